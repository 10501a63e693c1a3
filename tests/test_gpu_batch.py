"""Batches of boxes of different sizes (one graph launch) give exactly the
per-box results."""
import numpy as np
import pytest

import prc_d2z
from prc_d2z import fields

pytestmark = pytest.mark.gpu


def _box(N, nr, seed):
    box = 1.5 * N
    p = prc_d2z.Parameters(N=N, Nscales=nr, BoxSize=box)
    cl = prc_d2z.CLParameters(Rmax=0.4 * box, zeta=30.0, M_min=1.47e9)
    t = prc_d2z.compute_tables(p, cl)
    d = dict(N=N, box_mpc=float(np.float32(box) / np.float32(0.68)), radii_mpc=t.radii_mpc,
             barrier_b=t.barrier_b, barrier_a=t.barrier_a, growth_init=t.DInit)
    return d, fields.gaussian_field(N, box, seed=seed)


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_per_box(use_graph):
    import torch
    spec = [(16, 5), (24, 7), (32, 9), (48, 6), (64, 11), (96, 8), (32, 4)]
    boxes, fields_ = zip(*[_box(N, nr, 100 + i) for i, (N, nr) in enumerate(spec)])
    ref = []
    for b, d in zip(boxes, fields_):
        with prc_d2z.Delta2Zreion(b["N"], b["box_mpc"], b["radii_mpc"], b["barrier_b"], b["barrier_a"],
                                  b["growth_init"]) as ctx:
            ref.append(ctx.forward(d, want_argmax=False)[0])
    batch = prc_d2z.Batch(list(boxes), n_streams=3)
    dev = [torch.from_numpy(d).cuda() for d in fields_]
    out = [torch.empty_like(x) for x in dev]
    for _ in range(2):  # the second call replays the captured graph
        batch.forward(dev, out, use_graph=use_graph)
        torch.cuda.synchronize()
        for r, o in zip(ref, out):
            assert np.array_equal(o.cpu().numpy(), r)
    assert batch.launches() > 0
    batch.close()
