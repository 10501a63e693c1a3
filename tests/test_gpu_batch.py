"""Batches of boxes of different sizes give exactly the per-box results, in
every batch mode: per-box launches (loop), the same captured into one graph,
and grouped launches (one launch per pass over all boxes of a grid size)."""
import numpy as np
import pytest

import prc_d2z
from prc_d2z import fields

pytestmark = pytest.mark.gpu


def _box(N, nr, seed, radius_batch=0):
    box = 1.5 * N
    p = prc_d2z.Parameters(N=N, Nscales=nr, BoxSize=box)
    cl = prc_d2z.CLParameters(Rmax=0.4 * box, zeta=30.0, M_min=1.47e9)
    t = prc_d2z.compute_tables(p, cl)
    d = dict(N=N, box_mpc=float(np.float32(box) / np.float32(0.68)), radii_mpc=t.radii_mpc,
             barrier_b=t.barrier_b, barrier_a=t.barrier_a, growth_init=t.DInit, radius_batch=radius_batch)
    return d, fields.gaussian_field(N, box, seed=seed)


def _reference(boxes, fields_, argmax):
    ref = []
    for b, d in zip(boxes, fields_):
        with prc_d2z.Delta2Zreion(b["N"], b["box_mpc"], b["radii_mpc"], b["barrier_b"], b["barrier_a"],
                                  b["growth_init"], radius_batch=b.get("radius_batch", 0)) as ctx:
            z, a, _ = ctx.forward(d, want_argmax=argmax)
            ref.append((z, a))
    return ref


# 16, 24 and 48 have no grouped kernels (they run per box inside a grouped
# batch); 32, 64 and 96 are grouped, with boxes of unequal radius counts
SPEC = [(16, 5), (24, 7), (32, 9), (48, 6), (64, 11), (96, 8), (32, 4), (64, 3), (32, 17)]


@pytest.mark.parametrize("mode", ["loop", "graph", "grouped"])
def test_batch_matches_per_box(mode):
    import torch
    boxes, fields_ = zip(*[_box(N, nr, 100 + i) for i, (N, nr) in enumerate(SPEC)])
    ref = _reference(boxes, fields_, False)
    batch = prc_d2z.Batch(list(boxes), n_streams=3)
    dev = [torch.from_numpy(d).cuda() for d in fields_]
    out = [torch.empty_like(x) for x in dev]
    for _ in range(2):  # the second call replays the captured graph
        batch.forward(dev, out, mode=mode)
        torch.cuda.synchronize()
        for (r, _), o in zip(ref, out):
            assert np.array_equal(o.cpu().numpy(), r)
    assert batch.launches() > 0
    batch.close()


def test_grouped_batch_argmax_new_pointers_and_radius_batches():
    """Grouped launches with argmax, with each box's own radius batch (4, 16
    or 3: 1 to 6 sweeps of unequal length per box), and with new output
    buffers on the second call (the tables change, the capture stays)."""
    import torch
    boxes, fields_ = zip(*[_box(N, nr, 200 + i, radius_batch=(4, 16, 3)[i % 3]) for i, (N, nr) in enumerate(SPEC)])
    ref = _reference(boxes, fields_, True)
    batch = prc_d2z.Batch(list(boxes), n_streams=2)
    dev = [torch.from_numpy(d).cuda() for d in fields_]
    for _ in range(2):
        out = [torch.full_like(x, -3.0) for x in dev]
        am = [torch.full(x.shape, 7, dtype=torch.uint8, device="cuda") for x in dev]
        batch.forward(dev, out, am, mode="grouped")
        torch.cuda.synchronize()
        for (rz, ra), o, a in zip(ref, out, am):
            assert np.array_equal(o.cpu().numpy(), rz)
            assert np.array_equal(a.cpu().numpy(), ra)
    # the groups of 32, 64 and 96 (3 + 3 x sweeps launches each) plus the
    # per-box launches of the other sizes
    assert batch.launches() < sum(1 for _ in SPEC) * 10
    batch.close()


def test_grouped_batch_with_a_faithful_window_box():
    """A box asking for the faithful float window is left out of the grouped
    launches of its size (they use the accurate window) and runs per box
    inside the same graph: its result equals a faithful single call, and the
    other boxes of its size still match theirs."""
    import torch
    spec = [(32, 6), (32, 7), (64, 5)]
    boxes, fields_ = zip(*[_box(N, nr, 400 + i) for i, (N, nr) in enumerate(spec)])
    boxes = [dict(b) for b in boxes]
    boxes[1]["faithful_window"] = True
    ref = []
    for b, d in zip(boxes, fields_):
        with prc_d2z.Delta2Zreion(b["N"], b["box_mpc"], b["radii_mpc"], b["barrier_b"], b["barrier_a"],
                                  b["growth_init"], faithful_window=b.get("faithful_window", False)) as ctx:
            ref.append(ctx.forward(d, want_argmax=False)[0])
    batch = prc_d2z.Batch(boxes, n_streams=2)
    dev = [torch.from_numpy(d).cuda() for d in fields_]
    out = [torch.empty_like(x) for x in dev]
    batch.forward(dev, out, mode="grouped")
    torch.cuda.synchronize()
    for r, o in zip(ref, out):
        assert np.array_equal(o.cpu().numpy(), r)
    batch.close()


def test_grouped_batch_rejects_partial_argmax():
    import torch
    boxes, fields_ = zip(*[_box(N, nr, 300 + i) for i, (N, nr) in enumerate([(32, 5), (64, 6)])])
    batch = prc_d2z.Batch(list(boxes), n_streams=1)
    dev = [torch.from_numpy(d).cuda() for d in fields_]
    out = [torch.empty_like(x) for x in dev]
    am = [torch.empty(dev[0].shape, dtype=torch.uint8, device="cuda"), None]
    from prc_d2z import _lib
    L = _lib.load()
    import ctypes
    dp = (ctypes.c_void_p * 2)(*[d.data_ptr() for d in dev])
    zp = (ctypes.c_void_p * 2)(*[o.data_ptr() for o in out])
    ap = (ctypes.c_void_p * 2)(am[0].data_ptr(), None)
    assert L.prc_d2z_batch_forward(batch._b, dp, zp, ap, _lib.PRC_BATCH_GROUPED) == _lib.PRC_ERR_INVALID
    assert L.prc_d2z_batch_forward(batch._b, dp, zp, None, 5) == _lib.PRC_ERR_INVALID
    batch.close()
