"""Tuning knobs and the autotuner: every window-pass variant and radius
batch gives the default's result within float rounding; the autotuner picks a
compiled choice and caches it; a tuned batch reproduces tuned per-box runs."""
import json

import numpy as np
import pytest

import prc_d2z
from prc_d2z import autotune, fields

pytestmark = pytest.mark.gpu


def _ctx(N, nr=10, **kw):
    box = 1.5 * N
    p = prc_d2z.Parameters(N=N, Nscales=nr, BoxSize=box)
    cl = prc_d2z.CLParameters(Rmax=0.4 * box, zeta=30.0, M_min=1.47e9)
    return prc_d2z.Delta2Zreion.from_parameters(p, cl, **kw), fields.gaussian_field(N, box, seed=N + 3)


@pytest.mark.parametrize("N", [128, 256, 512])
def test_every_variant_matches_default(N):
    nv = prc_d2z.win_variants(N)
    assert nv >= 1
    ctx, d = _ctx(N, radius_batch=16)
    z0, a0, _ = ctx.forward(d)
    A = ctx.tables.barrier_a
    for v in range(nv):
        for B in (4, 16, 32):
            ctx.tune(B, v)
            z, a, _ = ctx.forward(d)
            # a different radix plan only changes float rounding of delta_R
            assert float(np.max(np.abs(z - z0))) <= A * 2e-5 * float(np.max(np.abs(d))) + 1e-5, (v, B)
            assert np.mean(a == a0) > 0.999, (v, B)
    with pytest.raises(prc_d2z.PrcError):
        ctx.tune(0, nv)
    with pytest.raises(prc_d2z.PrcError):
        ctx.tune(65, 0)   # more radii per sweep than the kernels' parameter arrays hold
    ctx.close()


def test_autotune_picks_and_caches(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("PRC_D2Z_TUNE_CACHE", str(path))
    e = autotune.tune(128, 12, reps=2)
    batches, variants = autotune.candidates(128, 12)
    assert e["radius_batch"] in batches and e["win_variant"] in variants
    assert len(e["times_ms"]) == len(batches) * len(variants)
    data = json.loads(path.read_text())
    assert any(k.endswith("|N=128|nr=12") for k in data)
    assert autotune.tuned(128, 12) == (e["radius_batch"], e["win_variant"])   # from the cache


def test_tuned_batch_matches_tuned_boxes():
    import torch
    spec = [(128, 9), (256, 7), (64, 5)]
    boxes, fl, ctxs = [], [], []
    for i, (N, nr) in enumerate(spec):
        box = 1.5 * N
        p = prc_d2z.Parameters(N=N, Nscales=nr, BoxSize=box)
        cl = prc_d2z.CLParameters(Rmax=0.4 * box, zeta=30.0, M_min=1.47e9)
        t = prc_d2z.compute_tables(p, cl)
        boxes.append(dict(N=N, box_mpc=float(np.float32(box) / np.float32(0.68)), radii_mpc=t.radii_mpc,
                          barrier_b=t.barrier_b, barrier_a=t.barrier_a, growth_init=t.DInit, radius_batch=4))
        fl.append(torch.from_numpy(fields.gaussian_field(N, box, seed=50 + i)).cuda())
    v_of = {N: prc_d2z.win_variants(N) - 1 for N, _ in spec}
    batch = prc_d2z.Batch(boxes, n_streams=2)
    for i, (N, _) in enumerate(spec):
        batch.tune(i, 0, v_of[N])
    out = [torch.empty_like(x) for x in fl]
    batch.forward(fl, out, use_graph=True)
    torch.cuda.synchronize()
    for b, x, o in zip(boxes, fl, out):
        with prc_d2z.Delta2Zreion(b["N"], b["box_mpc"], b["radii_mpc"], b["barrier_b"], b["barrier_a"],
                                  b["growth_init"], radius_batch=4, argmax=False) as c:
            c.tune(0, v_of[b["N"]])
            z, _, _ = c.forward(x, want_argmax=False)
            torch.cuda.synchronize()
            assert torch.equal(z, o)
    batch.close()
