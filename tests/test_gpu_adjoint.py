"""GPU adjoint (prc_d2z_backward) against the FP64 oracle adjoint and central
finite differences of the GPU forward."""
import math

import numpy as np
import pytest

import prc_d2z
from oracle import d2z_ref as orc
from prc_d2z import fields

pytestmark = pytest.mark.gpu
H_ = 0.68


def _setup(N, nscales=10, seed=None):
    box = 1.5 * N
    p = prc_d2z.Parameters(N=N, Nscales=nscales, BoxSize=box)
    cl = prc_d2z.CLParameters(Rmax=0.4 * box, zeta=30.0, M_min=1.47e9)
    delta = fields.gaussian_field(N, box, seed=seed if seed is not None else 100 + N)
    t = prc_d2z.compute_tables(p, cl)
    return p, cl, delta, t, float(np.float32(box) / np.float32(H_))


@pytest.mark.parametrize("N", [16, 32, 48, 64, 96, 128])
def test_backward_matches_fp64_adjoint(N):
    p, cl, delta, t, box_mpc = _setup(N)
    rng = np.random.default_rng(N)
    g = rng.standard_normal(delta.shape).astype(np.float32)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
        z, am, _ = ctx.forward(delta)
        dd, dB = ctx.backward(g, am)
    ref, dBref = orc.adjoint(g, am, box_mpc, t.radii_mpc, t.barrier_a, t.DInit)
    rel = np.linalg.norm(dd - ref) / np.linalg.norm(ref)
    assert rel < 1e-5, rel
    np.testing.assert_allclose(dB, dBref, rtol=1e-5, atol=1e-9 * np.abs(dBref).max())


def test_backward_device_path_and_batches():
    import torch
    p, cl, delta, t, box_mpc = _setup(32, nscales=12)
    g = np.random.default_rng(3).standard_normal(delta.shape).astype(np.float32)
    outs = []
    for B in (1, 5, 12):
        with prc_d2z.Delta2Zreion.from_parameters(p, cl, radius_batch=B) as ctx:
            z, am, _ = ctx.forward(torch.from_numpy(delta).cuda())
            dd, dB = ctx.backward(torch.from_numpy(g).cuda(), am)
            torch.cuda.synchronize()
            outs.append((dd.cpu().numpy(), dB))
    for dd, dB in outs[1:]:
        np.testing.assert_allclose(dd, outs[0][0], rtol=0, atol=1e-6 * np.abs(outs[0][0]).max())
        np.testing.assert_allclose(dB, outs[0][1], rtol=1e-6)


def test_gpu_gradient_matches_finite_differences_of_the_model():
    """Loss L = mean((z - z_t)^2) against a target from another seed; the GPU
    gradient dL/d delta_lin at 64 random cells vs central differences (step
    1e-3 sigma) of the FP64 forward model.  Both use the FP64 argmax; cells
    whose perturbation flips an argmax are not checkable and are counted."""
    N = 32
    p, cl, delta, t, box_mpc = _setup(N, nscales=8)
    _, _, target, _, _ = _setup(N, nscales=8, seed=999)
    R, A, B, D = t.radii_mpc, t.barrier_a, t.barrier_b, t.DInit
    d64 = delta.astype(np.float64)
    zt, _, _ = orc.d2z(target.astype(np.float64), box_mpc, R, A, B, D, mode="fp64")

    def loss(d):
        z, am, _ = orc.d2z(d, box_mpc, R, A, B, D, mode="fp64")
        return float(np.mean((z - zt) ** 2)), am

    L0, am0 = loss(d64)
    z0, _, _ = orc.d2z(d64, box_mpc, R, A, B, D, mode="fp64")
    g = (2.0 * (z0 - zt) / N ** 3).astype(np.float32)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl, radius_batch=3) as ctx:
        grad, _ = ctx.backward(g, am0)
    h = 1e-3 * float(delta.std())
    rng = np.random.default_rng(11)
    ok = checked = 0
    for c in rng.choice(N ** 3, 64, replace=False):
        idx = np.unravel_index(c, delta.shape)
        dp, dm = d64.copy(), d64.copy()
        dp[idx] += h
        dm[idx] -= h
        Lp, amp = loss(dp)
        Lm, amm = loss(dm)
        if not (np.array_equal(amp, am0) and np.array_equal(amm, am0)):
            continue
        checked += 1
        fd = (Lp - Lm) / (2 * h)
        if abs(fd - grad[idx]) <= 1e-3 * abs(fd) + 1e-12:
            ok += 1
    assert checked >= 48, checked
    assert ok == checked, (ok, checked)
