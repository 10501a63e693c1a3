"""The adjoint at 256^3 x 64 radii (300 Mpc/h): loss L = mean((z - z_t)^2)
against a target from another seed; the GPU gradient dL/d delta_lin at 64
random cells against central differences (step 1e-3 sigma) of the FP64 model
(fp64_chain, cuFFT in double precision).  Both use the FP64 argmax; cells whose
perturbation flips an argmax anywhere are not checkable and are counted."""
import math

import numpy as np
import pytest

import prc_d2z
from prc_d2z import fields

pytestmark = pytest.mark.gpu


def test_gradient_matches_fp64_finite_differences_256():
    import torch
    from fp64_chain import kmag, tophat64
    N, box, nr = 256, 300.0, 64
    free, _ = torch.cuda.mem_get_info()
    if free < 24 * 2 ** 30:
        pytest.skip("not enough device memory for the FP64 model")
    p = prc_d2z.Parameters(N=N, Nscales=nr, BoxSize=box, Rmin=2.0)
    cl = prc_d2z.CLParameters(Rmax=60.0, zeta=80.5091, M_min=1e9 / 0.68)
    delta = fields.gaussian_field(N, box, seed=1, backend="torch").contiguous()
    target = fields.gaussian_field(N, box, seed=2, backend="torch").contiguous()
    ctx = prc_d2z.Delta2Zreion.from_parameters(p, cl, argmax=True)
    t = ctx.tables
    box_mpc = float(np.float32(box) / np.float32(0.68))
    km = kmag(N, box_mpc, delta.device)
    Ws = []
    for r in range(nr):
        W = tophat64(km * t.radii_mpc[r])
        W[0, 0, 0] = 0.0
        Ws.append(W)
    del km

    def model(d):
        spec = torch.fft.rfftn(d.double() / t.DInit)
        best = torch.full(d.shape, -math.inf, dtype=torch.float64, device=d.device)
        am = torch.full(d.shape, 255, dtype=torch.uint8, device=d.device)
        for r in range(nr):
            z = t.barrier_a * (torch.fft.irfftn(spec * Ws[r], s=(N, N, N)) + t.barrier_b[r]) - 1.0
            gt = z > best
            best = torch.where(gt, z, best)
            am[gt] = r
        z = torch.where(best > 0, best, torch.zeros_like(best))
        am = torch.where(best > 0, am, torch.full_like(am, 255))
        return z, am

    zt, _ = model(target.double())
    d64 = delta.double()
    z0, am0 = model(d64)
    g = (2.0 * (z0 - zt) / N ** 3).float().contiguous()
    grad, _ = ctx.backward(g, am0.contiguous())
    torch.cuda.synchronize()
    grad = grad.double()

    def loss(d):
        z, am = model(d)
        return float(((z - zt) ** 2).mean()), am

    h = 1e-3 * float(delta.std())
    rng = np.random.default_rng(256)
    ok = checked = 0
    worst = 0.0
    for c in rng.choice(N ** 3, 64, replace=False):
        idx = np.unravel_index(int(c), delta.shape)
        dp = d64.clone()
        dp[idx] += h
        Lp, amp = loss(dp)
        dp[idx] -= 2 * h
        Lm, amm = loss(dp)
        if not (torch.equal(amp, am0) and torch.equal(amm, am0)):
            continue
        checked += 1
        fd = (Lp - Lm) / (2 * h)
        gv = float(grad[idx])
        err = abs(fd - gv)
        worst = max(worst, err / max(abs(fd), 1e-30))
        if err <= 1e-3 * abs(fd) + 1e-14:
            ok += 1
    ctx.close()
    print(f"checked {checked} of 64 cells, worst relative difference {worst:.2e}")
    assert checked >= 32, checked
    assert ok == checked, (ok, checked, worst)
