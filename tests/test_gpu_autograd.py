"""delta2zreion as a torch autograd operation: gradients equal the C ABI
adjoint, and dL/dzeta agrees with a finite difference of the FP64 model."""
import math

import numpy as np
import pytest

import prc_d2z
from oracle import d2z_ref as orc
from prc_d2z import fields
from prc_d2z.autograd import barrier_derivatives, delta2zreion_fn, param_gradients

pytestmark = pytest.mark.gpu


def _setup(N=32, nscales=8):
    box = 1.5 * N
    p = prc_d2z.Parameters(N=N, Nscales=nscales, BoxSize=box)
    cl = prc_d2z.CLParameters(Rmax=0.4 * box, zeta=30.0, M_min=1.47e9)
    return p, cl, fields.gaussian_field(N, box, seed=7), fields.gaussian_field(N, box, seed=8)


def test_autograd_matches_backward():
    import torch
    p, cl, d, dt = _setup()
    eng = prc_d2z.Delta2Zreion.from_parameters(p, cl, argmax=True)
    x = torch.from_numpy(d).cuda().requires_grad_(True)
    B = torch.tensor(eng.tables.barrier_b, dtype=torch.float64, requires_grad=True)
    zt = torch.from_numpy(dt).cuda() * 0.5
    z = delta2zreion_fn(x, eng, B)
    loss = ((z - zt) ** 2).mean()
    loss.backward()
    z2, am2, _ = eng.forward(x.detach(), want_argmax=True)
    assert torch.equal(z.detach(), z2) and torch.equal(eng.last_argmax, am2)
    g = (2.0 / z.numel()) * (z2 - zt)
    dd, dB = eng.backward(g, am2)
    np.testing.assert_allclose(x.grad.cpu().numpy(), dd.cpu().numpy(), rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(B.grad.numpy(), dB, rtol=1e-6)
    eng.close()


def test_dzeta_matches_fp64_finite_difference():
    """L(zeta) = mean((z - z_t)^2) with B_r(zeta) = s_r erfc^-1(1/zeta) (exact
    inverse): the GPU dL/dB_r mapped to dL/dzeta vs a central difference of the
    FP64 model in zeta."""
    special = pytest.importorskip("scipy.special")
    import torch
    p, cl, d, dt = _setup()
    eng = prc_d2z.Delta2Zreion.from_parameters(p, cl, argmax=True)
    t = eng.tables
    box_mpc = float(np.float32(p.BoxSize) / np.float32(p.h))
    ok = np.isfinite(t.barrier_b)
    s = np.where(ok, t.barrier_b / t.erfizeta, np.nan)

    def B_of(zeta):
        return s * special.erfcinv(1.0 / zeta)

    zt = 0.5 * dt.astype(np.float64)

    def L(zeta):
        z, am, _ = orc.d2z(d.astype(np.float64), box_mpc, t.radii_mpc, t.barrier_a, B_of(zeta), t.DInit, mode="fp64")
        return float(np.mean((z - zt) ** 2)), z, am

    z0 = cl.zeta
    L0, zf, amf = L(z0)
    eng.set_barrier(B_of(z0), t.barrier_a)
    g = (2.0 / d.size * (zf - zt)).astype(np.float32)
    _, dB = eng.backward(torch.from_numpy(g).cuda(), torch.from_numpy(amf).cuda())
    t.erfizeta = float(special.erfcinv(1.0 / z0))
    t.barrier_b = B_of(z0)
    dBz, _ = barrier_derivatives(t, z0)
    grad = float(np.dot(np.nan_to_num(dB), dBz))
    h = 1e-4 * z0
    fd = (L(z0 + h)[0] - L(z0 - h)[0]) / (2 * h)
    assert abs(grad - fd) <= 1e-3 * abs(fd) + 1e-12, (grad, fd)
    eng.close()
