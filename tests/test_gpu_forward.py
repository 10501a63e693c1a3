"""GPU parity of the forward path (delta_lin -> zreion, argmax, delta_R, sigma_grid)
against the CPU oracle, through the C ABI."""
import math

import numpy as np
import pytest

import prc_d2z
from oracle import d2z_ref as orc
from prc_d2z import fields

pytestmark = pytest.mark.gpu

H_ = 0.68


def _setup(N, nscales=12, seed=None, rmax=None, zeta=30.0):
    box = 1.5 * N                                   # Mpc/h, 1.5 Mpc/h cells
    p = prc_d2z.Parameters(N=N, Nscales=nscales, BoxSize=box)
    cl = prc_d2z.CLParameters(Rmax=rmax or 0.4 * box, zeta=zeta, M_min=1.47e9)
    delta = fields.gaussian_field(N, box, seed=seed if seed is not None else N)
    t = prc_d2z.compute_tables(p, cl)
    box_mpc = float(np.float32(box) / np.float32(H_))
    return p, cl, delta, t, box_mpc


def _eps_z(A, dmax, z):
    return A * 1e-5 * dmax + 2 * np.spacing(np.abs(z).astype(np.float32)).astype(np.float64)


@pytest.mark.parametrize("N", [8, 12, 16, 24, 32, 48, 64, 96, 128])
def test_forward_zreion_argmax(N):
    p, cl, delta, t, box_mpc = _setup(N)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
        z, am, _ = ctx.forward(delta)
    zs, dmax = orc.z_stack(delta, box_mpc, t.radii_mpc, t.barrier_a, t.barrier_b, t.DInit, mode="fp32")
    best, rbest, gap = orc.margins(zs)
    zo = np.where(best > 0, best, 0.0)
    amo = np.where(best > 0, rbest, 255)
    eps = _eps_z(t.barrier_a, dmax, zo)
    clear = gap > eps
    frac_near = 1.0 - clear.mean()
    assert frac_near < 0.01, frac_near
    dz = np.abs(z.astype(np.float64) - zo)
    assert np.all(dz[clear] <= eps[clear]), float(dz[clear].max())
    assert np.array_equal(am[clear], amo[clear].astype(np.uint8))
    # near-barrier cells still land on one of the two candidates
    assert np.all(dz <= eps + np.maximum(gap, 0) + 1e-6)


@pytest.mark.parametrize("N", [16, 32, 64, 128])
def test_forward_matches_full_oracle_run(N):
    """The whole oracle chain (fp32 mode) gives the same zreion/argmax."""
    p, cl, delta, t, box_mpc = _setup(N, nscales=10)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl, sigma_grid=True) as ctx:
        z, am, sig = ctx.forward(delta, want_sigma_grid=True)
    zo, amo, sigo = orc.d2z(delta, box_mpc, t.radii_mpc, t.barrier_a, t.barrier_b, t.DInit, mode="fp32")
    agree = np.mean(am == amo)
    assert agree > 0.999, agree
    same = am == amo
    assert np.max(np.abs(z[same] - zo[same])) < 1e-4
    np.testing.assert_allclose(sig, sigo, rtol=1e-5)


@pytest.mark.parametrize("N", [16, 32, 64, 96, 128])
@pytest.mark.parametrize("r", [0, 5, 11])
def test_delta_R_relative_rms(N, r):
    """delta_R within 1e-5 relative RMS of the FP64 oracle."""
    p, cl, delta, t, box_mpc = _setup(N)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
        dR = ctx.smooth(delta, r)
    ref = orc.delta_R(delta.astype(np.float64), box_mpc, t.radii_mpc[r], t.DInit, mode="fp64")
    rel = math.sqrt(np.mean((dR - ref) ** 2) / np.mean(ref ** 2))
    assert rel < 1e-5, rel


def test_device_and_host_paths_agree():
    import torch
    p, cl, delta, t, box_mpc = _setup(32)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
        zh, ah, _ = ctx.forward(delta)
        zd, ad, _ = ctx.forward(torch.from_numpy(delta).cuda())
        torch.cuda.synchronize()
    assert np.array_equal(zh, zd.cpu().numpy())
    assert np.array_equal(ah, ad.cpu().numpy())


@pytest.mark.parametrize("B", [1, 3, 5, 16, 24, 32])
def test_radius_batch_invariance(B):
    """The result does not depend on how radii are grouped into sweeps."""
    p, cl, delta, t, box_mpc = _setup(32, nscales=40)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl, radius_batch=1) as c1:
        z1, a1, _ = c1.forward(delta)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl, radius_batch=B) as cb:
        zb, ab, _ = cb.forward(delta)
    assert np.array_equal(z1, zb) and np.array_equal(a1, ab)


def test_history_counts_exact():
    p, cl, delta, t, box_mpc = _setup(64)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
        z, _, _ = ctx.forward(delta)
        counts, hist, hz = ctx.history(z)
    co, ho, hzo = orc.history(z)
    assert np.array_equal(counts, co)
    np.testing.assert_array_equal(hist, ho)
    np.testing.assert_array_equal(hz[1:], hzo[1:])


@pytest.mark.parametrize("want_argmax", [False, True])
def test_pinned_host_buffers_read_and_written_in_place(want_argmax):
    """Pinned (mapped) host buffers are read by the forward R2C and written by
    the last sweep in place; the result is bit-identical to the device path
    and to the staged path of pageable buffers."""
    import torch
    p, cl, delta, t, box_mpc = _setup(64, nscales=12)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl, radius_batch=5) as ctx:
        zd, ad, _ = ctx.forward(torch.from_numpy(delta).cuda(), want_argmax=want_argmax)
        torch.cuda.synchronize()
        hd = torch.empty(delta.shape, dtype=torch.float32, pin_memory=True)
        hd.copy_(torch.from_numpy(delta))
        hz = torch.full(delta.shape, -7.0, dtype=torch.float32, pin_memory=True)
        ha = torch.zeros(delta.shape, dtype=torch.uint8, pin_memory=True) if want_argmax else None
        for _ in range(2):  # twice: the running max must not leak between calls
            ctx.forward(hd.numpy(), zreion=hz.numpy(), argmax=ha.numpy() if want_argmax else None,
                        want_argmax=want_argmax)
            assert np.array_equal(hz.numpy(), zd.cpu().numpy())
            if want_argmax:
                assert np.array_equal(ha.numpy(), ad.cpu().numpy())
        zp, ap, _ = ctx.forward(delta.copy(), want_argmax=want_argmax)   # pageable: staged copies
        assert np.array_equal(zp, zd.cpu().numpy())


@pytest.mark.parametrize("want_argmax,pinned", [(False, True), (True, True), (True, False)])
def test_forward_many_equals_single_calls(want_argmax, pinned):
    """prc_d2z_forward_many over five boxes (two device buffer sets reused
    alternately, copies overlapping the neighbouring boxes' kernels) gives
    each box's single-call result bit for bit."""
    import torch
    N, n = 64, 5
    p, cl, _, t, box_mpc = _setup(N, nscales=12)
    deltas = [fields.gaussian_field(N, p.BoxSize, seed=100 + i) for i in range(n)]

    def host(shape, dtype, fill=0):
        if pinned:
            return torch.full(shape, fill, dtype=dtype, pin_memory=True).numpy()
        return np.full(shape, fill, dtype=torch.empty(0, dtype=dtype).numpy().dtype)

    with prc_d2z.Delta2Zreion.from_parameters(p, cl, radius_batch=5) as ctx:
        ref = [ctx.forward(d.copy(), want_argmax=want_argmax) for d in deltas]
        hd = [host(d.shape, torch.float32) for d in deltas]
        for h, d in zip(hd, deltas):
            h[...] = d
        hz = [host(deltas[0].shape, torch.float32, -7.0) for _ in range(n)]
        ha = [host(deltas[0].shape, torch.uint8, 0) for _ in range(n)] if want_argmax else None
        for _ in range(2):  # twice: buffers and events are reused across calls
            ctx.forward_many(hd, hz, ha)
            for i in range(n):
                assert np.array_equal(hz[i], ref[i][0]), i
                if want_argmax:
                    assert np.array_equal(ha[i], ref[i][1]), i
        # one output buffer for every box: the last box's result remains
        ctx.forward_many(hd, [hz[0]] * n, [ha[0]] * n if want_argmax else None)
        assert np.array_equal(hz[0], ref[-1][0])
        if want_argmax:
            assert np.array_equal(ha[0], ref[-1][1])
        # a single box, and an empty list
        ctx.forward_many(hd[:1], hz[:1], ha[:1] if want_argmax else None)
        assert np.array_equal(hz[0], ref[0][0])
        ctx.forward_many([], [], [] if want_argmax else None)
