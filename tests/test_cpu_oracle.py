"""The oracle itself: known-answer cases (plane waves, a zero field, Parseval,
the NaN barrier, ties), fp32 vs fp64 agreement, the history binning and the
adjoint against finite differences.  CPU only."""
import math

import numpy as np
import pytest

from oracle import d2z_ref as orc

H_ = 0.68


def test_plane_wave_is_scaled_by_the_window():
    N, box = 32, 40.0
    x = np.arange(N)
    m = (3, 1, 2)
    arg = 2 * np.pi * (m[0] * x[:, None, None] + m[1] * x[None, :, None] + m[2] * x[None, None, :]) / N
    d = np.cos(arg)
    R = 3.0
    dR = orc.delta_R(d, box, R, mode="fp64")
    k = 2 * np.pi / box * math.sqrt(sum(q * q for q in m))
    xk = k * R
    W = 3 * (math.sin(xk) - xk * math.cos(xk)) / xk ** 3
    np.testing.assert_allclose(dR, W * d, atol=1e-12)
    # float32 faithful chain agrees to float precision
    dR32 = orc.delta_R(d.astype(np.float32), box, np.float32(R), mode="fp32")
    assert np.max(np.abs(dR32 - W * d)) < 2e-6


def test_zero_field_gives_uniform_zreion_at_the_largest_radius():
    N = 16
    R = np.linspace(2.0, 10.0, 6)
    B = np.linspace(5.0, 7.0, 6)          # B grows with R as for a real sigma(R)
    A = 0.75
    z, am, sig = orc.d2z(np.zeros((N, N, N), np.float32), 30.0, R, A, B, mode="fp32")
    expect = np.float32(A * B[-1] - 1)
    assert np.all(z == expect) and np.all(am == 5) and np.all(sig == 0)


def test_nan_barrier_never_updates_and_ties_keep_the_smaller_radius():
    N = 8
    rng = np.random.default_rng(0)
    d = rng.standard_normal((N, N, N)).astype(np.float32) * 0.1
    R = np.array([2.0, 2.0, 3.0])
    B = np.array([4.0, 4.0, float("nan")])  # radius 1 repeats radius 0; radius 2 is NaN
    z, am, _ = orc.d2z(d, 20.0, R, 0.75, B, mode="fp32")
    assert np.all(am[z > 0] == 0)          # strict > : the repeat never wins, NaN never wins


def test_parseval_of_the_forward_transform():
    rng = np.random.default_rng(1)
    d = rng.standard_normal((16, 16, 16))
    S = orc.forward_spectrum(d, 1.0, "fp64")
    w = np.full(S.shape, 2.0)
    w[..., 0] = 1
    w[..., -1] = 1
    np.testing.assert_allclose(np.sum(w * np.abs(S) ** 2) / d.size, np.sum(d * d), rtol=1e-12)


def test_fp32_and_fp64_chains_agree():
    N, box = 32, 48.0
    from prc_d2z import fields
    d = fields.gaussian_field(N, box, seed=5)
    p = orc.Parameters(N=N, Nscales=8, BoxSize=box, Rmax=12.0, zeta=30.0, M_min=1.47e9)
    T = orc.tables(p)
    bm = float(np.float32(box) / np.float32(H_))
    z32, a32, _ = orc.d2z(d, bm, T.R, T.A, T.B, T.DInit, mode="fp32")
    z64, a64, _ = orc.d2z(d, bm, T.R, T.A, T.B, T.DInit, mode="fp64")
    assert np.mean(a32 == a64) > 0.999
    assert np.max(np.abs(z32 - z64)[a32 == a64]) < 1e-4


def test_history_binning_matches_the_reference_formula():
    rng = np.random.default_rng(2)
    edge = [0.0, 49.9, 49.9001, 0.01, 0.005, 50.5]
    zz = np.concatenate([rng.uniform(0, 20, 4096 - len(edge)), edge]).astype(np.float32)
    counts, hist, hz = orc.history(zz.reshape(16, 16, 16))
    dz = np.float32((0.01 - 49.9) / 99999)
    ref = np.zeros(100000, np.int64)
    for v in zz:
        b = int((float(v) - 49.9) / float(dz))
        if 0 <= b < 100000:
            ref[b] += 1
    assert np.array_equal(counts, ref)
    assert hist[-1] == pytest.approx(ref.sum() / 4096, rel=1e-5)


def test_adjoint_matches_finite_differences_fp64():
    N, box = 16, 24.0
    from prc_d2z import fields
    d = fields.gaussian_field(N, box, seed=9).astype(np.float64)
    R = np.array([1.5, 2.5, 4.0, 6.0])
    B = np.array([5.0, 5.6, 6.1, 6.5])
    A = 0.75
    z, am, _ = orc.d2z(d, box, R, A, B, mode="fp64")
    g = np.random.default_rng(4).standard_normal(d.shape)
    grad, dB = orc.adjoint(g, am, box, R, A)
    h = 1e-6
    rng = np.random.default_rng(5)
    for c in rng.choice(N ** 3, 16, replace=False):
        idx = np.unravel_index(c, d.shape)
        dp, dm = d.copy(), d.copy()
        dp[idx] += h
        dm[idx] -= h
        zp, amp, _ = orc.d2z(dp, box, R, A, B, mode="fp64")
        zm, amm, _ = orc.d2z(dm, box, R, A, B, mode="fp64")
        if not (np.array_equal(amp, am) and np.array_equal(amm, am)):
            continue
        fd = np.sum(g * (zp - zm)) / (2 * h)
        assert fd == pytest.approx(grad[idx], rel=1e-5, abs=1e-9)
    # dL/dB_r by finite differences of B
    for r in range(len(R)):
        Bp, Bm = B.copy(), B.copy()
        Bp[r] += 1e-6
        Bm[r] -= 1e-6
        zp, _, _ = orc.d2z(d, box, R, A, Bp, mode="fp64")
        zm, _, _ = orc.d2z(d, box, R, A, Bm, mode="fp64")
        fd = np.sum(g * (zp - zm)) / 2e-6
        assert fd == pytest.approx(dB[r], rel=1e-5, abs=1e-8)
