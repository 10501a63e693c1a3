"""The C++ host tables (csrc/cosmo.cpp) against the oracle, one by one.

The reference computes these scalars in cosmology.C and math.C with GSL
(QAGS at epsrel 1e-7, Brent with a 1e-4 bracket).  The product restates them
in C++ (its own Gauss-Kronrod and Brent); the oracle restates them with scipy
(QUADPACK at epsrel 1e-9, the exact erfc^-1).  Every value is a float in the
reference, so agreement is stated in float ulps.
"""
import ctypes

import numpy as np
import pytest

import prc_d2z
from oracle import d2z_ref as orc
from prc_d2z import _lib

COSMOLOGIES = [
    dict(),  # the workloads' cosmology: Omega_m 0.31, Omega_b 0.049, h 0.68, n_s 0.965, sigma_8 0.81
    dict(Omegam=0.3, Omegab=0.045, Omegal=0.7, h=0.7, ns=0.96, sigma8=0.8),
]


def _ulps(a, b):
    a, b = np.float32(a), np.float32(b)
    return float(abs(np.float64(a) - np.float64(b)) / np.spacing(np.abs(b)))


@pytest.mark.parametrize("cos", COSMOLOGIES)
def test_pnorm_matches_quadrature(cos):
    """normalize (cosmology.C:246-272): sigma_8 normalisation, same float."""
    t = prc_d2z.compute_tables(prc_d2z.Parameters(**cos), prc_d2z.CLParameters(Rmax=60, zeta=50, M_min=1e9))
    assert _ulps(t.pnorm, orc.normalize(orc.Parameters(**cos))) <= 1


@pytest.mark.parametrize("cos", COSMOLOGIES)
def test_sigma2_matches_quadrature(cos):
    """cdmehint (cosmology.C:214-244) over 1e7..1e16 Msun, the masses of every
    radius of the workloads (2 cells of 1.5 Mpc/h to 60 Mpc/h) and M_min:
    within 2 float ulps (2.4e-7) of scipy's quad, the agreement the
    reference's own epsrel 1e-7 allows."""
    L = _lib.load()
    op = orc.Parameters(**cos)
    pn = orc.normalize(op)
    for m in np.logspace(7, 16, 14).astype(np.float32):
        out = ctypes.c_float()
        _lib.check(L.prc_sigma2(op.Omegam, op.Omegab, op.h, op.ns, pn, float(m), ctypes.byref(out)))
        assert _ulps(out.value, orc.cdmehint(op, pn, m)) <= 2, m


@pytest.mark.parametrize("N,box,nr,zeta,zinit", [(128, 200.0, 32, 82.44, 0.0), (64, 96.0, 24, 30.0, 6.0)])
def test_sigma_tables_match_oracle(N, box, nr, zeta, zinit):
    """sigma_min, every sigma_r, the radii and B_r of prc_compute_tables
    against the oracle's tables (delta2zreion_d2z.C:14-38,55,97-100).  With
    the oracle given the product's erfizeta, B_r agrees to 1e-6 relative (it
    differs only through the ulps of sigma_r and R); the product's erfizeta
    lies in the reference's bracket, at most 1e-4 below the exact root."""
    p = prc_d2z.Parameters(N=N, Nscales=nr, BoxSize=box, zInit=zinit)
    cl = prc_d2z.CLParameters(Rmax=60.0, zeta=zeta, M_min=1e9 / 0.68)
    t = prc_d2z.compute_tables(p, cl)
    op = orc.Parameters(N=N, Nscales=nr, BoxSize=box, Rmax=60.0, zeta=zeta, M_min=1e9 / 0.68, zInit=zinit)
    ot = orc.tables(op, erfizeta=t.erfizeta)
    assert _ulps(t.sigma_min, ot.sigma_min) <= 2
    # float pow(10, .) and log10f of the C library and of numpy may differ by
    # an ulp or two, so R does too, and sigma_r through R
    np.testing.assert_allclose(t.radii_mpc, ot.R, rtol=4e-7)
    np.testing.assert_allclose(t.sigma_r, ot.sigma_r, rtol=4e-7)
    ok = np.isfinite(ot.B)
    assert np.array_equal(np.isfinite(t.barrier_b), ok)
    np.testing.assert_allclose(t.barrier_b[ok], ot.B[ok], rtol=1e-6)
    exact = orc.inverse_erfc(np.float32(1.0 / np.float64(np.float32(zeta))))
    assert exact * (1 - 1e-4) - 1e-7 <= t.erfizeta <= exact + np.spacing(exact)
    assert _ulps(t.DInit, orc.growth(zinit, 0.31, 0.69, -1.0)) == 0
    assert t.barrier_a == pytest.approx(float(ot.A), rel=0, abs=0)


@pytest.mark.parametrize("z", [0.0, 6.0, 20.0, 3.5, 49.9])
def test_growth_matches_oracle(z):
    """growth (cosmology.C:174-212) bit for bit, including D(0) = 1."""
    g = prc_d2z.growth(z, 0.31, 0.69, -1.0)
    assert np.float32(g) == orc.growth(z, 0.31, 0.69, -1.0)
    if z == 0.0:
        assert g == 1.0


def test_tau_matches_oracle():
    """tau (cosmology.C:52-83) of a GetHistory-shaped history: the oracle's
    float restatement and the product agree to 2 ulps."""
    za = orc.history(np.zeros((4, 4, 4), np.float32))[2]
    xa = np.clip((12.0 - za) / 6.0, 0.0, 1.0).astype(np.float32)
    a = prc_d2z.tau(za, xa, 0.31, 0.049, 0.68)
    b = orc.tau(za, xa, 0.31, 0.049, 0.68)
    assert 0.03 < b < 0.2
    assert _ulps(a, b) <= 2


def test_inverse_erfc_bracket():
    """inverse_erfc (math.C:23-61): within the reference's 1e-4 bracket below
    the exact root for the zeta of every workload."""
    for zeta in (10.0, 30.0, 73.16, 80.51, 80.54, 81.69, 82.44):
        x = np.float32(1.0 / np.float64(np.float32(zeta)))
        got = prc_d2z.inverse_erfc(float(x))
        exact = orc.inverse_erfc(x)
        assert exact * (1 - 1e-4) - 1e-7 <= got <= exact + np.spacing(exact), zeta
