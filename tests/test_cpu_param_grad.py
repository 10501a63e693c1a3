"""Host mapping of dL/dB_r to dL/dzeta and dL/dM_min (prc_d2z.autograd),
against finite differences of the barrier table.  CPU only."""
import math

import numpy as np
import pytest

import prc_d2z
from prc_d2z.autograd import barrier_derivatives, param_gradients


def _tables(zeta=30.0, mmin=1.47e9):
    p = prc_d2z.Parameters(N=64, Nscales=12, BoxSize=96.0)
    cl = prc_d2z.CLParameters(Rmax=38.4, zeta=zeta, M_min=mmin)
    return p, cl, prc_d2z.compute_tables(p, cl)


def test_dB_dzeta_matches_exact_inverse_erfc_differences():
    special = pytest.importorskip("scipy.special")
    p, cl, t = _tables()
    dBz, _ = barrier_derivatives(t, cl.zeta)
    ok = np.isfinite(t.barrier_b)
    s = t.barrier_b[ok] / t.erfizeta            # sqrt(2(smin^2 - s_r^2))
    h = 1e-4 * cl.zeta
    fd = s * (special.erfcinv(1 / (cl.zeta + h)) - special.erfcinv(1 / (cl.zeta - h))) / (2 * h)
    # the tables hold the reference's bracketed erfc^-1 (1e-4 below the exact
    # root), which the analytic derivative evaluates at
    np.testing.assert_allclose(dBz[ok], fd, rtol=1e-3)


def test_dM_min_matches_table_differences():
    p, cl, t = _tables()
    g = np.random.default_rng(1).standard_normal(len(t.barrier_b))
    g[~np.isfinite(t.barrier_b)] = 0.0
    _, dm = param_gradients(t, p, cl, g)
    eps = 0.01
    hi = prc_d2z.compute_tables(p, prc_d2z.CLParameters(Rmax=cl.Rmax, zeta=cl.zeta, M_min=cl.M_min * math.exp(eps)))
    lo = prc_d2z.compute_tables(p, prc_d2z.CLParameters(Rmax=cl.Rmax, zeta=cl.zeta, M_min=cl.M_min * math.exp(-eps)))
    ok = np.isfinite(hi.barrier_b) & np.isfinite(lo.barrier_b)
    fd = float(np.dot(g[ok], (hi.barrier_b[ok] - lo.barrier_b[ok]))) / (2 * eps * cl.M_min)
    assert abs(dm - fd) <= 2e-2 * abs(fd), (dm, fd)


def test_nan_barriers_get_no_gradient():
    p, cl, t = _tables()
    t.barrier_b = t.barrier_b.copy()
    t.barrier_b[-1] = np.nan
    dBz, dBs = barrier_derivatives(t, cl.zeta)
    assert dBz[-1] == 0.0 and dBs[-1] == 0.0
    dz, dm = param_gradients(t, p, cl, np.ones(len(t.barrier_b)))
    assert np.isfinite(dz) and np.isfinite(dm)
