"""The committed golden fixtures (tests/golden, written by make_golden.py)
against the CPU oracle, the field generator and the host tables."""
import os

import numpy as np
import pytest

import prc_d2z
from oracle import d2z_ref as orc
from prc_d2z import fields

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(f for f in os.listdir(GOLD) if f.endswith(".npz"))


def _load(name):
    return dict(np.load(os.path.join(GOLD, name)))


def test_fixtures_present():
    assert len(CASES) >= 2


@pytest.mark.parametrize("name", CASES)
def test_field_generator_reproduces_fixture(name):
    g = _load(name)
    d = fields.gaussian_field(int(g["N"]), float(g["box_hmpc"]), seed=int(g["seed"]))
    rel = np.linalg.norm(d - g["delta"]) / np.linalg.norm(g["delta"])
    assert rel < 1e-6, rel


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_fixture(name):
    g = _load(name)
    d = g["delta"]
    args = (float(g["box_mpc"]), g["radii_mpc"], float(g["barrier_a"]), g["barrier_b"], float(g["dinit"]))
    z64, a64, _ = orc.d2z(d.astype(np.float64), *args, mode="fp64")
    gap = g["gap64"]
    clear = gap > 1e-9
    np.testing.assert_allclose(z64, g["zreion64"], rtol=0, atol=1e-10)
    assert np.array_equal(a64[clear], g["argmax64"][clear])
    z32, a32, _ = orc.d2z(d, *args, mode="fp32")
    eps = 1e-5 * float(g["dmax64"])
    ok32 = gap > eps
    np.testing.assert_allclose(z32[ok32], g["zreion32"][ok32], rtol=0, atol=eps)
    assert np.array_equal(a32[ok32], g["argmax32"][ok32])
    counts, _, _ = orc.history(g["zreion64"].astype(np.float32))
    nz = np.nonzero(counts)[0]
    assert np.array_equal(nz, g["hist_bins"]) and np.array_equal(counts[nz], g["hist_counts"])


@pytest.mark.parametrize("name", CASES)
def test_host_tables_match_fixture(name):
    """The C++ host tables (prc_compute_tables) give the fixture's radii and,
    within the reference's 1e-4 bracket of erfc^-1 (the fixtures hold the
    exact root), its barrier offsets; tests/test_cpu_tables.py pins every
    other factor of B_r to 1e-6."""
    g = _load(name)
    N = int(g["N"])
    p = prc_d2z.Parameters(N=N, Nscales=len(g["radii_mpc"]), BoxSize=float(g["box_hmpc"]), Rmin=2.0)
    cl = prc_d2z.CLParameters(Rmax=float(g["rmax"]), zeta=float(g["zeta"]), M_min=1.47e9)
    t = prc_d2z.compute_tables(p, cl)
    # float pow(10, .) of the C library and of numpy may differ by an ulp
    np.testing.assert_allclose(t.radii_mpc, g["radii_mpc"], rtol=4e-7)
    np.testing.assert_allclose(t.barrier_a, float(g["barrier_a"]), rtol=1e-7)
    np.testing.assert_allclose(t.DInit, float(g["dinit"]), rtol=1e-7)
    ok = np.isfinite(g["barrier_b"])
    assert np.array_equal(np.isfinite(t.barrier_b), ok)
    np.testing.assert_allclose(t.barrier_b[ok], g["barrier_b"][ok], rtol=1e-4)
