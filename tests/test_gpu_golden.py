"""The GPU path against the committed golden fixtures (tests/golden)."""
import os

import numpy as np
import pytest

import prc_d2z

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(f for f in os.listdir(GOLD) if f.endswith(".npz"))


def _ctx(g, **kw):
    return prc_d2z.Delta2Zreion(int(g["N"]), float(g["box_mpc"]), g["radii_mpc"], g["barrier_b"],
                                float(g["barrier_a"]), float(g["dinit"]), **kw)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("batch", [1, 4])
def test_gpu_zreion_argmax_match_fixture(name, batch):
    g = dict(np.load(os.path.join(GOLD, name)))
    with _ctx(g, radius_batch=batch) as ctx:
        z, am, _ = ctx.forward(g["delta"])
    zo, amo, gap = g["zreion64"], g["argmax64"], g["gap64"]
    eps = float(g["barrier_a"]) * 1e-5 * float(g["dmax64"]) + 2 * np.spacing(np.abs(zo).astype(np.float32))
    clear = gap > eps
    assert 1.0 - clear.mean() < 0.01
    dz = np.abs(z.astype(np.float64) - zo)
    assert np.all(dz[clear] <= eps[clear]), float(dz[clear].max())
    assert np.array_equal(am[clear], amo[clear])


@pytest.mark.parametrize("name", CASES)
def test_gpu_delta_r_matches_fixture(name):
    g = dict(np.load(os.path.join(GOLD, name)))
    with _ctx(g) as ctx:
        for r, key in ((0, "delta_r_first"), (len(g["radii_mpc"]) - 1, "delta_r_last")):
            dR = ctx.smooth(g["delta"], r).astype(np.float64)
            ref = g[key]
            rel = np.sqrt(np.mean((dR - ref) ** 2) / np.mean(ref ** 2))
            assert rel < 1e-5, (r, rel)


@pytest.mark.parametrize("name", CASES)
def test_gpu_history_counts_match_fixture(name):
    g = dict(np.load(os.path.join(GOLD, name)))
    with _ctx(g) as ctx:
        counts, _, _ = ctx.history(g["zreion64"].astype(np.float32))
    nz = np.nonzero(counts)[0]
    assert np.array_equal(nz, g["hist_bins"]) and np.array_equal(counts[nz], g["hist_counts"])
