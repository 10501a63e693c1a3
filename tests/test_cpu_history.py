"""Host side of the history-correction chain against its oracle (CPU only)."""
import subprocess
import sys

import numpy as np

import prc_d2z
from oracle import history_ref as hr


def _fcoll_table(path, n=2001, zmin=0.0, zmax=50.0, smin=4.63):
    z = np.linspace(zmin, zmax, n)
    tab = np.array([hr.fcoll(v, 0.31, 0.69, -1.0, smin) for v in z], np.float32)
    with open(path, "wb") as fh:
        np.array([zmin, zmax], np.float32).tofile(fh)
        np.array([n], np.int32).tofile(fh)
        tab.tofile(fh)
    return path


def test_unseeded_rand_sequence_is_reproduced():
    """random_r from initstate_r(1) is the sequence a fresh process's rand() gives."""
    code = "import ctypes, ctypes.util; c = ctypes.CDLL(ctypes.util.find_library('c')); print([c.rand() for _ in range(8)])"
    fresh = eval(subprocess.run([sys.executable, "-c", code], capture_output=True, text=True).stdout)
    g = hr.GlibcRand()
    assert [g.rand() for _ in range(8)] == fresh


def test_float2float_table(tmp_path):
    path = _fcoll_table(str(tmp_path / "fcoll_table.tab"))
    t = prc_d2z.Float2FloatTable(path)
    o = hr.f2f_load(path)
    for z in [-1.0, 0.0, 0.013, 3.7, 8.0, 12.345, 49.99, 50.0, 60.0]:
        assert np.float32(t.Float2Float(z)) == hr.f2f_eval(o, z)


def test_fcoll_matches_the_oracle():
    for z in [0.5, 6.0, 8.0, 15.0, 30.0]:
        assert np.float32(prc_d2z.fcoll(z, 0.0, 0.31, 0.69, -1.0, 4.63)) == hr.fcoll(z, 0.31, 0.69, -1.0, 4.63)


def test_chistory_and_zvz_match_the_oracle(tmp_path):
    path = _fcoll_table(str(tmp_path / "fcoll_table.tab"))
    rng = np.random.default_rng(0)
    mfp = np.sort(rng.uniform(1.0, 80.0, 64)).astype(np.float32)
    ch = prc_d2z.chistory(prc_d2z.Float2FloatTable(path), mfp, 60.0, 30.0)
    cho = hr.chistory(hr.f2f_load(path), mfp, 60.0, 30.0)
    np.testing.assert_array_equal(ch, cho)
    counts = np.zeros(100000)
    counts[70000:99000] = rng.poisson(3.0, 29000)
    hist = np.cumsum((counts / counts.sum()).astype(np.float32), dtype=np.float32)
    np.testing.assert_array_equal(prc_d2z.zvz_map(hist, ch), hr.zvz(hist, ch))
