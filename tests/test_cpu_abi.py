"""CPU-only checks of the shared library: it loads, exports every symbol the
header declares, and validates arguments before touching a device."""
import ctypes
import os
import re

import numpy as np
import pytest

import prc_d2z
from prc_d2z import _lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    src = open(os.path.join(REPO, "include", "prc_d2z.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(prc_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = _header_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(_lib.EXPORTS)


def test_supported_sizes():
    s = prc_d2z.supported_sizes()
    assert s == [8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024]


def _desc(N=32, nr=4, **kw):
    R = np.linspace(2.0, 8.0, nr)
    B = np.full(nr, 5.0)
    d = _lib.prc_d2z_desc()
    d.N = N
    d.n_radii = nr
    d.box_mpc = 70.0
    d.radii_mpc = R.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.barrier_b = B.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.barrier_a = 0.75
    d.growth_init = 1.0
    for k, v in kw.items():
        setattr(d, k, v)
    return d, (R, B)


@pytest.mark.parametrize("kw,code", [
    ({"N": 100}, _lib.PRC_ERR_UNSUPPORTED),
    ({"N": 640}, _lib.PRC_ERR_UNSUPPORTED),
    ({"N": 2048}, _lib.PRC_ERR_UNSUPPORTED),
    ({"n_radii": 0}, _lib.PRC_ERR_INVALID),
    ({"n_radii": 300}, _lib.PRC_ERR_INVALID),
    ({"box_mpc": 0.0}, _lib.PRC_ERR_INVALID),
    ({"growth_init": -1.0}, _lib.PRC_ERR_INVALID),
    ({"barrier_a": 0.0}, _lib.PRC_ERR_INVALID),
    ({"radius_batch": 99}, _lib.PRC_ERR_INVALID),
])
def test_create_rejects_bad_descriptors(kw, code):
    L = _lib.load()
    nr = kw.get("n_radii", 4)
    d, keep = _desc(**{k: v for k, v in kw.items() if k != "n_radii"}, n_radii=nr) if "n_radii" in kw else _desc(**kw)
    ctx = ctypes.c_void_p()
    st = L.prc_d2z_create(ctypes.byref(d), ctypes.byref(ctx))
    assert st == code
    assert not ctx.value
    assert len(L.prc_last_error()) > 0


def test_null_arguments_are_errors_not_crashes():
    L = _lib.load()
    assert L.prc_d2z_create(None, None) == _lib.PRC_ERR_INVALID
    assert L.prc_d2z_forward(None, None, 0, None, None, 0, None) == _lib.PRC_ERR_INVALID
    assert L.prc_d2z_forward_many(None, 1, None, None, None) == _lib.PRC_ERR_INVALID
    assert L.prc_d2z_history(None, None, 0, None, None, None) == _lib.PRC_ERR_INVALID
    assert L.prc_d2z_backward(None, None, None, 0, None, 0, None) == _lib.PRC_ERR_INVALID
    assert L.prc_d2z_destroy(None) == _lib.PRC_OK
    assert L.prc_compute_tables(None, None) == _lib.PRC_ERR_INVALID


def test_python_binding_raises_loudly_without_library(tmp_path):
    with pytest.raises(RuntimeError, match="missing"):
        _lib._lib_saved = _lib._lib
        try:
            _lib._lib = None
            _lib.load(str(tmp_path / "nope.so"))
        finally:
            _lib._lib = _lib._lib_saved


@pytest.mark.parametrize("nscales", [1, 255])
def test_tables_reject_radius_counts_the_reference_does_not_check(nscales):
    # Nscales = 1 makes the reference's radius spacing a division by zero
    # (delta2zreion_d2z.C:38); more than 254 radii do not fit the argmax byte
    p = prc_d2z.Parameters(N=32, Nscales=nscales, BoxSize=100.0)
    cl = prc_d2z.CLParameters(Rmax=60.0, zeta=80.5, M_min=1e9 / 0.68)
    with pytest.raises(_lib.PrcError) as e:
        prc_d2z.compute_tables(p, cl)
    assert e.value.code == _lib.PRC_ERR_INVALID


def test_autotuner_candidates_and_cache_path(monkeypatch, tmp_path):
    """The tuner's search space (radius batches up to the kernels' 64 and to
    60 GB of slots: at most 32 at 768 and 12 at 1024, where a slot is 1.8 and
    4.3 GB; never above the radius count; every compiled window variant) and
    its cache location, without a GPU."""
    from prc_d2z import autotune
    b, v = autotune.candidates(512, 64)
    assert b == [4, 8, 12, 16, 24, 32, 48, 64] and v == list(range(prc_d2z.win_variants(512)))
    b, _ = autotune.candidates(1024, 96)
    assert max(b) == 12
    b, _ = autotune.candidates(768, 64)
    assert max(b) == 32
    b, _ = autotune.candidates(128, 10)
    assert b == [4, 8, 10]
    assert prc_d2z.win_variants(100) == 0
    monkeypatch.setenv("PRC_D2Z_TUNE_CACHE", str(tmp_path / "t.json"))
    assert autotune.cache_path() == str(tmp_path / "t.json")
