"""ctypes binding of libprc_d2z.so (the C ABI declared in include/prc_d2z.h).

Loading fails loudly: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libprc_d2z.so")

PRC_OK = 0
PRC_ERR_INVALID = -1
PRC_ERR_UNSUPPORTED = -2
PRC_ERR_CUDA = -3
PRC_ERR_ALLOC = -4
PRC_ERR_IO = -5
PRC_ERR_NUMERIC = -6
PRC_FLAG_ARGMAX = 1
PRC_FLAG_SIGMA_GRID = 2
PRC_FLAG_FAITHFUL_WINDOW = 4
PRC_BATCH_LOOP = 0
PRC_BATCH_GRAPH = 1
PRC_BATCH_GROUPED = 2
PRC_NHISTORY = 100000
PRC_ARGMAX_NONE = 255
PRC_MAX_RADII = 254
KINDS = ["r2c_z", "col_fwd", "win_x", "col_inv", "c2r_z", "adj_z", "adj_x", "c2r_plain"]
PRC_NKINDS = len(KINDS)

# every symbol the header declares (checked by the CPU tests)
EXPORTS = [
    "prc_compute_tables", "prc_growth", "prc_sigma2", "prc_inverse_erfc", "prc_tau",
    "prc_d2z_supported", "prc_d2z_create", "prc_d2z_forward", "prc_d2z_forward_many", "prc_d2z_smooth",
    "prc_d2z_history",
    "prc_d2z_backward", "prc_d2z_last_timing", "prc_d2z_last_launches", "prc_d2z_profile",
    "prc_d2z_profile_read", "prc_d2z_destroy", "prc_d2z_forward_static",
    "prc_f2f_load", "prc_f2f_eval", "prc_f2f_free", "prc_deltac", "prc_fcoll", "prc_d2z_bubble_mfp",
    "prc_chistory", "prc_zvz", "prc_d2z_correct", "prc_d2z_batch_create", "prc_d2z_batch_forward",
    "prc_d2z_batch_launches", "prc_d2z_batch_destroy", "prc_d2z_set_barrier",
    "prc_white_noise", "prc_d2z_gaussian_field", "prc_d2z_win_variants", "prc_d2z_tune",
    "prc_d2z_batch_tune", "prc_d2z_test_withhold_copy", "prc_last_error",
]


class PrcError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"prc error {code}: {msg}")
        self.code = code


class prc_params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("Omegam", "Omegab", "Omegal", "h", "ns", "sigma8", "w",
                                                "BoxSize", "zInit", "Rmin")] + [
        ("N", ctypes.c_int), ("Nscales", ctypes.c_int),
        ("Rmax", ctypes.c_float), ("zeta", ctypes.c_float), ("M_min", ctypes.c_float)]


class prc_tables(ctypes.Structure):
    _fields_ = [("DInit", ctypes.c_float), ("zHigh", ctypes.c_float), ("DHigh", ctypes.c_float),
                ("pnorm", ctypes.c_float), ("erfizeta", ctypes.c_float), ("sigma_min", ctypes.c_float),
                ("barrier_a", ctypes.c_double),
                ("radii_mpc", ctypes.POINTER(ctypes.c_double)),
                ("sigma_r", ctypes.POINTER(ctypes.c_float)),
                ("barrier_b", ctypes.POINTER(ctypes.c_double))]


class prc_d2z_desc(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("n_radii", ctypes.c_int), ("box_mpc", ctypes.c_double),
                ("radii_mpc", ctypes.POINTER(ctypes.c_double)),
                ("barrier_b", ctypes.POINTER(ctypes.c_double)),
                ("barrier_a", ctypes.c_double), ("growth_init", ctypes.c_double),
                ("radius_batch", ctypes.c_int), ("flags", ctypes.c_int), ("stream", ctypes.c_void_p)]


class prc_f2f_table(ctypes.Structure):
    _fields_ = [("minval", ctypes.c_float), ("maxval", ctypes.c_float), ("delta", ctypes.c_float),
                ("n", ctypes.c_int), ("table", ctypes.POINTER(ctypes.c_float))]


class prc_mfp_setup(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("box_mpc", ctypes.c_float), ("n_x", ctypes.c_int),
                ("n_skewers", ctypes.c_int)]


PRC_NCHISTORY = 10000
PRC_NX_MFP = 1000
PRC_NMFP = 200
PRC_NSKEWERS = 20000

_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load (once) the shared library; raise if it has not been built.
    PRC_D2Z_LIB in the environment overrides the in-tree path."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("PRC_D2Z_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(path)
    P, c_int, c_float, c_double, vp = ctypes.POINTER, ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_void_p
    L.prc_last_error.restype = ctypes.c_char_p
    L.prc_compute_tables.argtypes = [P(prc_params), P(prc_tables)]
    L.prc_growth.argtypes = [c_float] * 4
    L.prc_growth.restype = c_float
    L.prc_sigma2.argtypes = [c_float] * 6 + [P(c_float)]
    L.prc_inverse_erfc.argtypes = [c_float, P(c_float)]
    L.prc_tau.argtypes = [vp, vp, c_int, c_float, c_float, c_float]
    L.prc_tau.restype = c_float
    L.prc_d2z_supported.argtypes = [c_int]
    L.prc_d2z_create.argtypes = [P(prc_d2z_desc), P(vp)]
    L.prc_d2z_forward.argtypes = [vp, vp, c_int, vp, vp, c_int, vp]
    L.prc_d2z_forward_many.argtypes = [vp, c_int, vp, vp, vp]
    L.prc_d2z_history.argtypes = [vp, vp, c_int, vp, vp, vp]
    L.prc_d2z_smooth.argtypes = [vp, vp, c_int, c_int, vp, c_int]
    L.prc_d2z_backward.argtypes = [vp, vp, vp, c_int, vp, c_int, vp]
    L.prc_d2z_last_timing.argtypes = [vp, P(c_float)]
    L.prc_d2z_last_launches.argtypes = [vp, P(c_int)]
    L.prc_d2z_destroy.argtypes = [vp]
    L.prc_d2z_profile.argtypes = [vp, c_int]
    L.prc_d2z_forward_static.argtypes = [c_int, c_int, c_double, vp, vp, c_double, c_double, vp, vp, vp, vp]
    L.prc_d2z_profile_read.argtypes = [vp, P(c_double), P(ctypes.c_longlong)]
    L.prc_f2f_load.argtypes = [ctypes.c_char_p, P(prc_f2f_table)]
    L.prc_f2f_eval.argtypes = [P(prc_f2f_table), c_float]
    L.prc_f2f_eval.restype = c_float
    L.prc_f2f_free.argtypes = [P(prc_f2f_table)]
    L.prc_f2f_free.restype = None
    L.prc_deltac.argtypes = [c_float] * 4 + [P(c_float)]
    L.prc_deltac.restype = c_float
    L.prc_fcoll.argtypes = [c_float] * 6
    L.prc_fcoll.restype = c_float
    L.prc_d2z_bubble_mfp.argtypes = [vp, P(prc_mfp_setup), vp, vp, vp, vp, vp]
    L.prc_chistory.argtypes = [P(prc_f2f_table), vp, c_int, c_float, c_float, vp]
    L.prc_zvz.argtypes = [vp, vp, vp]
    L.prc_d2z_correct.argtypes = [vp, vp, vp, c_int]
    L.prc_d2z_batch_create.argtypes = [c_int, P(prc_d2z_desc), c_int, P(vp)]
    L.prc_d2z_batch_forward.argtypes = [vp, P(vp), P(vp), P(vp), c_int]
    L.prc_d2z_batch_launches.argtypes = [vp, P(c_int)]
    L.prc_d2z_batch_destroy.argtypes = [vp]
    L.prc_d2z_set_barrier.argtypes = [vp, vp, c_double]
    L.prc_d2z_win_variants.argtypes = [c_int]
    L.prc_d2z_tune.argtypes = [vp, c_int, c_int]
    L.prc_d2z_batch_tune.argtypes = [vp, c_int, c_int, c_int]
    L.prc_white_noise.argtypes = [vp, ctypes.c_longlong, ctypes.c_uint, vp]
    L.prc_d2z_gaussian_field.argtypes = [vp, ctypes.c_uint, vp, c_int, vp, c_int]
    L.prc_d2z_test_withhold_copy.argtypes = [c_int]
    for name in EXPORTS:
        if name in ("prc_f2f_free",):
            continue
        getattr(L, name).restype = getattr(L, name).restype or c_int
    L.prc_growth.restype = c_float
    L.prc_tau.restype = c_float
    L.prc_f2f_eval.restype = c_float
    L.prc_deltac.restype = c_float
    L.prc_fcoll.restype = c_float
    L.prc_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


def check(status: int) -> None:
    if status != PRC_OK:
        msg = load().prc_last_error().decode(errors="replace")
        raise PrcError(status, msg)
