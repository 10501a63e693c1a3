"""prc_d2z -- the excursion-set reionization step (pr-calc's delta2zreion) on
one GB300, called through the C ABI of libprc_d2z.so.

Host-side mirror of the reference's interface for this path (pr-calc c++/src):

  Parameters / CLParameters  the structs of allvars_d2z.h:58-70, same names
  read_parameter_file        io_d2z.C:16-162 (tags, comments, -usedvalues echo)
  compute_tables             delta2zreion_d2z.C:14-38,55,97-100 and
                             main_d2z.C:57-64 through prc_compute_tables
  Delta2Zreion               the device context: forward() replaces
                             main_d2z.C:57-71 + delta2zreion(), history()
                             GetHistory (bubblehistory_d2z.C:5-43), backward()
                             the adjoint (new)
  delta2zreion               one call from delta_lin to (zreion, argmax,
                             sigma_grid), like the reference's function

Arrays may be numpy arrays (host; the library copies through) or CUDA torch
tensors (device pointers, no copies).  Everything runs on the GPU; without the
built library every entry point raises.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import (PRC_ARGMAX_NONE, PRC_FLAG_ARGMAX, PRC_FLAG_SIGMA_GRID, PRC_NHISTORY, PrcError,
                   check, load)

__all__ = ["Parameters", "CLParameters", "Tables", "read_parameter_file", "compute_tables",
           "Delta2Zreion", "delta2zreion", "PrcError", "PRC_ARGMAX_NONE", "PRC_NHISTORY",
           "supported_sizes", "growth", "inverse_erfc", "tau", "Float2FloatTable", "fcoll",
           "chistory", "zvz_map", "Batch", "win_variants"]


@dataclass
class Parameters:
    """Parameter (allvars_d2z.h:58-64); BoxSize in Mpc/h as read."""
    Omegam: float = 0.31
    Omegab: float = 0.049
    Omegal: float = 0.69
    h: float = 0.68
    ns: float = 0.965
    sigma8: float = 0.81
    w: float = -1.0
    BoxSize: float = 200.0
    zInit: float = 0.0
    Rmin: float = 2.0
    N: int = 128
    Nscales: int = 32
    DeltaFile: str = ""
    RecordBubbleSizes: int = 0


@dataclass
class CLParameters:
    """clParameter (allvars_d2z.h:66-70) with the defaults of commandline_d2z.C:47-52."""
    Rmax: float = 256.0
    zeta: float = 10.0
    M_min: float = 1e8
    verbose: int = 0
    everbose: int = 0
    lean: int = 0
    Paramfile: str = ""
    Basename: str = "output/output"


@dataclass
class Tables:
    DInit: float
    zHigh: float
    DHigh: float
    pnorm: float
    erfizeta: float
    sigma_min: float
    barrier_a: float
    radii_mpc: np.ndarray = field(repr=False)
    sigma_r: np.ndarray = field(repr=False)
    barrier_b: np.ndarray = field(repr=False)


_TAGS = {"Omegam": "f", "Omegab": "f", "Omegal": "f", "h": "f", "ns": "f", "sigma8": "f", "w": "f",
         "BoxSize": "f", "zInit": "f", "Rmin": "f", "N": "i", "Nscales": "i", "DeltaFile": "s",
         "RecordBubbleSizes": "i"}


def _atof(s: str) -> float:
    import re
    m = re.match(r"\s*[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?)", s)
    return float(np.float32(float(m.group(0)))) if m else 0.0


def _atoi(s: str) -> int:
    import re
    m = re.match(r"\s*[+-]?\d+", s)
    return int(m.group(0)) if m else 0


def read_parameter_file(path: str, echo: bool = True) -> tuple[Parameters, list[str]]:
    """io_d2z.C:16-162.  Unknown or repeated tags are reported and skipped;
    the values used are echoed to `<path>-usedvalues`.  Raises OSError when the
    file cannot be opened (the reference only prints, io_d2z.C:150-153)."""
    p = Parameters()
    seen: set[str] = set()
    errors: list[str] = []
    lines_out = []
    with open(path) as fh:
        for line in fh:
            tok = line.split()
            if len(tok) < 2 or tok[0][0] in "%#":
                continue
            key, val = tok[0], tok[1]
            if key not in _TAGS or key in seen:
                errors.append(f"Error in {path}: Tag '{key}' not allowed or multiple defined.")
                continue
            seen.add(key)
            t = _TAGS[key]
            if t == "f":
                setattr(p, key, _atof(val))
                lines_out.append(f"{key:<35s}{getattr(p, key):f}\n")
            elif t == "i":
                setattr(p, key, _atoi(val))
                lines_out.append(f"{key:<35s}{getattr(p, key):d}\n")
            else:
                setattr(p, key, val)
                lines_out.append(f"{key:<35s}{val}\n")
    if echo:
        with open(path + "-usedvalues", "w") as fo:
            fo.writelines(lines_out)
    return p, errors


def growth(z: float, omegam: float, omegal: float, w: float) -> float:
    """Growth factor D(z), cosmology.C:174-212."""
    return float(load().prc_growth(z, omegam, omegal, w))


def inverse_erfc(x: float) -> float:
    """erfc^-1 as math.C:23-61 returns it (low end of a 1e-4 bracket)."""
    out = ctypes.c_float()
    check(load().prc_inverse_erfc(x, ctypes.byref(out)))
    return float(out.value)


def tau(history_z: np.ndarray, history: np.ndarray, omegam: float, omegab: float, h: float) -> float:
    """Thomson optical depth of an ionisation history, cosmology.C:52-83."""
    za = np.ascontiguousarray(history_z, np.float32)
    xa = np.ascontiguousarray(history, np.float32)
    return float(load().prc_tau(za.ctypes.data, xa.ctypes.data, len(za), omegam, omegab, h))


class Float2FloatTable:
    """Float2FloatTable (tables.C:9-38): f32 min, f32 max, i32 n, f32 table[n],
    linear interpolation with spacing (max - min)/n."""

    def __init__(self, path: str):
        self._t = _lib.prc_f2f_table()
        check(load().prc_f2f_load(path.encode(), ctypes.byref(self._t)))

    def Float2Float(self, x: float) -> float:
        return float(load().prc_f2f_eval(ctypes.byref(self._t), x))

    def __del__(self):
        try:
            load().prc_f2f_free(ctypes.byref(self._t))
        except Exception:
            pass


def fcoll(z: float, zInit: float, omegam: float, omegal: float, w: float, sigma_min: float) -> float:
    """Press-Schechter collapsed fraction (cosmology.C:311-324)."""
    return float(load().prc_fcoll(z, zInit, omegam, omegal, w, sigma_min))


def chistory(table: Float2FloatTable, mfp, rmfp: float, zeta: float) -> np.ndarray:
    """GetCHistory (bubblehistory_d2z.C:45-80): the MFP-corrected history."""
    m = np.ascontiguousarray(mfp, np.float32)
    out = np.zeros(_lib.PRC_NCHISTORY, np.float32)
    check(load().prc_chistory(ctypes.byref(table._t), m.ctypes.data, len(m), rmfp, zeta, out.ctypes.data))
    return out


def zvz_map(history, chist) -> np.ndarray:
    """CorrectHistory's z -> corrected z table (bubblehistory_d2z.C:314-326)."""
    h = np.ascontiguousarray(history, np.float32)
    c = np.ascontiguousarray(chist, np.float32)
    out = np.zeros(PRC_NHISTORY, np.float32)
    check(load().prc_zvz(h.ctypes.data, c.ctypes.data, out.ctypes.data))
    return out


def compute_tables(p: Parameters, cl: CLParameters) -> Tables:
    """Host tables of the step (FP32/FP64 as the reference keeps them)."""
    L = load()
    pp = _lib.prc_params(p.Omegam, p.Omegab, p.Omegal, p.h, p.ns, p.sigma8, p.w, p.BoxSize, p.zInit,
                         p.Rmin, p.N, p.Nscales, cl.Rmax, cl.zeta, cl.M_min)
    R = np.zeros(p.Nscales, np.float64)
    S = np.zeros(p.Nscales, np.float32)
    B = np.zeros(p.Nscales, np.float64)
    t = _lib.prc_tables()
    t.radii_mpc = R.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    t.sigma_r = S.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    t.barrier_b = B.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    check(L.prc_compute_tables(ctypes.byref(pp), ctypes.byref(t)))
    return Tables(t.DInit, t.zHigh, t.DHigh, t.pnorm, t.erfizeta, t.sigma_min, t.barrier_a, R, S, B)


def win_variants(N: int) -> int:
    """Window-pass variants compiled for grid side N (prc_d2z_win_variants)."""
    return int(load().prc_d2z_win_variants(int(N)))


def supported_sizes() -> list[int]:
    L = load()
    return [n for n in range(2, 2049) if L.prc_d2z_supported(n)]


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _dev_ptr(x, dtype_name: str, n: int):
    if not x.is_cuda:
        raise ValueError("torch tensors passed to prc_d2z must live on a CUDA device")
    if not x.is_contiguous():
        raise ValueError("tensor must be contiguous")
    if str(x.dtype) != f"torch.{dtype_name}" or x.numel() != n:
        raise ValueError(f"expected {n} elements of {dtype_name}, got {x.numel()} of {x.dtype}")
    return ctypes.c_void_p(x.data_ptr())


def _host_ptr(x, dtype, n: int):
    if not isinstance(x, np.ndarray) or x.dtype != dtype or x.size != n or not x.flags.c_contiguous:
        raise ValueError(f"expected a contiguous numpy array of {n} {np.dtype(dtype).name}")
    return ctypes.c_void_p(x.ctypes.data)


class Delta2Zreion:
    """One box on the GPU (prc_d2z_create .. prc_d2z_destroy)."""

    def __init__(self, N: int, box_mpc: float, radii_mpc, barrier_b, barrier_a: float, growth_init: float = 1.0,
                 radius_batch: int = 0, argmax: bool = True, sigma_grid: bool = False, stream=None,
                 faithful_window: bool = False):
        L = load()
        self.N = int(N)
        self.n3 = self.N ** 3
        self.radii = np.ascontiguousarray(radii_mpc, np.float64)
        self.barrier_b = np.ascontiguousarray(barrier_b, np.float64)
        self.n_radii = len(self.radii)
        self.barrier_a = float(barrier_a)
        self.growth_init = float(growth_init)
        d = _lib.prc_d2z_desc()
        d.N = self.N
        d.n_radii = self.n_radii
        d.box_mpc = float(box_mpc)
        d.radii_mpc = self.radii.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.barrier_b = self.barrier_b.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.barrier_a = self.barrier_a
        d.growth_init = self.growth_init
        d.radius_batch = int(radius_batch)
        d.flags = ((PRC_FLAG_ARGMAX if argmax else 0) | (PRC_FLAG_SIGMA_GRID if sigma_grid else 0)
                   | (_lib.PRC_FLAG_FAITHFUL_WINDOW if faithful_window else 0))
        d.stream = ctypes.c_void_p(int(stream)) if stream is not None else None
        self._ctx = ctypes.c_void_p()
        check(L.prc_d2z_create(ctypes.byref(d), ctypes.byref(self._ctx)))

    @classmethod
    def from_parameters(cls, p: Parameters, cl: CLParameters, **kw) -> "Delta2Zreion":
        t = compute_tables(p, cl)
        obj = cls(p.N, float(np.float32(p.BoxSize) / np.float32(p.h)), t.radii_mpc, t.barrier_b, t.barrier_a,
                  t.DInit, **kw)
        obj.tables = t
        return obj

    def close(self):
        if getattr(self, "_ctx", None) and self._ctx.value:
            load().prc_d2z_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- forward
    def forward(self, delta_lin, zreion=None, argmax=None, want_argmax: bool = True,
                want_sigma_grid: bool = False):
        """delta_lin (N^3 float32, file order) -> (zreion, argmax | None, sigma_grid | None).

        numpy in -> numpy out (host copies inside the call); CUDA tensor in ->
        CUDA tensors out (no copies)."""
        L = load()
        n3 = self.n3
        sig = np.zeros(self.n_radii, np.float64) if want_sigma_grid else None
        sig_p = ctypes.c_void_p(sig.ctypes.data) if sig is not None else None
        if _is_torch(delta_lin):
            import torch
            dp = _dev_ptr(delta_lin.reshape(-1), "float32", n3)
            if zreion is None:
                zreion = torch.empty(delta_lin.shape, dtype=torch.float32, device=delta_lin.device)
            if want_argmax and argmax is None:
                argmax = torch.empty(delta_lin.shape, dtype=torch.uint8, device=delta_lin.device)
            zp = _dev_ptr(zreion.reshape(-1), "float32", n3)
            ap = _dev_ptr(argmax.reshape(-1), "uint8", n3) if argmax is not None else None
            check(L.prc_d2z_forward(self._ctx, dp, 1, zp, ap, 1, sig_p))
        else:
            d = np.ascontiguousarray(delta_lin, np.float32)
            dp = _host_ptr(d, np.float32, n3)
            if zreion is None:
                zreion = np.empty(d.shape, np.float32)
            if want_argmax and argmax is None:
                argmax = np.empty(d.shape, np.uint8)
            zp = _host_ptr(zreion, np.float32, n3)
            ap = _host_ptr(argmax, np.uint8, n3) if argmax is not None else None
            check(L.prc_d2z_forward(self._ctx, dp, 0, zp, ap, 0, sig_p))
        return zreion, argmax, sig

    def forward_many(self, deltas, zreions, argmaxes=None):
        """prc_d2z_forward_many: boxes deltas[i] -> zreions[i] (argmaxes[i]), all
        contiguous host numpy arrays of N^3 (pinned ones overlap the copies with
        the kernels of the neighbouring boxes).  Returns zreions."""
        n = len(deltas)
        if len(zreions) != n or (argmaxes is not None and len(argmaxes) != n):
            raise ValueError("deltas, zreions (and argmaxes) must have the same length")
        dp = (ctypes.c_void_p * n)(*[_host_ptr(d, np.float32, self.n3).value for d in deltas])
        zp = (ctypes.c_void_p * n)(*[_host_ptr(z, np.float32, self.n3).value for z in zreions])
        ap = None
        if argmaxes is not None:
            ap = (ctypes.c_void_p * n)(*[_host_ptr(a, np.uint8, self.n3).value for a in argmaxes])
        check(load().prc_d2z_forward_many(self._ctx, n, dp, zp, ap))
        return zreions

    def smooth(self, delta_lin, radius: int):
        """delta_R of one radius (diagnostic; host or device like forward)."""
        L = load()
        if _is_torch(delta_lin):
            import torch
            out = torch.empty(delta_lin.shape, dtype=torch.float32, device=delta_lin.device)
            check(L.prc_d2z_smooth(self._ctx, _dev_ptr(delta_lin.reshape(-1), "float32", self.n3), 1, int(radius),
                                   _dev_ptr(out.reshape(-1), "float32", self.n3), 1))
            return out
        d = np.ascontiguousarray(delta_lin, np.float32)
        out = np.empty(d.shape, np.float32)
        check(L.prc_d2z_smooth(self._ctx, _host_ptr(d, np.float32, self.n3), 0, int(radius),
                               _host_ptr(out, np.float32, self.n3), 0))
        return out

    def gaussian_field(self, seed: int, amp, out=None):
        """A Gaussian random field on this context's grid (prc_d2z_gaussian_field):
        amp is the |m|^2-indexed amplitude table (fields.amplitude_table).  out:
        a CUDA float32 tensor (N^3) or None for a host array."""
        a = np.ascontiguousarray(amp, np.float32)
        L = load()
        if out is not None and _is_torch(out):
            check(L.prc_d2z_gaussian_field(self._ctx, int(seed) & 0xFFFFFFFF, a.ctypes.data, len(a),
                                           _dev_ptr(out.reshape(-1), "float32", self.n3), 1))
            return out
        res = np.empty((self.N,) * 3, np.float32) if out is None else out
        check(L.prc_d2z_gaussian_field(self._ctx, int(seed) & 0xFFFFFFFF, a.ctypes.data, len(a),
                                       _host_ptr(res, np.float32, self.n3), 0))
        return res

    def tune(self, radius_batch: int = 0, win_variant: int = 0) -> None:
        """Radius batch (0 = keep) and window-pass variant (prc_d2z_tune)."""
        check(load().prc_d2z_tune(self._ctx, int(radius_batch), int(win_variant)))
        self.radius_batch, self.win_variant = int(radius_batch), int(win_variant)

    def set_barrier(self, barrier_b, barrier_a: float) -> None:
        """New barrier table for the same radii (prc_d2z_set_barrier)."""
        b = np.ascontiguousarray(barrier_b, np.float64)
        check(load().prc_d2z_set_barrier(self._ctx, b.ctypes.data, float(barrier_a)))
        self.barrier_b, self.barrier_a = b, float(barrier_a)

    def last_timing(self):
        ms = (ctypes.c_float * 3)()
        check(load().prc_d2z_last_timing(self._ctx, ms))
        return tuple(ms)

    def profile(self, enable: bool = True) -> None:
        """Per-kernel CUDA-event timing on/off (resets the totals)."""
        check(load().prc_d2z_profile(self._ctx, 1 if enable else 0))

    def profile_read(self) -> dict:
        """{kind: (total ms, launches)} since the last profile() call."""
        ms = (ctypes.c_double * _lib.PRC_NKINDS)()
        n = (ctypes.c_longlong * _lib.PRC_NKINDS)()
        check(load().prc_d2z_profile_read(self._ctx, ms, n))
        return {k: (ms[i], n[i]) for i, k in enumerate(_lib.KINDS)}

    def last_launches(self) -> int:
        n = ctypes.c_int()
        check(load().prc_d2z_last_launches(self._ctx, ctypes.byref(n)))
        return n.value

    # ---------------------------------------------------------------- history
    def history(self, zreion):
        """GetHistory: (counts, history, history_z), each PRC_NHISTORY long."""
        L = load()
        counts = np.zeros(PRC_NHISTORY, np.uint32)
        hist = np.zeros(PRC_NHISTORY, np.float32)
        hz = np.zeros(PRC_NHISTORY, np.float32)
        if _is_torch(zreion):
            zp, on_dev = _dev_ptr(zreion.reshape(-1), "float32", self.n3), 1
        else:
            z = np.ascontiguousarray(zreion, np.float32)
            zp, on_dev = _host_ptr(z, np.float32, self.n3), 0
        check(L.prc_d2z_history(self._ctx, zp, on_dev, ctypes.c_void_p(counts.ctypes.data),
                                ctypes.c_void_p(hist.ctypes.data), ctypes.c_void_p(hz.ctypes.data)))
        return counts, hist, hz

    # ---------------------------------------------------------------- correction chain
    def bubble_mfp(self, zreion, history, box_mpc: float, n_x: int = _lib.PRC_NX_MFP,
                   n_skewers: int = _lib.PRC_NSKEWERS):
        """GetBubbleMFP (bubblehistory_d2z.C:82-252): (mfp, mfp_x, dfdmfp)."""
        z = np.ascontiguousarray(zreion, np.float32)
        h = np.ascontiguousarray(history, np.float32)
        s = _lib.prc_mfp_setup(self.N, box_mpc, n_x, n_skewers)
        mfp = np.zeros(n_x, np.float32)
        mfp_x = np.zeros(n_x, np.float32)
        dfd = np.zeros(_lib.PRC_NMFP * n_x, np.float32)
        check(load().prc_d2z_bubble_mfp(self._ctx, ctypes.byref(s), _host_ptr(z, np.float32, self.n3),
                                        h.ctypes.data, mfp.ctypes.data, mfp_x.ctypes.data, dfd.ctypes.data))
        return mfp, mfp_x, dfd

    def correct(self, zreion, zvz):
        """CorrectHistory's per-cell map, in place (host array or CUDA tensor)."""
        zv = np.ascontiguousarray(zvz, np.float32)
        if _is_torch(zreion):
            check(load().prc_d2z_correct(self._ctx, zv.ctypes.data, _dev_ptr(zreion.reshape(-1), "float32", self.n3), 1))
        else:
            check(load().prc_d2z_correct(self._ctx, zv.ctypes.data, _host_ptr(zreion, np.float32, self.n3), 0))
        return zreion

    def correct_history(self, zreion, fcoll_table: str, box_mpc: float, rmfp: float, zeta: float,
                        n_x: int = _lib.PRC_NX_MFP, n_skewers: int = _lib.PRC_NSKEWERS):
        """main_d2z.C:76-87 on a host zreion grid, in place: GetHistory,
        GetBubbleMFP, GetCHistory, CorrectHistory.  Returns (mfp, chistory)."""
        _, hist, _ = self.history(zreion)
        mfp, _, _ = self.bubble_mfp(zreion, hist, box_mpc, n_x, n_skewers)
        ch = chistory(Float2FloatTable(fcoll_table), mfp, rmfp, zeta)
        self.correct(zreion, zvz_map(hist, ch))
        return mfp, ch

    # ---------------------------------------------------------------- adjoint
    def backward(self, dL_dz, argmax, dL_ddelta=None, want_dB: bool = True):
        """(dL/dz, argmax) -> (dL/d delta_lin, dL/dB_r | None)."""
        L = load()
        dB = np.zeros(self.n_radii, np.float64) if want_dB else None
        dBp = ctypes.c_void_p(dB.ctypes.data) if dB is not None else None
        if _is_torch(dL_dz):
            import torch
            gp = _dev_ptr(dL_dz.reshape(-1), "float32", self.n3)
            ap = _dev_ptr(argmax.reshape(-1), "uint8", self.n3)
            if dL_ddelta is None:
                dL_ddelta = torch.empty(dL_dz.shape, dtype=torch.float32, device=dL_dz.device)
            op = _dev_ptr(dL_ddelta.reshape(-1), "float32", self.n3)
            check(L.prc_d2z_backward(self._ctx, gp, ap, 1, op, 1, dBp))
        else:
            g = np.ascontiguousarray(dL_dz, np.float32)
            a = np.ascontiguousarray(argmax, np.uint8)
            if dL_ddelta is None:
                dL_ddelta = np.empty(g.shape, np.float32)
            check(L.prc_d2z_backward(self._ctx, _host_ptr(g, np.float32, self.n3),
                                     _host_ptr(a, np.uint8, self.n3), 0,
                                     _host_ptr(dL_ddelta, np.float32, self.n3), 0, dBp))
        return dL_ddelta, dB


class Batch:
    """Many boxes (any mix of supported grid sizes) run together: one
    workspace per box, n_streams CUDA streams (prc_d2z_batch_*).  forward's
    mode: "loop" (each box's launches), "graph" (those launches captured into
    one CUDA graph) or "grouped" (one launch per pass over all boxes of a grid
    size, the groups side by side, captured into one CUDA graph).

    boxes: list of dicts with the Delta2Zreion arguments (N, box_mpc,
    radii_mpc, barrier_b, barrier_a, growth_init, radius_batch,
    faithful_window)."""

    def __init__(self, boxes, n_streams: int = 4):
        L = load()
        self.n = len(boxes)
        self.N = [int(b["N"]) for b in boxes]
        self._keep = []
        descs = (_lib.prc_d2z_desc * self.n)()
        for i, b in enumerate(boxes):
            R = np.ascontiguousarray(b["radii_mpc"], np.float64)
            B = np.ascontiguousarray(b["barrier_b"], np.float64)
            self._keep += [R, B]
            d = descs[i]
            d.N = int(b["N"])
            d.n_radii = len(R)
            d.box_mpc = float(b["box_mpc"])
            d.radii_mpc = R.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            d.barrier_b = B.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            d.barrier_a = float(b["barrier_a"])
            d.growth_init = float(b.get("growth_init", 1.0))
            d.radius_batch = int(b.get("radius_batch", 0))
            d.flags = _lib.PRC_FLAG_FAITHFUL_WINDOW if b.get("faithful_window") else 0
        self._b = ctypes.c_void_p()
        check(L.prc_d2z_batch_create(self.n, descs, int(n_streams), ctypes.byref(self._b)))

    MODES = {"loop": _lib.PRC_BATCH_LOOP, "graph": _lib.PRC_BATCH_GRAPH, "grouped": _lib.PRC_BATCH_GROUPED}

    def forward(self, deltas, zreions, argmaxes=None, use_graph: bool = True, mode: str | None = None):
        """deltas/zreions (/argmaxes): lists of contiguous CUDA tensors.  mode:
        "loop", "graph" or "grouped" (default: "graph" if use_graph else "loop")."""
        m = self.MODES[mode] if mode is not None else (_lib.PRC_BATCH_GRAPH if use_graph else _lib.PRC_BATCH_LOOP)
        L = load()
        n = self.n
        dp = (ctypes.c_void_p * n)(*[_dev_ptr(d.reshape(-1), "float32", self.N[i] ** 3).value
                                    for i, d in enumerate(deltas)])
        zp = (ctypes.c_void_p * n)(*[_dev_ptr(z.reshape(-1), "float32", self.N[i] ** 3).value
                                    for i, z in enumerate(zreions)])
        ap = None
        if argmaxes is not None:
            ap = (ctypes.c_void_p * n)(*[_dev_ptr(a.reshape(-1), "uint8", self.N[i] ** 3).value
                                        for i, a in enumerate(argmaxes)])
        check(L.prc_d2z_batch_forward(self._b, dp, zp, ap, m))
        return zreions

    def launches(self) -> int:
        n = ctypes.c_int()
        check(load().prc_d2z_batch_launches(self._b, ctypes.byref(n)))
        return n.value

    def tune(self, box: int, radius_batch: int = 0, win_variant: int = 0) -> None:
        """Radius batch and window-pass variant of one box (prc_d2z_batch_tune)."""
        check(load().prc_d2z_batch_tune(self._b, int(box), int(radius_batch), int(win_variant)))

    def close(self):
        if getattr(self, "_b", None) and self._b.value:
            load().prc_d2z_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def delta2zreion(delta_lin, p: Parameters, cl: CLParameters, **kw):
    """delta_lin -> (zreion, argmax, sigma_grid, tables): main_d2z.C:57-71 in one call."""
    with Delta2Zreion.from_parameters(p, cl, sigma_grid=True, **kw) as ctx:
        z, a, s = ctx.forward(delta_lin, want_sigma_grid=True)
        return z, a, s, ctx.tables
