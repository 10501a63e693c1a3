"""TEST INFRASTRUCTURE -- the CPU oracle of the delta2zreion step.

A restatement of pr-calc's ``delta2zreion`` chain (c++/src) in numpy/scipy,
used only by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline / reference arm, and only to check results against it.  The product
never imports it.

Parity is unpinned: the reference needs MPI, FFTW 3.3.3 and GSL (not installed
where this code is built and run) and ships no golden vectors or tests for this path, so
these functions follow its source, each citing the lines it restates:

  read_parameter_file   io_d2z.C:16-162
  growth                cosmology.C:174-212
  transeh / sgm2k       cosmology.C:290-309 / :274-288
  normalize / cdmehint  cosmology.C:246-272 / :214-244 (GSL QAGS -> scipy quad)
  inverse_erfc          math.C:23-61 (GSL Brent -> exact erfcinv, see below)
  radii / tables        delta2zreion_d2z.C:14-38,55,97-100; main_d2z.C:57-64
  forward_spectrum      main_d2z.C:57-59,67 (FFTW r2c -> scipy.fft.rfftn)
  window                delta2zreion_d2z.C:41-43,58-89
  smooth                delta2zreion_d2z.C:92-93 (FFTW c2r + NormalizeArray)
  barrier / d2z         delta2zreion_d2z.C:105-146,206-216
  sigma_grid            arrayoperations.C:4-35
  history               bubblehistory_d2z.C:5-43
  tau                   cosmology.C:52-83

Two precisions:
  mode="fp32"  the reference's own arithmetic: float32 transforms (scipy's
               pocketfft in single precision stands in for FFTW float), the
               float window of delta2zreion_d2z.C:77 and the double barrier
               bracket (loops in the C helper d2z_cells.c);
  mode="fp64"  the same chain in float64 with the exact window, the FP64
               oracle used to report the error of both.
The third-party pieces (FFTW, GSL QAGS, GSL Brent) are replaced by their
mathematical definitions: the DFT, an adaptive quadrature (QUADPACK via
scipy.integrate.quad) and the exact inverse (scipy.special.erfcinv, refined);
GSL's Brent returns the low end of a 1e-4-relative bracket, so the
reference's erfizeta lies within 1e-4 relative below the exact value.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NHISTORY = 100000
HISTORY_INITIAL = 49.9
HISTORY_FINAL = 0.01

f32 = np.float32
f64 = np.float64


# ---------------------------------------------------------------- C helper
_lib = None


def lib():
    """The compiled per-cell helper (oracle/_build/liborc_cells.so)."""
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "_build", "liborc_cells.so")
        if not os.path.exists(path):
            import importlib.util
            spec = importlib.util.spec_from_file_location("_orc_build", os.path.join(HERE, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        L.orc_window_faithful.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float, P(ctypes.c_float)]
        L.orc_apply_window_c64.argtypes = [ctypes.c_long, P(ctypes.c_float), P(ctypes.c_float)]
        L.orc_barrier_update.argtypes = [ctypes.c_long, P(ctypes.c_float), ctypes.c_float, ctypes.c_double,
                                         ctypes.c_int, P(ctypes.c_float), P(ctypes.c_uint8), P(ctypes.c_double)]
        L.orc_hist.argtypes = [ctypes.c_long, P(ctypes.c_float), ctypes.c_float, ctypes.c_int,
                               P(ctypes.c_uint32)]
        L.orc_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a, t=ctypes.c_float):
    return a.ctypes.data_as(ctypes.POINTER(t))


# ---------------------------------------------------------------- parameters
@dataclass
class Parameters:
    """Parameter (allvars_d2z.h:58-64) and clParameter (:66-70) in one."""
    Omegam: float = 0.31
    Omegab: float = 0.049
    Omegal: float = 0.69
    h: float = 0.68
    ns: float = 0.965
    sigma8: float = 0.81
    w: float = -1.0
    BoxSize: float = 200.0          # Mpc/h as read
    zInit: float = 0.0
    Rmin: float = 2.0               # cells
    N: int = 128
    Nscales: int = 32
    DeltaFile: str = ""
    RecordBubbleSizes: int = 0
    Rmax: float = 60.0              # Mpc/h (-r)
    zeta: float = 10.0              # (-z)
    M_min: float = 1e8              # Msun (-m)


_TAGS = [("Omegam", "f"), ("Omegab", "f"), ("Omegal", "f"), ("h", "f"), ("ns", "f"), ("sigma8", "f"),
         ("w", "f"), ("BoxSize", "f"), ("zInit", "f"), ("Rmin", "f"), ("N", "i"), ("Nscales", "i"),
         ("DeltaFile", "s"), ("RecordBubbleSizes", "i")]


def _atof(s: str) -> float:
    import re
    m = re.match(r"\s*[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?)", s)
    return float(m.group(0)) if m else 0.0


def _atoi(s: str) -> int:
    import re
    m = re.match(r"\s*[+-]?\d+", s)
    return int(m.group(0)) if m else 0


def read_parameter_file(path: str, p: Parameters | None = None) -> tuple[Parameters, list[str]]:
    """io_d2z.C:89-149: first two tokens per line, '%'/'#' comments, each tag
    once; floats through atof into float.  Returns (params, error lines)."""
    p = p or Parameters()
    p.RecordBubbleSizes = 0
    seen, errors = set(), []
    types = dict(_TAGS)
    with open(path) as fh:
        for line in fh:
            tok = line.split()
            if len(tok) < 2 or tok[0][0] in "%#":
                continue
            key, val = tok[0], tok[1]
            if key not in types or key in seen:
                errors.append(f"Error in {path}: Tag '{key}' not allowed or multiple defined.")
                continue
            seen.add(key)
            t = types[key]
            if t == "f":
                setattr(p, key, float(f32(_atof(val))))
            elif t == "i":
                setattr(p, key, _atoi(val))
            else:
                setattr(p, key, val)
    return p, errors


# ---------------------------------------------------------------- cosmology
def growth(z, omegam, omegal, w):
    """cosmology.C:174-212 with its float/double conversions."""
    z, om, ol, w = f32(z), f32(omegam), f32(omegal), f32(w)
    x = f32(1) + z
    x2 = f32(x * x)
    x3 = f32(x * x * x)
    x3w = f32(np.power(x3, w, dtype=f32))
    omega = f32(om * x3 / (om * x3 + (f32(1) - om - ol) * x2 + ol))
    lam = f32(ol * x3 * x3w / (om * x3 + (f32(1) - om - ol) * x2 + ol * x3 * x3w))

    def gfun(o, l):
        return f32(2.5 * f64(o) / (math.pow(f64(o), 4. / 7.) - f64(l)
                                   + f64(f32((f32(1) + o / f32(2)) * (f32(1) + l / f32(70))))))

    g, g0 = gfun(omega, lam), gfun(om, ol)
    wd = f64(w)
    a1, a2 = (0.255 + 0.305 * wd + 0.0027 / wd), (0.366 + 0.266 * wd - 0.0700 / wd)
    t = f32(-a1 * f64(f32(1) - omega) - a2 * f64(np.log(omega, dtype=f32)))
    t0 = f32(-a1 * f64(f32(1) - om) - a2 * f64(np.log(om, dtype=f32)))
    g = f32(g * np.power(-w, t, dtype=f32))
    g0 = f32(g0 * np.power(-w, t0, dtype=f32))
    return f32(f32(g / x) / g0)


def transeh(k, om, ob, hh):
    """Eisenstein-Hu no-wiggle transfer function, cosmology.C:290-309."""
    alpha = (1 - 0.328 * math.log(431 * om * hh * hh) * (ob / om)
             + 0.38 * math.log(22.3 * om * hh * hh) * (ob / om) ** 2)
    sound = 44.5 * math.log(9.83 / (om * hh * hh)) / math.sqrt(1 + 10 * (ob * hh * hh) ** 0.75)
    shape = om * hh * (alpha + (1 - alpha) / (1 + (0.43 * k * sound) ** 4))
    q = (k / hh) * (2.728 / 2.7) ** 2 / shape
    L = math.log(2 * math.e + 1.8 * q)
    return L / (L + (14.2 + 731 / (1 + 62.5 * q)) * q * q)


def sigma2_of_R(R, om, ob, hh, ns, pnorm):
    """Integral of sgm2k (cosmology.C:274-288) over ln k in [ln(1e-5/R), ln(1e5/R)]."""
    from scipy.integrate import quad

    def f(lk):
        k = math.exp(lk)
        kR = k * R
        W = 3 * (math.sin(kR) - kR * math.cos(kR)) / kR ** 3
        T = transeh(k, om, ob, hh)
        return k ** (3 + ns) * T * T * W * W * pnorm ** 2

    a, b = math.log(1e-5 / R), math.log(1e5 / R)
    # split at the first few oscillations of W so the adaptive rule converges
    pts = sorted({math.log(x / R) for x in (0.1, 1.0, 4.49, 10.0, 100.0) if a < math.log(x / R) < b})
    edges = [a] + pts + [b]
    tot = 0.0
    for lo, hi in zip(edges[:-1], edges[1:]):
        v, _ = quad(f, lo, hi, epsabs=0, epsrel=1e-9, limit=5000)
        tot += v
    return tot


def normalize(p: Parameters):
    """cosmology.C:246-272: pnorm = sigma8 / sigma_unnorm(8/h Mpc), float."""
    om, ob, hh, ns = (f64(f32(v)) for v in (p.Omegam, p.Omegab, p.h, p.ns))
    R = f64(f32(8) / f32(p.h))
    s2 = sigma2_of_R(R, om, ob, hh, ns, 1.0)
    return f32(f64(f32(p.sigma8)) / math.sqrt(s2))


def cdmehint(p: Parameters, pnorm, mass):
    """cosmology.C:214-244: sigma^2 of a top-hat of mass `mass` [Msun], float."""
    om, ob, hh, ns = (f64(f32(v)) for v in (p.Omegam, p.Omegab, p.h, p.ns))
    rhoc = f32(2.775e11)
    pi = f32(3.141592654)
    fourpi = f32(4 * pi)
    dens = f64(f32(f32(f32(f32(p.Omegam) * rhoc) * f32(p.h)) * f32(p.h)))
    num = f32(f32(3 * f32(mass)) / fourpi)
    R = (f64(num) / dens) ** (1. / 3.)
    return f32(sigma2_of_R(R, om, ob, hh, ns, f64(f32(pnorm))))


def inverse_erfc(x):
    """math.C:23-61 returns the low end of a Brent bracket of relative width
    1e-4 around erfc^{-1}(x); the oracle returns the exact root (float)."""
    from scipy.special import erfcinv
    return f32(erfcinv(f64(f32(x))))


@dataclass
class Tables:
    DInit: float
    zHigh: float
    DHigh: float
    pnorm: float
    erfizeta: float
    sigma_min: float
    A: float
    R: np.ndarray = field(repr=False)        # Mpc (float32 values)
    sigma_r: np.ndarray = field(repr=False)
    B: np.ndarray = field(repr=False)        # float64


def radii(p: Parameters):
    """delta2zreion_d2z.C:32-38,55 (float arithmetic, pow in double)."""
    box = f32(f32(p.BoxSize) / f32(p.h))
    Ri = f32(f32(box * f32(p.Rmin)) / f32(p.N))
    Rf = f32(f32(p.Rmax) / f32(p.h))
    dS = f32(f32(np.log10(Rf, dtype=f32) - np.log10(Ri, dtype=f32)) / f32(p.Nscales - 1))
    lRi = np.log10(Ri, dtype=f32)
    return np.array([f32(10.0 ** f64(f32(lRi + f32(f32(r) * dS)))) for r in range(p.Nscales)], dtype=f32)


def tables(p: Parameters, erfizeta: float | None = None) -> Tables:
    """Host tables of the step; `erfizeta` overrides the exact inverse."""
    DInit = growth(p.zInit, p.Omegam, p.Omegal, p.w)
    zHigh = f32(20.0)
    DHigh = growth(zHigh, p.Omegam, p.Omegal, p.w)
    pnorm = normalize(p)
    ez = f32(erfizeta) if erfizeta is not None else inverse_erfc(f32(1.0 / f64(f32(p.zeta))))
    smin = np.sqrt(cdmehint(p, pnorm, p.M_min), dtype=f32)
    R = radii(p)
    rho0 = f32(2.775e11 * f64(f32(p.Omegam)) * f64(f32(p.h)) * f64(f32(p.h)))
    sig = np.zeros(p.Nscales, f32)
    B = np.zeros(p.Nscales, f64)
    for r, Rr in enumerate(R):
        mass = f32(4 * math.pi / 3 * f64(rho0) * f64(Rr) * f64(Rr) * f64(Rr))
        sig[r] = np.sqrt(cdmehint(p, pnorm, mass), dtype=f32)
        dvar = f32(f32(smin * smin) - f32(sig[r] * sig[r]))
        with np.errstate(invalid="ignore"):
            B[r] = math.sqrt(2. * f64(dvar)) * f64(ez) if dvar >= 0 else float("nan")
    A = f32(f32(f32(f32(1) + zHigh) * DHigh) / f32(1.686))
    return Tables(DInit, zHigh, DHigh, pnorm, ez, smin, A, R, sig, B)


# ---------------------------------------------------------------- the grid chain
def forward_spectrum(delta: np.ndarray, dinit: float, mode: str = "fp32"):
    """main_d2z.C:57-59,67: delta /= DInit, then the unnormalised R2C."""
    import scipy.fft as sfft
    workers = os.cpu_count()
    if mode == "fp32":
        d = (delta.astype(f32) / f32(dinit)).astype(f32)
        return sfft.rfftn(d, workers=workers).astype(np.complex64)
    d = delta.astype(f64) / f64(dinit)
    return sfft.rfftn(d, workers=workers)


def window(N: int, box_mpc: float, R: float, mode: str = "fp32"):
    """|k| R top-hat window on the half spectrum (delta2zreion_d2z.C:58-89)."""
    if mode == "fp32":
        dk = f32(2. * math.pi / f64(f32(box_mpc)))
        W = np.empty((N, N, N // 2 + 1), f32)
        lib().orc_window_faithful(N, dk, f32(R), _p(W))
        return W
    f = np.fft.fftfreq(N, 1.0 / N)
    fz = np.arange(N // 2 + 1, dtype=f64)
    m2 = f[:, None, None] ** 2 + f[None, :, None] ** 2 + fz[None, None, :] ** 2
    x = np.sqrt(m2) * (2 * math.pi / box_mpc) * f64(R)
    with np.errstate(divide="ignore", invalid="ignore"):
        W = 3 * (np.sin(x) - x * np.cos(x)) / x ** 3
        small = x < 1e-2
        x2 = x[small] ** 2
        W[small] = 1 - x2 / 10 + x2 * x2 / 280
    W[0, 0, 0] = 0.0
    return W


def smooth(spec, W, N: int, mode: str = "fp32"):
    """FFTW c2r of spec*W followed by /N^3 (delta2zreion_d2z.C:92-93)."""
    import scipy.fft as sfft
    workers = os.cpu_count()
    if mode == "fp32":
        s = np.ascontiguousarray(spec, dtype=np.complex64).copy()
        lib().orc_apply_window_c64(s.size, _p(s.view(f32)), _p(np.ascontiguousarray(W, dtype=f32)))
        # scipy's default "backward" normalisation is exactly the 1/N^3 of NormalizeArray
        return sfft.irfftn(s, s=(N, N, N), workers=workers).astype(f32)
    return sfft.irfftn(spec * W, s=(N, N, N), workers=workers)


def barrier_update(dR, A, B, r, zreion, argmax=None, mode="fp32"):
    """d2z + running max (delta2zreion_d2z.C:105-146,206-216); returns sum dR^2."""
    if mode == "fp32":
        s2 = ctypes.c_double(0)
        d = np.ascontiguousarray(dR, dtype=f32)
        lib().orc_barrier_update(d.size, _p(d), f32(A), f64(B), int(r), _p(zreion),
                                 _p(argmax, ctypes.c_uint8) if argmax is not None else None,
                                 ctypes.byref(s2))
        return s2.value
    z = f64(A) * (dR + f64(B)) - 1.0
    with np.errstate(invalid="ignore"):
        upd = z > zreion
    zreion[upd] = z[upd]
    if argmax is not None:
        argmax[upd] = r
    return float(np.sum(dR * dR))


def d2z(delta: np.ndarray, box_mpc: float, R, A, B, dinit: float = 1.0, mode: str = "fp32",
        radii_idx=None, want_argmax: bool = True):
    """The whole step: zreion (0-initialised), argmax (255 = never), sigma_grid.

    `radii_idx` restricts the loop to those radii (a bounded sample); the
    remaining outputs then cover only those radii."""
    N = delta.shape[0]
    spec = forward_spectrum(delta, dinit, mode)
    dt = f32 if mode == "fp32" else f64
    zreion = np.zeros(delta.shape, dt)
    argmax = np.full(delta.shape, 255, np.uint8) if want_argmax else None
    sig = np.zeros(len(R))
    for r in (range(len(R)) if radii_idx is None else radii_idx):
        W = window(N, box_mpc, R[r], mode)
        dR = smooth(spec, W, N, mode)
        s2 = barrier_update(dR, A, B[r], r, zreion, argmax, mode)
        sig[r] = math.sqrt(s2 / N ** 3)
    return zreion, argmax, sig


def z_stack(delta, box_mpc, R, A, B, dinit=1.0, mode="fp64"):
    """Per-radius z_R = A (delta_R + B_R) - 1 for every cell (small grids only),
    as float64 (mode fp64) or with the reference's float rounding (fp32);
    also returns max |delta_R| over all radii."""
    N = delta.shape[0]
    spec = forward_spectrum(delta, dinit, mode)
    zs = np.empty((len(R),) + delta.shape, f64)
    dmax = 0.0
    for r in range(len(R)):
        dR = smooth(spec, window(N, box_mpc, R[r], mode), N, mode)
        dmax = max(dmax, float(np.max(np.abs(dR))))
        z = f64(A) * (dR.astype(f64) + f64(B[r])) - 1.0
        zs[r] = z.astype(f32) if mode == "fp32" else z
    return zs, dmax


def margins(zs):
    """Best z, its radius, and the gap to the runner-up (including the
    initial 0 of zreion as a competitor), per cell."""
    with np.errstate(invalid="ignore"):
        zz = np.where(np.isnan(zs), -np.inf, zs)
    order = np.argsort(-zz, axis=0, kind="stable")
    best = np.take_along_axis(zz, order[:1], 0)[0]
    second = np.take_along_axis(zz, order[1:2], 0)[0] if len(zs) > 1 else np.full(best.shape, -np.inf)
    gap_r = best - second
    gap_0 = np.abs(best)          # against the initial zreion = 0
    return best, order[0], np.minimum(gap_r, gap_0)


def delta_R(delta, box_mpc, R, dinit=1.0, mode="fp64"):
    """The smoothed field of one radius (for the delta_R accuracy checks)."""
    N = delta.shape[0]
    spec = forward_spectrum(delta, dinit, mode)
    return smooth(spec, window(N, box_mpc, R, mode), N, mode)


def history(zreion: np.ndarray):
    """GetHistory (bubblehistory_d2z.C:5-43): counts, cumulative x_i, z grid."""
    dzf = f32((HISTORY_FINAL - HISTORY_INITIAL) / (NHISTORY - 1))
    z = np.ascontiguousarray(zreion, dtype=f32).ravel()
    q = (z.astype(f64) - HISTORY_INITIAL) / f64(dzf)
    b = np.trunc(q)
    ok = (b >= 0) & (b < NHISTORY)
    counts = np.bincount(b[ok].astype(np.int64), minlength=NHISTORY).astype(np.uint32)
    n3 = f64(zreion.shape[0]) ** 3
    hist = (counts.astype(f32).astype(f64) / n3).astype(f32)
    for i in range(1, NHISTORY):
        hist[i] = f32(hist[i] + hist[i - 1])
    # i*dz is an int x float product, rounded to float before the double sum
    hz = np.array([f32(HISTORY_INITIAL + f64(f32(i * dzf))) for i in range(NHISTORY)], f32)
    return counts, hist, hz


def tau(za, xa, omegam, omegab, h):
    """cosmology.C:52-83."""
    thompson, YHe = f32(6.65e-25), f32(0.25)
    hubble0 = f32(100. / 3.086e19 * f64(f32(h)))
    ne0 = f32(f64(f32(f32(omegab) * f32(h)) * f32(h)) * 1.88e-29 / 1.67e-24)
    c = f32(3e10)
    dtau0 = f32(f32(f32(thompson * ne0) * c) / hubble0)
    t = f32(0)
    for i in range(1, len(za) - 1):
        z, x = f32(za[i]), f32(xa[i])
        dz = f32(abs(f32(za[i + 1]) - f32(za[i])))
        NHe = f32(2) if z < 3 else f32(1)
        num = f64(f32(x * dtau0)) * f64(f32(1) + z) ** 2
        den = math.sqrt(f64(f32(omegam)) * f64(f32(1) + z) ** 3 + 1 - f64(f32(omegam)))
        t = f32(t + f32(num / den * f64(f32(f32(1) - YHe + f32(NHe * YHe) / f32(4))) * f64(dz)))
    return t


# ---------------------------------------------------------------- adjoint (FP64)
def adjoint(g: np.ndarray, argmax: np.ndarray, box_mpc: float, R, A: float, dinit: float = 1.0):
    """FP64 vector-Jacobian product of d2z (no reference counterpart):
    dL/d delta_lin = (1/(N^3 D)) IDFT(sum_R W_R DFT(A g [argmax == R])),
    dL/dB_R = A sum_{argmax == R} g."""
    import scipy.fft as sfft
    N = g.shape[0]
    acc = np.zeros((N, N, N // 2 + 1), np.complex128)
    dB = np.zeros(len(R))
    g64 = g.astype(f64)
    for r in range(len(R)):
        m = argmax == r
        if not m.any():
            continue
        h = np.where(m, f64(A) * g64, 0.0)
        dB[r] = f64(A) * float(g64[m].sum())
        acc += window(N, box_mpc, R[r], "fp64") * sfft.rfftn(h, workers=os.cpu_count())
    return sfft.irfftn(acc, s=(N, N, N), workers=os.cpu_count()) / f64(dinit), dB
