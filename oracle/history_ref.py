"""TEST INFRASTRUCTURE -- oracle of pr-calc's history-correction chain.

Restates, for the tests only (the product never imports it):
  f2f_load / f2f_eval   Float2FloatTable, tables.C:9-38
  deltac / fcoll        cosmology.C:141-172, 311-324 (float arithmetic)
  bubble_mfp            GetBubbleMFP, bubblehistory_d2z.C:82-252 (one rank)
  chistory              GetCHistory + BubbleMFP, bubblehistory_d2z.C:45-80, 254-276
  zvz / correct         CorrectHistory, bubblehistory_d2z.C:278-343
The skewer starts draw from glibc's generator in its unseeded state (the
state srand(1) gives), through libc's random_r, so the accepted cells are the
ones the reference's rand() would pick at one rank.  Pure Python loops: keep
the skewer counts small.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math

import numpy as np

f32, f64 = np.float32, np.float64
NHISTORY, NCHISTORY, NMFP = 100000, 10000, 200
H0, H1 = 49.9, 0.01
X0, X1 = 0.01, 0.999


class GlibcRand:
    """rand() of glibc from its initial state, via initstate_r/random_r."""

    class _RD(ctypes.Structure):
        _fields_ = [("fptr", ctypes.c_void_p), ("rptr", ctypes.c_void_p), ("state", ctypes.c_void_p),
                    ("rand_type", ctypes.c_int), ("rand_deg", ctypes.c_int), ("rand_sep", ctypes.c_int),
                    ("end_ptr", ctypes.c_void_p)]

    def __init__(self):
        libc = ctypes.CDLL(ctypes.util.find_library("c"))
        self._buf = ctypes.create_string_buffer(128)
        self._rd = self._RD()
        libc.initstate_r.argtypes = [ctypes.c_uint, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(self._RD)]
        libc.random_r.argtypes = [ctypes.POINTER(self._RD), ctypes.POINTER(ctypes.c_int32)]
        assert libc.initstate_r(1, self._buf, 128, ctypes.byref(self._rd)) == 0
        self._libc = libc
        self._out = ctypes.c_int32()

    def rand(self) -> int:
        self._libc.random_r(ctypes.byref(self._rd), ctypes.byref(self._out))
        return self._out.value

    def frand(self):
        # (float)rand()/RAND_MAX: RAND_MAX converts to float 2^31
        return f32(f32(self.rand()) / f32(2147483647))


def f2f_load(path):
    raw = open(path, "rb").read()
    mn, mx = np.frombuffer(raw[:8], f32)
    n = int(np.frombuffer(raw[8:12], np.int32)[0])
    tab = np.frombuffer(raw[12:12 + 4 * n], f32).copy()
    return dict(minval=f32(mn), maxval=f32(mx), n=n, delta=f32(f32(mx - mn) / f32(n)), table=tab)


def f2f_eval(t, x):
    x = f32(x)
    if x <= t["minval"]:
        return t["table"][0]
    if x >= t["maxval"]:
        return t["table"][t["n"] - 1]
    b = int(f32(f32(x - t["minval"]) / t["delta"]))
    if b >= t["n"] - 1:
        return t["table"][t["n"] - 1]
    f = f32(f32(x - f32(t["minval"] + f32(b * t["delta"]))) / t["delta"])
    return f32(f32(f32(1) - f) * t["table"][b] + f32(f * t["table"][b + 1]))


def deltac(z, om, ol, w):
    from oracle.d2z_ref import growth
    z, om, ol = f32(z), f32(om), f32(ol)
    x = f32(1) + z
    x2, x3 = f32(x * x), f32(f32(x * x) * x)
    omega = f32(f32(om * x3) / f32(f32(om * x3) + f32(f32(f32(1) - om - ol) * x2) + ol))
    a = f32(f32(2) / omega - f32(1))
    eta = f32(math.log(f64(a) + math.sqrt(f64(a) ** 2 - 1)))
    if om < 1 and ol == 0:
        raise NotImplementedError
    pi = f32(3.14159265358979)
    dc = f32(3 * (f64(f32(12 * pi)) ** (2. / 3.)) / 20 * (1 + 0.0123 * f64(np.log10(omega, dtype=f32))))
    return f32(dc / growth(z, om, ol, w))


_libm = None


def fcoll(z, om, ol, w, smin):
    """erfc of a float argument is the C library's erfcf (C++ overload of erfc)."""
    global _libm
    if _libm is None:
        _libm = ctypes.CDLL(ctypes.util.find_library("m"))
        _libm.erfcf.argtypes = [ctypes.c_float]
        _libm.erfcf.restype = ctypes.c_float
    arg = f32(f64(deltac(z, om, ol, w)) / math.sqrt(2.) / f64(f32(smin)))
    return f32(_libm.erfcf(arg))


def bubble_mfp(zreion, history, box_mpc, n_x, n_s):
    """GetBubbleMFP at one rank; returns mfp[n_x], mfp_x[n_x], dfdmfp[NMFP*n_x]."""
    N = zreion.shape[0]
    z = zreion.astype(f32)
    rng = GlibcRand()
    cell = f32(f32(box_mpc) / f32(N))
    mfp_final = f32(math.log(1.0 * f64(f32(box_mpc))))
    mfp_init = f32(np.log(f32(1 * cell), dtype=f32))
    dmfp = f32(f32(mfp_final - mfp_init) / f32(NMFP))
    dxmfp = f32((X1 - X0) / (n_x - 1))
    dzh = f32((H1 - H0) / (NHISTORY - 1))
    hist = np.asarray(history, f32)
    mfp = np.zeros(n_x, f32)
    dfd = np.zeros(NMFP * n_x, f32)
    zcur = f32(0)

    def account(ix, m, frac):
        clow = f32(math.log(m - 0.5))
        if m > 1:
            clow = f32(math.log(m - 1.0))
        chigh = f32(math.log(m * 1.0))
        cd = f32(np.exp(f32(clow + f32(f32(chigh - clow) * frac)), dtype=f32) * cell)
        lcd = np.log(cd, dtype=f32)
        imfp = int(f32(f32(lcd - mfp_init) / dmfp))
        if 0 <= imfp < NMFP and lcd < mfp_final and lcd > mfp_init:
            dfd[ix * NMFP + imfp] += 1
        return cd

    for ix in range(n_x):
        xcur = f32(X0 + f64(f32(ix * dxmfp)))
        if xcur < hist[0]:
            zcur = f32(H0)
        elif xcur > hist[-1]:
            zcur = f32(H1)
        else:
            i = int(np.searchsorted(hist, xcur, side="left")) - 1   # last i with hist[i] < xcur
            if 0 <= i < NHISTORY - 1 and hist[i] < xcur < hist[i + 1]:
                fint = f32(f32(xcur - hist[i]) / f32(hist[i + 1] - hist[i]))
                zcur = f32(f64(f32(1) - fint) * (H0 + f64(f32(i * dzh))) + f64(fint) * (H0 + f64(f32((i + 1) * dzh))))
        ml = f32(0)
        for _ in range(n_s):
            while True:
                sx, sy, sz = rng.frand(), rng.frand(), rng.frand()
                i0, j0, k0 = int(f32(sx * f32(N))), int(f32(sy * f32(N))), int(f32(sz * f32(N)))
                i0, j0, k0 = i0 % N if i0 >= N else i0, j0 - N if j0 >= N else j0, k0 - N if k0 >= N else k0
                if z[i0, j0, k0] > zcur and j0 < N - 2 and k0 < N - 2:
                    break
            j, m = j0, 0
            while True:
                j = j + 1 - (N if j + 1 >= N else 0)
                m += 1
                if z[i0, j, k0] < zcur or j == j0:
                    break
            fy = rng.frand()
            ml = f32(ml + account(ix, m, fy))
            k, m = k0, 0
            while True:
                k = k + 1 - (N if k + 1 >= N else 0)
                m += 1
                if z[i0, j0, k] < zcur or k == k0:
                    break
            fz = rng.frand()
            ml = f32(ml + account(ix, m, fz))
        mfp[ix] = f32(f64(ml) / (2. * n_s))
    mfp_x = np.array([f32(X0 + f64(f32(i * dxmfp))) for i in range(n_x)], f32)
    return mfp, mfp_x, dfd


def chistory(fct, mfp, rmfp, zeta):
    n_x = len(mfp)
    dzch = f32((H1 - H0) / (NCHISTORY - 1))
    dxmfp = f32((X1 - X0) / (n_x - 1))
    rmfp, zeta = f32(rmfp), f32(zeta)

    def bmfp(x):
        itab = int((f64(x) - X0) / f64(dxmfp))
        f = f32((f64(f32(x - f32(itab * dxmfp))) - X0) / f64(dxmfp))
        if itab < 0:
            return mfp[0]
        if itab >= n_x - 1:
            return mfp[n_x - 1]
        return f32(f32(f32(1) - f) * mfp[itab] + f32(f * mfp[itab + 1]))

    ch = np.zeros(NCHISTORY, f32)
    for i in range(1, NCHISTORY):
        x1 = ch[i - 1]
        z1 = f32(H0 + f64(f32(i * dzch)))
        z2 = f32(H0 + f64(f32((i + 1) * dzch)))
        df = f32(f2f_eval(fct, z2) - f2f_eval(fct, z1))
        rb = bmfp(x1)
        v = f32(ch[i - 1] + f32(f32(df / f32(f32(1) + f32(rb / rmfp))) * zeta))
        ch[i] = f32(1) if v >= 1 else v
    return ch


def zvz(history, ch):
    dzch = f32((H1 - H0) / (NCHISTORY - 1))
    out = np.full(NHISTORY, f32(-1), f32)
    for i in range(1, NHISTORY):
        x = history[i]
        if x == 0:
            continue
        if x < ch[0]:
            out[i] = f32(H0)
        elif x > ch[-1]:
            out[i] = f32(H1)
        else:
            hits = np.nonzero((x >= ch[:-1]) & (x <= ch[1:]))[0]
            j = int(hits[0])
            f = f32(f32(x - ch[j]) / f32(ch[j + 1] - ch[j]))
            out[i] = f32(f64(f32(1) - f) * (H0 + f64(f32(j * dzch))) + f64(f) * (H0 + f64(f32((j + 1) * dzch))))
    for i in range(NHISTORY - 2, -1, -1):
        if out[i] < 0:
            out[i] = out[i + 1]
    return out


def correct(zreion, zv):
    dz = f32((H1 - H0) / (NHISTORY - 1))
    z = zreion.astype(f32).copy()
    q = np.trunc((z.astype(f64) - H0) / f64(dz))
    ok = (q >= 0) & (q < NHISTORY)
    z[ok] = zv[q[ok].astype(np.int64)]
    return z
