"""Synthetic linear density fields for the delta2zreion workloads.

Unit Gaussian white noise from Philox4x32-10 (Salmon, Moraes, Dror & Shaw,
"Parallel random numbers: as easy as 1, 2, 3", SC 2011; counter = cell index,
key = (seed, 0)) and a Box-Muller transform in FP64, shaped by a BBKS power
spectrum (Bardeen, Bond, Kaiser & Szalay 1986; shape parameter Gamma =
Omega_m h, no baryon correction) normalised to sigma_8 with an 8 Mpc/h top hat:

    delta_hat(k) = DFT(w)(k) * sqrt(N^3 P(k) / L^3),  delta_hat(0) = 0,
    delta = IDFT(delta_hat) / N^3,

the normalisation of pr-calc's own generator (grf_ics.C:20-28,49-78).  The field
is a z = 0 float32 grid in file order (x-major, z fastest).  numpy serves small
grids; `backend="torch"` runs the same arithmetic on a CUDA device.
"""
from __future__ import annotations

import math

import numpy as np

PHILOX_M0, PHILOX_M1 = 0xD2511F53, 0xCD9E8D57
PHILOX_W0, PHILOX_W1 = 0x9E3779B9, 0xBB67AE85
M32 = 0xFFFFFFFF


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 on uint64 arrays holding 32-bit words."""
    c0, c1, c2, c3 = (np.asarray(x, np.uint64) & M32 for x in (c0, c1, c2, c3))
    k0 = np.uint64(k0 & M32)
    k1 = np.uint64(k1 & M32)
    for r in range(10):
        if r:
            k0 = np.uint64((int(k0) + PHILOX_W0) & M32)
            k1 = np.uint64((int(k1) + PHILOX_W1) & M32)
        p0 = c0 * np.uint64(PHILOX_M0)
        p1 = c2 * np.uint64(PHILOX_M1)
        hi0, lo0 = p0 >> np.uint64(32), p0 & np.uint64(M32)
        hi1, lo1 = p1 >> np.uint64(32), p1 & np.uint64(M32)
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return c0, c1, c2, c3


def white_noise(N: int, seed: int) -> np.ndarray:
    """Unit Gaussian per cell: Box-Muller on words 0 and 1 of Philox(cell, seed)."""
    n = N ** 3
    out = np.empty(n, np.float64)
    chunk = 1 << 22
    for s in range(0, n, chunk):
        idx = np.arange(s, min(n, s + chunk), dtype=np.uint64)
        x0, x1, _, _ = philox4x32_10(idx & np.uint64(M32), idx >> np.uint64(32), 0, 0, seed, 0)
        u1 = (x0.astype(np.float64) + 0.5) / 4294967296.0
        u2 = (x1.astype(np.float64) + 0.5) / 4294967296.0
        out[s:s + len(idx)] = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)
    return out.reshape(N, N, N)


def white_noise_torch(N: int, seed: int, device="cuda"):
    """white_noise() on a CUDA device (int64 tensors holding 32-bit words)."""
    import torch
    n = N ** 3
    out = torch.empty(n, dtype=torch.float64, device=device)
    chunk = 1 << 24
    m32 = 0xFFFFFFFF
    for s in range(0, n, chunk):
        idx = torch.arange(s, min(n, s + chunk), dtype=torch.int64, device=device)
        c0, c1 = idx & m32, idx >> 32
        c2 = torch.zeros_like(c0)
        c3 = torch.zeros_like(c0)
        k0, k1 = seed & m32, 0
        for r in range(10):
            if r:
                k0 = (k0 + PHILOX_W0) & m32
                k1 = (k1 + PHILOX_W1) & m32
            p0 = c0 * PHILOX_M0          # wraps mod 2^64; the masks below recover both halves
            p1 = c2 * PHILOX_M1
            hi0, lo0 = (p0 >> 32) & m32, p0 & m32
            hi1, lo1 = (p1 >> 32) & m32, p1 & m32
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        u1 = (c0.to(torch.float64) + 0.5) / 4294967296.0
        u2 = (c1.to(torch.float64) + 0.5) / 4294967296.0
        out[s:s + len(idx)] = torch.sqrt(-2.0 * torch.log(u1)) * torch.cos(2.0 * math.pi * u2)
    return out.reshape(N, N, N)


def white_noise_native(N: int, seed: int, device="cuda"):
    """white_noise() by this library's kernel (prc_white_noise), float32, on
    the current CUDA stream of `device`."""
    import torch
    from . import _lib
    out = torch.empty(N ** 3, dtype=torch.float32, device=device)
    st = torch.cuda.current_stream(out.device).cuda_stream
    _lib.check(_lib.load().prc_white_noise(out.data_ptr(), N ** 3, int(seed) & 0xFFFFFFFF, st))
    return out.reshape(N, N, N)


def bbks_transfer(k_hmpc, omegam: float, h: float):
    """T(q), q = k / Gamma with k in h/Mpc and Gamma = Omega_m h."""
    q = np.asarray(k_hmpc, np.float64) / (omegam * h)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.log1p(2.34 * q) / (2.34 * q) * (1 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3
                                               + (6.71 * q) ** 4) ** -0.25
    return np.where(q > 0, t, 1.0)


def power_norm(omegam: float, h: float, ns: float, sigma8: float) -> float:
    """Amplitude so that sigma(8 Mpc/h) = sigma8 for P = amp k^ns T^2 (k in h/Mpc)."""
    from scipy.integrate import quad

    def f(lk):
        k = math.exp(lk)
        x = 8.0 * k
        W = 3 * (math.sin(x) - x * math.cos(x)) / x ** 3 if x > 1e-3 else 1 - x * x / 10
        T = float(bbks_transfer(k, omegam, h))
        return k ** 3 * k ** ns * T * T * W * W / (2 * math.pi ** 2)

    s2 = 0.0
    edges = [math.log(x) for x in (1e-5, 1e-2, 0.1, 0.3, 1.0, 3.0, 10.0, 30.0, 100.0, 1e3)]
    for a, b in zip(edges[:-1], edges[1:]):
        s2 += quad(f, a, b, epsabs=0, epsrel=1e-9, limit=2000)[0]
    return sigma8 ** 2 / s2


def spectrum_amplitude(N: int, box_hmpc: float, omegam=0.31, h=0.68, ns=0.965, sigma8=0.81):
    """sqrt(N^3 P(k) / L^3) on the rfft grid (N, N, N//2+1), L in Mpc/h."""
    amp = power_norm(omegam, h, ns, sigma8)
    f = np.fft.fftfreq(N, 1.0 / N)
    fz = np.arange(N // 2 + 1, dtype=np.float64)
    dk = 2 * math.pi / box_hmpc
    k = dk * np.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + fz[None, None, :] ** 2)
    with np.errstate(divide="ignore"):
        P = np.where(k > 0, amp * k ** ns * bbks_transfer(k, omegam, h) ** 2, 0.0)
    return np.sqrt(N ** 3 * P / box_hmpc ** 3)


def amplitude_table(N: int, box_hmpc: float, omegam=0.31, h=0.68, ns=0.965, sigma8=0.81) -> np.ndarray:
    """sqrt(N^3 P(k) / L^3) / N^3 indexed by the integer |m|^2 = fx^2 + fy^2 + fz^2
    (0 .. 3 (N/2)^2), k = (2 pi / L) sqrt(|m|^2): the table prc_d2z_gaussian_field
    takes (the 1/N^3 is the inverse transform's normalisation)."""
    amp = power_norm(omegam, h, ns, sigma8)
    m2 = np.arange(3 * (N // 2) ** 2 + 1, dtype=np.float64)
    k = (2 * math.pi / box_hmpc) * np.sqrt(m2)
    with np.errstate(divide="ignore"):
        P = np.where(k > 0, amp * k ** ns * bbks_transfer(k, omegam, h) ** 2, 0.0)
    return (np.sqrt(N ** 3 * P / box_hmpc ** 3) / N ** 3).astype(np.float32)


def gaussian_field(N: int, box_hmpc: float, seed: int = 1, omegam=0.31, h=0.68, ns=0.965, sigma8=0.81,
                   backend: str = "numpy", device="cuda", engine=None):
    """float32 delta_lin (N, N, N) at z = 0 in file order.

    backend "numpy" (host, FP64 transforms), "torch" (the same on a CUDA device
    through torch.fft) or "native" (this library's kernels: Philox noise, the
    float32 R2C / C2R passes of the step; `engine` is an optional
    Delta2Zreion context of this N to use, else one is made)."""
    if backend == "native":
        import torch
        from . import Delta2Zreion
        tab = amplitude_table(N, box_hmpc, omegam, h, ns, sigma8)
        own = engine is None
        if own:
            engine = Delta2Zreion(N, box_hmpc / h, [1.0], [0.0], 1.0, 1.0)
        try:
            out = torch.empty((N, N, N), dtype=torch.float32, device=device)
            engine.gaussian_field(seed, tab, out=out)
            return out
        finally:
            if own:
                engine.close()
    S = spectrum_amplitude(N, box_hmpc, omegam, h, ns, sigma8)
    if backend == "torch":
        import torch
        wt = white_noise_torch(N, seed, device)
        St = torch.from_numpy(S).to(device)
        d = torch.fft.irfftn(torch.fft.rfftn(wt) * St, s=(N, N, N))
        return d.to(torch.float32)
    import scipy.fft as sfft
    w = white_noise(N, seed)
    d = sfft.irfftn(sfft.rfftn(w, workers=-1) * S, s=(N, N, N), workers=-1)
    return d.astype(np.float32)
