"""FP64 restatement of the whole delta2zreion chain with torch on the GPU
(cuFFT in double precision): the full-size reference of the precision and
adjoint tests.  Test-only; the product never calls it."""
import math


def kmag(N, box_mpc, device):
    import torch
    f = torch.fft.fftfreq(N, d=1.0 / N, device=device, dtype=torch.float64)
    fz = torch.arange(N // 2 + 1, device=device, dtype=torch.float64)
    dk = 2.0 * math.pi / box_mpc
    k2 = (f[:, None, None] ** 2 + f[None, :, None] ** 2 + fz[None, None, :] ** 2) * dk * dk
    return torch.sqrt(k2)


def tophat64(x):
    import torch
    small = x < 1e-2
    xs = torch.where(small, torch.ones_like(x), x)
    w = 3.0 * (torch.sin(xs) - xs * torch.cos(xs)) / xs ** 3
    x2 = x * x
    ws = 1.0 - x2 / 10.0 + x2 * x2 / 280.0
    return torch.where(small, ws, w)


def chain(delta, box_mpc, R, A, B, dinit, radii_check=(), km=None):
    """zreion / argmax / top-two margin / max|delta_R| and delta_R of the
    radii in radii_check, all in FP64 on delta's device."""
    import torch
    N = delta.shape[0]
    dev = delta.device
    spec = torch.fft.rfftn(delta.double() / dinit)
    km = kmag(N, box_mpc, dev) if km is None else km
    best = torch.full(delta.shape, -math.inf, dtype=torch.float64, device=dev)
    second = best.clone()
    am = torch.full(delta.shape, 255, dtype=torch.uint8, device=dev)
    dmax = 0.0
    keep = {}
    for r in range(len(R)):
        W = tophat64(km * R[r])
        W[0, 0, 0] = 0.0
        dR = torch.fft.irfftn(spec * W, s=(N, N, N))
        del W
        dmax = max(dmax, float(dR.abs().max()))
        if r in radii_check:
            keep[r] = dR.clone()
        z = A * (dR + B[r]) - 1.0
        del dR
        gt = z > best
        second = torch.where(gt, best, torch.where(z > second, z, second))
        best = torch.where(gt, z, best)
        am[gt] = r
        del z, gt
    zo = torch.where(best > 0, best, torch.zeros_like(best))
    am = torch.where(best > 0, am, torch.full_like(am, 255))
    gap = torch.minimum(best - second, best.abs())
    return zo, am, gap, dmax, keep
