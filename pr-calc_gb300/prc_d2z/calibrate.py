"""Calibration of the ionising efficiency zeta for a workload.

The benchmark configurations fix zeta so that the ionisation midpoint is at
z = 8: the raw (uncorrected) zreion field has x_i(z=8) = 0.5, x_i(z) being
the fraction of cells with zreion > z (GetHistory's cumulative history).
zeta only enters through erfizeta = erfc^-1(1/zeta), so the bisection in
log zeta recomputes the host tables and swaps the barrier table of one
device context per step (prc_d2z_set_barrier).

    python -m prc_d2z.calibrate --n 512 --box 600 --nr 64 --rmax 60
"""
from __future__ import annotations

import argparse
import math

import numpy as np

from . import CLParameters, Delta2Zreion, Parameters, compute_tables, fields


def ionised_fraction(ctx, delta_dev, z: float) -> float:
    import torch
    zr, _, _ = ctx.forward(delta_dev, want_argmax=False)
    return float((zr > z).to(torch.float64).mean().item())


def calibrate(N: int, box_hmpc: float, n_radii: int, rmax_hmpc: float, rmin_cells: float = 2.0,
              mmin_msun: float = 1e9 / 0.68, seed: int = 1, z_mid: float = 8.0, x_mid: float = 0.5,
              lo: float = 2.0, hi: float = 2000.0, iters: int = 30):
    import torch
    p = Parameters(N=N, Nscales=n_radii, BoxSize=box_hmpc, Rmin=rmin_cells)
    delta = fields.gaussian_field(N, box_hmpc, seed=seed, backend="torch").contiguous()
    cl = CLParameters(Rmax=rmax_hmpc, zeta=math.sqrt(lo * hi), M_min=mmin_msun)
    ctx = Delta2Zreion.from_parameters(p, cl, argmax=False)
    f_lo, f_hi = None, None
    for _ in range(iters):
        mid = math.sqrt(lo * hi)
        cl.zeta = mid
        t = compute_tables(p, cl)
        ctx.set_barrier(t.barrier_b, t.barrier_a)
        x = ionised_fraction(ctx, delta, z_mid)
        if x < x_mid:
            lo = mid
        else:
            hi = mid
        if hi / lo < 1 + 1e-5:
            break
    torch.cuda.synchronize()
    ctx.close()
    return math.sqrt(lo * hi)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, required=True)
    ap.add_argument("--box", type=float, required=True)
    ap.add_argument("--nr", type=int, required=True)
    ap.add_argument("--rmax", type=float, default=60.0)
    ap.add_argument("--rmin", type=float, default=2.0)
    ap.add_argument("--seed", type=int, default=1)
    a = ap.parse_args()
    print(f"N={a.n} box={a.box} nr={a.nr} zeta={calibrate(a.n, a.box, a.nr, a.rmax, a.rmin, seed=a.seed):.6g}")
