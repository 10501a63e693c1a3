"""Writes the golden fixtures of the delta2zreion step (tests/golden/*.npz).

The reference ships no golden vectors for this path and cannot be built here
(MPI, FFTW and GSL are absent), so the fixtures are the CPU oracle's outputs
(oracle/d2z_ref.py, FP64 and the reference's float arithmetic) on seeded
synthetic fields, frozen so that later changes to the oracle, the field
generator or the GPU path are all checked against the same numbers.

    python tests/golden/make_golden.py          # from the repository root

Each case: delta_lin (Philox4x32-10 + BBKS field), the host tables (radii,
barrier B_r, A, D_init), zreion / argmax in both precisions, the FP64 top-two
margin of every cell, delta_R of the first and last radius (FP64) and the
GetHistory bin counts of the FP64 zreion.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for _p in (REPO, os.path.join(REPO, "pr-calc_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

# (N, box Mpc/h, n_radii, Rmax Mpc/h, zeta, seed)
CASES = [(16, 24.0, 6, 9.6, 30.0, 11), (24, 36.0, 5, 14.4, 30.0, 12)]
H = 0.68
M_MIN = 1.47e9


def case_name(N):
    return os.path.join(HERE, f"d2z_n{N}.npz")


def make(N, box, nr, rmax, zeta, seed):
    from oracle import d2z_ref as orc
    from prc_d2z import fields
    op = orc.Parameters(N=N, Nscales=nr, BoxSize=box, Rmin=2.0, Rmax=rmax, zeta=zeta, M_min=M_MIN)
    t = orc.tables(op)
    delta = fields.gaussian_field(N, box, seed=seed)
    box_mpc = float(np.float32(box) / np.float32(H))
    z64, a64, _ = orc.d2z(delta.astype(np.float64), box_mpc, t.R, t.A, t.B, t.DInit, mode="fp64")
    z32, a32, s32 = orc.d2z(delta, box_mpc, t.R, t.A, t.B, t.DInit, mode="fp32")
    zs, dmax = orc.z_stack(delta, box_mpc, t.R, t.A, t.B, t.DInit, mode="fp64")
    _, _, gap = orc.margins(zs)
    dR0 = orc.delta_R(delta, box_mpc, t.R[0], t.DInit, mode="fp64")
    dRl = orc.delta_R(delta, box_mpc, t.R[-1], t.DInit, mode="fp64")
    counts, _, _ = orc.history(z64.astype(np.float32))
    nz = np.nonzero(counts)[0]
    np.savez_compressed(
        case_name(N), N=N, box_hmpc=box, box_mpc=box_mpc, seed=seed, zeta=zeta, rmax=rmax,
        delta=delta, radii_mpc=np.asarray(t.R, np.float64), barrier_b=np.asarray(t.B, np.float64),
        barrier_a=float(t.A), dinit=float(t.DInit), erfizeta=float(t.erfizeta), sigma_min=float(t.sigma_min),
        zreion64=z64.astype(np.float64), argmax64=a64, zreion32=z32.astype(np.float32), argmax32=a32,
        sigma_grid32=np.asarray(s32, np.float64), gap64=gap.astype(np.float64), dmax64=float(dmax),
        delta_r_first=dR0.astype(np.float64), delta_r_last=dRl.astype(np.float64),
        hist_bins=nz.astype(np.int32), hist_counts=counts[nz].astype(np.uint32))


if __name__ == "__main__":
    for c in CASES:
        make(*c)
        print("wrote", case_name(c[0]))
