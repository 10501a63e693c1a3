"""Grid files of the delta2zreion step, as the reference's producers and
consumers read and write them: headerless float32 N^3, x-major, z fastest.

  read_delta_file   ReadDeltaFile  (io_d2z.C:164-207): x-slab i of rank q at
                    byte offset (q*Nlocal + i)*N^2*4; mean and sigma in double
  write_zreion_file WriteZreionFile (io_d2z.C:209-245): the unpadded field
  read_reion_file   ReadReionFile of the consumers (flatskymap io_map.C:179-214,
                    allskymap io_asm.C:183, limber io_lmb.C:182): the same slab
                    layout; flatskymap also prints the local mean in double

Nlocal = N / nproc (the FFTW-MPI slab decomposition the reference assumes).
"""
from __future__ import annotations

import numpy as np

__all__ = ["read_delta_file", "write_zreion_file", "read_reion_file", "write_delta_file"]


def _slabs(path: str, N: int, nproc: int, rank: int) -> np.ndarray:
    if N % nproc:
        raise ValueError(f"N={N} is not divisible by nproc={nproc}")
    nloc = N // nproc
    out = np.empty((nloc, N, N), np.float32)
    with open(path, "rb") as fh:
        for i in range(nloc):
            fh.seek((rank * nloc + i) * N * N * 4)
            buf = fh.read(N * N * 4)
            if len(buf) != N * N * 4:
                raise IOError(f"{path}: short read of slab {rank * nloc + i} (file smaller than N^3 floats)")
            out[i] = np.frombuffer(buf, np.float32).reshape(N, N)
    return out


def _seq_sum(a: np.ndarray) -> float:
    """Sequential double accumulation in file order (the reference's loops)."""
    return float(np.add.accumulate(a.astype(np.float64).ravel())[-1]) if a.size else 0.0


def read_delta_file(path: str, N: int, nproc: int = 1, rank: int = 0):
    """(local slab (Nlocal, N, N), mean, sigma) -- mean and sigma over the whole
    grid when nproc == 1 (otherwise of the local slab; the reference sums them
    over ranks with MPI_Allreduce)."""
    s = _slabs(path, N, nproc, rank)
    n3 = float(np.float32(N)) ** 3
    lmean = _seq_sum(s)
    lsig = _seq_sum(s.astype(np.float64) ** 2)
    return s, lmean / n3, float(np.sqrt(lsig / n3))


def write_delta_file(path: str, delta: np.ndarray) -> None:
    np.ascontiguousarray(delta, np.float32).tofile(path)


def write_zreion_file(path: str, zreion) -> None:
    """Unpadded float32 N^3 in file order (host array or CUDA tensor)."""
    if hasattr(zreion, "detach"):
        zreion = zreion.detach().cpu().numpy()
    np.ascontiguousarray(zreion, np.float32).tofile(path)


def read_reion_file(path: str, N: int, nproc: int = 1, rank: int = 0):
    """(local slab (Nlocal, N, N), local mean in double) as the consumers read it."""
    s = _slabs(path, N, nproc, rank)
    return s, _seq_sum(s) / (N * N * s.shape[0])
