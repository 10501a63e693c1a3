"""Build recipe of the oracle's C helper (test infrastructure only).

Compiles oracle/d2z_cells.c into oracle/_build/liborc_cells.so with gcc,
OpenMP and -ffp-contract=off (the reference's float expressions round per
operation).  The reference itself is not built: it needs MPI, FFTW 3.3.3 and
GSL, none of which are installed where this code is built and run, so there is no
oracle/_ref.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "liborc_cells.so")


def build() -> str:
    src = os.path.join(HERE, "d2z_cells.c")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(src):
        cmd = [os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               src, "-o", OUT, "-lm"]
        subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build())
