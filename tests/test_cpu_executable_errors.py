"""Failure paths of the delta2zreion executable that end before any device
work: a missing parameter file, a grid size without a plan, a truncated
delta file.  Each exits non-zero with a message (no crash, no output file)."""
import os
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(REPO, "pr-calc_gb300", "bin", "delta2zreion")
pytestmark = pytest.mark.skipif(not os.access(EXE, os.X_OK), reason="executable not built")

PARAMS = ("Omegam 0.31\nOmegal 0.69\nOmegab 0.049\nh 0.68\nns 0.965\nsigma8 0.81\nw -1\n"
          "BoxSize {box}\nN {N}\nzInit 0\nDeltaFile delta\nRmin 2\nNscales 4\n")


def _run(tmp_path, *args):
    return subprocess.run([EXE, *args, "-v", "-e"], cwd=tmp_path, capture_output=True, text=True, timeout=120)


def test_missing_parameter_file(tmp_path):
    r = _run(tmp_path, "nope.d2z", "-f", "run")
    assert r.returncode != 0
    assert "not found" in r.stdout


def test_grid_size_without_plan(tmp_path):
    (tmp_path / "p.d2z").write_text(PARAMS.format(box=30.0, N=20))
    np.zeros(20 ** 3, np.float32).tofile(tmp_path / "delta")
    r = _run(tmp_path, "p.d2z", "-f", "run")
    assert r.returncode != 0
    assert "no GPU FFT plan" in r.stdout


def test_truncated_delta_file(tmp_path):
    (tmp_path / "p.d2z").write_text(PARAMS.format(box=24.0, N=16))
    np.zeros(16 ** 3 - 1, np.float32).tofile(tmp_path / "delta")
    r = _run(tmp_path, "p.d2z", "-f", "run")
    assert r.returncode != 0
    assert "cannot read" in r.stdout
    assert not (tmp_path / "output" / "run.zreion").exists()
