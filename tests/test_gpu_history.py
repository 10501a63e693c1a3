"""GPU parts of the history-correction chain (skewer walks, per-cell map) and
the drop-in executable end to end."""
import os
import subprocess

import numpy as np
import pytest

import prc_d2z
from oracle import history_ref as hr
from prc_d2z import fields

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
H_ = 0.68


def _zreion(N=32, seed=5, zeta=30.0):
    box = 1.5 * N
    p = prc_d2z.Parameters(N=N, Nscales=10, BoxSize=box)
    cl = prc_d2z.CLParameters(Rmax=0.4 * box, zeta=zeta, M_min=1.47e9)
    delta = fields.gaussian_field(N, box, seed=seed)
    ctx = prc_d2z.Delta2Zreion.from_parameters(p, cl)
    z, _, _ = ctx.forward(delta)
    return ctx, z, float(np.float32(box) / np.float32(H_)), delta, p, cl


def test_bubble_mfp_matches_the_oracle():
    ctx, z, box_mpc, *_ = _zreion()
    _, hist, _ = ctx.history(z)
    mfp, mfp_x, dfd = ctx.bubble_mfp(z, hist, box_mpc, n_x=16, n_skewers=48)
    mo, mxo, dfo = hr.bubble_mfp(z, hist, box_mpc, 16, 48)
    np.testing.assert_array_equal(mfp, mo)
    np.testing.assert_array_equal(mfp_x, mxo)
    np.testing.assert_array_equal(dfd, dfo)
    ctx.close()


def test_correct_matches_the_oracle(tmp_path):
    ctx, z, box_mpc, *_ = _zreion(seed=6)
    _, hist, _ = ctx.history(z)
    ch = np.minimum(np.cumsum(np.full(10000, 1.2e-4, np.float32), dtype=np.float32), 1).astype(np.float32)
    ch[0] = 0
    zv = prc_d2z.zvz_map(hist, ch)
    zc = ctx.correct(z.copy(), zv)
    np.testing.assert_array_equal(zc, hr.correct(z, zv))
    ctx.close()


def test_executable_end_to_end(tmp_path):
    """delta2zreion with the reference's command line and files."""
    exe = os.path.join(REPO, "pr-calc_gb300", "bin", "delta2zreion")
    N, box = 32, 48.0
    delta = fields.gaussian_field(N, box, seed=7)
    delta.tofile(tmp_path / "delta")
    smin = prc_d2z.compute_tables(prc_d2z.Parameters(N=N, Nscales=10, BoxSize=box),
                                  prc_d2z.CLParameters(Rmax=20.0, zeta=30.0, M_min=1.47e9)).sigma_min
    z = np.linspace(0.0, 50.0, 2001)
    with open(tmp_path / "fcoll_table.tab", "wb") as fh:
        np.array([0.0, 50.0], np.float32).tofile(fh)
        np.array([len(z)], np.int32).tofile(fh)
        np.array([hr.fcoll(v, 0.31, 0.69, -1.0, smin) for v in z], np.float32).tofile(fh)
    (tmp_path / "param.d2z").write_text(
        "# cosmology\nOmegam 0.31\nOmegal 0.69\nOmegab 0.049\nh 0.68\nns 0.965\nsigma8 0.81\nw -1\n"
        f"BoxSize {box}\nN {N}\nzInit 0\nDeltaFile delta\nRmin 2\nNscales 10\nBogus 3\n")
    r = subprocess.run([exe, "param.d2z", "-f", "run", "-m", "1.47e9", "-z", "30", "-r", "20", "-v", "-e"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Tag 'Bogus' not allowed" in r.stdout
    assert "tau =" in r.stdout
    used = (tmp_path / "param.d2z-usedvalues").read_text()
    assert "Nscales" in used and "Bogus" not in used
    out = tmp_path / "output"
    zfile = np.fromfile(out / "run.zreion", np.float32).reshape(N, N, N)
    # the consumers' slab reader (ReadReionFile at two ranks) sees the same field
    from prc_d2z import io as pio
    slabs = [pio.read_reion_file(str(out / "run.zreion"), N, 2, q)[0] for q in range(2)]
    assert np.array_equal(np.concatenate(slabs), zfile)
    # the same chain through the Python API
    p = prc_d2z.Parameters(N=N, Nscales=10, BoxSize=box)
    cl = prc_d2z.CLParameters(Rmax=20.0, zeta=30.0, M_min=1.47e9)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
        zr, _, _ = ctx.forward(delta)
        ctx.correct_history(zr, str(tmp_path / "fcoll_table.tab"), float(np.float32(box) / np.float32(0.68)),
                            20.0, 30.0)
    np.testing.assert_array_equal(zfile, zr)
    hist = np.loadtxt(out / "run.history")
    assert hist.shape == (100000, 4)
    assert (out / "run.mfp").exists() and (out / "run.mfppdf").stat().st_size == 8 + 16 + 4 * 200 * 1000


def test_executable_requires_fcoll_table(tmp_path):
    """Without fcoll_table.tab the history correction cannot run: the
    executable stops with a message and writes no .zreion."""
    exe = os.path.join(REPO, "pr-calc_gb300", "bin", "delta2zreion")
    N, box = 16, 24.0
    fields.gaussian_field(N, box, seed=7).tofile(tmp_path / "delta")
    (tmp_path / "param.d2z").write_text(
        "Omegam 0.31\nOmegal 0.69\nOmegab 0.049\nh 0.68\nns 0.965\nsigma8 0.81\nw -1\n"
        f"BoxSize {box}\nN {N}\nzInit 0\nDeltaFile delta\nRmin 2\nNscales 4\n")
    r = subprocess.run([exe, "param.d2z", "-f", "run", "-r", "9", "-v", "-e"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode != 0
    assert "fcoll_table.tab" in r.stdout
    assert not (tmp_path / "output" / "run.zreion").exists()


def test_executable_records_bubble_sizes(tmp_path):
    """RecordBubbleSizes 1: the executable writes <base>.rbubble, the radius
    [Mpc] of each cell's winning scale (delta2zreion_d2z.C:117-120, written as
    by WriteRbubbleFile, io_d2z.C:248-282: raw float32 N^3, file order), and 0
    where no scale won (the reference leaves those cells unset).  It equals
    R[argmax] of the forward call and of the fp32 oracle on clear cells."""
    from oracle import d2z_ref as orc
    exe = os.path.join(REPO, "pr-calc_gb300", "bin", "delta2zreion")
    N, box = 32, 48.0
    delta = fields.gaussian_field(N, box, seed=8)
    delta.tofile(tmp_path / "delta")
    smin = prc_d2z.compute_tables(prc_d2z.Parameters(N=N, Nscales=10, BoxSize=box),
                                  prc_d2z.CLParameters(Rmax=20.0, zeta=30.0, M_min=1.47e9)).sigma_min
    z = np.linspace(0.0, 50.0, 2001)
    with open(tmp_path / "fcoll_table.tab", "wb") as fh:
        np.array([0.0, 50.0], np.float32).tofile(fh)
        np.array([len(z)], np.int32).tofile(fh)
        np.array([hr.fcoll(v, 0.31, 0.69, -1.0, smin) for v in z], np.float32).tofile(fh)
    (tmp_path / "param.d2z").write_text(
        "Omegam 0.31\nOmegal 0.69\nOmegab 0.049\nh 0.68\nns 0.965\nsigma8 0.81\nw -1\n"
        f"BoxSize {box}\nN {N}\nzInit 0\nDeltaFile delta\nRmin 2\nNscales 10\nRecordBubbleSizes 1\n")
    r = subprocess.run([exe, "param.d2z", "-f", "run", "-m", "1.47e9", "-z", "30", "-r", "20", "-v", "-e"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Bubble sizes written" in r.stdout
    rb = np.fromfile(tmp_path / "output" / "run.rbubble", np.float32)
    assert rb.size == N ** 3
    rb = rb.reshape(N, N, N)
    p = prc_d2z.Parameters(N=N, Nscales=10, BoxSize=box, RecordBubbleSizes=1)
    cl = prc_d2z.CLParameters(Rmax=20.0, zeta=30.0, M_min=1.47e9)
    with prc_d2z.Delta2Zreion.from_parameters(p, cl) as ctx:
        _, am, _ = ctx.forward(delta)
        t = ctx.tables
    Rf = t.radii_mpc.astype(np.float32)
    want = np.where(am == 255, np.float32(0), Rf[np.minimum(am, len(Rf) - 1)])
    assert np.array_equal(rb, want)
    assert (rb > 0).mean() > 0.05
    box_mpc = float(np.float32(box) / np.float32(H_))
    _, amo, _ = orc.d2z(delta, box_mpc, t.radii_mpc, t.barrier_a, t.barrier_b, t.DInit, mode="fp32")
    wo = np.where(amo == 255, np.float32(0), Rf[np.minimum(amo, len(Rf) - 1)])
    assert np.mean(rb == wo) > 0.999
