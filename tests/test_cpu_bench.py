"""bench.py's reference arm on CPU at a small grid: the JSON line's contract
(impl, metric, cpu_baseline, e2e with no host copies) and how a step is
sampled: whole steps while the K steps fit in the CPU budget, else the
forward R2C plus an evenly spread sample of the radii."""
import argparse
import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture
def bench(monkeypatch):
    monkeypatch.syspath_prepend(REPO)
    import bench as b
    b._use_config("C2")
    # four radii keep the oracle's FP64 tables (scipy quadrature) to seconds
    monkeypatch.setattr(b, "NR", 4)
    return b


def _run(bench, capsys, **kw):
    args = argparse.Namespace(n=16, steps=2, warmup=1, ref_radii=0, gpus=1)
    for k, v in kw.items():
        setattr(args, k, v)
    bench.run_reference(args, 0)
    line = capsys.readouterr().out.strip().splitlines()[-1]
    return json.loads(line)


def test_reference_arm_whole_steps(bench, capsys):
    d = _run(bench, capsys)
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "cell*radii/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"].startswith("whole steps")
    assert d["e2e"] == {"value": d["value"], "unit": "cell*radii/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["N"] == 16 and d["config"]["radii"] == bench.NR


def test_reference_arm_samples_radii_beyond_the_budget(bench, capsys, monkeypatch):
    monkeypatch.setattr(bench, "REF_BUDGET_S", 1e-9)
    d = _run(bench, capsys)
    assert f"2 of {bench.NR} radii" in d["cpu_baseline"]["sample"]
    d = _run(bench, capsys, ref_radii=3)
    assert f"3 of {bench.NR} radii" in d["cpu_baseline"]["sample"]


def test_other_ranks_print_nothing(bench, capsys):
    args = argparse.Namespace(n=16, steps=1, warmup=1, ref_radii=0, gpus=2)
    bench.run_reference(args, 1)
    assert capsys.readouterr().out == ""


def test_step_bytes_at_512(monkeypatch):
    """The roofline arithmetic of the 512^3 x 64 line: the compulsory floor
    8 N_c + 8 N^3 per radius (103.2 GB), the canonical 3-pass model
    40 N_c + 8 N^3 per radius plus the forward R2C's 4 N^3 + 40 N_c (241.2 GB
    + 3.2 GB), and the kernels' own bytes: one sweep of 64 radii reads the
    spectrum and writes zreion once (142.3 GB), two sweeps of 32 read them
    twice (143.9 GB)."""
    monkeypatch.syspath_prepend(REPO)
    import bench as b
    b._use_config("C2")
    N = 512
    Nc = N * N * (N // 2 + 1)
    own64, floor, canon = b._step_bytes(N, 64)
    own32, _, _ = b._step_bytes(N, 32)
    assert floor == 64 * (8 * Nc + 8 * N ** 3) and abs(floor / 1e9 - 103.21) < 0.01
    assert canon == 64 * (40 * Nc + 8 * N ** 3) + 4 * N ** 3 + 40 * Nc
    assert abs((canon - 4 * N ** 3 - 40 * Nc) / 1e9 - 241.19) < 0.01
    # forward (r2c: 4 N^3 + 8 N_c; two column passes: 16 N_c each), window
    # (8 N_c + 8 N_c b), y pass (16 N_c b), z pass (8 N_c b + 4 N^3, +4 N^3 a later sweep)
    fwd = 4 * N ** 3 + 8 * Nc + 32 * Nc
    assert own64 == fwd + 8 * Nc + 8 * Nc * 64 + 16 * Nc * 64 + 8 * Nc * 64 + 4 * N ** 3
    assert own32 - own64 == 8 * Nc + 8 * N ** 3
