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
