"""Autotuner for the delta2zreion step.

For a grid side N and a radius count it times every compiled window-pass
variant (tile width and radix plan, prc_d2z_win_variants) at several radius
batches (radii per sweep) on a synthetic field of this library's generator,
and keeps the fastest pair in a JSON cache keyed by the device name, its SM
count, N and the radius count.  For batches of boxes it also picks the number
of streams by timing the whole captured batch.

    from prc_d2z import autotune
    B, v = autotune.tuned(512, 64)          # cached or measured now
    ctx.tune(B, v)

The cache lives at $PRC_D2Z_TUNE_CACHE, else ~/.cache/prc_d2z/tune.json.
Results do not depend on the choice beyond the float rounding of the
transforms (the tests check every variant against the default).
"""
from __future__ import annotations

import json
import os
import statistics

import numpy as np

from . import CLParameters, Delta2Zreion, Parameters, compute_tables, fields, win_variants

__all__ = ["tuned", "tune", "tune_batch_streams", "cache_path", "candidates"]


def cache_path() -> str:
    p = os.environ.get("PRC_D2Z_TUNE_CACHE")
    return p or os.path.join(os.path.expanduser("~"), ".cache", "prc_d2z", "tune.json")


def _device_key() -> str:
    import torch
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{props.name}|sm{props.multi_processor_count}"


def _load(path):
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _save(path, data):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def candidates(N: int, n_radii: int):
    """(radius batches, window variants) tried for a grid side N."""
    # radius slots up to 60 GB (a slot is N^2 (N/2 + 2) complex64: 0.54 GB at
    # 512, 1.8 GB at 768, 4.3 GB at 1024), so at most 64, 32 and 12 radii
    slot = N * N * (N // 2 + 2) * 8
    batches = sorted({min(b, n_radii) for b in (4, 8, 12, 16, 24, 32, 48, 64) if b * slot <= 60e9})
    return batches, list(range(win_variants(N)))


def _time_forward(ctx, delta, z, reps: int) -> float:
    import torch
    ctx.forward(delta, zreion=z, want_argmax=False)
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ctx.forward(delta, zreion=z, want_argmax=False)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def tune(N: int, n_radii: int, reps: int = 5, force: bool = False, path: str | None = None) -> dict:
    """Measure (or read from the cache) the fastest radius batch and window
    variant for N and n_radii; returns the cache entry."""
    import torch
    path = path or cache_path()
    data = _load(path)
    key = f"{_device_key()}|N={N}|nr={n_radii}"
    if key in data and not force:
        return data[key]
    box = 1.5 * N
    p = Parameters(N=N, Nscales=n_radii, BoxSize=box)
    cl = CLParameters(Rmax=min(60.0, 0.4 * box), zeta=80.0, M_min=1e9 / 0.68)
    t = compute_tables(p, cl)
    batches, variants = candidates(N, n_radii)
    delta = fields.gaussian_field(N, box, seed=1, backend="native")
    z = torch.empty_like(delta)
    # rounds over all candidates (not one candidate after another), so that a
    # slow drift of the clocks under sustained load biases none of them
    samples = {}
    with Delta2Zreion(N, float(np.float32(box) / np.float32(p.h)), t.radii_mpc, t.barrier_b, t.barrier_a, t.DInit,
                      radius_batch=max(batches), argmax=False) as ctx:
        for _ in range(reps):
            for B in batches:
                for v in variants:
                    ctx.tune(B, v)
                    samples.setdefault(f"B{B}_v{v}", []).append(_time_forward(ctx, delta, z, 1))
    times = {k: statistics.median(v) for k, v in samples.items()}
    # within 0.3% of the fastest (the spread of repeated steps) the larger
    # radius batch wins: it reads the spectrum and zreion fewer times
    fastest = min(times.values())
    near = [k for k in times if times[k] <= fastest * 1.003]
    best = max(near, key=lambda k: (int(k.split("_")[0][1:]), -times[k]))
    B, v = (int(x[1:]) for x in best.split("_"))
    entry = {"radius_batch": B, "win_variant": v, "ms": times[best], "times_ms": times}
    data = _load(path)
    data[key] = entry
    _save(path, data)
    return entry


def tuned(N: int, n_radii: int, **kw):
    """(radius batch, window variant) for N and n_radii, tuning on first use."""
    e = tune(N, n_radii, **kw)
    return e["radius_batch"], e["win_variant"]


def tune_batch_streams(make_batch, run, streams=(1, 2, 4), reps: int = 3):
    """Time run(batch) for batches made by make_batch(n_streams); returns
    (best n_streams, {n_streams: ms}).  The batches are closed afterwards."""
    import torch
    times = {}
    for s in streams:
        b = make_batch(s)
        try:
            run(b)
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                run(b)
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            times[s] = statistics.median(ts)
        finally:
            b.close()
    return min(times, key=times.get), times
