"""Benchmark of the delta2zreion step on GB300 (one JSON line on stdout).

Workload (the 512^3 plain configuration): a float32 linear density field at
z = 0 in a periodic 600 Mpc/h box, N = 512, from Philox4x32-10 white noise
(seed 1 + rank) shaped by a BBKS P(k) (n_s 0.965, Omega_m 0.31, h 0.68,
sigma_8 0.81); 64 log-spaced top-hat radii from 2 cells to 60 Mpc/h;
M_min = 1e9 Msun/h; zeta calibrated so the ionisation midpoint is z ~ 8.
A step is one delta2zreion pass: the forward R2C of delta_lin and all 64
radii (window, C2R, barrier, running max) into zreion.

  value : cell*radii/s with delta_lin resident in HBM (CUDA events over K steps)
  e2e   : the same through the public API with host (pinned) buffers: each step
          copies delta_lin in and zreion out inside the timed region
          (prc_d2z_forward_many: box i+1's input and box i-1's output move on
          the copy engines while box i computes; the median of three streams
          of K boxes; single_call_value: K separate prc_d2z_forward calls)
Multi-GPU (torchrun): replicas, one box per rank, no collective on the data
path; value = all ranks' cell*radii / max-over-ranks time.

The default line also carries the rest of the headline metric, each timed
with CUDA events under its own clock record: "adjoint" (backward / forward
time at 256^3 x 64, loss mean((z - z_t)^2)), "batched" (96 boxes of
64..256^3 in one captured launch against a per-box loop of the plain path,
bit-identity checked) and "step_frac" (the whole step's rate on the kernels'
own algorithmic bytes, on the compulsory floor and on the canonical 3-pass
model, each against the measured HBM copy rate).  "batched" also carries
"small_boxes": 96 boxes of 64^3, where the per-box loop is bound by launches
and tails rather than by the kernels.

--impl reference times the CPU implementation of the same step (the oracle's
faithful-fp32 restatement: scipy.fft with all host threads plus the OpenMP
C loops of oracle/d2z_cells.c): every step is a whole step, all radii, while
the K steps fit in REF_BUDGET_S seconds of CPU time; beyond that each step is
the forward R2C plus an evenly spread sample of the radii, scaled to all of
them (the cost per radius does not depend on the radius), and the line says
which.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "pr-calc_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "zreion cell*radii/s at 512^3 (64 radii)"
UNIT = "cell*radii/s"
N_DEF, BOX, NR, RMIN_CELLS, RMAX, H_ = 512, 600.0, 64, 2.0, 60.0, 0.68
MMIN_MSUN = 1e9 / H_
# zeta from prc_d2z.calibrate: raw zreion with x_i(z=8) = 0.5 at seed 1
ZETA = 80.5404       # 512^3, 600 Mpc/h, 64 radii to 60 Mpc/h
ZETA_BATCH = 81.6855 # 256^3, 384 Mpc/h (1.5 Mpc/h cells), 48 radii to 60 Mpc/h
REF_BUDGET_S = 600.0 # reference arm: CPU seconds for the K timed steps (whole steps at K = 20)
# plain configurations: N, box [Mpc/h], radii, calibrated zeta (x_i(z=8) = 0.5 at seed 1)
CONFIGS = {"C1": (128, 200.0, 32, 82.4429), "C2": (512, 600.0, 64, 80.5404), "C3": (1024, 1200.0, 96, 73.1587)}


def _use_config(name):
    """Select a plain configuration (C2, 512^3 x 64, is the default workload)."""
    global N_DEF, BOX, NR, ZETA, METRIC
    N_DEF, BOX, NR, ZETA = CONFIGS[name]
    METRIC = f"zreion cell*radii/s at {N_DEF}^3 ({NR} radii)"


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _params(N):
    import prc_d2z
    p = prc_d2z.Parameters(N=N, Nscales=NR, BoxSize=BOX * N / N_DEF if N != N_DEF else BOX, Rmin=RMIN_CELLS)
    cl = prc_d2z.CLParameters(Rmax=RMAX, zeta=ZETA, M_min=MMIN_MSUN)
    return p, cl


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons, watts = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            try:
                watts.append(float(f[3]))
            except ValueError:
                pass
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w": round(statistics.median(watts), 1) if watts else None}


def _config(N, box):
    """The workload keys, identical in both arms' lines."""
    return {"workload": f"plain delta2zreion {N}^3, {box:g} Mpc/h, {NR} radii", "N": N, "radii": NR,
            "box_mpc_h": box, "zeta": ZETA, "l2": "inputs larger than L2 (no flush)"}


def _algo_bytes(kind, N, nb, first):
    """Algorithmic DRAM bytes of one launch (what the kernel must read + write)."""
    Nc = N * N * (N // 2 + 1)
    n3 = N ** 3
    if kind == "win_x":            # spectrum once, nb slot outputs
        return 8 * Nc + 8 * Nc * nb
    if kind == "col_inv":          # nb slots read + written
        return 16 * Nc * nb
    if kind == "c2r_z":            # nb slots read, zreion written (+ read after the first sweep)
        return 8 * Nc * nb + (4 if first else 8) * n3
    if kind == "r2c_z":
        return 4 * n3 + 8 * Nc
    if kind == "col_fwd":
        return 16 * Nc
    return None


def _traffic(kind, N):
    """DRAM bytes per launch from the committed ncu summary, or None."""
    path = os.path.join(REPO, "profiles", f"{kind}_n{N}.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def _step_bytes(N, B):
    """Algorithmic bytes of one whole step as these kernels move them: the
    forward R2C (z pass, two column passes), then per sweep of up to B radii
    the window + x pass, the y pass and the z pass with the running max."""
    Nc = N * N * (N // 2 + 1)
    tot = _algo_bytes("r2c_z", N, 1, True) + 2 * _algo_bytes("col_fwd", N, 1, True)
    for s, r0 in enumerate(range(0, NR, B)):
        nb = min(B, NR - r0)
        tot += sum(_algo_bytes(k, N, nb, s == 0) for k in ("win_x", "col_inv", "c2r_z"))
    return tot, NR * (8 * Nc + 8 * N ** 3), NR * (40 * Nc + 8 * N ** 3) + 4 * N ** 3 + 40 * Nc


def cpu_sample(delta_np, tables, box_mpc, n_radii_sample, threads):
    """Oracle (faithful fp32): forward + n radii (all NR: one whole step);
    returns the full-workload cell*radii/s and the timings."""
    from oracle import d2z_ref as orc
    orc.lib().orc_set_threads(threads)
    N = delta_np.shape[0]
    t0 = time.perf_counter()
    spec = orc.forward_spectrum(delta_np, tables.DInit, "fp32")
    t1 = time.perf_counter()
    zreion = np.zeros(delta_np.shape, np.float32)
    idx = np.linspace(0, NR - 1, n_radii_sample).round().astype(int)
    for r in idx:
        W = orc.window(N, box_mpc, tables.radii_mpc[r], "fp32")
        dR = orc.smooth(spec, W, N, "fp32")
        orc.barrier_update(dR, tables.barrier_a, tables.barrier_b[r], int(r), zreion, None, "fp32")
    t2 = time.perf_counter()
    t_fwd, t_rad = t1 - t0, (t2 - t1) / len(idx)
    t_full = t_fwd + NR * t_rad
    return N ** 3 * NR / t_full, t_fwd, t_rad


def run_reference(args, rank):
    """CPU implementation of the path on the host cores (rank 0 only)."""
    if rank != 0:
        return
    import prc_d2z  # noqa: F401  (tables only; the oracle does the grid work)
    from oracle import d2z_ref as orc
    from prc_d2z import fields
    N = args.n
    threads = os.cpu_count() or 1
    p, cl = _params(N)
    op = orc.Parameters(N=N, Nscales=NR, BoxSize=p.BoxSize, Rmin=RMIN_CELLS, Rmax=RMAX, zeta=ZETA, M_min=MMIN_MSUN)
    tables = orc.tables(op)

    class T:  # adapter with the field names cpu_sample uses
        DInit, radii_mpc, barrier_a, barrier_b = tables.DInit, tables.R, tables.A, tables.B

    delta = fields.gaussian_field(N, p.BoxSize, seed=1)
    box_mpc = float(np.float32(p.BoxSize) / np.float32(H_))
    vals = []
    warm = None
    for s in range(max(1, args.warmup)):  # warm-up: the FFT plans, thread pools and caches (not timed)
        warm = cpu_sample(delta, T, box_mpc, 2, threads)
    # radii per step: all of them (whole steps) while K whole steps fit in
    # REF_BUDGET_S, else as many as fit, evenly spread over the radius grid
    nr_s = args.ref_radii
    if nr_s <= 0:
        t_fwd, t_rad = warm[1], warm[2]
        fit = int((REF_BUDGET_S / max(1, args.steps) - t_fwd) / max(t_rad, 1e-9))
        nr_s = max(2, min(NR, fit))
    nr_s = min(nr_s, NR)
    for s in range(args.steps):
        vals.append(cpu_sample(delta, T, box_mpc, nr_s, threads))
    v = statistics.median(x[0] for x in vals)
    ms = N ** 3 * NR / v * 1e3
    if nr_s >= NR:
        sample = (f"whole steps: forward R2C + all {NR} radii at {N}^3 "
                  f"(t_fwd {statistics.median(x[1] for x in vals):.2f} s, "
                  f"t_radius {statistics.median(x[2] for x in vals):.3f} s)")
    else:
        sample = (f"forward R2C + {nr_s} of {NR} radii per step at {N}^3, extrapolated to all {NR} radii "
                  f"(t_fwd {statistics.median(x[1] for x in vals):.2f} s, "
                  f"t_radius {statistics.median(x[2] for x in vals):.3f} s)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (Philox4x32-10 + BBKS, seed 1)",
        "config": _config(N, p.BoxSize), "parallelism": f"{threads} host threads",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch

    import prc_d2z
    from prc_d2z import fields
    from prc_d2z.parallel import max_over_ranks
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    N = args.n
    p, cl = _params(N)
    tuned = None
    if args.batch == 0:
        # radius batch and window-pass variant from the autotuner (cached per device)
        from prc_d2z import autotune
        tuned = autotune.tuned(N, NR)
    B_use = tuned[0] if tuned else args.batch
    ctx = prc_d2z.Delta2Zreion.from_parameters(p, cl, radius_batch=B_use, argmax=False)
    if tuned:
        ctx.tune(0, tuned[1])
    t = ctx.tables
    delta = fields.gaussian_field(N, p.BoxSize, seed=1 + rank, backend="torch", device=dev).contiguous()
    zreion = torch.empty_like(delta)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        ctx.forward(delta, zreion=zreion, want_argmax=False)
    ctx.profile(True)
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local_rank) as clk:
        ev0.record()
        for _ in range(args.steps):
            ctx.forward(delta, zreion=zreion, want_argmax=False)
        ev1.record()
        torch.cuda.synchronize()
    barrier()
    ms_total = ev0.elapsed_time(ev1)
    prof = ctx.profile_read()
    ctx.profile(False)
    launches = ctx.last_launches() * args.steps
    ms_total = max_over_ranks(ms_total, device=dev)
    ms_step = ms_total / args.steps
    value = world * N ** 3 * NR / (ms_step * 1e-3)

    # end to end through the public API with pinned host buffers.  Headline: a
    # stream of K boxes through prc_d2z_forward_many (every step copies its
    # delta_lin in and its zreion out; the copy engines move box i+1's input
    # and box i-1's output while box i's kernels run).  Also reported: K
    # separate prc_d2z_forward calls (each copy on the critical path).
    h_delta = torch.empty(delta.shape, dtype=torch.float32, pin_memory=True)
    h_delta.copy_(delta.cpu())
    h_z = [torch.empty(delta.shape, dtype=torch.float32, pin_memory=True) for _ in range(2)]
    hd, hz = h_delta.numpy(), [h.numpy() for h in h_z]
    for _ in range(max(1, args.warmup // 2)):
        ctx.forward(hd, zreion=hz[0], want_argmax=False)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.forward(hd, zreion=hz[0], want_argmax=False)
    torch.cuda.synchronize()
    single_s = max_over_ranks(time.perf_counter() - t0, device=dev)
    e2e_single = world * N ** 3 * NR * args.steps / single_s
    # the copy engines' rate on this machine, for reading the pipelined number
    scratch = torch.empty_like(delta)
    copy_gbs = {}
    for kind, dst, src in (("h2d", scratch, h_delta), ("d2h", h_z[1], scratch)):
        dst.copy_(src, non_blocking=True)
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record()
        dst.copy_(src, non_blocking=True)
        c1.record()
        c1.synchronize()
        copy_gbs[kind] = 4 * N ** 3 / (c0.elapsed_time(c1) * 1e6)
    del scratch
    ctx.forward_many([hd, hd], hz)
    # three streams of K boxes, the median reported: the pipelined rate
    # varies from run to run on a shared machine (28.3 to 34.0 ms a box for
    # the same build, the device-resident step taking 28.2-28.4 ms); clocks
    # and power are sampled over the three
    e2e_reps = []
    with Clocks(local_rank) as clk_e2e:
        for _ in range(3):
            barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.forward_many([hd] * args.steps, [hz[i % 2] for i in range(args.steps)])
            torch.cuda.synchronize()
            e2e_reps.append(max_over_ranks(time.perf_counter() - t0, device=dev))
    e2e_s = statistics.median(e2e_reps)
    e2e = world * N ** 3 * NR * args.steps / e2e_s

    if rank != 0:
        return
    # roofline of the dominant kernel
    peak, peak_kind = _peaks()
    B = min(B_use, NR)
    sweeps = math.ceil(NR / B)
    dom = max((k for k in prof if prof[k][1] > 0), key=lambda k: prof[k][0])
    tot_ms, n_l = prof[dom]
    per_launch_ms = tot_ms / n_l
    if dom in ("win_x", "col_inv", "c2r_z"):
        # average over sweeps: every sweep but possibly the last has B radii
        byts = [_algo_bytes(dom, N, min(B, NR - s * B), s == 0) for s in range(sweeps)]
        bytes_launch = sum(byts) / len(byts)
    else:
        bytes_launch = _algo_bytes(dom, N, 1, True) or 0
    achieved = bytes_launch / (per_launch_ms * 1e-3) / 1e9
    traffic = _traffic(dom, N)
    if traffic is not None and dom in ("win_x", "col_inv", "c2r_z"):
        # the committed summaries are for a radius batch of 8: scale by the units processed
        s8 = math.ceil(NR / 8)
        b8 = sum(_algo_bytes(dom, N, min(8, NR - s * 8), s == 0) for s in range(s8)) / s8
        traffic *= bytes_launch / b8
    rl = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
          "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
          "bytes_per_launch": bytes_launch, "ms_per_launch": per_launch_ms,
          "kernel_share": {k: v[0] / sum(x[0] for x in prof.values()) for k, v in prof.items() if v[1]}}
    # the whole step against the measured copy rate, on three byte counts: the
    # kernels' own algorithmic bytes, the compulsory floor (read the spectrum
    # and write the cells once per radius) and the canonical 3-pass model
    # (40 Nc + 8 N^3 per radius, 4 N^3 + 40 Nc once)
    own, floor, canon = _step_bytes(N, B)
    step_s = ms_step * 1e-3
    step_frac = {"own_bytes": own, "own_gbs": own / step_s / 1e9, "own_frac": own / step_s / 1e9 / peak,
                 "floor_bytes": floor, "floor_gbs": floor / step_s / 1e9, "floor_frac": floor / step_s / 1e9 / peak,
                 "canonical_bytes": canon, "canonical_gbs": canon / step_s / 1e9,
                 "canonical_frac": canon / step_s / 1e9 / peak, "peak_gbs": peak, "peak_source": peak_kind}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (Philox4x32-10 + BBKS, seed 1+rank)",
        "config": _config(N, p.BoxSize), "parallelism": f"replicas x{world}",
        "tuning": {"radius_batch": B, "win_variant": tuned[1] if tuned else 0, "autotuned": tuned is not None},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 4 * N ** 3, "d2h_bytes_per_step": 4 * N ** 3,
                "api": "prc_d2z_forward_many (K boxes, pinned host buffers, copies overlapped; median of 3 runs)",
                "runs_ms_per_box": [round(t / args.steps * 1e3, 3) for t in e2e_reps], "clocks": clk_e2e.summary(),
                "single_call_value": e2e_single, "copy_engine_gbs": copy_gbs},
        "gpu_launches": launches,
        "roofline": rl,
        "step_frac": step_frac,
        "clocks": clk.summary(),
    }
    ctx.close()
    del zreion, h_delta, h_z, hd, hz
    torch.cuda.empty_cache()
    if world == 1 and not args.no_extras:
        # the metric's other two parts, each under its own clock record
        out["adjoint"] = adjoint_measure(256, steps=5, warmup=3)
        out["batched"] = batched_measure(steps=5, warmup=3, streams=0)
        # north star (b): small boxes batched against the per-box loop
        sb = batched_measure(steps=5, warmup=3, streams=0, small_only=True)
        out["batched"]["small_boxes"] = {k: sb[k] for k in ("workload", "ms_per_step", "value", "per_box_loop",
                                                            "per_box_graph", "speedup_vs_loop",
                                                            "identical_to_loop", "gpu_launches", "clocks")}
    if world == 1 and not args.no_cpu:
        from oracle import d2z_ref as orc  # noqa: F401
        threads = os.cpu_count() or 1
        d_np = delta.cpu().numpy()

        class T:
            DInit, radii_mpc, barrier_a, barrier_b = t.DInit, t.radii_mpc, t.barrier_a, t.barrier_b

        v, tf, tr = cpu_sample(d_np, T, float(np.float32(p.BoxSize) / np.float32(H_)), NR, threads)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"oracle fp32, one whole step: forward R2C ({tf:.2f} s) + all {NR} radii "
                                         f"({tr:.3f} s each) at {N}^3"}
    print(json.dumps(out), flush=True)


def _cfg_box(N, nr, seed, zeta, box=None, rmax=RMAX):
    import prc_d2z
    box = box if box is not None else 1.5 * N
    p = prc_d2z.Parameters(N=N, Nscales=nr, BoxSize=box, Rmin=RMIN_CELLS)
    cl = prc_d2z.CLParameters(Rmax=rmax, zeta=zeta, M_min=MMIN_MSUN)
    t = prc_d2z.compute_tables(p, cl)
    return dict(N=N, box_mpc=float(np.float32(box) / np.float32(H_)), radii_mpc=t.radii_mpc,
                barrier_b=t.barrier_b, barrier_a=t.barrier_a, growth_init=t.DInit), box


def batched_measure(steps, warmup, streams, small_only=False):
    """96 realisations, grids 64/96/128/192/256 at 1.5 Mpc/h cells, 24-48 radii
    each (small_only: 96 boxes of 64^3), seeds 1000..1095: a per-box loop of
    the plain path, the same launches captured in one graph, and grouped
    launches (one launch per pass and grid size).  Every box sweeps all its
    radii at once (radius batch = its radius count: one read of its spectrum
    and one write of its zreion, the fastest batch at every size) with the
    autotuned window-pass variant of its grid size; each batch mode picks its
    stream count by timing.  The modes run one after another, each freeing its
    workspaces before the next.  Returns a dict (times, speed-ups,
    bit-identity, clocks)."""
    import torch

    import prc_d2z
    from prc_d2z import autotune, fields
    rng = np.random.default_rng(2024)
    sizes = [64] * 96 if small_only else [64] * 20 + [96] * 19 + [128] * 19 + [192] * 19 + [256] * 19
    rng.shuffle(sizes)
    nrs = rng.integers(24, 49, len(sizes))
    boxes, deltas = [], []
    for i, (N, nr) in enumerate(zip(sizes, nrs)):
        b, box = _cfg_box(int(N), int(nr), 1000 + i, ZETA_BATCH)
        b["radius_batch"] = int(nr)
        boxes.append(b)
        deltas.append(fields.gaussian_field(int(N), box, seed=1000 + i, backend="torch").contiguous())
    work = sum(b["N"] ** 3 * len(b["radii_mpc"]) for b in boxes)
    nr_rep = int(np.median(nrs))
    variant = {int(N): autotune.tuned(int(N), nr_rep)[1] for N in sorted(set(sizes))}

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with Clocks(torch.cuda.current_device()) as clk:
            e0.record()
            for _ in range(steps):
                fn()
            e1.record()
            torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, clk.summary()

    # the plain per-box loop
    outs_loop = [torch.empty_like(d) for d in deltas]
    ctxs = [prc_d2z.Delta2Zreion(b["N"], b["box_mpc"], b["radii_mpc"], b["barrier_b"], b["barrier_a"],
                                 b["growth_init"], radius_batch=b["radius_batch"], argmax=False) for b in boxes]
    for c, b in zip(ctxs, boxes):
        c.tune(0, variant[b["N"]])

    def loop():
        for c, d, o in zip(ctxs, deltas, outs_loop):
            c.forward(d, zreion=o, want_argmax=False)

    ms_loop, clk_loop = timed(loop)
    for c in ctxs:
        c.close()
    del ctxs
    torch.cuda.empty_cache()

    def make_batch(n_streams):
        bt = prc_d2z.Batch(boxes, n_streams=n_streams)
        for i, b in enumerate(boxes):
            bt.tune(i, 0, variant[b["N"]])
        return bt

    res = {}
    for mode, choices in (("graph", (1, 2, 4)), ("grouped", (1, 2, 3, 5))):
        outs = [torch.empty_like(d) for d in deltas]

        def run(bt, mode=mode, outs=outs):
            bt.forward(deltas, outs, mode=mode)

        ns, ns_ms = streams, None
        if streams <= 0:
            ns, ns_ms = autotune.tune_batch_streams(make_batch, run, streams=choices)
        bt = make_batch(ns)
        ms, clk = timed(lambda: run(bt))
        res[mode] = {"ms_per_step": ms, "value": work / (ms * 1e-3), "streams": ns, "streams_ms": ns_ms,
                     "identical_to_loop": all(torch.equal(a, o) for a, o in zip(outs_loop, outs)),
                     "gpu_launches": bt.launches(), "clocks": clk}
        bt.close()
        del outs
        torch.cuda.empty_cache()
    g = res["grouped"]
    mix = "N = 64 (96 boxes)" if small_only else "N in {64,96,128,192,256} (20/19/19/19/19)"
    out = {"workload": f"96 boxes, {mix}, 1.5 Mpc/h cells, radii U{{24..48}} from 2 cells to 60 Mpc/h",
           "zeta": ZETA_BATCH,
           "mode": "grouped: one launch per pass over all boxes of a grid size, sizes side by side, one graph",
           "radius_batch": "each box's radius count (one sweep per box)",
           "steps": steps, "warmup": warmup, "ms_per_step": g["ms_per_step"], "value": g["value"], "unit": UNIT,
           "per_box_loop": {"ms_per_step": ms_loop, "value": work / (ms_loop * 1e-3), "clocks": clk_loop},
           "per_box_graph": res["graph"], "grouped": g,
           "speedup_vs_loop": ms_loop / g["ms_per_step"], "identical_to_loop": g["identical_to_loop"],
           "win_variant": {str(N): v for N, v in variant.items()},
           "gpu_launches": g["gpu_launches"], "clocks": g["clocks"]}
    del deltas, outs_loop
    torch.cuda.empty_cache()
    return out


def run_batched(args):
    r = batched_measure(args.steps, args.warmup, args.streams)
    print(json.dumps({
        "metric": "batched zreion cell*radii/s (96 boxes, 64-256^3, 24-48 radii)", "value": r["value"],
        "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (Philox4x32-10 + BBKS, seeds 1000..1095)",
        "config": {"workload": "batched: " + r["workload"], "zeta": ZETA_BATCH},
        "mode": r["mode"], "radius_batch": r["radius_batch"], "per_box_loop": r["per_box_loop"],
        "per_box_graph": r["per_box_graph"], "speedup_vs_loop": r["speedup_vs_loop"],
        "identical_to_loop": r["identical_to_loop"], "win_variant": r["win_variant"],
        "gpu_launches": r["gpu_launches"], "clocks": r["clocks"]}), flush=True)


def adjoint_measure(N, steps, warmup, batch=0):
    """Adjoint at N^3 with 64 radii and the 512^3 workload's cell size:
    loss = mean((z - z_t)^2), z_t from seed 2; forward (with argmax) and
    backward timed with CUDA events; returns a dict with t_bwd / t_fwd."""
    import torch

    import prc_d2z
    from prc_d2z import fields
    box = 600.0 * N / 512
    nr, zeta = 64, CONFIGS["C2"][3]
    p = prc_d2z.Parameters(N=N, Nscales=nr, BoxSize=box, Rmin=RMIN_CELLS)
    cl = prc_d2z.CLParameters(Rmax=RMAX, zeta=zeta, M_min=MMIN_MSUN)
    ctx = prc_d2z.Delta2Zreion.from_parameters(p, cl, radius_batch=batch, argmax=True)
    delta = fields.gaussian_field(N, box, seed=1, backend="torch").contiguous()
    target = fields.gaussian_field(N, box, seed=2, backend="torch").contiguous()
    zt, _, _ = ctx.forward(target, want_argmax=False)
    zt = zt.clone()
    z = torch.empty_like(delta)
    am = torch.empty(delta.shape, dtype=torch.uint8, device=delta.device)
    grad = torch.empty_like(delta)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for _ in range(warmup):
        ctx.forward(delta, zreion=z, argmax=am)
        g = (2.0 / N ** 3) * (z - zt)
        ctx.backward(g, am, dL_ddelta=grad)
    torch.cuda.synchronize()
    tf = tb = 0.0
    with Clocks(torch.cuda.current_device()) as clk:
        for _ in range(steps):
            ev[0].record()
            ctx.forward(delta, zreion=z, argmax=am)
            ev[1].record()
            g = (2.0 / N ** 3) * (z - zt)
            ev[2].record()
            ctx.backward(g, am, dL_ddelta=grad)
            ev[3].record()
            torch.cuda.synchronize()
            tf += ev[0].elapsed_time(ev[1])
            tb += ev[2].elapsed_time(ev[3])
    tf /= steps
    tb /= steps
    ctx.close()
    del delta, target, zt, z, am, grad
    torch.cuda.empty_cache()
    return {"workload": f"adjoint {N}^3, {box:g} Mpc/h, 64 radii, loss mean((z-z_t)^2)", "N": N,
            "ratio": tb / tf, "forward_ms": tf, "backward_ms": tb, "steps": steps, "warmup": warmup,
            "backward_cell_radii_per_s": N ** 3 * nr / (tb * 1e-3), "clocks": clk.summary()}


def run_adjoint(args):
    r = adjoint_measure(args.n, args.steps, args.warmup, args.batch)
    print(json.dumps({
        "metric": f"adjoint/forward time ratio at {args.n}^3 (64 radii)", "value": r["ratio"], "unit": "ratio",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["forward_ms"] + r["backward_ms"],
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (Philox4x32-10 + BBKS, field seed 1, target seed 2)",
        "config": {"workload": r["workload"], "zeta": CONFIGS["C2"][3]},
        "forward_ms": r["forward_ms"], "backward_ms": r["backward_ms"],
        "backward_cell_radii_per_s": r["backward_cell_radii_per_s"], "clocks": r["clocks"]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="C2", choices=sorted(CONFIGS))
    ap.add_argument("--n", type=int, default=0, help="grid side (default: the config's; keeps its cell size)")
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--ref-radii", type=int, default=0,
                    help="reference arm: radii per step (0: all of them, a whole step, while the K steps fit in "
                         f"{REF_BUDGET_S:g} s; else as many as fit)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="default line without the adjoint and batched parts")
    ap.add_argument("--workload", default="plain", choices=["plain", "batched", "adjoint"])
    ap.add_argument("--streams", type=int, default=0, help="batched: streams (0: autotuned)")
    args = ap.parse_args()
    _use_config(args.config)
    if args.n == 0:
        args.n = N_DEF
    elif args.n != N_DEF:
        global METRIC
        METRIC = f"zreion cell*radii/s at {args.n}^3 ({NR} radii)"
    if args.workload == "batched" and args.impl == "ours":
        run_batched(args)
        return
    if args.workload == "adjoint" and args.impl == "ours":
        run_adjoint(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
