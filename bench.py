"""Benchmark of the FDTD time-stepping path: Yee cell-steps per second on the 512^3 plain-method
workload (thin-wire dipole with a 50-ohm pulsed feed among 5% random dielectric blocks, 16-cell
absorber, port series recorded every step, far-field DFT at 32 frequencies on a box 20 cells
inside the absorber), with the HBM roofline of the fused Yee kernel and the CPU restatement's
throughput beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--size 512]

One JSON line on rank 0. A step is one leapfrog step (B, E, sources) plus the per-step monitors,
over the whole grid. Inputs (6.4 GB of field state) are far larger than L2 (129 MB), so no flush
is needed between steps. Multi-GPU runs are replicas: each rank steps its own copy of the scene
(weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

BYTES_PER_CELL_STEP = 60  # E and B read + write in FP32 (48 B) + six binary16 edge materials (12 B)
METRIC = "Yee Mcells/s (cell-steps per second, 1e6)"


def _rank_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                self.out = ""

    def summary(self):
        rows = []
        for line in (getattr(self, "out", "") or "").splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def replica_throughput(cells_done: float, elapsed_s: float, dist=None, device=None):
    """Whole-job throughput of independent replicas: the cell-steps every rank processed, divided by
    the slowest rank's time (max over ranks). Returns (Mcells/s, max elapsed seconds)."""
    if dist is None:
        return cells_done / elapsed_s / 1e6, elapsed_s
    import torch
    t = torch.tensor([elapsed_s], dtype=torch.float64, device=device)
    c = torch.tensor([cells_done], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(c.item()) / float(t.item()) / 1e6, float(t.item())


def build_scene(args):
    from em_lab_gb300 import configs
    if args.workload == "plain_small":
        return configs.plain_small(steps=args.steps)
    return configs.plain_large(steps=args.steps, size=args.size)


def workload_text(args, sc, dft_points=None):
    n = "x".join(str(v) for v in sc.grid.size)
    if args.workload == "plain_small":
        return (f"plain_small {n}, 10-cell absorber, vacuum, glass sphere eps 2.25 r 10, z point dipole "
                f"CW lambda 16 amplitude 7 with 3-period ramp, far-field monitor at one frequency "
                f"(two-stage running average, every step)")
    text = (f"plain_large {n}, 16-cell absorber, thin-wire half-wave dipole with a 50-ohm Gaussian-pulse "
            f"feed, 5% seeded random dielectric blocks, port series recorded every step")
    if dft_points is not None:
        text += (f", far-field DFT at {DFT_FREQS} frequencies on a box {DFT_MARGIN} cells inside the absorber "
                 f"({dft_points} nodes)")
    return text


def attach_monitors(grid, sc, args):
    """Per-step monitors of the workload. Returns the DFT node count (None without the DFT)."""
    if sc.ports:
        grid.ports_configure([p.to_c() for p in sc.ports], sc.ports[0].wavelength, 4.0, sweep=True)
    if args.workload == "plain_small":
        ff = sc.far_field
        grid.ntff_configure(ff["box_min"], ff["box_max"], ff["wavelength"], ff["averaging"])
        return None
    _, points = dft_setup(grid, sc)
    return points


def frame_reads(sc):
    """The headless frame loop's reads: the probe neighbourhood and the six planes of the flux box."""
    from em_lab_gb300 import abi
    if sc.probes:
        probe = [tuple(int(v) - 1 for v in sc.probes[0][1])]
    else:
        probe = [(int(sc.grid.nx * 0.25), sc.grid.ny // 2, sc.grid.nz // 2)]
    if sc.fluxes:
        bmin, bmax = sc.fluxes[0].box_min, sc.fluxes[0].box_max
    else:
        c = [v // 2 for v in sc.grid.size]
        bmin, bmax = [v - 12 for v in c], [v + 12 for v in c]
    planes = []
    for ax in range(3):
        u, v = (1, 2) if ax == 0 else ((0, 2) if ax == 1 else (0, 1))
        for idx in (bmin[ax], bmax[ax]):
            planes.append(abi.FluxPlane(ax, idx, (bmin[u], bmin[v]), (bmax[u] + 1, bmax[v] + 1)))
    return probe, planes, bmin, bmax


def load_grid(grid, sc):
    m = sc.materials
    grid.upload_materials(m.sigma, m.epsilon_r, sc.edges, sc.wires)
    grid.set_sources(sc.sources)


DFT_FREQS = 32      # far-field spectrum: 32 frequencies over 0.3-1.7 x the design frequency
SWEEP_POINTS = 128  # port Z / S11 sweep points
DFT_MARGIN = 20     # Huygens box this many cells inside the absorber


def dft_setup(grid, sc):
    """Far-field DFT box 20 cells inside the absorber at 32 frequencies covering 0.3-1.7 f0."""
    L = sc.grid.pml_thickness
    lo = [L + DFT_MARGIN] * 3
    hi = [n - L - DFT_MARGIN - 1 for n in sc.grid.size]
    wl0 = sc.ports[0].wavelength
    wls = [wl0 / f for f in np.linspace(0.3, 1.7, DFT_FREQS)]
    grid.ntff_dft_configure(lo, hi, wls)
    points, _ = grid.ntff_dft_info()
    return wls, points


def kernel_name(kernel: str, tiling: int) -> str:
    if kernel == "fused":
        return "yee_tma2" if tiling in (0, 32, 64, 128) else "yee_tma"
    return {"fused_ldg": "yee_fused", "split": "yee_split_b+yee_split_e"}[kernel]


def read_traffic(key: str):
    """DRAM bytes per launch of the stencil kernel from an ncu capture, kept in profiles/traffic.txt
    as lines `<kernel>_<size> <bytes per launch>`."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            parts = line.split("#")[0].split()
            if len(parts) == 2 and parts[0] == key:
                return float(parts[1])
    return None


def cpu_sample(sc, seconds_budget: float = 20.0, max_steps: int = 8, dft: bool = False):
    """The FP32 CPU restatement on every host thread, over the full grid, for a few steps, with the
    same per-step monitors as the GPU arm (port series; the 32-frequency far-field DFT if `dft`)."""
    import oracle
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    o = oracle.Oracle(sc.grid, "f32")
    t0 = time.perf_counter()
    oracle.load_scene(o, sc)
    if sc.ports:
        o.ports_configure([p.to_c() for p in sc.ports], sc.ports[0].wavelength, 4.0, sweep=True)
    if dft:
        dft_setup(o, sc)
    setup = time.perf_counter() - t0
    cells = float(np.prod(sc.grid.size))
    o.step(1)  # warm-up (first touch of every page)
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps:
        o.step(1)
        steps += 1
        if time.perf_counter() - t0 > seconds_budget:
            break
    el = time.perf_counter() - t0
    o.close()
    return {"value": cells * steps / el / 1e6, "unit": "Mcells/s", "cores": threads, "kind": "port",
            "sample": f"{steps} full-grid steps (B, E, sources{', port monitor' if sc.ports else ''}"
                      f"{', 32-frequency far-field DFT' if dft else ''}) of the "
                      f"{'x'.join(str(v) for v in sc.grid.size)} workload after 1 warm-up step "
                      f"(oracle/emlab_oracle.c FP32, OpenMP {threads} threads, set-up {setup:.1f} s excluded)"}


COMPONENTS = ("Ex", "Ey", "Ez", "Bx", "By", "Bz")


def parity_sample(steps: int = 200, size: int = 128):
    """Part of the CPU-baseline leg: the workload's scene cropped to size^3 (16-cell absorber,
    thin-wire dipole with its 50-ohm pulsed feed, random dielectric blocks, port series) stepped
    `steps` times on the GPU and by the CPU restatement in FP32 and FP64. Reports whether the GPU
    fields and port series equal the FP32 restatement bit for bit (the restatement is itself equal
    to the reference's shaders compiled as C++), and the relative L2 of every field component and
    of the port series against the FP64 restatement (the FP32 error floor of the update)."""
    import oracle
    from em_lab_gb300 import SimulationGrid, configs
    oracle.set_threads(os.cpu_count() or 1)
    sc = configs.plain_large(size=size)
    port = [sc.ports[0].to_c()]
    out = {}
    t0 = time.perf_counter()
    for label, t in (("gpu", SimulationGrid(sc.grid)), ("f32", oracle.Oracle(sc.grid, "f32")),
                     ("f64", oracle.Oracle(sc.grid, "f64"))):
        oracle.load_scene(t, sc)
        t.ports_configure(port, sc.wavelength, 4.0, False, steps)
        t.step(steps)
        out[label] = ([np.asarray(c, np.float64) for c in t.read_components()], np.asarray(t.ports_series(), np.float64))
        t.close()
    gpu_f, gpu_s = out["gpu"]
    f32_f, f32_s = out["f32"]
    f64_f, f64_s = out["f64"]

    def rel(a, b):
        n = np.linalg.norm(b)
        return float(np.linalg.norm(a - b) / n) if n > 0 else 0.0
    return {"workload": f"{size}^3 crop of the workload's scene (absorber, thin-wire dipole, 50-ohm pulsed feed, "
                        f"random blocks, port series), {steps} steps",
            "bit_exact_vs_fp32_oracle": bool(all(np.array_equal(a, b) for a, b in zip(gpu_f, f32_f)) and
                                             np.array_equal(gpu_s, f32_s)),
            "max_abs_vs_fp32_oracle": float(max(np.abs(a - b).max() for a, b in zip(gpu_f, f32_f))),
            "rel_l2_vs_fp64_oracle": {n: rel(a, b) for n, a, b in zip(COMPONENTS, gpu_f, f64_f)},
            # the same per field vector (E, B): a component much smaller than its field's others (Bz of a
            # z dipole, 1 % of |B| here) has a larger error relative to its own norm at the same absolute error
            "rel_l2_vs_fp64_oracle_per_field": {
                "E": rel(np.stack(gpu_f[:3]), np.stack(f64_f[:3])), "B": rel(np.stack(gpu_f[3:]), np.stack(f64_f[3:]))},
            "rms_abs_error_vs_fp64_oracle": {n: float(np.sqrt(np.mean((a - b) ** 2))) for n, a, b in zip(COMPONENTS, gpu_f, f64_f)},
            "port_series_rel_l2_vs_fp64_oracle": rel(gpu_s, f64_s),
            "seconds": round(time.perf_counter() - t0, 1)}


def run_reference(args):
    """The reference's CPU implementation of the path on the host cores: its shaders compiled as C++
    (oracle/_ref) where that library was built, else the FP32 restatement, on every host thread."""
    rank, world, _ = _rank_env()
    if rank != 0:
        return 0
    sc = build_scene(args)
    kind = "port"
    try:
        from oracle import ref as refmod  # the reference's shaders compiled through the GLSL shim
        if refmod.available():
            kind = "reference"
    except Exception:
        refmod = None
    cells = float(np.prod(sc.grid.size))
    threads = os.cpu_count() or 1
    if kind == "reference":
        runner = refmod.RefGrid(sc.grid)
        refmod.set_threads(threads)
        runner.load_scene(sc)
    else:
        import oracle
        oracle.set_threads(threads)
        runner = oracle.Oracle(sc.grid, "f32")
        oracle.load_scene(runner, sc)
    if sc.ports:
        runner.ports_configure([p.to_c() for p in sc.ports], sc.ports[0].wavelength, 4.0, sweep=True)
    # the same per-step monitors as the GPU arm: the 32-frequency far-field DFT (FP64 sums every
    # step) runs in the restatement; the reference's own shaders have no multi-frequency monitor
    dft_points = None
    if args.workload == "plain_large" and kind == "port":
        _, dft_points = dft_setup(runner, sc)
    # each bench step is a bounded sample: one full-grid leapfrog step
    for _ in range(max(1, min(args.warmup, 1))):
        runner.step(1)
    # the timed sample is bounded: full-grid steps until K are done or the time budget is spent
    budget = float(os.environ.get("EMLAB_REFERENCE_BUDGET_S", "120"))
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        runner.step(1)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    value = cells * done / el / 1e6
    monitors = (", port monitor" if sc.ports else "") + (", 32-frequency far-field DFT" if dft_points else "")
    sample = (f"{done} of {args.steps} requested full-grid leapfrog steps (B, E, sources"
              f"{monitors}) of the {'x'.join(str(v) for v in sc.grid.size)} workload "
              f"within a {budget:.0f} s budget, "
              f"{'reference shaders compiled as C++ (oracle/_ref)' if kind == 'reference' else 'CPU restatement oracle/emlab_oracle.c FP32'}, "
              f"{threads} host threads")
    line = {"metric": METRIC, "value": value, "unit": "Mcells/s", "n_gpus": world, "steps": done,
            "warmup": args.warmup, "ms_per_step": el * 1e3 / done, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": workload_text(args, sc, dft_points) + (
                "" if dft_points or args.workload != "plain_large" else
                " (the far-field DFT is omitted: the reference's shaders have no multi-frequency monitor)"),
                       "cells": int(cells)},
            "cpu_baseline": {"value": value, "unit": "Mcells/s", "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "Mcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_batched(args):
    """--workload batched: the batched antenna sweep (256 seeded scenes, cube edges 48-160, 8-cell
    absorber, thin-wire dipole or monopole over ground with a 50-ohm Gaussian-pulse feed, one random
    dielectric sphere or box), every scene run to -60 dB port ring-down and its 128-point Z(f) sweep
    evaluated. value = sweeps per hour of the batched path (scene stacks, one launch per pass for all
    scenes of a cross-section); beside it the same scenes one grid at a time."""
    import torch
    from em_lab_gb300 import batch, configs, launch_count

    rank, world, local = _rank_env()
    if world > 1 and rank != 0:
        return 0  # one GPU per run in this mode
    torch.cuda.set_device(local)
    n = args.scenes
    t0 = time.perf_counter()
    scenes = configs.batched_scenes(n, seed=args.seed)
    build_s = time.perf_counter() - t0
    # warm-up: a few chunks of a small batch (kernel loading, allocator)
    warm = batch.BatchRunner([configs.batched_scene(args.seed + 1, i) for i in range(4)], max_steps=64 * args.warmup,
                             layout=args.layout)
    warm.run()
    warm.close()
    l0 = launch_count()
    runner = batch.BatchRunner(scenes, chunk=64, layout=args.layout)
    with ClockSampler(local) as clk:
        results = runner.run()
    launches = launch_count() - l0
    done = sum(r.done for r in results)
    steps = [r.steps for r in results]
    scene_cells = [int(np.prod(sc.grid.size)) for sc in scenes]
    useful = float(sum(c * st for c, st in zip(scene_cells, steps)))
    value = done / runner.wall_s * 3600.0
    other = None
    if args.layout == "ragged" and not args.no_single:
        # the same scenes in one stack per cross-section, each on its own stream and host thread
        alt = batch.BatchRunner(scenes, chunk=64, layout="cross_section")
        alt_res = alt.run()
        alt.close()
        other = {"layout": "one stack per cross-section, each on its own CUDA stream", "groups": len(alt.groups),
                 "sweeps_per_hour": sum(r.done for r in alt_res) / alt.wall_s * 3600.0,
                 "mcells_per_s": float(sum(c * r.steps for c, r in zip(scene_cells, alt_res))) / alt.wall_s / 1e6,
                 "identical_results": all(np.array_equal(a.sweep["z"], b.sweep["z"]) for a, b in zip(results, alt_res)
                                          if a.sweep is not None and b.sweep is not None)}
    single = None
    if not args.no_single:
        ts = []
        sample = scenes if args.single_all else scenes[:: max(1, n // 32)]
        for sc in sample:
            tm = {}
            batch.run_single(sc, chunk=64, timing=tm)
            ts.append(tm)
        run_s = sum(t["run_s"] for t in ts)
        cells_single = sum(int(np.prod(sc.grid.size)) * t["steps"] for sc, t in zip(sample, ts))
        single = {"scenes": len(sample), "sweeps_per_hour": len(sample) / run_s * 3600.0,
                  "mcells_per_s": cells_single / run_s / 1e6, "setup_s_per_scene": sum(t["setup_s"] for t in ts) / len(ts),
                  "note": "the same scenes, one SimulationGrid each, same ring-down rule; stepping + sweep timed, set-up excluded"}
    line = {
        "metric": "Z(f) sweeps/hr (batched, run to -60 dB port ring-down)", "value": value, "unit": "sweeps/hr",
        "n_gpus": 1, "steps": int(max(steps)), "warmup": args.warmup, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched antenna sweep: {n} seeded scenes (seed {args.seed}), cube edges 48-160 cells, "
                               "8-cell absorber, thin-wire dipole or monopole over ground, 50-ohm Gaussian-pulse feed, "
                               "one random dielectric sphere or box, 128-point Z(f) sweep per scene",
                   "groups": len(runner.groups), "chunk_steps": 64, "l2": "inputs larger than L2 (stack state > 129 MB)",
                   "layout": ("one stack of scenes with their own cross-sections per solver setting: one persistent "
                              "Yee launch per step for all scenes" if args.layout == "ragged" else
                              "one stack per cross-section, each on its own CUDA stream")},
        "scenes_done": done, "scenes_rung_down": sum(r.rung_down for r in results), "scene_steps": {"min": int(min(steps)), "median": int(np.median(steps)), "max": int(max(steps))},
        "mcells_per_s": useful / runner.wall_s / 1e6,
        "setup_s": {"scene_build": build_s, "stack_upload_and_tiling": runner.setup_s},
        "host_s": {"between_chunks": runner.host_s, "of_which_compaction": runner.compact_s,
                   "note": "summed over the stacks' host threads"},
        "tiling": {"x".join(str(v) for v in g.scenes[0].grid.size) if args.layout != "ragged" else f"stack {k}":
                   min(g.tiling, key=g.tiling.get) if g.tiling else None for k, g in enumerate(runner.groups)},
        "per_cross_section": other,
        "single_grid": single,
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    runner.close()
    return 0


def run_learned(args):
    """--workload learned: the learned ring-down extrapolator. Training
    runs of the batched generator's scenes (seed --seed) to -60 dB ring-down, training on the GPU
    with this library's kernels, then on held-out scenes (seed --seed + 1): sweeps/hr of the plain
    solver to ring-down (the reference result) against the learned path (early window + inference), the
    |dZ| and S11 error of the network and of the early window's truncated DFT, and the same for the
    32-frequency far-field spectra (directivity and radiated energy, dB)."""
    import torch
    from em_lab_gb300 import extrap, launch_count

    rank, world, local = _rank_env()
    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    periods = [float(v) for v in str(args.periods).split(",") if v.strip()]
    l0 = launch_count()
    with ClockSampler(local) as clk:
        out, _ = extrap.experiment(args.seed, args.train_scenes, args.seed + 1, args.scenes, epochs=args.epochs,
                                   periods=periods, members=args.members, val_frac=args.val_frac, single=True,
                                   log=lambda m: print(m, file=sys.stderr))
    windows = {k: {"sweeps_per_hour": v["sweeps_per_hour"], "speedup_vs_batched_plain": v["speedup_vs_batched_plain"],
                   "speedup_vs_single_plain": v.get("speedup_vs_single_plain"), "network_only": v["network_only"],
                   "eval": v["eval"], "validation": v.get("validation"), "wall": v["wall"],
                   "early_steps_median": v["early_steps_median"], "training": v["training"]}
               for k, v in out["windows"].items()}
    # headline: the network alone at the shortest window meeting the medians on validation runs;
    # beside it the strict operating point (p90 bound with the plain-solver fallback)
    strict = out["windows"][out["chosen_window"]]
    net_key = out["chosen_window_network_only"]
    if net_key is not None:
        head = dict(out["windows"][net_key]["network_only"], window=net_key, accuracy=out["windows"][net_key]["eval"]["network"],
                    accuracy_far_field=out["windows"][net_key]["eval"]["network_far"],
                    truncated_far_field=out["windows"][net_key]["eval"]["truncated_dft_far"],
                    criterion="median over scenes of band-median |dZ|/|Z| <= 2 % and S11 error <= 0.5 dB "
                              "(checked on validation runs)")
    else:
        head = {"sweeps_per_hour": strict["sweeps_per_hour"], "window": out["chosen_window"]}
    strict_line = {"window": out["chosen_window"], "sweeps_per_hour": strict["sweeps_per_hour"],
                   "speedup_vs_batched_plain": strict["speedup_vs_batched_plain"],
                   "speedup_vs_single_plain": strict.get("speedup_vs_single_plain"),
                   "accuracy": strict["eval"].get("with_fallback"), "fallback_scenes": strict["eval"].get("fallback_scenes"),
                   "accuracy_far_field": strict["eval"].get("with_fallback_far"),
                   "criterion": "p90 over scenes of band-median |dZ|/|Z| <= 2 % and of the S11 error <= 0.5 dB on "
                                "validation runs; scenes above the ensemble-spread threshold run the plain solver"}
    # what the learned path costs once, before any sweep: generating the training runs with the
    # batched solver, and training the ensemble of the window in use (sweeps/hr excludes both)
    for entry, key in ((head, head.get("window", out["chosen_window"])), (strict_line, out["chosen_window"])):
        entry["one_time_cost_s"] = {"training_runs_generation": out["train_runs"]["wall_s"],
                                    "ensemble_training": out["windows"][key]["training"]["wall_s"]}
    line = {
        "metric": "Z(f) sweeps/hr learned vs plain (held-out scenes)", "value": head["sweeps_per_hour"],
        "unit": "sweeps/hr", "n_gpus": 1, "steps": None, "warmup": args.warmup, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 GEMMs, fp32 accumulation",
        "data": "synthetic (runs generated by the batched solver)",
        "config": {"workload": f"learned ring-down extrapolator: {args.train_scenes} training scenes (seed {args.seed}; "
                               f"{args.val_frac:g} of them held for the fallback threshold), {args.scenes} held-out "
                               f"scenes (seed {args.seed + 1}), early windows {','.join(f'{p:g}' for p in periods)} "
                               f"design periods, ensembles of {args.members}, {args.epochs} epochs; inputs: early port "
                               f"V, I and 32 surface-DFT channels (the Huygens box's far-field spectra over the early "
                               f"window); outputs: Z(f) at 128 frequencies and the 32-frequency far-field spectra "
                               f"(directivity, radiated energy)",
                   "plain_reference": "batched stacks and one SimulationGrid per scene, each run to -60 dB ring-down"},
        "headline": head, "strict": strict_line, "plain": out["plain"], "windows": windows,
        "train_runs": out["train_runs"], "gpu_launches": int(launch_count() - l0), "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_phased(args):
    """--workload phased_array: 16 x 16 dipoles at half-wavelength pitch
    (lambda 24 cells) a quarter wavelength over a ground sheet under a radome slab (eps_r 3.5, 6
    cells), 384 x 384 x 256 cells with a 12-cell absorber, 50-ohm feeds with a Taylor taper and
    true-time-delay steering to 8 seeded directions (8 scenes); the 32-frequency tensor-core
    far-field DFT every step, then the pattern at 181 x 361 angles and all 32 frequencies.
    value = cell-steps per second of the stepping (DFT included) over the 8 scenes."""
    import torch
    from em_lab_gb300 import launch_count, phased

    rank, world, local = _rank_env()
    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    dirs = phased.steering_directions(args.seed, 8)
    warm = phased.build(0.0, 0.0, elements=4, nxy=128, nz=128)
    phased.run_scene(warm, 64 * args.warmup, 19, 37, freqs=[16])
    l0 = launch_count()
    res = []
    with ClockSampler(local) as clk:
        for k, (th, ph) in enumerate(dirs):
            sc = phased.build(th, ph)
            r = phased.run_scene(sc, args.array_steps, compare=(k == 0))
            r.pop("pattern")
            r["steer"] = (th, ph)
            r["pointing_error_deg"] = phased.angular_error(r["beam_theta"], r["beam_phi"], th, ph)
            res.append(r)
    launches = launch_count() - l0
    cell_steps = sum(r["cells"] * r["steps"] for r in res)
    step_s = sum(r["step_s"] for r in res)
    pat_s = sum(r["pattern_s"] for r in res)
    line = {
        "metric": "Yee Mcells/s (phased-array scenes, far-field DFT every step)", "value": cell_steps / step_s / 1e6,
        "unit": "Mcells/s", "n_gpus": 1, "steps": args.array_steps, "warmup": args.warmup,
        "ms_per_step": step_s / (len(res) * args.array_steps) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "phased array: 8 scenes of 384x384x256 (12-cell absorber), 16x16 thin-wire dipoles at "
                               "lambda/2 pitch (lambda 24), ground sheet, radome eps_r 3.5, 50-ohm Taylor-tapered "
                               "time-delay-steered feeds, 32-frequency far-field DFT, pattern 181x361 x 32 frequencies",
                   "directions_seed": args.seed, "l2": "inputs larger than L2 (1.8 GB of field state per scene)"},
        "pattern": {"evaluations": sum(r["pattern_evaluations"] for r in res), "seconds": pat_s,
                    "huygens_points": res[0]["points"],
                    "method": "per-face tensor-core GEMMs (emlab_ntff_dft_pattern_gemm)",
                    "first_scene_direct_sums_s": res[0].get("other_pattern_s"),
                    "first_scene_gemm_s": res[0]["pattern_s"],
                    "first_scene_max_diff_of_peak": res[0].get("max_diff_of_peak"),
                    "first_scene_power_rel_diff": res[0].get("power_rel_diff")},
        "beams": [{"steer": r["steer"], "beam": (r["beam_theta"], r["beam_phi"]),
                   "error_deg": round(r["pointing_error_deg"], 2)} for r in res],
        "gpu_launches": int(launches), "clocks": clk.summary(), "finite": all(r["finite"] for r in res),
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--workload", default="plain_large",
                    choices=["plain_large", "plain_small", "batched", "learned", "phased_array"],
                    help="plain_large: the 512^3 dipole + blocks workload (default); plain_small: 128^3 sphere; "
                         "batched: 256 antenna scenes to port ring-down (sweeps/hr)")
    ap.add_argument("--scenes", type=int, default=256, help="batched: number of scenes")
    ap.add_argument("--seed", type=int, default=2024, help="batched: scene seed")
    ap.add_argument("--no-single", action="store_true", help="batched: skip the one-grid-per-scene comparison")
    ap.add_argument("--single-all", action="store_true", help="batched: compare on every scene, not a sample")
    ap.add_argument("--layout", default="ragged", choices=["ragged", "cross_section"],
                    help="batched: one stack of all cross-sections (one launch per step) or one stack per cross-section")
    ap.add_argument("--train-scenes", type=int, default=20000, help="learned: training scenes")
    ap.add_argument("--epochs", type=int, default=100, help="learned: training epochs")
    ap.add_argument("--periods", default="1.5,2,3,4", help="learned: early windows to try, design periods")
    ap.add_argument("--members", type=int, default=3, help="learned: networks per ensemble")
    ap.add_argument("--val-frac", type=float, default=0.1, help="learned: training runs held for the fallback rule")
    ap.add_argument("--array-steps", type=int, default=12000, help="phased_array: steps per scene")
    ap.add_argument("--size", type=int, default=512, help="edge of the plain_large grid")
    ap.add_argument("--kernel", default="fused", choices=["fused", "fused_ldg", "split"])
    ap.add_argument("--tile-rows", type=int, default=0, choices=[0, 8, 16, 32, 64, 128])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the FP32/FP64 parity sample of the CPU leg")
    ap.add_argument("--e2e-steps", type=int, default=0, help="steps of the end-to-end leg (default: --steps)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    args.warmup = max(args.warmup, 3)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "learned":
        return run_learned(args)
    if args.workload == "phased_array":
        return run_phased(args)

    import torch
    rank, world, local = _rank_env()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)

    from em_lab_gb300 import SimulationGrid, abi, launch_count

    sc = build_scene(args)
    cells = float(np.prod(sc.grid.size))
    grid = SimulationGrid(sc.grid)
    grid.set_kernel({"fused": abi.KERNEL_FUSED, "fused_ldg": abi.KERNEL_FUSED_LDG, "split": abi.KERNEL_SPLIT}[args.kernel])
    grid.set_tiling(args.tile_rows)
    load_grid(grid, sc)
    dft_points = attach_monitors(grid, sc, args)
    stream = torch.cuda.ExternalStream(grid.stream_handle())

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        grid.synchronize(600000)

    # --- device-resident leg: inputs already in HBM -----------------------------------------
    grid.step(args.warmup)
    barrier()
    grid.set_timing(True)
    grid.kernel_time(reset=True)
    l0 = launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        grid.step(args.steps)
        ev1.record(stream)
        barrier()
    launches = launch_count() - l0
    kernel_ms, kernel_n = grid.kernel_time(reset=True)
    grid.set_timing(False)
    value, elapsed_s = replica_throughput(cells * args.steps, ev0.elapsed_time(ev1) * 1e-3, dist, "cuda")
    elapsed_ms = elapsed_s * 1e3
    peak, peak_kind = _peaks()
    per_launch_ms = kernel_ms / max(kernel_n, 1)
    achieved = BYTES_PER_CELL_STEP * cells / (per_launch_ms * 1e-3) / 1e9

    # --- end-to-end leg through the C ABI with host buffers ------------------------------------
    # The headless frame loop of the reference (Main.cpp:1074-1099): each frame steps the grid
    # (the host computes the source signals and monitor rotations in FP64 and uploads them), then
    # reads back the probe neighbourhood and the flux box the way FieldAnalyzer does, one frame
    # late (submit after the steps, collect at the next frame); the port (V, I) series is read
    # back at the end. Host<->device copies are inside the timed region.
    e2e_steps = args.e2e_steps or args.steps
    frame = 2
    probe, planes, bmin, bmax = frame_reads(sc)
    attach_monitors(grid, sc, args)  # fresh monitor state for the end-to-end leg
    from em_lab_gb300 import configs
    dirs = configs.fibonacci_directions(1024)
    barrier()
    t0 = time.perf_counter()
    frames = 0
    for _ in range(e2e_steps // frame):
        grid.step(frame)
        # FieldAnalyzer::submit / collect: this frame's probe and flux box are queued behind its
        # steps; the previous frame's values are read while the GPU runs on
        grid.analyzer_collect()
        grid.analyzer_submit(probe, planes)
        frames += 1
    grid.analyzer_collect()
    tail = []  # end-of-run reads: port series and sweep, far-field pattern
    if sc.ports:
        wl = sc.ports[0].wavelength
        tail.append(grid.ports_series())
        tail.append(grid.ports_sweep_sums(wl / 1.7, wl / 0.3, SWEEP_POINTS)[0])
    if dft_points is not None:
        tail.append(grid.ntff_dft_evaluate(DFT_FREQS // 2, dirs))
    else:
        tail.append(grid.ntff_evaluate(dirs))
    barrier()
    e2e_value, _ = replica_throughput(cells * frames * frame, time.perf_counter() - t0, dist, "cuda")
    # per step: FP64-evaluated source signals (FP32) and the monitor rotations (cos/sin pairs)
    h2d = 4 * len(sc.sources) + 16 * (1 if sc.ports else 0) + 16 * (1 if args.workload == "plain_small" else 0)
    # per frame: the probe's 54 texels and the flux planes' 16 x 16 workgroup partials; per step: the
    # port series; once: the sweep and the pattern
    parts = 0
    for ax in range(3):
        u, v = (1, 2) if ax == 0 else ((0, 2) if ax == 1 else (0, 1))
        parts += 2 * ((bmax[u] - bmin[u] + 16) // 16) * ((bmax[v] - bmin[v] + 16) // 16)
    d2h = (len(probe) * 54 * 16 + 4 * parts) / frame + sum(t.nbytes for t in tail) / (frames * frame)
    finite = grid.check_finite()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_sample(sc, dft=dft_points is not None)
        except Exception as e:  # pragma: no cover - reported, not fatal
            cpu = {"value": None, "unit": "Mcells/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {e}"}
        if args.workload == "plain_large" and not args.no_parity:
            try:
                cpu["parity"] = parity_sample()
            except Exception as e:  # pragma: no cover - reported, not fatal
                cpu["parity"] = {"failed": str(e)}

    if rank == 0:
        kname = kernel_name(args.kernel, args.tile_rows)
        traffic = read_traffic(f"{kname}_{args.workload}_{'x'.join(str(v) for v in sc.grid.size)}")
        state_gb = 48.0 * cells / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": "Mcells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_text(args, sc, dft_points), "cells": int(cells), "kernel": args.kernel,
                       "tiling": args.tile_rows or "auto (64x8 pair tiles)",
                       "l2": (f"inputs larger than L2 ({state_gb:.1f} GB of field state per step)" if state_gb > 0.129
                              else f"field state {state_gb * 1e3:.0f} MB fits in L2 (129 MB); no flush between steps"),
                       "e2e_extra": "probe + 6-plane flux box read every 2 steps; " + (
                           f"port series, {SWEEP_POINTS}-point port sweep and " if sc.ports else "") +
                                    "a 1024-direction far-field pattern at the end",
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_source": peak_kind,
                         "traffic_source": ("DRAM bytes read + written per launch from one ncu capture of the "
                                            "256^3 case, scaled by the cells a launch updates (profiles/traffic.txt); "
                                            "not measured in this run") if traffic else None,
                         "kernel": kname, "kernel_ms_per_launch": per_launch_ms,
                         "algorithmic_bytes_per_cell_step": BYTES_PER_CELL_STEP},
            "cpu_baseline": cpu,
            "parity": (cpu or {}).get("parity"),
            "e2e": {"value": e2e_value, "unit": "Mcells/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "frames": frames, "steps_per_frame": frame},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "finite": bool(finite),
        }
        print(json.dumps(line), flush=True)
    grid.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
