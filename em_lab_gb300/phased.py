"""Planar phased-array workload: N x N dipoles over a ground sheet under a radome,
Taylor-tapered and steered by true time delays, in eight seeded directions; the far field at
181 x 361 angles and 32 frequencies from the tensor-core DFT of the Huygens-box fields, the pattern
sums factorised face by face into tensor-core GEMMs.

The scene is the script `scenes/phased_array.lua`; each steering direction is one scene on a grid
of its own (a 384 x 384 x 256 scene fills the GPU by itself), stepped with the far-field DFT
attached, then evaluated at every frequency over the full angle grid by emlab_ntff_dft_pattern_gemm
(the sums of ntff_pattern.comp / ntff_reduce.comp split per face into a u and a v factor: the sum over
v one complex GEMM on the tcgen05 tensor cores, csrc/pattern_tc.cu) or, with pattern="direct",
emlab_ntff_dft_evaluate_all (the direct sums with range-reduced hardware sin/cos, csrc/monitors.cu).
"""
from __future__ import annotations

import math
import os
import time

import numpy as np

from .grid import SimulationGrid
from .script import ScriptEngine

SCENE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "scenes", "phased_array.lua")
DFT_MARGIN = 20
DFT_FREQS = 32


def steering_directions(seed: int = 5, count: int = 8):
    """(theta, phi) in degrees: theta uniform in [0, 40], phi uniform in [0, 360)."""
    rng = np.random.default_rng(seed)
    return [(round(float(rng.uniform(0.0, 40.0)), 1), round(float(rng.uniform(0.0, 360.0)), 1)) for _ in range(count)]


def build(theta, phi, **overrides):
    ov = {"theta": str(theta), "phi": str(phi)}
    ov.update({k: str(v) for k, v in overrides.items()})
    return ScriptEngine(ov, echo=False).run_file(SCENE).scene


def angle_grid(n_theta: int = 181, n_phi: int = 361):
    """Unit vectors on a theta x phi grid (degrees, theta from +z), as (n_theta * n_phi, 3) float32."""
    th = np.radians(np.linspace(0.0, 180.0, n_theta))
    ph = np.radians(np.linspace(0.0, 360.0, n_phi))
    T, P = np.meshgrid(th, ph, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], axis=-1).reshape(-1, 3)
    return d.astype(np.float32), np.degrees(th), np.degrees(ph)


def run_scene(sc, steps: int, n_theta: int = 181, n_phi: int = 361, freqs=None, pattern: str = "gemm",
              compare: bool = False):
    """Steps one scene with the 32-frequency far-field DFT and evaluates the pattern. Returns timing,
    the main-beam direction at the frequency nearest the design frequency and the pattern there.
    compare: also evaluate the direct sums and report the largest difference and their time."""
    L = sc.grid.pml_thickness
    g = SimulationGrid(sc.grid)
    m = sc.materials
    g.upload_materials(m.sigma, m.epsilon_r, sc.edges, sc.wires)
    g.set_sources(sc.sources)
    lo = [L + DFT_MARGIN] * 3
    hi = [n - L - DFT_MARGIN - 1 for n in sc.grid.size]
    wl0 = sc.wavelength
    rel = np.linspace(0.3, 1.7, DFT_FREQS)
    g.ntff_dft_configure(lo, hi, [wl0 / f for f in rel])
    points, _ = g.ntff_dft_info()
    g.synchronize()
    t0 = time.perf_counter()
    g.step(steps)
    g.synchronize(600000)
    t1 = time.perf_counter()
    dirs, th, ph = angle_grid(n_theta, n_phi)
    f0 = int(np.argmin(np.abs(rel - 1.0)))
    extra = {}
    if freqs is None:  # every frequency in one call
        which = range(DFT_FREQS)
        full = g.ntff_dft_pattern_gemm(0, dirs) if pattern == "gemm" else g.ntff_dft_evaluate_all(dirs)
        pat0 = full[f0, :, 0].reshape(n_theta, n_phi)
        if compare:
            g.synchronize()
            tc = time.perf_counter()
            other = g.ntff_dft_evaluate_all(dirs) if pattern == "gemm" else g.ntff_dft_pattern_gemm(0, dirs)
            g.synchronize()
            extra = {"other_pattern_s": time.perf_counter() - tc,
                     "max_diff_of_peak": float(np.max(np.abs(full[:, :, 0] - other[:, :, 0]).max(axis=1) /
                                                      np.maximum(np.abs(other[:, :, 0]).max(axis=1), 1e-30))),
                     "power_rel_diff": float(np.max(np.abs(full[:, 0, 1] - other[:, 0, 1]) /
                                                    np.maximum(np.abs(other[:, 0, 1]), 1e-30)))}
            t_extra = time.perf_counter() - tc
    else:
        which = freqs
        pat0 = None
        for f in which:
            out = g.ntff_dft_evaluate(f, dirs)
            if f == f0:
                pat0 = out[:, 0].reshape(n_theta, n_phi)
        if pat0 is None:
            pat0 = g.ntff_dft_evaluate(f0, dirs)[:, 0].reshape(n_theta, n_phi)
    g.synchronize()
    t2 = time.perf_counter() - (t_extra if extra else 0.0)
    finite = g.check_finite()
    g.close()
    upper = pat0[: n_theta // 2 + 1]  # theta <= 90 deg: the half space above the ground sheet
    i, j = np.unravel_index(int(np.argmax(upper)), upper.shape)
    return {"cells": int(np.prod(sc.grid.size)), "steps": steps, "points": points, "step_s": t1 - t0,
            "pattern_s": t2 - t1, "pattern_evaluations": len(list(which)) * len(dirs),
            "beam_theta": float(th[i]), "beam_phi": float(ph[j]), "f_rel": float(rel[f0]), "finite": bool(finite),
            "pattern": pat0, **extra}


def angular_error(t1, p1, t2, p2):
    """Angle between two directions given as (theta, phi) in degrees."""
    a = [math.radians(v) for v in (t1, p1, t2, p2)]
    u = (math.sin(a[0]) * math.cos(a[1]), math.sin(a[0]) * math.sin(a[1]), math.cos(a[0]))
    v = (math.sin(a[2]) * math.cos(a[3]), math.sin(a[2]) * math.sin(a[3]), math.cos(a[2]))
    return math.degrees(math.acos(max(-1.0, min(1.0, sum(x * y for x, y in zip(u, v))))))
