"""Scene builders for the benchmark workloads and the parity-test scenes.

`plain_small` is the 128^3 point-dipole + dielectric-sphere scene (the scene of README.md:39-48
with eps_r = 2.25); `plain_large` is the 512^3 thin-wire half-wave dipole with a 50-ohm pulsed
feed among seeded random dielectric blocks. Both use seeded synthetic geometry; there is no
external dataset. `random_scene` builds small seeded scenes that exercise every solver feature
(lossy and metal cells, absorber, thin wires, feeds, several sources) for the parity tests.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .scene import EnvironmentBuilder, FluxSetup, Material, SourceDesc, resolve_material

f32 = np.float32


def plain_small(steps: int = 2000):
    """128^3 grid, FP32, vacuum, 10-cell absorber, Courant 0.5; eps_r 2.25 sphere of radius 10 at
    centre + 30 x; z point dipole at the centre, CW lambda = 16, amplitude 7, 3-period ramp; probe at
    centre - 30 x; 24-cell flux box; far-field box with the default 4-cell margin."""
    grid = abi.GridConfig((128, 128, 128), courant=0.5, pml_thickness=10, pml_sigma_max=1.6, pml_grading=3.0)
    b = EnvironmentBuilder("plain_small", grid, wavelength=16.0)
    c = (64.0, 64.0, 64.0)
    b.sphere((94.0, 64.0, 64.0), 10.0, Material(0.0, 2.25))
    src = SourceDesc.dipole(c, (0.0, 0.0, 1.0), 16.0, 7.0, 0.0)
    b.scene.sources.append(src)
    b.scene.probes.append(("behind", (34.0, 64.0, 64.0)))
    b.scene.fluxes.append(FluxSetup("radiated", "box", (52, 52, 52), (76, 76, 76)))
    L = grid.pml_thickness
    b.scene.far_field = {"box_min": (L + 1 + 4,) * 3, "box_max": tuple(n - L - 2 - 4 for n in grid.size),
                         "wavelength": 16.0, "averaging": 4.0}
    sc = b.build()
    sc.steps = steps
    return sc


def random_blocks(builder: EnvironmentBuilder, fraction: float, seed: int, lo: int, hi: int, keep_out=None,
                  cell_size=1.0e-3, edge_range=(4, 24)):
    """Seeded dielectric blocks until `fraction` of the cells is filled: edges uniform in
    edge_range, eps_r uniform in [1, 10], sigma log-uniform in [1e-4, 1e-1] S/m."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = builder.scene.grid.size
    target = fraction * nx * ny * nz
    filled = np.zeros((nz, ny, nx), bool)
    count = 0
    blocks = 0
    attempts = 0
    while count < target and attempts < 200_000:
        attempts += 1
        e = rng.integers(edge_range[0], edge_range[1] + 1, size=3)
        p = np.array([rng.integers(lo, max(lo + 1, hi - e[a])) for a in range(3)])
        if keep_out is not None:
            kc, kr = keep_out
            if np.all(p + e > np.asarray(kc) - kr) and np.all(p < np.asarray(kc) + kr):
                continue
        eps = float(rng.uniform(1.0, 10.0))
        sig_si = float(10.0 ** rng.uniform(-4.0, -1.0))
        m = resolve_material(eps, cell_size, builder.scene.wavelength, conductivity=sig_si)
        builder.box(tuple(float(v) for v in p), tuple(float(v) for v in p + e), m)
        sl = (slice(p[2], p[2] + e[2]), slice(p[1], p[1] + e[1]), slice(p[0], p[0] + e[0]))
        count += int((~filled[sl]).sum())
        filled[sl] = True
        blocks += 1
    return blocks, count / float(nx * ny * nz)


def plain_large(steps: int = 20000, size: int = 512, seed: int = 12345):
    """512^3 grid, 16-cell absorber; thin-wire half-wave z dipole (lambda = 40, length 20, radius
    0.05) with a 50-ohm resistive voltage feed driven by a Gaussian pulse (pulse_width 0.4 periods:
    the spectrum covers about 0.3-1.7 f0); 5% of the cells in seeded random dielectric blocks; port
    sweep at 128 frequencies; far-field box 20 cells inside the absorber."""
    L = 16
    grid = abi.GridConfig((size, size, size), courant=0.5, pml_thickness=L, pml_sigma_max=1.6, pml_grading=3.0)
    wl = 40.0
    b = EnvironmentBuilder("plain_large", grid, wavelength=wl)
    c = (size * 0.5,) * 3
    box_lo, box_hi = L + 20, size - L - 21
    random_blocks(b, 0.05, seed, box_lo + 1, box_hi - 1, keep_out=(c, 24), edge_range=(4, 24))
    wave = SourceDesc(wavelength=wl, waveform=abi.WAVE_PULSE, ramp_periods=0.4)
    b.thin_dipole(wave, c, 2, 20.0, radius=0.05, impedance_ohm=50.0, drive=1.0, name="dipole")
    b.scene.far_field = {"box_min": (box_lo,) * 3, "box_max": (box_hi,) * 3, "wavelength": wl, "averaging": 4.0}
    b.scene.sweep = {"wavelength_min": wl / 1.7, "wavelength_max": wl / 0.3, "points": 128}
    sc = b.build()
    sc.steps = steps
    return sc


def random_scene(size=(24, 20, 18), pml=4, seed=1, thin_wire=True, lossy=True, sources=2, courant=0.5):
    """Small seeded scene exercising every solver feature (parity tests)."""
    rng = np.random.default_rng(seed)
    grid = abi.GridConfig(size, courant=courant, pml_thickness=pml, pml_sigma_max=1.6, pml_grading=3.0)
    b = EnvironmentBuilder(f"random{seed}", grid, wavelength=12.0)
    nx, ny, nz = size
    for _ in range(4):
        e = rng.integers(2, 6, size=3)
        p = np.array([rng.integers(0, max(1, n - 2)) for n in size])
        m = Material(float(10 ** rng.uniform(-3, 0.5)) if lossy else 0.0, float(rng.uniform(1.0, 6.0)))
        b.box(tuple(float(v) for v in p), tuple(float(v) for v in p + e), m)
    if lossy:
        p = np.array([rng.integers(pml, max(pml + 1, n - pml - 3)) for n in size])
        b.box(tuple(float(v) for v in p), tuple(float(v) for v in p + 2), Material(100.0, 1.0))  # metal block
    b.sphere((nx * 0.3, ny * 0.6, nz * 0.5), 3.0, Material(0.02, 2.25))
    srcs = []
    for k in range(sources):
        cpos = tuple(float(v) for v in rng.uniform(pml + 2, np.asarray(size) - pml - 2))
        ax = [0.0, 0.0, 0.0]
        ax[k % 3] = 1.0
        s = SourceDesc.dipole(cpos, ax, 12.0, float(rng.uniform(0.5, 3.0)), float(rng.integers(0, 4)))
        s.phase = float(rng.uniform(0, 6.28))
        if k % 2:
            s.waveform = abi.WAVE_PULSE
            s.ramp_periods = 0.5
        srcs.append(s)
    b.scene.sources.extend(srcs)
    if thin_wire:
        c = (nx * 0.5 + 0.3, ny * 0.5 - 0.2, nz * 0.5)
        wave = SourceDesc(wavelength=12.0, waveform=abi.WAVE_CW, ramp_periods=1.0)
        b.thin_dipole(wave, c, 2, 7.0, radius=0.05, impedance_ohm=50.0, drive=1.0, name="feed")
    sc = b.build()
    return sc


def fibonacci_directions(n: int) -> np.ndarray:
    """n unit vectors spread over the sphere (far-field test directions)."""
    i = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * i / n)
    th = math.pi * (1 + 5 ** 0.5) * i
    return np.stack([np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)], 1).astype(np.float32)


BATCH_EDGES = tuple(range(48, 161, 16))


def batched_scene(seed: int, index: int, pml: int = 8, edges=BATCH_EDGES):
    """One scene of the batched antenna sweep: a cube of edge 48, 64, ..., 160 cells (uniform) with an
    8-cell absorber; a thin-wire z dipole at the centre or a monopole over a PEC ground plate (50/50),
    length uniform in [0.3, 0.7] lambda, wire radius uniform in [0.02, 0.2] cell, fed by a 50-ohm
    resistive voltage source with a Gaussian pulse (0.4 periods: about 0.3-1.7 f0); one dielectric
    sphere or box (eps_r uniform in [1, 10], sigma log-uniform in [1e-4, 1e-1] S/m) beside it.
    lambda = 0.6 (edge - 2 pml) cells. Port sweep 0.3-1.7 f0 at 128 points. Seeded by (seed, index)."""
    rng = np.random.default_rng([int(seed), int(index)])
    n = int(rng.choice(edges))
    grid = abi.GridConfig((n, n, n), courant=0.5, pml_thickness=pml, pml_sigma_max=1.6, pml_grading=3.0)
    wl = float(f32(0.6 * (n - 2 * pml)))
    b = EnvironmentBuilder(f"batch{seed}_{index}", grid, wavelength=wl)
    monopole = bool(rng.random() < 0.5)
    length = float(f32(rng.uniform(0.3, 0.7) * wl))
    radius = float(f32(rng.uniform(0.02, 0.2)))
    wave = SourceDesc(wavelength=wl, waveform=abi.WAVE_PULSE, ramp_periods=0.4)
    c = n * 0.5
    lo, hi = pml + 3, n - pml - 3
    if monopole:
        zg = pml + 4  # ground plate: one metal layer below the surface plane zg
        b.box((float(lo), float(lo), float(zg - 1)), (float(hi), float(hi), float(zg)), Material(1.0e7, 1.0))
        node = [int(math.floor(c + 0.5)), int(math.floor(c + 0.5)), zg]
        rod = max(1, int(math.floor(length + 0.5)) - 1)
        b.add_thin_wire(node, 2, zg, zg + 1 + rod, radius, zg)
        b.add_feed(wave, node, 2, 1.0, 1, 50.0, 1.0, True, "monopole")
        ant_lo, ant_hi = zg, zg + 1 + rod
    else:
        b.thin_dipole(wave, (c, c, c), 2, length, radius=radius, impedance_ohm=50.0, drive=1.0, name="dipole")
        arm = EnvironmentBuilder.dipole_arm(length)
        ant_lo, ant_hi = int(math.floor(c)) - arm, int(math.floor(c)) + 1 + arm
    # the obstacle: beside the antenna (at least 3 cells of clearance from its axis)
    eps = float(rng.uniform(1.0, 10.0))
    m = resolve_material(eps, 1.0e-3, wl, conductivity=float(10.0 ** rng.uniform(-4.0, -1.0)))
    if rng.random() < 0.5:
        r = float(rng.uniform(2.0, max(2.5, n / 10.0)))
        off = float(rng.uniform(r + 3.0, max(r + 3.5, hi - c - r)))
        ang = float(rng.uniform(0.0, 2.0 * math.pi))
        zc = float(rng.uniform(max(lo + r, ant_lo - 2.0), min(hi - r, ant_hi + 2.0)))
        b.sphere((c + off * math.cos(ang), c + off * math.sin(ang), zc), r, m)
    else:
        e = rng.integers(3, max(4, n // 5) + 1, size=3)
        side = 1 if rng.random() < 0.5 else -1
        x0 = c + side * 3.0 if side > 0 else c - 3.0 - float(e[0])
        y0 = float(rng.uniform(lo, max(lo + 1.0, hi - e[1])))
        z0 = float(rng.uniform(lo, max(lo + 1.0, hi - e[2])))
        b.box((x0, y0, z0), (x0 + float(e[0]), y0 + float(e[1]), z0 + float(e[2])), m)
    b.scene.sweep = {"wavelength_min": wl / 1.7, "wavelength_max": wl / 0.3, "points": 128}
    sc = b.build()
    sc.description = f"{'monopole' if monopole else 'dipole'} L={length:.2f} a={radius:.3f} eps={eps:.2f}"
    return sc


def batched_scenes(count: int = 256, seed: int = 2024, edges=BATCH_EDGES):
    return [batched_scene(seed, i, edges=edges) for i in range(count)]
