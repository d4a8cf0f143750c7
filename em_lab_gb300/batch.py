"""Batched antenna sweeps: many independent scenes stepped together until their ports ring down.

Scenes of equal solver settings become one `SceneStack` of scenes with their own cross-sections: a
single grid whose every solver launch covers all of its scenes (csrc/stack.cu), one launch of the
persistent pair kernel per step whose work items are the tiles of each scene's own nx x ny. With
layout="cross_section" the scenes are instead grouped by (nx, ny), one stack per group, each group
on its own CUDA stream so that the groups' launches overlap on the device. Every `chunk` steps the port series of the
chunk is read back; a scene is done when the reference's ring-down residual (the largest |V| of
the last 5 % of its series over the peak, Ports.cpp:206-213) is 60 dB down, after at least four
design periods (at most 120). A finished scene's impedance sweep Z(f) is
evaluated on the host from its whole series (Ports.cpp:187-278: the FP64 DFT of V and I with the
half-step phase correction of I, Z = -V/I * eta0), and the scene is dropped from its stack by
compaction once a quarter of the stack has finished.

The single-scene reference path steps one SimulationGrid per scene (src/SimulationGrid.cpp:368-433);
`run_single` does that with this library, for comparison and as the reference result for the batched runs.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .grid import SceneStack, SimulationGrid
from .scene import K_ETA0

DB_RINGDOWN = -60.0


@dataclass
class SceneResult:
    index: int
    steps: int = 0
    series: list = field(default_factory=list)  # chunks of (steps, 2) float32: V, I of the scene's port
    done: bool = False
    rung_down: bool = False  # False when done at the step cap
    wall_s: float = 0.0
    sweep: dict | None = None
    accepted: bool = False  # stopped at its decision step (BatchRunner decide): no sweep of its own
    far: dict = field(default_factory=dict)  # far-field spectra by step (BatchRunner far_field)


def sweep_sums(series: np.ndarray, lambda_min: float, lambda_max: float, points: int, dt: float) -> np.ndarray:
    """(points, 4): Re V(f), Im V(f), Re I(f), Im I(f) of one port series (Ports.cpp:187-238; the
    library's sweep_kernel computes the same sums on the device). I is shifted by half a step."""
    nu_lo = 1.0 / max(lambda_max, lambda_min)
    nu_hi = 1.0 / min(lambda_max, lambda_min)
    nu = nu_lo + (nu_hi - nu_lo) * np.arange(points) / (points - 1)
    w = 2.0 * math.pi * nu
    k = np.arange(series.shape[0], dtype=np.float64)
    ph = -np.outer(w * dt, k)
    c, s = np.cos(ph), np.sin(ph)
    V = series[:, 0].astype(np.float64)
    I = series[:, 1].astype(np.float64)
    out = np.empty((points, 4))
    out[:, 0], out[:, 1] = c @ V, s @ V
    ic, is_ = c @ I, s @ I
    ch, sh = np.cos(w * 0.5 * dt), np.sin(w * 0.5 * dt)
    out[:, 2] = ic * ch - is_ * sh
    out[:, 3] = ic * sh + is_ * ch
    return out


def impedance(sums: np.ndarray, lambda_min: float, lambda_max: float, z0: float = 50.0):
    """Z(f) (ohm), S11 (dB) and the best-match wavelength from sweep sums (Ports.cpp:240-278)."""
    pts = sums.shape[0]
    nu_lo = 1.0 / max(lambda_max, lambda_min)
    nu_hi = 1.0 / min(lambda_max, lambda_min)
    nu = nu_lo + (nu_hi - nu_lo) * np.arange(pts) / (pts - 1)
    sv = sums[:, 0] + 1j * sums[:, 1]
    si = sums[:, 2] + 1j * sums[:, 3]
    z = np.where(np.abs(si) > 1e-30, -sv / np.where(np.abs(si) > 1e-30, si, 1.0) * K_ETA0, 0.0)
    g = np.abs((z - z0) / (z + z0))
    s11 = np.where(g > 1e-12, 20.0 * np.log10(np.maximum(g, 1e-300)), -200.0)
    return {"nu": nu, "z": z, "s11": s11, "best_wl": float(1.0 / nu[int(np.argmin(s11))])}


def scene_sweep(sc, series: np.ndarray, dt: float):
    sw = sc.sweep
    sums = sweep_sums(series, sw["wavelength_min"], sw["wavelength_max"], int(sw["points"]), dt)
    z0 = float(sc.ports[0].impedance_ohm) if sc.ports else 50.0
    return impedance(sums, sw["wavelength_min"], sw["wavelength_max"], z0)


class FarField:
    """The far-field spectra a batched run records per scene: a Huygens box just inside the scene's
    absorber (FarFieldMonitor::configure's box, FarField.cpp:126-174) with the multi-frequency DFT
    at `nf` frequencies uniform in 1/lambda over the scene's port sweep band, evaluated over a fixed
    grid of directions (polar angle 5..175 deg and azimuth 0..350 deg in 10-degree steps, plus the
    poles). A scene's spectra are, per frequency, the largest directivity over those directions in
    dBi (D = k^2 |N_perp - r x L|^2 / (8 pi P), FarField.cpp:198-217) and the radiated energy
    10 log10(P_sum / lambda0^2) dB, P_sum the radiated power of the unscaled DFT sums: the energy
    the pulse has radiated at that frequency, over the square of the design wavelength (the feed's
    pulse lasts a fixed number of periods, so its energy spectrum scales with lambda0^2)."""

    def __init__(self, nf: int = 32, block: int = 64):
        self.nf = int(nf)
        self.block = int(block)  # samples per fold: 64 keeps the per-node time block small
        th = np.radians(np.arange(5.0, 180.0, 10.0))
        ph = np.radians(np.arange(0.0, 360.0, 10.0))
        t, p = np.meshgrid(th, ph, indexing="ij")
        d = np.stack([np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)], axis=-1).reshape(-1, 3)
        self.dirs = np.concatenate([d, [[0.0, 0.0, 1.0], [0.0, 0.0, -1.0]]]).astype(np.float32)

    def wavelengths(self, sc):
        sw = sc.sweep
        nu_lo = 1.0 / max(sw["wavelength_max"], sw["wavelength_min"])
        nu_hi = 1.0 / min(sw["wavelength_max"], sw["wavelength_min"])
        return 1.0 / (nu_lo + (nu_hi - nu_lo) * np.arange(self.nf) / max(self.nf - 1, 1))

    @staticmethod
    def box(sc, z0: int = 0):
        """The scene's Huygens box in stack coordinates (its first plane at z0)."""
        n, L = sc.grid.size, int(sc.grid.pml_thickness)
        return [L + 1, L + 1, z0 + L + 1, n[0] - L - 2, n[1] - L - 2, z0 + n[2] - L - 2]

    def spectra(self, sc, out: np.ndarray, samples: int):
        """(D_max dBi, radiated energy dB) per frequency from an evaluation (nf, dirs, 2) of the sums
        scaled by 2 / samples."""
        wl = self.wavelengths(sc)
        k = 2.0 * math.pi / wl
        P = out[:, 0, 1].astype(np.float64)
        F2 = out[:, :, 0].astype(np.float64).max(axis=1)
        ok = P > 1e-30
        d = np.where(ok, k * k * F2 / (8.0 * math.pi * np.where(ok, P, 1.0)), 0.0)
        dbi = np.where(d > 1e-12, 10.0 * np.log10(np.maximum(d, 1e-300)), -120.0)
        energy = P * (0.5 * samples) ** 2 / float(sc.wavelength) ** 2
        db = np.where(energy > 1e-30, 10.0 * np.log10(np.maximum(energy, 1e-300)), -300.0)
        return np.stack([dbi, db]).astype(np.float32)


def residual(v: np.ndarray) -> float:
    """The reference's ring-down residual of a port voltage series (PortMonitor::evaluateSweep,
    Ports.cpp:206-213): the largest |V| of the last max(n / 20, 1) samples over the largest |V| of
    all n (1 without signal). emlab_ports_residuals computes the same on the device."""
    a = np.abs(np.asarray(v, np.float32))
    if a.size == 0:
        return 1.0
    peak = float(a.max())
    return float(a[a.size - max(a.size // 20, 1):].max()) / peak if peak > 0.0 else 1.0


class RingDown:
    """-60 dB watch on one port voltage with the reference's criterion: the sweep has settled once
    the residual (largest |V| of the last 5 % of the series over its peak, Ports.cpp:206-213) is at
    most -60 dB, checked wherever the runner reads the series; at least `min_steps` must have run,
    and the watch gives up (not rung down) at `max_steps`."""

    def __init__(self, min_steps: int, max_steps: int = 1 << 62, db: float = DB_RINGDOWN):
        self.min_steps, self.max_steps = int(min_steps), int(max_steps)
        self.ratio = 10.0 ** (db / 20.0)
        self.peak = 0.0
        self.steps = 0
        self.parts = []  # |V| of the series so far, in the chunks it arrived in

    def feed(self, v: np.ndarray) -> bool:
        a = np.abs(np.asarray(v, np.float32))
        if a.size:
            self.parts.append(a)
            self.peak = max(self.peak, float(a.max()))
        self.steps += a.size
        return self.done()

    def residual(self) -> float:
        if not (self.peak > 0.0):
            return 1.0
        tail, late, k = max(self.steps // 20, 1), 0.0, len(self.parts) - 1
        while tail > 0 and k >= 0:  # the last `tail` samples, from the newest chunk backwards
            part = self.parts[k][-tail:]
            late = max(late, float(part.max()))
            tail -= part.size
            k -= 1
        return late / self.peak

    def rung_down(self) -> bool:
        return self.peak > 0.0 and self.steps >= self.min_steps and self.residual() <= self.ratio

    def done(self) -> bool:
        return self.steps >= self.max_steps or self.rung_down()


MAX_PERIODS = 120  # a scene that has not rung down after this many design periods stops there (flagged)


def _watch(sc, dt: float) -> RingDown:
    period = sc.wavelength / dt  # steps per period of the design wavelength
    return RingDown(min_steps=int(math.ceil(4.0 * period)), max_steps=int(math.ceil(MAX_PERIODS * period)))


TILINGS = (64, 32, 128, 8)  # 64 x 8, 64 x 4, 64 x 16 pair tiles; 32 x 8 single-cell tiles
PAIR_TILINGS = (64, 32, 128)  # a stack of scenes with their own cross-sections: pair tiles only


def autotune_tiling(grid, modes=TILINGS, steps=4):
    """Times a few steps of the solver pass under each tiling (CUDA events around the launches) and
    keeps the fastest; the fields and the step count are reset afterwards, so the run starts as if
    untouched. Returns {mode: ms per launch} and leaves the best mode set."""
    times = {}
    for m in modes:
        grid.set_tiling(m)
        grid.step(1)  # first launch of a mode: attribute set-up outside the timing
        grid.set_timing(True)
        grid.kernel_time(reset=True)
        grid.step(steps)
        ms, n = grid.kernel_time(reset=True)
        grid.set_timing(False)
        times[m] = ms / max(n, 1)
    best = min(times, key=times.get)
    grid.set_tiling(best)
    grid.reset_fields()
    return times


class _Group:
    def __init__(self, scenes, indices, chunk, tune=True, far=None, ragged=False):
        self.indices = list(indices)  # scene indices into the batch, in stack order
        self.scenes = [scenes[i] for i in indices]
        first = self.scenes[0]
        if ragged:
            self.stack = SceneStack(first.grid, scene_dims=[tuple(sc.grid.size) for sc in self.scenes])
        else:
            self.stack = SceneStack(first.grid, [sc.grid.size[2] for sc in self.scenes])
        for k, sc in enumerate(self.scenes):
            m = sc.materials
            self.stack.upload_scene_materials(k, m.sigma, m.epsilon_r, sc.edges, sc.wires)
        self.stack.set_scene_sources([sc.sources for sc in self.scenes])
        self.stack.commit()
        self.tiling = autotune_tiling(self.stack, PAIR_TILINGS if ragged else TILINGS) if tune else None
        self.chunk = chunk
        self.stack.set_graph(chunk)  # each chunk replays one captured graph of its launches
        self.attach_ports()
        self.far = far
        if far is not None:
            z0, _ = self.stack.layout()
            self.stack.ntff_dft_configure_boxes([far.box(sc, z) for sc, z in zip(self.scenes, z0)],
                                                far.wavelengths(first), block=far.block)

    def attach_ports(self):
        z0, _ = self.stack.layout()
        ports = []
        for k, sc in enumerate(self.scenes):
            p = sc.ports[0]
            ports.append(abi.Port(int(p.texel[0]), int(p.texel[1]), int(p.texel[2]) + z0[k], int(p.axis),
                                  int(p.edges), 1 if p.sign >= 0 else -1))
        self.stack.ports_configure(ports, self.scenes[0].wavelength, 4.0, False, self.chunk)

    def far_spectra(self, k: int):
        """The far-field spectra of the stack's scene k now."""
        _, samples = self.stack.ntff_dft_info()
        return self.far.spectra(self.scenes[k], self.stack.ntff_dft_spectra(k, self.far.dirs), samples)

    def compact(self, keep):
        self.stack.compact(keep)  # the far-field boxes of the kept scenes keep their sums
        self.indices = [i for i, k in zip(self.indices, keep) if k]
        self.scenes = [s for s, k in zip(self.scenes, keep) if k]
        self.attach_ports()


class BatchRunner:
    """Steps `scenes` (each with one feed port) to port ring-down in stacks grouped by cross-section."""

    def __init__(self, scenes, chunk: int = 64, max_steps: int = 200_000, compact_fraction: float = 0.25,
                 stop_steps=None, tune: bool = True, decide_at=None, decide=None, far_field=None, snap_at=None,
                 layout: str = "ragged"):
        """stop_steps: per scene, stop after this many steps without waiting for the ring-down (the
        early window of a learned extrapolation); None: run every scene to ring-down.
        decide_at / decide: once scene i has run decide_at[i] steps (at a chunk boundary) without
        ringing down, decide(indices, series[, spectra]) is called for the scenes of a stack that reached it in
        the same chunk (under the runner's lock) and returns one flag per scene: True stops the scene
        there (result.accepted), False lets it run on to ring-down from where it is.
        far_field: a FarField; every scene then records its far-field spectra (result.far[step]) when
        it is done and, with snap_at (per scene, a list of steps), at each of those steps on the way.
        The boxes of one stack share the DFT's frequencies, so scenes of other sweep bands go to other
        stacks.
        layout: "ragged" (scenes of all cross-sections in one stack per solver setting) or
        "cross_section" (one stack per (nx, ny))."""
        if layout not in ("ragged", "cross_section"):
            raise ValueError("layout must be 'ragged' or 'cross_section'")
        for sc in scenes:
            if not sc.ports:
                raise ValueError(f"{sc.name}: a batched scene needs a feed port")
        self.scenes = list(scenes)
        self.chunk = int(chunk)
        self.max_steps = int(max_steps)
        self.compact_fraction = float(compact_fraction)
        self.far = far_field
        if far_field is not None and decide_at is not None:  # decide() sees the decision step's spectra
            snap_at = [list(a) + [d] for a, d in zip(snap_at or [[]] * len(self.scenes), decide_at)]
        self.snap_at = [sorted(set(int(v) for v in a)) for a in snap_at] if snap_at is not None else None
        groups = {}
        ragged = layout == "ragged"
        for i, sc in enumerate(self.scenes):
            key = (sc.grid.pml_thickness, float(sc.grid.courant), float(sc.grid.pml_sigma_max),
                   float(sc.grid.pml_grading))
            if not ragged:
                key += (sc.grid.size[0], sc.grid.size[1])
            if far_field is not None:  # the boxes of one stack share the DFT frequencies
                key += tuple(float(v) for v in far_field.wavelengths(sc))
            groups.setdefault(key, []).append(i)
        t0 = time.perf_counter()
        self.groups = [_Group(self.scenes, idx, self.chunk, tune, far_field, ragged) for _, idx in
                       sorted(groups.items(), key=lambda kv: kv[0])]
        self.setup_s = time.perf_counter() - t0
        self.results = [SceneResult(i) for i in range(len(self.scenes))]
        self.stop_steps = list(stop_steps) if stop_steps is not None else None
        self.decide_at = list(decide_at) if decide_at is not None else None
        self.decide = decide
        self.decided = [False] * len(self.scenes)
        if stop_steps is None:
            self.watch = [_watch(sc, float(sc.grid.courant)) for sc in self.scenes]
        else:
            self.watch = [RingDown(min_steps=int(n), max_steps=int(n)) for n in stop_steps]
        self.cell_steps = 0
        self.steps = 0
        self.host_s = 0.0     # host seconds between a chunk's read-back and the next chunk's launch
        self.compact_s = 0.0  # of which in compaction

    def _next_chunk(self, g, steps):
        """Steps of the stack's next chunk after the `steps` already queued (every scene of a stack
        has run the same steps): up to the next multiple of the chunk length (a whole chunk replays
        one captured graph), or fewer when a scene's stop, decision or snapshot step comes sooner,
        so an early window ends exactly there and the chunk grid stays where it was."""
        n = self.chunk - steps % self.chunk
        for i in g.indices:
            if self.results[i].done:
                continue
            for marks in (self.stop_steps, None if self.decide_at is None or self.decided[i] else self.decide_at):
                if marks is not None and marks[i] > steps:
                    n = min(n, marks[i] - steps)
            if self.snap_at is not None:
                later = [v for v in self.snap_at[i] if v > steps]
                if later:
                    n = min(n, later[0] - steps)
        return n

    def _compact_now(self, g, keep) -> bool:
        """Compact once the finished scenes hold compact_fraction of the stack's cells (their steps
        are wasted until then; each compaction copies the rest of the stack)."""
        cells = [int(np.prod(sc.grid.size)) for sc in g.scenes]
        done = sum(c for c, k in zip(cells, keep) if not k)
        return done > 0 and done >= self.compact_fraction * sum(cells)

    def _process(self, g, ser, t0, on_done, lock):
        """One chunk's port series of stack g: watch every scene, evaluate the finished ones, call
        decide() for the scenes at their decision step."""
        cells = sum(int(np.prod(sc.grid.size)) for sc in g.scenes) * ser.shape[0]  # the scenes' own cells
        finished = []
        for k, i in enumerate(g.indices):
            r = self.results[i]
            if r.done:
                continue
            r.series.append(ser[:, k].copy())
            r.steps += ser.shape[0]
            if self.snap_at is not None and r.steps in self.snap_at[i]:
                r.far[r.steps] = g.far_spectra(k)
            # the ring-down watch concludes only at whole chunks, as in a run without stop or
            # decision steps; a stop step ends the scene wherever it falls
            fed = self.watch[i].feed(ser[:, k, 0])
            if fed and (self.stop_steps is not None or r.steps % self.chunk == 0):
                r.done = True
                r.rung_down = self.watch[i].rung_down()
                r.wall_s = time.perf_counter() - t0
                sc = self.scenes[i]
                r.sweep = scene_sweep(sc, np.concatenate(r.series), float(sc.grid.courant))
                if g.far is not None and r.steps not in r.far:
                    r.far[r.steps] = g.far_spectra(k)
                finished.append(i)
        pending = [i for i in g.indices if self.decide_at is not None and not self.results[i].done
                   and not self.decided[i] and self.results[i].steps >= self.decide_at[i]]
        with lock:
            if pending:
                args = (pending, [np.concatenate(self.results[i].series) for i in pending])
                if self.far is not None:
                    args += ([self.results[i].far.get(self.decide_at[i]) for i in pending],)
                flags = self.decide(*args)
                for i, stop in zip(pending, flags):
                    self.decided[i] = True
                    if stop:
                        r = self.results[i]
                        r.done = r.accepted = True
                        r.wall_s = time.perf_counter() - t0
                        finished.append(i)
            self.cell_steps += cells
            if on_done:
                for i in finished:
                    on_done(i, self.results[i])

    def _run_group(self, g, t0, on_done, lock):
        """One stack's loop (its own host thread and CUDA stream): step a chunk, read the chunk's port
        series back, watch every scene, evaluate the finished ones, compact. The library releases the
        interpreter lock inside its calls, so the stacks' chunks overlap on the device.

        Without far-field monitors the loop runs one chunk ahead: chunk n+1 is queued before the
        series of chunk n is processed (asynchronous takes), so the device never waits for the host.
        A scene found done in chunk n has been stepped through chunk n+1 as well; that chunk's rows
        are not added to its series (its results are those of the chunk that finished it), and the
        compaction waits until the chunk in flight has been processed. With far-field monitors every
        chunk is processed before the next is queued (a snapshot reads the sums at its own step)."""
        from collections import deque
        steps = 0
        host = comp = 0.0
        ahead = 1 if self.far is None else 0
        inflight = deque()  # (slot, steps) of queued chunks not processed yet
        while True:
            while g.indices and steps < self.max_steps and len(inflight) <= ahead:
                n = self._next_chunk(g, steps)
                g.stack.step(n)
                inflight.append(g.stack.ports_take_series_async())
                steps += n
            if not inflight:
                break
            slot, rows = inflight.popleft()
            ser = g.stack.ports_collect_series(slot, rows)
            th = time.perf_counter()
            self._process(g, ser, t0, on_done, lock)
            keep = [not self.results[i].done for i in g.indices]
            if not any(keep) or self._compact_now(g, keep):
                while inflight:  # the chunk in flight ran with this layout: process it first
                    slot, rows = inflight.popleft()
                    self._process(g, g.stack.ports_collect_series(slot, rows), t0, on_done, lock)
                keep = [not self.results[i].done for i in g.indices]
                if not any(keep):
                    g.indices = []
                else:
                    tc = time.perf_counter()
                    g.compact(keep)
                    comp += time.perf_counter() - tc
            host += time.perf_counter() - th
        with lock:
            self.steps = max(self.steps, steps)
            self.host_s += host
            self.compact_s += comp

    def run(self, on_done=None):
        import threading
        t0 = time.perf_counter()
        lock = threading.Lock()
        errors = []

        def body(g):
            try:
                self._run_group(g, t0, on_done, lock)
            except BaseException as e:  # re-raised on the calling thread
                errors.append(e)
        threads = [threading.Thread(target=body, args=(g,)) for g in self.groups]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        self.wall_s = time.perf_counter() - t0
        if errors:
            raise errors[0]
        return self.results

    def close(self):
        for g in self.groups:
            g.stack.close()


def run_single(sc, chunk: int = 64, max_steps: int = 200_000, timing: dict | None = None, far_field=None):
    """One scene on its own SimulationGrid to the same ring-down rule: (series (steps, 2), sweep).
    `timing`, if given, receives the set-up and the stepping wall-clock seconds and the steps. With a
    FarField the grid carries its Huygens box and sweep["far"] holds the spectra at the end."""
    t0 = time.perf_counter()
    g = SimulationGrid(sc.grid)
    m = sc.materials
    g.upload_materials(m.sigma, m.epsilon_r, sc.edges, sc.wires)
    g.set_sources(sc.sources)
    g.ports_configure([sc.ports[0].to_c()], sc.wavelength, 4.0, False, chunk)
    g.set_graph(chunk)
    if far_field is not None:
        g.ntff_dft_configure_boxes([far_field.box(sc)], far_field.wavelengths(sc), block=far_field.block)
    g.synchronize()
    t1 = time.perf_counter()
    dt = float(sc.grid.courant)
    watch = _watch(sc, dt)
    parts = []
    steps = 0
    while steps < max_steps:
        g.step(chunk)
        ser = g.ports_take_series(chunk)
        parts.append(ser[:, 0].copy())
        steps += ser.shape[0]
        if watch.feed(ser[:, 0, 0]):
            break
    series = np.concatenate(parts)
    sweep = scene_sweep(sc, series, dt)
    if far_field is not None:
        sweep["far"] = far_field.spectra(sc, g.ntff_dft_spectra(0, far_field.dirs), g.ntff_dft_info()[1])
    t2 = time.perf_counter()
    g.close()
    if timing is not None:
        timing.update(setup_s=t1 - t0, run_s=t2 - t1, steps=steps)
    return series, sweep
