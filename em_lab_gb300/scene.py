"""Scene description for the solver: materials, sources, thin wires, feeds and ports.

Mirrors the parts of src/Environment.{hpp,cpp}, src/SimulationGrid.{hpp,cpp} (MaterialVolume,
SourceDesc and its factories) and src/ScriptEngine.cpp (material resolution, addThinWire,
addFeed, dipoleArm, buildDipole, emitThinWires) that produce the solver's inputs, with the
reference's float32 arithmetic. The output of `EnvironmentBuilder.build()` is exactly what
SimulationGrid::uploadMaterials / setSources and the monitors' configure calls consume.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi

f32 = np.float32
K_ETA0 = 376.730313668                 # free-space impedance, ohm (ScriptEngine.cpp:26)
K_ETA0_F = f32(376.730313668)
K_PERFECT_EDGE_SIGMA = f32(6.0e4)      # SimulationGrid.hpp:103
K_DIPOLE_SOFTNESS = f32(0.75)          # SimulationGrid.hpp:114
K_SHEET_SOFTNESS = f32(1.0)


# ---------------------------------------------------------------------------------------------
@dataclass
class Material:
    """Material (src/SimulationGrid.hpp:36-44): normalised conductivity and relative permittivity."""

    sigma: float = 0.0
    epsilon_r: float = 1.0


def resolve_material(eps_r, cell_size, wavelength, sigma_norm=None, conductivity=None, loss_tangent=None) -> Material:
    """resolve (ScriptEngine.cpp:458-465): S/m -> sigma * dx * eta0; loss tangent -> tan d * k * eps_r."""
    sigma = 0.0
    if sigma_norm is not None:
        sigma = sigma_norm
    elif conductivity is not None:
        sigma = conductivity * float(f32(cell_size)) * K_ETA0
    elif loss_tangent is not None:
        sigma = loss_tangent * (2.0 * math.pi / float(f32(wavelength))) * float(f32(eps_r))
    return Material(float(f32(sigma)), float(max(f32(eps_r), f32(1.0))))


class MaterialVolume:
    """MaterialVolume (src/SimulationGrid.hpp:46-69): per-cell sigma (>= 0) and eps_r (>= 1)."""

    def __init__(self, size):
        self.size = tuple(int(max(s, 0)) for s in size)
        nx, ny, nz = self.size
        self.sigma = np.zeros((nz, ny, nx), np.float32)
        self.epsilon_r = np.ones((nz, ny, nx), np.float32)

    def set_mask(self, mask_zyx, lo, m: Material):
        """MaterialVolume::set on every cell of a boolean block whose (x,y,z) origin is `lo`."""
        nz, ny, nx = mask_zyx.shape
        sl = (slice(lo[2], lo[2] + nz), slice(lo[1], lo[1] + ny), slice(lo[0], lo[0] + nx))
        self.sigma[sl][mask_zyx] = max(f32(m.sigma), f32(0.0))
        self.epsilon_r[sl][mask_zyx] = max(f32(m.epsilon_r), f32(1.0))
        return int(mask_zyx.sum())

    def get(self, p) -> Material:
        x, y, z = p
        nx, ny, nz = self.size
        if not (0 <= x < nx and 0 <= y < ny and 0 <= z < nz):
            return Material()
        return Material(float(self.sigma[z, y, x]), float(self.epsilon_r[z, y, x]))


# ---------------------------------------------------------------------------------------------
class BoxShape:
    """BoxShape (Environment.hpp:42-51): p >= min && p < max."""

    def __init__(self, mn, mx):
        mn, mx = np.asarray(mn, f32), np.asarray(mx, f32)
        self.min, self.max = np.minimum(mn, mx), np.maximum(mn, mx)

    def bounds(self):
        return self.min, self.max

    def contains(self, x, y, z):
        return ((x >= self.min[0]) & (y >= self.min[1]) & (z >= self.min[2]) & (x < self.max[0]) &
                (y < self.max[1]) & (z < self.max[2]))


class EllipsoidShape:
    """EllipsoidShape (Environment.hpp:54-61): |(p - c) / r|^2 <= 1."""

    def __init__(self, c, radii):
        self.c = np.asarray(c, f32)
        self.r = np.maximum(np.asarray(radii, f32), f32(1e-3))

    def bounds(self):
        return self.c - self.r, self.c + self.r

    def contains(self, x, y, z):
        dx = (x - self.c[0]) / self.r[0]
        dy = (y - self.c[1]) / self.r[1]
        dz = (z - self.c[2]) / self.r[2]
        return (dx * dx + dy * dy) + dz * dz <= f32(1.0)


class CylinderShape:
    """CylinderShape (Environment.hpp:64-75, Environment.cpp:11-22): |axial| <= h and radial^2 <= r^2."""

    def __init__(self, c, axis, radius, half_length):
        self.c = np.asarray(c, f32)
        self.axis = int(axis)
        self.r = f32(radius)
        self.h = f32(half_length)

    def bounds(self):
        ext = np.full(3, self.r, f32)
        ext[self.axis] = self.h
        return self.c - ext, self.c + ext

    def contains(self, x, y, z):
        d = [x - self.c[0], y - self.c[1], z - self.c[2]]
        a = d[self.axis]
        r2 = ((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) - a * a
        return (np.abs(a) <= self.h) & (r2 <= self.r * self.r)


class DifferenceShape:
    """DifferenceShape (Environment.hpp:92-100): in `a` and not in `b`; bounds of `a`."""

    def __init__(self, a, b):
        self.a, self.b = a, b

    def bounds(self):
        return self.a.bounds()

    def contains(self, x, y, z):
        return self.a.contains(x, y, z) & ~self.b.contains(x, y, z)


def rotation_from_euler_degrees(deg):
    """rotationFromEulerDegrees (Environment.cpp:66-71): R = Rz Ry Rx (x first, then y, then z)."""
    ax, ay, az = (math.radians(float(f32(v))) for v in deg)
    cx, sx, cy, sy, cz, sz = math.cos(ax), math.sin(ax), math.cos(ay), math.sin(ay), math.cos(az), math.sin(az)
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return (rz @ ry @ rx).astype(f32)


class TransformedShape:
    """TransformedShape (Environment.hpp:78-89, Environment.cpp:24-39): a local shape around the
    origin, rotated and moved to `center`; bounds = the rotated local box's 8 corners."""

    def __init__(self, local, center, rotation):
        self.local = local
        self.center = np.asarray(center, f32)
        self.rot = np.asarray(rotation, f32)
        self.inv = self.rot.T
        lo, hi = local.bounds()
        corners = np.array([[hi[0] if i & 1 else lo[0], hi[1] if i & 2 else lo[1], hi[2] if i & 4 else lo[2]]
                            for i in range(8)], f32)
        w = self.center + corners @ self.rot.T
        self.lo, self.hi = w.min(axis=0), w.max(axis=0)

    def bounds(self):
        return self.lo, self.hi

    def contains(self, x, y, z):
        d = [x - self.center[0], y - self.center[1], z - self.center[2]]
        m = self.inv
        lx = (m[0, 0] * d[0] + m[0, 1] * d[1]) + m[0, 2] * d[2]
        ly = (m[1, 0] * d[0] + m[1, 1] * d[1]) + m[1, 2] * d[2]
        lz = (m[2, 0] * d[0] + m[2, 1] * d[1]) + m[2, 2] * d[2]
        return self.local.contains(lx, ly, lz)


class WallShape:
    """WallShape (Environment.hpp:115-135, Environment.cpp:41-64): the slab [x0, x1) normal to
    `axis` minus rectangular (|d| < half size) and circular (|d|^2 <= r^2) apertures."""

    def __init__(self, axis, x0, x1, apertures, grid_size):
        self.axis = min(max(int(axis), 0), 2)
        self.u = 1 if self.axis == 0 else 0
        self.v = 1 if self.axis == 2 else 2
        self.x0, self.x1 = f32(min(x0, x1)), f32(max(x0, x1))
        self.apertures = apertures  # dicts: circular, center (u, v), half (u, v), radius
        self.lo = np.zeros(3, f32)
        self.hi = np.asarray(grid_size, f32).copy()
        self.lo[self.axis], self.hi[self.axis] = self.x0, self.x1

    def bounds(self):
        return self.lo, self.hi

    def contains(self, x, y, z):
        p = (x, y, z)
        a = p[self.axis]
        inside = (a >= self.x0) & (a < self.x1)
        tu, tv = p[self.u], p[self.v]
        for ap in self.apertures:
            du, dv = tu - f32(ap["center"][0]), tv - f32(ap["center"][1])
            if ap["circular"]:
                hole = du * du + dv * dv <= f32(ap["radius"]) * f32(ap["radius"])
            else:
                hole = (np.abs(du) < f32(ap["half"][0])) & (np.abs(dv) < f32(ap["half"][1]))
            inside &= ~hole
        return inside


class LambdaShape:
    """LambdaShape (Environment.hpp:102-110): a predicate over cell centres within given bounds.
    `fn(x, y, z)` takes arrays and returns a boolean array."""

    def __init__(self, lo, hi, fn):
        self.lo, self.hi = np.asarray(lo, f32), np.asarray(hi, f32)
        self.fn = fn

    def bounds(self):
        return self.lo, self.hi

    def contains(self, x, y, z):
        return self.fn(x, y, z)


# ---------------------------------------------------------------------------------------------
@dataclass
class SourceDesc:
    """SourceDesc (src/SimulationGrid.hpp:113-150)."""

    center: tuple = (0.0, 0.0, 0.0)
    half_extent: tuple = (0.0, 0.0, 0.0)
    softness: tuple = (0.75, 0.75, 0.75)
    polarization: tuple = (0.0, 0.0, 1.0)
    amplitude: float = 1.0
    wavelength: float = 16.0
    phase: float = 0.0
    waveform: int = abi.WAVE_CW
    ramp_periods: float = 3.0
    repeat_periods: float = 0.0
    delay_periods: float = 0.0
    enabled: bool = True
    emitter: int = -1
    port: int = -1

    @staticmethod
    def wire_current_density(current, softness):
        """SourceDesc::wireCurrentDensity (SimulationGrid.cpp:65-68)."""
        s = max(f32(softness), f32(0.25))
        return f32(current) / (f32(math.pi) * s * s)

    @staticmethod
    def dipole(center, axis, wavelength, current, length=0.0) -> "SourceDesc":
        """SourceDesc::dipole (SimulationGrid.cpp:70-82)."""
        ax = np.asarray(axis, f32)
        len2 = f32(ax[0] * ax[0] + ax[1] * ax[1]) + ax[2] * ax[2]
        n = ax / np.sqrt(len2) if len2 > 0 else np.array([0, 0, 1], f32)
        he = np.abs(n) * (f32(0.5) * max(f32(length), f32(0.0)))
        return SourceDesc(center=tuple(float(v) for v in np.asarray(center, f32)),
                          half_extent=tuple(float(v) for v in he),
                          softness=(float(K_DIPOLE_SOFTNESS),) * 3,
                          polarization=tuple(float(v) for v in ax),
                          amplitude=float(SourceDesc.wire_current_density(current, K_DIPOLE_SOFTNESS)),
                          wavelength=float(wavelength))

    def to_c(self) -> abi.Source:
        s = abi.Source()
        for i in range(3):
            s.center[i] = self.center[i]
            s.half_extent[i] = self.half_extent[i]
            s.softness[i] = self.softness[i]
            s.polarization[i] = self.polarization[i]
        s.amplitude = self.amplitude
        s.wavelength = self.wavelength
        s.phase = self.phase
        s.waveform = int(self.waveform)
        s.ramp_periods = self.ramp_periods
        s.repeat_periods = self.repeat_periods
        s.delay_periods = self.delay_periods
        s.enabled = 1 if self.enabled else 0
        return s


@dataclass
class PortSetup:
    """PortSetup (src/Ports.hpp:30-40)."""

    name: str
    texel: tuple
    axis: int = 2
    sign: float = 1.0
    edges: int = 1
    wavelength: float = 16.0
    voltage_feed: bool = True
    impedance_ohm: float = 50.0
    drive: float = 1.0

    def to_c(self) -> abi.Port:
        return abi.Port(int(self.texel[0]), int(self.texel[1]), int(self.texel[2]), int(self.axis), int(self.edges),
                        1 if self.sign >= 0 else -1)


@dataclass
class ThinWireSpec:
    node: tuple
    axis: int
    i0: int
    i1: int
    radius: float
    gap_edge: int | None = None


@dataclass
class FluxSetup:
    """FluxSetup / FluxSurface (Environment.hpp, FieldAnalyzer.hpp:28-45): a plane (axis, index,
    rectangle in the two tangential coordinates) or a closed box (outward normal)."""

    name: str
    kind: str = "box"                  # "box" or "plane"
    box_min: tuple = (0, 0, 0)
    box_max: tuple = (0, 0, 0)
    axis: int = 0
    index: int = 0
    rect_min: tuple = (0, 0)
    rect_max: tuple = (0, 0)
    log: str = ""

    def planes(self):
        """(sign, axis, index, rect_min, rect_max) per plane; a box has six with outward signs
        (FieldAnalyzer.cpp:175-190)."""
        if self.kind == "plane":
            return [(1.0, self.axis, self.index, self.rect_min, self.rect_max)]
        out = []
        for ax in range(3):
            u, v = (1, 2) if ax == 0 else ((0, 2) if ax == 1 else (0, 1))
            rmin = (self.box_min[u], self.box_min[v])
            rmax = (self.box_max[u] + 1, self.box_max[v] + 1)
            out.append((-1.0, ax, self.box_min[ax], rmin, rmax))
            out.append((1.0, ax, self.box_max[ax], rmin, rmax))
        return out


@dataclass
class CoaxSetup:
    """CoaxSetup (src/Coax.hpp:25-45): a voxel coaxial cable and what its monitor needs."""

    name: str
    axis: int = 0
    sign: int = 1
    start: int = 0
    center: tuple = (0.0, 0.0, 0.0)
    length: int = 0
    inner: int = 1
    outer: int = 5
    wall: int = 1
    sleeve_start: int = -1
    sleeve_end: int = -1
    sleeve_outer: int = 0
    epsilon_r: float = 1.0
    z0_ohm: float = 50.0
    wavelength: float = 16.0
    cell_size: float = 1e-3
    termination: str = "load"
    source_ohm: float = 50.0
    load_ohm: float = 50.0
    drive: float = 1.0
    pulsed: bool = False


@dataclass
class Scene:
    """The solver-facing part of Environment (src/Environment.hpp:165-187)."""

    name: str
    grid: abi.GridConfig
    materials: MaterialVolume
    edges: list = field(default_factory=list)      # EdgeOverride
    wires: list = field(default_factory=list)      # WireTerm
    sources: list = field(default_factory=list)    # SourceDesc
    ports: list = field(default_factory=list)      # PortSetup
    probes: list = field(default_factory=list)     # (name, position)
    probe_logs: list = field(default_factory=list) # CSV path per probe ("" = none)
    fluxes: list = field(default_factory=list)     # FluxSetup
    far_field: dict | None = None                  # box_min, box_max, wavelength, averaging
    sweep: dict | None = None                      # wavelength_min, wavelength_max, points
    cell_size: float = 1.0e-3
    wavelength: float = 16.0
    description: str = ""
    view: dict = field(default_factory=dict)       # ViewHints used by the headless runner
    coaxes: list = field(default_factory=list)     # CoaxSetup
    radar: dict | None = None                      # RadarSetup (radar{})
    emitters: list = field(default_factory=list)   # EmitterSetup (emitter{})
    crpa: dict | None = None                       # CrpaSetup (crpa{})
    targets: list = field(default_factory=list)    # TargetInfo of target = true objects


class EnvironmentBuilder:
    """EnvironmentBuilder (src/Environment.hpp:189-212) plus the antenna helpers of ScriptEngine.cpp."""

    def __init__(self, name, grid: abi.GridConfig, cell_size=1.0e-3, wavelength=16.0):
        self.scene = Scene(name=name, grid=grid, materials=MaterialVolume(grid.size), cell_size=cell_size,
                           wavelength=wavelength)
        self.thin_wires: list[ThinWireSpec] = []

    # --- voxeliser (Environment.cpp:82-97) -------------------------------------------------------
    def fill(self, shape, m: Material) -> int:
        size = np.asarray(self.scene.grid.size)
        bmin, bmax = shape.bounds()
        lo = np.clip(np.floor(np.asarray(bmin, f32) - f32(0.5)).astype(np.int64), 0, size)
        hi = np.clip(np.ceil(np.asarray(bmax, f32) + f32(0.5)).astype(np.int64), 0, size)
        if np.any(hi <= lo):
            return 0
        xs = np.arange(lo[0], hi[0], dtype=f32) + f32(0.5)
        ys = np.arange(lo[1], hi[1], dtype=f32) + f32(0.5)
        zs = np.arange(lo[2], hi[2], dtype=f32) + f32(0.5)
        Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
        mask = shape.contains(X, Y, Z)
        return self.scene.materials.set_mask(mask, lo, m)

    def box(self, mn, mx, m):
        return self.fill(BoxShape(mn, mx), m)

    def sphere(self, c, r, m):
        return self.fill(EllipsoidShape(c, (r, r, r)), m)

    # --- antennas (ScriptEngine.cpp:1183-1287) -----------------------------------------------------
    def add_thin_wire(self, node, axis, i0, i1, radius, gap_edge=None):
        if i1 <= i0:
            return
        self.thin_wires.append(ThinWireSpec(tuple(int(v) for v in node), int(axis), int(i0), int(i1),
                                            float(f32(radius)), gap_edge))

    def add_feed(self, wave: SourceDesc, texel, axis, sign, edges, impedance_ohm=50.0, drive=1.0, voltage=True,
                 name="port"):
        """addFeed (ScriptEngine.cpp:1205-1253): Norton resistive voltage source + port."""
        u, v = (axis + 1) % 3, (axis + 2) % 3
        eu = [0, 0, 0]
        ev = [0, 0, 0]
        eu[u] = 1
        ev[v] = 1
        s = SourceDesc(**{k: getattr(wave, k) for k in wave.__dataclass_fields__})
        s.softness = (0.25, 0.25, 0.25)
        pol = [0.0, 0.0, 0.0]
        pol[axis] = float(sign)
        s.polarization = tuple(pol)
        t = np.asarray(texel, f32)
        if edges == 4:
            s.center = tuple(float(c) for c in t + f32(0.5))
            he = [0.5, 0.5, 0.5]
            he[axis] = 0.0
            s.half_extent = tuple(he)
        else:
            c = t.copy()
            c[axis] += f32(0.5)
            s.center = tuple(float(x) for x in c)
            s.half_extent = (0.0, 0.0, 0.0)
        if voltage:
            sigma = K_ETA0_F / (f32(edges) * f32(impedance_ohm))
            offs = [(0, 0, 0), tuple(eu), tuple(ev), tuple(a + b for a, b in zip(eu, ev))]
            for i in range(edges):
                p = [int(texel[k]) + offs[i][k] for k in range(3)]
                self.scene.edges.append(abi.EdgeOverride(p[0], p[1], p[2], int(axis), float(sigma)))
            s.amplitude = float(-sigma * f32(drive))
        else:
            s.amplitude = float(f32(drive) / f32(edges))
        s.port = len(self.scene.ports)
        if s.enabled:
            self.scene.sources.append(s)
        self.scene.ports.append(PortSetup(name, tuple(int(x) for x in texel), int(axis), float(sign), int(edges),
                                          float(wave.wavelength), voltage, float(impedance_ohm), float(drive)))

    @staticmethod
    def dipole_arm(length: float) -> int:
        """dipoleArm (ScriptEngine.cpp:1255-1269): two arms plus a one-cell feed gap."""
        half = (float(f32(length)) - 1.0) * 0.5
        return max(1, int(math.floor(half + 0.5)) if half >= 0 else -int(math.floor(-half + 0.5)))

    def thin_dipole(self, wave: SourceDesc, center, axis, length, radius=None, impedance_ohm=50.0, drive=1.0,
                    sign=1.0, name="dipole"):
        """buildDipole, thin-wire model (ScriptEngine.cpp:1271-1287)."""
        if radius is None:
            radius = wave.wavelength / 400.0
        arm = self.dipole_arm(length)
        c = np.asarray(center, f32)
        node = [int(math.floor(float(v) + 0.5)) if v >= 0 else -int(math.floor(-float(v) + 0.5)) for v in c]
        node[axis] = int(math.floor(float(c[axis])))
        g = node[axis]
        self.add_thin_wire(node, axis, g - arm, g + 1 + arm, radius, g)
        self.add_feed(wave, node, axis, sign, 1, impedance_ohm, drive, True, name)

    def emit_thin_wires(self):
        """emitThinWires (ScriptEngine.cpp:2346-2419): PEC edges, end correction, 2/ln(1/a) factors."""
        key = lambda p: (int(p[0]), int(p[1]), int(p[2]))
        nodes = []
        for t in self.thin_wires:
            s = set()
            for k in range(t.i0, t.i1 + 1):
                p = list(t.node)
                p[t.axis] = k
                s.add(key(p))
            nodes.append(s)
        sheet_nodes = set()
        for e in self.scene.edges:
            if e.sigma < 0.5 * float(K_PERFECT_EDGE_SIGMA):
                continue
            end = [e.x, e.y, e.z]
            end[e.axis] += 1
            sheet_nodes.add((e.x, e.y, e.z))
            sheet_nodes.add(key(end))
        mats = self.scene.materials

        def touches(self_idx, p):
            if key(p) in sheet_nodes:
                return True
            for w, s in enumerate(nodes):
                if w != self_idx and key(p) in s:
                    return True
            for dz in (-1, 0):
                for dy in (-1, 0):
                    for dx in (-1, 0):
                        if mats.get((p[0] + dx, p[1] + dy, p[2] + dz)).sigma >= 1.0:
                            return True
            return False

        for w, t0 in enumerate(self.thin_wires):
            t = ThinWireSpec(**t0.__dict__)
            a = list(t.node)
            b = list(t.node)
            a[t.axis] = t.i0
            b[t.axis] = t.i1
            free_a = not touches(w, a) and t.gap_edge != t.i0
            free_b = not touches(w, b) and t.gap_edge != t.i1 - 1
            keep = 2 if (t.gap_edge is not None and t.i0 <= t.gap_edge < t.i1) else 1
            if (t.i1 - t.i0) - (1 if free_a else 0) - (1 if free_b else 0) >= keep:
                if free_a:
                    t.i0 += 1
                if free_b:
                    t.i1 -= 1
            f = f32(2.0) / np.log(f32(1.0) / f32(t.radius))
            u, v = (t.axis + 1) % 3, (t.axis + 2) % 3
            term = lambda comp: 0 if (comp + 2) % 3 == t.axis else 1
            for k in range(t.i0, t.i1):
                q = list(t.node)
                q[t.axis] = k
                if k != t.gap_edge:
                    self.scene.edges.append(abi.EdgeOverride(q[0], q[1], q[2], t.axis, float(K_PERFECT_EDGE_SIGMA)))
                qv = list(q)
                qv[v] -= 1
                qu = list(q)
                qu[u] -= 1
                W = self.scene.wires
                W.append(abi.WireTerm(q[0], q[1], q[2], u, term(u), float(f)))
                W.append(abi.WireTerm(qv[0], qv[1], qv[2], u, term(u), float(f)))
                W.append(abi.WireTerm(q[0], q[1], q[2], v, term(v), float(f)))
                W.append(abi.WireTerm(qu[0], qu[1], qu[2], v, term(v), float(f)))
        self.thin_wires = []

    def build(self) -> Scene:
        self.emit_thin_wires()
        return self.scene
