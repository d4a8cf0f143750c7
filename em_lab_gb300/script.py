"""Scene scripts: the reference's Lua scene API over the solver's scene description.

Runs a scene file (scenes/*.lua of the reference) with the Lua subset of `lua.py` and turns its
calls into a `scene.Scene`: src/ScriptEngine.cpp (SceneSettings :90-101, Args :226-400, materials
:409-520, scene/view/material/param :605-842, geometry :843-1075, sources and antennas :1077-1460,
plane waves :1526-1590, instruments :1737-1805, far_field :2160-2190, final checks :2420-2520).
The vector prelude (vec, X/Y/Z, deg, wavelengths, meters, mm, lerp, clamp, range) is provided as
native functions with the same behaviour. Every function of the reference's API is
provided, loop{} and frame{} included (:1022-1030, :1456-1524).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .lua import Interpreter, LuaError, LuaFunction, LuaTable, tostr
from .scene import (K_PERFECT_EDGE_SIGMA, BoxShape, CoaxSetup, CylinderShape, DifferenceShape, EllipsoidShape,
                    EnvironmentBuilder, FluxSetup, LambdaShape, Material, SourceDesc, TransformedShape, WallShape,
                    rotation_from_euler_degrees)

f32 = np.float32
K_C0 = 299792458.0
K_ETA0 = 376.730313668
K_SHEET_SOFTNESS = 1.0   # SourceDesc::kSheetSoftness (SimulationGrid.hpp)
K_DIPOLE_SOFTNESS = 0.75

# name: (eps_r, sigma (normalised), conductivity (S/m), loss tangent) -- the built-in material library
BUILTIN_MATERIALS = {
    "vacuum": (1.0, 0.0, None, None), "air": (1.0, 0.0, None, None), "pec": (1.0, 1.0e7, None, None),
    "metal": (1.0, None, 5.8e7, None), "copper": (1.0, None, 5.8e7, None), "silver": (1.0, None, 6.3e7, None),
    "gold": (1.0, None, 4.1e7, None), "aluminum": (1.0, None, 3.77e7, None), "brass": (1.0, None, 1.5e7, None),
    "steel": (1.0, None, 1.45e6, None), "absorber": (1.0, 0.3, None, None), "ptfe": (2.1, None, None, 2e-4),
    "teflon": (2.1, None, None, 2e-4), "polyethylene": (2.25, None, None, 3e-4),
    "rexolite": (2.53, None, None, 5e-4), "polystyrene": (2.6, None, None, 5e-4),
    "acrylic": (2.6, None, None, 8e-3), "quartz": (3.8, None, None, 1e-4), "fr4": (4.4, None, None, 0.02),
    "glass": (6.3, None, 0.004, None), "alumina": (9.8, None, None, 1e-4), "silicon": (11.7, 0.0, None, None),
    "concrete": (5.24, None, 0.05, None), "brick": (3.91, None, 0.024, None), "wood": (1.99, None, 0.005, None),
    "drywall": (2.73, None, 0.0085, None), "ground_dry": (4.0, None, 0.001, None),
    "ground_wet": (25.0, None, 0.02, None), "water": (78.0, None, None, 0.1), "seawater": (74.0, None, 4.0, None),
}

WAVEFORM_KEYS = ["wavelength", "frequency", "phase", "waveform", "ramp", "pulse_width", "interval", "delay", "enabled"]


class ScriptError(Exception):
    pass


@dataclass
class Settings:
    name: str = "Untitled scene"
    description: str = ""
    size: tuple = (128, 128, 128)
    courant: float = 0.5
    pml: int = 16
    pml_sigma_max: float = 1.6
    pml_grading: float = 3.0
    cell_size: float = 1.0e-3
    wavelength: float = 16.0
    output_dir: str = ""


@dataclass
class Param:
    name: str
    label: str
    kind: str                      # "number", "bool", "choice"
    value: object = None
    default: object = None
    choices: list = field(default_factory=list)
    lo: float = -1e300
    hi: float = 1e300
    step: float = 1.0


@dataclass
class ScriptResult:
    scene: object
    settings: Settings
    params: list
    warnings: list
    output: list
    output_dir: str = ""      # where relative log paths go (ScriptEngine.cpp:2647-2651)
    background: object = None  # radar scenes: the scene without its targets (the calibration run)


def _round_half_away(x: float) -> int:
    """glm::round / std::lround: halves away from zero."""
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


class Args:
    """Validated access to the table passed to a builder function (ScriptEngine.cpp:226-400)."""

    def __init__(self, eng, what, keys, tbl):
        self.eng, self.what, self.keys, self.t = eng, what, list(keys), tbl
        if type(tbl) is not LuaTable:
            self.fail(f"expects a table argument, e.g. {what}{{ key = value, ... }}")

    def fail(self, msg):
        raise LuaError(f"{self.what}: {msg}")

    def raw(self, key):
        return self.eng.I.index(self.t, key)

    def has(self, key):
        return self.raw(key) is not None

    def opt_num(self, key):
        v = self.raw(key)
        if v is None:
            return None
        if type(v) not in (int, float):
            self.fail(f"'{key}' must be a number")
        if not math.isfinite(v):
            self.fail(f"'{key}' must be finite")
        return float(v)

    def num(self, key, default):
        v = self.opt_num(key)
        return default if v is None else v

    def req_num(self, key):
        v = self.opt_num(key)
        if v is None:
            self.fail(f"missing required number '{key}'")
        return v

    def positive(self, key, default):
        v = self.num(key, default)
        if not v > 0.0:
            self.fail(f"'{key}' must be > 0 (got {v:g})")
        return v

    def integer(self, key, default):
        v = self.num(key, default)
        if math.floor(v) != v:
            self.fail(f"'{key}' must be an integer (got {v:g})")
        return int(v)

    def _vec(self, v, n):
        if type(v) in (int, float):
            return (float(f32(v)),) * n if math.isfinite(v) else None
        if type(v) is not LuaTable:
            return None
        out = []
        for i, k in enumerate("xyz"[:n] if n == 3 else "uv"):
            x = v.rawget(i + 1)
            if x is None:
                x = self.eng.I.index(v, k)
            if type(x) not in (int, float) or not math.isfinite(x):
                return None
            out.append(float(f32(x)))
        return tuple(out)

    def opt_vec(self, key):
        v = self.raw(key)
        if v is None:
            return None
        r = self._vec(v, 3)
        if r is None:
            self.fail(f"'{key}' must be a 3-vector: {{x, y, z}}, vec(x, y, z) or a number")
        return r

    def vec(self, key, default):
        v = self.opt_vec(key)
        return default if v is None else v

    def req_vec(self, key):
        v = self.opt_vec(key)
        if v is None:
            self.fail(f"missing required vector '{key}'")
        return v

    def opt_vec2(self, key):
        v = self.raw(key)
        if v is None:
            return None
        r = self._vec(v, 2)
        if r is None:
            self.fail(f"'{key}' must be a 2-vector {{u, v}} (tangential coordinates)")
        return r

    def opt_str(self, key):
        v = self.raw(key)
        if v is None:
            return None
        if type(v) is not str:
            self.fail(f"'{key}' must be a string")
        return v

    def str(self, key, default):
        v = self.opt_str(key)
        return default if v is None else v

    def boolean(self, key, default):
        v = self.raw(key)
        if v is None:
            return default
        if type(v) is not bool:
            self.fail(f"'{key}' must be true or false")
        return v

    def axis(self, key, default):
        v = self.raw(key)
        if v is None:
            return default
        a = None
        if type(v) is str:
            a = _parse_axis(v)
        elif type(v) in (int, float) and v in (0, 1, 2):
            a = int(v)
        if a is None:
            self.fail(f"'{key}' must be an axis: \"x\", \"y\" or \"z\"")
        return a

    def opt_direction(self, key):
        v = self.raw(key)
        if v is None:
            return None
        if type(v) is str:
            a = _parse_axis(v)
            if a is None:
                self.fail(f"'{key}' must be an axis (\"x\", \"-y\", ...) or a vector")
            d = [0.0, 0.0, 0.0]
            d[a] = -1.0 if v.startswith("-") else 1.0
            return tuple(d)
        r = self._vec(v, 3)
        if r is None:
            self.fail(f"'{key}' must be an axis (\"x\", \"-y\", ...) or a vector")
        n = math.sqrt(float(f32(r[0] * r[0] + r[1] * r[1] + r[2] * r[2])))
        if n < 1e-6:
            self.fail(f"'{key}' must not be the zero vector")
        return tuple(float(f32(c / n)) for c in r)

    def check_unknown(self):
        for k in list(self.t.hash.keys()):
            if isinstance(k, str):
                if k not in self.keys:
                    self.eng.warn(f"{self.what}: unknown field '{k}' ignored{suggestion(k, self.keys)}")
            else:
                self.eng.warn(f"{self.what}: positional (unnamed) values are ignored; use key = value")


def edit_distance(a: str, b: str) -> int:
    """Levenshtein distance (ScriptEngine.cpp:47-57)."""
    prev = list(range(len(b) + 1))
    for i in range(1, len(a) + 1):
        cur = [i] + [0] * len(b)
        for j in range(1, len(b) + 1):
            cur[j] = min(prev[j] + 1, cur[j - 1] + 1, prev[j - 1] + (a[i - 1] != b[j - 1]))
        prev = cur
    return prev[len(b)]


def suggestion(word: str, candidates) -> str:
    """' (did you mean 'x'?)' for the closest candidate within edit distance 2 (ScriptEngine.cpp:59-70)."""
    best, best_d = "", 3
    for c in candidates:
        d = edit_distance(word.lower(), c.lower())
        if d < best_d:
            best_d, best = d, c
    return f" (did you mean '{best}'?)" if best else ""


def _parse_axis(s: str):
    a = s.lower()
    if a[:1] in "+-":
        a = a[1:]
    return {"x": 0, "y": 1, "z": 2}.get(a)


class ScriptEngine:
    """One scene-script run (ScriptEngine::run / runOnce, ScriptEngine.cpp:2560-2654)."""

    def __init__(self, overrides=None, echo=True, with_targets=True):
        self.with_targets = with_targets  # False: the radar's calibration run leaves out target = true objects
        self.targets = []
        self.radar = None
        self.emitters = []
        self.crpa = None
        self.overrides = dict(overrides or {})
        self.output = []
        self.echo = echo

        def out(line):
            self.output.append(line)
            if self.echo:
                print(line, flush=True)
        self.I = Interpreter(out=out)
        self.settings = Settings()
        self.locked = False
        self.builder = None
        self.warnings = []
        self.params = []
        self.materials = {k: v for k, v in BUILTIN_MATERIALS.items()}
        self.material_names = {k: k for k in BUILTIN_MATERIALS}
        self.used_dielectrics = {}
        self.monopoles = []
        self.sheet_sources = 0
        self.view = {}
        self._install()

    # ------------------------------------------------------------------ helpers
    def warn(self, msg):
        self.warnings.append(msg)

    def vec(self, x, y, z):
        return LuaTable([float(x), float(y), float(z)], meta=self.V)

    def lock(self):
        if self.locked:
            return
        self.locked = True
        s = self.settings
        grid = abi.GridConfig(tuple(s.size), courant=s.courant, pml_thickness=s.pml, pml_sigma_max=s.pml_sigma_max,
                              pml_grading=s.pml_grading)
        self.builder = EnvironmentBuilder(s.name, grid, cell_size=s.cell_size, wavelength=s.wavelength)
        self.builder.scene.description = s.description
        g = self.grid
        n = [float(v) for v in s.size]
        g.rawset("size", self.vec(*n))
        g.rawset("center", self.vec(*(0.5 * v for v in n)))
        g.rawset("interior_min", self.vec(*(float(s.pml),) * 3))
        g.rawset("interior_max", self.vec(*(v - s.pml for v in n)))
        g.rawset("nx", int(s.size[0]))
        g.rawset("ny", int(s.size[1]))
        g.rawset("nz", int(s.size[2]))
        g.rawset("pml", int(s.pml))
        g.rawset("wavelength", float(f32(s.wavelength)))
        g.rawset("cell_size", float(f32(s.cell_size)))
        g.rawset("dt", float(f32(s.courant)))

    def env(self):
        self.lock()
        return self.builder.scene

    def resolve(self, spec):
        eps, sig, cond, tand = spec
        sigma = 0.0
        if sig is not None:
            sigma = sig
        elif cond is not None:
            sigma = cond * float(f32(self.settings.cell_size)) * K_ETA0
        elif tand is not None:
            sigma = tand * (2.0 * math.pi / float(f32(self.settings.wavelength))) * float(f32(eps))
        return Material(float(f32(sigma)), float(max(f32(eps), f32(1.0))))

    def spec_from(self, a, name):
        eps = a.num("epsilon_r", 1.0)
        if float(f32(eps)) < 1.0:
            a.fail(f"epsilon_r must be >= 1 (got {eps:g})")
        sig, cond, tand = a.opt_num("sigma"), a.opt_num("conductivity"), a.opt_num("loss_tangent")
        if sum(v is not None for v in (sig, cond, tand)) > 1:
            a.fail("give only one of sigma, conductivity (S/m) or loss_tangent")
        if any(v is not None and v < 0 for v in (sig, cond, tand)):
            a.fail("losses must be >= 0")
        return (float(f32(eps)), sig, cond, tand)

    def read_material(self, a, default):
        v = a.raw("material")
        if v is None:
            name, spec = default, self.materials[default]
        elif type(v) is str:
            name = v.lower()
            if name not in self.materials:
                a.fail(f"unknown material '{v}'{suggestion(v, list(self.materials))}. "
                       f"Define it with material{{ name = \"{v}\", epsilon_r = ..., ... }}")
            spec = self.materials[name]
        elif type(v) is LuaTable:
            m = Args(self, "material (inline)", ["epsilon_r", "sigma", "conductivity", "loss_tangent", "name"], v)
            name = m.str("name", "inline material")
            spec = self.spec_from(m, name)
            m.check_unknown()
        else:
            a.fail("'material' must be a material name or a table { epsilon_r = ..., conductivity = ... }")
        if spec[0] > 1.0:
            self.used_dielectrics[name] = max(self.used_dielectrics.get(name, 0.0), spec[0])
        return self.resolve(spec)

    def read_wavelength(self, a):
        wl, fr = a.opt_num("wavelength"), a.opt_num("frequency")
        if wl is not None and fr is not None:
            a.fail("give either wavelength (cells) or frequency (Hz), not both")
        if fr is not None:
            if fr <= 0.0:
                a.fail("frequency must be > 0")
            return float(f32(K_C0 / (fr * float(f32(self.settings.cell_size)))))
        if wl is not None:
            if wl < 2.0:
                a.fail(f"wavelength must be >= 2 cells (got {wl:g})")
            return float(f32(wl))
        return float(f32(self.settings.wavelength))

    def read_box(self, a):
        mm = a.has("min") or a.has("max")
        cs = a.has("center") or a.has("size")
        if mm and cs:
            a.fail("give either min/max or center/size, not both")
        if mm:
            mn, mx = np.asarray(a.req_vec("min"), f32), np.asarray(a.req_vec("max"), f32)
            return np.minimum(mn, mx), np.maximum(mn, mx)
        if not a.has("size"):
            a.fail("needs min/max or center/size")
        c = np.asarray(a.vec("center", tuple(v * 0.5 for v in self.settings.size)), f32)
        sz = np.abs(np.asarray(a.req_vec("size"), f32))
        return c - f32(0.5) * sz, c + f32(0.5) * sz

    def target_info(self, shape, name):
        """targetInfo (ScriptEngine.cpp:798-827): a radar target's bounds and the centres of its
        cells, subsampled to about 200 000 points."""
        lo_b, hi_b = shape.bounds()
        n = np.asarray(self.settings.size)
        lo = np.clip(np.floor(np.asarray(lo_b, np.float64)).astype(int), 0, n - 1)
        hi = np.clip(np.ceil(np.asarray(hi_b, np.float64)).astype(int), 0, n - 1)
        span = (hi - lo + 1).astype(np.float32)
        stride = max(1, int(math.ceil(float(np.cbrt(f32(span[0] * span[1] * span[2]) / f32(200000.0))))))
        zz, yy, xx = np.meshgrid(np.arange(lo[2], hi[2] + 1, stride), np.arange(lo[1], hi[1] + 1, stride),
                                 np.arange(lo[0], hi[0] + 1, stride), indexing="ij")
        px, py, pz = (xx + f32(0.5)).astype(f32), (yy + f32(0.5)).astype(f32), (zz + f32(0.5)).astype(f32)
        inside = np.asarray(shape.contains(px, py, pz), bool)
        pts = np.stack([px[inside], py[inside], pz[inside]], axis=1).astype(f32)
        if pts.size:
            mn, mx = pts.min(axis=0) - f32(0.5), pts.max(axis=0) + f32(0.5)
        else:
            mn, mx = np.asarray(lo_b, f32), np.asarray(hi_b, f32)
        return {"name": name, "min": tuple(float(v) for v in mn), "max": tuple(float(v) for v in mx), "points": pts}

    def take_target(self, a, shape) -> bool:
        """target = true: record the target; True when the object is left out (calibration run)."""
        if a.boolean("target", False):
            self.targets.append(self.target_info(shape, a.str("name", a.what)))
            return not self.with_targets
        return False

    def fill_shape(self, a, local, center, m):
        r = a.opt_vec("rotate")
        if r is not None and math.sqrt(sum(v * v for v in r)) != 0.0:
            rot = rotation_from_euler_degrees(r)
        else:
            rot = np.eye(3, dtype=f32)
        shape = TransformedShape(local, center, rot)
        if self.take_target(a, shape):
            return 0
        n = self.env_builder().fill(shape, m)
        if n == 0:
            self.warn(f"{a.what}: shape is empty or lies completely outside the grid")
        return n

    def env_builder(self):
        self.lock()
        return self.builder

    def read_waveform(self, a, s: SourceDesc):
        s.wavelength = self.read_wavelength(a)
        s.phase = float(f32(math.radians(a.num("phase", 0.0))))
        wf = a.str("waveform", "cw").lower()
        if wf in ("cw", "continuous", "sine"):
            s.waveform = abi.WAVE_CW
            s.ramp_periods = float(f32(a.num("ramp", 3.0)))
            if a.has("pulse_width"):
                self.warn(f"{a.what}: pulse_width is ignored for waveform = \"cw\"")
        elif wf in ("pulse", "gaussian"):
            s.waveform = abi.WAVE_PULSE
            s.ramp_periods = float(f32(a.positive("pulse_width", 1.0)))
            if a.has("ramp"):
                self.warn(f"{a.what}: ramp is ignored for waveform = \"pulse\" (use pulse_width)")
        else:
            a.fail(f"waveform must be \"cw\" or \"pulse\" (got \"{wf}\")")
        s.repeat_periods = float(f32(a.num("interval", 0.0)))
        s.delay_periods = float(f32(a.num("delay", 0.0)))
        s.enabled = a.boolean("enabled", True)
        if s.wavelength < 8.0:
            self.warn(f"{a.what}: wavelength {s.wavelength:.1f} cells is under-resolved (< 8 cells)")

    def add_source(self, s):
        if s.enabled:
            self.env().sources.append(s)

    def wire_axis(self, a, d):
        ad = [abs(v) for v in d]
        ax = 0 if (ad[0] >= ad[1] and ad[0] >= ad[2]) else (1 if ad[1] >= ad[2] else 2)
        if ad[ax] < 0.9999:
            a.fail("extended (length > 0) wires must be aligned with x, y or z; use length = 0 for an arbitrarily "
                   "oriented point dipole")
        return ax

    def read_conductor(self, a):
        m = a.str("model", "thin").lower()
        if m in ("thin", "wire"):
            return "thin"
        if m == "rod":
            return "rod"
        if m in ("current", "ideal"):
            return "current"
        a.fail("model must be \"thin\" (thin wire, default), \"rod\" (1x1-cell metal conductor) or \"current\" "
               "(ideal uniform current)")

    def read_feed(self, a):
        kind = a.str("feed", "voltage").lower()
        if kind not in ("voltage", "current"):
            a.fail("feed must be \"voltage\" (resistive voltage source, default) or \"current\" (ideal current "
                   "source)")
        imp = float(f32(a.positive("impedance", 50.0)))
        if kind == "current" and a.has("impedance"):
            self.warn(f"{a.what}: 'impedance' only applies to feed = \"voltage\"")
        return kind == "voltage", imp, float(f32(a.num("amplitude", 1.0)))

    def read_radius(self, a, wavelength):
        r = float(f32(a.num("radius", wavelength / 400.0)))
        if not r > 0.0:
            a.fail("radius must be > 0")
        if r > 0.4:
            a.fail(f"radius {r:.2f} cells is too thick for the thin-wire model (max 0.4 cells); use model = \"rod\" "
                   f"for a 1x1-cell conductor or refine the grid")
        return r

    def fill_rod(self, cell, axis, lo_i, hi_i, m):
        if hi_i <= lo_i:
            return 0
        lo = [float(c) for c in cell]
        hi = [float(c) + 1.0 for c in cell]
        lo[axis], hi[axis] = float(lo_i), float(hi_i)
        return self.env_builder().box(lo, hi, m)

    def dipole_arm(self, a, length):
        if length < 3.0:
            a.fail("a dipole needs length >= 3 cells (two arms plus the feed gap); use model = \"current\" for "
                   "shorter ideal elements, or length = 0 for an ideal point dipole")
        if length < 5.0 and a.str("model", "thin").lower() != "rod":
            a.fail("a thin-wire dipole needs length >= 5 cells (each free end is built one cell short to correct "
                   "the grid's end effect); refine the grid, or use model = \"rod\"")
        arm = max(1, _round_half_away((float(f32(length)) - 1.0) * 0.5))
        realized = 2 * arm + 1
        if abs(realized - length) >= 1.0:
            self.warn(f"{a.what}: length {length:.1f} realised as {realized} cells (two {arm}-cell arms + 1-cell "
                      f"feed gap)")
        return arm

    # ------------------------------------------------------------------ API
    def _install(self):
        I = self.I
        G = I.globals
        eng = self
        # sandbox: no file access
        for name in ("dofile", "loadfile", "require"):
            G.rawset(name, None)

        # -- vector prelude
        V = LuaTable()
        self.V = V

        def v_index(args):
            t, k = args[0], args[1]
            if k == "x":
                return [t.rawget(1)]
            if k == "y":
                return [t.rawget(2)]
            if k == "z":
                return [t.rawget(3)]
            return [V.rawget(k)]
        V.rawset("__index", LuaFunction("vec.__index", v_index))

        def comp(t, i, key):
            v = t.rawget(i)
            if v is None:
                v = I.index(t, key)
            return v

        def vec(x=None, y=None, z=None, *r):
            if type(x) is LuaTable:
                vals = []
                for i, k in enumerate("xyz"):
                    v = x.rawget(i + 1)
                    if v is None:
                        v = I.index(x, k)
                    vals.append(0 if v is None or v is False else v)
                return LuaTable(vals, meta=V)
            if y is None and z is None:
                x = 0 if x is None else x
                return LuaTable([x, x, x], meta=V)
            return LuaTable([0 if x is None else x, 0 if y is None else y, 0 if z is None else z], meta=V)
        I.register("vec", vec)

        def lift(a):
            return vec(a)

        def binop(op):
            def f(a, b=None, *r):
                a, b = lift(a), lift(b)
                return vec(*(I.arith(op, a.rawget(i), b.rawget(i)) for i in (1, 2, 3)))
            return f
        for mm, op in (("__add", "__add"), ("__sub", "__sub"), ("__mul", "__mul"), ("__div", "__div")):
            I.register(mm, binop(op), V)
        I.register("__unm", lambda a, *r: vec(*(I.arith("__unm", a.rawget(i), None) for i in (1, 2, 3))), V)
        I.register("__eq", lambda a, b, *r: all(I.equal(a.rawget(i), b.rawget(i)) for i in (1, 2, 3)), V)
        I.register("__tostring", lambda a, *r: "vec(%s, %s, %s)" % tuple(
            ("%g" % float(a.rawget(i))) for i in (1, 2, 3)), V)

        def dot(a, b, *r):
            b = lift(b)
            return I.arith("__add", I.arith("__add", I.arith("__mul", a.rawget(1), b.rawget(1)),
                                            I.arith("__mul", a.rawget(2), b.rawget(2))),
                           I.arith("__mul", a.rawget(3), b.rawget(3)))
        I.register("dot", dot, V)

        def length(a, *r):
            return math.sqrt(float(dot(a, a)))
        I.register("length", length, V)

        def normalize(a, *r):
            n = length(a)
            if n == 0:
                return vec(0, 0, 0)
            return binop("__div")(a, n)
        I.register("normalize", normalize, V)

        def cross(a, b, *r):
            b = lift(b)
            a1, a2, a3 = a.rawget(1), a.rawget(2), a.rawget(3)
            b1, b2, b3 = b.rawget(1), b.rawget(2), b.rawget(3)
            sub, mul = (lambda x, y: I.arith("__sub", x, y)), (lambda x, y: I.arith("__mul", x, y))
            return vec(sub(mul(a2, b3), mul(a3, b2)), sub(mul(a3, b1), mul(a1, b3)), sub(mul(a1, b2), mul(a2, b1)))
        I.register("cross", cross, V)

        def with_(a, axis, value, *r):
            i = {"x": 1, "y": 2, "z": 3}.get(axis, axis)
            out = vec(a)
            out.rawset(i, value)
            return out
        I.register("with", with_, V)
        G.rawset("X", vec(1, 0, 0))
        G.rawset("Y", vec(0, 1, 0))
        G.rawset("Z", vec(0, 0, 1))
        G.rawset("c0", K_C0)
        G.rawset("pi", math.pi)

        def gridfield(k):
            return I.index(G.rawget("grid"), k)
        I.register("deg", lambda x, *r: I.arith("__div", I.arith("__mul", x, math.pi), 180))
        I.register("wavelengths", lambda n, *r: I.arith("__mul", n, gridfield("wavelength")))
        I.register("meters", lambda x, *r: I.arith("__div", x, gridfield("cell_size")))
        I.register("mm", lambda x, *r: I.arith("__div", I.arith("__mul", x, 1e-3), gridfield("cell_size")))
        I.register("lerp", lambda a, b, t, *r: I.arith("__add", a, I.arith("__mul", I.arith("__sub", b, a), t)))
        M = G.rawget("math")
        I.register("clamp", lambda x, lo, hi, *r: I.call(M.rawget("max"), [lo, I.call(M.rawget("min"), [hi, x])[0]])[0])

        def range_(a, b, step=None, *r):
            step = 1 if step is None else step
            state = {"i": I.arith("__sub", a, step)}

            def it(args):
                i = I.arith("__add", state["i"], step)
                state["i"] = i
                if (step > 0 and i <= b + 1e-9) or (step < 0 and i >= b - 1e-9):
                    return [i]
                return [None]
            return LuaFunction("range_iter", it)
        I.register("range", range_)

        # -- grid: reading it before scene{} locks the default settings
        grid = LuaTable()
        gm = LuaTable()

        def grid_index(args):
            eng.lock()
            return [args[0].rawget(args[1])]
        gm.rawset("__index", LuaFunction("grid.__index", grid_index))
        grid.meta = gm
        G.rawset("grid", grid)
        self.grid = grid

        api = {"radar": self.api_radar, "emitter": self.api_emitter, "crpa": self.api_crpa, "scene": self.api_scene, "view": self.api_view, "material": self.api_material, "param": self.api_param,
               "box": self.api_box, "sphere": self.api_sphere, "cylinder": self.api_cylinder,
               "wall": self.api_wall, "grating": self.api_grating, "shape": self.api_shape,
               "cage": self.api_cage, "frame": self.api_frame, "loop": self.api_loop,
               "array": self.api_array, "coax": self.api_coax,
               "dipole": self.api_dipole, "monopole": self.api_monopole, "wire": self.api_wire,
               "sheet": self.api_sheet, "sweep": self.api_sweep, "plane_wave": self.api_plane_wave,
               "gaussian_beam": self.api_gaussian_beam, "current_source": self.api_current_source,
               "probe": self.api_probe, "flux_plane": self.api_flux_plane, "flux_box": self.api_flux_box,
               "far_field": self.api_far_field, "warning": self.api_warning}
        for name, fn in api.items():
            I.register(name, fn)

    # -- radar (ScriptEngine.cpp:1804-1848)
    def api_radar(self, t=None, *r):
        a = Args(self, "radar", ["range", "fov", "noise", "threshold", "dynamic_range", "reference", "phase_center",
                                 "tx", "taper", "log", "name"], t)
        self.lock()
        rs = {"range_min": 0.0, "range_max": 0.0, "fov_az": 40.0, "fov_el": 40.0, "noise_db": -300.0,
              "threshold_db": 13.0, "dynamic_range_db": 25.0, "reference": 0.0, "taper": 1,
              "phase_center": (0.0, 0.0, 0.0), "tx": None, "log": ""}
        rg = a.opt_vec2("range")
        if rg is not None:
            if not (rg[0] >= 0.0) or not (rg[1] > rg[0]):
                a.fail("range = {min, max} needs 0 <= min < max (cells)")
            rs["range_min"], rs["range_max"] = float(f32(rg[0])), float(f32(rg[1]))
        if a.has("fov"):
            v = a.raw("fov")
            if type(v) in (int, float):
                rs["fov_az"] = rs["fov_el"] = float(f32(a.opt_num("fov")))
            else:
                f2 = a.opt_vec2("fov")
                if f2 is not None:
                    rs["fov_az"], rs["fov_el"] = float(f32(f2[0])), float(f32(f2[1]))
            if not (0.0 < rs["fov_az"] <= 80.0 and 0.0 < rs["fov_el"] <= 80.0):
                a.fail("fov = half-angle in degrees (0..80), or {azimuth, elevation}")
        nz = a.opt_num("noise")
        if nz is not None:
            if nz > 0.0:
                a.fail("noise is in dB relative to the transmit pulse at a port, so it must be negative (e.g. -70)")
            rs["noise_db"] = float(f32(nz))
        rs["threshold_db"] = float(f32(a.num("threshold", 13.0)))
        rs["dynamic_range_db"] = float(f32(a.positive("dynamic_range", 25.0)))
        rs["reference"] = float(f32(a.num("reference", 0.0)))
        rs["phase_center"] = tuple(float(v) for v in a.vec("phase_center", (0.0, 0.0, 0.0)))
        tx = a.opt_vec("tx")
        rs["tx"] = tuple(float(v) for v in tx) if tx is not None else None
        taper = a.str("taper", "hamming").lower()
        if taper in ("uniform", "none"):
            rs["taper"] = 0
        elif taper == "hamming":
            rs["taper"] = 1
        elif taper in ("hann", "hanning"):
            rs["taper"] = 2
        else:
            a.fail(f"taper must be \"uniform\", \"hamming\" or \"hann\" (got \"{taper}\")")
        rs["log"] = a.str("log", "")
        if self.radar is not None:
            self.warn("radar: only one radar per scene; replacing the previous one")
        self.radar = rs
        a.check_unknown()

    # -- emitters and the adaptive array (ScriptEngine.cpp:1850-1948)
    def api_emitter(self, t=None, *r):
        """A transmitter at a point: one ideal dipole (linear) or two crossed dipoles 90 degrees apart
        in phase, perpendicular to the line toward `toward` (circular; IEEE handedness)."""
        a = Args(self, "emitter", ["position", "name", "polarization", "toward", "amplitude"] + WAVEFORM_KEYS, t)
        self.lock()
        w = SourceDesc()
        self.read_waveform(a, w)
        pos = np.asarray(a.req_vec("position"), f32)
        name = a.str("name", f"emitter {len(self.emitters) + 1}")
        if any(e["name"] == name for e in self.emitters):
            a.fail(f"an emitter named '{name}' already exists")
        index = len(self.emitters)
        amp = float(f32(a.num("amplitude", 1.0)))

        def add(direction, extra_phase):
            s = SourceDesc.dipole(tuple(float(v) for v in pos), tuple(float(v) for v in direction), w.wavelength, amp,
                                  0.0)
            for k in ("wavelength", "phase", "waveform", "ramp_periods", "repeat_periods", "delay_periods", "enabled"):
                setattr(s, k, getattr(w, k))
            s.phase = float(f32(f32(s.phase) + f32(extra_phase)))
            s.emitter = index
            self.add_source(s)
        pv = a.raw("polarization")
        pol = pv.lower() if type(pv) is str else "linear"
        if pol in ("rhcp", "lhcp"):
            toward = np.asarray(a.vec("toward", tuple(v * 0.5 for v in self.settings.size)), f32)
            d = toward - pos
            d = (d / f32(np.sqrt(np.sum(d * d, dtype=f32)))).astype(f32)  # propagation direction
            ref = np.array([0, 0, 1], f32) if abs(d[2]) < 0.9 else np.array([1, 0, 0], f32)
            ea = np.cross(d, ref).astype(f32)
            ea = (ea / f32(np.sqrt(np.sum(ea * ea, dtype=f32)))).astype(f32)
            eb = np.cross(d, ea).astype(f32)  # (ea, eb, d) right-handed
            add(ea, f32(math.pi / 2))
            add(eb, 0.0 if pol == "rhcp" else f32(math.pi))
        else:
            direction = a.opt_direction("polarization")
            if direction is None:
                a.fail("polarization must be \"rhcp\", \"lhcp\" or a direction vector (linear)")
            add(direction, 0.0)
            pol = "linear"
        self.emitters.append({"name": name, "position": tuple(float(v) for v in pos), "polarization": pol})
        a.check_unknown()

    def api_crpa(self, t=None, *r):
        a = Args(self, "crpa", ["satellite", "elements", "jnr", "snr", "steering", "weights", "periods", "north", "log",
                                "name", "adapt", "snapshot_periods", "snapshot_rate", "noise_seed"], t)
        self.lock()
        c = {"satellite": a.str("satellite", ""), "elements": []}
        if not c["satellite"]:
            a.fail("needs satellite = <emitter name>")
        els = a.raw("elements")
        if type(els) is not LuaTable:
            a.fail("needs elements = { {x = \"port\", y = \"port\", center = vec(...)}, ... }")
        n = self.I.length(els)
        for i in range(1, n + 1):
            e = self.I.index(els, i)
            if type(e) is not LuaTable:
                a.fail(f"elements[{i}] must be a table {{x = ..., y = ..., center = ...}}")
            px, py, ctr = self.I.index(e, "x"), self.I.index(e, "y"), self.I.index(e, "center")
            el = {"x": px if type(px) is str else "", "y": py if type(py) is str else "", "center": (0.0, 0.0, 0.0)}
            if type(ctr) is LuaTable:
                vals = [self.I.index(ctr, k + 1) for k in range(3)]
                el["center"] = tuple(float(f32(v)) if type(v) in (int, float) else 0.0 for v in vals)
            if not el["x"] or not el["y"]:
                a.fail(f"elements[{i}] needs x and y port names")
            c["elements"].append(el)
        if len(c["elements"]) < 2:
            a.fail("a CRPA needs at least 2 elements")
        c["jnr_db"] = float(f32(a.num("jnr", 40.0)))
        c["snr_db"] = float(f32(a.num("snr", -20.0)))
        steering = a.str("steering", "model").lower()
        if steering not in ("model", "measured"):
            a.fail("steering must be \"model\" or \"measured\"")
        c["measured_steering"] = steering == "measured"
        weights = a.str("weights", "mvdr").lower()
        if weights not in ("mvdr", "steering"):
            a.fail("weights must be \"mvdr\" or \"steering\"")
        c["mvdr"] = weights == "mvdr"
        c["pass_periods"] = float(f32(a.positive("periods", 36.0)))
        adapt = a.str("adapt", "blind").lower()
        if adapt not in ("blind", "ideal"):
            a.fail("adapt must be \"blind\" or \"ideal\"")
        c["blind"] = adapt == "blind"
        c["snapshot_periods"] = float(f32(_round_half_away(a.positive("snapshot_periods", 40.0))))
        if c["snapshot_periods"] < 8.0:
            a.fail("snapshot_periods must be at least 8")
        c["snapshots_per_period"] = min(max(int(_round_half_away(a.positive("snapshot_rate", 4.0))), 1), 16)
        c["noise_seed"] = int(max(0.0, a.num("noise_seed", 1.0)))
        nv = a.opt_vec("north")
        c["north"] = (0.0, 1.0, 0.0)
        if nv is not None:
            v = np.asarray(nv, f32)
            c["north"] = tuple(float(x) for x in v / f32(np.sqrt(np.sum(v * v, dtype=f32))))
        c["log"] = a.str("log", "")
        self.crpa = c
        a.check_unknown()

    # -- scene / view / material / param (ScriptEngine.cpp:605-842)
    def api_scene(self, t=None, *r):
        a = Args(self, "scene", ["name", "description", "size", "cell_size", "wavelength", "frequency", "courant",
                                 "pml", "output_dir"], t)
        if self.locked:
            a.fail("scene{} must be the first call in the script (before any objects, sources or use of 'grid')")
        s = self.settings
        s.name = a.str("name", s.name)
        s.description = a.str("description", "")
        s.output_dir = a.str("output_dir", "")
        s.cell_size = float(f32(a.positive("cell_size", s.cell_size)))
        s.courant = float(f32(a.positive("courant", s.courant)))
        if s.courant >= float(f32(0.577)):
            a.fail(f"courant must be < 1/sqrt(3) ~ 0.577 for stability (got {s.courant:g})")
        v = a.opt_vec("size")
        if v is not None:
            rv = [_round_half_away(c) for c in v]
            if any(c < 16 for c in rv):
                a.fail("size must be at least 16 cells per axis")
            s.size = tuple(rv)
        p = a.raw("pml")
        if type(p) in (int, float):
            s.pml = int(p)
        elif type(p) is LuaTable:
            pa = Args(self, "scene.pml", ["thickness", "sigma_max", "grading"], p)
            s.pml = pa.integer("thickness", s.pml)
            s.pml_sigma_max = float(f32(pa.num("sigma_max", s.pml_sigma_max)))
            s.pml_grading = float(f32(pa.num("grading", s.pml_grading)))
            pa.check_unknown()
        elif p is not None:
            a.fail("'pml' must be a number (thickness) or { thickness, sigma_max, grading }")
        if s.pml < 0 or s.pml > 64:
            a.fail("pml thickness must be within 0..64 cells")
        if any(c < 2 * s.pml + 8 for c in s.size):
            a.fail(f"size must exceed 2 * pml + 8 = {2 * s.pml + 8} cells per axis")
        s.wavelength = self.read_wavelength(a)
        mem = 48.0 * s.size[0] * s.size[1] * s.size[2] / (1024.0 * 1024.0)
        if mem > 2048.0:
            self.warn(f"scene: grid needs {mem:.0f} MB of GPU memory")
        if s.wavelength < 10.0:
            self.warn(f"scene: reference wavelength is only {s.wavelength:.1f} cells; >= 12 cells per wavelength "
                      f"keeps numerical dispersion small")
        a.check_unknown()
        self.lock()

    def api_view(self, t=None, *r):
        a = Args(self, "view", ["mode", "component", "gain", "gain_e", "gain_b", "exposure", "density", "step",
                                "steps_per_frame", "distance", "yaw", "pitch", "target", "overlay", "metal_opacity"], t)
        v = self.view
        m = a.opt_str("mode")
        if m is not None:
            modes = ["fields", "e", "b", "poynting", "signed"]
            if m.lower() not in modes:
                a.fail("mode must be one of \"fields\", \"e\", \"b\", \"poynting\", \"signed\""
                       + suggestion(m, modes))
            v["mode"] = modes.index(m.lower())
        if a.has("component"):
            v["component"] = a.axis("component", 2)
        g = a.opt_num("gain")
        if g is not None:
            v["gain_e"] = v["gain_b"] = float(g)
        for key, name in (("gain_e", "gain_e"), ("gain_b", "gain_b"), ("exposure", "exposure"),
                          ("density", "density"), ("step", "step")):
            x = a.opt_num(key)
            if x is not None:
                v[name] = float(x)
        x = a.opt_num("metal_opacity")
        if x is not None:
            v["metal_opacity"] = min(max(float(x), 0.0), 1.0)
        if a.has("steps_per_frame"):
            v["steps_per_frame"] = min(max(a.integer("steps_per_frame", 2), 1), 64)
        v["distance"] = float(a.num("distance", v.get("distance", 3.0)))
        v["yaw"] = float(a.num("yaw", v.get("yaw", -55.0)))
        v["pitch"] = float(a.num("pitch", v.get("pitch", 30.0)))
        t = a.opt_vec("target")
        if t is not None:
            v["target"] = tuple(float(c) for c in t)
        if a.has("overlay"):
            v["overlay"] = a.boolean("overlay", True)
        a.check_unknown()

    def api_material(self, t=None, *r):
        a = Args(self, "material", ["name", "epsilon_r", "sigma", "conductivity", "loss_tangent"], t)
        name = a.opt_str("name")
        if not name:
            a.fail("needs a name, e.g. material{ name = \"foam\", epsilon_r = 1.1 }")
        spec = self.spec_from(a, name)
        key = name.lower()
        if key in BUILTIN_MATERIALS:
            self.warn(f"material: '{name}' overrides the built-in material")
        self.materials[key] = spec
        a.check_unknown()
        return name

    def api_param(self, t=None, *r):
        a = Args(self, "param", ["name", "label", "default", "min", "max", "step", "key", "keys", "choices", "wrap"], t)
        name = a.opt_str("name")
        if not name:
            a.fail("needs a name")
        if any(p.name == name for p in self.params):
            a.fail(f"parameter '{name}' is declared twice")
        label = a.str("label", name)
        override = self.overrides.get(name)
        ch = a.raw("choices")
        if type(ch) is LuaTable:
            choices = []
            for i in range(1, ch.length() + 1):
                v = ch.rawget(i)
                if type(v) is not str:
                    a.fail("choices must be a list of strings")
                choices.append(v)
            if not choices:
                a.fail("choices must not be empty")
            default = a.str("default", choices[0])
            if default not in choices:
                a.fail(f"default '{default}' is not one of the choices")
            value = override if override in choices else default
            p = Param(name, label, "choice", value, default, choices)
        elif type(a.raw("default")) is bool:
            d = a.raw("default")
            value = d
            if override is not None:
                value = override.lower() in ("true", "1", "on")
            p = Param(name, label, "bool", value, d)
        else:
            d = a.req_num("default")
            lo, hi = a.num("min", -1e300), a.num("max", 1e300)
            step = a.positive("step", 1.0)
            a.boolean("wrap", False)
            if lo > hi:
                a.fail("min must be <= max")
            value = d
            if override is not None:
                try:
                    value = float(override.strip().split()[0])
                except (ValueError, IndexError):
                    pass
            value = min(max(value, lo), hi)
            p = Param(name, label, "number", value, d, lo=lo, hi=hi, step=step)
        a.raw("key")
        a.raw("keys")
        a.check_unknown()
        self.params.append(p)
        return p.value

    # -- geometry (ScriptEngine.cpp:843-1075)
    def api_box(self, t=None, *r):
        a = Args(self, "box", ["min", "max", "center", "size", "material", "rotate", "thickness", "name", "target"], t)
        mn, mx = self.read_box(a)
        m = self.read_material(a, "metal")
        c, h = f32(0.5) * (mn + mx), f32(0.5) * (mx - mn)
        local = BoxShape(-h, h)
        th = a.opt_num("thickness")
        if th is not None:
            if th <= 0.0:
                a.fail("thickness must be > 0")
            hi = np.maximum(h - f32(th), f32(0.0))
            local = DifferenceShape(local, BoxShape(-hi, hi))
        self.fill_shape(a, local, c, m)
        a.check_unknown()

    def api_sphere(self, t=None, *r):
        a = Args(self, "sphere", ["center", "radius", "material", "rotate", "thickness", "name", "target"], t)
        c = np.asarray(a.vec("center", tuple(v * 0.5 for v in self.settings.size)), f32)
        rad = np.asarray(a.req_vec("radius"), f32)
        if np.any(rad <= 0):
            a.fail("radius must be > 0")
        m = self.read_material(a, "metal")
        local = EllipsoidShape((0, 0, 0), rad)
        th = a.opt_num("thickness")
        if th is not None:
            if th <= 0.0:
                a.fail("thickness must be > 0")
            ri = rad - f32(th)
            if np.all(ri > 0):
                local = DifferenceShape(local, EllipsoidShape((0, 0, 0), ri))
        self.fill_shape(a, local, c, m)
        a.check_unknown()

    def api_cylinder(self, t=None, *r):
        a = Args(self, "cylinder", ["center", "axis", "radius", "length", "material", "rotate", "thickness",
                                    "inner_radius", "capped", "name", "target"], t)
        c = np.asarray(a.vec("center", tuple(v * 0.5 for v in self.settings.size)), f32)
        axis = a.axis("axis", 2)
        rad = f32(a.positive("radius", 1.0))
        ln = f32(a.positive("length", 1.0))
        m = self.read_material(a, "metal")
        local = CylinderShape((0, 0, 0), axis, rad, f32(0.5) * ln)
        th, ri = a.opt_num("thickness"), a.opt_num("inner_radius")
        if th is not None and ri is not None:
            a.fail("give thickness or inner_radius, not both")
        if th is not None or ri is not None:
            inner = f32(ri) if ri is not None else rad - f32(th)
            if inner <= 0 or inner >= rad:
                a.fail("inner radius must be within (0, radius)")
            capped = a.boolean("capped", False)
            wall = rad - inner
            inner_half = f32(0.5) * ln - wall if capped else f32(0.5) * ln + f32(1.0)
            local = DifferenceShape(local, CylinderShape((0, 0, 0), axis, inner, max(inner_half, f32(0.0))))
        self.fill_shape(a, local, c, m)
        a.check_unknown()

    def read_apertures(self, a, axis):
        out = []
        n = self.settings.size
        u, v = (1 if axis == 0 else 0), (1 if axis == 2 else 2)
        mid = (0.5 * n[u], 0.5 * n[v])
        aps = a.raw("apertures")
        if type(aps) is LuaTable:
            for i in range(1, aps.length() + 1):
                ap = Args(self, "wall.apertures[]", ["center", "size", "radius"], aps.rawget(i))
                c = ap.opt_vec2("center") or mid
                rr = ap.opt_num("radius")
                if rr is not None:
                    out.append({"circular": True, "center": c, "radius": float(f32(rr)), "half": (0, 0)})
                else:
                    sz = ap.opt_vec2("size")
                    if sz is None:
                        a.fail("each aperture needs size = {w, h} or radius = r")
                    out.append({"circular": False, "center": c, "radius": 0.0,
                                "half": (0.5 * abs(sz[0]), 0.5 * abs(sz[1]))})
                ap.check_unknown()
        sl = a.raw("slits")
        if type(sl) is LuaTable:
            s = Args(self, "wall.slits", ["count", "width", "spacing", "length", "direction", "center"], sl)
            count = s.integer("count", 2)
            width = float(f32(s.positive("width", 6.0)))
            spacing = float(f32(s.num("spacing", 4.0 * width)))
            length = float(f32(s.num("length", 1.0e6)))
            d = s.axis("direction", v)
            center = s.opt_vec2("center") or mid
            s.check_unknown()
            if d == axis:
                a.fail("slits.direction must lie in the wall plane")
            if count < 1:
                a.fail("slits.count must be >= 1")
            long_u = d == u
            for i in range(count):
                off = float(f32((i - 0.5 * (count - 1)) * spacing))
                c = (center[0], center[1] + off) if long_u else (center[0] + off, center[1])
                half = (0.5 * length, 0.5 * width) if long_u else (0.5 * width, 0.5 * length)
                out.append({"circular": False, "center": c, "radius": 0.0, "half": half})
        return out

    def api_wall(self, t=None, *r):
        a = Args(self, "wall", ["axis", "position", "thickness", "material", "apertures", "slits", "name"], t)
        axis = a.axis("axis", 0)
        pos = float(f32(a.req_num("position")))
        th = float(f32(a.positive("thickness", 2.0)))
        m = self.read_material(a, "metal")
        aps = self.read_apertures(a, axis)
        self.lock()
        wall = WallShape(axis, pos, float(f32(pos + th)), aps, self.settings.size)
        if self.env_builder().fill(wall, m) == 0:
            self.warn(f"{a.what}: shape is empty or lies completely outside the grid")
        a.check_unknown()

    def api_grating(self, t=None, *r):
        a = Args(self, "grating", ["axis", "position", "thickness", "period", "width", "direction", "min", "max",
                                   "material", "name"], t)
        axis = a.axis("axis", 0)
        x0 = f32(a.req_num("position"))
        th = f32(a.positive("thickness", 1.0))
        period = f32(a.positive("period", 4.0))
        width = f32(a.positive("width", 1.0))
        if width >= period:
            a.fail("width must be smaller than period")
        u, v = (1 if axis == 0 else 0), (1 if axis == 2 else 2)
        d = a.axis("direction", v)
        if d == axis:
            a.fail("direction (bar axis) must lie in the grating plane")
        across = v if d == u else u
        n = np.asarray(self.settings.size, f32)
        lo2 = a.opt_vec2("min") or (0.0, 0.0)
        hi2 = a.opt_vec2("max") or (float(n[u]), float(n[v]))
        m = self.read_material(a, "metal")
        bmin, bmax = np.zeros(3, f32), n.copy()
        bmin[axis], bmax[axis] = x0, x0 + th
        bmin[u], bmax[u] = lo2[0], hi2[0]
        bmin[v], bmax[v] = lo2[1], hi2[1]
        start = bmin[across]

        def inside(x, y, z):
            p = (x, y, z)
            ok = np.ones(np.shape(x), bool)
            for i in range(3):
                ok &= (p[i] >= bmin[i]) & (p[i] < bmax[i])
            q = np.fmod(p[across] - start, period)
            return ok & (q >= 0) & (q < width)
        if self.env_builder().fill(LambdaShape(bmin, bmax, inside), m) == 0:
            self.warn(f"{a.what}: shape is empty or lies completely outside the grid")
        a.check_unknown()

    def api_shape(self, t=None, *r):
        a = Args(self, "shape", ["min", "max", "center", "size", "inside", "material", "name", "target"], t)
        mn, mx = self.read_box(a)
        fn = a.raw("inside")
        if type(fn) is not LuaFunction:
            a.fail("needs inside = function(x, y, z) return <boolean> end")
        m = self.read_material(a, "metal")
        I = self.I

        def inside(x, y, z):
            ok = ((x >= mn[0]) & (y >= mn[1]) & (z >= mn[2]) & (x < mx[0]) & (y < mx[1]) & (z < mx[2]))
            out = np.zeros(np.shape(x), bool)
            idx = np.nonzero(ok)
            for k in zip(*idx):
                try:
                    res = I.call(fn, [float(x[k]), float(y[k]), float(z[k])])
                except LuaError as e:
                    raise LuaError(f"shape.inside(): {e}")
                v = res[0] if res else None
                out[k] = v is not None and v is not False
            return out
        shape = LambdaShape(mn, mx, inside)
        if self.take_target(a, shape):
            a.check_unknown()
            return
        if self.env_builder().fill(shape, m) == 0:
            self.warn(f"{a.what}: shape is empty or lies completely outside the grid")
        a.check_unknown()

    def api_cage(self, t=None, *r):
        """cage{} (ScriptEngine.cpp:1010-1020) with EnvironmentBuilder::meshCage (Environment.cpp:129-156):
        bars of `bar` cells every `spacing` cells on the faces of a box, plus the far rims."""
        a = Args(self, "cage", ["min", "max", "center", "size", "spacing", "bar", "material", "name"], t)
        mn, mx = self.read_box(a)
        spacing = a.integer("spacing", 4)
        bar = a.integer("bar", 2)
        if bar < 1 or spacing <= bar:
            a.fail("need bar >= 1 and spacing > bar")
        m = self.read_material(a, "metal")
        lo = np.array([_round_half_away(float(v)) for v in mn])
        hi = np.array([_round_half_away(float(v)) for v in mx]) - 1
        tk = max(bar, 1)
        sp = max(spacing, tk + 1)
        size = np.asarray(self.settings.size)
        clo, chi = np.maximum(lo, 0), np.minimum(hi, size - 1)
        written = 0
        if np.all(chi >= clo):
            zz, yy, xx = np.meshgrid(*(np.arange(clo[k], chi[k] + 1) for k in (2, 1, 0)), indexing="ij")
            P = (xx, yy, zz)
            solid = np.zeros(xx.shape, bool)
            for ax in range(3):
                on_face = (P[ax] < lo[ax] + tk) | (P[ax] > hi[ax] - tk)
                u, v = (ax + 1) % 3, (ax + 2) % 3

                def on_bar(k):
                    return ((P[k] - lo[k]) % sp < tk) | (P[k] > hi[k] - tk)
                solid |= on_face & (on_bar(u) | on_bar(v))
            written = self.env().materials.set_mask(solid, (int(clo[0]), int(clo[1]), int(clo[2])), m)
        if written == 0:
            self.warn(f"{a.what}: shape is empty or lies completely outside the grid")
        a.check_unknown()

    def api_frame(self, t=None, *r):
        """frame{} (ScriptEngine.cpp:1022-1030) with EnvironmentBuilder::wireframeBox
        (Environment.cpp:111-127): the twelve edges of a box as square bars `bar` cells thick."""
        a = Args(self, "frame", ["min", "max", "center", "size", "bar", "material", "name"], t)
        mn, mx = self.read_box(a)
        bar = float(f32(a.positive("bar", 2.0)))
        m = self.read_material(a, "metal")
        mn = [float(f32(v)) for v in mn]
        mx = [float(f32(v)) for v in mx]
        written = 0
        for axis in range(3):
            u, v = (axis + 1) % 3, (axis + 2) % 3
            for su in (0, 1):
                for sv in (0, 1):
                    lo, hi = list(mn), list(mx)
                    lo[u] = float(f32(mx[u] - bar)) if su else mn[u]
                    hi[u] = float(f32(lo[u] + bar))
                    lo[v] = float(f32(mx[v] - bar)) if sv else mn[v]
                    hi[v] = float(f32(lo[v] + bar))
                    written += self.env_builder().box(tuple(lo), tuple(hi), m)
        if written == 0:
            self.warn(f"{a.what}: shape is empty or lies completely outside the grid")
        a.check_unknown()

    def api_loop(self, t=None, *r):
        """loop{} (ScriptEngine.cpp:1456-1524): a square loop antenna of `size` cells in the plane normal
        to `normal`, current counter-clockwise about +normal. model "thin": four thin wires on the
        node lattice fed across one edge in the middle of the -v side; "rod": a ring of 1x1-cell rods
        fed in the middle of the -v side (4-edge gap); "current": four ideal current segments."""
        a = Args(self, "loop", ["center", "normal", "size", "amplitude", "name", "model", "radius", "feed",
                                "impedance", "material", *WAVEFORM_KEYS], t)
        self.lock()
        base = SourceDesc()
        self.read_waveform(a, base)
        c = [float(f32(v)) for v in a.vec("center", tuple(float(f32(v)) * 0.5 for v in self.settings.size))]
        n = a.axis("normal", 2)
        side = float(f32(a.positive("size", 4.0)))
        u, v = (n + 1) % 3, (n + 2) % 3  # u x v = n (right-handed)
        model = self.read_conductor(a)
        name = a.str("name", "loop")
        if model == "thin":
            sz = _round_half_away(side)
            if sz < 2:
                a.fail("a thin-wire loop needs size >= 2 cells")
            radius = self.read_radius(a, base.wavelength)
            n0 = [_round_half_away(x) for x in c]
            u0, v0 = n0[u] - sz // 2, n0[v] - sz // 2
            ug = u0 + sz // 2
            bottom, top, left, right = list(n0), list(n0), list(n0), list(n0)
            bottom[v], top[v], left[u], right[u] = v0, v0 + sz, u0, u0 + sz
            self.add_thin_wire(bottom, u, u0, u0 + sz, radius, ug)
            self.add_thin_wire(top, u, u0, u0 + sz, radius)
            self.add_thin_wire(left, v, v0, v0 + sz, radius)
            self.add_thin_wire(right, v, v0, v0 + sz, radius)
            gap = list(bottom)
            gap[u] = ug
            self.add_feed(base, gap, u, 1.0, 1, self.read_feed(a), name)
            a.check_unknown()
            return
        if model == "rod":
            sz = _round_half_away(side)
            if sz < 3:
                a.fail("a rod loop needs size >= 3 cells")
            m = self.read_material(a, "metal")
            g0 = [int(math.floor(x)) for x in c]
            u0, v0 = g0[u] - sz // 2, g0[v] - sz // 2
            ug = u0 + sz // 2
            bottom, top, left, right = list(g0), list(g0), list(g0), list(g0)
            bottom[v], top[v], left[u], right[u] = v0, v0 + sz - 1, u0, u0 + sz - 1
            self.fill_rod(bottom, u, u0, ug, m)
            self.fill_rod(bottom, u, ug + 1, u0 + sz, m)
            self.fill_rod(top, u, u0, u0 + sz, m)
            self.fill_rod(left, v, v0 + 1, v0 + sz - 1, m)
            self.fill_rod(right, v, v0 + 1, v0 + sz - 1, m)
            gap = list(bottom)
            gap[u] = ug
            self.add_feed(base, gap, u, 1.0, 4, self.read_feed(a), name)
            a.check_unknown()
            return
        amp = float(f32(a.num("amplitude", 1.0)))
        for along, at, at_sign, dir_sign in ((u, v, -1.0, 1.0), (v, u, 1.0, 1.0), (u, v, 1.0, -1.0), (v, u, -1.0, -1.0)):
            center = list(c)
            center[at] = float(f32(center[at] + f32(f32(at_sign * 0.5) * f32(side))))
            axis_vec = [0.0, 0.0, 0.0]
            axis_vec[along] = dir_sign
            d = SourceDesc.dipole(tuple(center), tuple(axis_vec), base.wavelength, amp, side)
            for k in ("wavelength", "phase", "waveform", "ramp_periods", "repeat_periods", "delay_periods", "enabled"):
                setattr(d, k, getattr(base, k))
            self.add_source(d)
        a.check_unknown()

    def taper_weights(self, a, n):
        """taperWeights (ScriptEngine.cpp:1592-1623): a name or an explicit list, normalised to a peak of 1."""
        v = a.raw("taper")
        if type(v) is LuaTable:
            if v.length() != n:
                a.fail(f"taper weights list needs {n} entries")
            return [float(f32(v.rawget(i + 1) or 0.0)) for i in range(n)]
        if v is not None and type(v) is not str:
            a.fail("taper must be a name or a list of weights")
        kind = (v or "uniform").lower()
        w = []
        for i in range(n):
            x = float(i)
            if kind == "uniform":
                val = 1.0
            elif kind == "binomial":
                val = 1.0
                for k in range(1, i + 1):
                    val = val * (n - k) / k
            elif kind == "hann":
                val = math.sin(math.pi * (x + 1.0) / (n + 1.0)) ** 2
            elif kind == "cosine":
                val = math.sin(math.pi * (x + 0.5) / n)
            elif kind == "triangular":
                val = 1.0 - abs((x - 0.5 * (n - 1)) / (0.5 * (n + 1)))
            else:
                a.fail("taper must be \"uniform\", \"binomial\", \"hann\", \"cosine\", \"triangular\" or a "
                       "weights list")
            w.append(float(f32(val)))
        mx = max(w)
        if mx > 0:
            w = [float(f32(f32(x) / f32(mx))) for x in w]
        return w

    def api_array(self, t=None, *r):
        """array{} (ScriptEngine.cpp:1625-1735): a 1-D or 2-D lattice of dipoles (fed wires or ideal
        currents) with amplitude taper and progressive phase (steer or phase_step)."""
        a = Args(self, "array", ["center", "elements", "axis", "spacing", "orientation", "length", "amplitude",
                                 "phase_step", "steer", "taper", "name", "model", "radius", "feed", "impedance",
                                 "material", "wavelength", "frequency", "phase", "waveform", "ramp", "pulse_width",
                                 "interval", "delay", "enabled"], t)
        self.lock()
        base = SourceDesc()
        self.read_waveform(a, base)
        c = a.vec("center", tuple(v * 0.5 for v in self.settings.size))
        n, ax = [1, 1], [1, 2]
        d = [float(f32(0.5 * base.wavelength))] * 2
        dphi = [0.0, 0.0]

        def read2(key, one):
            v = a.raw(key)
            if type(v) is LuaTable:
                if v.length() != 2:
                    a.fail(f"'{key}' must have two entries for a 2-D array")
                for i in range(2):
                    one(i, v.rawget(i + 1))
                return 2
            if v is not None:
                one(0, v)
                return 1
            return 0

        def as_int(v, what):
            if type(v) not in (int, float):
                a.fail(f"'{what}' entries must be numbers")
            return int(v)
        dims = read2("elements", lambda i, v: n.__setitem__(i, as_int(v, "elements")))
        if dims == 0:
            dims, n[0] = 1, 4

        def set_axis(i, v):
            p = _parse_axis(v) if type(v) is str else None
            if p is None:
                a.fail("'axis' entries must be \"x\", \"y\" or \"z\"")
            ax[i] = p
        axis_dims = read2("axis", set_axis)
        if axis_dims not in (0, dims):
            a.fail(f"'axis' needs {dims} entr{'y' if dims == 1 else 'ies'} to match 'elements'")
        if dims == 2 and axis_dims == 0:
            ax = [1, 0]
        if dims == 2 and ax[0] == ax[1]:
            a.fail("2-D array axes must differ")

        def set_spacing(i, v):
            if type(v) not in (int, float):
                a.fail("'spacing' must be a number")
            d[i] = float(f32(v))
            if dims == 2 and i == 0:
                d[1] = d[0]
        read2("spacing", set_spacing)
        has_steer, has_step = a.has("steer"), a.has("phase_step")
        if has_steer and has_step:
            a.fail("give steer (degrees from broadside) or phase_step (degrees), not both")

        def set_phase(i, v):
            if type(v) not in (int, float):
                a.fail("steer / phase_step must be numbers (degrees)")
            if has_steer:
                k = 2.0 * math.pi / base.wavelength
                dphi[i] = float(f32(-k * d[i] * math.sin(math.radians(v))))
            else:
                dphi[i] = float(f32(math.radians(v)))
        read2("steer" if has_steer else "phase_step", set_phase)
        for i in range(dims):
            if n[i] < 1 or n[i] > 64:
                a.fail("elements must be within 1..64 per axis")
            if d[i] <= 0:
                a.fail("spacing must be > 0")
            if d[i] > base.wavelength:
                self.warn(f"array: spacing {d[i]:.1f} > wavelength {base.wavelength:.1f} produces grating lobes")
        if n[0] * n[1] > 256:
            a.fail("too many elements (max 256)")
        o = a.opt_direction("orientation") or (0.0, 0.0, 1.0)
        ln = float(f32(a.num("length", 0.45 * base.wavelength)))
        if ln < 0:
            a.fail("length must be >= 0")
        elem_axis = self.wire_axis(a, o) if ln > 0 else 2
        model = self.read_conductor(a) if ln > 0 else "current"
        wire = model != "current"
        arm = self.dipole_arm(a, ln) if wire else 0
        metal = self.read_material(a, "metal") if model == "rod" else Material()
        radius = self.read_radius(a, base.wavelength) if model == "thin" else 0.0
        feed = self.read_feed(a) if wire else (True, 50.0, 1.0)
        base_name = a.str("name", "array")
        amp = float(f32(a.num("amplitude", 1.0)))
        w0 = self.taper_weights(a, n[0])
        w1 = self.taper_weights(a, n[1]) if dims == 2 else [1.0]
        sign = 1.0 if o[elem_axis] >= 0 else -1.0
        for j in range(n[1]):
            for i in range(n[0]):
                p = list(c)
                p[ax[0]] = float(f32(p[ax[0]] + f32((i - 0.5 * (n[0] - 1)) * d[0])))
                if dims == 2:
                    p[ax[1]] = float(f32(p[ax[1]] + f32((j - 0.5 * (n[1] - 1)) * d[1])))
                current = float(f32(f32(amp) * f32(w0[i]) * f32(w1[j if dims == 2 else 0])))
                timing = SourceDesc(**{k: getattr(base, k) for k in base.__dataclass_fields__})
                timing.phase = float(f32(f32(base.phase) + f32(i) * f32(dphi[0]) + f32(j) * f32(dphi[1])))
                if wire:
                    ef = (feed[0], feed[1], current)
                    ename = f"{base_name}[{i},{j}]" if dims == 2 else f"{base_name}[{i}]"
                    if model == "thin":
                        node = [_round_half_away(v) for v in p]
                        node[elem_axis] = int(math.floor(p[elem_axis]))
                        g = node[elem_axis]
                        self.add_thin_wire(node, elem_axis, g - arm, g + 1 + arm, radius, g)
                        self.add_feed(timing, node, elem_axis, sign, 1, ef, ename)
                    else:
                        cell = [int(math.floor(v)) for v in p]
                        self.fill_rod(cell, elem_axis, cell[elem_axis] - arm, cell[elem_axis], metal)
                        self.fill_rod(cell, elem_axis, cell[elem_axis] + 1, cell[elem_axis] + 1 + arm, metal)
                        self.add_feed(timing, cell, elem_axis, sign, 4, ef, ename)
                elif current != 0.0:
                    e = SourceDesc.dipole(p, o, base.wavelength, current, ln)
                    for k in ("wavelength", "phase", "waveform", "ramp_periods", "repeat_periods", "delay_periods",
                              "enabled"):
                        setattr(e, k, getattr(timing, k))
                    self.add_source(e)
        a.check_unknown()

    def api_coax(self, t=None, *r):
        """coax{} (ScriptEngine.cpp:1964-2152): a square coaxial cable of voxels (shield with end
        plates, dielectric, 1x1-cell inner conductor), a resistive generator across the first gap
        cell, a load / open / short / antenna-terminal far end, an optional sleeve balun, and the
        line monitor's set-up. Returns z0, z0_air, epsilon_r, velocity_factor, wavelength, far_end
        (and inner_terminal / outer_terminal for termination = "terminals")."""
        a = Args(self, "coax", ["from", "axis", "length", "inner", "outer", "wall", "z0", "material", "termination",
                                "load", "terminals", "balun", "balun_length", "balun_gap", "amplitude", "impedance",
                                "name", "wavelength", "frequency", "phase", "waveform", "ramp", "pulse_width",
                                "interval", "delay", "enabled"], t)
        self.lock()
        wave = SourceDesc()
        self.read_waveform(a, wave)
        frm = a.req_vec("from")
        d = a.opt_direction("axis") or (1.0, 0.0, 0.0)
        ax = self.wire_axis(a, d)
        u, v = (ax + 1) % 3, (ax + 2) % 3
        sg = 1 if d[ax] >= 0 else -1
        ln = _round_half_away(a.positive("length", 4.0 * wave.wavelength))
        inner = _round_half_away(a.num("inner", 1.0))
        outer = _round_half_away(a.num("outer", 5.0))
        wall = _round_half_away(a.num("wall", 1.0))
        if inner != 1:
            a.fail("inner must be 1 cell (the generator drives the inner conductor across a 1x1-cell gap)")
        if outer < 3 or outer % 2 == 0:
            a.fail("outer (the inside of the shield, cells) must be odd and >= 3")
        if wall < 1:
            a.fail("wall must be >= 1 cell")
        term = a.str("termination", "load").lower()
        if term not in ("load", "open", "short", "terminals"):
            a.fail("termination must be \"load\", \"open\", \"short\" or \"terminals\" (connect an antenna)")
        if ln < 2 * outer + 12:
            a.fail(f"length must be at least {2 * outer + 12} cells for this cross-section")
        name = a.str("name", "cable")
        g = coax_geometry_factor(inner, outer)
        z0_air = K_ETA0 / g
        if a.has("material"):
            diel = self.read_material(a, "vacuum")
        else:
            target = a.positive("z0", 50.0)
            er = (z0_air / target) * (z0_air / target)
            if er < 1.0:
                self.warn(f"coax: {target:.1f} ohm needs a wider shield; with outer = {outer} the air-filled line "
                          f"is {z0_air:.1f} ohm")
                er = 1.0
            diel = Material(0.0, float(max(f32(er), f32(1.0))))
            if er > 1.0:
                key = name + " dielectric"
                self.used_dielectrics[key] = max(self.used_dielectrics.get(key, 0.0), diel.epsilon_r)
        z0 = z0_air / math.sqrt(max(diel.epsilon_r, 1.0))
        tdir = a.opt_direction("terminals") or ((0.0, 1.0, 0.0) if ax == 2 else (0.0, 0.0, 1.0))
        tax = self.wire_axis(a, tdir)
        if tax == ax:
            a.fail("terminals must be perpendicular to the cable axis")
        ts = 1 if tdir[tax] >= 0 else -1
        start = _round_half_away(frm[ax])
        centre = [0.0, 0.0, 0.0]
        centre[ax] = float(start)
        centre[u] = float(f32(math.floor(frm[u]) + 0.5))
        centre[v] = float(f32(math.floor(frm[v]) + 0.5))
        b = self.env_builder()

        def put(t0, t1, size, m):
            lo, hi = [0.0] * 3, [0.0] * 3
            lo[ax] = float(start + t0 if sg > 0 else start - t1)
            hi[ax] = float(start + t1 if sg > 0 else start - t0)
            for k in (u, v):
                lo[k] = float(f32(centre[k] - 0.5 * size))
                hi[k] = float(f32(centre[k] + 0.5 * size))
            b.box(lo, hi, m)
        metal = Material(float(f32(4.0 * float(K_PERFECT_EDGE_SIGMA))), 1.0)
        shield = outer + 2 * wall
        capped = term != "terminals"
        c = CoaxSetup(name, ax, sg, start, tuple(centre), ln, inner, outer, wall, epsilon_r=diel.epsilon_r,
                      z0_ohm=float(f32(z0)), wavelength=wave.wavelength, cell_size=float(f32(self.settings.cell_size)),
                      termination=term, pulsed=wave.waveform == abi.WAVE_PULSE)
        if a.boolean("balun", False):
            bl = _round_half_away(a.positive("balun_length", 0.25 * wave.wavelength))
            gap = _round_half_away(a.positive("balun_gap", 2.0))
            sleeve = shield + 2 * (gap + wall)
            if bl + wall >= ln - 4:
                a.fail("balun_length is too long for this cable")
            put(ln - bl - wall, ln, sleeve, metal)
            put(ln - bl, ln, shield + 2 * gap, Material())
            c.sleeve_start, c.sleeve_end, c.sleeve_outer = ln - bl - wall, ln, sleeve
        put(-wall, ln + wall if capped else ln, shield, metal)
        put(0, ln, outer, diel)
        inner_end = {"terminals": ln + 3, "short": ln, "load": ln - 1}.get(term, ln - 2)
        put(1, inner_end, inner, metal)
        gen_ohm = float(f32(a.positive("impedance", z0)))
        drive = float(f32(a.num("amplitude", 1.0)))
        gap_cell = [0, 0, 0]
        gap_cell[ax] = start if sg > 0 else start - 1
        gap_cell[u] = int(math.floor(centre[u]))
        gap_cell[v] = int(math.floor(centre[v]))
        self.add_feed(wave, gap_cell, ax, float(sg), 4, (True, gen_ohm, drive), name)
        c.source_ohm, c.drive = gen_ohm, drive
        c.load_ohm = float(f32(a.positive("load", z0)))
        if term == "load":
            cell = list(gap_cell)
            cell[ax] = start + ln - 1 if sg > 0 else start - ln
            quiet = SourceDesc(**{k: getattr(wave, k) for k in wave.__dataclass_fields__})
            quiet.enabled = True
            self.add_feed(quiet, cell, ax, float(-sg), 4, (True, c.load_ohm, 0.0), name + " load")
        elif a.has("load"):
            self.warn("coax: 'load' only applies to termination = \"load\"")
        inner_node, outer_node = [0.0] * 3, [0.0] * 3
        if term == "terminals":
            tu = v if tax == u else u
            lo, hi = [0.0] * 3, [0.0] * 3
            lo[ax] = float(start + ln if sg > 0 else start - ln - 3)
            hi[ax] = float(start + ln + 3 if sg > 0 else start - ln)
            lo[tu], hi[tu] = centre[tu] - 0.5, centre[tu] + 0.5
            wall_in = 0.5 * outer
            wall_out = wall_in + wall
            lo[tax] = centre[tax] - wall_out if ts > 0 else centre[tax] + wall_in
            hi[tax] = centre[tax] - wall_in if ts > 0 else centre[tax] + wall_out
            b.box(lo, hi, metal)
            inner_node[ax] = outer_node[ax] = float(start + sg * (ln + 2))
            inner_node[tu] = outer_node[tu] = centre[tu] - 0.5
            inner_node[tax] = centre[tax] + 0.5 * ts
            outer_node[tax] = centre[tax] - ts * wall_out
        self.env().coaxes.append(c)
        a.check_unknown()
        out = LuaTable()
        out.rawset("z0", z0)
        out.rawset("z0_air", z0_air)
        out.rawset("epsilon_r", diel.epsilon_r)
        out.rawset("velocity_factor", 1.0 / math.sqrt(max(diel.epsilon_r, 1.0)))
        out.rawset("wavelength", wave.wavelength / math.sqrt(max(diel.epsilon_r, 1.0)))
        end = list(centre)
        end[ax] = float(start + sg * ln)
        out.rawset("far_end", self.vec(*end))
        if term == "terminals":
            out.rawset("inner_terminal", self.vec(*inner_node))
            out.rawset("outer_terminal", self.vec(*outer_node))
        return out

    # -- antennas (ScriptEngine.cpp:1077-1460)
    def add_thin_wire(self, node, axis, i0, i1, radius, gap=None):
        if i1 <= i0:
            return
        self.env_builder().add_thin_wire(node, axis, i0, i1, radius, gap)

    def add_feed(self, wave, texel, axis, sign, edges, feed, name):
        voltage, imp, drive = feed
        self.env_builder().add_feed(wave, texel, axis, sign, edges, imp, drive, voltage, name)

    def api_dipole(self, t=None, *r):
        a = Args(self, "dipole", ["center", "orientation", "length", "amplitude", "name", "model", "radius", "feed",
                                  "impedance", "material", "wavelength", "frequency", "phase", "waveform", "ramp",
                                  "pulse_width", "interval", "delay", "enabled"], t)
        self.lock()
        s = SourceDesc()
        self.read_waveform(a, s)
        c = a.vec("center", tuple(v * 0.5 for v in self.settings.size))
        o = a.opt_direction("orientation") or (0.0, 0.0, 1.0)
        ln = a.num("length", 0.0)
        if ln < 0.0:
            a.fail("length must be >= 0")
        model = self.read_conductor(a) if ln > 0.0 else "current"
        if model != "current":
            ax = self.wire_axis(a, o)
            radius = self.read_radius(a, s.wavelength) if model == "thin" else 0.0
            metal = self.read_material(a, "metal") if model == "rod" else Material()
            if model == "thin" and a.has("material"):
                self.warn("dipole: thin wires are perfect conductors; 'material' applies to model = \"rod\"")
            sign = 1.0 if o[ax] >= 0.0 else -1.0
            arm = self.dipole_arm(a, ln)
            feed = self.read_feed(a)
            name = a.str("name", "dipole")
            if model == "thin":
                node = [_round_half_away(v) for v in c]
                node[ax] = int(math.floor(c[ax]))
                g = node[ax]
                self.add_thin_wire(node, ax, g - arm, g + 1 + arm, radius, g)
                self.add_feed(s, node, ax, sign, 1, feed, name)
            else:
                cell = [int(math.floor(v)) for v in c]
                self.fill_rod(cell, ax, cell[ax] - arm, cell[ax], metal)
                self.fill_rod(cell, ax, cell[ax] + 1, cell[ax] + 1 + arm, metal)
                self.add_feed(s, cell, ax, sign, 4, feed, name)
        else:
            if ln > 0.0:
                self.wire_axis(a, o)
            for k in ("radius", "feed", "impedance", "material"):
                if a.has(k):
                    self.warn(f"dipole: '{k}' does not apply to an ideal current element")
            d = SourceDesc.dipole(c, o, s.wavelength, float(f32(a.num("amplitude", 1.0))), ln)
            for k in ("wavelength", "phase", "waveform", "ramp_periods", "repeat_periods", "delay_periods",
                      "enabled"):
                setattr(d, k, getattr(s, k))
            self.add_source(d)
        a.check_unknown()

    def api_monopole(self, t=None, *r):
        a = Args(self, "monopole", ["base", "orientation", "length", "amplitude", "name", "model", "radius", "feed",
                                    "impedance", "material", "wavelength", "frequency", "phase", "waveform", "ramp",
                                    "pulse_width", "interval", "delay", "enabled"], t)
        self.lock()
        s = SourceDesc()
        self.read_waveform(a, s)
        base = a.req_vec("base")
        o = a.opt_direction("orientation") or (0.0, 0.0, 1.0)
        ax = self.wire_axis(a, o)
        sign = 1.0 if o[ax] >= 0.0 else -1.0
        ln = float(f32(a.positive("length", 0.25 * s.wavelength)))
        if ln < 2.0:
            a.fail("length must be >= 2 cells (feed gap plus rod)")
        rod = max(1, _round_half_away(ln) - 1)
        if abs(rod + 1 - ln) >= 1.0:
            self.warn(f"monopole: length {ln:.1f} realised as {rod + 1} cells (1-cell feed gap + {rod}-cell "
                      f"conductor)")
        model = self.read_conductor(a)
        if model == "current":
            a.fail("a monopole needs a conductor: use model = \"thin\" or \"rod\"")
        feed = self.read_feed(a)
        name = a.str("name", "monopole")
        surface = _round_half_away(base[ax])
        g = surface if sign > 0 else surface - 1
        if model == "thin":
            node = [_round_half_away(v) for v in base]
            node[ax] = g
            radius = self.read_radius(a, s.wavelength)
            if sign > 0:
                self.add_thin_wire(node, ax, g, g + 1 + rod, radius, g)
            else:
                self.add_thin_wire(node, ax, g - rod, g + 1, radius, g)
            self.add_feed(s, node, ax, sign, 1, feed, name)
            chk = list(node)
            chk[ax] = surface
            self.monopoles.append((True, tuple(chk), ax, sign))
        else:
            cell = [int(math.floor(v)) for v in base]
            cell[ax] = g
            m = self.read_material(a, "metal")
            if sign > 0:
                self.fill_rod(cell, ax, g + 1, g + 1 + rod, m)
            else:
                self.fill_rod(cell, ax, g - rod, g, m)
            self.add_feed(s, cell, ax, sign, 4, feed, name)
            chk = list(cell)
            chk[ax] -= int(sign)
            self.monopoles.append((False, tuple(chk), ax, sign))
        a.check_unknown()

    def api_wire(self, t=None, *r):
        a = Args(self, "wire", ["from", "to", "radius", "name"], t)
        self.lock()
        p0 = [_round_half_away(v) for v in a.req_vec("from")]
        p1 = [_round_half_away(v) for v in a.req_vec("to")]
        d = [p1[i] - p0[i] for i in range(3)]
        if sum(1 for v in d if v != 0) != 1:
            a.fail("from and to must differ along exactly one axis (thin wires run along x, y or z); build bent or "
                   "slanted conductors from several wires or from metal shapes")
        ax = 0 if d[0] != 0 else (1 if d[1] != 0 else 2)
        self.add_thin_wire(p0, ax, min(p0[ax], p1[ax]), max(p0[ax], p1[ax]),
                           self.read_radius(a, self.settings.wavelength))
        a.check_unknown()

    def api_sheet(self, t=None, *r):
        a = Args(self, "sheet", ["min", "max", "center", "size", "name"], t)
        self.lock()
        mn, mx = self.read_box(a)
        lo = [_round_half_away(float(v)) for v in mn]
        hi = [_round_half_away(float(v)) for v in mx]
        normal = -1
        for i in range(3):
            if lo[i] == hi[i]:
                if normal >= 0:
                    a.fail("a sheet needs a non-zero extent along two axes (use wire{} for a line)")
                normal = i
        if normal < 0:
            a.fail("a sheet has zero thickness: give min and max equal along its normal axis (e.g. min.z == max.z), "
                   "or a size with one zero component; use box{} for solid metal")
        u, v = (normal + 1) % 3, (normal + 2) % 3
        edges = self.env().edges
        sig = float(K_PERFECT_EDGE_SIGMA)
        for iu in range(lo[u], hi[u] + 1):
            for iv in range(lo[v], hi[v] + 1):
                q = list(lo)
                q[u], q[v] = iu, iv
                if iu < hi[u]:
                    edges.append(abi.EdgeOverride(q[0], q[1], q[2], u, sig))
                if iv < hi[v]:
                    edges.append(abi.EdgeOverride(q[0], q[1], q[2], v, sig))
        a.check_unknown()

    def api_sweep(self, t=None, *r):
        a = Args(self, "sweep", ["wavelengths", "frequencies", "points", "log", "name"], t)
        self.lock()
        hw, hf = a.has("wavelengths"), a.has("frequencies")
        if hw == hf:
            a.fail("give the band as wavelengths = {lo, hi} (cells) or frequencies = {lo, hi} (Hz)")
        band = a.opt_vec2("wavelengths" if hw else "frequencies")
        if band is None or not band[0] > 0 or not band[1] > 0 or band[0] == band[1]:
            a.fail("the band needs two different positive values")
        if hw:
            wmin, wmax = min(band), max(band)
        else:
            cell = float(f32(self.settings.cell_size))
            wmin = float(f32(K_C0 / (max(band) * cell)))
            wmax = float(f32(K_C0 / (min(band) * cell)))
        if wmin < 6.0:
            self.warn(f"sweep: the band reaches {wmin:.1f} cells per wavelength; below ~10 the results are inaccurate")
        self.env().sweep = {"wavelength_min": wmin, "wavelength_max": wmax,
                            "points": min(max(a.integer("points", 81), 2), 2001), "log": a.str("log", "")}
        a.check_unknown()

    # -- plane waves and current sources (ScriptEngine.cpp:1526-1590, 1737-1755)
    def add_sheet(self, a, axis, pos, center, half, soft):
        self.lock()
        base = SourceDesc()
        self.read_waveform(a, base)
        pol = a.opt_direction("polarization")
        if pol is None:
            p = [0.0, 0.0, 0.0]
            p[0 if axis == 2 else 2] = 1.0
            pol = tuple(p)
        pol = list(pol)
        if abs(pol[axis]) > 1e-4:
            self.warn(f"{a.what}: polarization has a component along the propagation axis; it was removed")
            pol[axis] = 0.0
            n = math.sqrt(sum(v * v for v in pol))
            if n < 1e-6:
                a.fail("polarization must be perpendicular to the propagation axis")
            pol = [float(f32(v / n)) for v in pol]
        d = a.str("direction", "+").lower()
        if d not in ("+", "-", "both"):
            a.fail("direction must be \"+\", \"-\" or \"both\"")
        e0 = a.num("amplitude", 1.0)
        one_way = d != "both"
        s = SourceDesc(**{k: getattr(base, k) for k in base.__dataclass_fields__})
        c = list(center)
        c[axis] = pos
        s.center = tuple(float(f32(v)) for v in c)
        s.half_extent = tuple(float(v) for v in half)
        s.softness = tuple(float(v) for v in soft)
        s.polarization = tuple(pol)
        s.amplitude = sheet_current_for_field(0.5 * e0 if one_way else e0, s.wavelength, soft[axis])
        self.add_source(s)
        if one_way:
            s2 = SourceDesc(**{k: getattr(s, k) for k in s.__dataclass_fields__})
            c2 = list(s.center)
            c2[axis] = float(f32(c2[axis] + (1.0 if d == "+" else -1.0) * float(f32(0.25 * s.wavelength))))
            s2.center = tuple(c2)
            s2.delay_periods = float(f32(s.delay_periods + 0.25))
            self.add_source(s2)
        self.sheet_sources += 1

    def api_plane_wave(self, t=None, *r):
        a = Args(self, "plane_wave", ["axis", "position", "polarization", "amplitude", "direction", "name",
                                      "wavelength", "frequency", "phase", "waveform", "ramp", "pulse_width",
                                      "interval", "delay", "enabled"], t)
        axis = a.axis("axis", 0)
        pos = float(f32(a.num("position", self.settings.pml + 8.0)))
        half = [1.0e5, 1.0e5, 1.0e5]
        half[axis] = 0.0
        soft = [K_SHEET_SOFTNESS] * 3
        self.add_sheet(a, axis, pos, (0.0, 0.0, 0.0), half, soft)
        a.check_unknown()

    def api_gaussian_beam(self, t=None, *r):
        a = Args(self, "gaussian_beam", ["axis", "position", "center", "waist", "polarization", "amplitude",
                                         "direction", "name", "wavelength", "frequency", "phase", "waveform", "ramp",
                                         "pulse_width", "interval", "delay", "enabled"], t)
        axis = a.axis("axis", 0)
        pos = float(f32(a.num("position", self.settings.pml + 8.0)))
        c = a.vec("center", tuple(v * 0.5 for v in self.settings.size))
        waist = float(f32(a.positive("waist", 2.0 * self.settings.wavelength)))
        soft = [waist] * 3
        soft[axis] = K_SHEET_SOFTNESS
        self.add_sheet(a, axis, pos, c, (0.0, 0.0, 0.0), soft)
        a.check_unknown()

    def api_current_source(self, t=None, *r):
        a = Args(self, "current_source", ["min", "max", "center", "size", "polarization", "amplitude", "softness",
                                          "name", "wavelength", "frequency", "phase", "waveform", "ramp",
                                          "pulse_width", "interval", "delay", "enabled"], t)
        self.lock()
        s = SourceDesc()
        self.read_waveform(a, s)
        mn, mx = self.read_box(a)
        s.center = tuple(float(v) for v in f32(0.5) * (mn + mx))
        s.half_extent = tuple(float(v) for v in f32(0.5) * (mx - mn))
        s.softness = a.vec("softness", (K_DIPOLE_SOFTNESS,) * 3)
        s.polarization = a.opt_direction("polarization") or (0.0, 0.0, 1.0)
        s.amplitude = float(f32(a.num("amplitude", 1.0)))
        self.add_source(s)
        a.check_unknown()

    # -- instruments (ScriptEngine.cpp:1757-1805, 2154-2190)
    def api_probe(self, t=None, *r):
        a = Args(self, "probe", ["position", "name", "log"], t)
        self.lock()
        pos = a.req_vec("position")
        sc = self.env()
        sc.probes.append((a.str("name", f"probe{len(sc.probes) + 1}"), pos))
        sc.probe_logs.append(a.str("log", ""))
        a.check_unknown()

    def api_flux_plane(self, t=None, *r):
        a = Args(self, "flux_plane", ["axis", "position", "min", "max", "name", "log"], t)
        self.lock()
        axis = a.axis("axis", 0)
        n = self.settings.size
        u, v = (1 if axis == 0 else 0), (1 if axis == 2 else 2)
        L0 = float(self.settings.pml)
        lo = a.opt_vec2("min") or (L0, L0)
        hi = a.opt_vec2("max") or (float(n[u] - L0), float(n[v] - L0))
        fl = self.env().fluxes
        f = FluxSetup(a.str("name", f"flux{len(fl) + 1}"), "plane", axis=axis,
                      index=_round_half_away(a.req_num("position")),
                      rect_min=tuple(_round_half_away(c) for c in lo), rect_max=tuple(_round_half_away(c) for c in hi),
                      log=a.str("log", ""))
        fl.append(f)
        a.check_unknown()

    def api_flux_box(self, t=None, *r):
        a = Args(self, "flux_box", ["min", "max", "center", "size", "name", "log"], t)
        self.lock()
        mn, mx = self.read_box(a)
        lo = [_round_half_away(float(v)) for v in mn]
        hi = [_round_half_away(float(v)) for v in mx]
        fl = self.env().fluxes
        fl.append(FluxSetup(a.str("name", f"flux{len(fl) + 1}"), "box",
                            tuple(min(p, q) for p, q in zip(lo, hi)), tuple(max(p, q) for p, q in zip(lo, hi)),
                            log=a.str("log", "")))
        a.check_unknown()

    def api_warning(self, msg=None, *r):
        if type(msg) not in (str, int, float):
            raise LuaError("bad argument #1 to 'warning' (string expected)")
        self.warn(tostr(msg))

    def api_far_field(self, t=None, *r):
        a = Args(self, "far_field", ["min", "max", "center", "size", "margin", "wavelength", "frequency",
                                     "averaging", "name", "log", "axis"], t)
        self.lock()
        s = self.settings
        if a.has("min") or a.has("max") or a.has("size"):
            mn, mx = self.read_box(a)
            bmin = tuple(_round_half_away(float(v)) for v in mn)
            bmax = tuple(_round_half_away(float(v)) for v in mx)
        else:
            margin = a.integer("margin", 4)
            bmin = (s.pml + 1 + margin,) * 3
            bmax = tuple(n - s.pml - 2 - margin for n in s.size)
        ff = {"box_min": bmin, "box_max": bmax, "wavelength": self.read_wavelength(a),
              "averaging": float(f32(a.positive("averaging", 4.0))), "name": a.str("name", "far field"),
              "log": a.str("log", ""), "axis": (0.0, 0.0, 1.0)}
        ax = a.opt_direction("axis")
        if ax is not None:
            d = [abs(v) for v in ax]
            i = 0 if (d[0] >= d[1] and d[0] >= d[2]) else (1 if d[1] >= d[2] else 2)
            if d[i] < 0.9999:
                a.fail("axis must be along x, y or z (\"+x\", \"-z\", ...)")
            m = [0.0, 0.0, 0.0]
            m[i] = 1.0 if ax[i] > 0 else -1.0
            ff["axis"] = tuple(m)
        if self.env().far_field is not None:
            self.warn("far_field: only one far-field monitor is supported; replacing the previous one")
        self.env().far_field = ff
        a.check_unknown()

    # ------------------------------------------------------------------ run
    def final_checks(self, sc):
        n = np.asarray(sc.grid.size, f32)
        L = f32(sc.grid.pml_thickness)

        def in_absorber(p):
            p = np.asarray(p, f32)
            return bool(np.any(p < L) or np.any(p >= n - L))
        if not sc.sources:
            self.warn("scene has no (enabled) sources: nothing will radiate")
        for thin, node, axis, sign in self.monopoles:
            grounded = False
            mats = sc.materials
            if not thin:
                grounded = mats.get(node).sigma >= 1.0
            else:
                u, v = (axis + 1) % 3, (axis + 2) % 3
                for du in (-1, 0):
                    for dv in (-1, 0):
                        cell = list(node)
                        cell[u] += du
                        cell[v] += dv
                        cell[axis] = node[axis] - 1 if sign > 0 else node[axis]
                        grounded = grounded or mats.get(cell).sigma >= 1.0
                for e in sc.edges:
                    if grounded:
                        break
                    if e.sigma < 0.5 * float(K_PERFECT_EDGE_SIGMA):
                        continue
                    end = [e.x, e.y, e.z]
                    end[e.axis] += 1
                    grounded = (e.x, e.y, e.z) == tuple(node) or tuple(end) == tuple(node)
            if not grounded:
                self.warn("monopole: no conductor touches the base of the feed gap, so the feed has nothing to drive "
                          "against. Add a ground plane, radials or wall at the base.")
        for name, eps in self.used_dielectrics.items():
            lam = sc.wavelength / math.sqrt(eps)
            if lam < 8.0:
                self.warn(f"material '{name}' (eps_r = {eps:g}) shortens the wavelength to {lam:.1f} cells; below ~8 "
                          f"cells per wavelength the results are inaccurate (increase scene.wavelength)")
        for name, pos in sc.probes:
            if in_absorber(pos):
                self.warn(f"probe '{name}' lies inside the absorbing boundary layer")
        for s in sc.sources:
            if math.sqrt(sum(v * v for v in s.half_extent)) < 1e3 and in_absorber(s.center):
                self.warn("a source lies inside the absorbing boundary layer (it will be damped)")
        if sc.sweep is not None:
            pulsed = any(s.waveform == abi.WAVE_PULSE for s in sc.sources)
            if not sc.ports:
                self.warn("sweep: the scene has no antenna feeds (ports) to sweep")
            elif not pulsed:
                self.warn("sweep: the antennas are driven with a continuous wave, which only contains one frequency; "
                          "use waveform = \"pulse\" for a frequency sweep")
        if sc.far_field is not None and self.sheet_sources > 0:
            self.warn("far_field: plane-wave / beam sources cross the Huygens box; the pattern is only meaningful "
                      "for localized sources (antennas)")

    def run_source(self, src: str, chunk: str = "scene") -> ScriptResult:
        try:
            self.I.execute(src, chunk)
            self.lock()
            sc = self.builder.build()  # emits the thin wires (PEC edges, end correction, 2/ln(1/a) terms)
            sc.view = dict(self.view)
            sc.cell_size = self.settings.cell_size
            sc.wavelength = self.settings.wavelength
            sc.radar = self.radar
            sc.targets = list(self.targets)
            sc.emitters = list(self.emitters)
            sc.crpa = self.crpa
            self.final_checks(sc)
        except LuaError as e:
            raise ScriptError(str(e)) from None
        except RecursionError:
            raise ScriptError(f"{chunk}: stack overflow") from None
        return ScriptResult(sc, self.settings, self.params, self.warnings, self.output)

    def run_file(self, path) -> ScriptResult:
        with open(path, "r", encoding="utf-8") as f:
            src = f.read()
        res = self.run_source(src, os.path.basename(str(path)))
        if self.radar is not None and self.with_targets:
            # the radar's calibration scene: everything except the targets (ScriptEngine.cpp:2581-2592)
            bg = ScriptEngine(self.overrides, echo=False, with_targets=False).run_source(src, os.path.basename(str(path)))
            res.background = bg.scene
            if not self.targets:
                res.warnings.append("radar: no object is marked target = true, so the calibration (which removes "
                                    "the targets) sees the same scene and every echo cancels; mark what the radar "
                                    "should detect with target = true")
        base = os.path.dirname(os.path.abspath(str(path)))
        od = self.settings.output_dir
        stem = os.path.splitext(os.path.basename(str(path)))[0]
        res.output_dir = (os.path.join(base, "output", stem) if not od else
                          (od if os.path.isabs(od) else os.path.join(base, od)))
        return res


def coax_geometry_factor(inner: int, outer: int) -> float:
    """CoaxMonitor::geometryFactor (Coax.cpp:43-78): Laplace's equation on the lattice nodes of
    the square cross-section (inner conductor at 1, shield at 0) by SOR in the same sweep order;
    G = sum over the transverse edges of (delta phi)^2, so Z0 = eta0 / (sqrt(eps_r) G)."""
    n = outer + 1
    lo = (outer - inner) // 2
    hi = lo + inner
    phi = [0.0] * (n * n)
    fixed = [False] * (n * n)
    for j in range(n):
        for i in range(n):
            k = j * n + i
            if i == 0 or j == 0 or i == n - 1 or j == n - 1:
                fixed[k] = True
            if lo <= i <= hi and lo <= j <= hi:
                fixed[k] = True
                phi[k] = 1.0
    omega = 2.0 / (1.0 + math.sin(math.pi / n))
    for _ in range(20000):
        change = 0.0
        for j in range(1, n - 1):
            for i in range(1, n - 1):
                k = j * n + i
                if fixed[k]:
                    continue
                target = 0.25 * (((phi[k - 1] + phi[k + 1]) + phi[k - n]) + phi[k + n])
                d = omega * (target - phi[k])
                phi[k] += d
                change = max(change, abs(d))
        if change < 1e-13:
            break
    g = 0.0
    for j in range(n):
        for i in range(n):
            k = j * n + i
            if i + 1 < n:
                g += (phi[k + 1] - phi[k]) * (phi[k + 1] - phi[k])
            if j + 1 < n:
                g += (phi[k + n] - phi[k]) * (phi[k + n] - phi[k])
    return g


def sheet_current_for_field(field_amplitude, wavelength, softness) -> float:
    """SourceDesc::sheetCurrentForField (SimulationGrid.cpp:58-63): the sheet current whose
    Gaussian footprint radiates a plane wave of the given field amplitude."""
    k = 2.0 * math.pi / max(float(wavelength), 1e-3)
    s = max(float(softness), 0.25)
    spectral = s * math.sqrt(math.pi) * math.exp(-0.25 * k * k * s * s)
    return float(f32(2.0 * float(f32(field_amplitude)) / spectral))


def run_script(path, overrides=None, echo=True) -> ScriptResult:
    return ScriptEngine(overrides, echo).run_file(path)
