"""Instruments of a headless run: probes, flux monitors, ports and sweep, far field, and the
console report, over the solver's C ABI.

Host arithmetic of the reference's instruments on the device readbacks: probe interpolation
(src/FieldAnalyzer.cpp:17-40, 237-262), flux sums with outward signs and their running average
(FieldAnalyzer.cpp:175-190, 264-270; Instruments.cpp:240-262), port readings
(src/Ports.cpp:159-185), the frequency sweep analysis (Ports.cpp:187-278; the FP64 DFT sums
themselves run on the device), the far-field direction set and pattern analysis
(src/FarField.cpp:27-53, 79-124, 294-335), and the periodic report (src/Instruments.cpp:317-444,
445-493) with the same line formats.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

from . import abi

K_ETA0 = 376.730313668
K_C0 = 299792458.0
K_CUT_SAMPLES = 180
K_MAP_SIZE = 81
NO_INSTRUMENTS_HINT = ("No instruments in this scene, so there are no readings to report. Add probe{}, flux_plane{}, "
                       "flux_box{} or far_field{} to the script, or feed an antenna, to measure fields, power, "
                       "impedance or radiation patterns.")


def boresight_frame(n):
    """boresightFrame (FarField.hpp:29-37): right and up as seen from behind, looking along n."""
    n = np.asarray(n, np.float32)
    if abs(n[2]) > 0.5:
        return np.array([1, 0, 0], np.float32), np.array([0, 1, 0], np.float32)
    up = np.array([0, 0, 1], np.float32)
    return np.cross(n, up).astype(np.float32), up


def far_field_directions(axis):
    """buildDirections (FarField.cpp:79-124): three principal cuts of 180 samples, then the two
    hemispheric u-v maps (81 x 81, directions inside the unit circle) around `axis`."""
    dirs = []
    cuts = []
    for name, a, b in (("xy", (1, 0, 0), (0, 1, 0)), ("xz", (1, 0, 0), (0, 0, 1)), ("yz", (0, 1, 0), (0, 0, 1))):
        a = np.asarray(a, np.float32)
        b = np.asarray(b, np.float32)
        angles = []
        for i in range(K_CUT_SAMPLES):
            deg = np.float32(360.0) * np.float32(i) / np.float32(K_CUT_SAMPLES)
            rad = np.float32(math.radians(float(deg)))
            angles.append(float(deg))
            dirs.append(np.float32(math.cos(rad)) * a + np.float32(math.sin(rad)) * b)
        cuts.append({"name": name, "angles": angles})
    ax = 2
    for i in range(3):
        if abs(axis[i]) > abs(axis[ax]):
            ax = i
    n = np.zeros(3, np.float32)
    n[ax] = 1.0 if axis[ax] >= 0 else -1.0
    eu, ev = boresight_frame(n)
    for h in range(2):
        for r in range(K_MAP_SIZE):
            for c in range(K_MAP_SIZE):
                # float arithmetic in the reference's order: -1 + (2 c) / (N - 1), 1 - (2 r) / (N - 1)
                u = np.float32(-1.0) + np.float32(np.float32(2.0 * c) / np.float32(K_MAP_SIZE - 1))
                v = np.float32(1.0) - np.float32(np.float32(2.0 * r) / np.float32(K_MAP_SIZE - 1))
                rho2 = np.float32(u * u) + np.float32(v * v)
                if rho2 > np.float32(1.0):
                    continue
                w = np.sqrt(max(np.float32(1.0) - rho2, np.float32(0.0)))
                dirs.append(u * eu + v * ev + (w if h == 0 else -w) * n)
    return np.array(dirs, np.float32), cuts


def _round_half_away(x: float) -> int:
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def _g(v):
    """A number as C++ streams print it by default (6 significant digits, %g)."""
    return "%g" % v


def to_dbi(d):
    return float(np.float32(10.0 * math.log10(d))) if d > 1e-12 else -120.0


def analyse_cut(cut, dbi):
    """analyseCut (FarField.cpp:27-53): peak, -3 dB beamwidth by linear interpolation, front/back."""
    n = len(dbi)
    peak = int(np.argmax(dbi))
    cut["peak_dbi"] = dbi[peak]
    cut["peak_angle"] = cut["angles"][peak]
    step = 360.0 / n
    thr = dbi[peak] - 3.0

    def at(i):
        return dbi[((i % n) + n) % n]
    half = [-1.0, -1.0]
    for k_dir, sgn in enumerate((1, -1)):
        for k in range(1, n // 2 + 1):
            a, b = at(peak + sgn * (k - 1)), at(peak + sgn * k)
            if b < thr:
                frac = (a - thr) / max(a - b, 1e-6)
                half[k_dir] = (k - 1 + frac) * step
                break
    cut["beamwidth"] = 360.0 if (half[0] < 0 or half[1] < 0) else half[0] + half[1]
    cut["dbi"] = dbi
    cut["front_back"] = dbi[peak] - at(peak + n // 2)


def _len32(v) -> float:
    """|v| of a float vector in float32, as glm::length: a diverged field gives inf (the non-finite
    check reports it), without numpy's overflow warnings."""
    a = np.asarray(v, np.float32)
    with np.errstate(over="ignore", invalid="ignore"):
        return math.sqrt(float(np.float32(np.dot(a, a))))


def _cross32(a, b):
    with np.errstate(over="ignore", invalid="ignore"):
        return np.cross(np.asarray(a, np.float32), np.asarray(b, np.float32))


def probe_origin(pos, size):
    p = [min(max(float(v), 0.0), float(n - 1)) for v, n in zip(pos, size)]
    return [min(max(int(math.floor(v)) - 1, 0), max(n - 3, 0)) for v, n in zip(p, size)]


def sample_block(block, origin, extent, q, ch):
    """sampleBlock (FieldAnalyzer.cpp:17-40): trilinear interpolation in a 3x3x3 block."""
    fl = [math.floor(v) for v in q]
    f = [np.float32(v - w) for v, w in zip(q, fl)]
    i0 = [int(fl[k]) - origin[k] for k in range(3)]
    res = np.float32(0.0)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = ((f[0] if dx else np.float32(1) - f[0]) * (f[1] if dy else np.float32(1) - f[1])
                     * (f[2] if dz else np.float32(1) - f[2]))
                if w != 0:
                    x = min(max(i0[0] + dx, 0), extent[0] - 1)
                    y = min(max(i0[1] + dy, 0), extent[1] - 1)
                    z = min(max(i0[2] + dz, 0), extent[2] - 1)
                    res = np.float32(res + w * block[(z * 3 + y) * 3 + x][ch])
    return float(res)


class Instruments:
    """Instruments::configure / measure / evaluate / printReport for one scene on one grid."""

    def __init__(self, grid, scene, out=print, output_dir=""):
        self.g = grid
        self.sc = scene
        self.out = out
        self.output_dir = output_dir
        self.warnings = []
        self.size = tuple(scene.grid.size)
        self.averaging_time = 3.0 * max(scene.wavelength, 2.0)
        self.unstable = False
        self.measure_time, self.measure_step = 0.0, 0
        self.probes = []
        logs = list(getattr(scene, "probe_logs", [])) + [""] * len(scene.probes)
        for (name, pos), log in zip(scene.probes, logs):
            p = tuple(min(max(float(v), 0.0), float(n - 1)) for v, n in zip(pos, self.size))
            self.probes.append({"name": name, "pos": p, "sample": None,
                                "log": self.open_log(log, "step,time,Ex,Ey,Ez,Bx,By,Bz,absE,absB,Sx,Sy,Sz")})
        self.fluxes = [{"setup": f, "inst": 0.0, "avg": 0.0, "peak": 0.0, "last": -1.0,
                        "log": self.open_log(f.log, "step,time,P,P_avg")} for f in scene.fluxes]
        self.ports = list(scene.ports)
        self.readings = [None] * len(self.ports)
        self.sweep_setup = scene.sweep if self.ports else None
        self.sweep_result = None
        self.ff = scene.far_field
        self.pattern = None
        self.port_start = 0.0
        self.ff_start = 0.0
        self.coaxes = list(getattr(scene, "coaxes", []))
        self.coax_readings = [None] * len(self.coaxes)
        self.radar = None
        self.crpa = None
        self.configure()

    # ------------------------------------------------------------------ set-up
    def resolve(self, path):
        if not path:
            return ""
        p = path if os.path.isabs(path) or not self.output_dir else os.path.join(self.output_dir, path)
        d = os.path.dirname(p)
        if d:
            os.makedirs(d, exist_ok=True)
        return p

    def open_log(self, path, header):
        """Instruments::openLog (Instruments.cpp:19-33): CSV with a header line, relative paths
        under the scene's output directory."""
        if not path:
            return None
        try:
            f = open(self.resolve(path), "w")
        except OSError:
            self.warnings.append(f"cannot open log file '{path}'")
            return None
        f.write(header + "\n")
        return f

    def close(self):
        for rec in self.probes + self.fluxes:
            if rec.get("log"):
                rec["log"].close()
                rec["log"] = None

    def configure(self):
        g, sc = self.g, self.sc
        t = g.time()
        if self.ports:
            avg = self.ff["averaging"] if self.ff else 4.0
            self.port_wavelength = max(self.ports[0].wavelength, 2.0)
            radar = getattr(sc, "radar", None)
            if radar is not None:
                # the radar records every element (and its reference channels) on the port monitor;
                # the elements' readings are its first channels (Instruments.cpp:81-95)
                from .radar import RadarMonitor
                rs = dict(radar)
                rs["log_path"] = self.resolve(rs.get("log", ""))
                self.radar = RadarMonitor(g, rs, self.ports, sc.sources, self.ports[0].wavelength, sc.cell_size,
                                          getattr(sc, "targets", []), self.warnings)
                if self.radar.phase == "off":
                    self.radar = None
            crpa = getattr(sc, "crpa", None)
            if crpa is not None and self.radar is None:
                # the adaptive array switches the sources between its passes and records every port
                # (Instruments.cpp:97-110); its first update, before the first step, starts a pass
                from .crpa import CrpaMonitor
                cs = dict(crpa)
                cs["log_path"] = self.resolve(cs.get("log", ""))
                self.crpa = CrpaMonitor(g, cs, getattr(sc, "emitters", []), sc.sources, self.ports,
                                        self.ports[0].wavelength, sc.cell_size, self.warnings)
                if self.crpa.phase == "off":
                    self.crpa = None
            if self.radar is None and self.crpa is None:
                g.ports_configure([p.to_c() for p in self.ports], self.port_wavelength, avg,
                                  sweep=self.sweep_setup is not None)
            self.port_start = t
        if self.ff:
            box = g.ntff_configure(self.ff["box_min"], self.ff["box_max"], self.ff["wavelength"], self.ff["averaging"])
            self.ff_box = box
            self.ff_start = t
            self.dirs, self.cuts = far_field_directions(self.ff.get("axis", (0.0, 0.0, 1.0)))
        if self.coaxes:
            self.configure_coax()
            self.coax_start = t
        self.planes = []
        for k, f in enumerate(sc.fluxes):
            for sign, axis, index, rmin, rmax in f.planes():
                self.planes.append((k, sign, abi.FluxPlane(axis, index, rmin, rmax)))

    def empty(self):
        return not (self.probes or self.fluxes or self.ff or self.ports or self.coaxes)

    # ------------------------------------------------------------------ coax lines (Coax.cpp)
    def configure_coax(self):
        """CoaxMonitor::configure (Coax.cpp:80-168): per station k = 1 .. length-1 of each cable, V
        (E line integral inner -> shield, averaged over the 4 sides), I (B loop round the inner
        conductor) and Icm (B loop round the whole shield, or the balun sleeve)."""
        quantities, terms, weights = [], [], []
        self.coax_layout = []

        def node_lo(c, size):
            return _round_half_away(float(np.float32(c) - np.float32(0.5) * np.float32(size)))

        def node_hi(c, size):
            return _round_half_away(float(np.float32(c) + np.float32(0.5) * np.float32(size)))
        for c in self.coaxes:
            a, u, v = c.axis, (c.axis + 1) % 3, (c.axis + 2) % 3

            def texel(ia, iu, iv):
                t = [0, 0, 0]
                t[a], t[u], t[v] = ia, iu, iv
                return t

            def add(t, comp, w):
                terms.append([t[0], t[1], t[2], comp])
                weights.append(w)

            def loop(ia, u0, u1, v0, v1, w):
                for iv in range(v0, v1 + 1):
                    add(texel(ia, u1, iv), 3 + v, w)
                    add(texel(ia, u0 - 1, iv), 3 + v, -w)
                for iu in range(u0, u1 + 1):
                    add(texel(ia, iu, v1), 3 + u, -w)
                    add(texel(ia, iu, v0 - 1), 3 + u, w)
            cu, cv = c.center[u], c.center[v]
            iu0, iu1, iv0, iv1 = node_lo(cu, c.inner), node_hi(cu, c.inner), node_lo(cv, c.inner), node_hi(cv, c.inner)
            su0, su1, sv0, sv1 = node_lo(cu, c.outer), node_hi(cu, c.outer), node_lo(cv, c.outer), node_hi(cv, c.outer)
            shield = c.outer + 2 * c.wall
            first = len(quantities)
            for k in range(1, c.length):
                ia = c.start + c.sign * k
                f0 = len(terms)
                w = float(np.float32(1.0) / (np.float32(4.0) * np.float32(c.inner + 1)))
                for r in range(iv0, iv1 + 1):
                    for i in range(iu1, su1):
                        add(texel(ia, i, r), u, w)
                    for i in range(su0, iu0):
                        add(texel(ia, i, r), u, -w)
                for r in range(iu0, iu1 + 1):
                    for i in range(iv1, sv1):
                        add(texel(ia, r, i), v, w)
                    for i in range(sv0, iv0):
                        add(texel(ia, r, i), v, -w)
                quantities.append([f0, len(terms) - f0, 0, 0])
                ib = c.start + k if c.sign > 0 else c.start - k - 1
                sgn = float(c.sign)
                f2 = len(terms)
                loop(ib, iu0, iu1, iv0, iv1, sgn)
                quantities.append([f2, len(terms) - f2, 1, 0])
                out = c.sleeve_outer if (c.sleeve_outer > 0 and c.sleeve_start <= k < c.sleeve_end) else shield
                f2 = len(terms)
                loop(ib, node_lo(cu, out), node_hi(cu, out), node_lo(cv, out), node_hi(cv, out), sgn)
                quantities.append([f2, len(terms) - f2, 1, 0])
            self.coax_layout.append((first, max(c.length - 1, 0)))
        self.g.lines_configure(quantities, terms, weights, max(self.coaxes[0].wavelength, 2.0), 4.0)
        self.coax_peak = [0.0] * len(self.coaxes)

    def poll_coax(self):
        """CoaxMonitor::analyse (Coax.cpp:214-288): two-wave least-squares fit of V(t) and I(t)
        with the lattice's TEM propagation constant."""
        if not self.coaxes:
            return
        ph, now = self.g.lines_read()
        dt = self.g.dt()
        for li, c in enumerate(self.coaxes):
            first, n = self.coax_layout[li]
            r = {"valid": False}
            tV = [k + 1.0 for k in range(n)]
            tI = [k + 1.5 for k in range(n)]
            q = [first + 3 * k for k in range(n)]
            V = [complex(float(ph[i, 2]), float(ph[i, 3])) for i in q]
            I = [complex(float(ph[i + 1, 2]), float(ph[i + 1, 3])) for i in q]
            Icm = [complex(float(ph[i + 2, 2]), float(ph[i + 2, 3])) for i in q]
            vmax = max((abs(float(now[i])) for i in q), default=0.0)
            self.coax_peak[li] = max(vmax, self.coax_peak[li] * 0.995)
            w = 2.0 * math.pi / max(c.wavelength, 2.0)
            s_arg = math.sqrt(float(c.epsilon_r)) * math.sin(0.5 * w * dt) / dt
            beta = 2.0 * math.asin(min(max(s_arg, -1.0), 1.0))
            r["beta"] = beta
            self.coax_readings[li] = r
            if c.pulsed or n < 8:
                continue
            edge = float(c.outer + 2)

            def fit(t, x):
                m11 = m12 = m22 = r1 = r2 = 0j
                for k in range(len(t)):
                    if t[k] < edge or t[k] > c.length - edge:
                        continue
                    e = complex(math.cos(-beta * t[k]), math.sin(-beta * t[k]))
                    f = e.conjugate()
                    m11 += abs(e) ** 2
                    m12 += e.conjugate() * f
                    m22 += abs(f) ** 2
                    r1 += e.conjugate() * x[k]
                    r2 += f.conjugate() * x[k]
                det = m11 * m22 - m12 * m12.conjugate()
                if abs(det) < 1e-30:
                    return None
                return (r1 * m22 - m12 * r2) / det, (m11 * r2 - m12.conjugate() * r1) / det
            fv, fi = fit(tV, V), fit(tI, I)
            if fv is None or fi is None or abs(fv[0]) < 1e-20:
                continue
            A, B = fv
            Ai = fi[0]
            res = tot = 0.0
            for k in range(n):
                if tV[k] < edge or tV[k] > c.length - edge:
                    continue
                model = (A * complex(math.cos(-beta * tV[k]), math.sin(-beta * tV[k])) +
                         B * complex(math.cos(beta * tV[k]), math.sin(beta * tV[k])))
                res += abs(V[k] - model) ** 2
                tot += abs(model) ** 2
            gam = B / A * complex(math.cos(2 * beta * c.length), math.sin(2 * beta * c.length))
            gg = min(abs(gam), 0.999999)
            z0n, rsn = c.z0_ohm / K_ETA0, c.source_ohm / K_ETA0
            p_fwd, p_avail = abs(A) ** 2 / (2.0 * z0n), c.drive * c.drive / (8.0 * rsn)
            i_fwd = abs(A) / z0n
            cm = max((abs(x) for x in Icm), default=0.0)
            r.update(valid=True, A=A, B=B, residual=math.sqrt(res / tot) if tot > 0 else 1.0,
                     z0m=abs(A / Ai) * K_ETA0 if abs(Ai) > 1e-30 else 0.0, gamma=gam,
                     vswr=(1.0 + gg) / (1.0 - gg), rl=-20.0 * math.log10(gg) if gg > 1e-12 else 200.0,
                     zend=c.z0_ohm * (1.0 + gam) / (1.0 - gam), fwd=p_fwd / p_avail if p_avail > 0 else 0.0,
                     cm_db=20.0 * math.log10(cm / i_fwd) if cm > 0 and i_fwd > 0 else -300.0)

    def print_coax(self):
        """Instruments::printCoax (Instruments.cpp:393-410)."""
        if not self.coaxes:
            return
        periods = max(self.g.time() - self.coax_start, 0.0) / max(self.coaxes[0].wavelength, 2.0)
        for c, r in zip(self.coaxes, self.coax_readings):
            self.out(f"    {c.name}: Z0 {c.z0_ohm:.1f} ohm (eps_r {c.epsilon_r:.2f}, velocity factor "
                     f"{1.0 / math.sqrt(c.epsilon_r):.2f}), {c.termination} end, {periods:.0f} periods")
            if not r or not r["valid"]:
                continue
            g = r["gamma"]
            self.out(f"      waves: Z0 measured {r['z0m']:.1f} ohm, end Gamma {abs(g):.3f} @ "
                     f"{math.degrees(math.atan2(g.imag, g.real)):+.0f} deg (RL {r['rl']:.1f} dB), VSWR {r['vswr']:.2f}, "
                     f"Z_end {r['zend'].real:.1f} {r['zend'].imag:+.1f}j ohm")
            self.out(f"      forward {100.0 * r['fwd']:.0f}% of available, delivered {100.0 * (1.0 - abs(g) ** 2):.0f}% "
                     f"of forward; shield outside current {max(r['cm_db'], -200.0):.1f} dB vs line current; fit "
                     f"residual {r['residual']:.1e}")

    # ------------------------------------------------------------------ measurement
    def measure(self):
        g = self.g
        self.measure_time, self.measure_step = g.time(), g.step_count()
        finite = True
        if self.probes:
            origins = [probe_origin(p["pos"], self.size) for p in self.probes]
            blocks = g.probe_gather(origins)
            for p, o, blk in zip(self.probes, origins, blocks):
                extent = [min(3, n - oo) for n, oo in zip(self.size, o)]
                e, b = blk[:27], blk[27:]
                pos = p["pos"]
                E = [sample_block(e, o, extent, (pos[0] - 0.5, pos[1], pos[2]), 0),
                     sample_block(e, o, extent, (pos[0], pos[1] - 0.5, pos[2]), 1),
                     sample_block(e, o, extent, (pos[0], pos[1], pos[2] - 0.5), 2)]
                B = [sample_block(b, o, extent, (pos[0], pos[1] - 0.5, pos[2] - 0.5), 0),
                     sample_block(b, o, extent, (pos[0] - 0.5, pos[1], pos[2] - 0.5), 1),
                     sample_block(b, o, extent, (pos[0] - 0.5, pos[1] - 0.5, pos[2]), 2)]
                S = _cross32(E, B)
                cell = [min(max(int(math.floor(v)), 0), n - 1) for v, n in zip(pos, self.size)]
                m = self.sc.materials.get(cell)
                p["sample"] = {"E": E, "B": B, "S": [float(v) for v in S], "sigma": m.sigma, "eps": m.epsilon_r}
                finite = finite and all(math.isfinite(v) for v in E + B)
                if p["log"]:
                    em = _len32(E)
                    bm = _len32(B)
                    p["log"].write(",".join([str(self.measure_step), _g(self.measure_time)] +
                                            [_g(v) for v in E + B + [em, bm] + list(p["sample"]["S"])]) + "\n")
        if self.planes:
            sums = g.flux_planes([pl for _, _, pl in self.planes])
            totals = [0.0] * len(self.fluxes)
            for (k, sign, _), v in zip(self.planes, sums):
                totals[k] += sign * float(v)
            for f, P in zip(self.fluxes, totals):
                finite = finite and math.isfinite(P)
                if f["last"] < 0 or self.measure_time < f["last"]:
                    f["avg"], f["peak"] = P, 0.0
                else:
                    a = 1.0 - math.exp(-(self.measure_time - f["last"]) / self.averaging_time)
                    f["avg"] += a * (P - f["avg"])
                f["inst"] = P
                f["peak"] = max(f["peak"], abs(P))
                f["last"] = self.measure_time
                if f["log"]:
                    f["log"].write(f"{self.measure_step},{_g(self.measure_time)},{_g(P)},{_g(f['avg'])}\n")
        if not finite and not self.unstable:
            self.unstable = True
            print(f"ERROR: non-finite field values detected at step {self.measure_step}", file=sys.stderr)

    def evaluate_ports(self):
        if not self.ports:
            return
        ph = self.g.ports_phasors()
        for i, p in enumerate(self.ports):
            s2 = ph[i, 4:8].astype(np.float64)
            V = -complex(s2[0], s2[1])
            I = complex(s2[2], s2[3])
            r = {"V": V, "I": I, "valid": abs(I) > 1e-12 and math.isfinite(abs(V)), "accepted": 0.0, "available": 0.0}
            if r["valid"]:
                z = V / I * K_ETA0
                z0 = max(float(p.impedance_ohm), 1e-6)
                gam = (z - z0) / (z + z0)
                gg = abs(gam)
                r.update(z=z, gamma=gam, vswr=(1.0 + min(gg, 0.999999)) / (1.0 - min(gg, 0.999999)),
                         rl=-20.0 * math.log10(gg) if gg > 1e-12 else 200.0,
                         accepted=0.5 * (V * I.conjugate()).real)
            if p.voltage_feed:
                rs = max(float(p.impedance_ohm), 1e-6) / K_ETA0
                r["available"] = float(p.drive) * float(p.drive) / (8.0 * rs)
            self.readings[i] = r

    def evaluate_far_field(self):
        if self.ff:
            out = self.g.ntff_evaluate(self.dirs).astype(np.float64)
            P = out[0, 1]
            pat = {"P": P, "valid": math.isfinite(P) and P > 1e-12}
            if pat["valid"]:
                k = 2.0 * math.pi / self.ff["wavelength"]
                scale = k * k / (8.0 * math.pi * P)
                d = scale * out[:, 0]
                best = int(np.argmax(d))
                pat["max_dir"] = self.dirs[best]
                pat["max_dbi"] = to_dbi(float(d[best]))
                cuts = []
                for c, cut in enumerate(self.cuts):
                    cc = dict(cut)
                    dbi = [to_dbi(float(v)) for v in d[c * K_CUT_SAMPLES:(c + 1) * K_CUT_SAMPLES]]
                    analyse_cut(cc, dbi)
                    cuts.append(cc)
                pat["cuts"] = cuts
                if self.ff.get("log"):
                    self.write_pattern_csv(self.resolve(self.ff["log"]), pat)
            self.pattern = pat
        self.evaluate_ports()

    def evaluate_sweep(self):
        """Ports.cpp:187-278 on the device's FP64 DFT sums."""
        s = self.sweep_setup
        if not s or not self.ports:
            return
        series_steps = self.g.ports_series().shape[0]
        if series_steps < 16:
            return
        pts = max(int(s["points"]), 2)
        sums, residual = self.g.ports_sweep_sums(s["wavelength_min"], s["wavelength_max"], pts)
        nu_lo = 1.0 / max(s["wavelength_max"], s["wavelength_min"])
        nu_hi = 1.0 / min(s["wavelength_max"], s["wavelength_min"])
        res = {"samples": series_steps, "residual": residual, "ports": [], "full": False}
        for pi, p in enumerate(self.ports):
            z0 = max(float(p.impedance_ohm), 1e-6)
            points = []
            for f in range(pts):
                nu = nu_lo + (nu_hi - nu_lo) * f / (pts - 1)
                sv = complex(sums[pi, f, 0], sums[pi, f, 1])
                si = complex(sums[pi, f, 2], sums[pi, f, 3])
                pt = {"wl": 1.0 / nu, "z": 0j, "s11": 0.0, "vswr": 1.0}
                if abs(si) > 1e-30:
                    z = -sv / si * K_ETA0
                    gg = abs((z - z0) / (z + z0))
                    pt.update(z=z, s11=20.0 * math.log10(gg) if gg > 1e-12 else -200.0,
                              vswr=(1.0 + min(gg, 0.999999)) / (1.0 - min(gg, 0.999999)))
                points.append(pt)
            best = min(range(len(points)), key=lambda i: (points[i]["s11"], i))
            nu_best = 1.0 / points[best]["wl"]
            if 0 < best < len(points) - 1:
                a, b, c = points[best - 1]["s11"], points[best]["s11"], points[best + 1]["s11"]
                den = a - 2.0 * b + c
                dnu = (nu_hi - nu_lo) / (pts - 1)
                if abs(den) > 1e-12:
                    nu_best += min(max(0.5 * (a - c) / den, -1.0), 1.0) * dnu
            ps = {"points": points, "best": best, "best_wl": 1.0 / nu_best, "band": None}
            if points[best]["s11"] < -10.0:
                def edge(direction):
                    i = best
                    while 0 <= i + direction < len(points) and points[i + direction]["s11"] < -10.0:
                        i += direction
                    j = i + direction
                    nu_i = 1.0 / points[i]["wl"]
                    if j < 0 or j >= len(points):
                        return nu_i
                    nu_j = 1.0 / points[j]["wl"]
                    s_i, s_j = points[i]["s11"], points[j]["s11"]
                    return nu_i + (nu_j - nu_i) * (-10.0 - s_i) / (s_j - s_i)
                ps["band"] = (1.0 / edge(-1), 1.0 / edge(+1))
            res["ports"].append(ps)
        self.sweep_result = res
        if s.get("log"):
            self.write_sweep_csv(self.resolve(s["log"]), res)

    def write_sweep_csv(self, path, res):
        """PortMonitor::writeSweepCsv (Ports.cpp:280-297)."""
        with open(path, "w") as f:
            f.write("frequency_Hz,wavelength_cells")
            for p in self.ports:
                f.write(f",{p.name}_R_ohm,{p.name}_X_ohm,{p.name}_S11_dB,{p.name}_VSWR")
            f.write("\n")
            for i in range(len(res["ports"][0]["points"])):
                wl = res["ports"][0]["points"][i]["wl"]
                row = [_g(K_C0 / (wl * float(np.float32(self.sc.cell_size)))), _g(wl)]
                for ps in res["ports"]:
                    pt = ps["points"][i]
                    row += [_g(pt["z"].real), _g(pt["z"].imag), _g(pt["s11"]), _g(pt["vswr"])]
                f.write(",".join(row) + "\n")

    def write_pattern_csv(self, path, pat):
        """FarFieldMonitor::writeCsv (FarField.cpp:336-349): angle and the three cuts in dBi."""
        with open(path, "w") as f:
            f.write("angle_deg" + "".join(f",{c['name']}_dBi" for c in pat["cuts"]) + "\n")
            for i, ang in enumerate(pat["cuts"][0]["angles"]):
                f.write(_g(ang) + "".join("," + _g(c["dbi"][i]) for c in pat["cuts"]) + "\n")

    # ------------------------------------------------------------------ report
    def print_ports(self, max_lines):
        if not self.ports:
            return
        out = self.out
        rd = self.readings
        periods = max(self.g.time() - self.port_start, 0.0) / self.port_wavelength
        accepted = sum(r["accepted"] for r in rd if r)
        available = sum(r["available"] for r in rd if r)
        cw_lines = 0 if (self.sweep_setup or self.radar or self.crpa) else max_lines
        if periods < 12.0 and cw_lines > 0:
            out(f"    ports: averaging ({periods:.0f} of ~12 periods), impedances still settling")
        for i, p in enumerate(self.ports[:cw_lines]):
            r = rd[i]
            if r is None or not r["valid"]:
                out(f"    port  {p.name:<14s} (no current yet)")
                continue
            if p.voltage_feed:
                pa = 100.0 * r["accepted"] / r["available"] if r["available"] > 0 else 0.0
                out(f"    port  {p.name:<14s} Z = {r['z'].real:7.1f} {r['z'].imag:+7.1f}j ohm | Gamma "
                    f"{abs(r['gamma']):.3f} @ {math.degrees(math.atan2(r['gamma'].imag, r['gamma'].real)):+5.0f} deg "
                    f"(S11 {-r['rl']:6.1f} dB), VSWR {r['vswr']:5.2f} vs {p.impedance_ohm:.0f} ohm | P_acc "
                    f"{r['accepted']:.3e} of {r['available']:.3e} avail ({pa:.0f}%)")
            else:
                out(f"    port  {p.name:<14s} Z = {r['z'].real:7.1f} {r['z'].imag:+7.1f}j ohm | current feed "
                    f"{p.drive:.3g} | P_acc {r['accepted']:.3e}")
        if cw_lines > 0 and len(self.ports) > max_lines:
            out(f"    ... {len(self.ports) - max_lines} more ports (press P for all) | total P_acc {accepted:.3e} of "
                f"{available:.3e} available")
        if self.sweep_setup:
            sw = self.sweep_result
            cell = self.sc.cell_size

            def ghz(wl):
                return K_C0 / (wl * cell) * 1e-9
            if sw is None:
                out("    sweep: recording the pulse response...")
            else:
                tail = " (settled)" if sw["residual"] <= 1e-3 else (
                    " (buffer full: results approximate)" if sw["full"] else " (still ringing: results settling)")
                out(f"    sweep: {sw['samples']} steps recorded, ring-down {sw['residual']:.1e} of peak{tail}")
                for i, ps in enumerate(sw["ports"][:max_lines]):
                    b = ps["points"][ps["best"]]
                    line = (f"    sweep {self.ports[i].name:<12s} best match {ghz(ps['best_wl']):.4f} GHz (lambda "
                            f"{ps['best_wl']:.2f} cells): S11 {b['s11']:.1f} dB, VSWR {b['vswr']:.2f}, Z = "
                            f"{b['z'].real:.1f} {b['z'].imag:+.1f}j ohm")
                    if ps["band"]:
                        f0, fl, fh = ghz(ps["best_wl"]), ghz(ps["band"][0]), ghz(ps["band"][1])
                        line += f" | -10 dB band {fl:.4f}-{fh:.4f} GHz ({100.0 * (fh - fl) / f0:.1f}%)"
                    else:
                        line += " | never below -10 dB in the sweep"
                    out(line)
        if self.ff and self.pattern and self.pattern["valid"] and accepted > 0.0:
            prad = self.pattern["P"]
            if len(self.ports) == 1 and rd[0] and rd[0]["valid"]:
                i2 = abs(rd[0]["I"]) ** 2
                out(f"    radiation resistance R_rad = 2 P_rad / |I|^2 = {2.0 * prad / i2 * K_ETA0:.1f} ohm, radiation "
                    f"efficiency P_rad / P_acc = {100.0 * prad / accepted:.0f}%")
            else:
                out(f"    radiation efficiency P_rad / total P_acc = {100.0 * prad / accepted:.0f}%")

    def print_report(self):
        out = self.out
        if self.empty():
            out(f"[t={self.g.time():8.1f} step {self.g.step_count():7d}] {NO_INSTRUMENTS_HINT}")
            return
        out(f"[t={self.measure_time:8.1f} step {self.measure_step:7d}]")
        for i, p in enumerate(self.probes):
            s = p["sample"]
            if s is None:
                continue
            E, B, S = s["E"], s["B"], s["S"]
            em = _len32(E)
            bm = _len32(B)
            pos = p["pos"]
            out(f"  {'>' if i == 0 else ' '} probe {p['name']:<14s} ({pos[0]:6.1f} {pos[1]:6.1f} {pos[2]:6.1f}): "
                f"|E|={em:.5f} E=({E[0]:+.4f} {E[1]:+.4f} {E[2]:+.4f}) |B|={bm:.5f} S=({S[0]:+.2e} {S[1]:+.2e} "
                f"{S[2]:+.2e}) sigma={s['sigma']:.3g} eps_r={s['eps']:.2f}")
        for f in self.fluxes:
            out(f"    flux  {f['setup'].name:<28s} P={f['inst']:+.4e}  <P>={f['avg']:+.4e}  peak|P|={f['peak']:.4e}")
        self.print_ports(4)
        if self.radar:
            self.radar.report(out)
        if self.crpa:
            self.crpa.report(out)
        self.print_coax()
        if self.ff:
            pat = self.pattern
            settle = max(self.g.time() - self.ff_start, 0.0) / max(self.ff["wavelength"], 1.0)
            if not pat or not pat["valid"]:
                out(f"    far field: accumulating ({settle:.1f} periods)...")
            else:
                d = pat["max_dir"]
                theta = math.degrees(math.acos(min(max(float(d[2]), -1.0), 1.0)))
                phi = math.degrees(math.atan2(float(d[1]), float(d[0])))
                settling = ", still settling" if settle < 3.0 * self.ff["averaging"] else ""
                out(f"    far field [lambda={self.ff['wavelength']:.1f} cells, {settle:.0f} periods averaged{settling}]: "
                    f"P_rad={pat['P']:.4e}  D_max={pat['max_dbi']:.2f} dBi ({10 ** (pat['max_dbi'] / 10):.2f}) @ "
                    f"theta={theta:.0f} phi={phi:.0f}")
                for c in pat["cuts"]:
                    bw = "omni" if c["beamwidth"] >= 359.0 else f"{c['beamwidth']:.1f} deg"
                    out(f"      {c['name']}-cut: peak {c['peak_dbi']:6.2f} dBi @ {c['peak_angle']:5.1f} deg, HPBW "
                        f"{bw}, front/back {c['front_back']:.1f} dB")
