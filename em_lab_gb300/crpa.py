"""Controlled-reception-pattern antenna (CRPA): an adaptive GPS array (src/Crpa.hpp, src/Crpa.cpp).

Dual-probe patches (a 90-degree hybrid forms each element's right-hand-circular channel) receive
a GPS satellite below the noise and jammers. In the ideal mode each emitter transmits alone in a
pass of its own and a least-squares fit over the last four periods gives its steady-state port
phasors (its steering vector); in the blind mode all emitters transmit at once (the jammers a few
percent off the carrier), the receiver downconverts every port to baseband (Blackman-Harris
low-pass), takes snapshots and estimates the covariance from them with its own thermal noise, and
a joint fit of every emitter's tone scores the result. MVDR weights w = R^-1 a / (a^H R^-1 a) put
unit gain toward the satellite and nulls on the jammers; the array then transmits with the
weights so the fields show the adapted pattern. The passes switch the grid's sources and reset
its fields; the port monitor records every port.

The receiver noise is the reference's: std::mt19937 seeded with noise_seed and the polar-method
normal distribution of the GNU C++ library, restated here (MT19937, generate_canonical with two
32-bit draws, Marsaglia polar pairs with the second value cached).
"""
from __future__ import annotations

import cmath
import math

import numpy as np

f32 = np.float32
MAP_SIZE = 61


# ---- the reference's random numbers ---------------------------------------------------------
class MT19937:
    """The Mersenne Twister of Matsumoto and Nishimura (1998), 32-bit, init_genrand seeding."""

    def __init__(self, seed: int):
        self.mt = [0] * 624
        self.mt[0] = seed & 0xFFFFFFFF
        for i in range(1, 624):
            self.mt[i] = (1812433253 * (self.mt[i - 1] ^ (self.mt[i - 1] >> 30)) + i) & 0xFFFFFFFF
        self.i = 624

    def next32(self) -> int:
        if self.i >= 624:
            mt = self.mt
            for k in range(624):
                y = (mt[k] & 0x80000000) | (mt[(k + 1) % 624] & 0x7FFFFFFF)
                mt[k] = mt[(k + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            self.i = 0
        y = self.mt[self.i]
        self.i += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y & 0xFFFFFFFF

    def canonical(self) -> float:
        """A double in [0, 1) from two 32-bit draws (low word first), as generate_canonical."""
        lo = self.next32()
        hi = self.next32()
        r = (lo + hi * 4294967296.0) / 18446744073709551616.0
        return r if r < 1.0 else math.nextafter(1.0, 0.0)


class Normal:
    """Marsaglia's polar method: pairs of normals, the second one kept for the next call."""

    def __init__(self, rng: MT19937, mean=0.0, stddev=1.0):
        self.rng, self.mean, self.stddev = rng, mean, stddev
        self.saved = None

    def __call__(self) -> float:
        if self.saved is not None:
            v, self.saved = self.saved, None
        else:
            while True:
                x = 2.0 * self.rng.canonical() - 1.0
                y = 2.0 * self.rng.canonical() - 1.0
                r2 = x * x + y * y
                if not (r2 > 1.0 or r2 == 0.0):
                    break
            mult = math.sqrt(-2.0 * math.log(r2) / r2)
            self.saved = x * mult
            v = y * mult
        return v * self.stddev + self.mean


def _db(p):
    return 10.0 * math.log10(p) if p > 1e-300 else -300.0


def _mean_power(v):
    v = np.asarray(v)
    return float(np.sum(np.abs(v) ** 2) / v.size) if v.size else 0.0


def _dot3_f32(a, b):
    """glm::dot of two vec3: (a.x b.x + a.y b.y) + a.z b.z, every operation rounded to FP32."""
    a, b = np.asarray(a, f32), np.asarray(b, f32)
    return f32(f32(f32(a[0] * b[0]) + f32(a[1] * b[1])) + f32(a[2] * b[2]))


def _normalize_f32(v):
    """glm::normalize: v * inversesqrt(dot(v, v)) with inversesqrt = 1 / sqrt in FP32."""
    v = np.asarray(v, f32)
    inv = f32(f32(1.0) / f32(np.sqrt(_dot3_f32(v, v))))
    return (v * inv).astype(f32)


def _dot_h(a, b):
    return complex(np.sum(np.conj(np.asarray(a)) * np.asarray(b)))


def solve(A, b, n):
    """Gaussian elimination with partial pivoting (Crpa.cpp:30-54), singular pivots skipped."""
    A = np.array(A, complex).reshape(n, n)
    b = np.array(b, complex)
    for col in range(n):
        piv = col
        for r in range(col + 1, n):
            if abs(A[r, col]) > abs(A[piv, col]):
                piv = r
        if piv != col:
            A[[col, piv]] = A[[piv, col]]
            b[[col, piv]] = b[[piv, col]]
        d = A[col, col]
        if abs(d) < 1e-300:
            continue
        for r in range(col + 1, n):
            f = A[r, col] / d
            A[r, col:] -= f * A[col, col:]
            b[r] -= f * b[col]
    x = np.zeros(n, complex)
    for i in range(n - 1, -1, -1):
        s = b[i] - np.sum(A[i, i + 1:] * x[i + 1:])
        x[i] = s / A[i, i] if abs(A[i, i]) > 1e-300 else 0.0
    return x


class CrpaMonitor:
    """CrpaMonitor (Crpa.hpp:96-157) driving the grid's sources and port monitor."""

    def __init__(self, grid, setup: dict, emitters, sources, ports, wavelength, cell_size, warnings):
        self.g = grid
        self.setup = dict(setup)
        self.emitters = list(emitters)
        self.sources = list(sources)
        self.ports = list(ports)
        self.wl = max(float(wavelength), 2.0)
        self.cell_size = float(cell_size)
        self.dt = float(grid.dt())
        self.phase = "off"
        self.result = None
        if not self.emitters:
            warnings.append("crpa: the scene has no emitter{} transmitters")
            return
        self.element_ports = []
        center = np.zeros(3, f32)
        names = [p.name for p in self.ports]
        for el in self.setup["elements"]:
            ix = max([k for k, n in enumerate(names) if n == el["x"]], default=-1)
            iy = max([k for k, n in enumerate(names) if n == el["y"]], default=-1)
            self.element_ports.append((ix, iy))
            center = (center + np.asarray(el["center"], f32)).astype(f32)
        self.center = (center / f32(max(len(self.setup["elements"]), 1))).astype(f32)
        self.satellite = 0
        for e, em in enumerate(self.emitters):
            if em["name"] == self.setup["satellite"]:
                self.satellite = e
        self.pass_steps = int(math.ceil(f32(self.setup["pass_periods"]) * f32(self.wl) / self.dt))
        self.blind_steps = int(math.ceil((self.setup["pass_periods"] + self.setup["snapshot_periods"] + 4.5) *
                                         self.wl / self.dt))
        E = len(self.emitters)
        self.emitter_wl = [self.wl] * E
        for s in self.sources:
            if 0 <= s.emitter < E:
                self.emitter_wl[s.emitter] = float(s.wavelength) / (1.0 + self.emitter_offset(s.emitter))
        near = 0.0
        for e, em in enumerate(self.emitters):
            if e != self.satellite:
                r = float(np.sqrt(np.sum((np.asarray(em["position"], f32) - self.center) ** 2, dtype=f32)))
                near = min(near, r) if near > 0.0 else r
        r_sat = float(np.sqrt(np.sum((np.asarray(self.emitters[self.satellite]["position"], f32) - self.center) ** 2,
                                     dtype=f32)))
        self.sat_amplitude = (0.5 * 10.0 ** ((self.setup["snr_db"] - self.setup["jnr_db"]) / 20.0) * r_sat / near
                              if near > 0.0 else 1.0)
        self.response = [None] * E
        self.settle = [1.0] * E
        self.baseband = []
        self.pass_ = 0
        self.phase = "listening" if self.setup["blind"] else "measuring"
        self.needs_apply = True

    # ---- passes (Crpa.cpp:163-245) ----------------------------------------------------------
    def emitter_offset(self, e):
        """Blind run: jammer k transmits (+1, -1, +2, -2, ...) / snapshot_periods off the carrier."""
        if not self.setup["blind"] or e == self.satellite:
            return 0.0
        rank = e if e < self.satellite else e - 1
        n = (rank // 2 + 1) * (1 if rank % 2 == 0 else -1)
        return float(n) / max(self.setup["snapshot_periods"], 1.0)

    def pass_progress(self):
        steps = self.pass_steps if self.phase == "measuring" else (self.blind_steps if self.phase == "listening" else 0)
        if steps == 0:
            return 1.0
        return min(1.0, self.g.ports_recorded() / steps)

    def start_pass(self):
        import copy
        active = []
        if self.phase == "measuring":
            active = [s for s in self.sources if s.emitter == self.pass_]
        elif self.phase == "listening":
            for s in self.sources:
                if s.emitter < 0:
                    continue
                t = copy.copy(s)
                t.wavelength = float(f32(float(s.wavelength) / (1.0 + self.emitter_offset(s.emitter))))
                if s.emitter == self.satellite:
                    t.amplitude = float(f32(float(s.amplitude) * self.sat_amplitude))
                active.append(t)
        else:
            # transmit with the receive weights: y = sum conj(w_i) (X_i - j Y_i) / sqrt 2, by reciprocity
            coef = [0j] * len(self.ports)
            r2 = 1.0 / math.sqrt(2.0)
            w = self.result["weights"] if self.result else []
            for i, (px, py) in enumerate(self.element_ports[: len(w)]):
                cw = complex(w[i]).conjugate()
                if px >= 0:
                    coef[px] = cw * r2
                if py >= 0:
                    coef[py] = cw * -1j * r2
            cmax = max((abs(c) for c in coef), default=0.0)
            for s in self.sources:
                if s.port < 0 or s.port >= len(coef) or cmax <= 0.0:
                    continue
                c = coef[s.port] / cmax
                if abs(c) < 1e-9:
                    continue
                t = copy.copy(s)
                t.amplitude = float(f32(float(s.amplitude) * abs(c)))
                t.phase = float(f32(float(s.phase) + math.atan2(c.imag, c.real)))
                active.append(t)
        self.g.set_sources(active)
        self.g.reset_fields()
        steps = self.pass_steps if self.phase == "measuring" else (self.blind_steps if self.phase == "listening" else 0)
        self.g.ports_configure([p.to_c() for p in self.ports], self.wl, 4.0, False, steps)

    def update(self):
        """Once per frame before the steps (Crpa.cpp:226-245)."""
        if self.phase == "off":
            return
        if self.needs_apply:
            self.needs_apply = False
            self.start_pass()
            return
        rec = self.g.ports_recorded()
        if self.phase == "measuring" and rec >= self.pass_steps:
            self.finish_pass()
            self.pass_ += 1
            if self.pass_ >= len(self.emitters):
                self.compute_weights()
                self.phase = "adapted"
                self.write_log()
            self.start_pass()
        elif self.phase == "listening" and rec >= self.blind_steps:
            self.finish_blind()
            self.compute_weights()
            self.phase = "adapted"
            self.write_log()
            self.start_pass()

    def series(self):
        return self.g.ports_series()[:, :, 0].astype(np.float64)  # V per [step][port]

    def finish_pass(self):
        """Steady-state phasor of every port: A cos + B sin over the last four periods (Crpa.cpp:340-375)."""
        v = self.series()
        N, P = v.shape
        w = 2.0 * math.pi / self.wl
        W = min(N // 2, int(round(4.0 * self.wl / self.dt)))

        def fit(p, end):
            t = (np.arange(end - W, end) + 1) * self.dt
            c, s, x = np.cos(w * t), np.sin(w * t), v[end - W:end, p]
            scc, sss, scs, svc, svs = (c * c).sum(), (s * s).sum(), (c * s).sum(), (x * c).sum(), (x * s).sum()
            det = scc * sss - scs * scs
            if abs(det) < 1e-30:
                return 0j
            A = (svc * sss - svs * scs) / det
            B = (svs * scc - svc * scs) / det
            return complex(A, -B)
        ph = np.zeros(P, complex)
        change = level = 0.0
        if W > 8:
            for p in range(P):
                ph[p] = fit(p, N)
                earlier = fit(p, N - W)
                change = max(change, abs(ph[p] - earlier))
                level = max(level, abs(ph[p]))
        if 0 <= self.pass_ < len(self.response):
            self.response[self.pass_] = ph
            self.settle[self.pass_] = change / level if level > 0.0 else 1.0

    def finish_blind(self):
        """Joint least-squares fit of every emitter's tone (scoring) and the receiver's I/Q snapshots
        (Crpa.cpp:247-338)."""
        v = self.series()
        N, P = v.shape
        E = len(self.emitters)
        lam0 = self.wl
        w0 = 2.0 * math.pi / lam0
        ta = (self.setup["pass_periods"] + 2.0) * lam0
        tb = ta + self.setup["snapshot_periods"] * lam0
        t = (np.arange(N) + 1) * self.dt
        sel = (t >= ta) & (t < tb)
        ts = t[sel]
        basis = np.zeros((ts.size, 2 * E))
        for e in range(E):
            w = 2.0 * math.pi / self.emitter_wl[e]
            basis[:, 2 * e], basis[:, 2 * e + 1] = np.cos(w * ts), np.sin(w * ts)
        G = basis.T @ basis
        rhs = v[sel].T @ basis  # (P, 2E)
        coef = np.stack([solve(G, rhs[p], 2 * E).real for p in range(P)])
        self.response = [np.array([complex(coef[p, 2 * e], -coef[p, 2 * e + 1]) for p in range(P)]) for e in range(E)]
        fitv = basis @ coef.T
        resid = float(np.sum((v[sel] - fitv) ** 2))
        count = int(sel.sum())
        resid_power = 2.0 * resid / (count * P) if count and P else 0.0
        self.settle = [math.sqrt(resid_power / _mean_power(self.response[e])) if _mean_power(self.response[e]) > 0
                       else 1.0 for e in range(E)]
        S = max(int(self.setup["snapshots_per_period"]), 1)
        K = int(round(self.setup["snapshot_periods"] * S))
        half = 2.0 * lam0
        self.baseband = []
        for k in range(K):
            tk = ta + k * lam0 / S
            n0 = int(max(0.0, math.ceil((tk - half) / self.dt - 1.0)))
            tt = (np.arange(n0, N) + 1) * self.dt
            m = tt <= tk + half
            tt = tt[m]
            u = (tt - tk) / (2.0 * half) + 0.5
            a = 2.0 * math.pi * u
            win = 0.35875 - 0.48829 * np.cos(a) + 0.14128 * np.cos(2.0 * a) - 0.01168 * np.cos(3.0 * a)
            lo = np.exp(-1j * w0 * tt)
            x = (win[:, None] * v[n0:n0 + tt.size] * lo[:, None]).sum(axis=0)
            wsum = win.sum()
            if wsum > 0.0:
                x = x * (2.0 / wsum)
            self.baseband.append(self.channels(x))

    def channels(self, ports, lhcp=False):
        """Each element's RHCP (or LHCP) channel: the 90-degree hybrid (X -/+ jY) / sqrt 2."""
        j = 1j if lhcp else -1j
        out = []
        for px, py in self.element_ports:
            x = ports[px] if 0 <= px < len(ports) else 0j
            y = ports[py] if 0 <= py < len(ports) else 0j
            out.append((x + j * y) / math.sqrt(2.0))
        return np.asarray(out, complex)

    def compass_angles(self, p):
        up = np.array([0, 0, 1], f32)
        north = np.asarray(self.setup["north"], f32)
        east = np.cross(north, up).astype(f32)
        d = (np.asarray(p, f32) - self.center).astype(f32)
        ln = max(float(np.sqrt(np.sum(d * d, dtype=f32))), 1e-6)
        az = math.degrees(math.atan2(float(np.dot(d, east)), float(np.dot(d, north))))
        if az < 0.0:
            az += 360.0
        return az, math.degrees(math.asin(min(max(float(np.dot(d, up)) / ln, -1.0), 1.0)))

    def compute_weights(self):
        """Covariance, steering vector, MVDR / steering weights and their scores (Crpa.cpp:389-520)."""
        N, E = len(self.element_ports), len(self.emitters)
        if N == 0 or any(r is None for r in self.response):
            self.result = None
            return
        s_raw = self.channels(self.response[self.satellite])
        jams = [self.channels(self.response[e]) for e in range(E) if e != self.satellite]
        strongest = max((_mean_power(j) for j in jams), default=0.0)
        ps = _mean_power(s_raw)
        gj = 10.0 ** (self.setup["jnr_db"] / 10.0) / strongest if strongest > 0 else 0.0
        gs = 10.0 ** (self.setup["snr_db"] / 10.0) / ps if ps > 0 else 0.0
        blind = self.setup["blind"] and len(self.baseband) > 0
        r = {"blind": False}
        if blind:
            sigma2 = (strongest / 10.0 ** (self.setup["jnr_db"] / 10.0) if strongest > 0
                      else ps / 10.0 ** (self.setup["snr_db"] / 10.0))
            gj = gs = 1.0 / sigma2 if sigma2 > 0 else 0.0
        Rin = np.eye(N, dtype=complex)
        for j in jams:
            Rin += gj * np.outer(j, np.conj(j))
        R = Rin + gs * np.outer(s_raw, np.conj(s_raw))
        if blind:
            rng = Normal(MT19937(int(self.setup["noise_seed"])), 0.0, math.sqrt(0.5))
            R = np.zeros((N, N), complex)
            amp = math.sqrt(gs)
            for snap in self.baseband:
                xk = np.empty(N, complex)
                for i in range(N):
                    # cd(gauss(rng), gauss(rng)) (Crpa.cpp:447): C++ leaves the order of the two
                    # draws to the compiler; GCC and MSVC evaluate the imaginary part's draw first
                    im = rng()
                    xk[i] = amp * snap[i] + complex(rng(), im)
                R += np.outer(xk, np.conj(xk))
            R /= len(self.baseband)
            r.update(blind=True, snapshots=len(self.baseband),
                     snapshot_us=self.setup["snapshot_periods"] * self.wl * self.cell_size / 299792458.0 * 1e6)
        # glm::normalize and glm::dot in FP32, operation by operation (Crpa.cpp:462-466)
        u = _normalize_f32((np.asarray(self.emitters[self.satellite]["position"], f32) - self.center).astype(f32))
        k = 2.0 * math.pi / self.wl
        if self.setup["measured_steering"]:
            a = s_raw.copy()
        else:
            a = np.array([cmath.rect(1.0, k * float(_dot3_f32((np.asarray(el["center"], f32) - self.center).astype(f32), u)))
                          for el in self.setup["elements"]])
        Ria = solve(R, a, N)
        denom = _dot_h(a, Ria)
        aa = _dot_h(a, a).real
        w_mvdr = Ria / denom if abs(denom) > 1e-300 else np.zeros(N, complex)
        w_steer = a / aa
        w = w_mvdr if self.setup["mvdr"] else w_steer
        r["weights"] = w

        def quad(x, M):
            return float(np.real(np.conj(x) @ M @ x))

        def sinr(ww):
            return gs * abs(_dot_h(ww, s_raw)) ** 2 / max(quad(ww, Rin), 1e-300)
        single = 0.0
        for i in range(N):
            interf = 1.0 + sum(gj * abs(j[i]) ** 2 for j in jams)
            single += gs * abs(s_raw[i]) ** 2 / interf
        r["sinr_single_db"] = _db(single / N)
        r["sinr_steering_db"] = _db(sinr(w_steer))
        r["sinr_mvdr_db"] = _db(sinr(w))
        wn, wsn = _dot_h(w, w).real, _dot_h(w_steer, w_steer).real
        r["satellite_gain_db"] = _db(gs * abs(_dot_h(w, s_raw)) ** 2 / wn) - _db(gs * ps)
        rows = []
        for e in range(E):
            em = self.emitters[e]
            az, el = self.compass_angles(em["position"])
            v = self.channels(self.response[e])
            g = gs if e == self.satellite else gj
            rows.append({"name": em["name"], "satellite": e == self.satellite, "az": az, "el": el,
                         "distance": float(np.sqrt(np.sum((np.asarray(em["position"], f32) - self.center) ** 2,
                                                          dtype=f32))),
                         "input_db": _db(g * _mean_power(v)), "output_db": _db(g * abs(_dot_h(w, v)) ** 2 / wn),
                         "steering_out_db": _db(g * abs(_dot_h(w_steer, v)) ** 2 / wsn),
                         "cross_pol_db": _db(_mean_power(self.channels(self.response[e], True))) - _db(_mean_power(v)),
                         "settle_db": 20.0 * math.log10(max(self.settle[e], 1e-12)),
                         "offset_pct": 100.0 * self.emitter_offset(e)})
        r["emitters"] = rows
        r["valid"] = True
        self.result = r

    def write_log(self, path=None):
        path = path or self.setup.get("log_path")
        r = self.result
        if not path or not r or not r.get("valid"):
            return
        with open(path, "w") as f:
            f.write("emitter,kind,azimuth_deg,elevation_deg,distance_cells,input_db,output_db,steering_output_db,"
                    "crosspol_db\n")
            for e in r["emitters"]:
                f.write(f"{e['name']},{'satellite' if e['satellite'] else 'jammer'},{e['az']:g},{e['el']:g},"
                        f"{e['distance']:g},{e['input_db']:g},{e['output_db']:g},{e['steering_out_db']:g},"
                        f"{e['cross_pol_db']:g}\n")
            f.write("\nelement,weight_mag,weight_phase_deg\n")
            for i, w in enumerate(r["weights"]):
                f.write(f"{i + 1},{abs(w):g},{math.degrees(math.atan2(w.imag, w.real)):g}\n")
            f.write(f"\nsinr_single_db,{r['sinr_single_db']:g}\nsinr_steering_db,{r['sinr_steering_db']:g}\n"
                    f"sinr_mvdr_db,{r['sinr_mvdr_db']:g}\n")

    def report(self, out):
        """Instruments::printCrpa (Instruments.cpp:366-393)."""
        if self.phase == "off":
            return
        if self.phase == "measuring":
            p = self.pass_
            name = self.emitters[p]["name"] if p < len(self.emitters) else "?"
            out(f"    crpa: measuring {name} at the array (pass {p + 1} of {len(self.emitters)}, "
                f"{100.0 * self.pass_progress():.0f}%)")
            return
        if self.phase == "listening":
            out(f"    crpa: listening, all {len(self.emitters)} emitters on ({100.0 * self.pass_progress():.0f}%)")
            return
        r = self.result
        if not r or not r.get("valid"):
            return
        if r["blind"]:
            out(f"    crpa: blind, covariance from {r['snapshots']} snapshots ({r['snapshot_us']:.3f} us)")
        out(f"    crpa ({'MVDR' if self.setup['mvdr'] else 'steering'} weights): SINR single element "
            f"{r['sinr_single_db']:.1f} dB, steering {r['sinr_steering_db']:.1f} dB, applied {r['sinr_mvdr_db']:.1f} dB")
        for e in r["emitters"]:
            out(f"      {e['name']:<12s} az {e['az']:5.1f} el {e['el']:5.1f}  f {e['offset_pct']:+4.1f}%  in "
                f"{e['input_db']:+6.1f} dB  out {e['output_db']:+6.1f} dB  (steering only {e['steering_out_db']:+6.1f} dB)"
                f"  cross-pol {e['cross_pol_db']:+.1f} dB  settled {e['settle_db']:.0f} dB")
