"""Pulsed phased-array radar over the antenna ports (src/Radar.hpp, src/Radar.cpp).

Every feed transmits a short pulse (or only some of them) and every feed receives: the grid's port
monitor records the voltage of each element and three reference channels (Ex, Ey, Ez at a point
on boresight) at every step. A first pass without the targets (calibration) records the radar's
own response and fixes the listening window from the antennas' ring-down; a second pass with the
targets is the measurement. Processing (RadarMonitor::computeImage): the echo (measurement minus
calibration) is pulse-compressed with the two-way template REF^2 / S in the frequency domain,
brought to complex baseband and decimated; back-projection over range x azimuth x elevation runs
on the GPU (csrc/radar.cu, emlab_radar_backproject); local maxima above the floor are the
detections, compared with the targets' true nearest points.

Receiver noise is the reference's: per element, MT19937 seeded with 20251105 + element and the
polar-method normal generator (em_lab_gb300/crpa.py restates both).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import abi
from .grid import _check, load_library
from .crpa import MT19937, Normal
from .instruments import boresight_frame

f32 = np.float32
REFERENCE_CHANNELS = 3
MAX_DETECTIONS = 8


def _to_db(p):
    return float(10.0 * math.log10(p)) if p > 1e-300 else -3000.0


def _vertex_offset(a, b, c):
    den = f32(a) - f32(2.0) * f32(b) + f32(c)
    if abs(den) < 1e-12:
        return f32(0.0)
    return f32(min(max(f32(0.5) * (f32(a) - f32(c)) / den, -0.5), 0.5))


def _round_half_away(x):
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


def _next_pow2(n):
    f = 1
    while f < n:
        f <<= 1
    return f


def source_signal(s, t):
    from .grid import source_signal as sig
    return sig(s, t)


class RadarMonitor:
    """RadarMonitor (Radar.hpp:99-205) with the grid's port monitor as its recorder."""

    def __init__(self, grid, setup: dict, elements, sources, wavelength, cell_size, targets, warnings):
        self.g = grid
        self.setup = dict(setup)
        self.targets = list(targets)
        self.wl = max(float(wavelength), 2.0)
        self.cell_size = float(cell_size)
        self.dt = float(grid.dt())
        self.elements = list(elements)
        self.phase = "off"
        self.image = None
        self.cal = None
        self.meas = None
        if not self.elements:
            warnings.append("radar: the scene has no antenna feeds to transmit and receive with")
            return
        p0 = self.elements[0]
        n = np.zeros(3, f32)
        n[p0.axis] = 1.0 if p0.sign >= 0 else -1.0
        right, up = boresight_frame(n)
        self.axes = [np.asarray(right, f32), np.asarray(up, f32), n]
        off = np.asarray(self.setup["phase_center"], f32)
        self.elem_pos = []
        for p in self.elements:
            c = np.asarray(p.texel, f32)
            c[p.axis] += f32(0.5)  # centre of the gap edge
            self.elem_pos.append(c + off)
        self.elem_pos = np.asarray(self.elem_pos, f32)
        # receive taper: a separable window over element rows and columns (Radar.cpp:152-171)
        self.weights = np.ones(len(self.elem_pos))
        taper = int(self.setup["taper"])
        if taper != 0:
            a = 0.54 if taper == 1 else 0.5
            for k in range(2):
                coords = [f32(np.round(f32(np.dot(p, self.axes[k])) * f32(4.0)) / f32(4.0)) for p in self.elem_pos]
                uniq = sorted(set(float(c) for c in coords))
                if len(uniq) < 2:
                    continue
                cnt = float(len(uniq))
                for i, c in enumerate(coords):
                    idx = float(uniq.index(float(c)))
                    self.weights[i] *= a - (1.0 - a) * math.cos(2.0 * math.pi * (idx + 1.0) / (cnt + 1.0))
        # transmit phase centre and pulse timing (drive-weighted over the pulsed feeds)
        wsum = tsum = tau_sum = t_end = 0.0
        csum = np.zeros(3)
        tx = []
        for s in sources:
            if not s.enabled or s.waveform != abi.WAVE_PULSE:
                continue
            w = abs(float(s.amplitude))
            if w <= 0.0:
                continue
            period = max(float(s.wavelength), 1e-3)
            tau = max(float(s.ramp_periods), 0.1) * period
            t0 = max(float(s.delay_periods), 0.0) * period + 3.0 * tau
            csum += w * np.asarray(s.center, np.float64)
            tsum += w * t0
            tau_sum += w * tau
            wsum += w
            t_end = max(t_end, t0 + 3.0 * tau)
            tx.append(s)
        if wsum <= 0.0:
            warnings.append("radar: no pulsed transmitter; drive the antennas with waveform = \"pulse\"")
            return
        txc = self.setup.get("tx")
        self.tx = np.asarray(txc, f32) if txc is not None else (np.asarray(csum / wsum, f32) + off).astype(f32)
        self.tx_sources = tx
        self.tx_weight = wsum
        if txc is not None:
            self.tx_pos, self.tx_amp = np.asarray([txc], f32), np.asarray([1.0])
        else:
            self.tx_pos = np.asarray([np.asarray(s.center, f32) + off for s in tx], f32)
            self.tx_amp = np.asarray([abs(float(s.amplitude)) for s in tx])
        self.tx_time = tsum / wsum
        self.target_nearest = []
        for t in self.targets:
            pts = t["points"]
            if len(pts):
                d = np.sqrt(((pts - self.tx) ** 2).sum(axis=1, dtype=f32))
                self.target_nearest.append(pts[int(np.argmin(d))])
            else:
                self.target_nearest.append(np.clip(self.tx, t["min"], t["max"]).astype(f32))
        self.pulse_width = tau_sum / wsum
        # image ranges (Radar.cpp:221-232)
        gs = np.asarray(grid.size(), f32)
        L = f32(grid.config().pml_thickness)
        self.interior_min = np.full(3, L, f32)
        self.interior_max = (gs - L).astype(f32)
        ax = p0.axis
        to_edge = (gs[ax] - L - f32(2.0) - self.tx[ax]) if n[ax] > 0 else (self.tx[ax] - L - f32(1.0))
        rmax = float(self.setup["range_max"])
        rmin = float(self.setup["range_min"])
        self.range_max = float(f32(rmax)) if rmax > 0.0 else float(max(to_edge, f32(2.0) * f32(self.wl)))
        self.range_min = float(f32(rmin)) if rmin > 0.0 else float(f32(self.wl))
        if self.range_max <= self.range_min:
            self.range_max = float(f32(self.range_min) + f32(self.wl))
        if self.range_max > float(to_edge) + 1.0:
            warnings.append("radar: the image range reaches into the absorbing layer along boresight")
        ref = float(self.setup["reference"])
        rd = f32(ref) if ref > 0.0 else f32(1.5) * f32(self.wl)
        rd = min(rd, f32(0.8) * to_edge)
        self.reference = np.asarray([_round_half_away(float(v)) for v in self.tx + n * f32(rd)], f32)
        self.reference_distance = float(np.sqrt(np.sum((self.reference - self.tx) ** 2, dtype=f32)))
        # listening window (Radar.cpp:234-249)
        self.extent = float(max(float(np.sqrt(np.sum((p - self.tx) ** 2, dtype=f32))) for p in self.elem_pos))
        self.pulse_end = t_end
        provisional = t_end + 2.0 * (self.range_max + self.extent) + 24.0 * self.wl
        self.provisional_steps = int(math.ceil(provisional / self.dt))
        self.drive = np.zeros(self.provisional_steps)
        for k in range(self.provisional_steps):
            t = (k + 0.5) * self.dt
            self.drive[k] = sum(float(s.amplitude) * source_signal(s, t) for s in tx) / wsum
        self.start_calibration()

    # ---- recording -------------------------------------------------------------------------
    def channels(self):
        ch = [p.to_c() for p in self.elements]
        for k in range(REFERENCE_CHANNELS):
            ch.append(abi.Port(int(self.reference[0]), int(self.reference[1]), int(self.reference[2]), k, 1, 1))
        return ch

    def start_recording(self):
        self.g.ports_configure(self.channels(), self.wl, 4.0, False, self.steps)

    def start_calibration(self):
        self.phase = "calibrating"
        self.steps = self.provisional_steps
        self.window_measured = False
        self.last_window_check = 0
        self.cal = None
        self.meas = None
        self.image = None
        self.start_recording()

    def begin_measurement(self):
        self.phase = "measuring"
        self.steps = self.cal_steps
        self.image = None
        self.start_recording()

    def recorded(self):
        return self.g.ports_recorded()

    def read_series(self):
        """V per [step][channel] (float32)."""
        return np.ascontiguousarray(self.g.ports_series()[:, :, 0])

    def progress(self):
        if self.phase == "done":
            return 1.0
        if self.phase == "off" or not self.steps:
            return 0.0
        return min(1.0, self.recorded() / self.steps)

    def fidelity(self):
        return 10.0 ** (-(float(self.setup["dynamic_range_db"]) + 10.0) / 20.0)

    def calibration_complete(self):
        return self.phase == "calibrating" and self.cal is not None

    def update(self):
        """RadarMonitor::update (Radar.cpp:371-408), with the measurement processed when complete."""
        if self.phase == "calibrating" and self.cal is None:
            rec = self.recorded()
            period = max(16, int(self.wl / self.dt))
            if not self.window_measured and rec >= self.last_window_check + period:
                self.last_window_check = rec
                self.measure_window()
            if rec >= self.steps:
                cal = self.read_series()[: self.steps]
                self.cal = cal
                self.cal_steps = cal.shape[0]
                self.build_template()
        elif self.phase == "measuring":
            if self.recorded() >= self.steps:
                self.meas = self.read_series()[: self.steps]
                self.image = self.compute_image(self.meas, self.meas.shape[0], True)
                self.phase = "done"
                self.write_log()

    # ---- template and window (Radar.cpp:414-544) ---------------------------------------------
    def reference_channel(self, rec, n):
        C = len(self.elements)
        pk = np.abs(rec[:n, C:C + REFERENCE_CHANNELS]).max(axis=0)
        return int(np.argmax(pk))

    def measure_window(self):
        rec = self.read_series()
        C = len(self.elements)
        n = rec.shape[0]
        period = max(1, int(_round_half_away(self.wl / self.dt)))
        blocks = n // period
        if blocks < 6:
            return
        best = self.reference_channel(rec, n)
        x = np.abs(rec[: blocks * period, C + best].astype(np.float64)).reshape(blocks, period).max(axis=1)
        peak = float(x.max())
        if not peak > 0.0:
            return
        if np.any(x[blocks - 3:] >= self.fidelity() * peak):
            return
        F = _next_pow2(2 * n)
        templ = self.template_spectrum(rec, n, F)
        response = self.response_length(templ)
        window = 2.0 * self.range_max + self.extent + response + self.wl
        self.steps = int(min(max(int(math.ceil(window / self.dt)), n), self.provisional_steps))
        self.window_measured = True

    def tx_array_factor(self, p, omega):
        v = (np.asarray(p, f32) - self.tx_pos).astype(f32)
        d = np.maximum(np.sqrt((v * v).sum(axis=1, dtype=f32)).astype(np.float64), 0.5)
        g = np.maximum((v @ self.axes[2]).astype(f32).astype(np.float64) / d, 0.0)
        return np.sum((self.tx_amp * g / d) * np.exp(-1j * omega * d))

    def response_length(self, templ):
        t = np.fft.ifft(templ)
        half = len(t) // 2
        a = np.abs(t[:half])
        tmax = a.max()
        idx = np.nonzero(a > self.fidelity() * tmax)[0]
        last = int(idx[-1]) if idx.size else 0
        return (last + 1) * self.dt

    def template_spectrum(self, rec, n, F):
        C = len(self.elements)
        w = 2.0 * math.pi / self.wl
        dw = 2.0 * math.pi / (F * self.dt)
        best = self.reference_channel(rec, n)
        ref = np.zeros(F, complex)
        drive = np.zeros(F, complex)
        ref[:n] = rec[:n, C + best]
        m = min(n, len(self.drive))
        drive[:m] = self.drive[:m]
        ref = np.fft.fft(ref)
        drive = np.fft.fft(drive)
        dmax = np.abs(drive).max()
        templ = np.zeros(F, complex)
        k = np.arange(1, F // 2)
        om = k * dw
        af = np.zeros(k.size, complex)
        band = np.abs(om - w) <= 0.6 * w
        for j in np.nonzero(band)[0]:
            af[j] = self.tx_array_factor(self.reference, om[j])
        afmax = np.abs(af).max() if af.size else 0.0
        ok = np.abs(af) >= 1e-12
        r = ref[k] * np.conj(af) / (np.abs(af) ** 2 + 0.05 * afmax * afmax)
        t = r * r * np.conj(drive[k]) / (np.abs(drive[k]) ** 2 + 1e-8 * dmax * dmax)
        templ[k[ok]] = t[ok]
        return templ

    def build_template(self):
        C = len(self.elements)
        N = self.cal_steps
        w = 2.0 * math.pi / self.wl
        self.peak_tx = float(np.abs(self.cal[:N, :C].astype(np.float64)).max())
        F = _next_pow2(2 * N)
        self.fft_size = F
        dw = 2.0 * math.pi / (F * self.dt)
        templ = self.template_spectrum(self.cal, N, F)
        k = np.arange(1, F // 2)
        om = k * dw
        self.filter = np.zeros(F, complex)
        self.filter[k] = np.conj(templ[k]) * np.exp(-(((om - w) / (0.3 * w)) ** 2))
        k0 = min(max(int(_round_half_away(w / dw)), 2), F // 2 - 2)
        slope = np.angle(templ[k0 + 1] * np.conj(templ[k0 - 1])) / (2.0 * dw)
        self.system_delay = float(-slope - self.tx_time)
        self.template_end = self.response_length(templ)

    # ---- imaging (Radar.cpp:546-745) ---------------------------------------------------------
    def direction(self, az, el):
        a, e = f32(math.radians(az)), f32(math.radians(el))
        return ((self.axes[0] * f32(math.sin(a) * math.cos(e))) + self.axes[1] * f32(math.sin(e)) +
                self.axes[2] * f32(math.cos(a) * math.cos(e))).astype(f32)

    def angles_of(self, p):
        u = np.asarray(p, f32) - self.tx
        u = u / f32(np.sqrt(np.sum(u * u, dtype=f32)))
        return (math.degrees(math.atan2(float(np.dot(u, self.axes[0])), float(np.dot(u, self.axes[2])))),
                math.degrees(math.asin(min(max(float(np.dot(u, self.axes[1])), -1.0), 1.0))))

    def baseband(self, meas, N):
        """Echoes (measurement minus calibration, plus receiver noise), pulse-compressed and decimated
        to complex baseband: z (M, C) complex64 and the decimation D."""
        C = len(self.elements)
        dt, w = self.dt, 2.0 * math.pi / self.wl
        noise = float(self.setup["noise_db"])
        in_band = self.peak_tx * 10.0 ** (noise / 20.0) if noise > -299.0 else 0.0
        sigma = in_band * math.sqrt((0.5 / dt) / (0.376 / self.wl))
        F = self.fft_size
        D = max(1, int(_round_half_away(0.25 * self.wl / dt)))
        M = (N + D - 1) // D
        z = np.zeros((M, C), np.complex64)
        lag = np.arange(M) * D * dt - 0.5 * dt
        rot = np.exp(-1j * w * lag)
        for i in range(C):
            buf = np.zeros(F, complex)
            buf[:N] = meas[:N, i].astype(np.float64) - self.cal[:N, i].astype(np.float64)
            if sigma > 0.0:  # each element's own seeded generator (Radar.cpp:590-596)
                gauss = Normal(MT19937((20251105 + i) & 0xFFFFFFFF))
                buf[:N] += sigma * np.array([gauss() for _ in range(N)])
            buf = np.fft.ifft(np.fft.fft(buf) * self.filter)
            z[:, i] = (buf[: M * D: D] * rot).astype(np.complex64)
        return z, D, M

    def geometry(self, nr, naz, nel, D):
        g = abi.RadarGeometry()
        for k in range(3):
            g.tx[k] = float(self.tx[k])
            g.interior_min[k], g.interior_max[k] = float(self.interior_min[k]), float(self.interior_max[k])
            for r in range(3):
                g.axes[3 * r + k] = float(self.axes[r][k])
        g.omega = 2.0 * math.pi / float(f32(self.wl))
        g.dt, g.sample_dt = self.dt, D * self.dt
        g.r0, g.dr = float(f32(self.range_min)), float(f32(0.125) * f32(self.wl))
        g.nr, g.naz, g.nel = nr, naz, nel
        d_ang = 1.5
        g.daz = g.del_ = d_ang
        g.az0 = float(-f32(d_ang) * f32(naz // 2))
        g.el0 = float(-f32(d_ang) * f32(nel // 2))
        return g

    def backproject(self, z, g):
        lib = load_library()
        M, Cn = z.shape
        total = g.nr * g.nel * g.naz
        zz = np.ascontiguousarray(z.view(np.float32).reshape(M, 2 * Cn))
        out = np.zeros(total, np.float64)
        fp = C.POINTER(C.c_float)
        dp = C.POINTER(C.c_double)
        ep = np.ascontiguousarray(self.elem_pos, np.float32)
        wt = np.ascontiguousarray(self.weights, np.float64)
        tp = np.ascontiguousarray(self.tx_pos, np.float32)
        ta = np.ascontiguousarray(self.tx_amp, np.float64)
        _check(lib.emlab_radar_backproject(C.byref(g), zz.ctypes.data_as(fp), M, Cn, ep.ctypes.data_as(fp),
                                           wt.ctypes.data_as(dp), tp.ctypes.data_as(fp), ta.ctypes.data_as(dp),
                                           len(ta), out.ctypes.data_as(dp)))
        return out.reshape(g.nr, g.nel, g.naz)

    def compute_image(self, meas, n_meas, final):
        Cn = len(self.elements)
        N = min(n_meas, self.cal_steps, meas.shape[0])
        img = {"valid": False}
        if N < 32 or self.fft_size < 2 * N or not self.peak_tx > 0.0:
            return img
        echo = np.abs(meas[:N, :Cn].astype(np.float64) - self.cal[:N, :Cn].astype(np.float64)).max()
        img["echo_db"] = _to_db((echo / self.peak_tx) ** 2)
        img["complete_range"] = self.range_max
        z, D, _ = self.baseband(meas, N)
        dr = f32(0.125) * f32(self.wl)
        nr = max(2, int((f32(self.range_max) - f32(self.range_min)) / dr) + 1)
        naz = 2 * int(_round_half_away(float(self.setup["fov_az"]) / 1.5)) + 1
        nel = 2 * int(_round_half_away(float(self.setup["fov_el"]) / 1.5)) + 1
        geo = self.geometry(nr, naz, nel, D)
        power = self.backproject(z, geo)
        return self.detect(power, geo, final, img)

    def detect(self, power, geo, final, img):
        nr, nel, naz = power.shape
        pmax = power.max()
        if not pmax > 0.0:
            return img
        inside_mask = power >= 0.0
        with np.errstate(divide="ignore"):
            db = np.where(power > 1e-300 * pmax, 10.0 * np.log10(np.maximum(power, 1e-300) / pmax), -3000.0)
        db = np.where(inside_mask, db, -3000.0).astype(np.float32)
        inside = db[inside_mask]
        floor = -100.0
        if inside.size >= 16:
            floor = float(np.partition(inside, inside.size // 2)[inside.size // 2])
        img.update(valid=True, floor_db=floor, nr=nr, naz=naz, nel=nel, power_db=db)
        min_level = max(floor + float(self.setup["threshold_db"]), -float(self.setup["dynamic_range_db"]))

        def at(ir, ie, ia):
            return db[min(max(ir, 0), nr - 1), min(max(ie, 0), nel - 1), min(max(ia, 0), naz - 1)]
        dets = []
        last = nr - 1
        if inside.size >= 16:
            for ir in range(1, last):
                cand = np.argwhere(db[ir] >= min_level)
                for ie, ia in cand:
                    v = db[ir, ie, ia]
                    peak = True
                    for a in (-1, 0, 1):
                        for b in (-1, 0, 1):
                            for c in (-1, 0, 1):
                                if not peak or (a == 0 and b == 0 and c == 0):
                                    continue
                                jr, je, ja = ir + a, ie + b, ia + c
                                if jr < 0 or je < 0 or ja < 0 or jr >= nr or je >= nel or ja >= naz:
                                    continue
                                u = db[jr, je, ja]
                                if u > v or (u == v and (a < 0 or (a == 0 and (b < 0 or (b == 0 and c < 0))))):
                                    peak = False
                    if not peak:
                        continue
                    fr = _vertex_offset(at(ir - 1, ie, ia), v, at(ir + 1, ie, ia))
                    fe = _vertex_offset(at(ir, ie - 1, ia), v, at(ir, ie + 1, ia))
                    fa = _vertex_offset(at(ir, ie, ia - 1), v, at(ir, ie, ia + 1))
                    d = {"range": float(f32(geo.r0) + (f32(ir) + fr) * f32(geo.dr)),
                         "el": float(f32(geo.el0) + (f32(ie) + fe) * f32(geo.del_)),
                         "az": float(f32(geo.az0) + (f32(ia) + fa) * f32(geo.daz)),
                         "rel_db": float(v), "snr_db": float(v) - floor, "target": -1}
                    d["position"] = self.tx + f32(d["range"]) * self.direction(d["az"], d["el"])
                    dets.append(d)
        dets.sort(key=lambda d: -d["rel_db"])
        dets = dets[:MAX_DETECTIONS]
        for d in dets:  # truth: the nearest marked target and its point nearest the radar
            nearest = 1e30
            for t, tg in enumerate(self.targets):
                pts = tg["points"]
                if len(pts):
                    dist = float(np.sqrt(((pts - d["position"]) ** 2).sum(axis=1)).min())
                else:
                    q = np.clip(d["position"], tg["min"], tg["max"])
                    dist = float(np.sqrt(((d["position"] - q) ** 2).sum()))
                if dist < nearest:
                    nearest, d["target"] = dist, t
            if d["target"] < 0:
                continue
            q = self.target_nearest[d["target"]]
            d["target_range"] = float(np.sqrt(np.sum((q - self.tx) ** 2, dtype=f32)))
            d["target_az"], d["target_el"] = self.angles_of(q)
        img["detections"] = dets
        return img

    def write_log(self, path=None):
        path = path or self.setup.get("log_path")
        img = self.image
        if not path or not img or not img.get("valid"):
            return
        with open(path, "w") as f:
            f.write("detection,range_cells,range_m,azimuth_deg,elevation_deg,above_floor_db,relative_db,target,"
                    "target_range_cells,target_azimuth_deg,target_elevation_deg\n")
            for k, d in enumerate(img["detections"]):
                name = self.targets[d["target"]]["name"] if d["target"] >= 0 else ""
                f.write(f"{k + 1},{d['range']:g},{d['range'] * self.cell_size:g},{d['az']:g},{d['el']:g},"
                        f"{d['snr_db']:g},{d['rel_db']:g},{name},{d.get('target_range', 0.0):g},"
                        f"{d.get('target_az', 0.0):g},{d.get('target_el', 0.0):g}\n")

    # ---- report (Instruments.cpp:412-444) ----------------------------------------------------
    def report(self, out):
        if self.phase == "off":
            return
        if self.phase == "calibrating":
            out(f"    radar: calibrating without the targets ({100.0 * self.progress():.0f}% of {self.steps} steps)")
            return
        img = self.image
        if self.phase == "measuring":
            out(f"    radar: measuring ({100.0 * self.progress():.0f}% of {self.steps} steps), image final out to "
                f"{(img['complete_range'] * self.cell_size * 1e3 if img and img.get('valid') else 0.0):.1f} mm")
            if not img or not img.get("valid"):
                return
        if not img or not img.get("valid"):
            out("    radar: no image")
            return
        cell = self.cell_size * 1e3
        out(f"    radar: strongest echo {-img['echo_db']:.1f} dB below the transmit pulse at an element, image floor "
            f"{img['floor_db']:.1f} dB, {len(img['detections'])} detection(s)")
        for k, d in enumerate(img["detections"]):
            line = (f"      #{k + 1} range {d['range'] * cell:6.1f} mm ({d['range'] / self.wl:5.2f} lambda)  az "
                    f"{d['az']:+5.1f}  el {d['el']:+5.1f} deg  {d['rel_db']:+6.1f} dB ({d['snr_db']:.1f} dB above floor)")
            if d["target"] >= 0:
                line += (f" | {self.targets[d['target']]['name']}: front at {d['target_range'] * cell:.1f} mm, az "
                         f"{d['target_az']:+.1f}, el {d['target_el']:+.1f}")
            out(line)
