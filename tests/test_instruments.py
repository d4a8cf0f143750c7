"""Instrument arithmetic of the headless runner on a stand-in grid (no GPU): far-field pattern
analysis, port readings, sweep analysis, probe interpolation, flux signs and the report lines."""
import math

import numpy as np
import pytest

from em_lab_gb300 import configs
from em_lab_gb300.instruments import Instruments, far_field_directions, sample_block
from em_lab_gb300.scene import FluxSetup, PortSetup


class FakeGrid:
    def __init__(self, t=100.0, step=200):
        self.t, self.n = t, step
        self.pattern = None
        self.phasors = None
        self.sweep = None

    def time(self):
        return self.t

    def step_count(self):
        return self.n

    def ports_configure(self, *a, **k):
        pass

    def ntff_configure(self, mn, mx, wl, avg):
        return tuple(mn), tuple(mx)

    def ntff_evaluate(self, dirs):
        return self.pattern(np.asarray(dirs, np.float64))

    def ports_phasors(self):
        return self.phasors

    def ports_series(self):
        return np.zeros((400, 1, 2), np.float32)

    def ports_sweep_sums(self, lo, hi, pts):
        return self.sweep(lo, hi, pts)

    def probe_gather(self, origins):
        out = np.zeros((len(origins), 54, 4), np.float32)
        for i, o in enumerate(origins):
            for t in range(27):
                x, y, z = o[0] + t % 3, o[1] + (t // 3) % 3, o[2] + t // 9
                out[i, t, :3] = (x, y, z)           # E = position: interpolation must reproduce it
                out[i, 27 + t, :3] = (2 * x, 0, 0)
        return out

    def flux_planes(self, planes):
        return np.array([1.0 + p.axis for p in planes])


def test_hertzian_pattern_directivity_and_beamwidth():
    sc = configs.plain_small()
    g = FakeGrid()
    wl = sc.far_field["wavelength"]
    k = 2 * math.pi / wl
    P = k * k / (8 * math.pi) / 1.5            # |F|^2 = sin^2(theta) has D_max = 1.5

    def pattern(d):
        out = np.zeros((len(d), 2))
        out[:, 0] = 1.0 - d[:, 2] ** 2
        out[0, 1] = P
        return out
    g.pattern = pattern
    inst = Instruments(g, sc)
    inst.evaluate_far_field()
    pat = inst.pattern
    assert pat["valid"] and pat["max_dbi"] == pytest.approx(10 * math.log10(1.5), abs=1e-3)
    cuts = {c["name"]: c for c in pat["cuts"]}
    assert cuts["xy"]["beamwidth"] >= 359.0                   # omni in the azimuth plane
    assert cuts["xz"]["beamwidth"] == pytest.approx(90.0, abs=0.3)
    assert cuts["yz"]["peak_angle"] in (0.0, 180.0)
    lines = []
    inst.out = lines.append
    inst.measure()
    inst.print_report()
    text = "\n".join(lines)
    assert "far field [lambda=16.0 cells" in text and "D_max=1.76 dBi (1.50)" in text
    # -3 dB crossings interpolated linearly in dB between 2-degree samples: 89.8 deg for sin^2
    assert "xz-cut: peak   1.76 dBi" in text and "HPBW 89.8 deg" in text and "HPBW omni" in text


def test_direction_set_sizes():
    dirs, cuts = far_field_directions((0, 0, 1))
    assert len(cuts) == 3 and all(len(c["angles"]) == 180 for c in cuts)
    assert np.allclose(np.linalg.norm(dirs, axis=1), 1.0, atol=1e-6)
    f = np.float32
    inside = 0
    for r in range(81):
        for c in range(81):
            u, v = f(-1) + f(f(2 * c) / f(80)), f(1) - f(f(2 * r) / f(80))
            inside += f(u * u) + f(v * v) <= f(1)
    assert len(dirs) == 540 + 2 * inside


def test_port_readings_and_sweep():
    sc = configs.plain_small()
    sc.ports = [PortSetup("feed", (64, 64, 64), 2, 1.0, 1, 16.0, True, 50.0, 1.0)]
    sc.sweep = {"wavelength_min": 10.0, "wavelength_max": 30.0, "points": 21, "log": ""}
    g = FakeGrid()
    z_norm = complex(73.0, 42.5) / 376.730313668
    I = complex(0.01, 0.002)
    V = z_norm * I
    ph = np.zeros((1, 8), np.float32)
    ph[0, 4:8] = (-V.real, -V.imag, I.real, I.imag)        # stage 2: gap field along the feed = -V
    g.phasors = ph

    def sweep(lo, hi, pts):  # an RLC-like impedance with a match near lambda = 20
        out = np.zeros((1, pts, 4))
        for f in range(pts):
            nu = 1 / hi + (1 / lo - 1 / hi) * f / (pts - 1)
            z = complex(50.0, 400.0 * (nu - 0.05) / 0.05) / 376.730313668
            out[0, f] = (-z.real, -z.imag, 1.0, 0.0)
        return out, 2e-4
    g.sweep = sweep
    inst = Instruments(g, sc)
    inst.evaluate_ports()
    r = inst.readings[0]
    assert r["z"] == pytest.approx(complex(73.0, 42.5), rel=1e-5)
    gam = (r["z"] - 50) / (r["z"] + 50)
    assert abs(r["gamma"] - gam) < 1e-9 and r["vswr"] == pytest.approx((1 + abs(gam)) / (1 - abs(gam)))
    inst.evaluate_sweep()
    ps = inst.sweep_result["ports"][0]
    assert ps["best_wl"] == pytest.approx(20.0, rel=1e-3) and ps["points"][ps["best"]]["s11"] < -100
    assert ps["band"] is not None
    lines = []
    inst.out = lines.append
    inst.print_ports(4)
    assert lines[0].startswith("    sweep: 400 steps recorded, ring-down 2.0e-04 of peak (settled)")
    assert "best match" in lines[1] and "-10 dB band" in lines[1]


def test_probe_interpolation_and_flux_signs():
    sc = configs.plain_small()
    sc.fluxes.append(FluxSetup("plane", "plane", axis=1, index=40, rect_min=(10, 10), rect_max=(20, 20)))
    g = FakeGrid()
    inst = Instruments(g, sc)
    inst.measure()
    s = inst.probes[0]["sample"]
    x, y, z = inst.probes[0]["pos"]
    assert s["E"] == pytest.approx([x - 0.5, y - 0.5, z - 0.5])  # E = position, each component at its stagger
    assert s["B"][0] == pytest.approx(2 * x)
    assert s["eps"] == 1.0 and s["sigma"] == 0.0
    # box: six planes, outward signs -1/+1 per axis with values 1 + axis -> total 0; plane: +2
    assert inst.fluxes[0]["inst"] == 0.0 and inst.fluxes[1]["inst"] == 2.0


def test_sample_block_matches_trilinear():
    rng = np.random.default_rng(3)
    blk = rng.standard_normal((27, 4)).astype(np.float32)
    q = (10.3, 20.7, 5.5)
    origin = [9, 20, 4]
    got = sample_block(blk, origin, [3, 3, 3], q, 1)
    f = [q[i] - math.floor(q[i]) for i in range(3)]
    i0 = [int(math.floor(q[i])) - origin[i] for i in range(3)]
    want = 0.0
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = (f[0] if dx else 1 - f[0]) * (f[1] if dy else 1 - f[1]) * (f[2] if dz else 1 - f[2])
                want += w * blk[((i0[2] + dz) * 3 + i0[1] + dy) * 3 + i0[0] + dx, 1]
    assert got == pytest.approx(want, rel=1e-5)


def test_csv_logs(tmp_path):
    sc = configs.plain_small()
    sc.probe_logs = ["probe.csv"]
    sc.fluxes[0].log = "logs/flux.csv"
    g = FakeGrid()
    inst = Instruments(g, sc, out=lambda s: None, output_dir=str(tmp_path))
    inst.measure()
    g.t, g.n = 101.0, 202
    inst.measure()
    inst.close()
    probe = (tmp_path / "probe.csv").read_text().splitlines()
    flux = (tmp_path / "logs" / "flux.csv").read_text().splitlines()
    assert probe[0] == "step,time,Ex,Ey,Ez,Bx,By,Bz,absE,absB,Sx,Sy,Sz"
    assert probe[1].startswith("200,100,33.5,63.5,63.5,68,0,0,") and len(probe) == 3
    assert flux == ["step,time,P,P_avg", "200,100,0,0", "202,101,0,0"]
