"""Radar set-up and detection on the host: the array frame, receive taper, transmit centre and
timing, listening window, and the local-maximum detector with its sub-bin refinement."""
import math
import os

import numpy as np
import pytest

from em_lab_gb300 import abi
from em_lab_gb300.radar import RadarMonitor
from em_lab_gb300.script import ScriptEngine

SCENES = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "em_lab_gb300", "scenes")


class FakeGrid:
    def __init__(self, sc):
        self.sc = sc
        self.configured = []

    def dt(self):
        return float(self.sc.grid.courant)

    def size(self):
        return tuple(self.sc.grid.size)

    def config(self):
        return self.sc.grid

    def ports_configure(self, ports, wl, avg, sweep, steps):
        self.configured.append((len(ports), steps))

    def ports_recorded(self):
        return 0


@pytest.fixture(scope="module")
def radar():
    res = ScriptEngine(echo=False).run_file(os.path.join(SCENES, "monopole_radar.lua"))
    sc = res.scene
    g = FakeGrid(sc)
    warns = []
    r = RadarMonitor(g, sc.radar, sc.ports, sc.sources, sc.ports[0].wavelength, sc.cell_size, sc.targets, warns)
    return r, sc, g, warns


def test_frame_taper_and_transmitter(radar):
    r, sc, g, warns = radar
    assert r.phase == "calibrating" and not warns
    np.testing.assert_array_equal(r.axes[2], [1, 0, 0])  # boresight along the feeds (+x)
    np.testing.assert_array_equal(r.axes[1], [0, 0, 1])  # up
    np.testing.assert_array_equal(r.axes[0], [0, -1, 0])  # right = n x up
    # Hamming over 6 rows and 6 columns: a - (1 - a) cos(2 pi (k + 1) / 7)
    w1 = [0.54 - 0.46 * math.cos(2 * math.pi * (k + 1) / 7) for k in range(6)]
    assert sorted(set(np.round(r.weights, 12))) == sorted(set(np.round([a * b for a in w1 for b in w1], 12)))
    # the 2 x 2 centre elements transmit: the phase centre is their mean + the phase-centre offset
    assert len(r.tx_sources) == 4
    np.testing.assert_allclose(r.tx, np.mean([s.center for s in r.tx_sources], axis=0) + [1.5, 2.0, 0.0], atol=1e-5)
    # 36 elements + 3 reference channels recorded for the provisional window
    assert g.configured[-1] == (39, r.provisional_steps)
    assert r.reference[0] == math.floor(float(r.tx[0]) + 1.5 * 20 + 0.5)  # glm::round: halves away from 0
    tau = 0.5 * 20
    assert r.pulse_end == pytest.approx(6 * tau)
    assert r.provisional_steps == math.ceil((6 * tau + 2 * (150 + r.extent) + 24 * 20) / 0.5)
    assert len(r.elements) == 36


def test_detector_finds_a_synthetic_peak(radar):
    r, sc, g, warns = radar
    geo = r.geometry(40, 21, 21, 10)
    power = np.full((40, 21, 21), 1e-4)
    power[0, 0, 0] = -1.0  # outside the volume
    power[17, 12, 8] = 1.0
    power[16, 12, 8] = power[18, 12, 8] = 0.5
    power[17, 12, 7], power[17, 12, 9] = 0.25, 0.5
    img = r.detect(power, geo, True, {"valid": False})
    assert img["valid"] and len(img["detections"]) == 1
    d = img["detections"][0]
    assert d["rel_db"] == 0.0 and d["snr_db"] == pytest.approx(40.0, abs=1e-4)
    # parabolic refinement: symmetric in range, skewed toward the larger azimuth neighbour
    assert d["range"] == pytest.approx(geo.r0 + 17 * geo.dr, abs=1e-5)
    assert d["az"] > geo.az0 + 8 * geo.daz
    assert d["target"] == 0 and "target_range" in d
