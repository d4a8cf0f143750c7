"""The radar on the GPU: the back-projection kernel against the CPU restatement, and a two-pass
radar scene (calibration without the target, measurement with it) run headless end to end."""
import math
import os

import numpy as np
import pytest

from em_lab_gb300 import abi, headless
from em_lab_gb300.radar import RadarMonitor
from oracle import radar_ref

pytestmark = pytest.mark.gpu
SCENES = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "em_lab_gb300", "scenes")


def test_backprojection_matches_the_cpu_restatement():
    rng = np.random.default_rng(5)
    C, M = 9, 60
    g = abi.RadarGeometry()
    tx = np.array([20.3, 40.1, 39.7], np.float32)
    for k in range(3):
        g.tx[k] = float(tx[k])
        g.interior_min[k] = 5.0
        g.interior_max[k] = 90.0
    for k, v in enumerate([0, -1, 0, 0, 0, 1, 1, 0, 0]):  # right, up, boresight (+x)
        g.axes[k] = float(v)
    g.omega, g.dt, g.sample_dt = 2 * math.pi / 16.0, 0.5, 2.0
    g.r0, g.dr, g.az0, g.daz, g.el0, g.del_ = 10.0, 2.0, -12.0, 3.0, -9.0, 3.0
    g.nr, g.naz, g.nel = 9, 9, 7
    z = (rng.standard_normal((M, C)) + 1j * rng.standard_normal((M, C))).astype(np.complex64)
    ep = (tx + rng.uniform(-6, 6, (C, 3))).astype(np.float32)
    w = rng.uniform(0.3, 1.0, C)
    tp = (tx + rng.uniform(-2, 2, (3, 3))).astype(np.float32)
    ta = rng.uniform(0.5, 1.5, 3)

    class Fake:
        elem_pos, weights, tx_pos, tx_amp = ep, w, tp, ta
    got = RadarMonitor.backproject(Fake(), z, g)
    ref = radar_ref.backproject(g, z, ep, w, tp, ta)
    inside = ref >= 0
    assert inside.sum() > 100 and np.array_equal(got < 0, ref < 0)
    np.testing.assert_allclose(got[inside], ref[inside], rtol=2e-4, atol=1e-6 * ref.max())


def test_backprojection_matches_the_reference_image():
    """The GPU kernel against the reference's own back-projection (Radar.cpp:606-646 compiled from
    the reference tree; tests/golden/radar_backproject.npz): same image points inside the volume,
    values within the tolerance of the FP32-geometry comparison above."""
    gold = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "radar_backproject.npz"))
    g = abi.RadarGeometry.from_buffer_copy(gold["geometry"].tobytes())

    class Fake:
        elem_pos, weights, tx_pos, tx_amp = gold["elem_pos"], gold["weights"], gold["tx_pos"], gold["tx_amp"]
    got = RadarMonitor.backproject(Fake(), gold["z"], g)
    ref = gold["power"]
    inside = ref >= 0
    assert inside.any() and (~inside).any() and np.array_equal(got < 0, ref < 0)
    np.testing.assert_allclose(got[inside], ref[inside], rtol=2e-4, atol=1e-6 * ref.max())


def test_radar_scene_detects_the_sphere(tmp_path, capsys):
    code, inst = headless.run(os.path.join(SCENES, "monopole_radar.lua"), 600, steps_per_frame=8)
    out = capsys.readouterr().out
    assert code == 0
    r = inst.radar
    assert r is not None and r.phase == "done", out[-2000:]
    img = r.image
    assert img["valid"] and img["detections"], out[-2000:]
    d = img["detections"][0]
    assert d["target"] == 0
    # the strongest return is the sphere's front: within a range bin and a few degrees of the truth
    assert abs(d["range"] - d["target_range"]) < 0.25 * 20
    assert abs(d["az"] - d["target_az"]) < 4.0 and abs(d["el"] - d["target_el"]) < 4.0
    assert "radar: strongest echo" in out and "| sphere: front at" in out
