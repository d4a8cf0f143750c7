"""CPU checks of the planar phased-array workload's host side: the seeded steering directions, the
angle grid, the pointing-error measure, and the scene script's taper and true-time delays."""
import math

import numpy as np
import pytest

from em_lab_gb300 import phased


def test_steering_directions_are_seeded_and_in_range():
    a, b = phased.steering_directions(5, 8), phased.steering_directions(5, 8)
    assert a == b and len(a) == 8
    assert all(0.0 <= t <= 40.0 and 0.0 <= p < 360.0 for t, p in a)
    assert phased.steering_directions(6, 8) != a


def test_angle_grid_unit_vectors():
    d, th, ph = phased.angle_grid(19, 37)
    assert d.shape == (19 * 37, 3) and d.dtype == np.float32
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    np.testing.assert_allclose(d[0], (0.0, 0.0, 1.0), atol=1e-7)   # theta 0: +z
    assert th[0] == 0.0 and th[-1] == 180.0 and ph[-1] == 360.0
    k = 9 * 37 + 9                                                  # theta 90, phi 90: +y
    np.testing.assert_allclose(d[k], (0.0, 1.0, 0.0), atol=1e-6)


def test_angular_error():
    assert phased.angular_error(20.0, 30.0, 20.0, 30.0) == pytest.approx(0.0, abs=1e-6)
    assert phased.angular_error(0.0, 0.0, 0.0, 123.0) == pytest.approx(0.0, abs=1e-6)  # the pole
    assert phased.angular_error(90.0, 0.0, 90.0, 90.0) == pytest.approx(90.0)
    assert phased.angular_error(10.0, 0.0, 10.0, 180.0) == pytest.approx(20.0)


def test_scene_taper_and_true_time_delays():
    """4 x 4 elements steered to (30, 0): symmetric Taylor amplitudes peaking at 1, and delays that
    grow by pitch * sin(theta) / lambda periods per column along +x, equal along y."""
    sc = phased.build(30.0, 0.0, elements=4, nxy=128, nz=128)
    assert len(sc.ports) == 16 and len(sc.sources) == 16
    amp = {p.name: p.drive for p in sc.ports}                          # the feed's drive voltage
    delay = {p.name: sc.sources[s_i].delay_periods for s_i, p in enumerate(sc.ports)}
    assert all(sc.sources[k].port == k for k in range(16))             # one source per feed, in order
    a = [[amp[f"d[{i},{j}]"] for j in range(1, 5)] for i in range(1, 5)]
    np.testing.assert_allclose(a, np.array(a).T, rtol=1e-6)            # separable and symmetric
    np.testing.assert_allclose(a[0], a[0][::-1], rtol=1e-6)
    assert max(max(r) for r in a) == pytest.approx(1.0)
    step = 12 * math.sin(math.radians(30.0)) / 24                       # pitch lambda/2, periods
    for j in range(1, 5):
        for i in range(1, 4):
            assert delay[f"d[{i + 1},{j}]"] - delay[f"d[{i},{j}]"] == pytest.approx(step, rel=1e-6)
    for i in range(1, 5):
        assert len({round(delay[f"d[{i},{j}]"], 6) for j in range(1, 5)}) == 1
    assert min(delay.values()) == pytest.approx(1.0)                    # the earliest feed fires after 1 period
