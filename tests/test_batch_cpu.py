"""Host side of the batched antenna sweep: the seeded scene generator, the -60 dB ring-down watch
and the FP64 impedance sweep (Ports.cpp:187-278) of a port series."""
import math

import numpy as np
import pytest

from em_lab_gb300 import batch, configs


def test_batched_scene_generator_is_seeded_and_in_range():
    a = configs.batched_scene(5, 3)
    b = configs.batched_scene(5, 3)
    assert a.grid.size == b.grid.size and a.description == b.description
    assert np.array_equal(a.materials.sigma, b.materials.sigma) and np.array_equal(a.materials.epsilon_r,
                                                                                    b.materials.epsilon_r)
    scs = configs.batched_scenes(64, seed=11)
    edges = {sc.grid.size[0] for sc in scs}
    assert edges <= set(configs.BATCH_EDGES) and len(edges) >= 6
    kinds = [sc.description.split()[0] for sc in scs]
    assert 15 < kinds.count("monopole") < 49
    for sc in scs:
        n = sc.grid.size[0]
        assert sc.grid.size == (n, n, n) and sc.grid.pml_thickness == 8
        assert len(sc.ports) == 1 and len(sc.sources) == 1 and sc.ports[0].impedance_ohm == 50.0
        wl = sc.wavelength
        assert wl == pytest.approx(0.6 * (n - 16), rel=1e-6)
        length = float(sc.description.split()[1][2:])
        assert 0.3 * wl <= length <= 0.7 * wl
        radius = float(sc.description.split()[2][2:])
        assert 0.02 <= radius <= 0.2
        eps = float(sc.description.split()[3][4:])
        assert 1.0 <= eps <= 10.0
        assert sc.sweep["points"] == 128
        # every scene fits its antenna inside the absorber-free region
        p = sc.ports[0].texel
        assert all(8 < v < n - 9 for v in p)


def test_ringdown_watch_on_a_damped_tone():
    """The reference's criterion (Ports.cpp:206-213): settled once the largest |V| of the last 5 %
    of the series is 60 dB below the peak."""
    dt, period = 0.5, 40.0  # steps per period = 80
    w = batch.RingDown(min_steps=320)
    k = np.arange(4000)
    tau = 150.0  # steps: amplitude e^{-k / tau}
    v = np.sin(2 * math.pi * k / (period / dt)) * np.exp(-k / tau)
    done_at = None
    for c in range(0, k.size, 64):
        if w.feed(v[c:c + 64]):
            done_at = c + 64
            break
    assert done_at is not None
    assert w.residual() == pytest.approx(batch.residual(v[:done_at]), rel=1e-6)
    # the late window starts at 0.95 n: e^{-0.95 n / tau} <= 1e-3 from n = tau ln(1000) / 0.95
    settle = tau * math.log(1000.0) / 0.95
    assert settle - 80 < done_at <= settle + 64 + 80
    assert batch.residual(v[:done_at]) <= 1e-3 < batch.residual(v[:done_at - 64])
    # a silent start (delayed pulse) does not count as ring-down
    w2 = batch.RingDown(min_steps=20)
    assert not w2.feed(np.zeros(200)) and w2.residual() == 1.0


def test_ringdown_stops_at_the_step_cap():
    w = batch.RingDown(min_steps=10, max_steps=256)
    v = np.sin(np.arange(300) * 0.3)  # never decays
    done = [w.feed(v[c:c + 64]) for c in range(0, 256, 64)]
    assert done == [False, False, False, True] and not w.rung_down()


def test_sweep_sums_match_a_direct_dft():
    rng = np.random.default_rng(4)
    ser = rng.standard_normal((300, 2)).astype(np.float32)
    dt = 0.5
    sums = batch.sweep_sums(ser, 10.0, 40.0, 7, dt)
    nu = 1 / 40.0 + (1 / 10.0 - 1 / 40.0) * np.arange(7) / 6
    for f in range(7):
        w = 2 * math.pi * nu[f]
        V = sum(float(ser[k, 0]) * complex(math.cos(-w * dt * k), math.sin(-w * dt * k)) for k in range(300))
        I = sum(float(ser[k, 1]) * complex(math.cos(-w * dt * k), math.sin(-w * dt * k)) for k in range(300))
        I *= complex(math.cos(w * 0.5 * dt), math.sin(w * 0.5 * dt))
        assert sums[f, 0] == pytest.approx(V.real, abs=1e-9) and sums[f, 1] == pytest.approx(V.imag, abs=1e-9)
        assert sums[f, 2] == pytest.approx(I.real, abs=1e-9) and sums[f, 3] == pytest.approx(I.imag, abs=1e-9)


def test_impedance_of_a_resistive_port():
    """V = -(R / eta0) * I at every frequency gives Z = R and the matched S11."""
    rng = np.random.default_rng(1)
    i = rng.standard_normal(256)
    sums = np.zeros((5, 4))
    sums[:, 2], sums[:, 3] = i[:5], i[5:10]
    r = 73.0
    sums[:, 0] = -(r / batch.K_ETA0) * sums[:, 2]
    sums[:, 1] = -(r / batch.K_ETA0) * sums[:, 3]
    z = batch.impedance(sums, 10.0, 20.0, 50.0)
    np.testing.assert_allclose(z["z"].real, r, rtol=1e-12)
    np.testing.assert_allclose(z["z"].imag, 0.0, atol=1e-9)
    g = (r - 50.0) / (r + 50.0)
    np.testing.assert_allclose(z["s11"], 20 * math.log10(g), rtol=1e-12)


def test_far_field_spectra_of_a_dipole_pattern():
    """FarField: the direction grid, the frequencies over the sweep band, the scene's box inside its
    absorber, and the spectra formula on a synthetic short-dipole pattern |F|^2 ~ sin^2(theta):
    D = 1.5 (1.76 dBi) and the radiated energy in dB over lambda0^2 of the unscaled sums."""
    ff = batch.FarField(8)
    d = ff.dirs.astype(np.float64)
    assert d.shape == (18 * 36 + 2, 3) and np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    sc = configs.batched_scene(4, 2)
    wl = ff.wavelengths(sc)
    sw = sc.sweep
    assert wl[0] == pytest.approx(sw["wavelength_max"]) and wl[-1] == pytest.approx(sw["wavelength_min"])
    assert np.all(np.diff(1.0 / wl) > 0)
    n, L = sc.grid.size, sc.grid.pml_thickness
    assert batch.FarField.box(sc, 100) == [L + 1, L + 1, 100 + L + 1, n[0] - L - 2, n[1] - L - 2, 100 + n[2] - L - 2]
    # a pattern |F|^2 = A sin^2(theta) whose peak gives D = k^2 A / (8 pi P) = 1.5 (a short dipole)
    k = 2.0 * math.pi / wl
    P = np.linspace(1.0, 2.0, 8)
    A = 1.5 * 8.0 * math.pi * P / (k * k)
    sin2 = 1.0 - d[:, 2] ** 2
    out = np.zeros((8, len(d), 2), np.float32)
    out[:, :, 0] = A[:, None] * sin2[None, :]
    out[:, 0, 1] = P
    samples = 1000
    spec = ff.spectra(sc, out, samples)
    assert spec.shape == (2, 8)
    np.testing.assert_allclose(spec[0], 10.0 * math.log10(1.5) + 10.0 * np.log10(sin2.max()), atol=1e-4)
    np.testing.assert_allclose(spec[1], 10.0 * np.log10(P * (samples / 2.0) ** 2 / sc.wavelength ** 2), rtol=1e-5)
