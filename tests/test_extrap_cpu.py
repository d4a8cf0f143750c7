"""The learned extrapolator's host side: the CPU restatement's backward formulas against finite
differences, its BF16 rounding, and the early-window features."""
import math

import numpy as np
import pytest

from em_lab_gb300 import batch, configs, extrap
from oracle import extrap_ref as R


def small_params(seed=1):
    p = extrap.init_params(seed)
    return {k: (w.astype(np.float64), b.astype(np.float64) + 0.01) for k, (w, b) in p.items()}


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 1e-30, 3.14159265], np.float32)
    r = R.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # a tie rounds to the even mantissa
    assert r[2] == np.float32(1.0 + 2 ** -7)  # above the tie: up
    assert r[3] == -2.5
    assert r[5] == np.float32(3.140625)
    assert np.all(R.bf16(r) == r)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = small_params()
    B, n = 3, 3
    x = rng.standard_normal((B, extrap.T_IN, 2))
    zt = rng.standard_normal((B, extrap.AUX)) * 0.5
    t = rng.standard_normal((B, extrap.OUT)) * 0.5
    y, cache = R.forward(p, x, zt, exact=True)
    g = R.backward(p, cache, t, n, exact=True)
    for name in ("conv1", "conv2", "fc1", "fc3", "out"):
        w, b = p[name]
        for _ in range(3):
            i, j = rng.integers(0, w.shape[0]), rng.integers(0, w.shape[1])
            h = 1e-6
            wp, wm = w.copy(), w.copy()
            wp[i, j] += h
            wm[i, j] -= h
            lp = R.loss({**p, name: (wp, b)}, x, zt, t, n)
            lm = R.loss({**p, name: (wm, b)}, x, zt, t, n)
            fd = (lp - lm) / (2 * h)
            assert g[name][0][i, j] == pytest.approx(fd, rel=1e-4, abs=1e-9), (name, i, j)
        k = rng.integers(0, b.shape[0])
        bp, bm = b.copy(), b.copy()
        bp[k] += 1e-6
        bm[k] -= 1e-6
        fd = (R.loss({**p, name: (w, bp)}, x, zt, t, n) - R.loss({**p, name: (w, bm)}, x, zt, t, n)) / 2e-6
        assert g[name][1][k] == pytest.approx(fd, rel=1e-4, abs=1e-9), (name, "bias", k)


def test_layer_shapes_follow_the_spec():
    shapes = {n: (o, i) for n, o, i in extrap.layer_shapes()}
    assert shapes["conv1"] == (32, 16) and shapes["conv2"] == (64, 256)
    # head inputs: 1024 encoder features, Re/Im of the 128-point truncated Z(f), the 32-frequency
    # surface-DFT spectra (directivity and radiated energy); outputs: Z(f) and the far-field spectra
    assert shapes["fc1"] == (256, 1024 + 256 + 64) and shapes["fc4"] == (256, 256) and shapes["out"] == (320, 256)
    hidden = [n for n, i, o, r in extrap.HEAD if r]
    assert len(hidden) == 4  # a 4-layer MLP head of width 256


def test_features_are_scale_invariant_and_match_the_sweep():
    sc = configs.batched_scene(4, 0)
    n = extrap.early_steps(sc)
    assert n == math.ceil(extrap.PERIODS_IN * sc.wavelength / 0.5)
    k = np.arange(n + 50)
    v = np.sin(k * 0.07) * np.exp(-k / 300.0)
    i = 0.1 * np.cos(k * 0.07 + 0.3) * np.exp(-k / 300.0)
    ser = np.stack([v, i], axis=1).astype(np.float32)
    far = np.stack([np.linspace(1.8, 2.6, extrap.NFF), np.linspace(-3.0, 14.0, extrap.NFF)])
    x1, z1, zt1 = extrap.features(sc, ser, far)
    x2, z2, zt2 = extrap.features(sc, ser * np.float32(8.0), far)
    np.testing.assert_allclose(x1, x2, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(zt1, zt2, rtol=1e-5)
    assert x1.shape == (extrap.T_IN, 2) and z1.shape == (extrap.AUX,)
    # the surface-DFT channels: the early window's spectra in network units
    np.testing.assert_allclose(z1[2 * extrap.NF:], far.reshape(-1) / 10.0, rtol=1e-6)
    assert np.abs(x1).max() == pytest.approx(1.0, rel=1e-6)
    # Z_trunc is the sweep of the early window alone
    sw = sc.sweep
    ref = batch.impedance(batch.sweep_sums(ser[:n], sw["wavelength_min"], sw["wavelength_max"], 128, 0.5),
                          sw["wavelength_min"], sw["wavelength_max"], 50.0)["z"]
    np.testing.assert_allclose(zt1, ref, rtol=1e-9)
    t = extrap.target(ref, far)
    np.testing.assert_allclose(extrap.to_z(t), np.clip(ref.real, -1000, 1000) +
                               1j * np.clip(ref.imag, -1000, 1000), rtol=1e-5)
    np.testing.assert_allclose(extrap.to_far(t), far, rtol=1e-5)


def test_record_keeps_what_features_read():
    """A run's record (no material arrays) gives the same features as the scene itself, and runs
    that did not ring down are dropped."""
    from types import SimpleNamespace as NS
    sc = configs.batched_scene(4, 1)
    n = extrap.early_steps(sc)
    k = np.arange(n + 200)
    ser = np.stack([np.sin(k * 0.05), 0.02 * np.cos(k * 0.05)], axis=1).astype(np.float32)
    z = np.full(extrap.NF, 50.0 + 10.0j)
    fe, ff = np.full((2, extrap.NFF), 1.5), np.full((2, extrap.NFF), 2.0)
    far = {n: fe, ser.shape[0]: ff}
    done = NS(done=True, rung_down=True, sweep={"z": z}, series=[ser[:100], ser[100:]], far=far)
    q = extrap.record(sc, done)
    assert q is not None and q.series.shape == ser.shape and q.far_final is ff
    for a, b in zip(extrap.features(q, q.series, fe), extrap.features(sc, ser, fe)):
        np.testing.assert_array_equal(a, b)
    assert extrap.record(sc, NS(done=True, rung_down=False, sweep={"z": z}, series=[ser], far=far)) is None
    x, zt, t, ztr, zc, ftr, fc = extrap.dataset_of([q, q])
    assert x.shape == (2, extrap.T_IN, 2) and t.shape == (2, extrap.OUT) and np.array_equal(zc[0], z)
    assert np.array_equal(ftr[0], fe) and np.array_equal(fc[1], ff)
    short = extrap.record(sc, NS(done=True, rung_down=True, sweep={"z": z}, series=[ser[: n - 1]], far=far))
    assert extrap.dataset_of([short]) is None
    # a run without the early window's far-field snapshot is not a sample of that window
    bare = extrap.record(sc, NS(done=True, rung_down=True, sweep={"z": z}, series=[ser], far={ser.shape[0]: ff}))
    assert extrap.dataset_of([bare]) is None


def test_ensemble_spread_and_fallback_threshold():
    """Spread = band median of the largest member deviation from the mean; the threshold is the
    largest that keeps the p90 (over all scenes, fallback scenes counting 0) of |dZ| <= 2 % and of
    the S11 error <= 0.5 dB."""
    from types import SimpleNamespace as NS
    rng = np.random.default_rng(3)
    y = rng.standard_normal((5, extrap.OUT)).astype(np.float32) * 0.3 + 1.0
    nets = [NS(predict=lambda x, zt, d=d: y * np.float32(1.0 + d)) for d in (-0.01, 0.0, 0.01)]
    zm, spread, fm = extrap.ensemble_predict(nets, None, None)
    np.testing.assert_allclose(zm, extrap.to_z(y), rtol=1e-6)
    np.testing.assert_allclose(fm, extrap.to_far(y), rtol=1e-6)
    np.testing.assert_allclose(spread, 0.01, rtol=1e-3)
    # 20 scenes: errors grow with spread; scenes 14.. exceed 2 %
    spread = np.linspace(0.001, 0.02, 20)
    dz = spread * 1.5
    ds11 = np.full(20, 0.1)
    tau = extrap.select_threshold(spread, dz, ds11)
    acc = spread <= tau
    assert np.percentile(np.where(acc, dz, 0.0), 90) <= 0.02
    nxt = spread[spread > tau]
    if nxt.size:  # the next threshold up would break the bound
        acc2 = spread <= nxt.min()
        assert np.percentile(np.where(acc2, dz, 0.0), 90) > 0.02
    # every accepted scene 25x over: the interpolated p90 of 20 values lies between the 18th and
    # 19th largest, so only the lowest-spread scene can be accepted; of 5 values, none
    assert extrap.select_threshold(spread, np.full(20, 0.5), ds11) == spread[0]
    assert extrap.select_threshold(spread[:5], np.full(5, 0.5), ds11[:5]) == -np.inf
    assert extrap.select_threshold(spread, dz * 0.0, ds11) == spread.max()
