"""CPU checks of the oracle: its arithmetic primitives, its pin to the reference's own shader code
(oracle/_ref, where the reference tree is present), and the committed golden fixtures."""
import math
import os
import struct

import numpy as np
import pytest

import oracle
from em_lab_gb300 import abi, configs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def f32(x):
    return struct.unpack("f", struct.pack("f", x))[0]


def test_expf_within_two_ulp_and_special_values():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-103, 88.7, 4000), rng.uniform(-1, 1, 2000), rng.uniform(-1e-4, 1e-4, 500)])
    worst = 0.0
    for x in xs.astype(np.float32):
        got = oracle.expf(float(x))
        ref = math.exp(float(x))
        if 1.2e-38 < ref < 3e38:
            ulp = float(np.spacing(np.float32(ref)))
            worst = max(worst, abs(got - ref) / ulp)
    assert worst <= 2.0, worst
    assert oracle.expf(0.0) == 1.0 and oracle.expf(-0.0) == 1.0
    assert oracle.expf(100.0) == math.inf
    assert oracle.expf(-200.0) == 0.0
    assert math.isnan(oracle.expf(math.nan))
    sub = oracle.expf(-100.0)  # subnormal result
    assert 0.0 < sub < 1.2e-38 and abs(sub - math.exp(-100.0)) <= 2 ** -149


def test_half_packing_is_ieee_round_to_nearest_even():
    rng = np.random.default_rng(1)
    vals = np.concatenate([rng.uniform(0, 70000, 3000), rng.uniform(0, 1e-4, 1000), 10 ** rng.uniform(-8, 4.8, 2000),
                           np.array([0.0, 1.0, 2.25, 6.0e4, 65504.0, 65519.0, 65520.0, 1e-8, 2 ** -24, 2 ** -25,
                                     3 * 2 ** -26, 1 + 2 ** -11, 1 + 3 * 2 ** -11])]).astype(np.float32)
    with np.errstate(over="ignore"):
        halves = vals.astype(np.float16).view(np.uint16)
    for v, want in zip(vals, halves):
        want = int(want)
        assert oracle.float_to_half(float(v)) == want, (float(v), want)


def test_fp32_oracle_error_floor():
    sc = configs.random_scene(size=(30, 26, 22), pml=5, seed=9)
    res = {}
    for prec in ("f32", "f64"):
        o = oracle.Oracle(sc.grid, prec)
        oracle.load_scene(o, sc)
        o.step(200)
        res[prec] = o.read_components()
    for a, b in zip(res["f32"], res["f64"]):
        rel = np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b)
        assert rel < 1e-5, rel


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref needs the reference tree (oracle/build_ref.py)")
@pytest.mark.parametrize("seed,size,pml", [(1, (24, 20, 18), 4), (2, (37, 29, 23), 5), (6, (20, 21, 22), 0)])
@pytest.mark.parametrize("exp", ["emlab", "libm"])
def test_oracle_equals_reference_shaders(seed, size, pml, exp):
    """The restatement against the reference's own shader code, every output, bit for bit."""
    import golden.make_golden as mg  # noqa: F401  (same monitor set-up as the fixtures)

    sc = configs.random_scene(size=size, pml=pml, seed=seed)
    a = mg.run(oracle.Oracle(sc.grid, "f32" if exp == "emlab" else "f32libm"), sc, 70)
    b = mg.run(oracle.Oracle(sc.grid, "ref" if exp == "emlab" else "reflibm"), sc, 70)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("name", ["random_s1", "random_s2", "vacuum_pml0"])
def test_oracle_matches_golden_fixtures(name):
    import golden.make_golden as mg

    case = {c[0]: c for c in mg.CASES}[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    sc = configs.random_scene(**case[1])
    out = mg.run(oracle.Oracle(sc.grid, "f32"), sc, int(g["steps"]))
    assert mg.field_hash([out[f"f{c}"] for c in range(6)]) == str(g["sha256"])
    for k in g.files:
        if k in ("steps", "sha256"):
            continue
        if k.startswith("mid"):
            f = out[f"f{k[3:]}"]
            assert np.array_equal(f[f.shape[0] // 2], g[k]), k
        else:
            assert np.array_equal(out[k], g[k]), k


def test_signal_waveforms():
    s = configs.SourceDesc(wavelength=16.0, ramp_periods=3.0)
    assert oracle.source_signal(s, 0.0) == 0.0
    T = 16.0
    t = 5.0 * T + 0.3
    assert abs(oracle.source_signal(s, t) - math.sin(2 * math.pi / T * t)) < 1e-15
    r = 0.5
    ramp = r ** 3 * (10 + r * (-15 + 6 * r))
    assert abs(oracle.source_signal(s, 1.5 * T) - ramp * math.sin(2 * math.pi / T * 1.5 * T)) < 1e-15
    p = configs.SourceDesc(wavelength=20.0, waveform=abi.WAVE_PULSE, ramp_periods=0.5, delay_periods=1.0)
    tau = 10.0
    assert oracle.source_signal(p, 20.0 + 3 * tau) == 0.0  # sin(0) at the packet centre
    assert oracle.source_signal(p, 19.0) == 0.0            # before the delay
    assert oracle.source_signal(p, 20.0 + 3 * tau + 7 * tau) == 0.0  # |u| > 6
