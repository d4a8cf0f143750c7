"""The opt-in convolutional PML in the CPU restatement (oracle/oracle_impl.h): its FP32 and FP64
instances agree to the FP32 error floor, and it absorbs a pulse far better than the reference's
graded absorber of the same thickness. (The GPU kernels are checked against this restatement bit
for bit in tests/test_gpu_cpml.py.)"""
import numpy as np

import oracle
from em_lab_gb300 import abi, configs, scene

DEFAULT = (3.2, 1.0, 0.05, 3.0)  # sigma_max = 0.8 (m + 1), kappa_max, alpha_max, m


def pulse_run(size, L, cpml, times, prec="f64"):
    o = oracle.Oracle(abi.GridConfig((size,) * 3, courant=0.5, pml_thickness=L), prec)
    if cpml:
        o.set_cpml(cpml)
    c = size / 2
    o.set_sources([scene.SourceDesc(center=(c, c, c), polarization=(0, 0, 1), wavelength=12.0,
                                    waveform=abi.WAVE_PULSE, ramp_periods=0.5, amplitude=1.0)])
    out, prev = [], 0
    for t in times:
        o.step(t - prev)
        prev = t
        out.append(o.read_components())
    o.close()
    return out


def reflection(small, big, L, cpml, times):
    """Largest deviation over `times` of the small grid's interior from the same region of a grid
    large enough that nothing returns from its boundary in that time, relative to the largest
    field norm there: the absorber's reflection."""
    ref = pulse_run(big, L, None, times)
    off = (big - small) // 2
    lo, hi = L + 1, small - L - 1

    def cut(f, o=0):
        return [a[o + lo:o + hi, o + lo:o + hi, o + lo:o + hi] for a in f]
    refc = [cut(f, off) for f in ref]
    peak = max(np.sqrt(sum(np.sum(b.astype(np.float64) ** 2) for b in f)) for f in refc)
    got = pulse_run(small, L, cpml, times)
    return max(np.sqrt(sum(np.sum((a.astype(np.float64) - b) ** 2) for a, b in zip(cut(f), r)))
               for f, r in zip(got, refc)) / peak


def test_cpml_absorbs_far_better_than_the_graded_absorber():
    oracle.set_threads(oracle.max_threads())
    times = list(range(20, 101, 10))  # the pulse reaches the absorber and is gone from the interior
    graded = reflection(40, 120, 8, None, times)
    cpml = reflection(40, 120, 8, DEFAULT, times)
    print(f"reflection, 8-cell absorber: graded {graded:.2e}, convolutional PML {cpml:.2e}")
    assert cpml < 5e-4 and cpml * 50 < graded


def test_cpml_fp32_against_fp64():
    sc = configs.random_scene(size=(30, 26, 24), pml=5, seed=3)
    out = []
    for prec in ("f32", "f64"):
        o = oracle.Oracle(sc.grid, prec)
        o.set_cpml(DEFAULT)
        oracle.load_scene(o, sc)
        o.step(120)
        out.append(o.read_components())
        o.close()
    for c, (a, b) in enumerate(zip(*out)):
        rel = np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b)
        assert rel < 1e-5, (c, rel)
