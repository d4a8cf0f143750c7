"""The opt-in convolutional PML on the GPU (csrc/cpml.cu) against its CPU restatement: fields bit for
bit after many steps on seeded scenes with lossy dielectrics, thin wires, feeds and sources reaching
into the absorber; the FP64 error stated; the reflection measured against the reference's graded
absorber on the GPU; switching back restores the reference absorber exactly."""
import numpy as np
import pytest

import oracle
from em_lab_gb300 import SimulationGrid, abi, configs, scene

pytestmark = pytest.mark.gpu
DEFAULT = (3.2, 1.0, 0.05, 3.0)


@pytest.mark.parametrize("seed,size,pml,params", [(1, (40, 34, 30), 6, DEFAULT), (2, (33, 41, 27), 4, (2.0, 4.0, 0.1, 2.0)),
                                                  (3, (64, 48, 40), 8, DEFAULT)])
def test_cpml_bit_exact_against_the_restatement(seed, size, pml, params):
    sc = configs.random_scene(size=size, pml=pml, seed=seed)
    out = {}
    for label, t in (("gpu", SimulationGrid(sc.grid)), ("f32", oracle.Oracle(sc.grid, "f32")),
                     ("f64", oracle.Oracle(sc.grid, "f64"))):
        t.set_cpml(params)
        oracle.load_scene(t, sc)
        t.step(150)
        out[label] = t.read_components()
        t.close()
    for c in range(6):
        assert np.array_equal(out["gpu"][c], out["f32"][c]), c
        b = out["f64"][c]
        rel = np.linalg.norm(out["gpu"][c].astype(np.float64) - b) / np.linalg.norm(b)
        print(f"CPML seed {seed} component {c}: relative L2 vs FP64 restatement {rel:.2e}")
        assert rel < 1e-5


def pulse_fields(size, L, cpml, times):
    g = SimulationGrid(abi.GridConfig((size,) * 3, courant=0.5, pml_thickness=L))
    if cpml:
        g.set_cpml(cpml)
    c = size / 2
    g.set_sources([scene.SourceDesc(center=(c, c, c), polarization=(0, 0, 1), wavelength=12.0,
                                    waveform=abi.WAVE_PULSE, ramp_periods=0.5, amplitude=1.0)])
    out, prev = [], 0
    for t in times:
        g.step(t - prev)
        prev = t
        out.append(g.read_components())
    g.close()
    return out


def test_cpml_reflection_against_the_graded_absorber():
    """A pulsed dipole in a 64^3 grid with an 8-cell absorber against the same region of a 224^3
    grid (nothing returns from its boundary in the window): the convolutional PML's reflection is
    below 5e-4 of the peak field and more than 50 times below the graded absorber's."""
    times = list(range(20, 141, 10))
    small, big, L = 64, 224, 8
    ref = pulse_fields(big, L, None, times)
    off = (big - small) // 2
    lo, hi = L + 1, small - L - 1

    def cut(f, o=0):
        return [a[o + lo:o + hi, o + lo:o + hi, o + lo:o + hi].astype(np.float64) for a in f]
    refc = [cut(f, off) for f in ref]
    peak = max(np.sqrt(sum(np.sum(b ** 2) for b in f)) for f in refc)
    errs = {}
    for name, p in (("graded", None), ("cpml", DEFAULT)):
        got = pulse_fields(small, L, p, times)
        errs[name] = max(np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(cut(f), r))) for f, r in zip(got, refc)) / peak
    print(f"reflection, 8-cell absorber on a 64^3 grid: graded {errs['graded']:.2e}, convolutional PML {errs['cpml']:.2e}")
    assert errs["cpml"] < 5e-4 and errs["cpml"] * 50 < errs["graded"]


def test_switching_back_restores_the_reference_absorber():
    sc = configs.random_scene(size=(36, 30, 28), pml=5, seed=9)
    g = SimulationGrid(sc.grid)
    g.set_cpml(DEFAULT)
    oracle.load_scene(g, sc)
    g.step(40)
    g.set_cpml(None)
    oracle.load_scene(g, sc)
    g.step(60)
    o = oracle.Oracle(sc.grid, "f32")
    oracle.load_scene(o, sc)
    o.step(60)
    for c, (a, b) in enumerate(zip(g.read_components(), o.read_components())):
        assert np.array_equal(a, b), c
    g.close()
    o.close()
