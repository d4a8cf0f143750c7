"""The planar phased-array workload on the GPU (reduced size): the beam of a Taylor-tapered,
time-delay-steered array, read from the tensor-core far-field DFT, points where it was steered."""
import pytest

from em_lab_gb300 import phased

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("theta,phi", [(0.0, 0.0), (25.0, 40.0), (30.0, 200.0)])
def test_beam_points_to_the_steering_direction(theta, phi):
    sc = phased.build(theta, phi, elements=8, nxy=192, nz=128)
    r = phased.run_scene(sc, 1400, n_theta=91, n_phi=181, freqs=[])
    assert r["finite"]
    err = phased.angular_error(r["beam_theta"], r["beam_phi"], theta, phi)
    assert err < 6.0, (r["beam_theta"], r["beam_phi"])


def test_cropped_array_bit_exact_against_the_oracle():
    """The phased-array scene itself (thin-wire dipoles with 50-ohm Taylor-tapered, time-delay-
    steered feeds, the PEC ground sheet, the radome slab, the 12-cell absorber) as a 4 x 4 subarray
    on a 128 x 128 x 96 grid: fields and every feed's (V, I) series bit-identical to the FP32
    oracle after 600 steps, the FP64 error of each field component stated."""
    import numpy as np
    import oracle
    from em_lab_gb300 import SimulationGrid
    sc = phased.build(25.0, 40.0, elements=4, nxy=128, nz=96)
    assert len(sc.ports) == 16
    ports = [p.to_c() for p in sc.ports]
    steps = 600
    oracle.set_threads(oracle.max_threads())
    out = {}
    for label, t in (("gpu", SimulationGrid(sc.grid)), ("f32", oracle.Oracle(sc.grid, "f32")),
                     ("f64", oracle.Oracle(sc.grid, "f64"))):
        oracle.load_scene(t, sc)
        t.ports_configure(ports, sc.wavelength, 4.0, False, steps)
        t.step(steps)
        out[label] = (t.read_components(), np.asarray(t.ports_series()))
        t.close()
    (fg, sg), (fo, so), (fd, _) = out["gpu"], out["f32"], out["f64"]
    for c in range(6):
        assert np.array_equal(fg[c], fo[c]), c
        rel = np.linalg.norm(fg[c].astype(np.float64) - fd[c]) / np.linalg.norm(fd[c])
        print(f"phased array crop, component {c}: relative L2 vs FP64 oracle {rel:.2e}")
        assert rel < 1e-4
    assert sg.shape == so.shape and np.array_equal(sg, so)
    assert np.abs(sg).max() > 0
