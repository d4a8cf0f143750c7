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
