"""The adaptive array's host arithmetic: the reference's random numbers (MT19937 and the polar
normal generator), the small complex solver, MVDR weights nulling a jammer, and the scene script."""
import math
import os

import numpy as np
import pytest

from em_lab_gb300 import crpa
from em_lab_gb300.script import ScriptEngine


def test_mt19937_known_answers():
    g = crpa.MT19937(5489)  # the default seed
    first = g.next32()
    assert first == 3499211612
    for _ in range(9998):
        g.next32()
    assert g.next32() == 4123659995  # the 10000th output of a default-constructed mt19937
    rs = np.random.RandomState(7)  # NumPy's legacy generator is the same twister with init_genrand seeding
    h = crpa.MT19937(7)
    raw = np.random.MT19937()
    raw.state = {"bit_generator": "MT19937", "state": {"key": rs.get_state()[1], "pos": rs.get_state()[2]}}
    assert [h.next32() for _ in range(1000)] == [int(v) for v in raw.random_raw(1000)]


def test_polar_normals_are_standard_and_paired():
    n = crpa.Normal(crpa.MT19937(1), 0.0, math.sqrt(0.5))
    x = np.array([n() for _ in range(20000)])
    assert abs(x.mean()) < 0.02 and abs(x.var() - 0.5) < 0.02
    # two draws of 32 bits per uniform, two uniforms per pair: the second value comes from the cache
    g = crpa.MT19937(3)
    u = [g.canonical() for _ in range(2)]
    a, b = 2 * u[0] - 1, 2 * u[1] - 1
    r2 = a * a + b * b
    m = crpa.Normal(crpa.MT19937(3))
    if r2 <= 1.0:
        mult = math.sqrt(-2 * math.log(r2) / r2)
        assert m() == pytest.approx(b * mult, abs=0) and m() == pytest.approx(a * mult, abs=0)


def test_solver_and_mvdr_null():
    rng = np.random.default_rng(2)
    A = rng.standard_normal((5, 5)) + 1j * rng.standard_normal((5, 5))
    b = rng.standard_normal(5) + 1j * rng.standard_normal(5)
    np.testing.assert_allclose(crpa.solve(A.ravel(), b, 5), np.linalg.solve(A, b), rtol=1e-10)
    # a 4-element array: a strong jammer and a weak satellite; MVDR keeps unit gain on the satellite
    k = 2 * math.pi / 20
    pos = np.array([[0, 0], [10, 0], [0, 10], [10, 10]], float)

    def steer(az):
        u = np.array([math.sin(az), math.cos(az)])
        return np.exp(1j * k * pos @ u)
    s, j = steer(0.3), steer(1.4)
    R = np.eye(4) + 1e4 * np.outer(j, j.conj()) + 1e-2 * np.outer(s, s.conj())
    Ria = crpa.solve(R.ravel(), s, 4)
    w = Ria / np.vdot(s, Ria)
    assert abs(np.vdot(w, s)) == pytest.approx(1.0, rel=1e-9)
    assert abs(np.vdot(w, j)) ** 2 < 1e-6


def test_crpa_scene_script():
    from oracle.build_ref import reference_root
    root = reference_root()
    ref = os.path.join(str(root), "scenes", "17_crpa_gps.lua") if root else ""
    if not os.path.exists(ref):
        pytest.skip("reference tree not present")
    sc = ScriptEngine(echo=False).run_file(ref).scene
    assert sc.crpa["satellite"] == "GPS" and len(sc.crpa["elements"]) == 4
    assert [e["name"] for e in sc.emitters][0] == "GPS" and sc.emitters[0]["polarization"] == "rhcp"
    gps = [s for s in sc.sources if s.emitter == 0]
    assert len(gps) == 2 and abs(gps[0].phase - gps[1].phase) == pytest.approx(math.pi / 2, abs=1e-6)
