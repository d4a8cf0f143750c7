"""Scene scripts through the scene API: the solver inputs a script produces (materials, edge
overrides, thin-wire terms, sources, ports and monitors) against the same scene built directly
with the scene builder, plus the API's validation and error messages."""
import os
import re

import numpy as np
import pytest

from em_lab_gb300 import abi, configs
from em_lab_gb300.scene import EnvironmentBuilder, SourceDesc
from em_lab_gb300.script import ScriptEngine, ScriptError

SCENES = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "em_lab_gb300", "scenes")


def run(src, overrides=None):
    return ScriptEngine(overrides, echo=False).run_source(src, "test.lua")


def edge_list(sc):
    return sorted((e.x, e.y, e.z, e.axis, e.sigma) for e in sc.edges)


def wire_list(sc):
    return sorted((w.x, w.y, w.z, w.component, w.term, w.factor) for w in sc.wires)


def src_tuple(s):
    return (s.center, s.half_extent, s.softness, s.polarization, s.amplitude, s.wavelength, s.phase, s.waveform,
            s.ramp_periods, s.repeat_periods, s.delay_periods, s.enabled)


def test_sphere_dipole_script_equals_plain_small_config():
    res = ScriptEngine(echo=False).run_file(os.path.join(SCENES, "sphere_dipole.lua"))
    a, b = res.scene, configs.plain_small()
    assert a.grid.size == b.grid.size and a.grid.pml_thickness == b.grid.pml_thickness
    assert a.grid.courant == b.grid.courant
    assert np.array_equal(a.materials.sigma, b.materials.sigma)
    assert np.array_equal(a.materials.epsilon_r, b.materials.epsilon_r)
    assert [src_tuple(s) for s in a.sources] == [src_tuple(s) for s in b.sources]
    assert [p[1] for p in a.probes] == [p[1] for p in b.probes]
    assert (a.fluxes[0].box_min, a.fluxes[0].box_max) == (b.fluxes[0].box_min, b.fluxes[0].box_max)
    for k in ("box_min", "box_max", "wavelength", "averaging"):
        assert tuple(np.atleast_1d(a.far_field[k])) == tuple(np.atleast_1d(b.far_field[k])), k


def test_fed_dipole_script_equals_builder():
    res = ScriptEngine({"length": "21"}, echo=False).run_file(os.path.join(SCENES, "fed_dipole.lua"))
    a = res.scene
    grid = abi.GridConfig((96, 96, 112), courant=0.5, pml_thickness=12)
    b = EnvironmentBuilder("ref", grid, wavelength=32.0)
    wave = SourceDesc(wavelength=32.0, waveform=abi.WAVE_PULSE, ramp_periods=float(np.float32(0.4)))
    b.thin_dipole(wave, (48.0, 48.0, 56.0), 2, 21, radius=float(np.float32(0.08)), name="feed")
    b = b.build()
    assert edge_list(a) == edge_list(b)
    assert wire_list(a) == wire_list(b)
    assert [src_tuple(s) for s in a.sources] == [src_tuple(s) for s in b.sources]
    assert [(p.texel, p.axis, p.edges, p.name) for p in a.ports] == [(p.texel, p.axis, p.edges, p.name) for p in b.ports]
    assert a.sweep == {"wavelength_min": 20.0, "wavelength_max": 60.0, "points": 64, "log": ""}
    assert [p.value for p in res.params] == [21.0, 0.08]


def test_geometry_primitives_voxelise_like_the_builder():
    res = run("""
        scene { size = {48, 40, 36}, pml = 4, wavelength = 20 }
        box { min = {10, 10, 10}, max = {20, 18, 16}, material = { name = "d", epsilon_r = 3 } }
        sphere { center = {30, 20, 20}, radius = {5, 4, 3}, material = "fr4" }
        cylinder { center = {24, 30, 18}, axis = "x", radius = 3, length = 12, thickness = 1, material = "pec" }
        box { center = {36, 12, 24}, size = 6, rotate = {0, 0, 45}, material = "glass" }
        shape { min = {4, 4, 4}, max = {12, 12, 12}, inside = function(x, y, z) return x + y < 16 end, material = "water" }
    """)
    sc = res.scene
    mats = sc.materials
    assert mats.epsilon_r[12, 12, 12] == np.float32(3.0)            # inside the first box
    assert mats.epsilon_r[9, 12, 12] == 1.0                           # just outside (z = 9)
    assert mats.epsilon_r[20, 20, 30] == np.float32(4.4)              # ellipsoid centre, fr4
    assert mats.sigma[18, 30, 24] == 0.0                              # hollow tube inside
    assert mats.sigma[18, 30 + 2, 24] == np.float32(1e7)              # tube wall (pec)
    assert mats.epsilon_r[24, 12, 36] == np.float32(6.3)              # rotated cube centre
    assert mats.epsilon_r[5, 5, 5] == np.float32(78.0) and mats.epsilon_r[5, 11, 11] == 1.0  # predicate shape


def test_wall_slits_and_plane_wave():
    res = ScriptEngine({"spacing": "16"}, echo=False).run_file(os.path.join(SCENES, "slit_wall.lua"))
    sc = res.scene
    s = sc.materials.sigma
    # [z, y, x]: slits of width 6 centred at y = 48 -+ 8 in the wall at x = 48..49; metal elsewhere
    assert s[32, 40, 48] == 0.0 and s[32, 56, 49] == 0.0
    assert s[32, 48, 48] > 1e6 and s[32, 36, 48] > 1e6 and s[32, 40, 50] == 0.0
    assert len(sc.sources) == 2                                   # one-way sheet: two quarter-wave-spaced sheets
    assert sc.sources[1].center[0] - sc.sources[0].center[0] == pytest.approx(4.0)
    assert sc.sources[1].delay_periods == pytest.approx(0.25)
    assert [f.kind for f in sc.fluxes] == ["plane"] and sc.fluxes[0].rect_min == (10, 10)


def test_array_and_cage():
    res = run("""
        scene { size = {96, 96, 64}, pml = 8, wavelength = 24 }
        array { elements = {2, 3}, spacing = 12, length = 11, steer = {10, 0}, taper = "hann", name = "ant" }
        cage { min = {10, 10, 10}, max = {30, 30, 30}, spacing = 5, bar = 1, material = "pec" }
    """)
    sc = res.scene
    assert len(sc.ports) == 6 and sc.ports[0].name == "ant[0,0]"
    assert len({s.phase for s in sc.sources}) == 2                 # progressive phase along the steered axis
    assert sc.materials.sigma[10, 10, 10] > 0 and sc.materials.sigma[12, 12, 10] == 0


@pytest.mark.parametrize("src,msg", [
    ("box { min = {1, 1, 1}, max = {2, 2, 2}, material = 'unobtainium' }", "unknown material 'unobtainium'"),
    ("box { min = {1, 1, 1} }", "missing required vector 'max'"),
    ("probe { position = 'here' }", "'position' must be a 3-vector"),
    ("box { min = {1, 1, 1}, max = {2, 2, 2} } scene { size = 64 }", "scene{} must be the first call"),
    ("scene { size = 8 }", "size must be at least 16 cells"),
    ("scene { courant = 0.6 }", "courant must be < 1/sqrt(3)"),
    ("dipole { length = 4 }", "thin-wire dipole needs length >= 5"),
    ("wire { from = {1, 1, 1}, to = {2, 2, 1} }", "differ along exactly one axis"),
    ("loop { size = 1 }", "a thin-wire loop needs size >= 2 cells"),
    ("loop { size = 2, model = 'rod' }", "a rod loop needs size >= 3 cells"),
    ("frame { min = {1, 1, 1}, max = {9, 9, 9}, bar = 0 }", "'bar' must be > 0"),
    ("radar { taper = 'kaiser' }", "taper must be \"uniform\", \"hamming\" or \"hann\""),
    ("view { mode = 'poyntng' }", "mode must be one of \"fields\", \"e\", \"b\", \"poynting\", \"signed\" "
                                  "(did you mean 'poynting'?)"),
    ("box { min = {1, 1, 1}, max = {2, 2, 2}, material = 'coper' }", "unknown material 'coper' (did you mean 'copper'?)"),
    ("local v = vec(1, 2, 3) + 'x'", "arithmetic"),
])
def test_errors(src, msg):
    with pytest.raises(ScriptError, match=re.escape(msg)):
        run(src)


def test_vector_prelude_and_grid_globals():
    res = run("""
        scene { size = {64, 48, 32}, pml = 6, wavelength = 20, cell_size = 0.002 }
        local a = vec(1, 2, 3)
        local b = a * 2 + 1 - vec(1)
        print(tostring(b), b.x, b:length() > 0, a:dot(X), tostring(a:cross(Y)), tostring(a:with('z', 9)))
        print(tostring(grid.center), grid.nx, grid.pml, grid.wavelength, deg(180), wavelengths(2), mm(4), lerp(1, 3, 0.5))
        local n = 0
        for x in range(0, 1, 0.25) do n = n + 1 end
        print(n, clamp(5, 0, 3), tostring(-a), a == vec(1, 2, 3))
    """)
    assert res.output == ["vec(2, 4, 6)\t2\ttrue\t1\tvec(-3, 0, 1)\tvec(1, 2, 9)",
                          # cell_size is the float32 value, as the reference exposes it
                          "vec(32, 24, 16)\t64\t6\t20.0\t3.1415926535898\t40.0\t1.9999999050051\t2.0",
                          "5\t3\tvec(-1, -2, -3)\ttrue"]


def test_warnings():
    res = run("""
        scene { size = 48, pml = 6 }
        probe { position = {2, 20, 20} }
        box { min = {0, 0, 0}, max = {4, 4, 4}, colour = 'red' }
        monopole { base = {24, 24, 24}, length = 6 }
    """)
    w = " | ".join(res.warnings)
    assert "unknown field 'colour'" in w
    assert "lies inside the absorbing boundary layer" in w
    assert "no conductor touches the base of the feed gap" in w


def test_view_hints():
    res = run("""
        scene { size = 48 }
        view { mode = "Signed", component = "y", gain = 3, gain_b = 5, exposure = 2, density = 0.5, step = 0.4,
               metal_opacity = 1.7, steps_per_frame = 300, distance = 2, yaw = 10, target = {1, 2, 3}, overlay = false }
        view { pitch = 45 }
    """)
    v = res.scene.view
    assert v["mode"] == 4 and v["component"] == 1
    assert (v["gain_e"], v["gain_b"], v["exposure"], v["density"], v["step"]) == (3.0, 5.0, 2.0, 0.5, 0.4)
    assert v["metal_opacity"] == 1.0 and v["steps_per_frame"] == 64
    assert (v["distance"], v["yaw"], v["pitch"], v["target"], v["overlay"]) == (2.0, 10.0, 45.0, (1.0, 2.0, 3.0), False)
    res = run("scene { size = 48 } view { colour = 1 }")
    assert "view: unknown field 'colour' ignored" in " | ".join(res.warnings)


def test_coax_builder_and_monitor_layout():
    from em_lab_gb300.instruments import Instruments
    from em_lab_gb300.script import coax_geometry_factor
    assert coax_geometry_factor(1, 5) == pytest.approx(4.8, abs=1e-12)   # square lattice coax, 5-cell shield
    res = ScriptEngine(echo=False).run_file(os.path.join(SCENES, "coax_load.lua"))
    sc = res.scene
    c = sc.coaxes[0]
    assert c.z0_ohm == pytest.approx(50.0, rel=1e-6) and c.epsilon_r == pytest.approx((376.730313668 / 4.8 / 50) ** 2, rel=1e-6)
    assert len(sc.ports) == 2 and [p.name for p in sc.ports] == ["cable", "cable load"]
    assert res.output[0].startswith("coax: Z0 50.00 ohm")
    m = sc.materials
    assert m.sigma[20, 20, 20 + 60] > 1e5 and m.epsilon_r[20, 21, 20 + 60] == np.float32(c.epsilon_r)  # inner / dielectric

    class Grid:
        def time(self):
            return 0.0

        def dt(self):
            return 0.5

        def lines_configure(self, q, t, w, wl, avg):
            self.q, self.t, self.w = q, t, w

        def ports_configure(self, *a, **k):
            pass
    g = Grid()
    Instruments(g, sc, out=lambda s: None)
    assert len(g.q) == 3 * (c.length - 1)
    kinds = [q[2] for q in g.q[:3]]
    assert kinds == [0, 1, 1]
    assert g.q[0][1] == 4 * 2 * 2 and g.q[1][1] == 8     # V: 4 sides x 2 node rows x 2 cells; I: 8 B terms


def test_frame_builds_the_twelve_edges_of_a_box():
    """frame{} (ScriptEngine.cpp:1022-1030, Environment.cpp:111-127): bars `bar` cells thick along the
    twelve edges of the box; faces and interior stay empty."""
    sc = run("""
        scene { size = 48, pml = 4 }
        frame { min = {10, 12, 14}, max = {30, 28, 34}, bar = 2, material = "pec" }
    """).scene
    sig = sc.materials.sigma  # (z, y, x)
    metal = sig > 0
    assert metal[14, 12, 10] and metal[33, 27, 29] and metal[20, 12, 10] and metal[14, 20, 29]
    assert not metal[20, 20, 20] and not metal[20, 20, 10] and not metal[14, 20, 20]
    # each edge bar: 2 x 2 cells across; edge lengths 20, 16, 20: 4 bars each, corners shared
    onx = np.isin(np.arange(48), [10, 11, 28, 29])
    ony = np.isin(np.arange(48), [12, 13, 26, 27])
    onz = np.isin(np.arange(48), [14, 15, 32, 33])
    inx = (np.arange(48) >= 10) & (np.arange(48) < 30)
    iny = (np.arange(48) >= 12) & (np.arange(48) < 28)
    inz = (np.arange(48) >= 14) & (np.arange(48) < 34)
    Z, Y, X = np.meshgrid(np.arange(48), np.arange(48), np.arange(48), indexing="ij")
    edge = inx[X] & iny[Y] & inz[Z] & ((onx[X] & ony[Y]) | (ony[Y] & onz[Z]) | (onx[X] & onz[Z]))
    np.testing.assert_array_equal(metal, edge)


def test_loop_models():
    """loop{} (ScriptEngine.cpp:1456-1524): thin-wire square fed across one edge of the -v side, a ring
    of rods with a four-edge gap, or four ideal current segments counter-clockwise about +normal."""
    thin = run("""
        scene { size = 48, pml = 4, wavelength = 24 }
        loop { center = {24, 24, 24}, normal = "z", size = 8, radius = 0.1 }
    """).scene
    assert len(thin.ports) == 1 and thin.ports[0].axis == 0 and thin.ports[0].edges == 1
    p = thin.ports[0]
    assert tuple(p.texel) == (24, 20, 24)      # the middle of the -y side (u = x, v = y)
    assert len(thin.wires) > 0 and all(w.z == 24 or w.z == 23 for w in thin.wires)
    rod = run("""
        scene { size = 48, pml = 4, wavelength = 24 }
        loop { center = {24, 24, 24}, normal = "x", size = 6, model = "rod" }
    """).scene
    assert len(rod.ports) == 1 and rod.ports[0].edges == 4 and rod.ports[0].axis == 1
    metal = rod.materials.sigma > 0  # (z, y, x): the ring lies in the plane x = 24
    assert metal[:, :, 24].sum() == 4 * 6 - 4 - 1 and not metal[:, :, 23].any()
    ideal = run("""
        scene { size = 48, pml = 4, wavelength = 24 }
        loop { center = {24, 24, 24}, normal = "z", size = 8, model = "current", amplitude = 2 }
    """).scene
    assert len(ideal.sources) == 4 and not ideal.ports
    cs = sorted((tuple(round(v, 3) for v in s.center), tuple(round(v, 3) for v in s.polarization)) for s in ideal.sources)
    assert cs == sorted([((24.0, 20.0, 24.0), (1.0, 0.0, 0.0)), ((28.0, 24.0, 24.0), (0.0, 1.0, 0.0)),
                         ((24.0, 28.0, 24.0), (-1.0, 0.0, 0.0)), ((20.0, 24.0, 24.0), (0.0, -1.0, 0.0))])
