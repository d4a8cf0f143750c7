"""The headless runner on the GPU: scene scripts stepped frame by frame with the reference's
report, and the report's readings against the oracle stepping the same scene."""
import os

import numpy as np
import pytest

import oracle
from em_lab_gb300 import headless
from em_lab_gb300.instruments import Instruments
from em_lab_gb300.script import ScriptEngine

pytestmark = pytest.mark.gpu
SCENES = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "em_lab_gb300", "scenes")


def test_sphere_dipole_report_matches_oracle(capsys):
    path = os.path.join(SCENES, "sphere_dipole.lua")
    code, inst = headless.run(path, 100)
    out = capsys.readouterr().out
    assert code == 0
    assert "=== Dipole beside a dielectric sphere ===  (sphere_dipole.lua)" in out
    assert "Grid 128x128x128 (2.1 M cells" in out and "1 source term(s)" in out
    assert "[t=   100.0 step     200]" in out
    assert "probe behind" in out and "flux  radiated" in out and "far field [lambda=16.0 cells" in out
    # the same scene stepped by the oracle, measured through the same host arithmetic
    sc = ScriptEngine(echo=False).run_file(path).scene
    o = oracle.Oracle(sc.grid, "f32")
    oracle.load_scene(o, sc)
    o.ntff_configure(sc.far_field["box_min"], sc.far_field["box_max"], sc.far_field["wavelength"],
                     sc.far_field["averaging"])
    o.step(200)

    class OracleGrid:
        def __getattr__(self, k):
            return getattr(o, k)

        def time(self):
            return 100.0

        def step_count(self):
            return 200
    ref = Instruments(OracleGrid(), sc, out=lambda s: None)
    ref.measure()
    assert ref.probes[0]["sample"] == inst.probes[0]["sample"]
    assert ref.fluxes[0]["inst"] == inst.fluxes[0]["inst"]


def test_fed_dipole_sweep_report(capsys):
    code, inst = headless.run(os.path.join(SCENES, "fed_dipole.lua"), 300, {"length": "17"})
    out = capsys.readouterr().out
    assert code == 0
    assert "Parameters:" in out and "= 17" in out
    assert "sweep: 600 steps recorded" in out and "sweep feed" in out and "best match" in out
    ps = inst.sweep_result["ports"][0]
    assert 20.0 < ps["best_wl"] < 60.0


def test_slit_wall_flux_plane(capsys):
    code, inst = headless.run(os.path.join(SCENES, "slit_wall.lua"), 120)
    out = capsys.readouterr().out
    assert code == 0
    assert "flux  transmitted" in out and "probe slit1" in out and "probe screen" in out
    assert np.isfinite(inst.fluxes[0]["inst"])


def test_coax_matched_line_measures_z0(capsys):
    code, inst = headless.run(os.path.join(SCENES, "coax_load.lua"), 200)
    out = capsys.readouterr().out
    assert code == 0
    assert "cable: Z0 50.0 ohm" in out and "waves: Z0 measured" in out
    r = inst.coax_readings[0]
    assert r["valid"]
    assert abs(r["z0m"] - 50.0) < 2.5            # the line's own V+/I+ against the lattice Z0
    assert abs(r["gamma"]) < 0.1                 # matched resistive load at the far end


def test_screenshot_of_last_frame(tmp_path, capsys):
    """--screenshot: the last frame ray-marched on the GPU and saved as a 24-bit BMP."""
    shot = tmp_path / "frame.bmp"
    code = headless.main(["--script", os.path.join(SCENES, "sphere_dipole.lua"), "--frames", "30",
                          "--screenshot", str(shot), "--width", "161", "--height", "90"])
    out = capsys.readouterr().out
    assert code == 0 and f"Saved screenshot {shot}" in out
    data = shot.read_bytes()
    row = (161 * 3 + 3) & ~3
    assert data[:2] == b"BM" and len(data) == 54 + 90 * row
    pix = np.frombuffer(data[54:], np.uint8).reshape(90, row)[:, :161 * 3].reshape(90, 161, 3)
    # the dipole's field glows over the dark background: some pixels are far brighter than the corner
    assert int(pix.max()) >= int(pix[0, 0].max()) + 30
    assert "render 0.000 ms" not in out
