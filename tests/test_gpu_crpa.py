"""The adaptive GPS array end to end on the GPU: measurement passes (or the blind recording), MVDR
weights, and the adapted transmission; MVDR nulls the jammer that plain steering lets through."""
import os

import pytest

from em_lab_gb300 import headless

pytestmark = pytest.mark.gpu
SCENES = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "em_lab_gb300", "scenes")


@pytest.mark.parametrize("adapt", ["ideal", "blind"])
def test_crpa_nulls_the_jammer(adapt, capsys):
    code, inst = headless.run(os.path.join(SCENES, "gps_array.lua"), 500, {"adapt": adapt})
    out = capsys.readouterr().out
    assert code == 0
    c = inst.crpa
    assert c is not None and c.phase == "adapted", out[-2000:]
    r = c.result
    assert r["valid"] and r["blind"] == (adapt == "blind")
    sat = [e for e in r["emitters"] if e["satellite"]][0]
    jam = [e for e in r["emitters"] if not e["satellite"]][0]
    assert r["sinr_mvdr_db"] > r["sinr_steering_db"] + 10.0
    assert jam["output_db"] < jam["steering_out_db"] - 15.0
    assert abs(sat["output_db"] - sat["steering_out_db"]) < 6.0
    assert "crpa (MVDR weights): SINR single element" in out
