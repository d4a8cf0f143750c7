"""The reference's bundled scene scripts, built by this package's Lua interpreter and scene API.

tests/golden/scenes/ holds the result of every bundled script (scenes/*.lua, scenes/validation/*.lua,
plus the parameter settings the validation headers quote), written by make_scenes.py from the
reference tree. Here: every saved scene loads back to the digest recorded when it was built; where
the reference tree is present, every script is built again and must give the recorded digest (the
interpreter, the scene API and the voxeliser reproduce their own earlier output bit for bit). The
GPU half (tests/test_gpu_scenes.py) runs the saved scenes headless and checks the results the
reference quotes.
"""
import json
import os

import numpy as np
import pytest

from em_lab_gb300 import headless, scene_io

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scenes")
TABLE = json.load(open(os.path.join(HERE, "digests.json")))

BUNDLED = 21  # scenes/*.lua (18) and scenes/validation/*.lua (3) in the reference tree


def test_every_bundled_script_has_a_fixture():
    scripts = {v["script"] for v in TABLE.values()}
    assert len(scripts) == BUNDLED
    assert sum(1 for v in TABLE.values() if not v["overrides"]) == BUNDLED
    for name in TABLE:
        assert os.path.exists(os.path.join(HERE, name + ".npz")), name


@pytest.mark.parametrize("name", sorted(TABLE))
def test_saved_scene_loads_to_its_digest(name):
    res = scene_io.load(os.path.join(HERE, name + ".npz"))
    assert scene_io.digest(res) == TABLE[name]["digest"]
    assert scene_io.summary(res) == TABLE[name]["summary"]


def _tree():
    from oracle.build_ref import reference_root
    root = reference_root()
    return str(root) if root and os.path.isdir(os.path.join(str(root), "scenes")) else None


@pytest.mark.parametrize("name", sorted(TABLE))
def test_script_rebuilds_to_the_saved_scene(name):
    tree = _tree()
    if tree is None:
        pytest.skip("reference tree not available (set EMLAB_REFERENCE)")
    from em_lab_gb300.script import ScriptEngine
    entry = TABLE[name]
    res = ScriptEngine(dict(entry["overrides"]), echo=False).run_file(os.path.join(tree, entry["script"]))
    assert scene_io.digest(res) == entry["digest"]


def test_round_trip_keeps_every_solver_input():
    res = scene_io.load(os.path.join(HERE, "04_dipole.npz"))
    again = scene_io.load_bytes(scene_io.to_bytes(res))
    a, b = res.scene, again.scene
    assert np.array_equal(a.materials.sigma, b.materials.sigma)
    assert np.array_equal(a.materials.epsilon_r, b.materials.epsilon_r)
    assert a.grid.as_tuple() == b.grid.as_tuple()
    assert [tuple(getattr(e, f) for f, _ in e._fields_) for e in a.edges] == \
        [tuple(getattr(e, f) for f, _ in e._fields_) for e in b.edges]
    assert [(w.x, w.y, w.z, w.component, w.term, w.factor) for w in a.wires] == \
        [(w.x, w.y, w.z, w.component, w.term, w.factor) for w in b.wires]
    assert a.sources == b.sources and a.ports == b.ports and a.far_field == b.far_field


def test_script_error_exits_with_code_3(tmp_path, capsys):
    """Main.cpp:1145-1157: a script that fails to load ends the run with exit code 3 (no GPU use)."""
    bad = tmp_path / "broken.lua"
    bad.write_text('scene { name = "broken", size = {32, 32, 32} }\nnot_a_function_of_the_api { }\n')
    code, inst = headless.run(str(bad), 10)
    assert code == 3 and inst is None
    assert "script error" in capsys.readouterr().err
