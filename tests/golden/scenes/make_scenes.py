"""Builds every scene script bundled with the reference (scenes/*.lua and scenes/validation/*.lua)
through em_lab_gb300.script and saves each result as tests/golden/scenes/<name>.npz, with its
SHA-256 digest and a summary in tests/golden/scenes/digests.json.

    python tests/golden/scenes/make_scenes.py [--reference PATH]

The tree comes from --reference, $EMLAB_REFERENCE or the tree oracle/build_ref.py last built from.
The saved results are the solver inputs the scripts produce (materials, sub-cell terms, sources,
monitors, parameters): the tests run them headless on the GPU where the scripts themselves are
absent, and rebuild the scripts to compare digests where the tree is present. Besides each
script's defaults, the parameter settings the validation scripts quote results for are saved:
dipole_impedance at lengths 7, 15, 19, 21 and coax_line with every termination.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, ROOT)

from em_lab_gb300 import scene_io  # noqa: E402
from em_lab_gb300.script import ScriptEngine  # noqa: E402

# (fixture name, script path in the tree, parameter overrides)
VARIANTS = [
    ("dipole_impedance_len7", "scenes/validation/dipole_impedance.lua", {"length": "7"}),
    ("dipole_impedance_len15", "scenes/validation/dipole_impedance.lua", {"length": "15"}),
    ("dipole_impedance_len21", "scenes/validation/dipole_impedance.lua", {"length": "21"}),
    ("coax_line_open", "scenes/validation/coax_line.lua", {"termination": "open"}),
    ("coax_line_short", "scenes/validation/coax_line.lua", {"termination": "short"}),
    ("coax_line_100ohm", "scenes/validation/coax_line.lua", {"termination": "100 ohm"}),
]


def reference_tree(argv):
    if "--reference" in argv:
        return argv[argv.index("--reference") + 1]
    from oracle.build_ref import reference_root
    root = reference_root()
    return str(root) if root else None


def scene_list(tree):
    """(fixture name, script path relative to the tree, overrides) for every bundled script."""
    out = []
    for sub in ("scenes", os.path.join("scenes", "validation")):
        d = os.path.join(tree, sub)
        for f in sorted(os.listdir(d)):
            if f.endswith(".lua"):
                out.append((os.path.splitext(f)[0], os.path.join(sub, f), {}))
    return out + VARIANTS


def build(tree, rel, overrides):
    return ScriptEngine(dict(overrides), echo=False).run_file(os.path.join(tree, rel))


def main(argv):
    tree = reference_tree(argv)
    if not tree or not os.path.isdir(os.path.join(tree, "scenes")):
        print("reference tree not found: nothing written")
        return 1
    table = {}
    for name, rel, overrides in scene_list(tree):
        res = build(tree, rel, overrides)
        scene_io.save(os.path.join(HERE, name + ".npz"), res)
        table[name] = {"script": rel.replace(os.sep, "/"), "overrides": overrides, "digest": scene_io.digest(res),
                       "summary": scene_io.summary(res)}
        print(f"{name:28s} {table[name]['digest'][:16]}  {table[name]['summary']['size']}")
    with open(os.path.join(HERE, "digests.json"), "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
        f.write("\n")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
