"""The C++ SimulationGrid facade on a device: configure -> uploadMaterials -> setSources -> step with
a per-step callback, the size-mismatch exception and the device field view, as the reference's
Application drives its solver."""
import subprocess

import pytest

from test_host_cpu import build_facade_demo

pytestmark = pytest.mark.gpu


def test_cpp_facade_runs_on_the_device(tmp_path):
    exe = build_facade_demo(tmp_path)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "steps 40" in res.stdout and "field-view 1" in res.stdout
