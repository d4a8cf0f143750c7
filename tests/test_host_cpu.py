"""CPU checks of the product's host side: the C ABI library loads and exports what include/emlab.h
declares, its set-up arithmetic equals the oracle's, the scene builders reproduce the reference's
antenna/feed construction, and the package fails loudly without a device."""
import math
import os
import re

import numpy as np
import pytest

import oracle
from em_lab_gb300 import abi, configs, grid, scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    """Every function declared in include/*.h (the C headers of the boundary)."""
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(emlab_\w+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = grid.load_library()
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.emlab_version() >= 1


def test_no_device_fails_loudly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(grid.EmlabError) as e:
        grid.SimulationGrid(abi.GridConfig((16, 16, 16)))
    assert e.value.code == abi.EMLAB_ERR_NO_DEVICE


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_edge_materials_equal_oracle(seed):
    sc = configs.random_scene(size=(23, 19, 17), pml=3, seed=seed)
    m = sc.materials
    es, ee, w0, w1, classes = grid.edge_materials(m.sigma, m.epsilon_r, sc.edges, sc.wires)
    o = oracle.Oracle(sc.grid, "f32")
    o.upload_materials(m.sigma, m.epsilon_r, sc.edges, sc.wires)
    os_, oe, ow0, ow1 = o.edge_materials()
    # the product table stores sigma >= 0, eps >= 1 (update_E.comp:48-49); the oracle the raw halves
    assert np.array_equal(es, np.maximum(os_, 0)) and np.array_equal(ee, np.maximum(oe, 1))
    assert np.array_equal(w0, ow0) and np.array_equal(w1, ow1)
    assert classes >= 2


def test_edge_materials_clamp_and_invalid_overrides_skipped():
    n = 8
    sig = np.zeros((n, n, n), np.float32)
    eps = np.ones((n, n, n), np.float32)
    sig[2:5, 2:5, 2:5] = 1e7  # PEC cells: clamped to 6e4 on the edges
    edges = [abi.EdgeOverride(1, 1, 1, 0, 123.0), abi.EdgeOverride(-1, 0, 0, 0, 5.0), abi.EdgeOverride(0, 0, 0, 3, 5.0),
             abi.EdgeOverride(1, 1, 1, 0, -3.0)]
    es, ee, w0, w1, classes = grid.edge_materials(sig, eps, edges, [])
    assert es.max() == np.float32(np.float16(6.0e4))
    assert es[1, 1, 1, 0] == 0.0  # the later override (negative -> 0) wins
    assert es[0, 0, 0, 0] == 0.0
    assert np.all(w0 == 1.0) and np.all(w1 == 1.0)


def test_source_signal_equals_oracle():
    rng = np.random.default_rng(3)
    for k in range(40):
        s = scene.SourceDesc(wavelength=float(rng.uniform(8, 60)), phase=float(rng.uniform(0, 6.3)),
                             waveform=int(k % 2), ramp_periods=float(rng.uniform(0.2, 4)),
                             repeat_periods=float(rng.choice([0.0, 3.0])), delay_periods=float(rng.uniform(0, 2)))
        for t in rng.uniform(0, 400, 20):
            assert grid.source_signal(s, float(t)) == oracle.source_signal(s, float(t))


def test_thin_wire_dipole_construction():
    """buildDipole / emitThinWires / addFeed for a centre-fed half-wave dipole (ScriptEngine.cpp)."""
    g = abi.GridConfig((64, 64, 64), pml_thickness=8)
    b = scene.EnvironmentBuilder("d", g, wavelength=40.0)
    wave = scene.SourceDesc(wavelength=40.0)
    b.thin_dipole(wave, (32.0, 32.0, 32.0), 2, 20.0, radius=0.05)
    sc = b.build()
    # 2 * 10 + 1 = 21 edges requested, both free ends one cell short, the gap edge left for the feed
    pec = [e for e in sc.edges if e.sigma == np.float32(6.0e4)]
    feed = [e for e in sc.edges if e.sigma != np.float32(6.0e4)]
    assert len(pec) == 18 and len(feed) == 1
    assert (feed[0].x, feed[0].y, feed[0].z, feed[0].axis) == (32, 32, 32, 2)
    assert feed[0].sigma == np.float32(np.float32(376.730313668) / np.float32(50.0))
    zs = sorted(e.z for e in pec)
    assert zs[0] == 23 and zs[-1] == 41 and 32 not in zs
    assert len(sc.wires) == 4 * 19
    assert all(abs(w.factor - 2.0 / math.log(20.0)) < 1e-6 for w in sc.wires)
    # the B components circling a z wire: Bx scales term0 (d_y E_z), By scales term1 (d_x E_z)
    assert {(w.component, w.term) for w in sc.wires} == {(0, 0), (1, 1)}
    src = sc.sources[0]
    assert src.center == (32.0, 32.0, 32.5) and src.softness == (0.25, 0.25, 0.25)
    assert src.amplitude == pytest.approx(-376.730313668 / 50.0, rel=1e-6)
    assert sc.ports[0].texel == (32, 32, 32)


def test_plain_workloads():
    small = configs.plain_small()
    assert small.grid.size == (128, 128, 128) and small.grid.pml_thickness == 10
    # radius-10 sphere: cells whose centres lie within distance 10 (cell-centre voxeliser test)
    assert int((small.materials.epsilon_r == np.float32(2.25)).sum()) == 4224
    src = small.sources[0]
    assert src.amplitude == pytest.approx(7.0 / (math.pi * 0.75 ** 2), rel=1e-6)
    large = configs.plain_large(size=256)
    frac = float((large.materials.epsilon_r > 1).mean())
    assert 0.049 < frac < 0.06
    assert len(large.ports) == 1 and large.sources[0].waveform == abi.WAVE_PULSE


def test_config_clamps():
    o = oracle.Oracle(abi.GridConfig((4, 500, 20), courant=0.9, pml_thickness=70, pml_sigma_max=-1, pml_grading=20),
                      "f32")
    c = o.config()
    assert c.pml_thickness == 64 and c.nx == 136 and c.ny == 500 and c.nz == 136
    assert c.courant == np.float32(np.float32(0.99) / np.float32(1.7320508))
    assert c.pml_sigma_max == 0.0 and c.pml_grading == 12.0


def build_facade_demo(tmp_path):
    import subprocess

    exe = tmp_path / "facade_demo"
    lib_dir = grid.library_path().parent
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "facade_main.cpp"),
           "-L", str(lib_dir), "-lemlab_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_facade_compiles_and_reports_missing_device(tmp_path):
    """The C++ SimulationGrid facade builds against the library; without a device its constructor
    throws std::runtime_error like the reference's does on GL failures."""
    import subprocess

    import torch

    exe = build_facade_demo(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present (the GPU test runs the demo)")
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    assert res.returncode == 3 and "no CUDA device" in res.stdout


def grid_handle_functions():
    """Functions of include/emlab.h whose first parameter is the grid handle."""
    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "emlab.h")).read(), flags=re.S)
    return sorted(set(re.findall(r"\b(emlab_\w+)\s*\(\s*(?:const\s+)?emlab_grid\s*\*\s*\w+", text)))


def test_null_grid_handle_is_an_invalid_argument():
    """Every entry point that takes a grid handle rejects a NULL handle with EMLAB_ERR_INVALID and a
    message, before touching the device or any other argument (no device needed)."""
    import ctypes as C

    lib = grid.load_library()
    names = grid_handle_functions()
    assert len(names) >= 30
    for name in names:
        fn = getattr(lib, name)
        assert fn.argtypes is not None, f"{name} has no ctypes signature"
        args = [0.0 if t in (C.c_float, C.c_double) else (0 if t in (C.c_int, C.c_size_t, C.c_longlong, C.c_uint64)
                                                           else None) for t in fn.argtypes[1:]]
        rc = fn(None, *args)
        if name == "emlab_grid_destroy":
            assert rc == abi.EMLAB_OK  # destroying nothing is allowed, as delete of a null pointer
            continue
        assert rc == abi.EMLAB_ERR_INVALID, f"{name}: {rc}"
        assert lib.emlab_last_error(), name
