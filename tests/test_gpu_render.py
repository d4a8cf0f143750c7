"""The CUDA volume pass (emlab_render) against the CPU restatement of raymarch.frag and the golden
frames of the reference shader.

Tolerance: every channel within 1 of 255 and at least 98 % of the channels equal. The two sides run
the same FP32 operations in the same order (no contraction, emlab_expf for exp); pow() is the
device's powf on one side and libm's powf on the other, and GLSL leaves pow's precision to the
implementation, so a last-bit difference there can move a channel across a rounding boundary."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

import oracle  # noqa: E402
from em_lab_gb300 import abi, configs, render  # noqa: E402

pytestmark = pytest.mark.gpu


def close_images(a, b, what):
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))
    assert d.max() <= 1, f"{what}: max channel difference {d.max()}"
    frac = float((d == 0).mean())
    assert frac >= 0.98, f"{what}: only {frac:.4f} of the channels equal"


@pytest.fixture(scope="module")
def stepped_grid():
    import make_golden
    from em_lab_gb300 import SimulationGrid
    sc = configs.random_scene(**make_golden.RENDER_SCENE)
    g = SimulationGrid(sc.grid)
    oracle.load_scene(g, sc)
    g.step(make_golden.RENDER_STEPS)
    g.synchronize()
    yield g, sc
    g.close()


def test_render_matches_golden_frames(stepped_grid):
    g, _ = stepped_grid
    z = np.load(os.path.join(ROOT, "tests", "golden", "raymarch.npz"))
    names = sorted(k[:-7] for k in z.files if k.endswith("_params"))
    for name in names:
        p = abi.RenderParams()
        C.memmove(C.byref(p), bytes(z[f"{name}_params"]), C.sizeof(p))
        img = g.render(p)
        assert img.shape == (p.height, p.width, 4) and (img[..., 3] == 255).all()
        close_images(img[..., :3], z[f"{name}_rgb"], name)


@pytest.mark.parametrize("mode", range(5))
def test_render_matches_restatement(stepped_grid, mode):
    g, _ = stepped_grid
    e, b = g.read_textures()
    size = g.size()
    gain = float(1.0 / (0.25 * np.abs(e[..., :3]).max()))
    for w, h, view in ((97, 61, {"distance": 2.2}), (16, 8, {"yaw": 150.0, "pitch": -40.0}),
                       (1, 1, {}), (130, 3, {"distance": 0.4, "step": 0.2})):
        v = dict(view, mode=mode, gain=gain, component=mode % 3)
        p = render.render_params(size, v, w, h)
        close_images(g.render(p), oracle.render(e, b, p), f"mode {mode} {w}x{h} {view}")


def test_render_edge_cases(stepped_grid):
    g, _ = stepped_grid
    e, b = g.read_textures()
    size = g.size()
    cases = []
    p = render.render_params(size, {"mode": 0, "gain": 50.0}, 45, 30)
    p.clip_min[2] = p.vol_min[2] + 0.5 * p.vol_size[2]  # cutaway
    cases.append(p)
    p = render.render_params(size, {"mode": 2}, 20, 10)
    for k in range(3):  # every ray misses
        p.clip_min[k] += 40.0
        p.clip_max[k] += 40.0
    cases.append(p)
    p = render.render_params(size, {"mode": 4, "gain": 80.0}, 24, 24)
    p.step_voxels, p.signed_axis = 100.0, 9  # clamped to 4 and to z
    cases.append(p)
    for p in cases:
        close_images(g.render(p), oracle.render(e, b, p), "edge case")


def test_render_rejects_bad_sizes(stepped_grid):
    g, _ = stepped_grid
    p = render.render_params(g.size(), {}, 4, 4)
    p.width = 0
    with pytest.raises(Exception):
        g.render(p)
    p.width, p.height = 4, 20000
    with pytest.raises(Exception):
        g.render(p)
    p.height, p.step_voxels = 4, float("nan")
    with pytest.raises(Exception):
        g.render(p)
