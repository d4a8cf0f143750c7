"""The headless volume pass on the CPU: the restatement (oracle/oracle_render.h) against the
reference's own raymarch.frag (compiled through the GLSL shim, when the reference tree is here) and
against the committed golden frames; the orbit camera, the view{} hints and the BMP writer."""
import ctypes as C
import math
import os
import struct
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from em_lab_gb300 import abi, render  # noqa: E402

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import make_golden  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden", "raymarch.npz")


def params_from_bytes(raw):
    p = abi.RenderParams()
    C.memmove(C.byref(p), bytes(raw), C.sizeof(p))
    return p


@pytest.fixture(scope="module")
def textures():
    return make_golden.render_textures()


def synthetic_textures(n=(21, 17, 13), seed=3):
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    r = np.sqrt((x - nx / 2) ** 2 + (y - ny / 2) ** 2 + (z - nz / 2) ** 2).astype(np.float32)
    e = np.zeros((nz, ny, nx, 4), np.float32)
    b = np.zeros_like(e)
    e[..., 0] = rng.standard_normal(r.shape) * 0.4
    e[..., 2] = np.sin(r * 0.7) * 2.0
    b[..., 1] = np.cos(r * 0.7) * 1.5
    b[..., 0] = rng.standard_normal(r.shape) * 0.2
    e[..., 3] = np.where((abs(x - 5) < 3) & (abs(y - 6) < 4), 1e7, np.where(r < 3, 0.4, 0.0))  # metal, lossy
    b[..., 3] = np.where(x > 15, 3.5, 1.0)  # glass slab
    return e, b


def test_golden_frames_match_restatement(textures):
    """The restatement reproduces the reference shader's frames bit for bit (committed fixture)."""
    e, b = textures
    z = np.load(GOLDEN)
    names = sorted(k[:-7] for k in z.files if k.endswith("_params"))
    assert len(names) == 7
    for name in names:
        p = params_from_bytes(z[f"{name}_params"])
        img = oracle.render(e, b, p)
        np.testing.assert_array_equal(img[..., :3], z[f"{name}_rgb"], err_msg=name)
        assert (img[..., 3] == 255).all()


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref (the reference's shaders) not built")
@pytest.mark.parametrize("mode", range(5))
def test_restatement_equals_reference_shader(mode):
    e, b = synthetic_textures()
    size = (e.shape[2], e.shape[1], e.shape[0])
    for axis in (0, 2, 7):  # 7: clamped to z
        view = {"mode": mode, "component": axis, "metal_opacity": 0.8, "gain": 0.9, "step": 0.6}
        p = render.render_params(size, view, 37, 23)
        p.signed_axis = axis
        a = oracle.render(e, b, p)
        r = oracle.render(e, b, p, ref=True)
        np.testing.assert_array_equal(a, r)


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref (the reference's shaders) not built")
def test_restatement_edge_cases_equal_reference_shader():
    """Cutaway box, a camera inside the volume, a ray that misses, clamped steps, a 1x1 target."""
    e, b = synthetic_textures((9, 30, 5))
    size = (e.shape[2], e.shape[1], e.shape[0])
    cases = []
    p = render.render_params(size, {"mode": 0}, 31, 19)
    p.clip_min[1] = p.vol_min[1] + 0.3 * p.vol_size[1]
    p.clip_max[2] = p.vol_min[2] + 0.6 * p.vol_size[2]
    cases.append(p)
    cases.append(render.render_params(size, {"mode": 3, "distance": 0.05, "yaw": 90.0, "pitch": 0.0}, 25, 25))
    p = render.render_params(size, {"mode": 2, "distance": 2.0, "yaw": 0.0, "pitch": 0.0}, 16, 9)
    for k in range(3):  # move the volume behind the camera: every ray misses
        p.clip_min[k] += 40.0
        p.clip_max[k] += 40.0
    cases.append(p)
    p = render.render_params(size, {"mode": 1}, 1, 1)
    p.step_voxels = 100.0  # clamped to 4
    cases.append(p)
    p = render.render_params(size, {"mode": 4}, 8, 8)
    p.step_voxels = 0.0  # clamped to 0.1
    cases.append(p)
    for p in cases:
        np.testing.assert_array_equal(oracle.render(e, b, p), oracle.render(e, b, p, ref=True))


def test_missed_rays_are_background():
    e, b = synthetic_textures((6, 6, 6))
    p = render.render_params((6, 6, 6), {}, 12, 10)
    for k in range(3):
        p.clip_min[k] += 40.0
        p.clip_max[k] += 40.0
    img = oracle.render(e, b, p).astype(int)
    # the background gradient is dark blue: blue above red and green everywhere, no field colour
    assert (img[..., 2] >= img[..., 0]).all() and img[..., :3].max() < 80


def test_orbit_camera_matches_reference_conventions():
    size = (40, 20, 10)
    assert render.world_scale(size) == np.float32(0.05)
    np.testing.assert_allclose(render.lattice_to_world(size, (20, 10, 5)), 0.0)
    eye, fwd = render.orbit_camera((0, 0, 0), 3.0, -55.0, 30.0)
    y, pch = math.radians(-55.0), math.radians(30.0)
    np.testing.assert_allclose(eye, 3.0 * np.array([math.cos(pch) * math.cos(y), math.cos(pch) * math.sin(y),
                                                      math.sin(pch)]), rtol=1e-6)
    np.testing.assert_allclose(fwd, -eye / 3.0, rtol=1e-6)
    # the distance and the pitch are clamped as Camera::setOrbit clamps them
    eye, _ = render.orbit_camera((0, 0, 0), 500.0, 0.0, 120.0)
    np.testing.assert_allclose(np.linalg.norm(eye), 50.0, rtol=1e-6)
    assert eye[2] == pytest.approx(50.0 * math.sin(math.radians(89.0)), rel=1e-6)
    # the centre pixel's ray of the inverse view-projection runs along the camera's forward axis
    p = render.render_params(size, {"distance": 2.5, "yaw": 10.0, "pitch": 20.0}, 64, 64)
    m = np.array(p.inv_view_proj, np.float64).reshape(4, 4).T
    far = m @ np.array([0.0, 0.0, 1.0, 1.0])
    d = far[:3] / far[3] - np.array(p.cam_pos)
    _, fwd = render.orbit_camera((0, 0, 0), 2.5, 10.0, 20.0)
    np.testing.assert_allclose(d / np.linalg.norm(d), fwd, atol=1e-5)
    # the marched box is the whole lattice, longest side 2 world units
    np.testing.assert_allclose(p.vol_size[:], [2.0, 1.0, 0.5])
    np.testing.assert_allclose(p.vol_min[:], [-1.0, -0.5, -0.25])


def test_view_hints_set_render_settings():
    defaults = render.render_params((8, 8, 8), {}, 4, 4)
    assert (defaults.mode, defaults.signed_axis) == (0, 2)
    assert defaults.exposure == pytest.approx(1.25) and defaults.material_opacity == pytest.approx(0.45)
    assert defaults.step_voxels == pytest.approx(0.75) and defaults.density == 1.0 and defaults.emission == 1.0
    p = render.render_params((8, 8, 8), {"mode": 3, "component": 0, "gain_e": 2.0, "gain_b": 3.0, "exposure": 0.5,
                                         "density": 4.0, "step": 9.0, "metal_opacity": 0.1}, 4, 4)
    assert (p.mode, p.signed_axis, p.gain_e, p.gain_b, p.exposure, p.density, p.step_voxels) == \
        (3, 0, 2.0, 3.0, 0.5, 4.0, 4.0)
    assert p.material_opacity == pytest.approx(0.1)


def test_bmp_writer(tmp_path):
    img = np.zeros((3, 5, 4), np.uint8)
    img[0, 0] = (10, 20, 30, 255)   # bottom-left pixel
    img[2, 4] = (200, 100, 50, 255)  # top-right pixel
    path = tmp_path / "f.bmp"
    render.write_bmp(path, img)
    data = path.read_bytes()
    assert data[:2] == b"BM"
    size, _, _, off = struct.unpack("<IHHI", data[2:14])
    hsz, w, h, planes, bpp = struct.unpack("<IiiHH", data[14:30])
    row = (5 * 3 + 3) & ~3
    assert (size, off, hsz, w, h, planes, bpp) == (54 + 3 * row, 54, 40, 5, 3, 1, 24)
    assert data[54:57] == bytes((30, 20, 10))  # BGR, bottom row first
    assert data[54 + 2 * row + 12:54 + 2 * row + 15] == bytes((50, 100, 200))
