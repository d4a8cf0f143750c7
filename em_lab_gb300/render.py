"""Headless rendering: the reference's orbit camera and render settings, the ray-march call, and
BMP output for --screenshot.

Camera (src/Camera.cpp: orbit offset, lookAt with +z up, 50-degree perspective) and the volume
pass's uniforms (src/VolumeRenderer.cpp:44-118: the lattice mapped to [-1, 1] along its longest
axis) in float32 with glm's matrix conventions; the ray march itself runs on the GPU
(csrc/render.cu, emlab_render).
"""
from __future__ import annotations

import math
import struct

import numpy as np

from . import abi

f32 = np.float32
MODES = {"fields": 0, "e": 1, "b": 2, "poynting": 3, "signed": 4}


def world_scale(size):
    return f32(2.0) / f32(max(max(size), 1))


def lattice_to_world(size, p):
    return (np.asarray(p, f32) - f32(0.5) * np.asarray(size, f32)) * world_scale(size)


def look_at(eye, center, up):
    """glm::lookAt (right-handed), column-major 4x4 as a row-major numpy array M[row, col]."""
    f = center - eye
    f = f / f32(np.sqrt(np.float32(np.dot(f, f))))
    s = np.cross(f, up).astype(f32)
    s = s / f32(np.sqrt(np.float32(np.dot(s, s))))
    u = np.cross(s, f).astype(f32)
    m = np.eye(4, dtype=f32)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -np.dot(s, eye), -np.dot(u, eye), np.dot(f, eye)
    return m


def perspective(fovy, aspect, near, far):
    """glm::perspective (right-handed, clip depth -1..1)."""
    t = f32(math.tan(float(fovy) / 2.0))
    m = np.zeros((4, 4), f32)
    m[0, 0] = f32(1.0) / (f32(aspect) * t)
    m[1, 1] = f32(1.0) / t
    m[2, 2] = -(f32(far) + f32(near)) / (f32(far) - f32(near))
    m[3, 2] = f32(-1.0)
    m[2, 3] = -(f32(2.0) * f32(far) * f32(near)) / (f32(far) - f32(near))
    return m


def orbit_camera(target, distance, yaw_deg, pitch_deg):
    """Camera::setOrbit / position / forward: the eye on the orbit sphere, looking at the target."""
    dist = min(max(float(distance), 0.05), 50.0)
    yaw = f32(math.radians(yaw_deg))
    pitch = f32(min(max(math.radians(pitch_deg), -math.radians(89.0)), math.radians(89.0)))
    cp = f32(math.cos(pitch))
    off = np.array([cp * f32(math.cos(yaw)), cp * f32(math.sin(yaw)), f32(math.sin(pitch))], f32)
    eye = np.asarray(target, f32) + f32(dist) * off
    return eye, -off


def render_params(size, view, width, height):
    """RenderSettings and camera of a scene's view{} hints (VolumeRenderer::render, Main.cpp
    applyView) as emlab_render_params."""
    p = abi.RenderParams()
    p.width, p.height = int(width), int(height)
    target = view.get("target")
    tgt = lattice_to_world(size, target) if target is not None else np.zeros(3, f32)
    eye, fwd = orbit_camera(tgt, view.get("distance", 3.0), view.get("yaw", -55.0), view.get("pitch", 30.0))
    vm = look_at(eye, eye + fwd, np.array([0, 0, 1], f32))
    pm = perspective(math.radians(50.0), f32(width) / f32(height), 0.01, 100.0)
    inv = np.linalg.inv((pm.astype(np.float64) @ vm.astype(np.float64))).astype(f32)
    for i, v in enumerate(inv.T.reshape(-1)):  # column-major
        p.inv_view_proj[i] = float(v)
    vmin = -f32(0.5) * np.asarray(size, f32) * world_scale(size)
    vsize = np.asarray(size, f32) * world_scale(size)
    for k in range(3):
        p.cam_pos[k] = float(eye[k])
        p.vol_min[k], p.vol_size[k] = float(vmin[k]), float(vsize[k])
        p.clip_min[k], p.clip_max[k] = float(vmin[k]), float(vmin[k] + vsize[k])
    p.step_voxels = min(max(float(view.get("step", 0.75)), 0.1), 4.0)
    p.gain_e = float(view.get("gain_e", view.get("gain", 1.0)))
    p.gain_b = float(view.get("gain_b", view.get("gain", 1.0)))
    p.density = float(view.get("density", 1.0))
    p.emission = 1.0
    p.material_opacity = float(view.get("metal_opacity", 0.45))
    p.exposure = float(view.get("exposure", 1.25))
    p.mode = int(view.get("mode", 0))
    p.signed_axis = int(view.get("component", 2))
    return p


def write_bmp(path, rgba_bottom_up):
    """24-bit BMP from RGBA rows ordered bottom-up (BMP's own row order)."""
    h, w = rgba_bottom_up.shape[:2]
    row = (w * 3 + 3) & ~3
    pix = np.zeros((h, row), np.uint8)
    bgr = rgba_bottom_up[:, :, 2::-1]
    pix[:, :w * 3] = bgr.reshape(h, w * 3)
    data = pix.tobytes()
    header = struct.pack("<2sIHHI", b"BM", 54 + len(data), 0, 0, 54)
    info = struct.pack("<IiiHHIIiiII", 40, w, h, 1, 24, 0, len(data), 2835, 2835, 0, 0)
    with open(path, "wb") as f:
        f.write(header + info + data)
