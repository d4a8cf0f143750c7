"""Generates tests/golden/*.npz from the reference's own shader code (oracle/_ref, built from the
reference tree by oracle/build_ref.py), so the CPU restatement and the GPU path can be checked
against it where the reference tree is absent.

    python tests/golden/make_golden.py

Each fixture is a seeded scene from em_lab_gb300.configs.random_scene stepped N times by the
reference shaders (emlab_expf as exp): the six field components, the port series and phasors, the
far-field phasors, the coax-line phasors, probe blocks, flux sums and the far-field pattern of 64
directions. radar_backproject.npz holds the reference's radar back-projection (its C++, compiled
by oracle/build_ref.py) of a seeded problem. raymarch.npz holds frames of the reference's volume pass (shaders/raymarch.frag through
the same shim) over the textures of a seeded scene: the render parameters as raw bytes and the
RGB of each frame.
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from em_lab_gb300 import abi, configs  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

CASES = [
    # name, scene kwargs, steps, keep the full field arrays (else: their sha256 and the mid-z plane)
    ("random_s1", dict(size=(24, 20, 18), pml=4, seed=1), 60, True),
    ("random_s2", dict(size=(37, 29, 23), pml=5, seed=2), 90, False),
    ("vacuum_pml0", dict(size=(16, 16, 16), pml=0, seed=5, thin_wire=False, lossy=False, sources=1), 50, True),
]

LINE_Q = [[0, 3, 0, 0], [3, 2, 1, 0]]
LINE_T = [[5, 5, 5, 2], [5, 5, 6, 2], [5, 5, 7, 2], [6, 6, 6, 3], [6, 7, 6, 4]]
LINE_W = [1.0, 1.0, 1.0, 0.5, -0.5]


def monitors_setup(o, sc, steps):
    L = sc.grid.pml_thickness
    size = sc.grid.size
    if sc.ports:
        o.ports_configure([p.to_c() for p in sc.ports], 12.0, 4.0, record_steps=steps)
    o.ntff_configure((L + 1,) * 3, tuple(n - L - 2 for n in size), 12.0, 4.0)
    o.lines_configure(LINE_Q, LINE_T, LINE_W, 12.0)


def flux_planes(size):
    return [abi.FluxPlane(0, 7, (2, 3), (15, 14)), abi.FluxPlane(2, size[2] // 2, (0, 0), (size[0], size[1])),
            abi.FluxPlane(1, 3, (1, 1), (size[0] - 1, size[2] - 1))]


def probe_origins(size):
    return [(3, 4, 5), (0, 0, 0), (size[0] - 2, size[1] - 3, size[2] - 2)]


def field_hash(comps):
    return hashlib.sha256(b"".join(np.ascontiguousarray(c, np.float32).tobytes() for c in comps)).hexdigest()


def run(o, sc, steps):
    oracle.load_scene(o, sc)
    monitors_setup(o, sc, steps)
    o.step(steps)
    out = {f"f{c}": a for c, a in enumerate(o.read_components())}
    if sc.ports:
        out["port_series"] = o.ports_series()
        out["port_phasors"] = o.ports_phasors()
    out["ntff"] = o.ntff_phasors()
    ph, now = o.lines_read()
    out["line_phasors"], out["line_now"] = ph, now
    out["probe"] = o.probe_gather(probe_origins(sc.grid.size))
    out["flux"] = o.flux_planes(flux_planes(sc.grid.size))
    out["pattern"] = o.ntff_evaluate(configs.fibonacci_directions(64))
    return out


RENDER_SCENE = dict(size=(20, 16, 14), pml=3, seed=4)
RENDER_STEPS = 40


def render_textures():
    """E and B textures (rgb = field, alpha = cell sigma / eps_r) of the render fixture's scene."""
    sc = configs.random_scene(**RENDER_SCENE)
    o = oracle.Oracle(sc.grid, "f32")
    oracle.load_scene(o, sc)
    o.step(RENDER_STEPS)
    f = o.read_components()
    e = np.stack([f[0], f[1], f[2], sc.materials.sigma], axis=-1).astype(np.float32)
    b = np.stack([f[3], f[4], f[5], sc.materials.epsilon_r], axis=-1).astype(np.float32)
    return e, b


def render_views(size, gain):
    """(name, view hints, width, height): every mode, a cutaway, a close and a far camera."""
    v = []
    for mode in range(5):
        v.append((f"mode{mode}", {"mode": mode, "gain": gain, "component": 1, "metal_opacity": 0.7}, 48, 32))
    v.append(("inside", {"mode": 0, "gain": gain, "distance": 0.3, "yaw": 20.0, "pitch": -10.0, "step": 0.3}, 40, 24))
    v.append(("far", {"mode": 0, "gain": gain * 4, "distance": 9.0, "pitch": 75.0, "exposure": 3.0}, 33, 21))
    return v


def make_render_golden():
    from em_lab_gb300 import render
    e, b = render_textures()
    size = (e.shape[2], e.shape[1], e.shape[0])
    gain = float(1.0 / (0.25 * np.abs(e[..., :3]).max()))
    out = {}
    for name, view, w, h in render_views(size, gain):
        p = render.render_params(size, view, w, h)
        if name == "mode3":  # cutaway: the upper half of x
            p.clip_min[0] = p.vol_min[0] + 0.5 * p.vol_size[0]
        img = oracle.render(e, b, p, ref=True)
        out[f"{name}_params"] = np.frombuffer(bytes(p), np.uint8)
        out[f"{name}_rgb"] = img[..., :3]
    out["steps"] = np.array(RENDER_STEPS)
    np.savez_compressed(os.path.join(OUT, "raymarch.npz"), **out)
    print("raymarch written")


def make_radar_golden():
    """The reference's back-projection (RadarMonitor::computeImage, compiled from the reference by
    oracle/build_ref.py) on a seeded problem, for the GPU kernel's test on machines without the tree."""
    from oracle import radar_ref
    g, wl, z, ep, w, tp, ta = radar_ref.random_case(5)
    power = oracle.ref_host_backproject(g, wl, z, ep, w, tp, ta)
    np.savez_compressed(os.path.join(OUT, "radar_backproject.npz"), geometry=np.frombuffer(bytes(g), np.uint8),
                        wavelength=np.array(wl), z=z, elem_pos=ep, weights=w, tx_pos=tp, tx_amp=ta, power=power)
    print("radar_backproject written")


def main():
    if "--radar-only" in sys.argv:
        make_radar_golden()
        return
    if not oracle.ref_available():
        sys.exit("oracle/_ref is not built: run python oracle/build_ref.py (needs the reference tree)")
    if "--render-only" in sys.argv:
        make_render_golden()
        return
    for name, kw, steps, full in CASES:
        sc = configs.random_scene(**kw)
        o = oracle.Oracle(sc.grid, "ref")
        out = run(o, sc, steps)
        out["steps"] = np.array(steps)
        out["sha256"] = np.array(field_hash([out[f"f{c}"] for c in range(6)]))
        if not full:
            for c in range(6):
                f = out.pop(f"f{c}")
                out[f"mid{c}"] = f[f.shape[0] // 2]
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
        print(name, "written")
    make_render_golden()
    if oracle.ref_host_available():
        make_radar_golden()


if __name__ == "__main__":
    main()
