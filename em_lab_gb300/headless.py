"""Headless runner: a scene script stepped for N frames with the reference's console output.

    python -m em_lab_gb300 --script FILE.lua --frames N [--set NAME=VALUE ...] [--steps N]
    python -m em_lab_gb300 --scene FILE.npz --frames N     (a scene built earlier, see scene_io)

Follows the unattended `--frames` mode of the reference application (src/Main.cpp:40-103 options,
464-540 scene load and header, 1043-1157 frame loop): each frame steps the grid (the monitors that
need every step run on the device inside the step), measures probes and fluxes every second frame,
evaluates the far field, port readings and sweep every 50th frame, prints the instrument report
every 100th frame and once more after the last frame. Exit code 2 = non-finite fields, 3 = script
error. There is no window: with --screenshot the last frame's volume pass is ray-marched on the GPU
(render.py, csrc/render.cu) at --width x --height and saved as a BMP (Main.cpp:814-829, 1122-1128);
the render timing is that pass, else 0.
"""
from __future__ import annotations

import argparse
import os
import sys
import time


def _load(path, overrides):
    from .script import ScriptEngine
    return ScriptEngine(overrides, echo=True).run_file(path)


def _value_string(p):
    if p.kind == "bool":
        return "on" if p.value else "off"
    if p.kind == "choice":
        return str(p.value)
    return "%g" % p.value


def print_header(res, grid, script_name):
    sc = res.scene
    s = grid.size()
    print(f"\n=== {sc.name} ===  ({script_name})")
    if sc.description:
        print(sc.description)
    n = s[0] * s[1] * s[2]
    print(f"Grid {s[0]}x{s[1]}x{s[2]} ({n * 1e-6:.1f} M cells, {grid.gpu_memory_bytes() / (1 << 20):.0f} MB GPU), "
          f"dt = {grid.dt():.3f}, PML {sc.grid.pml_thickness}, lambda_ref = {sc.wavelength:.1f} cells "
          f"({299792458.0 / (sc.wavelength * sc.cell_size) * 1e-9:.4g} GHz at {sc.cell_size * 1e3:.3g} mm cells), "
          f"{len(sc.sources)} source term(s)")
    if res.params:
        print("Parameters:")
        for p in res.params:
            print(f"  {'':<8s} {p.label:<24s} = {_value_string(p)}")


def view_settings(sc):
    """The scene's view{} hints with the signed-mode axis defaulting to the first source's dominant
    polarization component (Main.cpp:542-569)."""
    v = dict(sc.view)
    if "component" not in v and sc.sources:
        px, py, pz = (abs(float(c)) for c in sc.sources[0].polarization)
        v["component"] = 0 if (px >= py and px >= pz) else (1 if py >= pz else 2)
    return v


def screenshot(grid, sc, path, width, height):
    """Ray-marches the current fields at width x height and writes a BMP; returns the render ms."""
    from .render import render_params, write_bmp
    params = render_params(grid.size(), view_settings(sc), width, height)
    t0 = time.perf_counter()
    img = grid.render(params)
    ms = (time.perf_counter() - t0) * 1e3
    write_bmp(path, img)
    print(f"Saved screenshot {path}")
    return ms


def run(script, frames, overrides=None, steps_per_frame=None, quiet=False, screenshot_path=None,
        width=1920, height=1080):
    """Runs `script` for `frames` frames; returns (exit code, Instruments)."""
    from .script import ScriptError

    try:
        res = _load(script, overrides or {})
    except ScriptError as e:
        print(f"script error: {e}", file=sys.stderr)
        return 3, None
    return run_result(res, frames, steps_per_frame, screenshot_path=screenshot_path, width=width, height=height,
                      script_name=os.path.basename(str(script)))


def run_result(res, frames, steps_per_frame=None, screenshot_path=None, width=1920, height=1080,
               script_name="scene", after_frame=None):
    """Runs an already built scene (a script's ScriptResult, e.g. loaded by scene_io) for `frames`
    frames exactly as `run` does; returns (exit code, Instruments). `after_frame(frame, inst)` is
    called after every frame's measurements (for callers that watch the readings)."""
    from . import SimulationGrid
    from .instruments import NO_INSTRUMENTS_HINT, Instruments

    sc = res.scene
    grid = SimulationGrid(sc.grid)
    # a radar first records the scene without its targets (Main.cpp:472-507)
    first = res.background if (getattr(sc, "radar", None) is not None and res.background is not None) else sc
    m = first.materials
    grid.upload_materials(m.sigma, m.epsilon_r, first.edges, first.wires)
    grid.set_sources(sc.sources)
    inst = Instruments(grid, sc, output_dir=res.output_dir)
    for w in res.warnings + inst.warnings:
        print(f"  warning: {w}", file=sys.stderr)
    print_header(res, grid, script_name)
    if inst.empty():
        print(NO_INSTRUMENTS_HINT)
    spf = steps_per_frame if steps_per_frame is not None else 2
    if sc.view.get("steps_per_frame"):
        spf = sc.view["steps_per_frame"]
    every_step = bool(inst.ports or inst.ff or inst.coaxes)
    sim_ms = 0.0
    frame = 0
    while frame < frames:
        if inst.crpa is not None:  # switches the sources between its passes (Main.cpp:1067)
            inst.crpa.update()
        t0 = time.perf_counter()
        if spf > 0:
            grid.step(spf)
        grid.synchronize(600000)
        sim_ms = (time.perf_counter() - t0) * 1e3
        if inst.radar is not None:  # swap in the targets once the calibration pass is recorded (Main.cpp:1079-1088)
            inst.radar.update()
            if inst.radar.calibration_complete():
                grid.upload_materials(sc.materials.sigma, sc.materials.epsilon_r, sc.edges, sc.wires)
                grid.reset_fields()
                inst.radar.begin_measurement()
        if frame % 2 == 0 or spf == 0:
            inst.measure()
        if every_step and frame % 50 == 49:
            inst.evaluate_far_field()
            if inst.sweep_setup:
                inst.evaluate_sweep()
        inst.poll_coax()  # the reference polls the line monitor once per frame
        frame += 1
        if after_frame is not None:
            after_frame(frame, inst)
        if frame % 100 == 0 and not inst.empty():
            inst.print_report()
        if frame >= frames:
            inst.measure()
            inst.evaluate_far_field()
            if inst.sweep_setup:
                inst.evaluate_sweep()
            if not inst.empty():
                inst.print_report()
            render_ms = 0.0
            if screenshot_path:
                render_ms = screenshot(grid, sc, screenshot_path, width, height)
            print(f"GPU timings: sim {sim_ms:.3f} ms/frame ({spf} steps), render {render_ms:.3f} ms")
    finite = grid.check_finite()
    inst.close()
    grid.close()
    return (2 if (inst.unstable or not finite) else 0), inst


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m em_lab_gb300", description=__doc__.split("\n\n")[0])
    src = ap.add_mutually_exclusive_group(required=True)
    src.add_argument("--script", help="scene script (.lua)")
    src.add_argument("--scene", help="a built scene saved by em_lab_gb300.scene_io (.npz)")
    ap.add_argument("--set", action="append", default=[], metavar="NAME=VALUE", help="override a script param{}")
    ap.add_argument("--frames", type=int, default=100, help="run this many frames, then exit")
    ap.add_argument("--steps", type=int, default=2, help="simulation steps per frame (the scene's view{} wins)")
    ap.add_argument("--width", type=int, default=1920, help="screenshot width")
    ap.add_argument("--height", type=int, default=1080, help="screenshot height")
    ap.add_argument("--screenshot", metavar="FILE.bmp", help="save the last frame of the run")
    a = ap.parse_args(argv)
    overrides = {}
    for kv in a.set:
        if "=" not in kv or kv.startswith("="):
            print(f"--set expects NAME=VALUE (got '{kv}')", file=sys.stderr)
            continue
        k, v = kv.split("=", 1)
        overrides[k] = v
    if a.scene:
        from . import scene_io
        res = scene_io.load(a.scene)
        code, _ = run_result(res, max(a.frames, 1), min(max(a.steps, 0), 64), screenshot_path=a.screenshot,
                             width=max(a.width, 1), height=max(a.height, 1), script_name=os.path.basename(a.scene))
        return code
    code, _ = run(a.script, max(a.frames, 1), overrides, min(max(a.steps, 0), 64), screenshot_path=a.screenshot,
                  width=max(a.width, 1), height=max(a.height, 1))
    return code


if __name__ == "__main__":
    sys.exit(main())
