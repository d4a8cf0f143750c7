"""Compiles the reference's own compute shaders as C++ (test infrastructure; the pin of the oracle).

Reads the shader files where they lie in the reference tree (`--reference PATH` or
$EMLAB_REFERENCE; without either the recipe does nothing), rewrites the GLSL-only syntax mechanically (resource declarations ->
globals, fragment inputs/outputs -> per-thread globals, `out` parameters -> references, swizzles
-> calls, `.a` -> `.w`, float literals -> float suffix, array constructors -> brace lists) into oracle/_ref/*.hpp, and builds oracle/_ref/libemlab_ref.so
from oracle/ref_driver.cpp, which runs every dispatch of SimulationGrid::step and the monitors over
the CPU with those shader bodies and the GLSL semantics of oracle/glsl_shim.hpp. Nothing under
oracle/_ref is committed. Without the reference tree the recipe does nothing. The tree it built
from is recorded in oracle/_ref/source_tree.txt, where the tests look for it when
$EMLAB_REFERENCE is unset.

    python oracle/build_ref.py --reference PATH [--force]
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libemlab_ref.so"
SHADERS = ["common.glsl", "field_sampling.glsl", "ntff_common.glsl", "update_B.comp", "update_E.comp",
           "apply_sources.comp", "clear_fields.comp", "port_accumulate.comp", "probe_gather.comp",
           "poynting_flux.comp", "ntff_accumulate.comp", "ntff_pattern.comp", "ntff_reduce.comp",
           "line_accumulate.comp", "raymarch.frag"]


_TREE_RECORD = OUT / "source_tree.txt"
_explicit_root: Path | None = None


def reference_root() -> Path | None:
    """The reference source tree: the recipe's `--reference` argument, else $EMLAB_REFERENCE, else the
    tree the last build recorded in oracle/_ref/source_tree.txt; None when none of them exists."""
    cands = [_explicit_root, os.environ.get("EMLAB_REFERENCE")]
    if _TREE_RECORD.exists():
        cands.append(_TREE_RECORD.read_text().strip())
    for c in cands:
        if c and Path(c).is_dir():
            return Path(c)
    return None


def reference_shaders() -> Path | None:
    base = reference_root()
    d = base / "shaders" if base else None
    return d if d is not None and d.is_dir() else None


_FLOAT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)(?![\w.])")


def _array_ctor(src: str) -> str:
    """`T[N](a, b, ...)` -> `{a, b, ...}`."""
    out = []
    i = 0
    pat = re.compile(r"\b\w+\[\d+\]\(")
    while True:
        m = pat.search(src, i)
        if not m:
            out.append(src[i:])
            return "".join(out)
        out.append(src[i:m.start()])
        depth, j = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(src[j], 0)
            j += 1
        out.append("{" + src[m.end():j - 1] + "}")
        i = j


def transform(text: str) -> str:
    lines = []
    for line in text.splitlines():
        s = line
        if s.lstrip().startswith("#version"):
            continue
        s = re.sub(r'#include\s+"([\w.]+)"', r'#include "\1.hpp"', s)
        if re.match(r"\s*layout\s*\(\s*local_size", s):
            continue
        s = re.sub(r"layout\s*\(\s*location[^)]*\)\s*(?:in|out)\s+(\w+)\s+(\w+)\s*;", r"thread_local \1 \2;", s)
        s = re.sub(r"layout\s*\(\s*std430[^)]*\)\s*(?:(?:readonly|writeonly|restrict)\s+)*buffer\s+\w+\s*\{\s*(\w+)\s+"
                   r"(\w+)\s*\[\s*\]\s*;\s*\}\s*;", r"\1* \2 = nullptr;", s)
        s = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+(?:restrict\s+)?(\w+)\s+(\w+)\s*;", r"\1 \2;", s)
        s = re.sub(r"^(\s*)uniform\s+", r"\1", s)
        s = re.sub(r"^(\s*)shared\s+", r"\1thread_local ", s)
        s = re.sub(r"\bout\s+(\w+)\s+(\w+)", r"\1& \2", s)
        code, sep, comment = s.partition("//")
        code = re.sub(r"\.(xyz|xy|zw|rgb)\b(?!\s*\()", r".\1()", code)
        code = re.sub(r"\.a\b(?!\s*\()", ".w", code)
        code = _FLOAT.sub(lambda m: m.group(1) + "f", code)
        lines.append(code + sep + comment)
    return _array_ctor("\n".join(lines)) + "\n"


def _lines_between(text: str, start: str, end: str, what: str, include_end: bool = False) -> str:
    """The lines from the first one containing `start` up to the next one containing `end` (that
    line excluded, or included with include_end). Raises if either anchor is missing, so a changed
    reference file fails loudly."""
    lines = text.splitlines()
    i = next((k for k, l in enumerate(lines) if start in l), None)
    if i is None:
        raise RuntimeError(f"build_ref: anchor of {what} not found: {start!r}")
    j = next((k for k in range(i + 1, len(lines)) if end in lines[k]), None)
    if j is None:
        raise RuntimeError(f"build_ref: end anchor of {what} not found: {end!r}")
    return "\n".join(lines[i:j + (1 if include_end else 0)]) + "\n"


def _braced(text: str, start: str, what: str) -> str:
    """The lines from the first one containing `start` through the line that closes the brace the
    start line opens (with whatever follows it on that line, e.g. `};`)."""
    lines = text.splitlines()
    i = next((k for k, l in enumerate(lines) if start in l), None)
    if i is None:
        raise RuntimeError(f"build_ref: anchor of {what} not found: {start!r}")
    depth, opened = 0, False
    for k in range(i, len(lines)):
        code = lines[k].split("//")[0]
        for ch in code:
            if ch == "{":
                depth, opened = depth + 1, True
            elif ch == "}":
                depth -= 1
        if opened and depth == 0:
            return "\n".join(lines[i:k + 1]) + "\n"
    raise RuntimeError(f"build_ref: unbalanced braces in {what}")


def host_sources(root: Path) -> dict[str, str]:
    """The pure-CPU spans of the reference's host code that oracle/ref_host.cpp compiles: the set-up
    types and member functions of SimulationGrid.hpp/.cpp, the host arithmetic of uploadMaterials
    and setSources up to their first graphics call, and the radar's direction, transmit delay and
    back-projection loop. Each span is cut at fixed anchors; the text is not otherwise changed
    (except `RadarMonitor::` -> `RadarCore::`, the wrapper struct that holds the members it reads)."""
    hpp = (root / "src" / "SimulationGrid.hpp").read_text()
    cpp = (root / "src" / "SimulationGrid.cpp").read_text()
    radar = (root / "src" / "Radar.cpp").read_text()
    crpa_h = (root / "src" / "Crpa.hpp").read_text()
    crpa = (root / "src" / "Crpa.cpp").read_text()
    return {
        # the adaptive array's weights: set-up and result types, the small dense complex algebra,
        # the hybrid channels and computeWeights from its covariance to its SINR scores
        "ref_crpa_types.inc": _lines_between(crpa_h, "struct EmitterSetup {", "class CrpaMonitor {", "CRPA types"),
        "ref_crpa_algebra.inc": _braced(crpa, "namespace {", "CRPA helpers"),
        "ref_crpa_channels.inc": _braced(crpa, "std::vector<cd> CrpaMonitor::channels(", "channels"
                                         ).replace("CrpaMonitor::", "CrpaCore::"),
        "ref_crpa_weights.inc": _lines_between(crpa, "const std::vector<cd> sRaw = channels(m_response",
                                               "r.satelliteGainDb =", "computeWeights", include_end=True),
        "ref_types.inc": _lines_between(hpp, "struct GridConfig {", "class SimulationGrid {", "set-up types"),
        "ref_gpusource.inc": _braced(cpp, "struct GPUSource {", "GPUSource"),
        "ref_defs.inc": _lines_between(cpp, "MaterialVolume::MaterialVolume(const glm::ivec3& size)",
                                       "SimulationGrid::SimulationGrid(", "MaterialVolume / SourceDesc members"),
        "ref_upload_edges.inc": _lines_between(cpp, "const glm::ivec3 s = m_config.size;",
                                               "glTextureSubImage3D(m_edgeMaterial", "edge materials"),
        "ref_upload_wires.inc": _lines_between(cpp, "std::vector<glm::vec2> factor(n * 3",
                                               "glTextureSubImage3D(m_wireCoef", "thin-wire factors"),
        "ref_sources_pack.inc": _lines_between(cpp, "m_sources.clear();", "if (!packed.empty())", "source packing"),
        "ref_sources_lists.inc": _lines_between(cpp, "std::vector<std::pair<std::uint32_t, std::uint32_t>> pairs;",
                                                "// Immutable storage", "source lists"),
        "ref_radar_members.inc": (_braced(radar, "glm::vec3 RadarMonitor::direction(", "direction") +
                                  _braced(radar, "double RadarMonitor::txDelay(", "txDelay")
                                  ).replace("RadarMonitor::", "RadarCore::"),
        "ref_radar_rows.inc": _braced(radar, "auto rows = [&](int ieBegin, int ieEnd) {", "back-projection rows"),
    }


HOST_LIB = OUT / "libemlab_ref_host.so"


def build_host(force: bool = False, verbose: bool = False) -> Path | None:
    """oracle/_ref/libemlab_ref_host.so from oracle/ref_host.cpp and the extracted spans."""
    root = reference_root()
    if root is None or not (root / "src" / "SimulationGrid.cpp").exists():
        return None
    OUT.mkdir(parents=True, exist_ok=True)
    changed = force or not HOST_LIB.exists()
    for name, text in host_sources(root).items():
        dst = OUT / name
        if not dst.exists() or dst.read_text() != text:
            dst.write_text(text)
            changed = True
    deps = [HERE / "ref_host.cpp", HERE / "glm_host.hpp", Path(__file__)]
    if not changed and all(HOST_LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return HOST_LIB
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
           "-I", str(OUT), "-I", str(HERE), str(HERE / "ref_host.cpp"), "-o", str(HOST_LIB)]
    if verbose:
        print(" ".join(cmd))
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(res.stdout + res.stderr)
        raise RuntimeError("building the reference host code failed")
    return HOST_LIB


def build(force: bool = False, verbose: bool = False) -> Path | None:
    src = reference_shaders()
    if src is None:
        return None
    OUT.mkdir(parents=True, exist_ok=True)
    deps = [HERE / "ref_driver.cpp", HERE / "glsl_shim.hpp", HERE / "emlab_oracle.c", HERE / "oracle_impl.h",
            HERE / "oracle_render.h",
            HERE.parent / "em_lab_gb300" / "csrc" / "emlab_math.h", Path(__file__)]
    changed = force or not LIB.exists()
    for name in SHADERS:
        dst = OUT / (name + ".hpp")
        text = transform((src / name).read_text())
        if not dst.exists() or dst.read_text() != text:
            dst.write_text(text)
            changed = True
    _TREE_RECORD.write_text(str(src.parent) + "\n")
    if not changed and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    # the host-side set-up comes from the restatement: link its object into the same library
    obj = OUT / "emlab_oracle.o"
    cmds = [[os.environ.get("CC", "gcc"), "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-c",
             str(HERE / "emlab_oracle.c"), "-o", str(obj)],
            [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
             "-I", str(OUT), "-I", str(HERE), str(HERE / "ref_driver.cpp"), str(obj), "-o", str(LIB)]]
    for cmd in cmds:
        if verbose:
            print(" ".join(cmd))
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            sys.stderr.write(res.stdout + res.stderr)
            raise RuntimeError("building the reference shaders failed")
    return LIB


if __name__ == "__main__":
    if "--reference" in sys.argv:
        _explicit_root = Path(sys.argv[sys.argv.index("--reference") + 1])
    lib = build(force="--force" in sys.argv, verbose=True)
    host = build_host(force="--force" in sys.argv, verbose=True) if lib else None
    print(lib if lib else "reference tree not found: nothing built")
    if host:
        print(host)
