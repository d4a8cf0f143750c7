"""Build recipe for the native library (nvcc, sm_103a) and the CPU restatement used by the tests.

Everything is compiled in-tree: objects under ``em_lab_gb300/_build/``, the shared library at
``em_lab_gb300/_lib/libemlab_gb300.so`` and the test oracle at ``oracle/_build/libemlab_oracle.so``.
Floating-point contraction is disabled everywhere (``-fmad=false`` for device code,
``-ffp-contract=off`` for host code) so the kernels, the host set-up code and the oracle round
every operation identically.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "libemlab_gb300.so"
ORACLE_SRC = ROOT / "oracle" / "emlab_oracle.c"
ORACLE_LIB = ROOT / "oracle" / "_build" / "libemlab_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = "-fPIC,-fopenmp,-ffp-contract=off,-O2"
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", HOST_FLAGS,
              "-I", str(ROOT / "include"), "-I", str(CSRC)]

SOURCES = ["yee.cu", "yee_tma.cu", "monitors.cu", "capi.cu", "noalloc.cu", "dft_tc.cu", "render.cu", "stack.cu", "learn.cu", "radar.cu", "cpml.cu", "pattern_tc.cu", "setup.cpp"]
HEADERS = ["emlab_math.h", "emlab_internal.h", "setup.h", "yee_common.cuh", "grid_state.h", "sincos_reduced.cuh"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build em_lab_gb300")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    res = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(map(str, cmd))}\n{res.stdout}\n{res.stderr}")
    return res


def build_library(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    headers = [CSRC / h for h in HEADERS] + [ROOT / "include" / "emlab.h"]
    jobs = []
    for src in SOURCES:
        obj = OBJ / (src + ".o")
        if force or _stale(obj, [CSRC / src] + headers):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", CSRC / src, "-o", obj]
            if src.endswith(".cpp"):
                cmd = [nvcc, *NVCC_FLAGS, "-x", "c++", "-c", CSRC / src, "-o", obj]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs))
    objs = [OBJ / (s + ".o") for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", LIB, *objs], verbose)
    return LIB


def build_oracle(verbose: bool = False, force: bool = False) -> Path:
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    deps = [ORACLE_SRC, ROOT / "oracle" / "oracle_impl.h", ROOT / "oracle" / "oracle_render.h", CSRC / "emlab_math.h",
            ROOT / "include" / "emlab.h"]
    if force or _stale(ORACLE_LIB, deps):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11",
              ORACLE_SRC, "-o", ORACLE_LIB, "-lm"], verbose)
    return ORACLE_LIB


def build_all(verbose: bool = False, force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, verbose, force)
        f2 = ex.submit(build_oracle, verbose, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    import sys
    build_all(verbose=True, force="--force" in sys.argv)
