"""Built scenes on disk: a scene script's result (materials, sub-cell terms, sources, monitors,
parameters) saved as one compressed .npz and loaded back without the script.

A scene script runs once on the machine that has it; the saved result then runs anywhere through
`headless.run_result` (or `python -m em_lab_gb300 --scene FILE.npz`), with the same solver inputs
bit for bit. `digest` is a SHA-256 over everything the solver and the instruments read, so two
builds of one script can be compared without keeping the arrays.

The format: an array `meta` holding UTF-8 JSON, plus one array per numpy array of the result.
Objects are written as tagged JSON: dataclasses of the scene and script modules by class name,
the ctypes structs of `abi` by class name and field values, tuples, and numpy arrays by reference
into the archive. Loading accepts only those classes (nothing is imported or executed by name).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import hashlib
import io
import json

import numpy as np

from . import abi, scene, script

_DATACLASSES = {cls.__name__: cls for cls in (
    scene.Material, scene.SourceDesc, scene.PortSetup, scene.ThinWireSpec, scene.FluxSetup, scene.CoaxSetup,
    scene.Scene, script.Settings, script.Param, script.ScriptResult)}
_STRUCTS = {cls.__name__: cls for cls in (abi.GridConfig, abi.EdgeOverride, abi.WireTerm, abi.Source, abi.Port,
                                          abi.FluxPlane)}
FORMAT = 1


def _encode(obj, arrays):
    if obj is None or isinstance(obj, (bool, int, float, str)):
        return obj
    if isinstance(obj, (np.bool_, np.integer)):
        return int(obj) if not isinstance(obj, np.bool_) else bool(obj)
    if isinstance(obj, np.floating):
        return float(obj)
    if isinstance(obj, np.ndarray):
        key = f"a{len(arrays)}"
        arrays[key] = obj
        return {"__np__": key}
    if isinstance(obj, tuple):
        return {"__tuple__": [_encode(v, arrays) for v in obj]}
    if isinstance(obj, list):
        return [_encode(v, arrays) for v in obj]
    if isinstance(obj, dict):
        if not all(isinstance(k, str) for k in obj):
            return {"__items__": [[_encode(k, arrays), _encode(v, arrays)] for k, v in obj.items()]}
        return {"__dict__": {k: _encode(v, arrays) for k, v in obj.items()}}
    if isinstance(obj, scene.MaterialVolume):
        return {"__materials__": {"size": list(obj.size), "sigma": _encode(obj.sigma, arrays),
                                  "epsilon_r": _encode(obj.epsilon_r, arrays)}}
    if isinstance(obj, C.Structure):
        name = type(obj).__name__
        if name not in _STRUCTS:
            raise TypeError(f"scene_io: cannot save ctypes struct {name}")
        vals = {}
        for f, _ in obj._fields_:
            v = getattr(obj, f)
            vals[f] = list(v) if isinstance(v, C.Array) else v
        return {"__struct__": name, "fields": vals}
    if dataclasses.is_dataclass(obj):
        name = type(obj).__name__
        if _DATACLASSES.get(name) is not type(obj):
            raise TypeError(f"scene_io: cannot save {type(obj).__module__}.{name}")
        return {"__dc__": name, "fields": {f.name: _encode(getattr(obj, f.name), arrays)
                                           for f in dataclasses.fields(obj)}}
    raise TypeError(f"scene_io: cannot save a {type(obj).__name__}")


def _decode(obj, arrays):
    if isinstance(obj, list):
        return [_decode(v, arrays) for v in obj]
    if not isinstance(obj, dict):
        return obj
    if "__np__" in obj:
        return np.array(arrays[obj["__np__"]])
    if "__tuple__" in obj:
        return tuple(_decode(v, arrays) for v in obj["__tuple__"])
    if "__dict__" in obj:
        return {k: _decode(v, arrays) for k, v in obj["__dict__"].items()}
    if "__items__" in obj:
        return {_decode(k, arrays): _decode(v, arrays) for k, v in obj["__items__"]}
    if "__materials__" in obj:
        m = obj["__materials__"]
        mv = scene.MaterialVolume(tuple(m["size"]))
        mv.sigma = _decode(m["sigma"], arrays).astype(np.float32)
        mv.epsilon_r = _decode(m["epsilon_r"], arrays).astype(np.float32)
        return mv
    if "__struct__" in obj:
        cls = _STRUCTS[obj["__struct__"]]
        s = cls.__new__(cls)
        C.Structure.__init__(s)
        for f, _ in cls._fields_:
            v = obj["fields"][f]
            if isinstance(v, list):
                arr = getattr(s, f)
                for i, x in enumerate(v):
                    arr[i] = x
            else:
                setattr(s, f, v)
        return s
    if "__dc__" in obj:
        cls = _DATACLASSES[obj["__dc__"]]
        return cls(**{k: _decode(v, arrays) for k, v in obj["fields"].items()})
    raise ValueError("scene_io: unknown tagged object")


def dumps(res) -> tuple[bytes, dict]:
    """(JSON meta, arrays) of a ScriptResult or Scene."""
    arrays: dict = {}
    meta = {"format": FORMAT, "root": _encode(res, arrays)}
    return json.dumps(meta, sort_keys=True).encode(), arrays


def save(path, res) -> None:
    """Writes a ScriptResult (or a bare Scene) to `path` (.npz, compressed)."""
    meta, arrays = dumps(res)
    np.savez_compressed(path, meta=np.frombuffer(meta, np.uint8), **arrays)


def load(path):
    """Reads what `save` wrote."""
    with np.load(path, allow_pickle=False) as z:
        meta = json.loads(bytes(z["meta"]).decode())
        if meta.get("format") != FORMAT:
            raise ValueError(f"scene_io: {path} has format {meta.get('format')}, expected {FORMAT}")
        arrays = {k: z[k] for k in z.files if k != "meta"}
    return _decode(meta["root"], arrays)


def digest(res) -> str:
    """SHA-256 of a ScriptResult or Scene as saved (JSON meta, then each array's dtype, shape and
    bytes in key order). Output directories (machine paths) are left out."""
    arrays: dict = {}
    root = _encode(res, arrays)
    _strip_paths(root)
    h = hashlib.sha256(json.dumps(root, sort_keys=True).encode())
    for k in sorted(arrays, key=lambda s: int(s[1:])):
        a = np.ascontiguousarray(arrays[k])
        h.update(f"{k}:{a.dtype.str}:{a.shape}".encode())
        h.update(a.tobytes())
    return h.hexdigest()


def _strip_paths(node):
    if isinstance(node, dict):
        for k in list(node):
            if k in ("output_dir",):
                node[k] = ""
            else:
                _strip_paths(node[k])
    elif isinstance(node, list):
        for v in node:
            _strip_paths(v)


def summary(res) -> dict:
    """Counts of what a built scene holds (for fixtures and reports)."""
    sc = res.scene if hasattr(res, "scene") else res
    m = sc.materials
    return {"name": sc.name, "size": list(sc.grid.size), "pml": int(sc.grid.pml_thickness),
            "courant": float(sc.grid.courant), "wavelength": float(sc.wavelength),
            "non_vacuum_cells": int(np.count_nonzero((m.sigma != 0) | (m.epsilon_r != 1))),
            "edge_overrides": len(sc.edges), "wire_terms": len(sc.wires), "sources": len(sc.sources),
            "ports": len(sc.ports), "probes": len(sc.probes), "fluxes": len(sc.fluxes),
            "far_field": sc.far_field is not None, "sweep": sc.sweep is not None, "coaxes": len(sc.coaxes),
            "radar": sc.radar is not None, "crpa": sc.crpa is not None, "emitters": len(sc.emitters),
            "targets": len(sc.targets)}


def load_bytes(data: bytes):
    """Reads what `to_bytes` returned."""
    return load(io.BytesIO(data))


def to_bytes(res) -> bytes:
    """The .npz archive of `save` in memory."""
    buf = io.BytesIO()
    meta, arrays = dumps(res)
    np.savez_compressed(buf, meta=np.frombuffer(meta, np.uint8), **arrays)
    return buf.getvalue()
