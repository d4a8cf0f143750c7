"""ctypes loader for the CPU restatement in emlab_oracle.c (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this package; the
product (em_lab_gb300) never does. `Oracle(cfg, precision)` mirrors the C-ABI grid object:
precision "f32" (parity oracle, deterministic emlab_expf), "f32libm" (FP32 with libm expf, the
tolerance variant) or "f64" (error floor).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from em_lab_gb300 import abi

_PATH = Path(__file__).resolve().parent / "_build" / "libemlab_oracle.so"
_REF_PATH = Path(__file__).resolve().parent / "_ref" / "libemlab_ref.so"
_lib = None
_ref_lib = None


def _grid_spec(R):
    P, I, SZ, F, D = C.c_void_p, C.c_int, C.c_size_t, C.c_float, C.c_double
    ip, dp, fp = C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_float)
    rp = C.POINTER(R)
    return {
        "oracle_create": ([C.POINTER(abi.GridConfig), I], P),
        "oracle_destroy": ([P], None),
        "oracle_get_config": ([P, C.POINTER(abi.GridConfig)], None),
        "oracle_step_count": ([P], C.c_uint64),
        "oracle_source_cells": ([P], I),
        "oracle_upload_materials": ([P, fp, fp, I, I, I, C.POINTER(abi.EdgeOverride), SZ,
                                     C.POINTER(abi.WireTerm), SZ], I),
        "oracle_edge_materials": ([P, fp, fp, fp, fp], None),
        "oracle_set_sources": ([P, C.POINTER(abi.Source), SZ], I),
        "oracle_reset_fields": ([P], None),
        "oracle_step": ([P, I], None),
        "oracle_read_components": ([P] + [rp] * 6, None),
        "oracle_write_components": ([P] + [rp] * 6, None),
        "oracle_ports_configure": ([P, C.POINTER(abi.Port), SZ, F, F, I, SZ], I),
        "oracle_ports_read_phasors": ([P, rp], None),
        "oracle_ports_read_series": ([P, rp, SZ], SZ),
        "oracle_ports_sweep_sums": ([P, D, D, I, dp, dp], None),
        "oracle_ntff_configure": ([P, ip, ip, F, F, ip], I),
        "oracle_ntff_point_count": ([P], I),
        "oracle_ntff_read_phasors": ([P, rp], None),
        "oracle_ntff_evaluate": ([P, fp, I, rp], None),
        "oracle_lines_configure": ([P, ip, I, ip, fp, I, F, F], I),
        "oracle_lines_read": ([P, rp, rp], None),
        "oracle_probe_gather": ([P, ip, I, rp], None),
        "oracle_flux_planes": ([P, C.POINTER(abi.FluxPlane), I, dp], None),
        "oracle_ntff_dft_configure": ([P, ip, ip, fp, I, ip], I),
        "oracle_ntff_dft_points": ([P], I),
        "oracle_ntff_dft_read": ([P, dp], None),
        "oracle_set_cpml": ([P, I, F, F, F, F], I),
    }


def ref_available() -> bool:
    """True when oracle/_ref (the reference's shaders compiled as C++) has been built."""
    return _REF_PATH.exists()


def load_ref():
    """The reference-shader library built by oracle/build_ref.py (raises if absent)."""
    global _ref_lib
    if _ref_lib is not None:
        return _ref_lib
    if not _REF_PATH.exists():
        raise FileNotFoundError(f"{_REF_PATH} is not built (python oracle/build_ref.py)")
    lib = C.CDLL(str(_REF_PATH))
    for name, (args, res) in _grid_spec(C.c_float).items():
        if name in ("oracle_ports_sweep_sums", "oracle_ntff_dft_configure", "oracle_ntff_dft_points",
                    "oracle_ntff_dft_read", "oracle_set_cpml"):
            continue
        fn = getattr(lib, f"{name}_ref")
        fn.argtypes, fn.restype = args, res
    lib.oracle_set_threads.argtypes, lib.oracle_set_threads.restype = [C.c_int], None
    _ref_lib = lib
    return lib


_REF_HOST_PATH = Path(__file__).resolve().parent / "_ref" / "libemlab_ref_host.so"
_ref_host = None


def ref_host_available() -> bool:
    """True when oracle/_ref/libemlab_ref_host.so (the reference's host set-up and radar C++,
    built by oracle/build_ref.py) exists."""
    return _REF_HOST_PATH.exists()


def load_ref_host():
    """The reference's host C++ (oracle/ref_host.cpp over the extracted spans; raises if absent)."""
    global _ref_host
    if _ref_host is not None:
        return _ref_host
    if not _REF_HOST_PATH.exists():
        raise FileNotFoundError(f"{_REF_HOST_PATH} is not built (python oracle/build_ref.py --reference PATH)")
    lib = C.CDLL(str(_REF_HOST_PATH))
    I, SZ, F, D = C.c_int, C.c_size_t, C.c_float, C.c_double
    fp, dp, ip = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int)
    u32p, i32p = C.POINTER(C.c_uint32), C.POINTER(C.c_int32)
    src = C.POINTER(abi.Source)
    spec = {
        "ref_host_signal": ([src, D], D),
        "ref_host_dipole": ([fp, fp, F, F, F, src], None),
        "ref_host_plane_wave": ([I, F, fp, F, F, src], None),
        "ref_host_upload_materials": ([fp, fp, I, I, I, C.POINTER(abi.EdgeOverride), SZ, C.POINTER(abi.WireTerm),
                                       SZ, u32p, u32p], I),
        "ref_host_set_sources": ([src, SZ, I, I, I, fp, i32p, i32p, ip, ip], I),
        "ref_host_radar_backproject": ([C.POINTER(abi.RadarGeometry), F, fp, I, I, fp, dp, fp, dp, I, dp], None),
    }
    for name, (args, res) in spec.items():
        fn = getattr(lib, name)
        fn.argtypes, fn.restype = args, res
    _ref_host = lib
    return lib


def ref_host_backproject(g, wavelength, z, elem_pos, weights, tx_pos, tx_amp):
    """RadarMonitor::computeImage's back-projection compiled from the reference: power (nr, nel, naz)."""
    lib = load_ref_host()
    M, C_ = z.shape
    out = np.zeros((g.nr, g.nel, g.naz))
    fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
    zz = np.ascontiguousarray(z, np.complex64).view(np.float32)
    ep = np.ascontiguousarray(elem_pos, np.float32)
    w = np.ascontiguousarray(weights, np.float64)
    tp = np.ascontiguousarray(tx_pos, np.float32)
    ta = np.ascontiguousarray(tx_amp, np.float64)
    lib.ref_host_radar_backproject(C.byref(g), float(wavelength), zz.ctypes.data_as(fp), M, C_, ep.ctypes.data_as(fp),
                                   w.ctypes.data_as(dp), tp.ctypes.data_as(fp), ta.ctypes.data_as(dp), len(ta),
                                   out.ctypes.data_as(dp))
    return out


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not _PATH.exists():
        from em_lab_gb300 import _build
        _build.build_oracle()
    lib = C.CDLL(str(_PATH))
    I, F, D = C.c_int, C.c_float, C.c_double
    lib.oracle_expf.argtypes, lib.oracle_expf.restype = [F], F
    lib.oracle_float_to_half.argtypes, lib.oracle_float_to_half.restype = [F], C.c_uint16
    lib.oracle_half_to_float.argtypes, lib.oracle_half_to_float.restype = [C.c_uint16], F
    lib.oracle_set_threads.argtypes, lib.oracle_set_threads.restype = [I], None
    lib.oracle_max_threads.argtypes, lib.oracle_max_threads.restype = [], I
    lib.oracle_signal.argtypes, lib.oracle_signal.restype = [C.POINTER(abi.Source), D], D
    for suf, R in (("f32", C.c_float), ("f64", C.c_double)):
        for name, (args, res) in _grid_spec(R).items():
            fn = getattr(lib, f"{name}_{suf}")
            fn.argtypes, fn.restype = args, res
    _lib = lib
    return lib


def set_threads(n: int):
    load().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(load().oracle_max_threads())


def expf(x: float) -> float:
    return load().oracle_expf(float(x))


def float_to_half(x: float) -> int:
    return int(load().oracle_float_to_half(float(x)))


def source_signal(src, t: float) -> float:
    s = src.to_c() if hasattr(src, "to_c") else src
    return load().oracle_signal(C.byref(s), float(t))


class Oracle:
    """The reference's solver + monitors on the CPU (same methods as em_lab_gb300.SimulationGrid)."""

    def __init__(self, config: abi.GridConfig, precision: str = "f32"):
        self.precision = precision
        if precision in ("ref", "reflibm"):
            self._lib = load_ref()
            self._suf = "ref"
        else:
            self._lib = load()
            self._suf = "f64" if precision == "f64" else "f32"
        self.dtype = np.float64 if precision == "f64" else np.float32
        self._R = C.c_double if precision == "f64" else C.c_float
        cfg = abi.GridConfig()
        C.memmove(C.byref(cfg), C.byref(config), C.sizeof(cfg))
        self._h = self._fn("oracle_create")(C.byref(cfg), 1 if precision in ("f32libm", "reflibm") else 0)
        if not self._h:
            raise MemoryError("oracle allocation failed")
        self._nports = 0
        self._nq = 0

    def _fn(self, name):
        return getattr(self._lib, f"{name}_{self._suf}")

    def _rp(self, a):
        return a.ctypes.data_as(C.POINTER(self._R))

    def close(self):
        if getattr(self, "_h", None):
            self._fn("oracle_destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def config(self) -> abi.GridConfig:
        c = abi.GridConfig()
        self._fn("oracle_get_config")(self._h, C.byref(c))
        return c

    def size(self):
        c = self.config()
        return (c.nx, c.ny, c.nz)

    def step_count(self) -> int:
        return int(self._fn("oracle_step_count")(self._h))

    def source_cells(self) -> int:
        return int(self._fn("oracle_source_cells")(self._h))

    def upload_materials(self, sigma, eps_r, edges=(), wires=()):
        nx, ny, nz = self.size()
        s = np.ascontiguousarray(sigma, np.float32)
        e = np.ascontiguousarray(eps_r, np.float32)
        ea, ne = abi.array_of(abi.EdgeOverride, edges)
        wa, nw = abi.array_of(abi.WireTerm, wires)
        fp = C.POINTER(C.c_float)
        rc = self._fn("oracle_upload_materials")(self._h, s.ctypes.data_as(fp), e.ctypes.data_as(fp), nx, ny, nz,
                                                 ea, ne, wa, nw)
        if rc:
            raise ValueError(f"oracle upload_materials failed ({rc})")

    def edge_materials(self):
        nx, ny, nz = self.size()
        out = [np.empty((nz, ny, nx, 3), np.float32) for _ in range(4)]
        fp = C.POINTER(C.c_float)
        self._fn("oracle_edge_materials")(self._h, *[o.ctypes.data_as(fp) for o in out])
        return out

    def set_sources(self, sources):
        arr, n = abi.array_of(abi.Source, [s.to_c() if hasattr(s, "to_c") else s for s in sources])
        if self._fn("oracle_set_sources")(self._h, arr, n):
            raise MemoryError("oracle set_sources failed")

    def reset_fields(self):
        self._fn("oracle_reset_fields")(self._h)

    def step(self, count: int = 1):
        self._fn("oracle_step")(self._h, int(count))

    def read_components(self):
        nx, ny, nz = self.size()
        out = [np.empty((nz, ny, nx), self.dtype) for _ in range(6)]
        self._fn("oracle_read_components")(self._h, *[self._rp(o) for o in out])
        return out

    def write_components(self, comps):
        arrs = [np.ascontiguousarray(c, self.dtype) for c in comps]
        self._fn("oracle_write_components")(self._h, *[self._rp(a) for a in arrs])

    def ports_configure(self, ports, wavelength, averaging_periods=4.0, sweep=False, record_steps=0):
        arr, n = abi.array_of(abi.Port, ports)
        self._fn("oracle_ports_configure")(self._h, arr, n, float(wavelength), float(averaging_periods),
                                           1 if sweep else 0, int(record_steps))
        self._nports = n

    def ports_phasors(self):
        out = np.zeros((max(1, self._nports), 8), self.dtype)
        self._fn("oracle_ports_read_phasors")(self._h, self._rp(out))
        return out[: self._nports]

    def ports_series(self):
        n = self._fn("oracle_ports_read_series")(self._h, None, 0)
        out = np.zeros((max(1, n), max(1, self._nports), 2), self.dtype)
        self._fn("oracle_ports_read_series")(self._h, self._rp(out), n)
        return out[:n, : self._nports]

    def ports_sweep_sums(self, lambda_min, lambda_max, points):
        out = np.zeros((self._nports, points, 4), np.float64)
        res = C.c_double()
        self._fn("oracle_ports_sweep_sums")(self._h, float(lambda_min), float(lambda_max), int(points),
                                            out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(res))
        return out, res.value

    def ntff_configure(self, box_min, box_max, wavelength, averaging_periods=4.0):
        mn = (C.c_int * 3)(*[int(v) for v in box_min])
        mx = (C.c_int * 3)(*[int(v) for v in box_max])
        out = (C.c_int * 6)()
        rc = self._fn("oracle_ntff_configure")(self._h, mn, mx, float(wavelength), float(averaging_periods), out)
        if rc:
            raise ValueError("far_field box is degenerate")
        return tuple(out[:3]), tuple(out[3:])

    def ntff_point_count(self):
        return int(self._fn("oracle_ntff_point_count")(self._h))

    def ntff_phasors(self):
        n = self.ntff_point_count()
        out = np.zeros((max(1, n), 32), self.dtype)
        self._fn("oracle_ntff_read_phasors")(self._h, self._rp(out))
        return out[:n]

    def ntff_evaluate(self, directions):
        d = np.zeros((len(directions), 4), np.float32)
        d[:, :3] = np.asarray(directions, np.float32)[:, :3]
        out = np.zeros((len(directions), 2), self.dtype)
        self._fn("oracle_ntff_evaluate")(self._h, d.ctypes.data_as(C.POINTER(C.c_float)), len(d), self._rp(out))
        return out

    def ntff_dft_configure(self, box_min, box_max, wavelengths, block_steps=64):
        mn = (C.c_int * 3)(*[int(v) for v in box_min])
        mx = (C.c_int * 3)(*[int(v) for v in box_max])
        out = (C.c_int * 6)()
        wl = np.ascontiguousarray(wavelengths, np.float32)
        rc = self._fn("oracle_ntff_dft_configure")(self._h, mn, mx, wl.ctypes.data_as(C.POINTER(C.c_float)), len(wl), out)
        if rc:
            raise ValueError("far-field DFT box is degenerate")
        self._dft_nf = len(wl)
        return tuple(out[:3]), tuple(out[3:])

    def set_cpml(self, params=None):
        """The opt-in convolutional PML (sigma_max, kappa_max, alpha_max, order) or None for the
        reference absorber; clears the fields and the auxiliary fields as the library does."""
        if params is None:
            rc = self._fn("oracle_set_cpml")(self._h, 0, 0.0, 1.0, 0.0, 1.0)
        else:
            rc = self._fn("oracle_set_cpml")(self._h, 1, *[float(v) for v in params])
        if rc:
            raise MemoryError("oracle CPML set-up failed")

    def ntff_dft_info(self):
        """(box nodes, samples accumulated) like the device monitor's emlab_ntff_dft_info."""
        return int(self._fn("oracle_ntff_dft_points")(self._h)), None

    def ntff_dft_read(self):
        n = int(self._fn("oracle_ntff_dft_points")(self._h))
        out = np.zeros((self._dft_nf, n, 6, 2), np.float64)
        self._fn("oracle_ntff_dft_read")(self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def lines_configure(self, quantities, terms, weights, wavelength, averaging_periods=4.0):
        q = np.ascontiguousarray(np.asarray(quantities, np.int32).reshape(-1, 4))
        t = np.ascontiguousarray(np.asarray(terms, np.int32).reshape(-1, 4))
        w = np.ascontiguousarray(weights, np.float32)
        ip = C.POINTER(C.c_int)
        self._fn("oracle_lines_configure")(self._h, q.ctypes.data_as(ip), len(q), t.ctypes.data_as(ip),
                                           w.ctypes.data_as(C.POINTER(C.c_float)), len(t), float(wavelength),
                                           float(averaging_periods))
        self._nq = len(q)

    def lines_read(self):
        ph = np.zeros((max(1, self._nq), 4), self.dtype)
        now = np.zeros(max(1, self._nq), self.dtype)
        self._fn("oracle_lines_read")(self._h, self._rp(ph), self._rp(now))
        return ph[: self._nq], now[: self._nq]

    def probe_gather(self, origins):
        o = np.zeros((len(origins), 4), np.int32)
        o[:, :3] = np.asarray(origins, np.int32)[:, :3]
        out = np.zeros((len(origins), 54, 4), self.dtype)
        self._fn("oracle_probe_gather")(self._h, o.ctypes.data_as(C.POINTER(C.c_int)), len(o), self._rp(out))
        return out

    def flux_planes(self, planes):
        arr, n = abi.array_of(abi.FluxPlane, planes)
        out = np.zeros(max(1, n), np.float64)
        self._fn("oracle_flux_planes")(self._h, arr, n, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out[:n]


def load_scene(target, scene):
    """Uploads a Scene (em_lab_gb300.scene) into an Oracle or a SimulationGrid."""
    m = scene.materials
    target.upload_materials(m.sigma, m.epsilon_r, scene.edges, scene.wires)
    target.set_sources(scene.sources)


def render(e_rgba, b_rgba, params: abi.RenderParams, ref: bool = False) -> np.ndarray:
    """The volume pass (raymarch.frag) on the CPU: the restatement (oracle_render.h) or, with
    ref=True, the reference's own shader compiled through the GLSL shim (oracle/_ref). e_rgba and
    b_rgba are (nz, ny, nx, 4) float32 textures; returns (height, width, 4) uint8, bottom row first."""
    e = np.ascontiguousarray(e_rgba, np.float32)
    b = np.ascontiguousarray(b_rgba, np.float32)
    assert e.shape == b.shape and e.ndim == 4 and e.shape[3] == 4
    nz, ny, nx = e.shape[:3]
    lib = load_ref() if ref else load()
    fn = lib.oracle_render_ref if ref else lib.oracle_render
    fp = C.POINTER(C.c_float)
    fn.argtypes = [fp, fp, C.c_int, C.c_int, C.c_int, C.POINTER(abi.RenderParams), C.POINTER(C.c_ubyte)]
    fn.restype = C.c_int
    out = np.zeros((params.height, params.width, 4), np.uint8)
    rc = fn(e.ctypes.data_as(fp), b.ctypes.data_as(fp), nx, ny, nz, C.byref(params),
            out.ctypes.data_as(C.POINTER(C.c_ubyte)))
    if rc != 0:
        raise ValueError("oracle render: bad arguments")
    return out
