"""Python mirror of EM_Lab's solver interface over the native C ABI (include/emlab.h).

`SimulationGrid` keeps the member names and semantics of src/SimulationGrid.hpp:155-216
(configure, uploadMaterials, setSources, resetFields, step, time, dt, stepCount, size, config,
gpuMemoryBytes); the monitors attach to the grid and run inside `step` on the device.
The library is loaded from the package's own `_lib/` directory; there is no fallback: if it is
missing or no CUDA device is visible, construction raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import abi

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libemlab_gb300.so"
_lib = None


class EmlabError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"emlab error {code}: {message}")
        self.code = code


def library_path() -> Path:
    return _LIB_PATH


def load_library() -> C.CDLL:
    """Loads libemlab_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise RuntimeError(f"{_LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(_LIB_PATH))
    P, I, SZ, F, D = C.c_void_p, C.c_int, C.c_size_t, C.c_float, C.c_double
    fp, dp, ip = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int)
    sig = {
        "emlab_last_error": ([], C.c_char_p),
        "emlab_version": ([], I),
        "emlab_launch_count": ([], C.c_uint64),
        "emlab_grid_create": ([C.POINTER(P)], I),
        "emlab_grid_destroy": ([P], I),
        "emlab_grid_configure": ([P, C.POINTER(abi.GridConfig)], I),
        "emlab_grid_get_config": ([P, C.POINTER(abi.GridConfig)], I),
        "emlab_grid_upload_materials": ([P, fp, fp, I, I, I, C.POINTER(abi.EdgeOverride), SZ,
                                         C.POINTER(abi.WireTerm), SZ], I),
        "emlab_grid_set_sources": ([P, C.POINTER(abi.Source), SZ], I),
        "emlab_grid_reset_fields": ([P], I),
        "emlab_grid_step": ([P, I], I),
        "emlab_grid_synchronize": ([P, I], I),
        "emlab_grid_get_state": ([P, C.POINTER(abi.GridState)], I),
        "emlab_grid_read_fields": ([P, fp, fp], I),
        "emlab_grid_read_components": ([P, fp, fp, fp, fp, fp, fp], I),
        "emlab_grid_write_components": ([P, fp, fp, fp, fp, fp, fp], I),
        "emlab_grid_set_kernel": ([P, I], I),
        "emlab_grid_set_tiling": ([P, I], I),
        "emlab_grid_stream": ([P, C.POINTER(P)], I),
        "emlab_grid_field_ptr": ([P, C.POINTER(C.c_void_p), C.POINTER(I), C.POINTER(C.c_longlong)], I),
        "emlab_grid_check_finite": ([P], I),
        "emlab_grid_set_timing": ([P, I], I),
        "emlab_grid_kernel_time": ([P, dp, C.POINTER(C.c_uint64), I], I),
        "emlab_ports_configure": ([P, C.POINTER(abi.Port), SZ, F, F, I, SZ], I),
        "emlab_ports_read_phasors": ([P, fp], I),
        "emlab_ports_read_series": ([P, fp, SZ, C.POINTER(SZ)], I),
        "emlab_ports_sweep_sums": ([P, D, D, I, dp, dp], I),
        "emlab_ports_residuals": ([P, dp], I),
        "emlab_ntff_configure": ([P, ip, ip, F, F, ip], I),
        "emlab_ntff_point_count": ([P, ip], I),
        "emlab_ntff_read_phasors": ([P, fp], I),
        "emlab_ntff_evaluate": ([P, fp, I, fp], I),
        "emlab_ntff_dft_configure": ([P, ip, ip, fp, I, ip], I),
        "emlab_ntff_dft_info": ([P, ip, C.POINTER(C.c_uint64)], I),
        "emlab_ntff_dft_engine": ([P, I], I),
        "emlab_ntff_dft_read": ([P, dp], I),
        "emlab_ntff_dft_evaluate": ([P, I, fp, I, fp], I),
        "emlab_ntff_dft_evaluate_all": ([P, fp, I, fp], I),
        "emlab_ntff_dft_configure_boxes": ([P, ip, I, fp, I, I], I),
        "emlab_ntff_dft_spectra": ([P, I, fp, I, fp], I),
        "emlab_ntff_dft_pattern_gemm": ([P, I, fp, I, fp], I),
        "emlab_probe_gather": ([P, ip, I, fp], I),
        "emlab_flux_planes": ([P, C.POINTER(abi.FluxPlane), I, dp], I),
        "emlab_flux_planes_noalloc": ([P, C.POINTER(abi.FluxPlane), I, dp], I),
        "emlab_render": ([P, C.POINTER(abi.RenderParams), C.POINTER(C.c_ubyte)], I),
        "emlab_ports_take_series": ([P, fp, SZ, C.POINTER(SZ)], I),
        "emlab_analyzer_submit": ([P, ip, I, C.POINTER(abi.FluxPlane), I], I),
        "emlab_analyzer_collect": ([P, fp, dp, ip], I),
        "emlab_radar_backproject": ([C.POINTER(abi.RadarGeometry), fp, I, I, fp, dp, fp, dp, I, dp], I),
        "emlab_grid_set_graph": ([P, I], I),
        "emlab_stack_configure": ([P, C.POINTER(abi.GridConfig), ip, I], I),
        "emlab_stack_info": ([P, ip, ip, ip], I),
        "emlab_ports_take_series_async": ([P, ip, C.POINTER(SZ)], I),
        "emlab_ports_collect_series": ([P, I, fp, SZ, I], I),
        "emlab_stack_configure_scenes": ([P, C.POINTER(abi.GridConfig), ip, I], I),
        "emlab_stack_scene_dims": ([P, ip], I),
        "emlab_stack_upload_materials": ([P, I, fp, fp, I, I, I, C.POINTER(abi.EdgeOverride), SZ,
                                          C.POINTER(abi.WireTerm), SZ], I),
        "emlab_stack_commit": ([P], I),
        "emlab_stack_set_sources": ([P, C.POINTER(abi.Source), ip, SZ], I),
        "emlab_stack_compact": ([P, C.POINTER(C.c_ubyte)], I),
        "emlab_lines_configure": ([P, ip, I, ip, fp, I, F, F], I),
        "emlab_lines_read": ([P, fp, fp], I),
        "emlab_debug_expf": ([fp, fp, SZ], I),
        "emlab_debug_set_wait_limit": ([I], I),
        "emlab_debug_pair_schedule": ([I, I, I, I, I, ip, ip], I),
        "emlab_debug_ragged_items": ([ip, ip, ip, ip, I, I, I, ip, SZ, C.POINTER(SZ)], I),
        "emlab_grid_set_cpml": ([P, C.POINTER(abi.Cpml)], I),
        "emlab_edge_materials": ([fp, fp, I, I, I, C.POINTER(abi.EdgeOverride), SZ, C.POINTER(abi.WireTerm), SZ,
                                  fp, fp, fp, fp, C.POINTER(C.c_uint32)], I),
        "emlab_source_signal": ([C.POINTER(abi.Source), D], D),
        "emlab_source_lists": ([C.POINTER(abi.Source), SZ, I, I, I, fp, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                C.POINTER(I), C.POINTER(I), C.POINTER(I)], I),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _check(rc: int):
    if rc != abi.EMLAB_OK:
        raise EmlabError(rc, load_library().emlab_last_error().decode())


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


def _f32(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def launch_count() -> int:
    return int(load_library().emlab_launch_count())


WAIT_POLLS_DEFAULT = 1 << 20


def debug_set_wait_limit(polls: int) -> None:
    """Test hook: polls of an on-device barrier wait before a kernel gives up and the grid reports
    EMLAB_ERR_TIMEOUT (0: the first wait of every launch gives up; WAIT_POLLS_DEFAULT restores)."""
    _check(load_library().emlab_debug_set_wait_limit(int(polls)))


def pair_schedule(nx: int, ny: int, nz: int, tile_rows: int, ctas: int):
    """The persistent pair kernel's schedule on a single grid (host arithmetic): (planes per z chunk,
    work items)."""
    zc, items = C.c_int(), C.c_int()
    _check(load_library().emlab_debug_pair_schedule(int(nx), int(ny), int(nz), int(tile_rows), int(ctas),
                                                    C.byref(zc), C.byref(items)))
    return zc.value, items.value


def ragged_items(z0, nx, ny, nz, tile_rows: int, ctas: int) -> np.ndarray:
    """The persistent pair kernel's work items on a stack of scenes with their own cross-sections
    (host arithmetic): (items, 5) int32 rows (x0, y0, first plane, end plane, scene)."""
    arrs = [np.ascontiguousarray(v, np.int32) for v in (z0, nx, ny, nz)]
    ptr = [a.ctypes.data_as(C.POINTER(C.c_int)) for a in arrs]
    lib, n = load_library(), C.c_size_t()
    _check(lib.emlab_debug_ragged_items(*ptr, len(arrs[0]), int(tile_rows), int(ctas), None, 0, C.byref(n)))
    out = np.zeros((n.value, 5), np.int32)
    _check(lib.emlab_debug_ragged_items(*ptr, len(arrs[0]), int(tile_rows), int(ctas),
                                        out.ctypes.data_as(C.POINTER(C.c_int)), n.value, C.byref(n)))
    return out


def device_expf(x) -> np.ndarray:
    x = _f32(np.asarray(x).ravel())
    out = np.empty_like(x)
    _check(load_library().emlab_debug_expf(_fptr(x), _fptr(out), x.size))
    return out


def edge_materials(sigma, eps_r, edges=(), wires=()):
    """Host-side uploadMaterials arithmetic: (edge sigma, edge eps, wire0, wire1, classes), each
    array (nz, ny, nx, 3) as the solver sees it; needs no device."""
    sigma = np.asarray(sigma, np.float32)
    nz, ny, nx = sigma.shape
    s = _f32(sigma)
    e = _f32(eps_r, s.size)
    ea, ne = abi.array_of(abi.EdgeOverride, edges)
    wa, nw = abi.array_of(abi.WireTerm, wires)
    outs = [np.empty((nz, ny, nx, 3), np.float32) for _ in range(4)]
    classes = C.c_uint32()
    _check(load_library().emlab_edge_materials(_fptr(s), _fptr(e), nx, ny, nz, ea, ne, wa, nw,
                                               *[_fptr(o) for o in outs], C.byref(classes)))
    return (*outs, int(classes.value))


def source_lists(sources, size):
    """Host-side setSources arithmetic on a grid of `size` cells: (packed (k, 16) float32 source
    records, cells (m + 1, 4) int32 with the sentinel, lists int32); needs no device."""
    arr, n = abi.array_of(abi.Source, [s.to_c() if hasattr(s, "to_c") else s for s in sources])
    nx, ny, nz = (int(v) for v in size)
    ns, nc, nl = C.c_int(), C.c_int(), C.c_int()
    lib = load_library()
    _check(lib.emlab_source_lists(arr, n, nx, ny, nz, None, None, None, C.byref(ns), C.byref(nc), C.byref(nl)))
    packed = np.zeros((max(ns.value, 1), 16), np.float32)
    cells = np.zeros((nc.value + 1, 4), np.int32)
    lists = np.zeros(max(nl.value, 1), np.int32)
    i32 = C.POINTER(C.c_int32)
    _check(lib.emlab_source_lists(arr, n, nx, ny, nz, _fptr(packed), cells.ctypes.data_as(i32),
                                  lists.ctypes.data_as(i32), C.byref(ns), C.byref(nc), C.byref(nl)))
    return packed[:ns.value], cells, lists[:nl.value]


def source_signal(src, t: float) -> float:
    """SourceDesc::signal through the library (FP64)."""
    s = src.to_c() if hasattr(src, "to_c") else src
    return float(load_library().emlab_source_signal(C.byref(s), float(t)))


class SimulationGrid:
    """The FDTD solver (src/SimulationGrid.hpp:155-216) on one CUDA device."""

    kMaxSources = 256

    def __init__(self, config: abi.GridConfig | None = None):
        self._lib = load_library()
        h = C.c_void_p()
        _check(self._lib.emlab_grid_create(C.byref(h)))
        self._h = h
        self._sources = []
        if config is not None:
            self.configure(config)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.emlab_grid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # --- SimulationGrid ---------------------------------------------------------------------
    def configure(self, config: abi.GridConfig):
        cfg = abi.GridConfig()
        C.memmove(C.byref(cfg), C.byref(config), C.sizeof(cfg))
        _check(self._lib.emlab_grid_configure(self._h, C.byref(cfg)))

    def config(self) -> abi.GridConfig:
        cfg = abi.GridConfig()
        _check(self._lib.emlab_grid_get_config(self._h, C.byref(cfg)))
        return cfg

    def size(self):
        c = self.config()
        return (c.nx, c.ny, c.nz)

    def upload_materials(self, sigma, eps_r, edges=(), wires=()):
        """uploadMaterials: sigma/eps_r are (nz, ny, nx) cell arrays (MaterialVolume)."""
        nx, ny, nz = self.size()
        s = _f32(sigma, nx * ny * nz)
        e = _f32(eps_r, nx * ny * nz)
        ea, ne = abi.array_of(abi.EdgeOverride, edges)
        wa, nw = abi.array_of(abi.WireTerm, wires)
        _check(self._lib.emlab_grid_upload_materials(self._h, _fptr(s), _fptr(e), nx, ny, nz, ea, ne, wa, nw))

    def set_sources(self, sources):
        arr, n = abi.array_of(abi.Source, [s.to_c() if hasattr(s, "to_c") else s for s in sources])
        _check(self._lib.emlab_grid_set_sources(self._h, arr, n))
        self._sources = list(sources)

    def sources(self):
        return list(self._sources)

    def reset_fields(self):
        _check(self._lib.emlab_grid_reset_fields(self._h))

    def step(self, count: int = 1, after_each_step=None):
        """step(count, afterEachStep): attached monitors run on the device inside every step; a
        Python callback, if given, runs on the host after each completed step."""
        if after_each_step is None:
            _check(self._lib.emlab_grid_step(self._h, int(count)))
            return
        for _ in range(int(count)):
            _check(self._lib.emlab_grid_step(self._h, 1))
            after_each_step()

    def synchronize(self, timeout_ms: int = 0):
        _check(self._lib.emlab_grid_synchronize(self._h, int(timeout_ms)))

    def state(self) -> abi.GridState:
        st = abi.GridState()
        _check(self._lib.emlab_grid_get_state(self._h, C.byref(st)))
        return st

    def time(self) -> float:
        return self.state().time

    def dt(self) -> float:
        return self.config().courant

    def step_count(self) -> int:
        return int(self.state().step_count)

    def gpu_memory_bytes(self) -> int:
        return int(self.state().device_bytes)

    def set_kernel(self, kernel: int):
        _check(self._lib.emlab_grid_set_kernel(self._h, int(kernel)))

    def set_cpml(self, params=None):
        """The opt-in convolutional PML: (sigma_max, kappa_max, alpha_max, order), or None for the
        reference's graded absorber. Clears the fields, the auxiliary fields and time."""
        if params is None:
            _check(self._lib.emlab_grid_set_cpml(self._h, None))
        else:
            p = abi.Cpml(*[float(v) for v in params])
            _check(self._lib.emlab_grid_set_cpml(self._h, C.byref(p)))

    def set_tiling(self, tile_rows: int):
        """Tile height of the fused kernels (8, 16, or 0 = automatic); results do not depend on it."""
        _check(self._lib.emlab_grid_set_tiling(self._h, int(tile_rows)))

    def set_graph(self, chunk: int):
        """Replay chunks of exactly `chunk` steps as captured CUDA graphs (0: off); same results."""
        _check(self._lib.emlab_grid_set_graph(self._h, int(chunk)))

    def stream_handle(self) -> int:
        p = C.c_void_p()
        _check(self._lib.emlab_grid_stream(self._h, C.byref(p)))
        return int(p.value or 0)

    def field_pointers(self):
        """(six device addresses Ex..Bz, row pitch, plane stride) of the current generation
        (emlab_grid_field_ptr); valid until the next step, reset or configure."""
        ptrs = (C.c_void_p * 6)()
        pitch = C.c_int()
        plane = C.c_longlong()
        _check(self._lib.emlab_grid_field_ptr(self._h, ptrs, C.byref(pitch), C.byref(plane)))
        return [int(p or 0) for p in ptrs], int(pitch.value), int(plane.value)

    def field_tensors(self):
        """Zero-copy torch views (nz, ny, nx) of Ex, Ey, Ez, Bx, By, Bz on the grid's device
        through __cuda_array_interface__; the grid's queued work is waited for first. Valid until
        the next step, reset or configure."""
        import torch

        self.synchronize()
        ptrs, pitch, plane = self.field_pointers()
        nx, ny, nz = self.size()

        class _View:
            def __init__(self, ptr):
                self.__cuda_array_interface__ = {"shape": (nz, ny, nx), "typestr": "<f4", "data": (ptr, False),
                                                 "strides": (plane * 4, pitch * 4, 4), "version": 2}

        dev = torch.device("cuda", torch.cuda.current_device())
        return [torch.as_tensor(_View(p), device=dev) for p in ptrs]

    def set_timing(self, enabled: bool):
        _check(self._lib.emlab_grid_set_timing(self._h, 1 if enabled else 0))

    def kernel_time(self, reset: bool = False):
        """(accumulated device ms of the solver launches, number of timed launches)."""
        ms = C.c_double()
        n = C.c_uint64()
        _check(self._lib.emlab_grid_kernel_time(self._h, C.byref(ms), C.byref(n), 1 if reset else 0))
        return ms.value, int(n.value)

    def check_finite(self) -> bool:
        rc = self._lib.emlab_grid_check_finite(self._h)
        if rc == abi.EMLAB_ERR_NONFINITE:
            return False
        _check(rc)
        return True

    # --- field access -----------------------------------------------------------------------
    def read_components(self):
        """(Ex, Ey, Ez, Bx, By, Bz), each (nz, ny, nx) float32."""
        nx, ny, nz = self.size()
        out = [np.empty((nz, ny, nx), np.float32) for _ in range(6)]
        _check(self._lib.emlab_grid_read_components(self._h, *[_fptr(o) for o in out]))
        return out

    def read_textures(self):
        """The E and B textures (nz, ny, nx, 4) in the reference's RGBA32F layout."""
        nx, ny, nz = self.size()
        e = np.empty((nz, ny, nx, 4), np.float32)
        b = np.empty((nz, ny, nx, 4), np.float32)
        _check(self._lib.emlab_grid_read_fields(self._h, _fptr(e), _fptr(b)))
        return e, b

    def write_components(self, comps):
        nx, ny, nz = self.size()
        arrs = [None if c is None else _f32(c, nx * ny * nz) for c in comps]
        _check(self._lib.emlab_grid_write_components(self._h, *[_fptr(a) for a in arrs]))

    # --- monitors (device side) -------------------------------------------------------------
    def ports_configure(self, ports, wavelength, averaging_periods=4.0, sweep=False, record_steps=0):
        arr, n = abi.array_of(abi.Port, ports)
        _check(self._lib.emlab_ports_configure(self._h, arr, n, float(wavelength), float(averaging_periods),
                                               1 if sweep else 0, int(record_steps)))
        self._nports = n

    def ports_phasors(self) -> np.ndarray:
        out = np.zeros((max(1, getattr(self, "_nports", 0)), 8), np.float32)
        _check(self._lib.emlab_ports_read_phasors(self._h, _fptr(out)))
        return out[: getattr(self, "_nports", 0)]

    def ports_series(self) -> np.ndarray:
        steps = C.c_size_t()
        _check(self._lib.emlab_ports_read_series(self._h, None, 0, C.byref(steps)))
        n = getattr(self, "_nports", 0)
        out = np.zeros((max(1, steps.value), max(1, n), 2), np.float32)
        _check(self._lib.emlab_ports_read_series(self._h, _fptr(out), steps.value, C.byref(steps)))
        return out[: steps.value, :n]

    def analyzer_submit(self, origins, planes):
        """FieldAnalyzer::submit: queue probe gathers and flux planes; returns at once."""
        o = np.zeros((max(1, len(origins)), 4), np.int32)
        if len(origins):
            o[: len(origins), :3] = np.asarray(origins, np.int32)[:, :3]
        arr, n = abi.array_of(abi.FluxPlane, planes)
        _check(self._lib.emlab_analyzer_submit(self._h, o.ctypes.data_as(C.POINTER(C.c_int)), len(origins), arr, n))
        self._analyzer = getattr(self, "_analyzer", []) + [(len(origins), n)]

    def analyzer_collect(self):
        """FieldAnalyzer::collect: (probe blocks (n, 54, 4), flux sums (m,)) of the oldest queued
        measurement, or None when nothing is pending."""
        q = getattr(self, "_analyzer", [])
        if not q:
            return None
        npr, npl = q[0]
        probe = np.zeros((max(1, npr), 54, 4), np.float32)
        flux = np.zeros(max(1, npl), np.float64)
        ready = C.c_int()
        _check(self._lib.emlab_analyzer_collect(self._h, _fptr(probe), flux.ctypes.data_as(C.POINTER(C.c_double)),
                                                C.byref(ready)))
        self._analyzer = q[1:]
        return probe[:npr], flux[:npl]

    def ports_recorded(self) -> int:
        """Steps recorded so far (PortMonitor::recordedSteps)."""
        steps = C.c_size_t()
        _check(self._lib.emlab_ports_read_series(self._h, None, 0, C.byref(steps)))
        return int(steps.value)

    def ports_take_series(self, max_steps: int) -> np.ndarray:
        """The steps recorded since the last take (at most max_steps), (steps, ports, 2); recording
        restarts at the start of the buffer."""
        n = getattr(self, "_nports", 0)
        out = np.zeros((max(1, int(max_steps)), max(1, n), 2), np.float32)
        steps = C.c_size_t()
        _check(self._lib.emlab_ports_take_series(self._h, _fptr(out), int(max_steps), C.byref(steps)))
        return out[: steps.value, :n]

    def ports_take_series_async(self):
        """Queues the copy of the steps recorded since the last take; returns (slot, steps) for
        ports_collect_series. Recording restarts at the start of the buffer."""
        slot, steps = C.c_int(), C.c_size_t()
        _check(self._lib.emlab_ports_take_series_async(self._h, C.byref(slot), C.byref(steps)))
        return slot.value, steps.value

    def ports_collect_series(self, slot: int, steps: int, timeout_ms: int = 0) -> np.ndarray:
        """Waits for a queued take and returns its (steps, ports, 2) series."""
        n = getattr(self, "_nports", 0)
        out = np.zeros((max(1, int(steps)), max(1, n), 2), np.float32)
        _check(self._lib.emlab_ports_collect_series(self._h, int(slot), _fptr(out), int(steps), int(timeout_ms)))
        return out[: int(steps), :n]

    def ports_sweep_sums(self, lambda_min, lambda_max, points):
        n = getattr(self, "_nports", 0)
        out = np.zeros((n, points, 4), np.float64)
        res = C.c_double()
        _check(self._lib.emlab_ports_sweep_sums(self._h, float(lambda_min), float(lambda_max), int(points),
                                                out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(res)))
        return out, res.value

    def ports_residuals(self):
        """Per port, the reference's ring-down residual of the recorded series (on the device)."""
        n = getattr(self, "_nports", 0)
        out = np.zeros(n, np.float64)
        _check(self._lib.emlab_ports_residuals(self._h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def ntff_configure(self, box_min, box_max, wavelength, averaging_periods=4.0):
        mn = (C.c_int * 3)(*[int(v) for v in box_min])
        mx = (C.c_int * 3)(*[int(v) for v in box_max])
        out = (C.c_int * 6)()
        _check(self._lib.emlab_ntff_configure(self._h, mn, mx, float(wavelength), float(averaging_periods), out))
        return tuple(out[:3]), tuple(out[3:])

    def ntff_point_count(self) -> int:
        p = C.c_int()
        _check(self._lib.emlab_ntff_point_count(self._h, C.byref(p)))
        return p.value

    def ntff_phasors(self) -> np.ndarray:
        n = self.ntff_point_count()
        out = np.zeros((max(1, n), 32), np.float32)
        _check(self._lib.emlab_ntff_read_phasors(self._h, _fptr(out)))
        return out[:n]

    def ntff_evaluate(self, directions) -> np.ndarray:
        d = np.zeros((len(directions), 4), np.float32)
        d[:, :3] = np.asarray(directions, np.float32)[:, :3]
        out = np.zeros((len(directions), 2), np.float32)
        _check(self._lib.emlab_ntff_evaluate(self._h, _fptr(d), len(d), _fptr(out)))
        return out

    def ntff_dft_configure(self, box_min, box_max, wavelengths):
        mn = (C.c_int * 3)(*[int(v) for v in box_min])
        mx = (C.c_int * 3)(*[int(v) for v in box_max])
        out = (C.c_int * 6)()
        wl = _f32(wavelengths)
        _check(self._lib.emlab_ntff_dft_configure(self._h, mn, mx, _fptr(wl), len(wl), out))
        self._dft_nf = len(wl)
        return tuple(out[:3]), tuple(out[3:])

    def ntff_dft_engine(self, engine: int):
        """abi.DFT_TENSOR (tcgen05 split-precision TF32, the default) or abi.DFT_CUDA_CORES."""
        _check(self._lib.emlab_ntff_dft_engine(self._h, int(engine)))

    def ntff_dft_info(self):
        p = C.c_int()
        n = C.c_uint64()
        _check(self._lib.emlab_ntff_dft_info(self._h, C.byref(p), C.byref(n)))
        return p.value, int(n.value)

    def ntff_dft_read(self) -> np.ndarray:
        points, _ = self.ntff_dft_info()
        out = np.zeros((self._dft_nf, points, 6, 2), np.float64)
        _check(self._lib.emlab_ntff_dft_read(self._h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def ntff_dft_evaluate(self, f, directions) -> np.ndarray:
        d = np.zeros((len(directions), 4), np.float32)
        d[:, :3] = np.asarray(directions, np.float32)[:, :3]
        out = np.zeros((len(directions), 2), np.float32)
        _check(self._lib.emlab_ntff_dft_evaluate(self._h, int(f), _fptr(d), len(d), _fptr(out)))
        return out

    def ntff_dft_evaluate_all(self, directions) -> np.ndarray:
        """(frequencies, directions, 2): the pattern at every configured frequency (fast surface
        phases; see emlab_ntff_dft_evaluate_all)."""
        d = np.zeros((len(directions), 4), np.float32)
        d[:, :3] = np.asarray(directions, np.float32)[:, :3]
        out = np.zeros((self._dft_nf, len(directions), 2), np.float32)
        _check(self._lib.emlab_ntff_dft_evaluate_all(self._h, _fptr(d), len(d), _fptr(out)))
        return out

    def ntff_dft_configure_boxes(self, boxes, wavelengths, block: int = 0):
        """The far-field DFT on several boxes ((k, 6) ints: min xyz, max xyz each, not clamped);
        block: samples per fold at most (0: the engine's own)."""
        b = np.ascontiguousarray(np.asarray(boxes, np.int32).reshape(-1, 6))
        wl = _f32(wavelengths)
        _check(self._lib.emlab_ntff_dft_configure_boxes(self._h, b.ctypes.data_as(C.POINTER(C.c_int)), len(b),
                                                        _fptr(wl), len(wl), int(block)))
        self._dft_nf = len(wl) if len(b) else 0

    def ntff_dft_spectra(self, box: int, directions) -> np.ndarray:
        """(frequencies, directions, 2) of one box of several, as ntff_dft_evaluate_all."""
        d = np.zeros((len(directions), 4), np.float32)
        d[:, :3] = np.asarray(directions, np.float32)[:, :3]
        out = np.zeros((self._dft_nf, len(directions), 2), np.float32)
        _check(self._lib.emlab_ntff_dft_spectra(self._h, int(box), _fptr(d), len(d), _fptr(out)))
        return out

    def ntff_dft_pattern_gemm(self, box: int, directions) -> np.ndarray:
        """(frequencies, directions, 2) as ntff_dft_spectra, the sums factorised into per-face
        tensor-core GEMMs (emlab_ntff_dft_pattern_gemm)."""
        d = np.zeros((len(directions), 4), np.float32)
        d[:, :3] = np.asarray(directions, np.float32)[:, :3]
        out = np.zeros((self._dft_nf, len(directions), 2), np.float32)
        _check(self._lib.emlab_ntff_dft_pattern_gemm(self._h, int(box), _fptr(d), len(d), _fptr(out)))
        return out

    def probe_gather(self, origins) -> np.ndarray:
        o = np.zeros((len(origins), 4), np.int32)
        o[:, :3] = np.asarray(origins, np.int32)[:, :3]
        out = np.zeros((len(origins), 54, 4), np.float32)
        _check(self._lib.emlab_probe_gather(self._h, o.ctypes.data_as(C.POINTER(C.c_int)), len(o), _fptr(out)))
        return out

    def flux_planes(self, planes) -> np.ndarray:
        arr, n = abi.array_of(abi.FluxPlane, planes)
        out = np.zeros(max(1, n), np.float64)
        _check(self._lib.emlab_flux_planes(self._h, arr, n, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out[:n]

    def flux_planes_noalloc(self, planes) -> np.ndarray:
        """flux_planes without device allocation, for callers that must not allocate: scratch is a
        fixed device array (at most 64 planes / 65536 workgroup partials) shared by all calls."""
        arr, n = abi.array_of(abi.FluxPlane, planes)
        out = np.zeros(max(1, n), np.float64)
        _check(self._lib.emlab_flux_planes_noalloc(self._h, arr, n, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out[:n]

    def render(self, params: abi.RenderParams) -> np.ndarray:
        """Ray-marched RGBA8 image of the current fields, (height, width, 4), rows bottom-up."""
        out = np.zeros((params.height, params.width, 4), np.uint8)
        _check(self._lib.emlab_render(self._h, C.byref(params), out.ctypes.data_as(C.POINTER(C.c_ubyte))))
        return out

    def lines_configure(self, quantities, terms, weights, wavelength, averaging_periods=4.0):
        q = np.ascontiguousarray(np.asarray(quantities, np.int32).reshape(-1, 4))
        t = np.ascontiguousarray(np.asarray(terms, np.int32).reshape(-1, 4))
        w = _f32(weights)
        _check(self._lib.emlab_lines_configure(self._h, q.ctypes.data_as(C.POINTER(C.c_int)), len(q),
                                               t.ctypes.data_as(C.POINTER(C.c_int)), _fptr(w), len(t),
                                               float(wavelength), float(averaging_periods)))
        self._nq = len(q)

    def lines_read(self):
        n = getattr(self, "_nq", 0)
        ph = np.zeros((max(1, n), 4), np.float32)
        now = np.zeros(max(1, n), np.float32)
        _check(self._lib.emlab_lines_read(self._h, _fptr(ph), _fptr(now)))
        return ph[:n], now[:n]




class SceneStack(SimulationGrid):
    """Independent scenes stepped as one grid (emlab_stack_*): scene i occupies planes z0[i] ..
    z0[i] + nz[i] - 1 with a frozen separator plane between scenes, and evolves bit for bit as it
    would on a SimulationGrid of its own. Scenes of equal nx x ny (`scene_nz`: their depths) or of
    their own cross-sections (`scene_dims`: (nx, ny, nz) each; every scene at x = y = 0 of its planes,
    the rest of the planes frozen). Materials and sources are given per scene in the scene's own
    coordinates; ports are attached in stack planes (scene z + z0)."""

    def __init__(self, config: abi.GridConfig, scene_nz=None, scene_dims=None):
        super().__init__(None)
        cfg = abi.GridConfig()
        C.memmove(C.byref(cfg), C.byref(config), C.sizeof(cfg))
        if scene_dims is not None:
            d = [int(v) for t in scene_dims for v in t]
            arr = (C.c_int * len(d))(*d)
            _check(self._lib.emlab_stack_configure_scenes(self._h, C.byref(cfg), arr, len(d) // 3))
        else:
            nz = (C.c_int * len(scene_nz))(*[int(v) for v in scene_nz])
            _check(self._lib.emlab_stack_configure(self._h, C.byref(cfg), nz, len(scene_nz)))

    def scene_dims(self):
        """(nx, ny, nz) of every scene now in the stack."""
        n = self.scenes()
        out = (C.c_int * max(3, 3 * n))()
        _check(self._lib.emlab_stack_scene_dims(self._h, out))
        return [tuple(out[3 * i: 3 * i + 3]) for i in range(n)]

    def layout(self):
        """(z0, nz) lists of the scenes now in the stack."""
        n = C.c_int()
        _check(self._lib.emlab_stack_info(self._h, C.byref(n), None, None))
        z0 = (C.c_int * max(1, n.value))()
        nz = (C.c_int * max(1, n.value))()
        _check(self._lib.emlab_stack_info(self._h, C.byref(n), z0, nz))
        return list(z0[: n.value]), list(nz[: n.value])

    def scenes(self) -> int:
        return len(self.layout()[0])

    def upload_scene_materials(self, scene: int, sigma, eps_r, edges=(), wires=()):
        nz_s, ny, nx = np.asarray(sigma).shape
        s = _f32(sigma)
        e = _f32(eps_r, s.size)
        ea, ne = abi.array_of(abi.EdgeOverride, edges)
        wa, nw = abi.array_of(abi.WireTerm, wires)
        _check(self._lib.emlab_stack_upload_materials(self._h, int(scene), _fptr(s), _fptr(e), nx, ny, nz_s, ea, ne,
                                                      wa, nw))

    def commit(self):
        _check(self._lib.emlab_stack_commit(self._h))

    def set_scene_sources(self, per_scene):
        """per_scene[i]: the sources of scene i (scene coordinates)."""
        flat, owner = [], []
        for i, srcs in enumerate(per_scene):
            for sdesc in srcs:
                flat.append(sdesc.to_c() if hasattr(sdesc, "to_c") else sdesc)
                owner.append(i)
        arr, n = abi.array_of(abi.Source, flat)
        own = (C.c_int * max(1, n))(*owner)
        _check(self._lib.emlab_stack_set_sources(self._h, arr, own, n))

    def compact(self, keep):
        k = (C.c_ubyte * len(keep))(*[1 if v else 0 for v in keep])
        _check(self._lib.emlab_stack_compact(self._h, k))
        self._nports = 0

    def scene_components(self, scene: int, comps=None):
        """The six components of one scene, each (nz_i, ny_i, nx_i)."""
        z0, nz = self.layout()
        nx, ny, _ = self.scene_dims()[scene]
        comps = self.read_components() if comps is None else comps
        return [c[z0[scene]: z0[scene] + nz[scene], :ny, :nx] for c in comps]
