"""ctypes mirrors of the structs declared in include/emlab.h (the C ABI of the solver)."""
from __future__ import annotations

import ctypes as C

EMLAB_OK = 0
EMLAB_ERR_INVALID = 1
EMLAB_ERR_OOM = 2
EMLAB_ERR_CUDA = 3
EMLAB_ERR_TIMEOUT = 4
EMLAB_ERR_NONFINITE = 5
EMLAB_ERR_NO_DEVICE = 6

KERNEL_FUSED = 0
KERNEL_SPLIT = 1
KERNEL_FUSED_LDG = 2
DFT_TENSOR = 0
DFT_CUDA_CORES = 1

WAVE_CW = 0
WAVE_PULSE = 1

# fixed scratch of emlab_flux_planes_noalloc
FLUX_NOALLOC_MAX_PLANES = 64
FLUX_NOALLOC_MAX_PARTIALS = 65536


class GridConfig(C.Structure):
    """GridConfig (src/SimulationGrid.hpp:25-31); defaults are the reference's."""

    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("courant", C.c_float),
                ("pml_thickness", C.c_int), ("pml_sigma_max", C.c_float), ("pml_grading", C.c_float)]

    def __init__(self, size=(128, 128, 128), courant=0.5, pml_thickness=16, pml_sigma_max=1.6, pml_grading=3.0):
        super().__init__(int(size[0]), int(size[1]), int(size[2]), float(courant), int(pml_thickness),
                         float(pml_sigma_max), float(pml_grading))

    @property
    def size(self):
        return (self.nx, self.ny, self.nz)

    def as_tuple(self):
        return (self.nx, self.ny, self.nz, self.courant, self.pml_thickness, self.pml_sigma_max, self.pml_grading)


class EdgeOverride(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int), ("axis", C.c_int), ("sigma", C.c_float)]


class WireTerm(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int), ("component", C.c_int), ("term", C.c_int),
                ("factor", C.c_float)]


class Source(C.Structure):
    """SourceDesc (src/SimulationGrid.hpp:113-150), solver-facing fields."""

    _fields_ = [("center", C.c_float * 3), ("half_extent", C.c_float * 3), ("softness", C.c_float * 3),
                ("polarization", C.c_float * 3), ("amplitude", C.c_float), ("wavelength", C.c_float),
                ("phase", C.c_float), ("waveform", C.c_int), ("ramp_periods", C.c_float),
                ("repeat_periods", C.c_float), ("delay_periods", C.c_float), ("enabled", C.c_int)]


class Cpml(C.Structure):
    """emlab_cpml: the opt-in convolutional PML's grading."""
    _fields_ = [("sigma_max", C.c_float), ("kappa_max", C.c_float), ("alpha_max", C.c_float), ("order", C.c_float)]


class Port(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int), ("axis", C.c_int), ("edges", C.c_int),
                ("sign", C.c_int)]


class FluxPlane(C.Structure):
    _fields_ = [("axis", C.c_int), ("index", C.c_int), ("rect_min", C.c_int * 2), ("rect_max", C.c_int * 2)]


class RenderParams(C.Structure):
    """emlab_render_params: camera and look of one rendered frame."""
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("inv_view_proj", C.c_float * 16),
                ("cam_pos", C.c_float * 3), ("vol_min", C.c_float * 3), ("vol_size", C.c_float * 3),
                ("clip_min", C.c_float * 3), ("clip_max", C.c_float * 3), ("step_voxels", C.c_float),
                ("gain_e", C.c_float), ("gain_b", C.c_float), ("density", C.c_float), ("emission", C.c_float),
                ("material_opacity", C.c_float), ("exposure", C.c_float), ("mode", C.c_int), ("signed_axis", C.c_int)]


class RadarGeometry(C.Structure):
    """emlab_radar_geometry: the back-projection image grid and array frame."""
    _fields_ = [("tx", C.c_float * 3), ("axes", C.c_float * 9), ("interior_min", C.c_float * 3),
                ("interior_max", C.c_float * 3), ("omega", C.c_double), ("dt", C.c_double), ("sample_dt", C.c_double),
                ("r0", C.c_float), ("dr", C.c_float), ("az0", C.c_float), ("daz", C.c_float), ("el0", C.c_float),
                ("del_", C.c_float), ("nr", C.c_int), ("naz", C.c_int), ("nel", C.c_int)]


class GridState(C.Structure):
    _fields_ = [("time", C.c_double), ("dt", C.c_float), ("step_count", C.c_uint64), ("nx", C.c_int),
                ("ny", C.c_int), ("nz", C.c_int), ("device_bytes", C.c_uint64), ("source_cells", C.c_int),
                ("kernel", C.c_int)]


def array_of(struct, items):
    items = list(items)
    arr = (struct * max(1, len(items)))()
    for i, it in enumerate(items):
        arr[i] = it
    return arr, len(items)
