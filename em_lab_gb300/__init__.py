"""GB300-native FDTD time-stepping path of EM_Lab: a C ABI (include/emlab.h) over sm_103a CUDA
kernels, with Python mirrors of the reference's solver, scene and monitor interfaces."""
from . import abi
from .grid import EmlabError, SimulationGrid, device_expf, launch_count, library_path, load_library
from .scene import EnvironmentBuilder, Material, MaterialVolume, PortSetup, Scene, SourceDesc

__all__ = ["abi", "EmlabError", "SimulationGrid", "device_expf", "launch_count", "library_path", "load_library",
           "EnvironmentBuilder", "Material", "MaterialVolume", "PortSetup", "Scene", "SourceDesc"]
