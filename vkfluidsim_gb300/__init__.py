"""GB300-native WCSPH step of VkFluidSim: sm_103a CUDA kernels behind a C ABI.

The compute path is ``_lib/libvfs_cuda.so`` (built by ``vkfluidsim_gb300.build``); this package
only binds it. Importing works without a GPU; every model call needs the library and a device.
"""
from ._abi import LIB_PATH, VfsError, load_library, SHAPE_SPHERE, SHAPE_BOX, SHAPE_CONTAINER
from .model import (AnalyticObject, Batch, MeshObject, mesh_signed_distance, SimulationParameters, SPHParameters, WCSPHParameters,
                    WCSPHWithBoundaryModel, generate_fourier_velocity, generate_lattice,
                    generate_uniform_blob, load_scene, look_at, perspective, read_state,
                    render_density_raymarch, to_rgba8, tune_cache_clear, tune_cache_load,
                    tune_cache_save, write_ppm)

__all__ = [
    "LIB_PATH", "VfsError", "load_library", "SHAPE_SPHERE", "SHAPE_BOX", "SHAPE_CONTAINER",
    "AnalyticObject", "Batch", "MeshObject", "mesh_signed_distance", "SimulationParameters", "SPHParameters", "WCSPHParameters",
    "WCSPHWithBoundaryModel", "generate_fourier_velocity", "generate_lattice",
    "generate_uniform_blob", "load_scene", "look_at", "perspective", "read_state",
    "render_density_raymarch", "to_rgba8", "tune_cache_clear", "tune_cache_load",
    "tune_cache_save", "write_ppm",
]
