"""ctypes declarations of ``include/vfs_cuda.h`` (the C ABI of the CUDA library).

Loading fails loudly when the in-tree library has not been built: there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libvfs_cuda.so"

VFS_OK = 0
STATUS_NAMES = {
    1: "VFS_ERR_INVALID_ARGUMENT",
    2: "VFS_ERR_CUDA",
    3: "VFS_ERR_OUT_OF_MEMORY",
    4: "VFS_ERR_IO",
    5: "VFS_ERR_PARSE",
    6: "VFS_ERR_CAPACITY",
    7: "VFS_ERR_DEVICE_CHECK",
    8: "VFS_ERR_NOT_READY",
}

SHAPE_SPHERE, SHAPE_BOX, SHAPE_CONTAINER = 0, 1, 2


class VfsError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


class SimParams(C.Structure):
    _fields_ = [("gravity", C.c_float * 3), ("smooth_radius", C.c_float)]


class SphParams(C.Structure):
    _fields_ = [
        ("time_scale", C.c_float),
        ("iterations", C.c_int32),
        ("n_particles", C.c_int32),
        ("fixed_dt", C.c_float),
        ("target_density", C.c_float),
        ("bbox_size", C.c_float * 3),
        ("bbox_pos", C.c_float * 3),
    ]


class WcsphParams(C.Structure):
    _fields_ = [
        ("wall_stiffness", C.c_float),
        ("stiffness", C.c_float),
        ("expoent", C.c_float),
        ("viscosity_strenght", C.c_float),
    ]


class BoundaryObject(C.Structure):
    _fields_ = [
        ("transform", C.c_float * 16),
        ("rotation", C.c_float * 16),
        ("box_size", C.c_float * 3),
        ("box_pos", C.c_float * 3),
        ("resolution", C.c_uint32 * 3),
        ("sdf_grid", C.POINTER(C.c_float)),
        ("volume_map_grid", C.POINTER(C.c_float)),
    ]


class AnalyticObject(C.Structure):
    _fields_ = [
        ("shape", C.c_int32),
        ("params", C.c_double * 3),
        ("position", C.c_float * 3),
        ("rotation_angle_deg", C.c_float),
        ("rotation_axis", C.c_float * 3),
        ("scale", C.c_float * 3),
        ("resolution", C.c_uint32 * 3),
    ]


_P = C.c_void_p
_F = C.POINTER(C.c_float)
_U = C.POINTER(C.c_uint32)
_I = C.c_int
_U32 = C.c_uint32

# name -> (restype, argtypes)
class MeshObject(C.Structure):
    _fields_ = [
        ("obj_path", C.c_char_p),
        ("vertices", C.POINTER(C.c_float)),
        ("n_vertices", C.c_uint32),
        ("triangles", C.POINTER(C.c_uint32)),
        ("n_triangles", C.c_uint32),
        ("position", C.c_float * 3),
        ("rotation_angle_deg", C.c_float),
        ("rotation_axis", C.c_float * 3),
        ("scale", C.c_float * 3),
        ("resolution", C.c_uint32 * 3),
    ]


class TuneConfig(C.Structure):
    _fields_ = [("sort_digit_bits", C.c_int32), ("sort_tile_items", C.c_int32),
                ("nbr_block", C.c_int32), ("nbr_min_blocks", C.c_int32), ("cell_block", C.c_int32),
                ("force_block", C.c_int32), ("force_min_blocks", C.c_int32),
                ("walk_staging", C.c_int32)]


SIGNATURES = {
    "vfs_last_error": (C.c_char_p, []),
    "vfs_version": (C.c_char_p, []),
    "vfs_device_count": (_I, []),
    "vfs_model_create": (_I, [C.POINTER(SimParams), C.POINTER(SphParams), C.POINTER(WcsphParams), C.POINTER(_P)]),
    "vfs_model_destroy": (_I, [_P]),
    "vfs_model_set_stream": (_I, [_P, _P]),
    "vfs_model_set_parameters": (_I, [_P, C.POINTER(SimParams), C.POINTER(SphParams), C.POINTER(WcsphParams)]),
    "vfs_model_get_parameters": (_I, [_P, C.POINTER(SimParams), C.POINTER(SphParams), C.POINTER(WcsphParams)]),
    "vfs_model_num_particles": (_U32, [_P]),
    "vfs_model_add_boundary_object": (_I, [_P, C.POINTER(BoundaryObject)]),
    "vfs_model_add_analytic_object": (_I, [_P, C.POINTER(AnalyticObject)]),
    "vfs_model_num_boundary_objects": (_U32, [_P]),
    "vfs_model_get_boundary_object": (_I, [_P, _U32, C.POINTER(BoundaryObject), _F, _F]),
    "vfs_model_set_particle_state": (_I, [_P, _F, _F, _U32, C.c_int64]),
    "vfs_model_set_particles_in_box": (_I, [_P, _F, _F, _U32, C.c_int64, C.c_int32, C.c_uint64]),
    "vfs_model_copy_data_buffers": (_I, [_P, _F, _F, _F, _F]),
    "vfs_model_step_host": (_I, [_P, _F, _F, _I, _F, _F, _F]),
    "vfs_model_get_ids": (_I, [_P, _U]),
    "vfs_model_get_neighbor_arrays": (_I, [_P, _U, _U, _U]),
    "vfs_model_get_boundary_fields": (_I, [_P, _F, _F]),
    "vfs_model_record_fields": (_I, [_P, C.c_int32]),
    "vfs_model_step": (_I, [_P]),
    "vfs_model_substeps": (_I, [_P, C.c_int32]),
    "vfs_model_use_graph": (_I, [_P, C.c_int32]),
    "vfs_model_synchronize": (_I, [_P]),
    "vfs_model_profile_substeps": (_I, [_P, C.c_int32, _F]),
    "vfs_model_set_sort_config": (_I, [_P, C.c_int32, C.c_int32]),
    "vfs_model_get_sort_config": (_I, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "vfs_model_device_state": (_I, [_P, C.POINTER(_P), C.POINTER(_P)]),
    "vfs_batch_create": (_I, [C.c_int32, C.POINTER(SimParams), C.POINTER(SphParams), C.POINTER(WcsphParams), C.POINTER(_P)]),
    "vfs_batch_destroy": (_I, [_P]),
    "vfs_batch_num_scenes": (C.c_int32, [_P]),
    "vfs_batch_num_particles": (_U32, [_P, C.c_int32]),
    "vfs_batch_set_stream": (_I, [_P, _P]),
    "vfs_batch_set_scene_parameters": (_I, [_P, C.c_int32, C.POINTER(SimParams), C.POINTER(SphParams), C.POINTER(WcsphParams)]),
    "vfs_batch_add_boundary_object": (_I, [_P, C.c_int32, C.POINTER(BoundaryObject)]),
    "vfs_batch_add_analytic_object": (_I, [_P, C.c_int32, C.POINTER(AnalyticObject)]),
    "vfs_batch_get_boundary_object": (_I, [_P, C.c_int32, _U32, C.POINTER(BoundaryObject), _F, _F]),
    "vfs_batch_set_particle_state": (_I, [_P, C.c_int32, _F, _F, _U32, C.c_int64]),
    "vfs_batch_copy_data_buffers": (_I, [_P, C.c_int32, _F, _F, _F, _F]),
    "vfs_batch_get_ids": (_I, [_P, C.c_int32, _U]),
    "vfs_batch_get_neighbor_arrays": (_I, [_P, C.c_int32, _U, _U, _U]),
    "vfs_batch_get_boundary_fields": (_I, [_P, C.c_int32, _F, _F]),
    "vfs_batch_record_fields": (_I, [_P, C.c_int32]),
    "vfs_batch_substeps": (_I, [_P, C.c_int32]),
    "vfs_batch_use_graph": (_I, [_P, C.c_int32]),
    "vfs_batch_synchronize": (_I, [_P]),
    "vfs_batch_profile_substeps": (_I, [_P, C.c_int32, _F]),
    "vfs_batch_set_sort_config": (_I, [_P, C.c_int32, C.c_int32]),
    "vfs_batch_set_neighbor_capacity": (_I, [_P, C.c_int32]),
    "vfs_model_set_neighbor_capacity": (_I, [_P, C.c_int32]),
    "vfs_model_set_skin": (_I, [_P, C.c_float]),
    "vfs_model_get_skin": (_I, [_P, C.POINTER(C.c_float)]),
    "vfs_model_set_walk_staging": (_I, [_P, C.c_int32]),
    "vfs_batch_set_walk_staging": (_I, [_P, C.c_int32]),
    "vfs_batch_set_skin": (_I, [_P, C.c_float]),
    "vfs_batch_get_skin": (_I, [_P, C.POINTER(C.c_float)]),
    "vfs_model_get_skin_builds": (_I, [_P, C.POINTER(C.c_uint32)]),
    "vfs_batch_get_skin_builds": (_I, [_P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "vfs_model_get_neighbor_capacity": (C.c_int32, [_P]),
    "vfs_batch_autotune": (_I, [_P, C.c_int32, C.c_int32, C.POINTER(TuneConfig)]),
    "vfs_batch_set_tune_config": (_I, [_P, C.POINTER(TuneConfig)]),
    "vfs_batch_get_tune_config": (_I, [_P, C.POINTER(TuneConfig)]),
    "vfs_model_autotune": (_I, [_P, C.c_int32, C.c_int32, C.POINTER(TuneConfig)]),
    "vfs_model_set_tune_config": (_I, [_P, C.POINTER(TuneConfig)]),
    "vfs_model_get_tune_config": (_I, [_P, C.POINTER(TuneConfig)]),
    "vfs_tune_cache_save": (_I, [C.c_char_p]),
    "vfs_model_export_state": (_I, [_P, C.c_char_p]),
    "vfs_model_add_mesh_object": (_I, [_P, C.POINTER(MeshObject)]),
    "vfs_batch_add_mesh_object": (_I, [_P, C.c_int32, C.POINTER(MeshObject)]),
    "vfs_mesh_signed_distance": (_I, [C.POINTER(C.c_float), C.c_uint32, C.POINTER(C.c_uint32),
                                      C.c_uint32, C.POINTER(C.c_float), C.c_uint32,
                                      C.POINTER(C.c_double)]),
    "vfs_model_render_particles": (_I, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32,
                                        C.c_int32, C.c_float, C.c_float, C.c_float,
                                        C.POINTER(C.c_uint8), C.POINTER(C.c_float)]),
    "vfs_batch_render_particles": (_I, [_P, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                        C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_float,
                                        C.POINTER(C.c_uint8), C.POINTER(C.c_float)]),
    "vfs_model_density_grid": (_I, [_P, _F, _F, C.POINTER(C.c_int32), _F]),
    "vfs_batch_density_grid": (_I, [_P, C.c_int32, _F, _F, C.POINTER(C.c_int32), _F]),
    "vfs_render_density_raymarch": (_I, [_F, C.POINTER(C.c_int32), _F, _F, _F, _F, C.c_int32,
                                         C.c_int32, C.c_float, C.c_int32, C.c_float, C.c_float,
                                         _F]),
    "vfs_model_import_state": (_I, [_P, C.c_char_p]),
    "vfs_model_record": (_I, [_P, C.c_int32, C.c_int32, C.c_char_p]),
    "vfs_batch_export_state": (_I, [_P, C.c_int32, C.c_char_p]),
    "vfs_batch_import_state": (_I, [_P, C.c_int32, C.c_char_p]),
    "vfs_batch_record": (_I, [_P, C.c_int32, C.c_int32, C.c_char_p]),
    "vfs_selftest_lookback": (_I, [C.c_int32, C.c_int32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "vfs_tune_cache_load": (_I, [C.c_char_p]),
    "vfs_tune_cache_clear": (_I, []),
    "vfs_rollout_create": (_I, [_P, C.c_int32, C.c_int32, C.POINTER(_P)]),
    "vfs_rollout_destroy": (_I, [_P]),
    "vfs_rollout_forward": (_I, [_P]),
    "vfs_rollout_backward": (_I, [_P, _F, _F, _F, _F, C.POINTER(C.c_double)]),
    "vfs_scene_load": (_I, [C.c_char_p, C.c_char_p, C.POINTER(_P)]),
    "vfs_scene_reset": (_I, [_P]),
    "vfs_sort_pairs": (_I, [_P, _P, _U32, _U32, _P]),
    "vfs_sort_pairs_noalloc": (_I, [_P, _P, _U32, _U32, _P]),
    "vfs_sort_pairs_status": (_I, [_P, _U]),
    "vfs_spatial_offsets": (_I, [_P, _P, _U32, _P]),
    "vfs_reorder_float3": (_I, [_P, _P, _P, _U32, _P]),
    "vfs_generate_lattice": (_I, [_U, _F, C.c_float, C.c_float, C.c_uint64, _F]),
    "vfs_generate_uniform_blob": (_I, [C.c_uint64, _F, _F, C.c_uint64, _F, C.c_float, C.c_uint64, _F]),
    "vfs_generate_fourier_velocity": (_I, [C.c_uint64, _F, C.c_int32, C.c_float, C.c_uint64, _F]),
}

_lib = None


def load_library(path: Path | None = None) -> C.CDLL:
    """Loads libvfs_cuda.so and binds every declared symbol; raises when it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: the CUDA library must be built first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(code: int) -> None:
    if code != VFS_OK:
        msg = load_library().vfs_last_error()
        raise VfsError(code, msg.decode() if msg else "")
