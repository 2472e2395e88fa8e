"""ctypes bindings of the reference's own code built by ``oracle/ref_build.py`` into
``oracle/_ref/``: ``libvfs_ref_shaders.so`` (its step shaders compiled as C++) and
``libvfs_ref_volume_map.so`` (its CPU mesh SDF and volume-map code), present only where the recipe
could run (the volume-map library needs the reference source tree itself).

TEST INFRASTRUCTURE ONLY: used by tests/ and the fixture script under tests/golden/ to pin the
oracle against the reference's code. The product package never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .binding import OracleParams

LIB_PATH = Path(__file__).resolve().parent / "_ref" / "libvfs_ref_shaders.so"
VOLUME_MAP_LIB_PATH = Path(__file__).resolve().parent / "_ref" / "libvfs_ref_volume_map.so"

_F = C.POINTER(C.c_float)
_U = C.POINTER(C.c_uint32)
_lib = None


def available() -> bool:
    return LIB_PATH.exists()


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing; build it with "
                          "python oracle/ref_build.py <VkFluidSim source tree>")
    lib = C.CDLL(str(LIB_PATH))
    sig = {
        "vfs_ref_create": (C.c_void_p, [C.POINTER(OracleParams), C.c_uint32]),
        "vfs_ref_destroy": (None, [C.c_void_p]),
        "vfs_ref_add_object": (C.c_int, [C.c_void_p, _F, _F, _F, _F, _U, _F, _F]),
        "vfs_ref_set_state": (None, [C.c_void_p, _F, _F]),
        "vfs_ref_step": (None, [C.c_void_p, C.c_int]),
        "vfs_ref_get": (None, [C.c_void_p, _F, _F, _F, _F, _F, _F, _U, _U, _U]),
        "vfs_ref_set_threads": (None, [C.c_int]),
        "vfs_ref_get_threads": (C.c_int, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def volume_map_available() -> bool:
    return VOLUME_MAP_LIB_PATH.exists()


def mesh_volume_map(vertices, triangles, h: float, res):
    """The reference's own MeshSDF + GenerateVolumeMap (src/util/mesh_sdf.cpp,
    src/util/volume_map.cpp) for a triangle mesh, margin 8 h, grids rounded to float as
    GenericScene uploads them: (box_size, box_pos, sdf, volume_map)."""
    lib = C.CDLL(str(VOLUME_MAP_LIB_PATH))
    fn = lib.vfs_ref_mesh_volume_map
    fn.restype = C.c_int
    fn.argtypes = [_F, C.c_uint32, _U, C.c_uint32, C.c_float, _U, _F, _F, _F, _F]
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, np.uint32).reshape(-1, 3)
    r = np.asarray(res, np.uint32)
    cnt = int(r[0]) * int(r[1]) * int(r[2])
    bs, bp = np.empty(3, np.float32), np.empty(3, np.float32)
    sdf, vm = np.empty(cnt, np.float32), np.empty(cnt, np.float32)
    rc = fn(_fp(v), len(v), t.ctypes.data_as(_U), len(t), h, r.ctypes.data_as(_U), _fp(bs), _fp(bp),
            _fp(sdf), _fp(vm))
    if rc != 0:
        raise ValueError("the reference volume-map code rejected the mesh")
    return bs, bp, sdf, vm


def set_threads(t: int) -> None:
    load().vfs_ref_set_threads(int(t))


def get_threads() -> int:
    return int(load().vfs_ref_get_threads())


def _fp(a):
    return a.ctypes.data_as(_F)


class RefShaderModel:
    """The reference's WCSPHWithBoundaryModel step run from its own shader code on the CPU (the
    counting sort's atomic passes in index order on one thread: a stable sort; the other
    dispatches across the host's threads)."""

    def __init__(self, params: OracleParams, n: int):
        self._lib = load()
        self.n = int(n)
        self._h = self._lib.vfs_ref_create(C.byref(params), self.n)
        if not self._h:
            raise ValueError("bad parameters")

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.vfs_ref_destroy(self._h)
            self._h = None

    def add_object(self, info) -> None:
        """A boundary object with the same fields the oracle takes (glm column-major matrices)."""
        arr = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
        res = np.asarray(info.resolution, np.uint32)
        rc = self._lib.vfs_ref_add_object(self._h, _fp(arr(info.transform)), _fp(arr(info.rotation)),
                                          _fp(arr(info.box_size)), _fp(arr(info.box_pos)),
                                          res.ctypes.data_as(_U), _fp(arr(info.sdf)),
                                          _fp(arr(info.volume_map)))
        if rc != 0:
            raise ValueError("bad boundary object")

    def set_state(self, pos, vel) -> None:
        p = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        v = np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        self._lib.vfs_ref_set_state(self._h, _fp(p), _fp(v))

    def step(self, count: int = 1) -> None:
        self._lib.vfs_ref_step(self._h, int(count))

    def state(self) -> dict:
        n = self.n
        out = {"positions": np.empty((n, 3), np.float32), "velocities": np.empty((n, 3), np.float32),
               "densities": np.empty(n, np.float32), "accelerations": np.empty((n, 3), np.float32),
               "boundary_density": np.empty(n, np.float32),
               "boundary_gradient": np.empty((n, 3), np.float32),
               "keys": np.empty(n, np.uint32), "sorted_indices": np.empty(n, np.uint32),
               "offsets": np.empty(n, np.uint32)}
        o = out
        self._lib.vfs_ref_get(self._h, _fp(o["positions"]), _fp(o["velocities"]), _fp(o["densities"]),
                              _fp(o["accelerations"]), _fp(o["boundary_density"]),
                              _fp(o["boundary_gradient"]), o["keys"].ctypes.data_as(_U),
                              o["sorted_indices"].ctypes.data_as(_U), o["offsets"].ctypes.data_as(_U))
        return out
