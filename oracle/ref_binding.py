"""ctypes binding of ``oracle/_ref/libvfs_ref_shaders.so``: the reference's own step shaders
compiled as C++ by ``oracle/ref_build.py`` (present only where the reference source tree was
available when the recipe ran).

TEST INFRASTRUCTURE ONLY: used by tests/ and the fixture script under tests/golden/ to pin the
oracle against the reference's code. The product package never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .binding import OracleParams

LIB_PATH = Path(__file__).resolve().parent / "_ref" / "libvfs_ref_shaders.so"

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
