"""ctypes binding of the CPU oracle (``oracle/_build/libvfs_oracle.so``).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline legs, as the reference results and the timed CPU baseline. The product package never
imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libvfs_oracle.so"


class OracleParams(C.Structure):
    _fields_ = [
        ("gravity", C.c_float * 3),
        ("smooth_radius", C.c_float),
        ("time_scale", C.c_float),
        ("iterations", C.c_int32),
        ("fixed_dt", C.c_float),
        ("target_density", C.c_float),
        ("bbox_size", C.c_float * 3),
        ("bbox_pos", C.c_float * 3),
        ("wall_stiffness", C.c_float),
        ("stiffness", C.c_float),
        ("expoent", C.c_float),
        ("viscosity_strenght", C.c_float),
    ]


_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_U = C.POINTER(C.c_uint32)
_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing; build it with vkfluidsim_gb300.build.build_oracle()")
    lib = C.CDLL(str(LIB_PATH))
    sig = {
        "vfs_oracle_create": (C.c_void_p, [C.POINTER(OracleParams), C.c_uint32, C.c_int]),
        "vfs_oracle_destroy": (None, [C.c_void_p]),
        "vfs_oracle_set_params": (None, [C.c_void_p, C.POINTER(OracleParams)]),
        "vfs_oracle_add_object": (C.c_int, [C.c_void_p, _F, _F, _F, _F, _U, _F, _F]),
        "vfs_oracle_set_state": (None, [C.c_void_p, _F, _F, _U]),
        "vfs_oracle_set_state_f64": (None, [C.c_void_p, _D, _D, _U]),
        "vfs_oracle_substeps": (None, [C.c_void_p, C.c_int]),
        "vfs_oracle_step": (None, [C.c_void_p]),
        "vfs_oracle_get_state": (None, [C.c_void_p, _F, _F, _F, _U]),
        "vfs_oracle_get_state_f64": (None, [C.c_void_p, _D, _D, _D, _U]),
        "vfs_oracle_get_neighbors": (None, [C.c_void_p, _U, _U, _U]),
        "vfs_oracle_get_fields": (None, [C.c_void_p, _F, _F, _F]),
        "vfs_oracle_set_threads": (None, [C.c_int]),
        "vfs_oracle_get_threads": (C.c_int, []),
        "vfs_oracle_hash_cell": (C.c_uint32, [C.c_int32, C.c_int32, C.c_int32]),
        "vfs_oracle_cell_coord": (C.c_int32, [C.c_float, C.c_float]),
        "vfs_oracle_gauss_legendre": (None, [C.c_int, _D, _D]),
        "vfs_oracle_volume_map": (C.c_int, [C.c_int, _D, C.c_float, _U, C.c_float, C.c_int, _F, _F,
                                            _F, _F]),
        "vfs_oracle_mesh_distance": (C.c_int, [_F, C.c_uint32, _U, C.c_uint32, _F, C.c_uint32, _D]),
        "vfs_oracle_mesh_volume_map": (C.c_int, [_F, C.c_uint32, _U, C.c_uint32, C.c_float, _U,
                                                 C.c_float, C.c_int, _F, _F, _F, _F]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _fp(a):
    return None if a is None else a.ctypes.data_as(_F)


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _up(a):
    return None if a is None else a.ctypes.data_as(_U)


def params_from(sim, sph, wcsph) -> OracleParams:
    """Builds the oracle's flat parameter block from the product's parameter dataclasses."""
    return OracleParams((C.c_float * 3)(*sim.gravity), sim.smooth_radius, sph.time_scale,
                        sph.iterations, sph.fixed_dt, sph.target_density,
                        (C.c_float * 3)(*sph.bbox_size), (C.c_float * 3)(*sph.bbox_pos),
                        wcsph.wall_stiffness, wcsph.stiffness, wcsph.expoent,
                        wcsph.viscosity_strenght)


def set_threads(t: int) -> None:
    load().vfs_oracle_set_threads(int(t))


def get_threads() -> int:
    return int(load().vfs_oracle_get_threads())


def hash_cell(x: int, y: int, z: int) -> int:
    return int(load().vfs_oracle_hash_cell(x, y, z))


def cell_coord(x: float, h: float) -> int:
    return int(load().vfs_oracle_cell_coord(x, h))


def gauss_legendre(n: int):
    x = np.empty(n, np.float64)
    w = np.empty(n, np.float64)
    load().vfs_oracle_gauss_legendre(n, _dp(x), _dp(w))
    return x, w


def volume_map(shape: int, params, h: float, res, margin: float, quad_n: int = 16):
    """Oracle SDF grid + volume map of an analytic shape (object-local), with its grid box."""
    prm = np.zeros(3, np.float64)
    prm[: len(params)] = params
    r = np.asarray(res, np.uint32)
    cnt = int(r[0]) * int(r[1]) * int(r[2])
    bs = np.empty(3, np.float32)
    bp = np.empty(3, np.float32)
    sdf = np.empty(cnt, np.float32)
    vm = np.empty(cnt, np.float32)
    rc = load().vfs_oracle_volume_map(shape, _dp(prm), h, _up(r), margin, quad_n, _fp(bs), _fp(bp),
                                      _fp(sdf), _fp(vm))
    if rc != 0:
        raise ValueError("oracle volume map rejected its arguments")
    return bs, bp, sdf, vm


def _mesh_args(vertices, triangles):
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, np.uint32).reshape(-1, 3)
    return v, t


def mesh_distance(vertices, triangles, points):
    """Oracle signed distances (double) of points to a triangle mesh."""
    v, t = _mesh_args(vertices, triangles)
    p = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    out = np.empty(len(p), np.float64)
    rc = load().vfs_oracle_mesh_distance(_fp(v), len(v), _up(t), len(t), _fp(p), len(p), _dp(out))
    if rc != 0:
        raise ValueError("oracle rejected the mesh")
    return out


def mesh_volume_map(vertices, triangles, h: float, res, margin: float, quad_n: int = 16):
    """Oracle SDF grid + volume map of a triangle mesh, with its grid box."""
    v, t = _mesh_args(vertices, triangles)
    r = np.asarray(res, np.uint32)
    cnt = int(r[0]) * int(r[1]) * int(r[2])
    bs = np.empty(3, np.float32)
    bp = np.empty(3, np.float32)
    sdf = np.empty(cnt, np.float32)
    vm = np.empty(cnt, np.float32)
    rc = load().vfs_oracle_mesh_volume_map(_fp(v), len(v), _up(t), len(t), h, _up(r), margin,
                                           quad_n, _fp(bs), _fp(bp), _fp(sdf), _fp(vm))
    if rc != 0:
        raise ValueError("oracle rejected the mesh")
    return bs, bp, sdf, vm


class OracleModel:
    """The oracle's model: FP32 restatement (fp64=False) or its FP64 twin (fp64=True)."""

    def __init__(self, params: OracleParams, n: int, fp64: bool = False):
        self._lib = load()
        self.n = int(n)
        self.fp64 = fp64
        self._params = params
        self._h = self._lib.vfs_oracle_create(C.byref(params), self.n, int(fp64))

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.vfs_oracle_destroy(self._h)
            self._h = None

    def set_params(self, params: OracleParams) -> None:
        self._params = params
        self._lib.vfs_oracle_set_params(self._h, C.byref(params))

    def add_object(self, info) -> None:
        """Adds a boundary object from a product BoundaryObjectInfo (same matrices and grids)."""
        t = np.ascontiguousarray(info.transform, np.float32)
        r = np.ascontiguousarray(info.rotation, np.float32)
        bs = np.ascontiguousarray(info.box_size, np.float32)
        bp = np.ascontiguousarray(info.box_pos, np.float32)
        res = np.asarray(info.resolution, np.uint32)
        sdf = np.ascontiguousarray(info.sdf, np.float32)
        vm = np.ascontiguousarray(info.volume_map, np.float32)
        rc = self._lib.vfs_oracle_add_object(self._h, _fp(t), _fp(r), _fp(bs), _fp(bp), _up(res),
                                             _fp(sdf), _fp(vm))
        if rc != 0:
            raise ValueError("oracle rejected the boundary object")

    def set_state(self, pos, vel, ids=None) -> None:
        ids_a = None if ids is None else np.ascontiguousarray(ids, np.uint32)
        if self.fp64 and (np.asarray(pos).dtype == np.float64):
            p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
            v = np.ascontiguousarray(vel, np.float64).reshape(-1, 3)
            self._lib.vfs_oracle_set_state_f64(self._h, _dp(p), _dp(v), _up(ids_a))
        else:
            p = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
            v = np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
            self._lib.vfs_oracle_set_state(self._h, _fp(p), _fp(v), _up(ids_a))

    def substeps(self, count: int) -> None:
        self._lib.vfs_oracle_substeps(self._h, int(count))

    def step(self) -> None:
        self._lib.vfs_oracle_step(self._h)

    def state(self) -> dict:
        n = self.n
        if self.fp64:
            pos = np.empty((n, 3), np.float64)
            vel = np.empty((n, 3), np.float64)
            dens = np.empty(n, np.float64)
            ids = np.empty(n, np.uint32)
            self._lib.vfs_oracle_get_state_f64(self._h, _dp(pos), _dp(vel), _dp(dens), _up(ids))
        else:
            pos = np.empty((n, 3), np.float32)
            vel = np.empty((n, 3), np.float32)
            dens = np.empty(n, np.float32)
            ids = np.empty(n, np.uint32)
            self._lib.vfs_oracle_get_state(self._h, _fp(pos), _fp(vel), _fp(dens), _up(ids))
        return {"positions": pos, "velocities": vel, "densities": dens, "ids": ids}

    def neighbors(self):
        n = self.n
        k = np.empty(n, np.uint32)
        p = np.empty(n, np.uint32)
        o = np.empty(n, np.uint32)
        self._lib.vfs_oracle_get_neighbors(self._h, _up(k), _up(p), _up(o))
        return k, p, o

    def fields(self) -> dict:
        n = self.n
        acc = np.empty((n, 3), np.float32)
        bd = np.empty(n, np.float32)
        bg = np.empty((n, 3), np.float32)
        self._lib.vfs_oracle_get_fields(self._h, _fp(acc), _fp(bd), _fp(bg))
        return {"accelerations": acc, "boundary_density": bd, "boundary_gradient": bg}
