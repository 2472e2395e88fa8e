"""Python mirror of VkFluidSim's model / scene interface over the C ABI.

Names follow the reference: ``SimulationParameters`` (src/simulation.h:10-13),
``SPHModel.Parameters`` (src/models/model.h:14-21), ``WCSPHWithBoundaryModel.Parameters``
(src/models/wcsph_with_boundary_model.h:26-33), ``set_particle_state`` / ``set_particles_in_box``
/ ``copy_data_buffers`` (src/models/model.h:68-84), ``step`` (wcsph_with_boundary_model.cpp:81-117)
and ``load_scene`` (src/util/scene_loader.h:8). Arrays are numpy; every call goes through
``libvfs_cuda.so`` and raises ``VfsError`` with the library's message on a non-zero status.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _abi
from ._abi import check, load_library

__all__ = [
    "SimulationParameters", "SPHParameters", "WCSPHParameters", "WCSPHWithBoundaryModel",
    "AnalyticObject", "Batch", "load_scene", "generate_lattice", "generate_uniform_blob",
    "generate_fourier_velocity",
]


def _fp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _up(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_uint32))


def _f32(a, shape=None) -> np.ndarray:
    out = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape is not None:
        out = out.reshape(shape)
    return out


@dataclass
class SimulationParameters:
    gravity: Sequence[float] = (0.0, -9.81, 0.0)
    smooth_radius: float = 0.2

    def to_c(self):
        return _abi.SimParams((C.c_float * 3)(*self.gravity), self.smooth_radius)


@dataclass
class SPHParameters:
    time_scale: float = 1.0
    iterations: int = 3
    n_particles: int = 8192
    fixed_dt: float = 1.0 / 60.0
    target_density: float = 100.0
    bbox_size: Sequence[float] = (10.0, 10.0, 10.0)
    bbox_pos: Sequence[float] = (0.0, 0.0, 0.0)

    def to_c(self):
        return _abi.SphParams(self.time_scale, self.iterations, self.n_particles, self.fixed_dt,
                              self.target_density, (C.c_float * 3)(*self.bbox_size),
                              (C.c_float * 3)(*self.bbox_pos))


@dataclass
class WCSPHParameters:
    wall_stiffness: float = 1e4
    stiffness: float = 1000.0
    expoent: float = 7.0
    viscosity_strenght: float = 0.01

    def to_c(self):
        return _abi.WcsphParams(self.wall_stiffness, self.stiffness, self.expoent,
                                self.viscosity_strenght)


@dataclass
class AnalyticObject:
    """Boundary shape whose SDF and volume map are generated on the GPU."""
    shape: int
    params: Sequence[float]
    position: Sequence[float] = (0.0, 0.0, 0.0)
    rotation_angle_deg: float = 0.0
    rotation_axis: Sequence[float] = (0.0, 1.0, 0.0)
    scale: Sequence[float] = (1.0, 1.0, 1.0)
    resolution: Sequence[int] = (64, 64, 64)

    def to_c(self):
        prm = list(self.params) + [0.0] * (3 - len(self.params))
        return _abi.AnalyticObject(self.shape, (C.c_double * 3)(*prm),
                                   (C.c_float * 3)(*self.position), self.rotation_angle_deg,
                                   (C.c_float * 3)(*self.rotation_axis),
                                   (C.c_float * 3)(*self.scale),
                                   (C.c_uint32 * 3)(*self.resolution))


@dataclass
class MeshObject:
    """A triangle-mesh boundary object (GenericScene ObjectDef with an OBJ resourcePath): either
    `obj_path` or `vertices` (V, 3) + `triangles` (T, 3)."""
    obj_path: Optional[str] = None
    vertices: Optional[np.ndarray] = None
    triangles: Optional[np.ndarray] = None
    position: Sequence[float] = (0.0, 0.0, 0.0)
    rotation_angle_deg: float = 0.0
    rotation_axis: Sequence[float] = (0.0, 0.0, 1.0)
    scale: Sequence[float] = (1.0, 1.0, 1.0)
    resolution: Sequence[int] = (32, 32, 32)

    def to_c(self):
        m = _abi.MeshObject()
        keep = []
        if self.obj_path is not None:
            m.obj_path = str(self.obj_path).encode()
        else:
            v = np.ascontiguousarray(self.vertices, np.float32).reshape(-1, 3)
            t = np.ascontiguousarray(self.triangles, np.uint32).reshape(-1, 3)
            keep += [v, t]
            m.vertices = v.ctypes.data_as(C.POINTER(C.c_float))
            m.n_vertices = len(v)
            m.triangles = t.ctypes.data_as(C.POINTER(C.c_uint32))
            m.n_triangles = len(t)
        m.position[:] = list(self.position)
        m.rotation_angle_deg = self.rotation_angle_deg
        m.rotation_axis[:] = list(self.rotation_axis)
        m.scale[:] = list(self.scale)
        m.resolution[:] = [int(r) for r in self.resolution]
        return m, keep


def mesh_signed_distance(vertices, triangles, points) -> np.ndarray:
    """Signed distances (double) of points to a triangle mesh, computed on the GPU."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, np.uint32).reshape(-1, 3)
    p = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    out = np.empty(len(p), np.float64)
    check(load_library().vfs_mesh_signed_distance(
        v.ctypes.data_as(C.POINTER(C.c_float)), len(v), t.ctypes.data_as(C.POINTER(C.c_uint32)),
        len(t), p.ctypes.data_as(C.POINTER(C.c_float)), len(p),
        out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


@dataclass
class BoundaryObjectInfo:
    transform: np.ndarray
    rotation: np.ndarray
    box_size: np.ndarray
    box_pos: np.ndarray
    resolution: tuple
    sdf: np.ndarray = field(repr=False)
    volume_map: np.ndarray = field(repr=False)


def read_state(prefix) -> dict:
    """Reads a snapshot written by export_state / record: {"positions" (N, 3), "velocities" (N, 3),
    "densities" (N,), each by particle id, plus the sidecar's "substeps", "time", "parameters"}."""
    import json
    from pathlib import Path

    meta = json.loads(Path(f"{prefix}.json").read_text())
    if meta.get("format") != "vkfluidsim_gb300.state" or meta.get("version") != 1:
        raise ValueError(f"{prefix}.json is not a version-1 state sidecar")
    raw = np.fromfile(Path(f"{prefix}.json").parent / meta["binary"], dtype="<u1")
    out = {k: meta[k] for k in ("substeps", "time", "parameters", "particles")}
    for name, a in meta["arrays"].items():
        count = int(np.prod(a["shape"]))
        out[name] = np.frombuffer(raw, dtype=a["dtype"], count=count,
                                  offset=a["offset"]).reshape(a["shape"])
    return out


def perspective(fovy: float, aspect: float, near: float, far: float, y_down: bool = True):
    """glm::perspective with depth in [0, 1] (GLM_FORCE_DEPTH_ZERO_TO_ONE), y optionally flipped
    as gfx::Camera does for Vulkan; column-major float32[16]."""
    f = 1.0 / np.tan(fovy / 2.0)
    m = np.zeros((4, 4), np.float64)  # m[col][row]
    m[0][0] = f / aspect
    m[1][1] = -f if y_down else f
    m[2][2] = far / (near - far)
    m[2][3] = -1.0
    m[3][2] = -(far * near) / (far - near)
    return m.astype(np.float32).ravel()


def look_at(eye, center, up=(0.0, 0.0, 1.0)):
    """glm::lookAt (right-handed); column-major float32[16]."""
    eye, center, up = (np.asarray(v, np.float64) for v in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)  # m[col][row]
    m[0][0], m[1][0], m[2][0] = s
    m[0][1], m[1][1], m[2][1] = u
    m[0][2], m[1][2], m[2][2] = -f
    m[3][0], m[3][1], m[3][2] = -s @ eye, -u @ eye, f @ eye
    return m.astype(np.float32).ravel()


def write_ppm(path, rgba) -> None:
    """Writes the RGB channels of an (H, W, 4) uint8 image as a binary PPM."""
    rgb = np.ascontiguousarray(np.asarray(rgba)[..., :3], dtype=np.uint8)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (rgb.shape[1], rgb.shape[0]))
        f.write(rgb.tobytes())


def _render(lib_fn, args, width, height, quad_side, depth_radius, v_max, with_depth):
    mv = np.ascontiguousarray(args[-2], np.float32)
    pj = np.ascontiguousarray(args[-1], np.float32)
    img = np.empty((height, width, 4), np.uint8)
    dep = np.empty((height, width), np.float32) if with_depth else None
    check(lib_fn(*args[:-2], _fp(mv), _fp(pj), width, height, quad_side, depth_radius, v_max,
                 img.ctypes.data_as(C.POINTER(C.c_uint8)), _fp(dep)))
    return (img, dep) if with_depth else img


def _density_grid(lib_fn, args, lo, hi, res) -> np.ndarray:
    lo = _f32(lo, (3,))
    hi = _f32(hi, (3,))
    r = np.ascontiguousarray(np.asarray(res, dtype=np.int32).reshape(3))
    grid = np.empty((int(r[2]), int(r[1]), int(r[0])), np.float32)
    check(lib_fn(*args, _fp(lo), _fp(hi), r.ctypes.data_as(C.POINTER(C.c_int32)), _fp(grid)))
    return grid


def render_density_raymarch(field, center, half_extent, view, proj, width: int, height: int,
                            step: float = 0.05, n_steps: int = 1000, color_scale: float = 5.0,
                            emission: float = 200.0, background=None) -> np.ndarray:
    """The reference's density raymarch (raymarch.slang) of a scalar field of shape
    (nz, ny, nx) occupying center +- half_extent, alpha-blended over `background` (an
    (height, width, 4) float RGBA image, transparent black by default). Returns the float image
    (row 0 at NDC y = -1); `to_rgba8` quantises it as the reference's 8-bit draw image does."""
    f = np.ascontiguousarray(field, dtype=np.float32)
    if f.ndim != 3:
        raise ValueError("field must have shape (nz, ny, nx)")
    res = np.array([f.shape[2], f.shape[1], f.shape[0]], np.int32)
    img = np.zeros((height, width, 4), np.float32)
    if background is not None:
        img[...] = np.asarray(background, np.float32)
    c = _f32(center, (3,))
    he = _f32(half_extent, (3,))
    v = np.ascontiguousarray(view, np.float32)
    pj = np.ascontiguousarray(proj, np.float32)
    check(load_library().vfs_render_density_raymarch(
        _fp(f), res.ctypes.data_as(C.POINTER(C.c_int32)), _fp(c), _fp(he), _fp(v), _fp(pj), width,
        height, step, n_steps, color_scale, emission, _fp(img)))
    return img


def to_rgba8(img) -> np.ndarray:
    """Float RGBA in [0, 1] to uint8, rounding to nearest (a UNORM attachment's conversion)."""
    return np.clip(np.rint(np.asarray(img, np.float32) * 255.0), 0, 255).astype(np.uint8)


def tune_dict(c) -> dict:
    return {k: int(getattr(c, k)) for k, _ in _abi.TuneConfig._fields_}


def tune_cache_save(path: str) -> None:
    check(load_library().vfs_tune_cache_save(str(path).encode()))


def tune_cache_load(path: str) -> None:
    check(load_library().vfs_tune_cache_load(str(path).encode()))


def tune_cache_clear() -> None:
    check(load_library().vfs_tune_cache_clear())


class WCSPHWithBoundaryModel:
    """A WCSPH-with-boundary model on the GPU (one handle of libvfs_cuda)."""

    def __init__(self, sim: SimulationParameters, sph: SPHParameters, wcsph: WCSPHParameters,
                 _handle: Optional[int] = None):
        self._lib = load_library()
        if _handle is not None:
            self._h = C.c_void_p(_handle)
        else:
            h = C.c_void_p()
            check(self._lib.vfs_model_create(C.byref(sim.to_c()), C.byref(sph.to_c()),
                                             C.byref(wcsph.to_c()), C.byref(h)))
            self._h = h

    # -- lifecycle
    def clear(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.vfs_model_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.clear()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.clear()

    @property
    def n_particles(self) -> int:
        return int(self._lib.vfs_model_num_particles(self._h))

    def get_parameters(self):
        s, p, w = _abi.SimParams(), _abi.SphParams(), _abi.WcsphParams()
        check(self._lib.vfs_model_get_parameters(self._h, C.byref(s), C.byref(p), C.byref(w)))
        return (SimulationParameters(tuple(s.gravity), s.smooth_radius),
                SPHParameters(p.time_scale, p.iterations, p.n_particles, p.fixed_dt,
                              p.target_density, tuple(p.bbox_size), tuple(p.bbox_pos)),
                WCSPHParameters(w.wall_stiffness, w.stiffness, w.expoent, w.viscosity_strenght))

    def set_parameters(self, sim=None, sph=None, wcsph=None) -> None:
        a = C.byref(sim.to_c()) if sim else None
        b = C.byref(sph.to_c()) if sph else None
        c = C.byref(wcsph.to_c()) if wcsph else None
        check(self._lib.vfs_model_set_parameters(self._h, a, b, c))

    def set_stream(self, stream_handle: int) -> None:
        check(self._lib.vfs_model_set_stream(self._h, C.c_void_p(stream_handle)))

    # -- boundary objects
    def add_boundary_object(self, transform, rotation, box_size, box_pos, resolution, sdf,
                            volume_map) -> None:
        sdf = _f32(sdf).ravel()
        vm = _f32(volume_map).ravel()
        o = _abi.BoundaryObject()
        o.transform[:] = [float(x) for x in np.asarray(transform, np.float32).ravel()]
        o.rotation[:] = [float(x) for x in np.asarray(rotation, np.float32).ravel()]
        o.box_size[:] = list(map(float, box_size))
        o.box_pos[:] = list(map(float, box_pos))
        o.resolution[:] = list(map(int, resolution))
        o.sdf_grid = _fp(sdf)
        o.volume_map_grid = _fp(vm)
        check(self._lib.vfs_model_add_boundary_object(self._h, C.byref(o)))

    def add_analytic_object(self, obj: AnalyticObject) -> None:
        check(self._lib.vfs_model_add_analytic_object(self._h, C.byref(obj.to_c())))

    def add_mesh_object(self, obj: MeshObject) -> None:
        m, keep = obj.to_c()
        check(self._lib.vfs_model_add_mesh_object(self._h, C.byref(m)))
        del keep

    @property
    def n_boundary_objects(self) -> int:
        return int(self._lib.vfs_model_num_boundary_objects(self._h))

    def get_boundary_object(self, idx: int) -> BoundaryObjectInfo:
        info = _abi.BoundaryObject()
        check(self._lib.vfs_model_get_boundary_object(self._h, idx, C.byref(info), None, None))
        res = tuple(int(x) for x in info.resolution)
        cnt = res[0] * res[1] * res[2]
        sdf = np.empty(cnt, np.float32)
        vm = np.empty(cnt, np.float32)
        check(self._lib.vfs_model_get_boundary_object(self._h, idx, None, _fp(sdf), _fp(vm)))
        return BoundaryObjectInfo(np.array(info.transform[:], np.float32),
                                  np.array(info.rotation[:], np.float32),
                                  np.array(info.box_size[:], np.float32),
                                  np.array(info.box_pos[:], np.float32), res, sdf, vm)

    # -- state
    def set_particle_state(self, pos, vel, offset: int = 0, count: int = -1) -> None:
        pos = _f32(pos, (-1, 3))
        vel = _f32(vel, (-1, 3))
        if count < 0:
            count = pos.shape[0]
        if pos.shape[0] < count or vel.shape[0] < count:
            raise ValueError("pos/vel hold fewer rows than count")
        check(self._lib.vfs_model_set_particle_state(self._h, _fp(pos), _fp(vel), offset, count))

    def set_particles_in_box(self, box_size, box_pos, offset: int = 0, count: int = -1,
                             mode: int = 0, seed: int = 0) -> None:
        bs = _f32(box_size, (3,))
        bp = _f32(box_pos, (3,))
        check(self._lib.vfs_model_set_particles_in_box(self._h, _fp(bs), _fp(bp), offset, count,
                                                       mode, seed))

    def copy_data_buffers(self, with_acc: bool = False) -> dict:
        n = self.n_particles
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        dens = np.empty(n, np.float32)
        acc = np.empty((n, 3), np.float32) if with_acc else None
        check(self._lib.vfs_model_copy_data_buffers(self._h, _fp(pos), _fp(vel), _fp(dens),
                                                    _fp(acc)))
        out = {"positions": pos, "velocities": vel, "densities": dens}
        if with_acc:
            out["accelerations"] = acc
        return out

    def step_host(self, pos=None, vel=None, substeps: int = 1, out: Optional[dict] = None) -> dict:
        """set_particle_state of every particle (when pos and vel are given), `substeps`
        substeps and copy_data_buffers, with one wait at the end (vfs_model_step_host). `out`
        may hold preallocated float32 arrays "positions" (N x 3), "velocities" (N x 3) and
        "densities" (N); when all of them are page-locked (e.g. numpy views of pinned torch
        tensors), the last substep writes them directly (its density pass the densities, its
        force pass positions and velocities)."""
        n = self.n_particles
        if (pos is None) != (vel is None):
            raise ValueError("pos and vel must both be given or both be None")
        p = v = None
        if pos is not None:
            p, v = _f32(pos, (-1, 3)), _f32(vel, (-1, 3))
            if p.shape[0] != n or v.shape[0] != n:
                raise ValueError("pos and vel must hold every particle")
        out = dict(out or {})
        shapes = {"positions": (n, 3), "velocities": (n, 3), "densities": (n,)}
        for k, shape in shapes.items():
            a = out.get(k)
            if a is None:
                out[k] = np.empty(shape, np.float32)
            elif a.dtype != np.float32 or a.shape != shape or not a.flags.c_contiguous:
                raise ValueError(f"out[{k!r}] must be a C-contiguous float32 array of shape {shape}")
        check(self._lib.vfs_model_step_host(self._h, _fp(p), _fp(v), substeps,
                                            _fp(out["positions"]), _fp(out["velocities"]),
                                            _fp(out["densities"])))
        return {k: out[k] for k in shapes}

    def get_ids(self) -> np.ndarray:
        ids = np.empty(self.n_particles, np.uint32)
        check(self._lib.vfs_model_get_ids(self._h, _up(ids)))
        return ids

    def get_neighbor_arrays(self):
        n = self.n_particles
        keys = np.empty(n, np.uint32)
        perm = np.empty(n, np.uint32)
        offs = np.empty(n, np.uint32)
        check(self._lib.vfs_model_get_neighbor_arrays(self._h, _up(keys), _up(perm), _up(offs)))
        return keys, perm, offs

    def get_boundary_fields(self):
        n = self.n_particles
        bd = np.empty(n, np.float32)
        bg = np.empty((n, 3), np.float32)
        check(self._lib.vfs_model_get_boundary_fields(self._h, _fp(bd), _fp(bg)))
        return bd, bg

    def record_fields(self, enable: bool = True) -> None:
        check(self._lib.vfs_model_record_fields(self._h, int(enable)))

    # -- stepping
    def step(self) -> None:
        check(self._lib.vfs_model_step(self._h))

    def substeps(self, count: int) -> None:
        check(self._lib.vfs_model_substeps(self._h, count))

    def use_graph(self, enable: bool) -> None:
        check(self._lib.vfs_model_use_graph(self._h, int(enable)))

    def synchronize(self) -> None:
        check(self._lib.vfs_model_synchronize(self._h))

    PHASES = ("keys", "sort", "cells_reorder", "density", "force", "clear")

    def profile_substeps(self, count: int) -> dict:
        ms = (C.c_float * 6)()
        check(self._lib.vfs_model_profile_substeps(self._h, count, ms))
        return dict(zip(self.PHASES, (float(x) for x in ms)))

    def set_sort_config(self, digit_bits: int, tile_items: int) -> None:
        check(self._lib.vfs_model_set_sort_config(self._h, digit_bits, tile_items))

    @property
    def neighbor_capacity(self) -> int:
        return int(self._lib.vfs_model_get_neighbor_capacity(self._h))

    def set_neighbor_capacity(self, slots: int) -> None:
        check(self._lib.vfs_model_set_neighbor_capacity(self._h, slots))

    @property
    def skin(self) -> float:
        """Skin of the candidate lists as a fraction of h (0: no lists, every particle walks)."""
        s = C.c_float()
        check(self._lib.vfs_model_get_skin(self._h, C.byref(s)))
        return float(s.value)

    def set_skin(self, skin: float) -> None:
        check(self._lib.vfs_model_set_skin(self._h, skin))

    def set_walk_staging(self, enable: bool) -> None:
        """Block-per-cell staging of the density walk (on by default; bit-identical results)."""
        check(self._lib.vfs_model_set_walk_staging(self._h, int(bool(enable))))

    def skin_builds(self) -> int:
        """Candidate-list builds so far."""
        b = C.c_uint32()
        check(self._lib.vfs_model_get_skin_builds(self._h, C.byref(b)))
        return int(b.value)

    def get_sort_config(self):
        d, t, p = C.c_int32(), C.c_int32(), C.c_int32()
        check(self._lib.vfs_model_get_sort_config(self._h, C.byref(d), C.byref(t), C.byref(p)))
        return d.value, t.value, p.value

    def export_state(self, prefix) -> None:
        """Writes `<prefix>.bin` + `<prefix>.json` (state by particle id; see read_state)."""
        check(self._lib.vfs_model_export_state(self._h, str(prefix).encode()))

    def import_state(self, prefix) -> None:
        check(self._lib.vfs_model_import_state(self._h, str(prefix).encode()))

    def record(self, substeps: int, every: int, prefix) -> None:
        """Runs `substeps` substeps, writing a snapshot `<prefix>_f<frame:06d>` every `every`."""
        check(self._lib.vfs_model_record(self._h, substeps, every, str(prefix).encode()))

    def render_particles(self, model_view, proj, width: int, height: int, quad_side: float = 0.15,
                         depth_radius: float = 0.15, v_max: float = 6.5, with_depth: bool = False):
        """The reference's particle pass into an (height, width, 4) uint8 RGBA image (row 0 at
        NDC y = -1), optionally with the depth buffer."""
        return _render(self._lib.vfs_model_render_particles, (self._h, model_view, proj), width,
                       height, quad_side, depth_radius, v_max, with_depth)

    def density_grid(self, lo, hi, res) -> np.ndarray:
        """SPH density of the current particles at the nodes of a regular grid over [lo, hi]
        (vfs_model_density_grid): shape (res_z, res_y, res_x), node (i, j, k) at
        lo + (i, j, k) (hi - lo) / (res - 1)."""
        return _density_grid(self._lib.vfs_model_density_grid, (self._h,), lo, hi, res)

    def autotune(self, repeats: int = 3, use_cache: bool = True) -> dict:
        """Runs the autotuner (vfs_model_autotune) and returns the chosen launch shapes."""
        c = _abi.TuneConfig()
        check(self._lib.vfs_model_autotune(self._h, repeats, int(use_cache), C.byref(c)))
        return tune_dict(c)

    def get_tune_config(self) -> dict:
        c = _abi.TuneConfig()
        check(self._lib.vfs_model_get_tune_config(self._h, C.byref(c)))
        return tune_dict(c)

    def set_tune_config(self, **kw) -> None:
        c = _abi.TuneConfig(**{**self.get_tune_config(), **kw})
        check(self._lib.vfs_model_set_tune_config(self._h, C.byref(c)))

    def device_state(self):
        p, v = C.c_void_p(), C.c_void_p()
        check(self._lib.vfs_model_device_state(self._h, C.byref(p), C.byref(v)))
        return p.value, v.value

    # -- scene
    def reset(self) -> None:
        check(self._lib.vfs_scene_reset(self._h))


def load_scene(json_path: str, resources_dir: str = "") -> WCSPHWithBoundaryModel:
    """LoadScene + GenericScene::Init/Reset (src/util/scene_loader.cpp:113-140)."""
    lib = load_library()
    h = C.c_void_p()
    check(lib.vfs_scene_load(str(json_path).encode(), str(resources_dir).encode(), C.byref(h)))
    return WCSPHWithBoundaryModel(None, None, None, _handle=h.value)


def generate_lattice(dims, origin, spacing: float, jitter: float, seed: int) -> np.ndarray:
    lib = load_library()
    d = np.asarray(dims, np.uint32)
    o = _f32(origin, (3,))
    out = np.empty((int(np.prod(d.astype(np.uint64))), 3), np.float32)
    check(lib.vfs_generate_lattice(_up(d), _fp(o), spacing, jitter, seed, _fp(out)))
    return out


def generate_uniform_blob(n_uniform: int, lo, hi, n_blob: int, center, sigma: float,
                          seed: int) -> np.ndarray:
    lib = load_library()
    out = np.empty((n_uniform + n_blob, 3), np.float32)
    check(lib.vfs_generate_uniform_blob(n_uniform, _fp(_f32(lo, (3,))), _fp(_f32(hi, (3,))),
                                        n_blob, _fp(_f32(center, (3,))), sigma, seed, _fp(out)))
    return out


def generate_fourier_velocity(pos, modes: int, amplitude: float, seed: int) -> np.ndarray:
    lib = load_library()
    pos = _f32(pos, (-1, 3))
    out = np.empty_like(pos)
    check(lib.vfs_generate_fourier_velocity(pos.shape[0], _fp(pos), modes, amplitude, seed,
                                            _fp(out)))
    return out


class Batch:
    """Many independent scenes advanced together (vfs_batch): every pass is one launch over all
    scenes; each scene's results equal those of its own WCSPHWithBoundaryModel."""

    def __init__(self, scenes):
        """scenes: sequence of (SimulationParameters, SPHParameters, WCSPHParameters)."""
        self._lib = load_library()
        k = len(scenes)
        sims = (_abi.SimParams * k)(*[s[0].to_c() for s in scenes])
        sphs = (_abi.SphParams * k)(*[s[1].to_c() for s in scenes])
        wcs = (_abi.WcsphParams * k)(*[s[2].to_c() for s in scenes])
        h = C.c_void_p()
        check(self._lib.vfs_batch_create(k, sims, sphs, wcs, C.byref(h)))
        self._h = h

    def clear(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.vfs_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.clear()
        except Exception:
            pass

    @property
    def n_scenes(self) -> int:
        return int(self._lib.vfs_batch_num_scenes(self._h))

    def n_particles(self, scene: int) -> int:
        return int(self._lib.vfs_batch_num_particles(self._h, scene))

    def set_stream(self, stream_handle: int) -> None:
        check(self._lib.vfs_batch_set_stream(self._h, C.c_void_p(stream_handle)))

    def set_scene_parameters(self, scene: int, sim=None, sph=None, wcsph=None) -> None:
        a = C.byref(sim.to_c()) if sim else None
        b = C.byref(sph.to_c()) if sph else None
        c = C.byref(wcsph.to_c()) if wcsph else None
        check(self._lib.vfs_batch_set_scene_parameters(self._h, scene, a, b, c))

    def add_analytic_object(self, scene: int, obj: AnalyticObject) -> None:
        check(self._lib.vfs_batch_add_analytic_object(self._h, scene, C.byref(obj.to_c())))

    def add_mesh_object(self, scene: int, obj: MeshObject) -> None:
        m, keep = obj.to_c()
        check(self._lib.vfs_batch_add_mesh_object(self._h, scene, C.byref(m)))
        del keep

    def get_boundary_object(self, scene: int, idx: int) -> BoundaryObjectInfo:
        info = _abi.BoundaryObject()
        check(self._lib.vfs_batch_get_boundary_object(self._h, scene, idx, C.byref(info), None,
                                                      None))
        res = tuple(int(x) for x in info.resolution)
        cnt = res[0] * res[1] * res[2]
        sdf = np.empty(cnt, np.float32)
        vm = np.empty(cnt, np.float32)
        check(self._lib.vfs_batch_get_boundary_object(self._h, scene, idx, None, _fp(sdf),
                                                      _fp(vm)))
        return BoundaryObjectInfo(np.array(info.transform[:], np.float32),
                                  np.array(info.rotation[:], np.float32),
                                  np.array(info.box_size[:], np.float32),
                                  np.array(info.box_pos[:], np.float32), res, sdf, vm)

    def set_particle_state(self, scene: int, pos, vel, offset: int = 0, count: int = -1) -> None:
        pos = _f32(pos, (-1, 3))
        vel = _f32(vel, (-1, 3))
        if count < 0:
            count = pos.shape[0]
        check(self._lib.vfs_batch_set_particle_state(self._h, scene, _fp(pos), _fp(vel), offset,
                                                     count))

    def copy_data_buffers(self, scene: int, with_acc: bool = False) -> dict:
        n = self.n_particles(scene)
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        dens = np.empty(n, np.float32)
        acc = np.empty((n, 3), np.float32) if with_acc else None
        check(self._lib.vfs_batch_copy_data_buffers(self._h, scene, _fp(pos), _fp(vel), _fp(dens),
                                                    _fp(acc)))
        out = {"positions": pos, "velocities": vel, "densities": dens}
        if with_acc:
            out["accelerations"] = acc
        return out

    def get_ids(self, scene: int) -> np.ndarray:
        ids = np.empty(self.n_particles(scene), np.uint32)
        check(self._lib.vfs_batch_get_ids(self._h, scene, _up(ids)))
        return ids

    def get_neighbor_arrays(self, scene: int):
        n = self.n_particles(scene)
        keys, perm, offs = (np.empty(n, np.uint32) for _ in range(3))
        check(self._lib.vfs_batch_get_neighbor_arrays(self._h, scene, _up(keys), _up(perm),
                                                      _up(offs)))
        return keys, perm, offs

    def get_boundary_fields(self, scene: int):
        n = self.n_particles(scene)
        bd = np.empty(n, np.float32)
        bg = np.empty((n, 3), np.float32)
        check(self._lib.vfs_batch_get_boundary_fields(self._h, scene, _fp(bd), _fp(bg)))
        return bd, bg

    def record_fields(self, enable: bool = True) -> None:
        check(self._lib.vfs_batch_record_fields(self._h, int(enable)))

    def substeps(self, count: int) -> None:
        check(self._lib.vfs_batch_substeps(self._h, count))

    def use_graph(self, enable: bool) -> None:
        check(self._lib.vfs_batch_use_graph(self._h, int(enable)))

    def synchronize(self) -> None:
        check(self._lib.vfs_batch_synchronize(self._h))

    def profile_substeps(self, count: int) -> dict:
        ms = (C.c_float * 6)()
        check(self._lib.vfs_batch_profile_substeps(self._h, count, ms))
        return dict(zip(WCSPHWithBoundaryModel.PHASES, (float(x) for x in ms)))

    def set_sort_config(self, digit_bits: int, tile_items: int) -> None:
        check(self._lib.vfs_batch_set_sort_config(self._h, digit_bits, tile_items))

    def set_neighbor_capacity(self, slots: int) -> None:
        check(self._lib.vfs_batch_set_neighbor_capacity(self._h, slots))

    @property
    def skin(self) -> float:
        s = C.c_float()
        check(self._lib.vfs_batch_get_skin(self._h, C.byref(s)))
        return float(s.value)

    def set_skin(self, skin: float) -> None:
        check(self._lib.vfs_batch_set_skin(self._h, skin))

    def set_walk_staging(self, enable: bool) -> None:
        check(self._lib.vfs_batch_set_walk_staging(self._h, int(bool(enable))))

    def skin_builds(self, scene: int) -> int:
        b = C.c_uint32()
        check(self._lib.vfs_batch_get_skin_builds(self._h, scene, C.byref(b)))
        return int(b.value)

    def export_state(self, scene: int, prefix) -> None:
        check(self._lib.vfs_batch_export_state(self._h, scene, str(prefix).encode()))

    def import_state(self, scene: int, prefix) -> None:
        check(self._lib.vfs_batch_import_state(self._h, scene, str(prefix).encode()))

    def record(self, substeps: int, every: int, prefix) -> None:
        """Snapshots `<prefix>_s<scene>_f<frame:06d>` of every scene every `every` substeps."""
        check(self._lib.vfs_batch_record(self._h, substeps, every, str(prefix).encode()))

    def render_particles(self, scene: int, model_view, proj, width: int, height: int,
                         quad_side: float = 0.15, depth_radius: float = 0.15, v_max: float = 6.5,
                         with_depth: bool = False):
        return _render(self._lib.vfs_batch_render_particles, (self._h, scene, model_view, proj),
                       width, height, quad_side, depth_radius, v_max, with_depth)

    def density_grid(self, scene: int, lo, hi, res) -> np.ndarray:
        return _density_grid(self._lib.vfs_batch_density_grid, (self._h, scene), lo, hi, res)

    def autotune(self, repeats: int = 3, use_cache: bool = True) -> dict:
        """Runs the autotuner (vfs_batch_autotune) and returns the chosen launch shapes."""
        c = _abi.TuneConfig()
        check(self._lib.vfs_batch_autotune(self._h, repeats, int(use_cache), C.byref(c)))
        return tune_dict(c)

    def get_tune_config(self) -> dict:
        c = _abi.TuneConfig()
        check(self._lib.vfs_batch_get_tune_config(self._h, C.byref(c)))
        return tune_dict(c)

    def set_tune_config(self, **kw) -> None:
        c = _abi.TuneConfig(**{**self.get_tune_config(), **kw})
        check(self._lib.vfs_batch_set_tune_config(self._h, C.byref(c)))
