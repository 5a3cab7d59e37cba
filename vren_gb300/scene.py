"""Seeded synthetic inputs (include/vren_scene.h), as numpy arrays."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _build

_LIB = None


class SceneCamera(C.Structure):
    _fields_ = [("fov_y", C.c_float), ("near_plane", C.c_float), ("far_plane", C.c_float),
                ("width", C.c_uint32), ("height", C.c_uint32)]


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = _build.SCENE_LIB
        if not path.exists():
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build()")
        _LIB = C.CDLL(str(path))
        u64, u32, i32, vp = C.c_uint64, C.c_uint32, C.c_int, C.c_void_p
        _LIB.vren_gen_u32.argtypes = [u64, u64, vp, u64, i32]
        _LIB.vren_gen_u32_masked.argtypes = [u64, u64, vp, u64, u32, i32]
        _LIB.vren_gen_depth_planes.argtypes = [u64, vp, u32, vp, vp, i32]
        _LIB.vren_gen_lights.argtypes = [u64, vp, u32, vp, vp]
        _LIB.vren_gen_gbuffer.argtypes = [u64, u32, u32, vp, vp, vp, vp, i32]
        _LIB.vren_gen_normal01.argtypes = [u64, u64, vp, u64, i32]
        _LIB.vren_gen_lights_near_surfaces.argtypes = [u64, vp, vp, u32, vp, vp]
    return _LIB


def _p(a):
    return a.ctypes.data if a is not None else None


def gen_u32(seed: int, stream: int, n: int, mask: int = 0xFFFFFFFF, threads: int = 0) -> np.ndarray:
    out = np.empty(n, np.uint32)
    lib().vren_gen_u32_masked(seed, stream, _p(out), n, mask, threads)
    return out


def scene_camera(width: int, height: int, fov_y_deg: float = 45.0, near: float = 0.1, far: float = 1000.0):
    return SceneCamera(np.float32(np.deg2rad(fov_y_deg)), near, far, width, height)


def depth_planes(seed: int, width: int, height: int, planes: int = 64, fov_y_deg: float = 45.0, near: float = 0.1,
                 far: float = 1000.0, threads: int = 0):
    cam = scene_camera(width, height, fov_y_deg, near, far)
    depth = np.empty(width * height, np.float32)
    normals = np.empty(width * height * 3, np.float32)
    lib().vren_gen_depth_planes(seed, C.byref(cam), planes, _p(depth), _p(normals), threads)
    return depth, normals


def lights(seed: int, count: int, width: int, height: int, fov_y_deg: float = 45.0, near: float = 0.1,
           far: float = 1000.0):
    cam = scene_camera(width, height, fov_y_deg, near, far)
    pos = np.empty(count * 4, np.float32)
    li = np.empty(count * 4, np.float32)
    lib().vren_gen_lights(seed, C.byref(cam), count, _p(pos), _p(li))
    return pos, li


def gbuffer(seed: int, width: int, height: int, threads: int = 0):
    n = width * height
    normals = np.empty(n * 3, np.float32)
    albedo = np.empty(n * 3, np.float32)
    rough = np.empty(n, np.float32)
    metal = np.empty(n, np.float32)
    lib().vren_gen_gbuffer(seed, width, height, _p(normals), _p(albedo), _p(rough), _p(metal), threads)
    return normals, albedo, rough, metal


def normal01(seed: int, stream: int, n: int, threads: int = 0) -> np.ndarray:
    out = np.empty(n, np.float32)
    lib().vren_gen_normal01(seed, stream, _p(out), n, threads)
    return out


def lights_near_surfaces(seed: int, count: int, depth: np.ndarray, width: int, height: int, fov_y_deg: float = 45.0,
                         near: float = 0.1, far: float = 1000.0):
    cam = scene_camera(width, height, fov_y_deg, near, far)
    pos = np.empty(count * 4, np.float32)
    li = np.empty(count * 4, np.float32)
    d = np.ascontiguousarray(depth, np.float32)
    lib().vren_gen_lights_near_surfaces(seed, C.byref(cam), _p(d), count, _p(pos), _p(li))
    return pos, li


def lights_near_camera(seed: int, count: int):
    """Lights packed in front of the camera (x in [-8, 8], y in [-5, 5], z in [0.5, 25], radius
    lognormal around 1): many lights per cluster.  Returns flat vec4 positions and point lights."""
    rng = np.random.default_rng(seed)
    p = np.zeros((count, 4), np.float32)
    p[:, 0] = rng.uniform(-8, 8, count)
    p[:, 1] = rng.uniform(-5, 5, count)
    p[:, 2] = rng.uniform(0.5, 25, count)
    p[:, 3] = 1
    q = np.zeros((count, 4), np.float32)
    q[:, 0:3] = rng.uniform(0, 1, (count, 3))
    q[:, 3] = np.exp(np.log(2.0) + 0.5 * rng.standard_normal(count)).astype(np.float32) * 0.5
    return p.reshape(-1), q.reshape(-1)
