"""ctypes bindings over oracle/_ref/ (TEST INFRASTRUCTURE ONLY): the reference's own shaders, rewritten
into C++ by oracle/ref_shaders.py and compiled for the CPU, in two variants ("glsl": as written;
"canonical": with the canonical decisions substituted).  Only the tests use it, to pin the oracle's
restatement to the reference's source.  available() is False where the libraries were not built (no
reference checkout on this machine)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_DIR = Path(__file__).resolve().parent / "_ref"
u32, u64, i32, vp, f32 = C.c_uint32, C.c_uint64, C.c_int, C.c_void_p, C.c_float

_PROTOS = {
    "ref_is_canonical": (i32, []),
    "ref_oob_count": (u64, [i32]),
    "ref_set_canonical": (None, [vp, vp, vp, vp, u32]),
    "ref_normal_bin": (None, [vp, u64, vp]),
    "ref_decode_cluster_key": (None, [vp, u64, vp]),
    "ref_cluster_boxes": (None, [vp, u64, u32, u32, f32, f32, vp, vp, vp]),
    "ref_test_aabb_aabb": (None, [vp, u64, vp]),
    "ref_test_sphere_aabb": (None, [vp, u64, vp]),
    "ref_view_space": (None, [vp, vp, u32, vp]),
    "ref_morton": (None, [vp, u32, vp, vp, vp]),
    "ref_leaves": (None, [vp, vp, vp, u32, u32, vp]),
    "ref_pixel_keys": (None, [u32, u32, vp, vp, f32, f32, vp, vp]),
    "ref_assign_lights": (None, [i32, vp, u32, u32, u32, f32, f32, vp, vp, u64, u32, u32, vp, u64, vp, u32, vp, vp,
                                 vp, u64]),
    "ref_shade": (None, [u32, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, u32, u64, vp, vp, u32, vp, u32, vp, f32, vp, vp,
                         vp]),
    "ref_bounce": (None, [vp, vp, u32, vp, vp, f32, f32]),
    "ref_depth_copy": (None, [vp, u32, u32, vp]),
    "ref_depth_reduce": (None, [vp, u32, u32, vp, u32, u32]),
    "ref_show_clusters": (None, [i32, u32, u32, u32, u32, vp, vp, u32, vp, vp, vp, u64, vp]),
}
_LIBS: dict = {}


def lib_path(variant: str) -> Path:
    return _DIR / f"libvren_ref_{variant}.so"


def available() -> bool:
    return all(lib_path(v).is_file() for v in ("glsl", "canonical"))


def lib(variant: str) -> C.CDLL:
    if variant not in _LIBS:
        dll = C.CDLL(str(lib_path(variant)))
        for name, (res, args) in _PROTOS.items():
            f = getattr(dll, name)
            f.restype = res
            f.argtypes = args
        _LIBS[variant] = dll
    return _LIBS[variant]


def _p(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _f(a):
    return np.ascontiguousarray(a, np.float32)


def _u(a):
    return np.ascontiguousarray(a, np.uint32)


def reference_projection(width: int, height: int, near: float, far: float, fov_y: float) -> np.ndarray:
    """vren::camera::get_projection (vren/vren/camera.cpp:40-50) in single precision, column-major."""
    f = np.float32
    tan_half = f(np.tan(f(f(fov_y) / f(2.0))))
    aspect = f(f(width) / f(height))
    m = np.zeros(16, np.float32)
    m[0] = f(1.0) / f(tan_half * aspect)
    m[5] = f(1.0) / tan_half
    m[10] = f(far) / f(f(far) - f(near))
    m[11] = f(1.0)
    m[14] = -f(f(far) * f(near)) / f(f(far) - f(near))
    return m


class Ref:
    """One variant; set_canonical() installs the host-built tables the canonical variant reads."""

    def __init__(self, variant: str):
        self.variant = variant
        self.L = lib(variant)
        self._keep = []

    def oob(self, clear=True) -> int:
        return int(self.L.ref_oob_count(1 if clear else 0))

    def set_canonical(self, view, slice_near, slice_far, max_slice: int):
        ip, iv = _f(view.inv_proj), _f(view.inv_view)
        sn, sf = _f(slice_near), _f(slice_far)
        self._keep = [ip, iv, sn, sf]  # the library keeps pointers to the tables
        self.L.ref_set_canonical(_p(ip), _p(iv), _p(sn), _p(sf), max_slice)

    def normal_bin(self, normals) -> np.ndarray:
        n = np.ascontiguousarray(_f(normals).reshape(-1, 3))
        out = np.zeros(len(n), np.uint32)
        self.L.ref_normal_bin(_p(n), len(n), _p(out))
        return out

    def decode_cluster_key(self, keys) -> np.ndarray:
        k = _u(keys)
        out = np.zeros((len(k), 4), np.uint32)
        self.L.ref_decode_cluster_key(_p(k), len(k), _p(out))
        return out

    def cluster_boxes(self, keys, tiles_x, tiles_y, near, half_fov, proj):
        k = _u(keys)
        mn = np.zeros((len(k), 4), np.float32)
        mx = np.zeros((len(k), 4), np.float32)
        self.L.ref_cluster_boxes(_p(k), len(k), tiles_x, tiles_y, near, half_fov, _p(_f(proj)), _p(mn), _p(mx))
        return mn, mx

    def test_aabb_aabb(self, t) -> np.ndarray:
        t = np.ascontiguousarray(_f(t).reshape(-1, 12))
        out = np.zeros(len(t), np.uint8)
        self.L.ref_test_aabb_aabb(_p(t), len(t), _p(out))
        return out

    def test_sphere_aabb(self, t) -> np.ndarray:
        t = np.ascontiguousarray(_f(t).reshape(-1, 10))
        out = np.zeros(len(t), np.uint8)
        self.L.ref_test_sphere_aabb(_p(t), len(t), _p(out))
        return out

    def view_space(self, view_matrix, positions, L) -> np.ndarray:
        out = np.zeros(L * 4, np.float32)
        self.L.ref_view_space(_p(_f(view_matrix)), _p(_f(positions)), L, _p(out))
        return out

    def morton(self, view_pos, L, mn, mx) -> np.ndarray:
        out = np.zeros((L, 2), np.uint32)
        self.L.ref_morton(_p(_f(view_pos)), L, _p(_f(mn)), _p(_f(mx)), _p(out))
        return out

    def leaves(self, view_pos, lights, sorted_pairs, L, padded) -> np.ndarray:
        out = np.zeros((padded, 8), np.uint32)
        self.L.ref_leaves(_p(_f(view_pos)), _p(_f(lights)), _p(_u(sorted_pairs)), L, padded, _p(out))
        return out

    def pixel_keys(self, W, H, depth, normals, near, half_fov, proj) -> np.ndarray:
        TX, TY = (W + 31) // 32, (H + 31) // 32
        out = np.zeros((TY * 32, TX * 32), np.uint32)
        self.L.ref_pixel_keys(W, H, _p(_f(depth)), _p(_f(normals)), near, half_fov, _p(_f(proj)), _p(out))
        return out

    def assign_lights(self, keys, tiles_x, tiles_y, near, half_fov, proj, bvh, root, levels, light_index, view_pos, L):
        """Count dispatch, offsets by exclusive sum, write dispatch (as the reference's host code runs them)."""
        k = _u(keys)
        U = len(k)
        bvh = _u(bvh).reshape(-1, 8)
        li = _u(light_index).reshape(-1)
        vpos = _f(view_pos)
        pr = _f(proj)
        counts = np.zeros(max(U, 1), np.uint32)
        self.L.ref_assign_lights(0, _p(k), U, tiles_x, tiles_y, near, half_fov, _p(pr), _p(bvh), len(bvh), root, levels,
                                 _p(li), len(li) // 2, _p(vpos), L, _p(counts), None, None, 0)
        counts = counts[:U]
        offsets = np.zeros(max(U, 1), np.uint32)
        offsets[:U] = np.concatenate([[0], np.cumsum(counts, dtype=np.uint64)[:-1]]).astype(np.uint32) if U else []
        total = int(counts.sum(dtype=np.uint64))
        indices = np.zeros(max(total, 1), np.uint32)
        cnt2 = counts.copy() if U else np.zeros(1, np.uint32)
        self.L.ref_assign_lights(1, _p(k), U, tiles_x, tiles_y, near, half_fov, _p(pr), _p(bvh), len(bvh), root, levels,
                                 _p(li), len(li) // 2, _p(vpos), L, _p(cnt2), _p(offsets), _p(indices), total)
        return counts, offsets[:U], indices[:total]

    def shade(self, W, H, gb, lists, light_pos, lights, L, eye, far, view_matrix, proj, directional=None):
        depth, normals, albedo, rough, metal = (_f(x) for x in gb)
        refs, counts, offsets, indices = (_u(x) for x in lists)
        dl = _f(directional) if directional is not None else np.zeros(8, np.float32)
        nd = 0 if directional is None else len(dl) // 8
        out = np.full(W * H * 4, np.nan, np.float32)
        self.L.ref_shade(W, H, _p(depth), _p(normals), _p(albedo), _p(rough), _p(metal), _p(refs), _p(counts),
                         _p(offsets), _p(indices), len(counts), len(indices), _p(_f(light_pos)), _p(_f(lights)), L,
                         _p(dl), nd, _p(_f(eye)), far, _p(_f(view_matrix)), _p(_f(proj)), _p(out))
        return out.reshape(H, W, 4)

    def bounce(self, positions, directions, L, mn, mx, speed, dt):
        p = np.array(_f(positions), copy=True)
        d = np.array(_f(directions), copy=True)
        self.L.ref_bounce(_p(p), _p(d), L, _p(_f(mn)), _p(_f(mx)), speed, dt)
        return p, d

    def depth_pyramid(self, depth, W, H, levels):
        """The reference's copy dispatch, then one reduce dispatch per level (max(1, size >> 1) each)."""
        out = [np.zeros(W * H, np.float32)]
        self.L.ref_depth_copy(_p(_f(depth)), W, H, _p(out[0]))
        w, h = W, H
        for _ in range(1, levels):
            tw, th = max(1, w >> 1), max(1, h >> 1)
            nxt = np.zeros(tw * th, np.float32)
            self.L.ref_depth_reduce(_p(out[-1]), w, h, _p(nxt), tw, th)
            out.append(nxt)
            w, h = tw, th
        return out

    def show_clusters(self, mode, W, H, refs, keys, counts=None, offsets=None, indices=None):
        TX, TY = (W + 31) // 32, (H + 31) // 32
        k = _u(keys)
        c = _u(counts) if counts is not None else None
        o = _u(offsets) if offsets is not None else None
        i = _u(indices) if indices is not None else np.zeros(1, np.uint32)
        out = np.zeros(W * H * 4, np.float32)
        self.L.ref_show_clusters(mode, W, H, TX, TY, _p(_u(refs)), _p(k), len(k), _p(c), _p(o), _p(i),
                                 0 if indices is None else len(i), _p(out))
        return out.reshape(H, W, 4)
