"""CPU oracle (TEST INFRASTRUCTURE ONLY) — ctypes bindings over oracle/_build/libvren_oracle.so.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this package, and
only as the oracle results are compared with, or as the timed CPU baseline.  See vren_oracle.h for what is pinned.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

_LIB = None
u32, u64, i32, vp = C.c_uint32, C.c_uint64, C.c_int, C.c_void_p

_PROTOS = {
    "oracle_round_to_next_power_of_2": (u32, [u32]),
    "oracle_round_to_next_power_of": (u32, [u32, u32]),
    "oracle_divide_and_ceil": (u32, [u32, u32]),
    "oracle_calc_bvh_padded_leaf_count": (u32, [u32]),
    "oracle_calc_bvh_buffer_length": (u32, [u32]),
    "oracle_calc_bvh_root_index": (u32, [u32]),
    "oracle_calc_bvh_level_count": (u32, [u32]),
    "oracle_reduce_tree_u32": (None, [i32, vp, u32, vp]),
    "oracle_reduce_tree_vec4": (None, [i32, vp, u32, vp]),
    "oracle_reduce_u32": (u32, [i32, vp, u64]),
    "oracle_reduce_f32": (C.c_float, [i32, vp, u64]),
    "oracle_exclusive_scan_u32": (None, [vp, u64]),
    "oracle_downsweep_u32": (None, [vp, u32, i32]),
    "oracle_stable_sort_u32": (None, [vp, vp, u64]),
    "oracle_bucket_sort_u32x2": (None, [vp, u32, u32, vp, vp]),
    "oracle_build_bvh": (None, [vp, u32]),
    "oracle_bvh_point_query": (u32, [vp, u32, vp, vp, u32]),
    "oracle_cs_slice_table": (None, [vp, u32, vp, vp]),
    "oracle_cs_light_bvh": (None, [vp, vp, u32, vp, u32, vp, vp, vp]),
    "oracle_cs_find_unique_clusters": (u32, [vp, vp, u32, u32, vp, i32, vp, u32, vp, i32]),
    "oracle_cs_assign_lights": (u64, [vp, u32, u32, u32, vp, vp, u32, vp, vp, vp, vp, vp, u64, i32]),
    "oracle_lbvh_build": (None, [vp, vp, u32, vp]),
    "oracle_bounce_point_lights": (None, [vp, vp, u32, vp, vp, C.c_float, C.c_float]),
    "oracle_depth_pyramid_level_count": (u32, [u32, u32]),
    "oracle_depth_pyramid": (None, [vp, u32, u32, vp]),
    "oracle_cs_show_clusters": (None, [i32, u32, u32, vp, vp, u32, vp, vp, vp, vp]),
    "oracle_cs_show_clusters_geometry": (None, [vp, u32, u32, vp, u32, vp]),
    "oracle_kd_tree_build": (u64, [vp, u64, vp, u64, vp, u64]),
    "oracle_kd_tree_search": (None, [vp, u64, vp, vp, u64, u32, vp, vp, vp]),
    "oracle_linear_nn_search": (None, [vp, u64, vp, u64, vp, u64, u32, vp, vp]),
    "oracle_cs_assign_lights_lbvh": (u64, [vp, u32, u32, u32, vp, vp, vp, vp, u32, vp, vp, vp, vp, vp, u64, i32]),
    "oracle_cs_shade_f64": (None, [vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, u32, i32, i32, vp, vp, i32]),
    "oracle_cs_shade_grad_f64": (None, [vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, u32, i32, vp, vp, i32]),
    "oracle_cs_shade_light_loss_f64": (C.c_double, [vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, u32, vp, i32, vp]),
    "oracle_cs_shade_grad_lights_f64": (None, [vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, u32, i32, vp,
                                               vp, u32, C.c_double, vp, vp, vp, i32]),
    "oracle_cs_light_codes": (None, [vp, u32, vp, u32, vp, vp, vp, vp]),
    "oracle_cs_normal_bins": (None, [vp, u64, vp]),
    "oracle_cs_pixel_keys": (None, [vp, vp, u32, u32, vp, vp]),
    "oracle_cs_cluster_boxes": (None, [vp, u64, u32, u32, vp, vp, vp]),
    "oracle_cs_test_aabb_aabb": (None, [vp, u64, vp]),
    "oracle_cs_test_sphere_aabb": (None, [vp, u64, vp]),
}

OPS = {"add": 0, "min": 1, "max": 2}


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = _build.build()
        dll = C.CDLL(str(path))
        for name, (res, args) in _PROTOS.items():
            f = getattr(dll, name)
            f.restype = res
            f.argtypes = args
        _LIB = dll
    return _LIB


def _p(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


# ---- primitives -------------------------------------------------------------------------------
def reduce_tree_u32(op: str, data: np.ndarray) -> np.ndarray:
    data = np.ascontiguousarray(data, dtype=np.uint32)
    P = int(lib().oracle_round_to_next_power_of_2(len(data)))
    out = np.empty(max(P, 0), dtype=np.uint32)
    if len(data):
        lib().oracle_reduce_tree_u32(OPS[op], _p(data), len(data), _p(out))
    return out


def reduce_tree_vec4(op: str, data: np.ndarray) -> np.ndarray:
    data = np.ascontiguousarray(data, dtype=np.float32).reshape(-1, 4)
    P = int(lib().oracle_round_to_next_power_of_2(len(data)))
    out = np.empty((P, 4), dtype=np.float32)
    if len(data):
        lib().oracle_reduce_tree_vec4(OPS[op], _p(data), len(data), _p(out))
    return out


def reduce_u32(op: str, data: np.ndarray) -> int:
    data = np.ascontiguousarray(data, dtype=np.uint32)
    return int(lib().oracle_reduce_u32(OPS[op], _p(data), len(data)))


def reduce_f32(op: str, data: np.ndarray) -> np.float32:
    data = np.ascontiguousarray(data, dtype=np.float32)
    return np.float32(lib().oracle_reduce_f32(OPS[op], _p(data), len(data)))


def exclusive_scan_u32(data: np.ndarray) -> np.ndarray:
    out = np.array(data, dtype=np.uint32, copy=True)
    lib().oracle_exclusive_scan_u32(_p(out), len(out))
    return out


def downsweep_u32(data: np.ndarray, clear_last: bool) -> np.ndarray:
    out = np.array(data, dtype=np.uint32, copy=True)
    lib().oracle_downsweep_u32(_p(out), len(out), 1 if clear_last else 0)
    return out


def stable_sort_u32(keys: np.ndarray, values: np.ndarray | None = None):
    k = np.array(keys, dtype=np.uint32, copy=True)
    v = None if values is None else np.array(values, dtype=np.uint32, copy=True)
    lib().oracle_stable_sort_u32(_p(k), _p(v), len(k))
    return k if v is None else (k, v)


def bucket_sort_u32x2(pairs: np.ndarray, key_bits: int):
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
    out = np.empty_like(pairs)
    ends = np.empty(1 << key_bits, dtype=np.uint32)
    lib().oracle_bucket_sort_u32x2(_p(pairs), len(pairs), key_bits, _p(out), _p(ends))
    return out, ends


def build_bvh(nodes: np.ndarray, padded_leaf_count: int) -> np.ndarray:
    """nodes: uint32 array of shape (buffer_length, 8) with the leaves filled."""
    out = np.array(nodes, dtype=np.uint32, copy=True)
    lib().oracle_build_bvh(_p(out), padded_leaf_count)
    return out


def bvh_point_query(nodes: np.ndarray, root_index: int, p) -> list[int]:
    nodes = np.ascontiguousarray(nodes, dtype=np.uint32)
    pt = np.asarray(p, dtype=np.float32)
    cap = max(1, len(nodes))
    out = np.empty(cap, dtype=np.uint32)
    n = int(lib().oracle_bvh_point_query(_p(nodes), root_index, _p(pt), _p(out), cap))
    return out[: min(n, cap)].tolist()


def size_helpers(n: int) -> dict:
    L = lib()
    return {
        "padded": int(L.oracle_calc_bvh_padded_leaf_count(n)),
        "length": int(L.oracle_calc_bvh_buffer_length(n)),
        "root": int(L.oracle_calc_bvh_root_index(n)),
        "levels": int(L.oracle_calc_bvh_level_count(n)),
    }


# ---- clustered shading --------------------------------------------------------------------------
def _view_ptr(view):
    import ctypes
    return ctypes.cast(ctypes.byref(view), ctypes.c_void_p).value


def cs_slice_table(view, tiles_y: int):
    near = np.empty(1024, np.float32)
    far = np.empty(1024, np.float32)
    lib().oracle_cs_slice_table(_view_ptr(view), tiles_y, _p(near), _p(far))
    return near, far


def cs_light_bvh(positions: np.ndarray, lights: np.ndarray, L: int, view, morton_bits: int = 15):
    P = int(lib().oracle_calc_bvh_padded_leaf_count(L))
    length = int(lib().oracle_calc_bvh_buffer_length(P))
    vp = np.zeros(L * 4, np.float32)
    bvh = np.zeros((length, 8), np.uint32)
    li = np.zeros(L * 2, np.uint32)
    if L:
        lib().oracle_cs_light_bvh(_p(np.ascontiguousarray(positions, np.float32)),
                                  _p(np.ascontiguousarray(lights, np.float32)), L, _view_ptr(view), morton_bits,
                                  _p(vp), _p(bvh), _p(li))
    return vp, bvh, li


def cs_find_unique_clusters(depth, normals, W: int, H: int, view, policy: int = 0, threads: int = 0):
    T = ((W + 31) // 32) * ((H + 31) // 32)
    keys = np.zeros(T * 1024, np.uint32)
    refs = np.zeros(W * H, np.uint32)
    U = lib().oracle_cs_find_unique_clusters(_p(np.ascontiguousarray(depth, np.float32)),
                                             _p(np.ascontiguousarray(normals, np.float32)), W, H, _view_ptr(view),
                                             policy, _p(keys), len(keys), _p(refs), threads)
    return keys[:U].copy(), refs


def cs_assign_lights(keys, W: int, H: int, view, bvh, L: int, light_index, view_pos, threads: int = 0,
                     index_cap: int | None = None):
    U = len(keys)
    counts = np.zeros(max(U, 1), np.uint32)
    offsets = np.zeros(max(U, 1), np.uint32)
    cap = index_cap if index_cap is not None else 1 << 26
    indices = np.zeros(cap, np.uint32)
    total = lib().oracle_cs_assign_lights(_p(np.ascontiguousarray(keys, np.uint32)), U, W, H, _view_ptr(view),
                                          _p(np.ascontiguousarray(bvh, np.uint32)), L,
                                          _p(np.ascontiguousarray(light_index, np.uint32)),
                                          _p(np.ascontiguousarray(view_pos, np.float32)), _p(counts), _p(offsets),
                                          _p(indices), cap, threads)
    return counts[:U], offsets[:U], indices[: min(total, cap)].copy(), int(total)


def cs_show_clusters(mode: int, W: int, H: int, refs, keys, counts=None, offsets=None, indices=None) -> np.ndarray:
    """vren_demo's show_clusters view (vren_oracle.c): (H, W, 4) float32 RGBA."""
    k = np.ascontiguousarray(keys, np.uint32)
    U = k.size
    z = np.zeros(1, np.uint32)
    c = np.ascontiguousarray(counts if counts is not None else z, np.uint32)
    o = np.ascontiguousarray(offsets if offsets is not None else z, np.uint32)
    i = np.ascontiguousarray(indices if indices is not None and len(indices) else z, np.uint32)
    out = np.empty((H, W, 4), np.float32)
    lib().oracle_cs_show_clusters(mode, W, H, _p(np.ascontiguousarray(refs, np.uint32)), _p(k if U else z), U,
                                  _p(c), _p(o), _p(i), _p(out))
    return out


def cs_show_clusters_geometry(view, W: int, H: int, keys) -> np.ndarray:
    """vren_demo's show_clusters_geometry (vren_oracle.c): (U, 32, 4) uint32 debug vertices
    (x, y, z float bits, colour)."""
    k = np.ascontiguousarray(keys, np.uint32)
    out = np.zeros((max(k.size, 1), 32, 4), np.uint32)
    lib().oracle_cs_show_clusters_geometry(_view_ptr(view), W, H, _p(k if k.size else np.zeros(1, np.uint32)),
                                           k.size, _p(out))
    return out[:k.size]


def kd_tree_build(points, stride: int = 3, max_leaf: int = 8, indices=None):
    """vren's kd_tree_build (vren_oracle.c): returns (nodes (n, 3) uint32, permuted indices)."""
    pts = np.ascontiguousarray(points, np.float32).reshape(-1)
    count = pts.size // stride
    idx = np.arange(count, dtype=np.uint32) if indices is None else np.array(indices, np.uint32)
    nodes = np.zeros((max(2 * len(idx), 1), 3), np.uint32)
    n = lib().oracle_kd_tree_build(_p(pts), stride, _p(idx), len(idx), _p(nodes), max_leaf)
    return nodes[:n].copy(), idx


def kd_tree_search(points, nodes, samples, stride: int = 3, sample_stride: int = 3, excluded=None):
    """Recursive kd_tree_search per sample from (UINT32_MAX, +inf): (best_points, best_dist)."""
    pts = np.ascontiguousarray(points, np.float32).reshape(-1)
    smp = np.ascontiguousarray(samples, np.float32).reshape(-1)
    q = smp.size // sample_stride
    bp = np.zeros(max(q, 1), np.uint32)
    bd = np.zeros(max(q, 1), np.float32)
    ex = None if excluded is None else np.ascontiguousarray(excluded, np.uint8)
    lib().oracle_kd_tree_search(_p(pts), stride, _p(np.ascontiguousarray(nodes, np.uint32)), _p(smp), sample_stride,
                                q, None if ex is None else _p(ex), _p(bp), _p(bd))
    return bp[:q], bd[:q]


def linear_nn_search(points, samples, stride: int = 3, sample_stride: int = 3, indices=None):
    pts = np.ascontiguousarray(points, np.float32).reshape(-1)
    smp = np.ascontiguousarray(samples, np.float32).reshape(-1)
    count = pts.size // stride
    idx = np.arange(count, dtype=np.uint32) if indices is None else np.ascontiguousarray(indices, np.uint32)
    q = smp.size // sample_stride
    bp = np.zeros(max(q, 1), np.uint32)
    bd = np.zeros(max(q, 1), np.float32)
    lib().oracle_linear_nn_search(_p(pts), stride, _p(idx), len(idx), _p(smp), sample_stride, q, _p(bp), _p(bd))
    return bp[:q], bd[:q]


def bounce_point_lights(positions, directions, L: int, aabb_min, aabb_max, speed: float, dt: float):
    """vren_demo's point-light bouncer (vren_oracle.c); returns new (positions, directions) arrays."""
    p = np.array(positions, np.float32).reshape(-1).copy()
    d = np.array(directions, np.float32).reshape(-1).copy()
    lo = np.array(aabb_min, np.float32)
    hi = np.array(aabb_max, np.float32)
    lib().oracle_bounce_point_lights(_p(p), _p(d), L, _p(lo), _p(hi), float(speed), float(dt))
    return p, d


def depth_pyramid_level_count(width: int, height: int) -> int:
    return int(lib().oracle_depth_pyramid_level_count(width, height))


def depth_pyramid(depth, width: int, height: int) -> list:
    """vren's depth-buffer pyramid (vren_oracle.c): one (h_l, w_l) float32 array per level."""
    d = np.ascontiguousarray(depth, np.float32).reshape(-1)
    assert d.size == width * height
    levels = depth_pyramid_level_count(width, height)
    sizes = [(max(height >> l, 1), max(width >> l, 1)) for l in range(levels)]
    out = np.empty(sum(h * w for h, w in sizes), np.float32)
    lib().oracle_depth_pyramid(_p(d), width, height, _p(out))
    res, o = [], 0
    for h, w in sizes:
        res.append(out[o:o + h * w].reshape(h, w))
        o += h * w
    return res


def lbvh_group_boxes(bvh, L: int) -> np.ndarray:
    """Per leaf, the box the reference's traversal effectively tests: its 32-leaf group's AABB (level 1
    of the 32-ary BVH), or an infinite box when L <= 32 (no box is tested then).  (L, 8) uint32."""
    b = np.ascontiguousarray(bvh, np.uint32).reshape(-1, 8)
    out = np.zeros((max(L, 1), 8), np.uint32)
    if L <= 32:
        f = out.view(np.float32)
        f[:, 0:3] = -np.inf
        f[:, 4:7] = np.inf
    else:
        P = 32
        while P < L:
            P *= 32
        out[:L] = b[P + np.arange(L) // 32]
    return out[:L]


def lbvh_build(light_index, boxes, L: int) -> np.ndarray:
    """Karras binary radix tree over the L sorted leaves with the given per-leaf boxes (vren_oracle.c):
    (L - 1, 8) uint32 nodes [min xyz, left, max xyz, right] as raw words; leaf children carry bit 31."""
    nodes = np.zeros((max(L - 1, 1), 8), np.uint32)
    lib().oracle_lbvh_build(_p(np.ascontiguousarray(light_index, np.uint32)),
                            _p(np.ascontiguousarray(boxes, np.uint32)), L, _p(nodes))
    return nodes[: max(L - 1, 0)]


def cs_assign_lights_lbvh(keys, W: int, H: int, view, nodes, boxes, bvh, L: int, light_index, view_pos,
                          threads: int = 0, index_cap: int | None = None):
    """assign_lights by the Karras tree built over `boxes`: lights whose box and sphere overlap."""
    U = len(keys)
    counts = np.zeros(max(U, 1), np.uint32)
    offsets = np.zeros(max(U, 1), np.uint32)
    cap = index_cap if index_cap is not None else 1 << 26
    indices = np.zeros(cap, np.uint32)
    nd = np.ascontiguousarray(nodes, np.uint32) if len(nodes) else np.zeros((1, 8), np.uint32)
    total = lib().oracle_cs_assign_lights_lbvh(_p(np.ascontiguousarray(keys, np.uint32)), U, W, H, _view_ptr(view),
                                               _p(nd), _p(np.ascontiguousarray(boxes, np.uint32)),
                                               _p(np.ascontiguousarray(bvh, np.uint32)), L,
                                               _p(np.ascontiguousarray(light_index, np.uint32)),
                                               _p(np.ascontiguousarray(view_pos, np.float32)), _p(counts),
                                               _p(offsets), _p(indices), cap, threads)
    return counts[:U], offsets[:U], indices[: min(total, cap)].copy(), int(total)


# ---- shading (FP64) -----------------------------------------------------------------------------
def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _u32(a):
    return np.ascontiguousarray(a, np.uint32)


def cs_shade_f64(view, W, H, gb, lists, lpos, lights, L, falloff=1, mode=1, threads=0):
    """gb = (depth, normals, albedo, roughness, metallic); lists = (refs, counts, offsets, indices)."""
    out = np.zeros(W * H * 3, np.float64)
    shaded = np.zeros(W * H, np.uint8)
    g = [_f32(x) for x in gb]
    ls = [_u32(x) for x in lists]
    lib().oracle_cs_shade_f64(_view_ptr(view), W, H, *(_p(x) for x in g), *(_p(x) for x in ls), _p(_f32(lpos)),
                              _p(_f32(lights)), L, falloff, mode, _p(out), _p(shaded), threads or 8)
    return out, shaded.astype(bool)


def cs_shade_grad_f64(view, W, H, gb, lists, lpos, lights, L, grad, falloff=1, threads=0):
    g7 = np.zeros(L * 7, np.float64)
    g = [_f32(x) for x in gb]
    ls = [_u32(x) for x in lists]
    lib().oracle_cs_shade_grad_f64(_view_ptr(view), W, H, *(_p(x) for x in g), *(_p(x) for x in ls),
                                   _p(_f32(lpos)), _p(_f32(lights)), L, falloff, _p(_f32(grad)), _p(g7), threads or 8)
    return g7.reshape(L, 7)


def cs_shade_light_loss_f64(view, W, H, gb, lists, l, theta, grad, falloff=1):
    g = [_f32(x) for x in gb]
    ls = [_u32(x) for x in lists]
    th = np.ascontiguousarray(theta, np.float64)
    return float(lib().oracle_cs_shade_light_loss_f64(_view_ptr(view), W, H, *(_p(x) for x in g),
                                                      *(_p(x) for x in ls), l, _p(th), falloff, _p(_f32(grad))))


def cs_shade_grad_lights_f64(view, W, H, gb, lists, lpos, lights, L, grad, sel, h=1e-4, falloff=1, threads=0):
    """FP64 gradient and central differences (step h) for the lights in `sel` only, over their own
    (pixel, light) pairs: returns (g7, fd7, pairs) with g7 and fd7 of shape (len(sel), 7)."""
    sel = _u32(sel)
    n = len(sel)
    g7 = np.zeros(n * 7, np.float64)
    fd7 = np.zeros(n * 7, np.float64)
    pairs = np.zeros(n, np.uint64)
    g = [_f32(x) for x in gb]
    ls = [_u32(x) for x in lists]
    lib().oracle_cs_shade_grad_lights_f64(_view_ptr(view), W, H, *(_p(x) for x in g), *(_p(x) for x in ls),
                                          _p(_f32(lpos)), _p(_f32(lights)), L, falloff, _p(_f32(grad)), _p(sel), n,
                                          float(h), _p(g7), _p(fd7), _p(pairs), threads or 8)
    return g7.reshape(n, 7), fd7.reshape(n, 7), pairs


# ---- per-element steps (compared with the reference's shaders run on the CPU, oracle/ref.py) --------
def cs_light_codes(positions, L: int, view, morton_bits: int = 15):
    """(view positions vec4[L], min vec4, max vec4, unsorted (code, light) pairs uint32[L, 2])."""
    vp = np.zeros(max(L, 1) * 4, np.float32)
    mn = np.zeros(4, np.float32)
    mx = np.zeros(4, np.float32)
    codes = np.zeros(max(L, 1) * 2, np.uint32)
    lib().oracle_cs_light_codes(_p(_f32(positions)), L, _view_ptr(view), morton_bits, _p(vp), _p(mn), _p(mx), _p(codes))
    return vp[: 4 * L], mn, mx, codes[: 2 * L].reshape(L, 2)


def cs_normal_bins(normals) -> np.ndarray:
    n = _f32(normals).reshape(-1, 3)
    out = np.zeros(len(n), np.uint32)
    lib().oracle_cs_normal_bins(_p(np.ascontiguousarray(n)), len(n), _p(out))
    return out


def cs_pixel_keys(depth, normals, W: int, H: int, view) -> np.ndarray:
    """Keys of every invocation of the unique-cluster dispatch: (TY*32, TX*32), overhang wrapped."""
    TX, TY = (W + 31) // 32, (H + 31) // 32
    out = np.zeros((TY * 32, TX * 32), np.uint32)
    lib().oracle_cs_pixel_keys(_p(_f32(depth)), _p(_f32(normals)), W, H, _view_ptr(view), _p(out))
    return out


def cs_cluster_boxes(keys, W: int, H: int, view):
    k = _u32(keys)
    mn = np.zeros((len(k), 3), np.float32)
    mx = np.zeros((len(k), 3), np.float32)
    lib().oracle_cs_cluster_boxes(_p(k), len(k), W, H, _view_ptr(view), _p(mn), _p(mx))
    return mn, mx


def cs_test_aabb_aabb(t) -> np.ndarray:
    t = _f32(t).reshape(-1, 12)
    out = np.zeros(len(t), np.uint8)
    lib().oracle_cs_test_aabb_aabb(_p(np.ascontiguousarray(t)), len(t), _p(out))
    return out


def cs_test_sphere_aabb(t) -> np.ndarray:
    t = _f32(t).reshape(-1, 10)
    out = np.zeros(len(t), np.uint8)
    lib().oracle_cs_test_sphere_aabb(_p(np.ascontiguousarray(t)), len(t), _p(out))
    return out
