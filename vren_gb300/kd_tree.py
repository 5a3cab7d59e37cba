"""k-d tree (vren/vren/base/kd_tree.{hpp,cpp}) over the C ABI: the host build and search of the
reference (same node array, same results), and the batched nearest-neighbour search on the GPU.

Nodes are (n, 3) uint32 arrays: split bits or point index, axis (3 = leaf), value (right-child
distance or leaf-run length, 30 bits).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import check, lib
from .primitives import _ptr, _stream

FILTER = C.CFUNCTYPE(C.c_int, C.c_uint32, C.c_void_p)
MAX_DEPTH = 128


def _host(a, dtype):
    return np.ascontiguousarray(a, dtype)


def kd_tree_build(points, point_stride: int = 3, indices=None, max_leaf_point_count: int = 8):
    """vren::kd_tree_build on the host: returns (nodes, indices) — the node array (at most 2 * count
    nodes) and the index array as the build leaves it permuted."""
    pts = _host(points, np.float32).reshape(-1)
    count = pts.size // point_stride
    idx = np.arange(count, dtype=np.uint32) if indices is None else np.array(indices, np.uint32)
    nodes = np.zeros((max(2 * idx.size, 1), 3), np.uint32)
    n = lib().vren_kd_tree_build(pts.ctypes.data, point_stride, idx.ctypes.data, idx.size, nodes.ctypes.data, 0,
                                 max_leaf_point_count)
    return nodes[:n].copy(), idx


def kd_tree_depth(nodes) -> int:
    nd = _host(nodes, np.uint32)
    return int(lib().vren_kd_tree_depth(nd.ctypes.data, 0)) if nd.size else 0


def kd_tree_search(points, nodes, sample, point_stride: int = 3, filter_predicate=None,
                   best_point: int = 0xFFFFFFFF, best_distance_squared: float = float("inf")):
    """vren::kd_tree_search on the host for one sample; filter_predicate(point) -> bool (None = all).
    Returns (best_point, best_distance_squared)."""
    pts = _host(points, np.float32).reshape(-1)
    nd = _host(nodes, np.uint32)
    s = _host(sample, np.float32).reshape(-1)
    bp = C.c_uint32(best_point)
    bd = C.c_float(best_distance_squared)
    cb = FILTER(lambda p, _u: 1 if filter_predicate(int(p)) else 0) if filter_predicate is not None else None
    lib().vren_kd_tree_search(pts.ctypes.data, point_stride, None, pts.size // point_stride, nd.ctypes.data, 0,
                              s.ctypes.data, cb, None, C.byref(bp), C.byref(bd))
    return int(bp.value), float(bd.value)


def kd_tree_search_batch(stream, points: torch.Tensor, nodes: torch.Tensor, samples: torch.Tensor, max_depth: int,
                         point_stride: int = 3, sample_stride: int = 3, excluded: torch.Tensor | None = None,
                         best_points: torch.Tensor | None = None, best_distances: torch.Tensor | None = None):
    """The nearest neighbour of every sample on the GPU (device tensors): (best_points int32 tensor,
    best_distances_squared float32 tensor), equal to the host search of each sample."""
    q = samples.numel() // sample_stride
    dev = samples.device
    if best_points is None:
        best_points = torch.empty(q, dtype=torch.int32, device=dev)
    if best_distances is None:
        best_distances = torch.empty(q, dtype=torch.float32, device=dev)
    check(lib().vren_kd_tree_search_batch(_stream(stream), _ptr(points), point_stride, points.numel() // point_stride,
                                          _ptr(nodes), nodes.numel() // 3, max_depth, _ptr(samples), sample_stride, q,
                                          _ptr(excluded) if excluded is not None else None, _ptr(best_points),
                                          _ptr(best_distances)), "kd_tree_search_batch")
    return best_points, best_distances
