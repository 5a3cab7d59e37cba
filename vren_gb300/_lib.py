"""Loader for the native libraries and the ctypes prototypes of the C ABI (include/vren_gb300.h).

The CUDA library must exist: nothing here falls back to another implementation.  Build it with
``python -c "import __graft_entry__ as g; g.build()"`` (or ``python -m vren_gb300._build``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import _build

VREN_OK = 0
VREN_ERR_ARG = 1
VREN_ERR_CAPACITY = 2
VREN_ERR_TIMEOUT = 3
VREN_ERR_CUDA = 4
VREN_ERR_STATE = 5

REDUCE_OPS = {"add": 0, "min": 1, "max": 2}
TUNE = {"scan_slices": 0, "spin_polls": 1, "radix_rank": 2, "radix_items": 3, "scan_staged": 4, "reduce_form": 5,
        "light_bvh_cluster": 6, "assign_fused": 7, "radix_persistent": 8, "fuc_fused": 9, "bucket_form": 10, "host_zero_copy": 11, "shade_packed": 12}

u32, u64, i32, sz, vp, fp = C.c_uint32, C.c_uint64, C.c_int, C.c_size_t, C.c_void_p, C.c_float

# name -> (restype, [argtypes])
PROTOTYPES: dict[str, tuple] = {
    "vren_status_string": (C.c_char_p, [i32]),
    "vren_device_error": (i32, [i32]),
    "vren_set_wait_limit": (u32, [u32]),
    "vren_test_withhold_scan_status": (i32, [u32]),
    "vren_test_withhold_bucket_scan_status": (i32, [u32]),
    "vren_tuning_set": (i32, [i32, i32]),
    "vren_tuning_get": (i32, [i32]),
    "vren_round_to_next_power_of_2": (u32, [u32]),
    "vren_round_to_next_power_of": (u32, [u32, u32]),
    "vren_divide_and_ceil": (u32, [u32, u32]),
    "vren_calc_reduce_output_buffer_length": (u32, [u32]),
    "vren_reduce_tree_u32": (i32, [vp, i32, vp, u32, vp, u32]),
    "vren_reduce_tree_vec4": (i32, [vp, i32, vp, u32, vp, u32]),
    "vren_reduce_scratch_bytes": (sz, [u32]),
    "vren_reduce_u32": (i32, [vp, i32, vp, u32, vp, vp]),
    "vren_reduce_f32": (i32, [vp, i32, vp, u32, vp, vp]),
    "vren_exclusive_scan_scratch_bytes": (sz, [u32, u32]),
    "vren_exclusive_scan_u32": (i32, [vp, vp, u32, u32, vp]),
    "vren_scan_downsweep_u32": (i32, [vp, vp, u32, u32, i32]),
    "vren_exclusive_scan_u32_noalloc": (i32, [vp, vp, u32, u32]),
    "vren_radix_sort_scratch1_bytes": (sz, [u32, u32]),
    "vren_radix_sort_u32": (i32, [vp, vp, u32, vp, vp]),
    "vren_radix_sort_u32_ex": (i32, [vp, vp, vp, u32, u32, vp, vp, vp]),
    "vren_bucket_sort_output_bytes": (sz, [u32, u32]),
    "vren_bucket_sort_scratch_bytes": (sz, [u32, u32]),
    "vren_bucket_sort_u32x2": (i32, [vp, vp, u32, vp, u32, vp]),
    "vren_calc_bvh_padded_leaf_count": (u32, [u32]),
    "vren_calc_bvh_buffer_length": (u32, [u32]),
    "vren_calc_bvh_buffer_size": (sz, [u32]),
    "vren_calc_bvh_root_index": (u32, [u32]),
    "vren_calc_bvh_level_count": (u32, [u32]),
    "vren_build_bvh": (i32, [vp, vp, u32]),
    "vren_lbvh_scratch_bytes": (C.c_size_t, [u32]),
    "vren_build_lbvh": (i32, [vp, vp, u32, vp, u32, vp, vp]),
    "vren_bounce_point_lights": (i32, [vp, vp, vp, u32, vp, vp, C.c_float, C.c_float]),
    "vren_depth_pyramid_level_count": (u32, [u32, u32]),
    "vren_depth_pyramid_level_offset": (sz, [u32, u32, u32]),
    "vren_depth_pyramid_scratch_bytes": (sz, [u32, u32]),
    "vren_depth_pyramid_copy_and_reduce": (i32, [vp, vp, u32, u32, vp, vp]),
    "vren_cs_show_clusters_scratch_bytes": (sz, [u32]),
    "vren_cs_show_clusters": (i32, [vp, i32, u32, u32, vp, vp, vp, u32, vp, vp, vp, u32, vp, vp]),
    "vren_cs_show_clusters_geometry": (i32, [vp, vp, vp, vp, u32, vp]),
    "vren_kd_tree_build": (sz, [vp, sz, vp, sz, vp, sz, sz]),
    "vren_kd_tree_depth": (u32, [vp, sz]),
    "vren_kd_tree_search": (None, [vp, sz, vp, sz, vp, sz, vp, vp, vp, vp, vp]),
    "vren_kd_tree_search_batch": (i32, [vp, vp, u32, u32, vp, u32, u32, vp, u32, u32, vp, vp, vp]),
}

_LIB: C.CDLL | None = None


def library_path() -> Path:
    return _build.CUDA_LIB


def lib() -> C.CDLL:
    """The loaded CUDA library (libvren_gb300.so).  Raises if it has not been built."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not path.exists():
            raise RuntimeError(
                f"{path} is missing: the CUDA extension of vren_gb300 has not been built "
                "(run __graft_entry__.build())")
        dll = C.CDLL(str(path))
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(dll, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = dll
    return _LIB


class VrenError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        msg = lib().vren_status_string(status).decode()
        super().__init__(f"{what}: {msg} (status {status})" if what else msg)
        self.status = status


def check(status: int, what: str = "") -> None:
    """Maps a C-ABI status to the reference's exception types: argument errors raise
    ValueError (std::invalid_argument in vren/primitives/radix_sort.cpp:158-161), the rest VrenError."""
    if status == VREN_OK:
        return
    if status == VREN_ERR_ARG:
        raise ValueError(f"{what}: invalid argument" if what else "invalid argument")
    raise VrenError(status, what)


def device_error(clear: bool = True) -> int:
    return int(lib().vren_device_error(1 if clear else 0))

# ---- clustered shading ----------------------------------------------------------------------------
PROTOTYPES_CS: dict[str, tuple] = {
    "vren_cs_view_from_camera": (None, [vp, u32, vp]),
    "vren_cs_frame_build": (i32, [vp, u32, u32, i32, vp]),
    "vren_cs_frame_upload": (i32, [vp, vp, vp]),
    "vren_cs_light_bvh_scratch_bytes": (sz, [u32, u32]),
    "vren_cs_construct_light_bvh": (i32, [vp, vp, vp, u32, vp, u32, vp, vp, vp, vp, vp]),
    "vren_cs_unique_clusters_scratch_bytes": (sz, [u32, u32]),
    "vren_cs_find_unique_clusters": (i32, [vp, vp, vp, u32, u32, vp, vp, u32, vp, vp, vp]),
    "vren_cs_assign_lights_scratch_bytes": (sz, [u32]),
    "vren_cs_assign_lights": (i32, [vp, vp, vp, u32, vp, vp, u32, vp, vp, vp, vp, vp, vp, u32, vp, vp]),
    "vren_cs_assign_lights_lbvh": (i32, [vp, vp, vp, u32, vp, vp, vp, u32, vp, vp, vp, vp, vp, vp, u32, vp, vp]),
    "vren_cs_create": (i32, [C.POINTER(vp), u32, u32, u32, u32]),
    "vren_cs_destroy": (None, [vp]),
    "vren_cs_set_options": (i32, [vp, vp]),
    "vren_cs_cluster": (i32, [vp, vp, vp, u32, u32, i32, vp, vp, vp, vp, u32]),
    "vren_cs_get_outputs": (i32, [vp, vp]),
    "vren_cs_cluster_and_shade": (i32, [vp, vp, vp, u32, u32, i32, vp, vp, vp, u32, vp, u32, i32, i32, vp]),
    "vren_cs_cluster_host": (i32, [vp, vp, vp, u32, u32, i32, vp, vp, vp, vp, u32, vp, vp, C.c_uint64]),
    "vren_cs_shade": (i32, [vp, vp, u32, u32, vp, vp, vp, vp, u32, vp, u32, i32, i32, vp]),
    "vren_cs_shade_backward_scratch_bytes": (sz, [u32, u32]),
    "vren_cs_shade_backward": (i32, [vp, vp, u32, u32, vp, vp, u32, vp, vp, u32, i32, vp, vp, vp, vp, vp]),
    "vren_cs_batch_create": (i32, [C.POINTER(vp)]),
    "vren_cs_batch_destroy": (None, [vp]),
    "vren_cs_batch_reserve": (i32, [vp, vp, u32, C.c_uint64]),
    "vren_cs_batch_set_options": (i32, [vp, vp]),
    "vren_cs_batch_get_options": (i32, [vp, vp]),
    "vren_cs_batch_run": (i32, [vp, vp, vp, u32]),
    "vren_cs_batch_autotune": (i32, [vp, vp, vp, u32, u32, vp]),
    "vren_cs_batch_frame_outputs": (i32, [vp, vp, u32, vp]),
}
PROTOTYPES.update(PROTOTYPES_CS)
