"""vren_gb300 — GB300-native (sm_103a) implementation of vren's parallel primitives and
clustered-shading light assignment.

The product is the C ABI in ``include/vren_gb300.h`` (``libvren_gb300.so``) and its C++20
mirror ``include/vren_gb300.hpp``.  This package is the Python host layer over the same ABI
(ctypes; torch tensors only as device memory and streams), used by the tests and the benchmark.
"""
from ._lib import VrenError, check, device_error, lib  # noqa: F401
from .primitives import (  # noqa: F401
    BVH_INVALID_NODE,
    BVH_LEAF_NODE,
    blelloch_scan,
    bucket_sort,
    build_bvh,
    calc_bvh_buffer_length,
    calc_bvh_buffer_size,
    calc_bvh_level_count,
    calc_bvh_padded_leaf_count,
    calc_bvh_root_index,
    calc_reduce_output_buffer_length,
    divide_and_ceil,
    radix_sort,
    reduce,
    reduce_scalar,
    round_to_next_power_of,
    round_to_next_power_of_2,
)
