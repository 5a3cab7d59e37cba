"""Python mirror of the reference's primitive call surface, over the C ABI.

Reference classes (loryruta/vren):
  vren::reduce<T, Op>   vren/vren/primitives/reduce.hpp:15-49
  vren::blelloch_scan   vren/vren/primitives/blelloch_scan.hpp:9-49
  vren::radix_sort      vren/vren/primitives/radix_sort.hpp:9-53
  vren::bucket_sort     vren/vren/primitives/bucket_sort.hpp:9-45
  vren::build_bvh       vren/vren/primitives/build_bvh.hpp:20-57

Buffers are CUDA tensors (the reference's vk_utils::buffer); offsets are in bytes, as in the
reference; the command buffer becomes a CUDA stream (default: torch's current stream).  Calls are
asynchronous and stream-ordered, like recording into a command buffer.
"""
from __future__ import annotations

import torch

from . import _lib
from ._lib import check, lib


def _stream(stream) -> int:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    return int(stream)


def _ptr(buf: torch.Tensor, offset_bytes: int = 0) -> int:
    if not buf.is_cuda:
        raise ValueError("device buffer expected")
    return buf.data_ptr() + int(offset_bytes)


def alloc_scratch(nbytes: int, device=None) -> torch.Tensor:
    """Caller-owned scratch, zero-filled (the primitives keep it reusable across calls)."""
    nwords = max(1, (int(nbytes) + 15) // 16 * 4)
    return torch.zeros(nwords, dtype=torch.int32, device=device or "cuda")


# ------------------------------------------------------------------------------------------------
# helpers of vren/vren/base/base.hpp
# ------------------------------------------------------------------------------------------------
def round_to_next_power_of_2(v: int) -> int:
    return int(lib().vren_round_to_next_power_of_2(v))


def round_to_next_power_of(n: int, base: int) -> int:
    return int(lib().vren_round_to_next_power_of(n, base))


def divide_and_ceil(value: int, divider: int) -> int:
    return int(lib().vren_divide_and_ceil(value, divider))


# ------------------------------------------------------------------------------------------------
# Reduce
# ------------------------------------------------------------------------------------------------
def calc_reduce_output_buffer_length(count: int) -> int:
    return int(lib().vren_calc_reduce_output_buffer_length(count))


class reduce:
    """vren::reduce<T, Op>: T in {"uint", "vec4"}, Op in {"add", "min", "max"}."""

    def __init__(self, data_type: str, operation: str):
        if data_type not in ("uint", "vec4") or operation not in _lib.REDUCE_OPS:
            raise ValueError("unsupported reduce instantiation")
        self.data_type = data_type
        self.op = _lib.REDUCE_OPS[operation]

    def __call__(self, stream, input_buffer: torch.Tensor, input_buffer_length: int, input_buffer_offset: int,
                 output_buffer: torch.Tensor | None = None, output_buffer_offset: int | None = None,
                 blocks_num: int = 1):
        if output_buffer is None:  # in-place form (reduce.hpp:39-46)
            output_buffer, output_buffer_offset = input_buffer, input_buffer_offset
        fn = lib().vren_reduce_tree_u32 if self.data_type == "uint" else lib().vren_reduce_tree_vec4
        check(fn(_stream(stream), self.op, _ptr(input_buffer, input_buffer_offset), input_buffer_length,
                 _ptr(output_buffer, output_buffer_offset), blocks_num), "reduce")


def reduce_scalar(stream, op: str, data: torch.Tensor, out: torch.Tensor, scratch: torch.Tensor) -> None:
    """Single-pass scalar reduction (u32 add/min/max, f32 min/max) into out[0]."""
    n = data.numel()
    if data.dtype == torch.float32:
        check(lib().vren_reduce_f32(_stream(stream), _lib.REDUCE_OPS[op], _ptr(data), n, _ptr(out), _ptr(scratch)),
              "reduce_f32")
    else:
        check(lib().vren_reduce_u32(_stream(stream), _lib.REDUCE_OPS[op], _ptr(data), n, _ptr(out), _ptr(scratch)),
              "reduce_u32")


def reduce_scratch_bytes(n: int) -> int:
    return int(lib().vren_reduce_scratch_bytes(n))


# ------------------------------------------------------------------------------------------------
# Blelloch scan
# ------------------------------------------------------------------------------------------------
class blelloch_scan:
    """vren::blelloch_scan.  The scan's scratch is owned by this object (grown on demand), the way
    the reference's toolbox owns the descriptor pools its dispatches use."""

    def __init__(self):
        self._scratch: torch.Tensor | None = None

    def _scratch_for(self, n: int, blocks: int, device) -> torch.Tensor:
        need = int(lib().vren_exclusive_scan_scratch_bytes(n, blocks))
        if self._scratch is None or self._scratch.numel() * 4 < need or self._scratch.device != device:
            self._scratch = alloc_scratch(need, device)
        return self._scratch

    def __call__(self, stream, buffer: torch.Tensor, length: int, offset: int = 0, blocks_num: int = 1):
        sc = self._scratch_for(length, blocks_num, buffer.device)
        check(lib().vren_exclusive_scan_u32(_stream(stream), _ptr(buffer, offset), length, blocks_num, _ptr(sc)),
              "blelloch_scan")

    def downsweep(self, stream, buffer: torch.Tensor, length: int, offset: int, blocks_num: int, clear_last: bool):
        check(lib().vren_scan_downsweep_u32(_stream(stream), _ptr(buffer, offset), length, blocks_num,
                                            1 if clear_last else 0), "blelloch_scan.downsweep")


# ------------------------------------------------------------------------------------------------
# Radix sort
# ------------------------------------------------------------------------------------------------
class radix_sort:
    """vren::radix_sort (keys only, in place) plus a key/value overload."""

    def __init__(self, digit_bits: int = 8):
        self.digit_bits = digit_bits

    def create_scratch_buffer_1(self, length: int, device=None) -> torch.Tensor:
        return alloc_scratch(lib().vren_radix_sort_scratch1_bytes(length, self.digit_bits), device)

    def create_scratch_buffer_2(self, length: int, device=None) -> torch.Tensor:
        return torch.empty(max(1, length), dtype=torch.int32, device=device or "cuda")

    def __call__(self, stream, buffer: torch.Tensor, length: int, scratch_buffer_1: torch.Tensor,
                 scratch_buffer_2: torch.Tensor):
        if self.digit_bits == 8:
            rc = lib().vren_radix_sort_u32(_stream(stream), _ptr(buffer), length, _ptr(scratch_buffer_1),
                                           _ptr(scratch_buffer_2))
            if rc == _lib.VREN_ERR_ARG:
                raise ValueError("Length must be higher than 1024 and a power of 2")
            check(rc, "radix_sort")
        else:
            self.sort(stream, buffer, None, length, scratch_buffer_1, scratch_buffer_2, None)

    def sort(self, stream, keys: torch.Tensor, values: torch.Tensor | None, length: int, scratch1: torch.Tensor,
             scratch_keys: torch.Tensor, scratch_values: torch.Tensor | None):
        check(lib().vren_radix_sort_u32_ex(_stream(stream), _ptr(keys), _ptr(values) if values is not None else None,
                                           length, self.digit_bits, _ptr(scratch1), _ptr(scratch_keys),
                                           _ptr(scratch_values) if scratch_values is not None else None),
              "radix_sort")


# ------------------------------------------------------------------------------------------------
# Bucket sort
# ------------------------------------------------------------------------------------------------
class bucket_sort:
    """vren::bucket_sort: uvec2(key, value) grouped by key & (2^key_bits - 1); stable."""

    k_key_bits = 16

    def __init__(self, key_bits: int = 16):
        self.key_bits = key_bits
        self._scratch: torch.Tensor | None = None

    def get_required_output_buffer_size(self, length: int) -> int:
        return int(lib().vren_bucket_sort_output_bytes(length, self.key_bits))

    def __call__(self, stream, input_buffer: torch.Tensor, input_buffer_length: int, input_buffer_offset: int,
                 output_buffer: torch.Tensor, output_buffer_offset: int):
        need = int(lib().vren_bucket_sort_scratch_bytes(input_buffer_length, self.key_bits))
        if self._scratch is None or self._scratch.numel() * 4 < need or self._scratch.device != input_buffer.device:
            self._scratch = alloc_scratch(need + 256, input_buffer.device)
        sc = _ptr(self._scratch)
        sc = (sc + 255) // 256 * 256
        check(lib().vren_bucket_sort_u32x2(_stream(stream), _ptr(input_buffer, input_buffer_offset),
                                           input_buffer_length, _ptr(output_buffer, output_buffer_offset),
                                           self.key_bits, sc), "bucket_sort")


# ------------------------------------------------------------------------------------------------
# BVH
# ------------------------------------------------------------------------------------------------
BVH_LEAF_NODE = 0xFFFFFFFF
BVH_INVALID_NODE = 0xFFFFFFFE


def calc_bvh_padded_leaf_count(n: int) -> int:
    return int(lib().vren_calc_bvh_padded_leaf_count(n))


def calc_bvh_buffer_length(n: int) -> int:
    return int(lib().vren_calc_bvh_buffer_length(n))


def calc_bvh_buffer_size(n: int) -> int:
    return int(lib().vren_calc_bvh_buffer_size(n))


def calc_bvh_root_index(n: int) -> int:
    return int(lib().vren_calc_bvh_root_index(n))


def calc_bvh_level_count(n: int) -> int:
    return int(lib().vren_calc_bvh_level_count(n))


class build_bvh:
    """vren::build_bvh: `buffer` holds bvh_node[calc_bvh_buffer_length(n)] (8 x 32-bit words each)
    with the leaves written; the parents are built in place."""

    def __call__(self, stream, buffer: torch.Tensor, leaf_count: int):
        check(lib().vren_build_bvh(_stream(stream), _ptr(buffer), leaf_count), "build_bvh")
