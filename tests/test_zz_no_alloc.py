"""The allocation-free scan entry point (vren_exclusive_scan_u32_noalloc) gives the same output as
the allocating one (vren_exclusive_scan_u32), on two calls in a row.

It exists for callers that cannot hand the library scratch memory — an engine whose allocator owns
all device memory, a plugin with no allocator, a frame loop that must not call cudaMalloc — and
keeps its look-back scratch in a fixed device array inside the library.  This file is collected
last so that a run stopping at the first failure has already run every other test; it also passes
on its own in a fresh process.
"""
import numpy as np
import pytest
import torch

import vren_gb300 as vg
from vren_gb300 import _lib

pytestmark = pytest.mark.gpu

MAX_ELEMENTS = 1 << 24


def _scan_both(cuda, x: np.ndarray, n: int, blocks: int):
    lib = vg.lib()
    stream = torch.cuda.current_stream().cuda_stream
    a = torch.from_numpy(x.view(np.int32)).to(cuda)
    b = a.clone()
    scratch = vg.primitives.alloc_scratch(lib.vren_exclusive_scan_scratch_bytes(n, blocks), cuda)
    assert lib.vren_exclusive_scan_u32(stream, a.data_ptr(), n, blocks, scratch.data_ptr()) == _lib.VREN_OK
    assert lib.vren_exclusive_scan_u32_noalloc(stream, b.data_ptr(), n, blocks) == _lib.VREN_OK
    torch.cuda.synchronize()
    return a.cpu().numpy().view(np.uint32), b.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("n,blocks", [(1, 1), (4095, 1), (4097, 1), (1 << 20, 1), (10000, 7), (MAX_ELEMENTS, 1)])
def test_noalloc_scan_matches_allocating_scan(cuda, n, blocks):
    rng = np.random.default_rng(n + blocks)
    for call in range(2):  # two calls in a row share (and must re-clear) the static scratch
        x = rng.integers(0, 256, n * blocks).astype(np.uint32)
        ref, got = _scan_both(cuda, x, n, blocks)
        assert np.array_equal(got, ref), f"call {call}"
        expect = np.concatenate([np.concatenate([[0], np.cumsum(s, dtype=np.uint64)[:-1]]).astype(np.uint32)
                                 for s in x.reshape(blocks, n)])
        assert np.array_equal(got, expect), f"call {call}"
    assert vg.device_error(clear=True) == 0


def test_noalloc_scan_rejects_inputs_beyond_its_capacity(cuda):
    lib = vg.lib()
    buf = torch.zeros(16, dtype=torch.int32, device=cuda)
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.vren_exclusive_scan_u32_noalloc(stream, buf.data_ptr(), MAX_ELEMENTS + 1, 1) == _lib.VREN_ERR_CAPACITY
    assert lib.vren_exclusive_scan_u32_noalloc(stream, buf.data_ptr(), MAX_ELEMENTS // 2, 3) == _lib.VREN_ERR_CAPACITY
    torch.cuda.synchronize()
    assert np.all(buf.cpu().numpy() == 0)  # nothing was enqueued
