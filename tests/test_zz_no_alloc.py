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


_CONTEXT_SCRIPT = r"""
import ctypes as C, sys
import numpy as np
lib = C.CDLL(sys.argv[1])
lib.vren_exclusive_scan_u32_noalloc.restype = C.c_int
lib.vren_exclusive_scan_u32_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32]
cu = C.CDLL("libcuda.so.1")
def ck(r, what):
    if r != 0:
        raise SystemExit(f"{what}: CUresult {r}")
ck(cu.cuInit(0), "cuInit")
dev = C.c_int()
ck(cu.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
def scan_in_current_context(seed):
    n = 100003
    x = np.random.default_rng(seed).integers(0, 256, n).astype(np.uint32)
    d = C.c_uint64()
    ck(cu.cuMemAlloc_v2(C.byref(d), C.c_size_t(n * 4)), "cuMemAlloc")
    ck(cu.cuMemcpyHtoD_v2(d, x.ctypes.data_as(C.c_void_p), C.c_size_t(n * 4)), "cuMemcpyHtoD")
    rc = lib.vren_exclusive_scan_u32_noalloc(None, C.c_void_p(d.value), n, 1)
    if rc != 0:
        raise SystemExit(f"scan status {rc}")
    ck(cu.cuCtxSynchronize(), "cuCtxSynchronize")
    y = np.empty(n, np.uint32)
    ck(cu.cuMemcpyDtoH_v2(y.ctypes.data_as(C.c_void_p), d, C.c_size_t(n * 4)), "cuMemcpyDtoH")
    ck(cu.cuMemFree_v2(d), "cuMemFree")
    expect = np.concatenate([[0], np.cumsum(x, dtype=np.uint64)[:-1]]).astype(np.uint32)
    if not np.array_equal(y, expect):
        raise SystemExit(f"wrong scan (seed {seed})")
primary = C.c_void_p()
ck(cu.cuDevicePrimaryCtxRetain(C.byref(primary), dev), "cuDevicePrimaryCtxRetain")
ck(cu.cuCtxSetCurrent(primary), "cuCtxSetCurrent")
scan_in_current_context(1)
other = C.c_void_p()
ck(cu.cuCtxCreate_v2(C.byref(other), 0, dev), "cuCtxCreate")  # current from here on
scan_in_current_context(2)
scan_in_current_context(3)
ck(cu.cuCtxDestroy_v2(other), "cuCtxDestroy")
ck(cu.cuCtxSetCurrent(primary), "cuCtxSetCurrent")
scan_in_current_context(4)
print("ok")
"""


def test_noalloc_scan_in_a_second_context(cuda, tmp_path):
    """A caller that runs the library under its own driver context (not the primary one, as an
    engine with its own CUDA context does) gets the static scratch of that context: the cached
    address is per context.  Runs in a child process, so this process's context stays untouched."""
    import subprocess
    import sys

    script = tmp_path / "noalloc_contexts.py"
    script.write_text(_CONTEXT_SCRIPT)
    r = subprocess.run([sys.executable, str(script), str(_lib.library_path())], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
