"""Bounded device-side waits on the GPU: one scan tile withholds its look-back status (a flag that
nothing ever publishes), so the look-back waits of the tiles after it run out after a short wait
limit.  The call returns, the kernels end, the device error word reports VREN_ERR_TIMEOUT, and after
the scratch is zero-filled again (the documented recovery) the next scan matches the oracle.  The
default wait limit and normal publication are restored whatever happens."""
import numpy as np
import pytest
import torch

import oracle
import vren_gb300 as vg
from vren_gb300 import _lib

pytestmark = pytest.mark.gpu

SHORT_WAIT = 4096  # polling rounds (a few milliseconds at most with the nanosleep back-off)
SCAN_FORM_KNOB = _lib.TUNE["scan_staged"]  # 0 automatic, 1 one tile per CTA in registers


def run_scan(lib, buf, n, scratch):
    return lib.vren_exclusive_scan_u32(None, buf.data_ptr(), n, 1, scratch.data_ptr())


@pytest.mark.parametrize("n,staged", [(100_000, 1), (1 << 22, 0)])  # one tile per CTA; the persistent grid
def test_scan_lookback_timeout_and_recovery(cuda, n, staged):
    lib = _lib.lib()
    data = np.random.default_rng(n).integers(0, 256, n, dtype=np.uint32)
    scratch = torch.zeros(int(lib.vren_exclusive_scan_scratch_bytes(n, 1)) // 4 + 4, dtype=torch.int32, device=cuda)
    buf = torch.from_numpy(data.view(np.int32)).to(cuda)
    knob = SCAN_FORM_KNOB
    old_mode = lib.vren_tuning_get(knob)
    lib.vren_tuning_set(knob, staged)
    torch.cuda.synchronize()
    vg.device_error(clear=True)
    prev = lib.vren_set_wait_limit(SHORT_WAIT)
    try:
        assert lib.vren_test_withhold_scan_status(2) == _lib.VREN_OK  # tile 1 never publishes
        assert run_scan(lib, buf, n, scratch) == _lib.VREN_OK
        torch.cuda.synchronize()  # the kernels ended: every wait gave up after the limit
        assert vg.device_error(clear=True) == _lib.VREN_ERR_TIMEOUT
    finally:
        lib.vren_test_withhold_scan_status(0)
        lib.vren_set_wait_limit(prev)
        lib.vren_tuning_set(knob, old_mode)
    # recovery: zero the scratch again, then a normal call is correct and records no error
    scratch.zero_()
    buf.copy_(torch.from_numpy(data.view(np.int32)))
    assert run_scan(lib, buf, n, scratch) == _lib.VREN_OK
    torch.cuda.synchronize()
    assert np.array_equal(buf.cpu().numpy().view(np.uint32), oracle.exclusive_scan_u32(data))
    assert vg.device_error(clear=True) == 0


def test_noalloc_scan_lookback_timeout_and_recovery(cuda):
    """The allocation-free scan clears its own scratch at every call, so the call after a timeout is
    correct without any action by the caller."""
    lib = _lib.lib()
    n = 200_000
    data = np.random.default_rng(3).integers(0, 256, n, dtype=np.uint32)
    buf = torch.from_numpy(data.view(np.int32)).to(cuda)
    torch.cuda.synchronize()
    vg.device_error(clear=True)
    prev = lib.vren_set_wait_limit(SHORT_WAIT)
    try:
        assert lib.vren_test_withhold_scan_status(3) == _lib.VREN_OK
        assert lib.vren_exclusive_scan_u32_noalloc(None, buf.data_ptr(), n, 1) == _lib.VREN_OK
        torch.cuda.synchronize()
        assert vg.device_error(clear=True) == _lib.VREN_ERR_TIMEOUT
    finally:
        lib.vren_test_withhold_scan_status(0)
        lib.vren_set_wait_limit(prev)
    buf.copy_(torch.from_numpy(data.view(np.int32)))
    assert lib.vren_exclusive_scan_u32_noalloc(None, buf.data_ptr(), n, 1) == _lib.VREN_OK
    torch.cuda.synchronize()
    assert np.array_equal(buf.cpu().numpy().view(np.uint32), oracle.exclusive_scan_u32(data))
    assert vg.device_error(clear=True) == 0


def test_bucket_column_scan_timeout_and_recovery(cuda):
    """The bucket sort's column scan (up to 10 key bits): row block 1 of 4 never publishes its
    look-back words, so blocks 2 and 3 wait until the short limit; the call returns, the device error
    word reports VREN_ERR_TIMEOUT, and the next call, with no action by the caller (the sort resets
    its look-back words itself), matches the oracle."""
    lib = _lib.lib()
    n = 1 << 22  # 1024 tile rows = 4 blocks of 256 rows
    rng = np.random.default_rng(11)
    pairs = np.stack([rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32),
                      np.arange(n, dtype=np.uint32)], 1).reshape(-1)
    bs = vg.bucket_sort(10)
    out = torch.zeros(bs.get_required_output_buffer_size(n) // 4, dtype=torch.int32, device=cuda)
    inp = torch.from_numpy(pairs.view(np.int32)).to(cuda)
    form = _lib.TUNE["bucket_form"]
    old_form = lib.vren_tuning_get(form)
    lib.vren_tuning_set(form, 0)
    torch.cuda.synchronize()
    vg.device_error(clear=True)
    prev = lib.vren_set_wait_limit(SHORT_WAIT)
    try:
        assert lib.vren_test_withhold_bucket_scan_status(2) == _lib.VREN_OK  # block 1 never publishes
        bs(None, inp, n, 0, out, 0)
        torch.cuda.synchronize()  # the kernels ended: every wait gave up after the limit
        assert vg.device_error(clear=True) == _lib.VREN_ERR_TIMEOUT
    finally:
        lib.vren_test_withhold_bucket_scan_status(0)
        lib.vren_set_wait_limit(prev)
    try:
        out.zero_()
        bs(None, inp, n, 0, out, 0)
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        exp_pairs, exp_ends = oracle.bucket_sort_u32x2(pairs.reshape(-1, 2), 10)
        assert np.array_equal(got[: 2 * n].reshape(-1, 2), exp_pairs)
        off = ((8 * n + 255) // 256 * 256) // 4
        assert np.array_equal(got[off: off + 1024], exp_ends)
        assert vg.device_error(clear=True) == 0
    finally:
        lib.vren_tuning_set(form, old_form)
