"""The depth-buffer pyramid (vren::depth_buffer_reductor::copy_and_reduce) against the CPU restatement
of the reference's copy dispatch and per-level reduce dispatches, bit for bit: odd sides, sides of 1,
NaN, -0, negative and infinite depths, the 128-bit and the scalar level-0 paths, every stage of the
one-launch hierarchy (levels 7..12 and 13..15), reuse of the scratch counters."""
import numpy as np
import pytest
import torch

import oracle
import vren_gb300 as vg
from vren_gb300._lib import lib
from vren_gb300.depth_pyramid import depth_buffer_pyramid, depth_buffer_reductor


def make_depth(w, h, seed):
    rng = np.random.default_rng(seed)
    d = rng.uniform(-0.1, 1.0, (h, w)).astype(np.float32)
    f = d.reshape(-1)
    f[rng.integers(0, f.size, max(f.size // 40, 1))] = np.nan
    f[rng.integers(0, f.size, max(f.size // 50, 1))] = -0.0
    f[rng.integers(0, f.size, max(f.size // 997, 1))] = np.inf
    return d


def check_pyramid(pyr, want):
    assert pyr.get_level_count() == len(want)
    for l, e in enumerate(want):
        g = pyr.level(l).cpu().numpy()
        assert g.shape == e.shape, l
        assert np.array_equal(g.view(np.uint32), e.view(np.uint32)), f"level {l}"


def test_level_layout_matches_reference_sizes(native):
    """Level count and sizes (depth_buffer_pyramid.cpp:18, :28-38, Vulkan mip sizes max(1, size >> level)); offsets 64-float aligned, disjoint."""
    for w, h in [(1, 1), (7, 3), (1920, 1080), (3840, 2160), (65535, 1), (1, 65535), (40000, 30000)]:
        n = lib().vren_depth_pyramid_level_count(w, h)
        assert n == oracle.depth_pyramid_level_count(w, h)
        end = 0
        for l in range(n):
            o = lib().vren_depth_pyramid_level_offset(w, h, l)
            assert o % 64 == 0 and o >= end
            end = o + max(w >> l, 1) * max(h >> l, 1)
        assert lib().vren_depth_pyramid_level_offset(w, h, n) >= end
    assert lib().vren_depth_pyramid_level_count(0, 4) == 0
    assert lib().vren_depth_pyramid_level_count(65536, 4) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("w,h", [(1, 1), (2, 1), (1, 9), (9, 1), (3, 5), (64, 64), (65, 127), (128, 1),
                                 (128, 128), (200, 77), (333, 257), (1920, 1080), (2560, 1440),
                                 (3840, 2160), (4100, 3), (8200, 3), (3, 8200), (260, 130), (4097, 4097)])
def test_pyramid_matches_oracle(cuda, w, h):
    d = make_depth(w, h, w * 7919 + h)
    pyr = depth_buffer_pyramid(w, h, cuda)
    depth = torch.from_numpy(d.reshape(-1)).to(cuda)
    depth_buffer_reductor().copy_and_reduce(None, depth, pyr)
    torch.cuda.synchronize()
    check_pyramid(pyr, oracle.depth_pyramid(d, w, h))
    assert vg.device_error() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("w,h", [(65535, 3), (3, 65535), (65535, 65)])
def test_pyramid_sixteen_levels(cuda, w, h):
    """The largest sides: 16 levels, the third stage of the hierarchy (levels 13..15)."""
    d = make_depth(w, h, w + h)
    pyr = depth_buffer_pyramid(w, h, cuda)
    assert pyr.get_level_count() == 16
    depth_buffer_reductor().copy_and_reduce(None, torch.from_numpy(d.reshape(-1)).to(cuda), pyr)
    torch.cuda.synchronize()
    check_pyramid(pyr, oracle.depth_pyramid(d, w, h))


@pytest.mark.gpu
def test_pyramid_scalar_level0_path(cuda):
    """Width a multiple of 4 but the depth buffer only 4-byte aligned: the scalar level-0 path."""
    w, h = 1024, 300
    d = make_depth(w, h, 5)
    buf = torch.zeros(w * h + 1, dtype=torch.float32, device=cuda)
    buf[1:] = torch.from_numpy(d.reshape(-1)).to(cuda)
    pyr = depth_buffer_pyramid(w, h, cuda)
    depth_buffer_reductor().copy_and_reduce(None, buf[1:], pyr)
    torch.cuda.synchronize()
    check_pyramid(pyr, oracle.depth_pyramid(d, w, h))


@pytest.mark.gpu
def test_pyramid_repeated_calls_reuse_scratch(cuda):
    """The arrival counters return to zero: the same reductor (scratch) serves many frames and sizes."""
    red = depth_buffer_reductor()
    s = torch.cuda.Stream()
    for i, (w, h) in enumerate([(1920, 1080), (1920, 1080), (8200, 3), (333, 257), (1920, 1080)]):
        d = make_depth(w, h, 100 + i)
        pyr = depth_buffer_pyramid(w, h, cuda)
        depth = torch.from_numpy(d.reshape(-1)).to(cuda)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            red.copy_and_reduce(s, depth, pyr)
        s.synchronize()
        check_pyramid(pyr, oracle.depth_pyramid(d, w, h))
    assert not red._scratch.any()


@pytest.mark.gpu
def test_pyramid_plain_depths_property(cuda):
    """Full-HD-plus size, depths in [0, 1): every level equals the max over its level-0 block
    (block 2^l per axis until the axis reaches one texel), computed with torch on the device."""
    w, h = 5120, 2880
    g = torch.Generator(device=cuda).manual_seed(9)
    depth = torch.rand(h * w, device=cuda, generator=g)
    pyr = depth_buffer_pyramid(w, h, cuda)
    depth_buffer_reductor().copy_and_reduce(None, depth, pyr)
    torch.cuda.synchronize()
    d0 = depth.view(h, w)
    kx, ky = w.bit_length() - 1, h.bit_length() - 1
    assert torch.equal(pyr.level(0), d0)
    for l in range(1, pyr.get_level_count()):
        wl, hl = max(w >> l, 1), max(h >> l, 1)
        bx, by = 1 << min(l, kx), 1 << min(l, ky)
        want = d0[:hl * by, :wl * bx].reshape(hl, by, wl, bx).amax(dim=(1, 3)).clamp_min(0.0)
        assert torch.equal(pyr.level(l), want), l


@pytest.mark.gpu
def test_pyramid_arguments(cuda):
    pyr = depth_buffer_pyramid(64, 64, cuda)
    red = depth_buffer_reductor()
    with pytest.raises(ValueError):
        red.copy_and_reduce(None, torch.zeros(10, device=cuda), pyr)
    with pytest.raises(ValueError):
        depth_buffer_pyramid(0, 4, cuda)
    with pytest.raises(ValueError):
        depth_buffer_pyramid(70000, 4, cuda)
    scratch = torch.zeros(16, dtype=torch.int32, device=cuda)
    depth = torch.zeros(64 * 64 + 1, device=cuda)
    assert lib().vren_depth_pyramid_copy_and_reduce(None, None, 64, 64, pyr.m_image.data_ptr(),
                                                    scratch.data_ptr()) == 1
    assert lib().vren_depth_pyramid_copy_and_reduce(None, depth.data_ptr(), 64, 64, pyr.m_image.data_ptr(),
                                                    None) == 1
    assert lib().vren_depth_pyramid_copy_and_reduce(None, depth.data_ptr() + 2, 64, 64, pyr.m_image.data_ptr(),
                                                    scratch.data_ptr()) == 1
    assert lib().vren_depth_pyramid_copy_and_reduce(None, depth.data_ptr(), 0, 64, pyr.m_image.data_ptr(),
                                                    scratch.data_ptr()) == 1
