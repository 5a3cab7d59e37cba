"""Depth-buffer pyramid: vren::depth_buffer_pyramid and vren::depth_buffer_reductor
(vren/vren/pipeline/depth_buffer_pyramid.hpp) over the C ABI.

The pyramid is one float32 device tensor holding every level back to back (level l starts at
``level_offset(l)`` floats and is ``get_image_height(l) x get_image_width(l)`` row-major); ``level(l)``
returns that level as a 2-D view.
"""
from __future__ import annotations

import torch

from ._lib import check, lib
from .primitives import _ptr, _stream, alloc_scratch


class depth_buffer_pyramid:
    """vren::depth_buffer_pyramid (depth_buffer_pyramid.cpp:12-24): storage for all levels."""

    k_max_depth_buffer_pyramid_level_count = 16

    def __init__(self, width: int, height: int, device=None):
        self.m_base_width, self.m_base_height = int(width), int(height)
        self.m_level_count = int(lib().vren_depth_pyramid_level_count(width, height))
        if self.m_level_count == 0:
            raise ValueError(f"depth_buffer_pyramid: unsupported size {width}x{height}")
        total = int(lib().vren_depth_pyramid_level_offset(width, height, self.m_level_count))
        self.m_image = torch.empty(total, dtype=torch.float32, device=device or "cuda")

    def get_image_width(self, level: int) -> int:
        return max(self.m_base_width >> level, 1)

    def get_image_height(self, level: int) -> int:
        return max(self.m_base_height >> level, 1)

    def get_level_count(self) -> int:
        return self.m_level_count

    def level_offset(self, level: int) -> int:
        return int(lib().vren_depth_pyramid_level_offset(self.m_base_width, self.m_base_height, level))

    def level(self, level: int) -> torch.Tensor:
        o, w, h = self.level_offset(level), self.get_image_width(level), self.get_image_height(level)
        return self.m_image[o:o + w * h].view(h, w)


class depth_buffer_reductor:
    """vren::depth_buffer_reductor (depth_buffer_pyramid.cpp:174-305): copy_and_reduce writes level 0
    (the depth buffer, copied exactly) and every level above it in one launch on `stream`."""

    k_workgroup_size_x = 32
    k_workgroup_size_y = 32

    def __init__(self):
        self._scratch = None

    def copy_and_reduce(self, stream, depth_buffer: torch.Tensor, pyramid: depth_buffer_pyramid) -> None:
        w, h = pyramid.m_base_width, pyramid.m_base_height
        if depth_buffer.numel() < w * h or depth_buffer.dtype != torch.float32:
            raise ValueError("depth_buffer: float32 tensor of width * height texels expected")
        need = int(lib().vren_depth_pyramid_scratch_bytes(w, h))
        if self._scratch is None or self._scratch.numel() * 4 < need:
            self._scratch = alloc_scratch(need, depth_buffer.device)
        check(lib().vren_depth_pyramid_copy_and_reduce(_stream(stream), _ptr(depth_buffer), w, h,
                                                       _ptr(pyramid.m_image), _ptr(self._scratch)),
              "depth_buffer_reductor::copy_and_reduce")
