"""Python mirror of vren::clustered_shading and vren::cluster_and_shade over the C ABI.

Reference: vren/vren/pipeline/clustered_shading.hpp:13-182.  The stage classes keep the reference
names; their buffers are CUDA tensors.  Frame parameters (camera matrices, slice tables) travel in a
device-resident ``vren_cs_frame`` block built on the host.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import check, lib
from .primitives import _ptr, _stream, alloc_scratch, calc_bvh_buffer_length, calc_bvh_padded_leaf_count

SLICES = 1024
SLICING = {"ref": 0, "fixed32": 1}
OFFSCREEN = {"wrap": 0, "skip": 1}


class Camera(C.Structure):
    """vren::camera (vren/vren/camera.hpp:14-33)."""
    _fields_ = [("position", C.c_float * 3), ("yaw", C.c_float), ("pitch", C.c_float), ("fov_y", C.c_float),
                ("aspect_ratio", C.c_float), ("near_plane", C.c_float), ("far_plane", C.c_float)]


class View(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("inv_proj", C.c_float * 16), ("inv_view", C.c_float * 16),
                ("eye", C.c_float * 3), ("near_plane", C.c_float), ("far_plane", C.c_float),
                ("half_fov_y", C.c_float), ("slicing", C.c_uint32), ("reserved", C.c_uint32)]


class Frame(C.Structure):
    _fields_ = [("view", View), ("width", C.c_uint32), ("height", C.c_uint32), ("tiles_x", C.c_uint32),
                ("tiles_y", C.c_uint32), ("max_slice", C.c_uint32), ("offscreen", C.c_uint32),
                ("normal_format", C.c_uint32), ("reserved", C.c_uint32), ("slice_near", C.c_float * SLICES),
                ("slice_far", C.c_float * SLICES)]


class Options(C.Structure):
    _fields_ = [("morton_bits", C.c_uint32), ("use_graph", C.c_uint32), ("sort_digit_bits", C.c_uint32),
                ("assign_warps", C.c_uint32), ("normal_format", C.c_uint32)]


class Outputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("view_positions", "bvh", "light_index", "leaf_spheres", "cluster_keys",
                                           "key_count", "cluster_refs", "counts", "offsets", "indices", "total",
                                           "frame")] + [("key_capacity", C.c_uint32), ("index_capacity", C.c_uint32)]


def scene_camera(width: int, height: int, fov_y_deg: float = 45.0, near: float = 0.1, far: float = 1000.0,
                 position=(0.0, 0.0, 0.0), yaw: float = 0.0, pitch: float = 0.0) -> Camera:
    cam = Camera()
    cam.position[:] = list(position)
    cam.yaw, cam.pitch = yaw, pitch
    cam.fov_y = np.float32(np.deg2rad(fov_y_deg))
    cam.aspect_ratio = width / height
    cam.near_plane, cam.far_plane = near, far
    return cam


def view_from_camera(cam: Camera, slicing: str = "ref") -> View:
    v = View()
    lib().vren_cs_view_from_camera(C.byref(cam), SLICING[slicing], C.byref(v))
    return v


NORMALS = {"f32x3": 0, "rgba16f": 1}


def normal_format_of(normals) -> int:
    """f32x3 normals for a float32 tensor, the reference's RGBA16F G-buffer layout for a float16 one."""
    return NORMALS["rgba16f"] if getattr(normals, "dtype", None) in (torch.float16, np.float16) else NORMALS["f32x3"]


def frame_build(view: View, width: int, height: int, offscreen: str = "wrap", normal_format: int = 0) -> Frame:
    f = Frame()
    check(lib().vren_cs_frame_build(C.byref(view), width, height, OFFSCREEN[offscreen], C.byref(f)), "frame_build")
    f.normal_format = normal_format
    return f


def frame_to_device(frame: Frame, device=None, stream=None) -> torch.Tensor:
    buf = torch.empty(C.sizeof(Frame) // 4, dtype=torch.int32, device=device or "cuda")
    check(lib().vren_cs_frame_upload(_stream(stream), C.byref(frame), _ptr(buf)), "frame_upload")
    return buf


class construct_point_light_bvh:
    """vren::clustered_shading::construct_point_light_bvh (clustered_shading.hpp:19-46)."""

    def __init__(self, morton_bits: int = 15):
        self.morton_bits = morton_bits
        self._scratch = None

    @staticmethod
    def get_required_bvh_buffer_size(light_count: int) -> int:
        return calc_bvh_buffer_length(light_count) * 32

    def __call__(self, stream, positions: torch.Tensor, lights: torch.Tensor, light_count: int,
                 frame_dev: torch.Tensor, view_positions: torch.Tensor, bvh: torch.Tensor,
                 light_index: torch.Tensor, leaf_spheres: torch.Tensor | None = None):
        need = int(lib().vren_cs_light_bvh_scratch_bytes(light_count, self.morton_bits))
        if self._scratch is None or self._scratch.numel() * 4 < need:
            self._scratch = alloc_scratch(need, positions.device)
        check(lib().vren_cs_construct_light_bvh(
            _stream(stream), _ptr(positions), _ptr(lights), light_count, _ptr(frame_dev), self.morton_bits,
            _ptr(view_positions), _ptr(bvh), _ptr(light_index),
            _ptr(leaf_spheres) if leaf_spheres is not None else None, _ptr(self._scratch)), "construct_point_light_bvh")


class find_unique_cluster_list:
    """vren::clustered_shading::find_unique_cluster_list (clustered_shading.hpp:52-74)."""

    def __init__(self):
        self._scratch = None

    def __call__(self, stream, width: int, height: int, frame_dev: torch.Tensor, depth: torch.Tensor,
                 normals: torch.Tensor, cluster_keys: torch.Tensor, key_count: torch.Tensor,
                 cluster_refs: torch.Tensor):
        need = int(lib().vren_cs_unique_clusters_scratch_bytes(width, height))
        if self._scratch is None or self._scratch.numel() * 4 < need:
            self._scratch = alloc_scratch(need, depth.device)
        check(lib().vren_cs_find_unique_clusters(
            _stream(stream), _ptr(depth), _ptr(normals), width, height, _ptr(frame_dev), _ptr(cluster_keys),
            cluster_keys.numel(), _ptr(key_count), _ptr(cluster_refs), _ptr(self._scratch)), "find_unique_cluster_list")


class assign_lights:
    """vren::clustered_shading::assign_lights (clustered_shading.hpp:80-108)."""

    def __init__(self):
        self._scratch = None

    def __call__(self, stream, cluster_keys: torch.Tensor, key_count: torch.Tensor, frame_dev: torch.Tensor,
                 bvh: torch.Tensor, light_count: int, light_index: torch.Tensor, view_positions: torch.Tensor,
                 counts: torch.Tensor, offsets: torch.Tensor, indices: torch.Tensor, total: torch.Tensor,
                 leaf_spheres: torch.Tensor | None = None):
        cap = cluster_keys.numel()
        need = int(lib().vren_cs_assign_lights_scratch_bytes(cap))
        if self._scratch is None or self._scratch.numel() * 4 < need:
            self._scratch = alloc_scratch(need, cluster_keys.device)
        check(lib().vren_cs_assign_lights(
            _stream(stream), _ptr(cluster_keys), _ptr(key_count), cap, _ptr(frame_dev),
            _ptr(bvh) if bvh is not None else None, light_count,
            _ptr(light_index) if light_index is not None else None,
            _ptr(view_positions) if view_positions is not None else None,
            _ptr(leaf_spheres) if leaf_spheres is not None else None,
            _ptr(counts), _ptr(offsets), _ptr(indices) if indices is not None else None,
            indices.numel() if indices is not None else 0, _ptr(total), _ptr(self._scratch)), "assign_lights")


def bounce_point_lights(stream, positions: torch.Tensor, directions: torch.Tensor, light_count: int, aabb_min,
                        aabb_max, speed: float, dt: float) -> None:
    """vren_demo's point-light bouncer (vren_bounce_point_lights): positions and directions (vec4 per
    light, float32 device tensors) updated in place."""
    lo = (C.c_float * 3)(*[float(x) for x in aabb_min])
    hi = (C.c_float * 3)(*[float(x) for x in aabb_max])
    check(lib().vren_bounce_point_lights(_stream(stream), _ptr(positions), _ptr(directions), light_count, lo, hi,
                                         float(speed), float(dt)), "bounce_point_lights")


class build_lbvh:
    """Karras binary radix tree over sorted leaves (extension; vren_build_lbvh).  `sorted_pairs` is a
    uvec2(key, payload) tensor in key order; leaf i's box is boxes[i >> box_shift] (None: infinite).
    Nodes: int32 tensor of (leaf_count - 1) * 8 words."""

    def __init__(self):
        self._scratch = None

    @staticmethod
    def group_boxes(bvh: torch.Tensor, light_count: int):
        """(boxes, box_shift) giving each light its 32-leaf group box: level 1 of the 32-ary BVH, or
        no boxes at all for at most 32 lights (the reference tests none then)."""
        if light_count <= 32:
            return None, 0
        P = calc_bvh_padded_leaf_count(light_count)
        return bvh[P * 8:], 5

    def __call__(self, stream, sorted_pairs: torch.Tensor, leaf_count: int, boxes: torch.Tensor | None,
                 box_shift: int, nodes: torch.Tensor):
        need = int(lib().vren_lbvh_scratch_bytes(leaf_count))
        if self._scratch is None or self._scratch.numel() * 4 < need:
            self._scratch = alloc_scratch(need, sorted_pairs.device)
        check(lib().vren_build_lbvh(_stream(stream), _ptr(sorted_pairs), leaf_count,
                                    _ptr(boxes) if boxes is not None else None, box_shift, _ptr(nodes),
                                    _ptr(self._scratch)), "build_lbvh")


class assign_lights_lbvh:
    """assign_lights through a Karras tree built over the group boxes (vren_cs_assign_lights_lbvh):
    the same counts, offsets and lists as assign_lights."""

    def __init__(self):
        self._scratch = None

    def __call__(self, stream, cluster_keys: torch.Tensor, key_count: torch.Tensor, frame_dev: torch.Tensor,
                 nodes: torch.Tensor | None, bvh: torch.Tensor, light_count: int, light_index: torch.Tensor,
                 view_positions: torch.Tensor, counts: torch.Tensor, offsets: torch.Tensor, indices: torch.Tensor,
                 total: torch.Tensor, leaf_spheres: torch.Tensor | None = None):
        cap = cluster_keys.numel()
        need = int(lib().vren_cs_assign_lights_scratch_bytes(cap))
        if self._scratch is None or self._scratch.numel() * 4 < need:
            self._scratch = alloc_scratch(need, cluster_keys.device)
        check(lib().vren_cs_assign_lights_lbvh(
            _stream(stream), _ptr(cluster_keys), _ptr(key_count), cap, _ptr(frame_dev),
            _ptr(nodes) if nodes is not None else None, _ptr(bvh) if bvh is not None else None, light_count,
            _ptr(light_index) if light_index is not None else None,
            _ptr(view_positions) if view_positions is not None else None,
            _ptr(leaf_spheres) if leaf_spheres is not None else None,
            _ptr(counts), _ptr(offsets), _ptr(indices) if indices is not None else None,
            indices.numel() if indices is not None else 0, _ptr(total), _ptr(self._scratch)), "assign_lights_lbvh")


class cluster_and_shade:
    """vren::cluster_and_shade (clustered_shading.hpp:147-182): owns an arena sized at creation."""

    def __init__(self, max_width: int, max_height: int, max_lights: int, max_assignments: int,
                 morton_bits: int = 15, use_graph: bool = True, sort_digit_bits: int = 8, assign_warps: int = 8):
        h = C.c_void_p()
        check(lib().vren_cs_create(C.byref(h), max_width, max_height, max_lights, max_assignments), "cs_create")
        self._h = h
        self.set_options(morton_bits, use_graph, sort_digit_bits, assign_warps)

    def set_options(self, morton_bits=15, use_graph=True, sort_digit_bits=8, assign_warps=8, normal_format=0):
        o = Options(morton_bits, 1 if use_graph else 0, sort_digit_bits, assign_warps, normal_format)
        check(lib().vren_cs_set_options(self._h, C.byref(o)), "cs_set_options")
        self._opts = o

    def _follow_normals(self, normals):
        """The normal format follows the normals' dtype (float16: the RGBA16F G-buffer layout)."""
        fmt = normal_format_of(normals)
        if fmt != self._opts.normal_format:
            o = self._opts
            self.set_options(o.morton_bits, bool(o.use_graph), o.sort_digit_bits, o.assign_warps, fmt)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().vren_cs_destroy(h)
            self._h = None

    def cluster(self, stream, view: View, width: int, height: int, depth: torch.Tensor, normals: torch.Tensor,
                positions: torch.Tensor | None, lights: torch.Tensor | None, light_count: int,
                offscreen: str = "wrap"):
        self._follow_normals(normals)
        check(lib().vren_cs_cluster(self._h, _stream(stream), C.byref(view), width, height, OFFSCREEN[offscreen],
                                    _ptr(depth), _ptr(normals), _ptr(positions) if positions is not None else None,
                                    _ptr(lights) if lights is not None else None, light_count), "cs_cluster")

    def cluster_host(self, stream, view: View, width: int, height: int, depth: torch.Tensor, normals: torch.Tensor,
                     positions: torch.Tensor | None, lights: torch.Tensor | None, light_count: int,
                     refs_out: torch.Tensor | None = None, lists_out: torch.Tensor | None = None,
                     offscreen: str = "wrap"):
        """The same frame from page-locked host tensors (uploads overlapped with the light BVH and the
        unique clusters; the references downloaded into refs_out while the light lists are assigned; the
        lists written by the device into lists_out as [U, total, keys, counts, offsets, indices])."""
        self._follow_normals(normals)
        check(lib().vren_cs_cluster_host(self._h, _stream(stream), C.byref(view), width, height, OFFSCREEN[offscreen],
                                         depth.data_ptr(), normals.data_ptr(),
                                         positions.data_ptr() if positions is not None else None,
                                         lights.data_ptr() if lights is not None else None, light_count,
                                         refs_out.data_ptr() if refs_out is not None else None,
                                         lists_out.data_ptr() if lists_out is not None else None,
                                         lists_out.numel() if lists_out is not None else 0), "cs_cluster_host")

    def __call__(self, stream, view: View, width: int, height: int, gbuf: "GBuffer", positions, lights,
                 light_count: int, out: torch.Tensor, directional=None, directional_count: int = 0,
                 falloff: str = "ref", mode: str = "color", offscreen: str = "wrap"):
        """cluster_and_shade::operator() (clustered_shading.cpp:924-1172): the clustering stages, then
        shade over this context's light lists into `out` (f32x3 per pixel), one graph per frame shape."""
        if self._opts.normal_format != 0:
            o = self._opts
            self.set_options(o.morton_bits, bool(o.use_graph), o.sort_digit_bits, o.assign_warps, 0)
        check(lib().vren_cs_cluster_and_shade(self._h, _stream(stream), C.byref(view), width, height,
                                              OFFSCREEN[offscreen], C.byref(gbuf), _addr(positions), _addr(lights),
                                              light_count, _addr(directional), directional_count, FALLOFF[falloff],
                                              SHADE_MODE[mode], _addr(out)), "cs_cluster_and_shade")

    def outputs(self) -> Outputs:
        o = Outputs()
        check(lib().vren_cs_get_outputs(self._h, C.byref(o)), "cs_get_outputs")
        return o


class BatchFrame(C.Structure):
    _fields_ = [("view", View), ("width", C.c_uint32), ("height", C.c_uint32), ("light_count", C.c_uint32),
                ("offscreen", C.c_int32), ("normal_format", C.c_uint32), ("reserved", C.c_uint32),
                ("depth", C.c_void_p), ("normals", C.c_void_p),
                ("light_positions", C.c_void_p), ("point_lights", C.c_void_p)]


class BatchOptions(C.Structure):
    _fields_ = [("sort_digit_bits", C.c_uint32), ("radix_items", C.c_uint32), ("scan_slices", C.c_uint32),
                ("assign_warps", C.c_uint32), ("use_graph", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class cluster_batch:
    """Batched cluster assignment over many frames (one graph per batch shape).  Frames are
    (view, width, height, depth, normals, positions, lights, light_count[, offscreen]) tuples of
    device tensors; each frame's outputs are bit-identical to cluster_and_shade.cluster."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().vren_cs_batch_create(C.byref(h)), "cs_batch_create")
        self._h = h
        self._frames = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().vren_cs_batch_destroy(h)
            self._h = None

    @staticmethod
    def _pack(frames):
        arr = (BatchFrame * len(frames))()
        keep = []
        for i, f in enumerate(frames):
            view, w, h, depth, normals, pos, lights, L = f[:8]
            off = f[8] if len(f) > 8 else "wrap"
            arr[i].view = view
            arr[i].width, arr[i].height, arr[i].light_count = w, h, L
            arr[i].offscreen = OFFSCREEN[off]
            arr[i].normal_format = normal_format_of(normals)
            arr[i].depth, arr[i].normals = _ptr(depth), _ptr(normals)
            arr[i].light_positions = _ptr(pos) if (pos is not None and L) else None
            arr[i].point_lights = _ptr(lights) if (lights is not None and L) else None
            keep.append(f)
        return arr, keep

    def reserve(self, frames, max_assignments: int):
        arr, _ = self._pack(frames)
        check(lib().vren_cs_batch_reserve(self._h, arr, len(frames), max_assignments), "cs_batch_reserve")

    def set_options(self, sort_digit_bits=8, radix_items=0, scan_slices=8, assign_warps=8, use_graph=True):
        o = BatchOptions(sort_digit_bits, radix_items, scan_slices, assign_warps, 1 if use_graph else 0)
        check(lib().vren_cs_batch_set_options(self._h, C.byref(o)), "cs_batch_set_options")

    def options(self) -> dict:
        o = BatchOptions()
        check(lib().vren_cs_batch_get_options(self._h, C.byref(o)), "cs_batch_get_options")
        return o.as_dict()

    def run(self, stream, frames):
        arr, keep = self._pack(frames)
        self._frames = (arr, keep)
        check(lib().vren_cs_batch_run(self._h, _stream(stream), arr, len(frames)), "cs_batch_run")

    def autotune(self, stream, frames, reps: int = 3) -> dict:
        arr, keep = self._pack(frames)
        self._frames = (arr, keep)
        o = BatchOptions()
        check(lib().vren_cs_batch_autotune(self._h, _stream(stream), arr, len(frames), reps, C.byref(o)),
              "cs_batch_autotune")
        return o.as_dict()

    def frame_outputs(self, stream, f: int) -> Outputs:
        o = Outputs()
        check(lib().vren_cs_batch_frame_outputs(self._h, _stream(stream), f, C.byref(o)), "cs_batch_frame_outputs")
        return o


_CUDART = None


def _cudart():
    global _CUDART
    if _CUDART is None:
        import ctypes.util
        import glob
        import os

        cands = [ctypes.util.find_library("cudart"), "libcudart.so"]
        cands += sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
        cands += sorted(glob.glob(os.path.join(os.path.dirname(torch.__file__), "lib", "libcudart*.so*")))
        for c in cands:
            if not c:
                continue
            try:
                _CUDART = C.CDLL(c)
                break
            except OSError:
                continue
        if _CUDART is None:
            raise RuntimeError("libcudart not found")
        _CUDART.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        _CUDART.cudaMemcpy.restype = C.c_int
    return _CUDART


FALLOFF = {"ref": 0, "windowed_inv_sq": 1}
SHADE_MODE = {"color": 0, "radiance": 1}


class GBuffer(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("depth", "normals", "albedo", "roughness", "metallic")]


class LightLists(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("cluster_refs", "counts", "offsets", "indices")] + \
               [("index_capacity", C.c_uint32), ("reserved", C.c_uint32)]


def _addr(x):
    if x is None:
        return None
    return x.data_ptr() if isinstance(x, torch.Tensor) else int(x)


def gbuffer(depth, normals, albedo, roughness, metallic) -> GBuffer:
    return GBuffer(*(_addr(t) for t in (depth, normals, albedo, roughness, metallic)))


def light_lists(cluster_refs, counts, offsets, indices, index_capacity: int | None = None) -> LightLists:
    """index_capacity: the entries `indices` holds (a tensor's size by default; required for an address)."""
    if index_capacity is None:
        if not isinstance(indices, torch.Tensor):
            raise ValueError("light_lists: index_capacity is required when indices is an address")
        index_capacity = indices.numel()
    return LightLists(*(_addr(t) for t in (cluster_refs, counts, offsets, indices)), int(index_capacity), 0)


class shade:
    """vren::clustered_shading::shade (clustered_shading.hpp:114-140)."""

    def __init__(self, falloff: str = "ref", mode: str = "color"):
        self.falloff = FALLOFF[falloff]
        self.mode = SHADE_MODE[mode]

    def __call__(self, stream, frame_dev, width: int, height: int, gbuf: GBuffer, lists: LightLists, positions,
                 lights, light_count: int, out: torch.Tensor, directional=None, directional_count: int = 0):
        check(lib().vren_cs_shade(_stream(stream), _addr(frame_dev), width, height, C.byref(gbuf), C.byref(lists),
                                  _addr(positions), _addr(lights), light_count, _addr(directional), directional_count,
                                  self.falloff, self.mode, _addr(out)), "shade")


class shade_backward:
    """Adjoint of the radiance image with respect to point-light positions, colours and radii."""

    def __init__(self, falloff: str = "windowed_inv_sq"):
        self.falloff = FALLOFF[falloff]
        self._scratch = None

    def __call__(self, stream, frame_dev, width: int, height: int, gbuf: GBuffer, lists: LightLists,
                 assignments: int, positions, lights, light_count: int, grad_radiance, grad_positions, grad_colors,
                 grad_radii):
        need = int(lib().vren_cs_shade_backward_scratch_bytes(light_count, assignments)) + 256
        dev = grad_radiance.device
        if self._scratch is None or self._scratch.numel() * 4 < need:
            self._scratch = alloc_scratch(need, dev)
        sc = (self._scratch.data_ptr() + 255) // 256 * 256
        check(lib().vren_cs_shade_backward(_stream(stream), _addr(frame_dev), width, height, C.byref(gbuf),
                                           C.byref(lists), assignments, _addr(positions), _addr(lights), light_count,
                                           self.falloff, _addr(grad_radiance), _addr(grad_positions),
                                           _addr(grad_colors), _addr(grad_radii), sc), "shade_backward")


def read_device(ptr: int, count: int, dtype=np.uint32) -> np.ndarray:
    """Copies `count` elements at a device address into a numpy array (synchronizes)."""
    out = np.empty(count, dtype=dtype)
    if count == 0:
        return out
    torch.cuda.synchronize()
    res = _cudart().cudaMemcpy(out.ctypes.data, ptr, out.nbytes, 2)  # cudaMemcpyDeviceToHost
    if res != 0:
        raise RuntimeError(f"cudaMemcpy failed: {res}")
    return out
