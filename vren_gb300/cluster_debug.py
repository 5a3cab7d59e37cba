"""Headless cluster debug views (vren_demo/vren_demo/clustered_shading_debug.cpp:6-202).

The reference draws these as Vulkan overlays.  Here the GPU writes the same data into device memory
(``show_clusters``: an RGBA float image; ``show_clusters_geometry``: the debug renderer's line
vertices), and host writers turn them into files: PPM (8-bit) and PFM (float) images, an OBJ line
set, a JSON table of the clusters and their light lists, and a comparison of two frames' outputs
(``diff_frames``) that marks the pixels whose cluster or light list differs, for inspecting parity
failures.  The writers are plain numpy and need no GPU.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import torch

from ._lib import check, lib
from .clustered_shading import Outputs, read_device
from .primitives import _stream, alloc_scratch

MODES = {"key": 0, "ijk": 1, "normal": 2, "light_counts": 3, "light_offsets": 4, "light_indices": 5}
NO_NORMAL = 0x3F


def _mode(mode) -> int:
    return MODES[mode] if isinstance(mode, str) else int(mode)


class show_clusters:
    """vren_demo::show_clusters: the per-pixel colour of each pixel's cluster (show_clusters.comp)."""

    def __init__(self):
        self._scratch = None

    def __call__(self, stream, mode, width: int, height: int, outputs: Outputs, rgba: torch.Tensor | None = None,
                 device=None) -> torch.Tensor:
        if rgba is None:
            rgba = torch.empty((height, width, 4), dtype=torch.float32, device=device or "cuda")
        need = int(lib().vren_cs_show_clusters_scratch_bytes(outputs.key_capacity))
        if self._scratch is None or self._scratch.numel() * 4 < need:
            self._scratch = alloc_scratch(need, rgba.device)
        check(lib().vren_cs_show_clusters(_stream(stream), _mode(mode), width, height, outputs.cluster_refs,
                                          outputs.cluster_keys, outputs.key_count, outputs.key_capacity,
                                          outputs.counts, outputs.offsets, outputs.indices, outputs.index_capacity,
                                          rgba.data_ptr(), self._scratch.data_ptr()), "show_clusters")
        return rgba


def show_clusters_geometry(stream, outputs: Outputs, vertices: torch.Tensor | None = None, device=None,
                           max_clusters: int | None = None) -> torch.Tensor:
    """vren_demo::show_clusters_geometry: (max_clusters, 32, 4) int32 debug vertices (x, y, z float
    bits, colour 0xRRGGBB) of each cluster's view-space box and normal arrow."""
    cap = int(max_clusters if max_clusters is not None else outputs.key_capacity)
    if vertices is None:
        vertices = torch.zeros((cap, 32, 4), dtype=torch.int32, device=device or "cuda")
    check(lib().vren_cs_show_clusters_geometry(_stream(stream), outputs.frame, outputs.cluster_keys,
                                               outputs.key_count, cap, vertices.data_ptr()),
          "show_clusters_geometry")
    return vertices


# ------------------------------------------------------------------------------------------------
# host-side readers and writers (numpy)
# ------------------------------------------------------------------------------------------------
def read_frame(outputs: Outputs, width: int, height: int) -> dict:
    """Copies one frame's cluster outputs to host arrays: keys, refs, counts, offsets, indices."""
    U = int(read_device(outputs.key_count, 1)[0])
    U = min(U, int(outputs.key_capacity))
    counts = read_device(outputs.counts, U)
    offsets = read_device(outputs.offsets, U)
    total = int(read_device(outputs.total, 1)[0]) if outputs.total else int(counts.sum())
    total = min(total, int(outputs.index_capacity))
    return {"keys": read_device(outputs.cluster_keys, U), "refs": read_device(outputs.cluster_refs, width * height),
            "counts": counts, "offsets": offsets, "indices": read_device(outputs.indices, total),
            "width": width, "height": height}


def decode_key(key: int) -> dict:
    """clustered_shading.glsl:45-70: (i, j, k) and the normal bin (face, u, v), or None."""
    key = int(key)
    n = key >> 26
    return {"ijk": [key & 0xFF, (key >> 8) & 0xFF, (key >> 16) & 0x3FF],
            "normal": None if n == NO_NORMAL else [n // 9, (n // 3) % 3, n % 3]}


def write_ppm(path, rgba) -> None:
    """Binary PPM (P6), 8 bits per channel: round(clamp(c, 0, 1) * 255); row 0 at the top."""
    a = np.asarray(rgba.cpu() if isinstance(rgba, torch.Tensor) else rgba, np.float32)
    h, w = a.shape[:2]
    rgb = np.rint(np.clip(np.nan_to_num(a[..., :3], nan=0.0), 0.0, 1.0) * 255.0).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(rgb).tobytes())


def write_pfm(path, rgba) -> None:
    """Portable float map (PF, little-endian, rows stored bottom to top): the exact float colours."""
    a = np.asarray(rgba.cpu() if isinstance(rgba, torch.Tensor) else rgba, np.float32)
    h, w = a.shape[:2]
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
        f.write(np.ascontiguousarray(a[::-1, :, :3], "<f4").tobytes())


def read_pfm(path) -> np.ndarray:
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = (int(x) for x in f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), "<f4" if scale < 0 else ">f4").reshape(h, w, 3)
    return data[::-1].astype(np.float32)


def write_obj(path, vertices, count: int | None = None) -> None:
    """The debug vertices as an OBJ line set: `v x y z r g b` per vertex, `l a b` per pair."""
    v = np.asarray(vertices.cpu() if isinstance(vertices, torch.Tensor) else vertices).view(np.uint32).reshape(-1, 4)
    if count is not None:
        v = v[: count * 32]
    pos = v[:, :3].copy().view(np.float32)
    col = v[:, 3]
    rgb = np.stack([(col >> 16) & 0xFF, (col >> 8) & 0xFF, col & 0xFF], 1) / 255.0
    with open(path, "w") as f:
        f.write("# cluster debug geometry: view-space boxes and normal arrows\n")
        for p, c in zip(pos, rgb):
            f.write(f"v {p[0]:.9g} {p[1]:.9g} {p[2]:.9g} {c[0]:.6g} {c[1]:.6g} {c[2]:.6g}\n")
        for i in range(0, len(pos), 2):
            f.write(f"l {i + 1} {i + 2}\n")


def cluster_table(frame: dict) -> list:
    """One record per cluster: index, key, (i, j, k), normal bin, light count, offset, lights."""
    out = []
    for c, key in enumerate(frame["keys"]):
        n, o = int(frame["counts"][c]), int(frame["offsets"][c])
        rec = {"cluster": c, "key": int(key), **decode_key(key), "light_count": n, "offset": o,
               "lights": [int(x) for x in frame["indices"][o:o + n]]}
        out.append(rec)
    return out


def write_cluster_json(path, frame: dict) -> None:
    with open(path, "w") as f:
        json.dump({"width": frame["width"], "height": frame["height"], "clusters": cluster_table(frame)}, f)


def _pixel_lists(frame: dict):
    """Per pixel: its cluster key, and per cluster its light list (a tuple, in list order)."""
    keys, refs = frame["keys"], frame["refs"]
    valid = refs < len(keys)
    pix_keys = np.where(valid, keys[np.minimum(refs, max(len(keys) - 1, 0))] if len(keys) else 0, 0xFFFFFFFF)
    lists = [tuple(int(x) for x in frame["indices"][o:o + n])
             for n, o in zip(frame["counts"], frame["offsets"])]
    return pix_keys.astype(np.uint32), lists, valid


def diff_frames(a: dict, b: dict, out_dir=None, max_report: int = 64) -> dict:
    """Compares two frames' cluster outputs pixel by pixel (e.g. the GPU's and the CPU oracle's).
    A pixel differs when its cluster key differs, or when its cluster's light list differs (contents
    or order).  Returns
    {"pixels": W*H, "key_mismatch": n, "light_mismatch": n, "clusters": [...first differing...]};
    with out_dir, also writes mismatch.ppm (red: key, yellow: light list, grey: equal) and
    mismatch.json."""
    W, H = a["width"], a["height"]
    ka, la, va = _pixel_lists(a)
    kb, lb, vb = _pixel_lists(b)
    key_bad = (ka != kb) | (va != vb)
    ra, rb = a["refs"], b["refs"]
    light_bad = np.zeros(W * H, bool)
    report, seen = [], set()
    for p in np.flatnonzero(~key_bad & va):
        ca, cb = int(ra[p]), int(rb[p])
        if la[ca] != lb[cb]:
            light_bad[p] = True
            if ca not in seen and len(report) < max_report:
                seen.add(ca)
                report.append({"pixel": [int(p % W), int(p // W)], "key": int(ka[p]), **decode_key(ka[p]),
                               "lights_a": list(la[ca]), "lights_b": list(lb[cb])})
    for p in np.flatnonzero(key_bad)[:max_report]:
        report.append({"pixel": [int(p % W), int(p // W)], "key_a": int(ka[p]), "key_b": int(kb[p])})
    res = {"pixels": W * H, "key_mismatch": int(key_bad.sum()), "light_mismatch": int(light_bad.sum()),
           "clusters": report}
    if out_dir is not None:
        d = Path(out_dir)
        d.mkdir(parents=True, exist_ok=True)
        img = np.full((H * W, 4), 0.25, np.float32)
        img[light_bad] = (1.0, 1.0, 0.0, 1.0)
        img[key_bad] = (1.0, 0.0, 0.0, 1.0)
        write_ppm(d / "mismatch.ppm", img.reshape(H, W, 4))
        with open(d / "mismatch.json", "w") as f:
            json.dump(res, f)
    return res
