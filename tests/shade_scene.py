"""Shared synthetic scene for the shading tests: G-buffer, lights on visible surfaces, and the light
lists computed by the CPU oracle pipeline (so the CPU tests need no GPU)."""
import numpy as np

import oracle
import vren_gb300.clustered_shading as cs
import vren_gb300.scene as scene


def make(W: int, H: int, L: int, seed: int = 5):
    view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
    depth, plane_normals = scene.depth_planes(seed, W, H)
    normals, albedo, rough, metal = scene.gbuffer(seed + 1, W, H)
    pos, lights = scene.lights_near_surfaces(seed + 2, L, depth, W, H)
    grad = scene.normal01(seed + 3, 9, W * H * 3)
    keys, refs = oracle.cs_find_unique_clusters(depth, plane_normals, W, H, view, 0)
    vp, bvh, lidx = oracle.cs_light_bvh(pos, lights, L, view, 15)
    counts, offsets, indices, total = oracle.cs_assign_lights(keys, W, H, view, bvh, L, lidx, vp)
    return dict(W=W, H=H, L=L, view=view, depth=depth, plane_normals=plane_normals, normals=normals, albedo=albedo,
                rough=rough, metal=metal, pos=pos, lights=lights, grad=grad, keys=keys, refs=refs, counts=counts,
                offsets=offsets, indices=indices, total=total)


def gb(s):
    return (s["depth"], s["normals"], s["albedo"], s["rough"], s["metal"])


def lists(s):
    return (s["refs"], s["counts"], s["offsets"], s["indices"])


def ndotv(s):
    """Per-pixel N.V in float64 (world position reconstructed from the depth as the oracle does)."""
    v, W, H = s["view"], s["W"], s["H"]
    ip = np.array(v.inv_proj, np.float64)
    iv = np.array(v.inv_view, np.float64)
    ys, xs = np.mgrid[0:H, 0:W]
    v0 = [xs.reshape(-1) / W * 2 - 1, (1 - ys.reshape(-1) / H) * 2 - 1, s["depth"].astype(np.float64),
          np.ones(W * H)]
    vv = [sum(ip[4 * k + r] * v0[k] for k in range(4)) for r in range(4)]
    vv = [x / vv[3] for x in vv]
    p = np.stack([sum(iv[4 * k + r] * vv[k] for k in range(4)) for r in range(3)], 1)
    e = np.array(v.eye, np.float64) - p
    V = e / np.linalg.norm(e, axis=1, keepdims=True)
    return (s["normals"].reshape(-1, 3).astype(np.float64) * V).sum(1)
