"""Animated frames (vren_demo's render loop: point_light_bouncer.cpp:17-57 moves the lights, then the
clustered light assignment runs on the moved positions): several frames on the GPU against the same
sequence on the CPU oracle, bit for bit at every frame."""
import numpy as np
import pytest
import torch

import oracle
import vren_gb300.clustered_shading as cs
import vren_gb300.scene as scene

pytestmark = pytest.mark.gpu


def test_bounce_then_cluster_frames(cuda):
    W, H, L, frames = 640, 360, 3000, 6
    view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
    depth, normals = scene.depth_planes(31, W, H)
    pos, lights = scene.lights_near_camera(32, L)
    rng = np.random.default_rng(33)
    dirs = np.zeros((L, 4), np.float32)
    dirs[:, :3] = rng.standard_normal((L, 3))
    lo, hi = [-8.0, -5.0, 0.5], [8.0, 5.0, 25.0]
    ctx = cs.cluster_and_shade(W, H, L, 1 << 22)
    st = torch.cuda.Stream(device=cuda)
    d_depth, d_norm = torch.from_numpy(depth).to(cuda), torch.from_numpy(normals).to(cuda)
    d_pos = torch.from_numpy(pos.copy()).to(cuda)
    d_dir = torch.from_numpy(dirs.reshape(-1).copy()).to(cuda)
    d_light = torch.from_numpy(lights).to(cuda)
    e_pos, e_dir = pos.copy(), dirs.reshape(-1).copy()
    for f in range(frames):
        with torch.cuda.stream(st):
            cs.bounce_point_lights(st, d_pos, d_dir, L, lo, hi, 3.0, 1.0 / 30.0)
            ctx.cluster(st, view, W, H, d_depth, d_norm, d_pos, d_light, L)
        st.synchronize()
        e_pos, e_dir = oracle.bounce_point_lights(e_pos, e_dir, L, lo, hi, 3.0, 1.0 / 30.0)
        assert np.array_equal(d_pos.cpu().numpy().view(np.uint32), e_pos.view(np.uint32)), f"positions, frame {f}"
        o = ctx.outputs()
        U = int(cs.read_device(o.key_count, 1)[0])
        ekeys, erefs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0)
        evp, ebvh, elidx = oracle.cs_light_bvh(e_pos, lights, L, view, 15)
        ec, eo, ei, et = oracle.cs_assign_lights(ekeys, W, H, view, ebvh, L, elidx, evp)
        assert U == len(ekeys) and int(cs.read_device(o.total, 1)[0]) == et, f"frame {f}"
        assert np.array_equal(cs.read_device(o.counts, U), ec), f"counts, frame {f}"
        assert np.array_equal(cs.read_device(o.indices, et), ei), f"lists, frame {f}"
