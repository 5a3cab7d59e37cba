"""GPU: show_clusters (every mode, invalid references) and show_clusters_geometry against the CPU
restatement of vren_demo's show_clusters.comp / show_clusters_geometry.comp, bit for bit, on the
clustering context's own outputs."""
import numpy as np
import pytest
import torch

import oracle
import vren_gb300 as vg
import vren_gb300.cluster_debug as cd
import vren_gb300.clustered_shading as cs
import vren_gb300.scene as scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def frame(cuda):
    W, H, L = 640, 360, 4096
    view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
    depth, normals = scene.depth_planes(77, W, H)
    pos, li = scene.lights_near_camera(78, L)
    ctx = cs.cluster_and_shade(W, H, L, 1 << 22)
    ins = [torch.from_numpy(np.ascontiguousarray(x)).to(cuda) for x in (depth, normals, pos, li)]
    torch.cuda.synchronize()
    ctx.cluster(None, view, W, H, *ins, L)
    torch.cuda.synchronize()
    out = ctx.outputs()
    host = cd.read_frame(out, W, H)
    assert host["counts"].max() >= 8, "scene should give clusters with many lights"
    return ctx, out, host, view


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4, 5, 6, -1])
def test_show_clusters_matches_oracle(frame, mode):
    ctx, out, h, _ = frame
    W, H = h["width"], h["height"]
    img = cd.show_clusters()(None, mode, W, H, out)
    torch.cuda.synchronize()
    want = oracle.cs_show_clusters(mode, W, H, h["refs"], h["keys"], h["counts"], h["offsets"], h["indices"])
    assert np.array_equal(img.cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert vg.device_error() == 0


def test_show_clusters_invalid_references_are_magenta(frame, cuda):
    ctx, out, h, _ = frame
    W, H = h["width"], h["height"]
    refs = torch.from_numpy(h["refs"].view(np.int32).copy()).to(cuda)
    refs[::97] = -1
    refs[5] = len(h["keys"])
    o2 = cs.Outputs.from_buffer_copy(out)
    o2.cluster_refs = refs.data_ptr()
    img = cd.show_clusters()(None, "key", W, H, o2).view(-1, 4).cpu().numpy()
    bad = np.zeros(W * H, bool)
    bad[::97] = True
    bad[5] = True
    assert np.array_equal(img[bad], np.tile([1.0, 0.0, 1.0, 1.0], (bad.sum(), 1)).astype(np.float32))
    want = oracle.cs_show_clusters(0, W, H, refs.cpu().numpy().view(np.uint32), h["keys"])
    assert np.array_equal(img.view(np.uint32), want.reshape(-1, 4).view(np.uint32))


def test_show_clusters_geometry_matches_oracle(frame):
    ctx, out, h, view = frame
    v = cd.show_clusters_geometry(None, out)
    torch.cuda.synchronize()
    U = len(h["keys"])
    got = v[:U].cpu().numpy().view(np.uint32)
    want = oracle.cs_show_clusters_geometry(view, h["width"], h["height"], h["keys"])
    assert np.array_equal(got, want)
    assert vg.device_error() == 0


def test_diff_of_gpu_and_oracle_frames_is_empty(frame, tmp_path):
    ctx, out, h, view = frame
    W, H = h["width"], h["height"]
    depth, normals = scene.depth_planes(77, W, H)
    pos, li = scene.lights_near_camera(78, 4096)
    keys, refs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0)
    vp, bvh, lidx = oracle.cs_light_bvh(pos, li, 4096, view, 15)
    c, o, i, _ = oracle.cs_assign_lights(keys, W, H, view, bvh, 4096, lidx, vp)
    ref = {"keys": keys, "refs": refs, "counts": c, "offsets": o, "indices": i, "width": W, "height": H}
    res = cd.diff_frames(h, ref, out_dir=tmp_path)
    assert res["key_mismatch"] == 0 and res["light_mismatch"] == 0
