"""GPU: the batched cluster assignment gives, frame by frame, the same bits as the plain per-frame
path (keys, references, counts, offsets, light lists, sorted light index, view positions, BVH, leaf
spheres), for mixed resolutions, light counts (0 to 40,000), off-screen policies and cameras; the
result does not depend on the tuning options; the autotuner returns valid options and caches them."""
import numpy as np
import pytest
import torch

import vren_gb300.clustered_shading as cs
import vren_gb300.scene as scene

pytestmark = pytest.mark.gpu

FRAMES = [  # (W, H, L, offscreen, moved camera)
    (640, 360, 1000, "wrap", False),
    (256, 192, 0, "wrap", False),
    (1280, 720, 5000, "wrap", True),
    (100, 37, 1, "wrap", False),
    (640, 360, 40000, "wrap", False),
    (320, 180, 3000, "skip", False),
    (96, 64, 20000, "wrap", True),
    (1920, 1080, 16384, "wrap", False),
]


def make_frames(device, specs=FRAMES, seed=100):
    out = []
    for k, (W, H, L, off, moved) in enumerate(specs):
        if moved:
            cam = cs.scene_camera(W, H, position=(3.0, -2.0, 1.5), yaw=0.3, pitch=-0.2)
        else:
            cam = cs.scene_camera(W, H)
        view = cs.view_from_camera(cam, "ref")
        depth, normals = scene.depth_planes(seed + 7 * k, W, H)
        if L:
            pos, lights = scene.lights(seed + 7 * k + 1, L, W, H)
            pos, lights = torch.from_numpy(pos).to(device), torch.from_numpy(lights).to(device)
        else:
            pos = lights = None
        out.append((view, W, H, torch.from_numpy(depth).to(device), torch.from_numpy(normals).to(device), pos, lights,
                    L, off))
    return out


def host_outputs(o, W, H, L, bvh=True):
    U = int(cs.read_device(o.key_count, 1)[0])
    total = int(cs.read_device(o.total, 1)[0])
    r = {
        "U": U,
        "total": total,
        "keys": cs.read_device(o.cluster_keys, U),
        "refs": cs.read_device(o.cluster_refs, W * H),
        "counts": cs.read_device(o.counts, U),
        "offsets": cs.read_device(o.offsets, U),
        "indices": cs.read_device(o.indices, total),
    }
    if L and bvh:
        P = cs.calc_bvh_padded_leaf_count(L)
        r["light_index"] = cs.read_device(o.light_index, 2 * L)
        r["view_pos"] = cs.read_device(o.view_positions, 4 * L)
        r["bvh"] = cs.read_device(o.bvh, 8 * cs.calc_bvh_buffer_length(L))
        r["spheres"] = cs.read_device(o.leaf_spheres, 4 * P)
    return r


def plain_outputs(device, frames):
    res = []
    stream = torch.cuda.Stream(device=device)
    for (view, W, H, depth, normals, pos, lights, L, off) in frames:
        ctx = cs.cluster_and_shade(W, H, max(L, 1), 1 << 22)
        with torch.cuda.stream(stream):
            ctx.cluster(stream, view, W, H, depth, normals, pos, lights, L, off)
        stream.synchronize()
        res.append(host_outputs(ctx.outputs(), W, H, L))
        del ctx
    return res


def batch_outputs(batch, stream, frames):
    return [host_outputs(batch.frame_outputs(stream, f), fr[1], fr[2], fr[7]) for f, fr in enumerate(frames)]


def assert_same(a, b, f):
    assert a.keys() == b.keys(), f
    for k in a:
        if isinstance(a[k], np.ndarray):
            assert np.array_equal(a[k], b[k]), (f, k)
        else:
            assert a[k] == b[k], (f, k)


@pytest.fixture(scope="module")
def frames_and_plain(cuda):
    frames = make_frames(cuda)
    return frames, plain_outputs(cuda, frames)


def test_batch_matches_plain(cuda, frames_and_plain):
    frames, plain = frames_and_plain
    stream = torch.cuda.Stream(device=cuda)
    b = cs.cluster_batch()
    b.reserve(frames, 1 << 24)
    with torch.cuda.stream(stream):
        b.run(stream, frames)
    got = batch_outputs(b, stream, frames)
    assert any(p["total"] > 0 for p in plain)
    for f in range(len(frames)):
        assert_same(got[f], plain[f], f)
    # replay of the captured graph gives the same bits
    with torch.cuda.stream(stream):
        b.run(stream, frames)
    again = batch_outputs(b, stream, frames)
    for f in range(len(frames)):
        assert_same(again[f], plain[f], f)


@pytest.mark.parametrize("opts", [dict(sort_digit_bits=4, radix_items=1, scan_slices=4, assign_warps=2),
                                  dict(sort_digit_bits=6, radix_items=0, scan_slices=8, assign_warps=4),
                                  dict(use_graph=False)])
def test_batch_options_do_not_change_results(cuda, frames_and_plain, opts):
    frames, plain = frames_and_plain
    stream = torch.cuda.Stream(device=cuda)
    b = cs.cluster_batch()
    b.reserve(frames, 1 << 24)
    b.set_options(**opts)
    with torch.cuda.stream(stream):
        b.run(stream, frames)
    got = batch_outputs(b, stream, frames)
    for f in range(len(frames)):
        assert_same(got[f], plain[f], f)


def test_batch_subset_and_reorder(cuda, frames_and_plain):
    """A smaller batch in another order inside the same reservation (graph re-captured)."""
    frames, plain = frames_and_plain
    order = [5, 0, 3]
    sub = [frames[i] for i in order]
    stream = torch.cuda.Stream(device=cuda)
    b = cs.cluster_batch()
    b.reserve(frames, 1 << 24)
    with torch.cuda.stream(stream):
        b.run(stream, frames)
        b.run(stream, sub)
    got = batch_outputs(b, stream, sub)
    for j, i in enumerate(order):
        assert_same(got[j], plain[i], i)


def test_batch_autotune(cuda, frames_and_plain):
    frames, plain = frames_and_plain
    stream = torch.cuda.Stream(device=cuda)
    b = cs.cluster_batch()
    b.reserve(frames, 1 << 24)
    chosen = b.autotune(stream, frames, reps=1)
    assert chosen["sort_digit_bits"] in (4, 6, 8) and chosen["scan_slices"] in (4, 8)
    assert 1 <= chosen["assign_warps"] <= 8 and chosen["radix_items"] in (0, 1)
    assert b.options() == chosen
    # the same shape bucket returns the cached choice
    assert b.autotune(stream, frames, reps=1) == chosen
    with torch.cuda.stream(stream):
        b.run(stream, frames)
    got = batch_outputs(b, stream, frames)
    for f in range(len(frames)):
        assert_same(got[f], plain[f], f)


def test_batch_capacity_and_arguments(cuda, frames_and_plain):
    frames, _ = frames_and_plain
    b = cs.cluster_batch()
    b.reserve(frames[:2], 1 << 20)
    with pytest.raises(Exception):
        b.run(torch.cuda.Stream(device=cuda), frames)  # more than reserved
    bad = list(frames[0])
    bad[1] = 9000  # width above 8192
    with pytest.raises(Exception):
        b.reserve([tuple(bad)], 1 << 20)


def test_batch_frame_groups(cuda):
    """A batch whose references exceed the unique-cluster group size (48 MB): eight 2560x1440 frames
    (118 MB of references) run as several groups and still match the plain path frame by frame."""
    specs = [(2560, 1440, 500 + 700 * k, "wrap", k % 2 == 1) for k in range(8)]
    frames = make_frames(cuda, specs, seed=900)
    plain = plain_outputs(cuda, frames)
    stream = torch.cuda.Stream(device=cuda)
    b = cs.cluster_batch()
    b.reserve(frames, 1 << 24)
    with torch.cuda.stream(stream):
        b.run(stream, frames)
    got = batch_outputs(b, stream, frames)
    for f in range(len(frames)):
        assert_same(got[f], plain[f], f)
