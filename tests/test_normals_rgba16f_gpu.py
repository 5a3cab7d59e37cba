"""Normals in the reference's G-buffer format (RGBA16F, vren/vren/pipeline/gbuffer.cpp:7-12): the
unique clusters, the clustering context (device and host inputs) and the batch read half x4 normals and
give exactly the outputs of the f32x3 path (and of the oracle) for the same values, half -> float being
exact."""
import numpy as np
import pytest
import torch

import oracle
import vren_gb300.clustered_shading as cs
import vren_gb300.scene as scene

pytestmark = pytest.mark.gpu


def rgba16f(normals_f32, seed=0, specials=False):
    """(half RGBA per pixel, the same normals as f32x3): w carries noise that must be ignored."""
    n = np.asarray(normals_f32, np.float32).reshape(-1, 3)
    h = np.zeros((len(n), 4), np.float16)
    h[:, :3] = n.astype(np.float16)
    h[:, 3] = np.random.default_rng(seed).uniform(-2, 2, len(n)).astype(np.float16)
    if specials:
        h[::23, 0] = np.float16(np.nan)
        h[1::29, 1] = np.float16(np.inf)
        h[2::31, :3] = np.float16(-0.0)
        h[3::37, 2] = np.float16(6e-8)   # subnormal half
    return h, np.ascontiguousarray(h[:, :3].astype(np.float32)).reshape(-1)


def u32(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("W,H", [(1920, 1080), (100, 37), (640, 360)])
@pytest.mark.parametrize("offscreen", ["wrap", "skip"])
def test_find_unique_clusters_rgba16f(cuda, W, H, offscreen):
    view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
    depth, normals = scene.depth_planes(W + H, W, H)
    half, f32 = rgba16f(normals, W, specials=True)
    frame = cs.frame_to_device(cs.frame_build(view, W, H, offscreen, cs.NORMALS["rgba16f"]), cuda)
    T = ((W + 31) // 32) * ((H + 31) // 32)
    keys = torch.zeros(T * 1024, dtype=torch.int32, device=cuda)
    kc = torch.zeros(1, dtype=torch.int32, device=cuda)
    refs = torch.zeros(W * H, dtype=torch.int32, device=cuda)
    cs.find_unique_cluster_list()(None, W, H, frame, torch.from_numpy(depth).to(cuda),
                                  torch.from_numpy(half).to(cuda), keys, kc, refs)
    ekeys, erefs = oracle.cs_find_unique_clusters(depth, f32, W, H, view, 0 if offscreen == "wrap" else 1)
    U = int(u32(kc)[0])
    assert U == len(ekeys) and np.array_equal(u32(keys)[:U], ekeys)
    assert np.array_equal(u32(refs), erefs)


def test_find_unique_clusters_rgba16f_unaligned(cuda):
    """Normals buffer only 8-byte aligned: the scalar load path."""
    W, H = 256, 96
    view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
    depth, normals = scene.depth_planes(5, W, H)
    half, f32 = rgba16f(normals, 5)
    buf = torch.zeros((W * H + 1, 4), dtype=torch.float16, device=cuda)
    buf[1:] = torch.from_numpy(half).to(cuda)
    frame = cs.frame_to_device(cs.frame_build(view, W, H, "wrap", cs.NORMALS["rgba16f"]), cuda)
    T = ((W + 31) // 32) * ((H + 31) // 32)
    keys = torch.zeros(T * 1024, dtype=torch.int32, device=cuda)
    kc = torch.zeros(1, dtype=torch.int32, device=cuda)
    refs = torch.zeros(W * H, dtype=torch.int32, device=cuda)
    cs.find_unique_cluster_list()(None, W, H, frame, torch.from_numpy(depth).to(cuda), buf[1:], keys, kc, refs)
    ekeys, erefs = oracle.cs_find_unique_clusters(depth, f32, W, H, view, 0)
    U = int(u32(kc)[0])
    assert U == len(ekeys) and np.array_equal(u32(keys)[:U], ekeys) and np.array_equal(u32(refs), erefs)


@pytest.mark.parametrize("use_graph", [True, False])
def test_context_device_and_host_inputs_rgba16f(cuda, use_graph):
    """The context follows the normals' dtype: the same frame with f32x3 and with RGBA16F normals (same
    values) gives identical outputs, from device and from page-locked host buffers."""
    W, H, L = 1280, 720, 4000
    view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
    depth, normals = scene.depth_planes(9, W, H)
    half, f32 = rgba16f(normals, 9)
    pos, li = scene.lights_near_camera(10, L)
    ctx = cs.cluster_and_shade(W, H, L, 1 << 22, use_graph=use_graph)
    st = torch.cuda.Stream(device=cuda)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    results = []
    for n in (dev(f32), dev(half), dev(f32)):
        with torch.cuda.stream(st):
            ctx.cluster(st, view, W, H, dev(depth), n, dev(pos), dev(li), L)
        st.synchronize()
        o = ctx.outputs()
        U = int(cs.read_device(o.key_count, 1)[0])
        tot = int(cs.read_device(o.total, 1)[0])
        results.append((cs.read_device(o.cluster_keys, U), cs.read_device(o.cluster_refs, W * H),
                        cs.read_device(o.counts, U), cs.read_device(o.indices, tot)))
    hp = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    h_refs = torch.zeros(W * H, dtype=torch.int32).pin_memory()
    h_lists = torch.zeros(1 << 22, dtype=torch.int32).pin_memory()
    for _ in range(2):
        with torch.cuda.stream(st):
            ctx.cluster_host(st, view, W, H, hp(depth), hp(half), hp(pos), hp(li), L, h_refs, h_lists)
        st.synchronize()
        assert np.array_equal(h_refs.numpy().view(np.uint32), results[0][1])
        U = int(h_lists[0])
        assert U == len(results[0][0]) and np.array_equal(h_lists[2:2 + U].numpy().view(np.uint32), results[0][0])
    ekeys, erefs = oracle.cs_find_unique_clusters(depth, f32, W, H, view, 0)
    for r in results:
        assert np.array_equal(r[0], ekeys) and np.array_equal(r[1], erefs)
        assert all(np.array_equal(a, b) for a, b in zip(r, results[0]))


def test_batch_mixed_normal_formats(cuda):
    """A batch whose frames alternate f32x3 and RGBA16F normals equals the per-frame context results."""
    frames, want = [], []
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    for k, (W, H, L) in enumerate([(640, 360, 500), (1280, 720, 3000), (320, 200, 40), (1920, 1080, 8000)]):
        view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
        depth, normals = scene.depth_planes(70 + k, W, H)
        half, f32 = rgba16f(normals, 70 + k)
        pos, li = scene.lights_near_camera(80 + k, L)
        n = dev(half) if k % 2 else dev(f32)
        frames.append((view, W, H, dev(depth), n, dev(pos), dev(li), L))
        ctx = cs.cluster_and_shade(W, H, L, 1 << 22)
        ctx.cluster(None, view, W, H, dev(depth), dev(f32), dev(pos), dev(li), L)
        torch.cuda.synchronize()
        o = ctx.outputs()
        U = int(cs.read_device(o.key_count, 1)[0])
        tot = int(cs.read_device(o.total, 1)[0])
        want.append((cs.read_device(o.cluster_keys, U), cs.read_device(o.cluster_refs, W * H),
                     cs.read_device(o.counts, U), cs.read_device(o.offsets, U), cs.read_device(o.indices, tot)))
    b = cs.cluster_batch()
    b.reserve(frames, 1 << 23)
    b.run(None, frames)
    torch.cuda.synchronize()
    for i, (f, w) in enumerate(zip(frames, want)):
        o = b.frame_outputs(None, i)
        U = int(cs.read_device(o.key_count, 1)[0])
        tot = int(cs.read_device(o.total, 1)[0])
        got = (cs.read_device(o.cluster_keys, U), cs.read_device(o.cluster_refs, f[1] * f[2]),
               cs.read_device(o.counts, U), cs.read_device(o.offsets, U), cs.read_device(o.indices, tot))
        assert all(np.array_equal(a, c) for a, c in zip(got, w)), f"frame {i}"
