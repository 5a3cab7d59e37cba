"""GPU: the Karras binary radix tree (an extension beside the reference's 32-ary BVH) against the
CPU oracle — topology and boxes bit-exact, over each leaf's own box and over its 32-leaf group box —
and light assignment through it, which must give exactly the 32-ary traversal's counts, offsets and
lists (and the oracle's)."""
import numpy as np
import pytest
import torch

import oracle
import vren_gb300 as vg
import vren_gb300.clustered_shading as cs
import vren_gb300.scene as scene

pytestmark = pytest.mark.gpu


def to_dev(a: np.ndarray, device) -> torch.Tensor:
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        return torch.from_numpy(a).to(device)
    return torch.from_numpy(a.astype(np.uint32).view(np.int32)).to(device)


def u32(t: torch.Tensor) -> np.ndarray:
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint32)


def make_view(W, H, moved=False):
    if moved:
        cam = cs.scene_camera(W, H, position=(3.0, -2.0, 1.5), yaw=0.3, pitch=-0.2)
    else:
        cam = cs.scene_camera(W, H)
    return cs.view_from_camera(cam, "ref")


def dense_lights(seed, L):
    """Lights packed near the camera (many lights per cluster)."""
    rng = np.random.default_rng(seed)
    pos = np.zeros((L, 4), np.float32)
    pos[:, 0] = rng.uniform(-8, 8, L)
    pos[:, 1] = rng.uniform(-5, 5, L)
    pos[:, 2] = rng.uniform(0.5, 25, L)
    pos[:, 3] = 1
    li = np.zeros((L, 4), np.float32)
    li[:, 0:3] = rng.uniform(0, 1, (L, 3))
    li[:, 3] = np.exp(np.log(2.0) + 0.5 * rng.standard_normal(L)).astype(np.float32) * 0.5
    return pos.reshape(-1), li.reshape(-1)


def light_bvh(device, pos, li, L, view, W, H, morton_bits=15):
    frame = cs.frame_to_device(cs.frame_build(view, W, H), device)
    P = vg.calc_bvh_padded_leaf_count(L)
    vp = torch.zeros(max(L, 1) * 4, dtype=torch.float32, device=device)
    bvh = torch.zeros(vg.calc_bvh_buffer_length(P) * 8, dtype=torch.int32, device=device)
    lidx = torch.zeros(max(L, 1) * 2, dtype=torch.int32, device=device)
    sph = torch.zeros(P * 4, dtype=torch.float32, device=device)
    cs.construct_point_light_bvh(morton_bits)(None, to_dev(pos, device), to_dev(li, device), L, frame, vp, bvh, lidx,
                                              sph)
    return frame, vp, bvh, lidx, sph


def build_tree(device, lidx, bvh, L, group):
    nodes = torch.zeros(max(L - 1, 1) * 8, dtype=torch.int32, device=device)
    if group:
        boxes, shift = cs.build_lbvh.group_boxes(bvh, L)
    else:
        boxes, shift = bvh, 0
    cs.build_lbvh()(None, lidx, L, boxes, shift, nodes)
    return nodes


@pytest.mark.parametrize("L", [2, 3, 31, 32, 33, 1000, 2049, 16384, 40000])
@pytest.mark.parametrize("morton_bits", [15, 30])
@pytest.mark.parametrize("group", [False, True])
def test_build_lbvh_matches_oracle(cuda, L, morton_bits, group):
    W, H = 1280, 720
    view = make_view(W, H, moved=(L % 2 == 1))
    pos, li = scene.lights(300 + L, L, W, H)
    _, vp, bvh, lidx, _ = light_bvh(cuda, pos, li, L, view, W, H, morton_bits)
    nodes = build_tree(cuda, lidx, bvh, L, group)
    evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, morton_bits)
    boxes = oracle.lbvh_group_boxes(ebvh, L) if group else ebvh[:L]
    expect = oracle.lbvh_build(elidx, boxes, L)
    assert np.array_equal(u32(nodes).reshape(-1, 8)[: L - 1], expect)
    # every leaf hangs below the root exactly once
    seen = np.zeros(L, np.int64)
    stack = [0]
    while stack:
        x = stack.pop()
        if x & 0x80000000:
            seen[x & 0x7FFFFFFF] += 1
        else:
            stack += [int(expect[x, 3]), int(expect[x, 7])]
    assert np.all(seen == 1)


def test_build_lbvh_equal_codes(cuda):
    """All lights at one position but one: equal Morton codes, ordered by leaf position."""
    W, H, L = 640, 360, 3000
    view = make_view(W, H)
    pos = np.tile(np.array([1.0, 2.0, 30.0, 1.0], np.float32), L)
    pos[4 * 7: 4 * 7 + 3] = [5.0, -1.0, 60.0]
    li = np.tile(np.array([0.5, 0.5, 0.5, 2.0], np.float32), L)
    _, vp, bvh, lidx, _ = light_bvh(cuda, pos, li, L, view, W, H)
    nodes = build_tree(cuda, lidx, bvh, L, False)
    evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, 15)
    assert np.array_equal(u32(nodes).reshape(-1, 8)[: L - 1], oracle.lbvh_build(elidx, ebvh[:L], L))


def unique_clusters(device, depth, normals, W, H, view):
    frame = cs.frame_to_device(cs.frame_build(view, W, H), device)
    T = ((W + 31) // 32) * ((H + 31) // 32)
    keys = torch.zeros(T * 1024, dtype=torch.int32, device=device)
    kc = torch.zeros(1, dtype=torch.int32, device=device)
    refs = torch.zeros(W * H, dtype=torch.int32, device=device)
    cs.find_unique_cluster_list()(None, W, H, frame, to_dev(depth, device), to_dev(normals, device), keys, kc, refs)
    return frame, keys, kc


def assign_both(device, W, H, view, depth, normals, pos, li, L, morton_bits=15, spheres=True, index_cap=1 << 22):
    frame, keys, kc = unique_clusters(device, depth, normals, W, H, view)
    _, vp, bvh, lidx, sph = light_bvh(device, pos, li, L, view, W, H, morton_bits)
    cap = keys.numel()
    out = []
    for kind in ("32ary", "lbvh"):
        counts = torch.zeros(cap, dtype=torch.int32, device=device)
        offsets = torch.zeros(cap, dtype=torch.int32, device=device)
        indices = torch.zeros(max(index_cap, 1), dtype=torch.int32, device=device)
        total = torch.zeros(1, dtype=torch.int32, device=device)
        s = sph if spheres else None
        if kind == "32ary":
            cs.assign_lights()(None, keys, kc, frame, bvh, L, lidx, vp, counts, offsets, indices, total, leaf_spheres=s)
        else:
            nodes = build_tree(device, lidx, bvh, L, True) if L > 1 else None
            cs.assign_lights_lbvh()(None, keys, kc, frame, nodes, bvh, L, lidx, vp, counts, offsets, indices, total,
                                    leaf_spheres=s)
        torch.cuda.synchronize()
        out.append((counts, offsets, indices, total))
    return keys, kc, out


@pytest.mark.parametrize("W,H,L,kind,morton_bits", [
    (640, 360, 1, "dense", 15), (640, 360, 20, "dense", 15), (640, 360, 32, "dense", 15),
    (640, 360, 33, "dense", 15), (1280, 720, 5000, "dense", 15), (1280, 720, 5000, "dense", 30),
    (640, 360, 40000, "dense", 15), (1920, 1080, 16384, "scene", 15)])
@pytest.mark.parametrize("spheres", [True, False])
def test_assign_lights_lbvh_equals_32ary(cuda, W, H, L, kind, morton_bits, spheres):
    view = make_view(W, H, moved=(L % 2 == 1))
    depth, normals = scene.depth_planes(W + L, W, H)
    pos, li = dense_lights(L, L) if kind == "dense" else scene.lights(L, L, W, H)
    keys, kc, ((c1, o1, i1, t1), (c2, o2, i2, t2)) = assign_both(cuda, W, H, view, depth, normals, pos, li, L,
                                                                 morton_bits, spheres)
    U = int(u32(kc)[0])
    tot = int(u32(t1)[0])
    assert int(u32(t2)[0]) == tot
    assert np.array_equal(u32(c2)[:U], u32(c1)[:U]) and np.array_equal(u32(o2)[:U], u32(o1)[:U])
    assert np.array_equal(u32(i2)[:tot], u32(i1)[:tot])
    # and the oracle's Karras traversal over the oracle's tree
    evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, morton_bits)
    boxes = oracle.lbvh_group_boxes(ebvh, L)
    enodes = oracle.lbvh_build(elidx, boxes, L)
    ec, eo, ei, et = oracle.cs_assign_lights_lbvh(u32(keys)[:U], W, H, view, enodes, boxes, ebvh, L, elidx, evp)
    assert et == tot and np.array_equal(u32(c2)[:U], ec) and np.array_equal(u32(i2)[:tot], ei)
    assert tot > 0 or L == 1


def test_assign_lights_lbvh_no_lights_and_capacity(cuda):
    W, H = 640, 360
    view = make_view(W, H)
    depth, normals = scene.depth_planes(77, W, H)
    frame, keys, kc = unique_clusters(cuda, depth, normals, W, H, view)
    cap = keys.numel()
    counts = torch.full((cap,), 7, dtype=torch.int32, device=cuda)
    offsets = torch.full((cap,), 7, dtype=torch.int32, device=cuda)
    total = torch.full((1,), 7, dtype=torch.int32, device=cuda)
    cs.assign_lights_lbvh()(None, keys, kc, frame, None, None, 0, None, None, counts, offsets, None, total)
    U = int(u32(kc)[0])
    assert np.all(u32(counts)[:U] == 0) and np.all(u32(offsets)[:U] == 0) and u32(total)[0] == 0
    pos, li = dense_lights(9, 5000)
    _, _, out = assign_both(cuda, W, H, view, depth, normals, pos, li, 5000, index_cap=100)
    assert vg.device_error(clear=True) == vg._lib.VREN_ERR_CAPACITY
    assert int(u32(out[1][3])[0]) > 100
