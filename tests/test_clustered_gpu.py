"""Clustered light assignment: GPU stages and the cluster_and_shade context against the CPU oracle,
bit-exact (keys, references, BVH, light index, counts, offsets, index lists)."""
import ctypes as C

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


def make_view(W, H, slicing="ref", moved=False):
    if moved:
        cam = cs.scene_camera(W, H, position=(3.0, -2.0, 1.5), yaw=0.3, pitch=-0.2)
    else:
        cam = cs.scene_camera(W, H)
    return cs.view_from_camera(cam, slicing)


def dense_lights(seed, L):
    """Lights packed near the camera so that clusters receive many lights (deep traversals)."""
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


# ------------------------------------------------------------------------------------------------
def run_light_bvh(device, pos, li, L, view, W, H, morton_bits=15):
    frame = cs.frame_to_device(cs.frame_build(view, W, H), device)
    P = vg.calc_bvh_padded_leaf_count(L)
    vp = torch.zeros(max(L, 1) * 4, dtype=torch.float32, device=device)
    bvh = torch.zeros(vg.calc_bvh_buffer_length(P) * 8, dtype=torch.int32, device=device)
    lidx = torch.zeros(max(L, 1) * 2, dtype=torch.int32, device=device)
    sph = torch.zeros(P * 4, dtype=torch.float32, device=device)
    cs.construct_point_light_bvh(morton_bits)(None, to_dev(pos, device), to_dev(li, device), L, frame, vp, bvh, lidx, sph)
    torch.cuda.synchronize()
    return frame, vp, bvh, lidx, sph


@pytest.mark.parametrize("L", [1, 5, 31, 32, 33, 1000, 1024, 1025, 2048, 2049, 16384, 40000])
@pytest.mark.parametrize("morton_bits", [15, 30])
def test_construct_light_bvh(cuda, L, morton_bits):
    W, H = 1920, 1080
    view = make_view(W, H, moved=(L % 2 == 1))
    pos, li = scene.lights(1000 + L, L, W, H)
    _, vp, bvh, lidx, sph = run_light_bvh(cuda, pos, li, L, view, W, H, morton_bits)
    evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, morton_bits)
    assert np.array_equal(vp.cpu().numpy().view(np.uint32)[: 4 * L], evp.view(np.uint32))
    assert np.array_equal(u32(lidx)[: 2 * L], elidx)
    assert np.array_equal(u32(bvh).reshape(-1, 8), ebvh)
    # leaf spheres: view position of the leaf's light and (max.x - min.x) / 2
    s = sph.cpu().numpy().reshape(-1, 4)
    fb = ebvh.view(np.float32)
    order = elidx.reshape(-1, 2)[:, 1]
    assert np.array_equal(s[:L, 0:3], evp.reshape(-1, 4)[order, 0:3])
    assert np.array_equal(s[:L, 3], ((fb[:L, 4] - fb[:L, 0]) / np.float32(2)).astype(np.float32))
    assert np.all(s[L:, 3] == -1)


@pytest.mark.parametrize("L", [2049, 5000, 16384, 32767, 32768])
@pytest.mark.parametrize("cluster", [1, 0])
@pytest.mark.parametrize("duplicates", [False, True])
def test_light_bvh_cluster_and_multi_kernel_paths(cuda, L, cluster, duplicates):
    """2049..32768 lights: the one-kernel 16-CTA cluster path and the multi-kernel path both give the
    oracle's BVH, light index, view positions and leaf spheres (equal Morton codes included)."""
    lib = vg.lib()
    knob = vg._lib.TUNE["light_bvh_cluster"]
    assert lib.vren_tuning_set(knob, cluster) == 0
    try:
        W, H = 1280, 720
        view = make_view(W, H, moved=(L % 2 == 1))
        if duplicates:
            pos = np.tile(np.array([1.0, 2.0, 30.0, 1.0], np.float32), L)
            pos[4 * 7: 4 * 7 + 3] = [5.0, -1.0, 60.0]
            li = np.tile(np.array([0.5, 0.5, 0.5, 2.0], np.float32), L)
        else:
            pos, li = scene.lights(77 + L, L, W, H)
        _, vp, bvh, lidx, sph = run_light_bvh(cuda, pos, li, L, view, W, H)
        assert vg.device_error() == 0
        evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, 15)
        assert np.array_equal(vp.cpu().numpy().view(np.uint32)[: 4 * L], evp.view(np.uint32))
        assert np.array_equal(u32(lidx)[: 2 * L], elidx)
        assert np.array_equal(u32(bvh).reshape(-1, 8), ebvh)
        s = sph.cpu().numpy().reshape(-1, 4)
        order = elidx.reshape(-1, 2)[:, 1]
        assert np.array_equal(s[:L, 0:3], evp.reshape(-1, 4)[order, 0:3])
        assert np.all(s[L:, 3] == -1)
    finally:
        lib.vren_tuning_set(knob, 1)


@pytest.mark.parametrize("L", [2000, 3000])
def test_construct_light_bvh_duplicate_positions(cuda, L):
    """Equal Morton codes (and a zero extent) exercise the stable tie order and the NaN path, in the
    one-CTA path (2000 lights) and the multi-CTA one (3000)."""
    W, H = 640, 360
    view = make_view(W, H)
    pos = np.tile(np.array([1.0, 2.0, 30.0, 1.0], np.float32), L)
    pos[4 * 7: 4 * 7 + 3] = [5.0, -1.0, 60.0]
    li = np.tile(np.array([0.5, 0.5, 0.5, 2.0], np.float32), L)
    _, vp, bvh, lidx, sph = run_light_bvh(cuda, pos, li, L, view, W, H)
    evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, 15)
    assert np.array_equal(u32(lidx)[: 2 * L], elidx)
    assert np.array_equal(u32(bvh).reshape(-1, 8), ebvh)


# ------------------------------------------------------------------------------------------------
def run_unique(device, depth, normals, W, H, view, offscreen="wrap", key_cap=None):
    frame = cs.frame_to_device(cs.frame_build(view, W, H, offscreen), device)
    T = ((W + 31) // 32) * ((H + 31) // 32)
    cap = T * 1024 if key_cap is None else key_cap
    keys = torch.zeros(max(cap, 1), dtype=torch.int32, device=device)
    kc = torch.zeros(1, dtype=torch.int32, device=device)
    refs = torch.zeros(W * H, dtype=torch.int32, device=device)
    cs.find_unique_cluster_list()(None, W, H, frame, to_dev(depth, device), to_dev(normals, device), keys, kc, refs)
    return frame, keys, kc, refs


@pytest.mark.parametrize("W,H", [(64, 64), (100, 37), (640, 360), (1280, 720), (1920, 1080), (2560, 1440)])
@pytest.mark.parametrize("offscreen", ["wrap", "skip"])
@pytest.mark.parametrize("slicing", ["ref", "fixed32"])
def test_find_unique_clusters(cuda, W, H, offscreen, slicing):
    view = make_view(W, H, slicing)
    depth, normals = scene.depth_planes(W * 7 + H, W, H)
    _, keys, kc, refs = run_unique(cuda, depth, normals, W, H, view, offscreen)
    ekeys, erefs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0 if offscreen == "wrap" else 1)
    U = int(u32(kc)[0])
    assert U == len(ekeys)
    assert np.array_equal(u32(keys)[:U], ekeys)
    assert np.array_equal(u32(refs), erefs)


def test_find_unique_clusters_special_normals(cuda):
    """Null normals (0x3F bin), axis-aligned and 45-degree normals, NaN depth and depth outside [0, 1]."""
    W, H = 96, 64
    view = make_view(W, H)
    rng = np.random.default_rng(3)
    depth = rng.uniform(0.0, 1.0, W * H).astype(np.float32)
    depth[::17] = np.nan
    depth[::29] = -0.5
    depth[::31] = 1.5
    normals = rng.standard_normal((W * H, 3)).astype(np.float32)
    normals[::5] = 0.0
    normals[1::7] = [0.0, -0.0, 1.0]
    normals[2::11] = [0.70710677, 0.70710677, 0.0]
    normals[3::13] = [-1.0, 1.0, -1.0]
    normals = normals.reshape(-1)
    _, keys, kc, refs = run_unique(cuda, depth, normals, W, H, view)
    ekeys, erefs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0)
    U = int(u32(kc)[0])
    assert U == len(ekeys) and np.array_equal(u32(keys)[:U], ekeys)
    assert np.array_equal(u32(refs), erefs)


def test_find_unique_clusters_many_tiles(cuda):
    """More than 16,384 tiles (the tile-count scan runs in several chunks)."""
    W, H = 4160, 4144  # 130 x 130 tiles
    view = make_view(W, H)
    depth, normals = scene.depth_planes(99, W, H)
    _, keys, kc, refs = run_unique(cuda, depth, normals, W, H, view)
    ekeys, erefs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0)
    U = int(u32(kc)[0])
    assert U == len(ekeys) and np.array_equal(u32(keys)[:U], ekeys)
    assert np.array_equal(u32(refs), erefs)


@pytest.mark.parametrize("slicing", ["ref", "fixed32"])
def test_find_unique_clusters_adversarial(cuda, slicing):
    """Depths at and one or two ulps either side of every slice boundary (the slice estimate must be
    corrected against the table), and normals whose largest components are equal, a few ulps apart,
    infinite, NaN, signed zero, subnormal or huge."""
    W, H = 256, 192
    view = make_view(W, H, slicing)
    fr = cs.frame_build(view, W, H)
    n, f = float(view.near_plane), float(view.far_plane)
    bounds = np.array(fr.slice_near[: fr.max_slice + 1], dtype=np.float64)
    bounds = bounds[np.isfinite(bounds) & (bounds < f)]
    d_at = (f / (f - n) * (1.0 - n / bounds)).astype(np.float32)
    cand = [d_at]
    for s in (1, 2):
        cand.append(np.nextafter(d_at, np.float32(2), dtype=np.float32) if s == 1 else
                    np.nextafter(np.nextafter(d_at, np.float32(2)), np.float32(2)))
        cand.append(np.nextafter(d_at, np.float32(-2)) if s == 1 else
                    np.nextafter(np.nextafter(d_at, np.float32(-2)), np.float32(-2)))
    cand = np.concatenate(cand + [np.array([0.0, 1.0, np.inf, -np.inf], np.float32)]).astype(np.float32)
    rng = np.random.default_rng(11)
    depth = cand[rng.integers(0, len(cand), W * H)].astype(np.float32)

    m = rng.uniform(0.2, 1.0, W * H).astype(np.float32)
    k = rng.integers(0, 4, W * H).astype(np.int32)
    near_m = m.view(np.int32) - k  # 0..3 ulps below m
    normals = np.zeros((W * H, 3), np.float32)
    perm = rng.permuted(np.tile([0, 1, 2], (W * H, 1)), axis=1)
    rows = np.arange(W * H)
    normals[rows, perm[:, 0]] = m * np.where(rng.random(W * H) < 0.5, -1, 1)
    normals[rows, perm[:, 1]] = near_m.view(np.float32) * np.where(rng.random(W * H) < 0.5, -1, 1)
    normals[rows, perm[:, 2]] = rng.uniform(-1, 1, W * H).astype(np.float32) * m
    special = np.array([[np.inf, 1, 0], [1, -np.inf, np.inf], [np.nan, 0.5, 0.5], [np.nan, np.nan, 0.0],
                        [-0.0, 0.0, 0.0], [0.0, -0.0, np.nan], [1e-38, 2e-38, -1e-45], [1e-36, 0, 0],
                        [3e38, -3e38, 1], [2e38, 1e38, 0], [0.5, 0.5, 0.5], [-0.5, 0.5, -0.5]], np.float32)
    normals[::3] = special[rng.integers(0, len(special), len(normals[::3]))]
    normals = normals.reshape(-1)
    _, keys, kc, refs = run_unique(cuda, depth, normals, W, H, view)
    ekeys, erefs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0)
    U = int(u32(kc)[0])
    assert U == len(ekeys) and np.array_equal(u32(keys)[:U], ekeys)
    assert np.array_equal(u32(refs), erefs)


def test_find_unique_clusters_repeated_calls(cuda):
    """The look-back scratch is reused across calls (epoch-tagged status words)."""
    W, H = 640, 360
    view = make_view(W, H)
    finder = cs.find_unique_cluster_list()
    frame = cs.frame_to_device(cs.frame_build(view, W, H), cuda)
    T = ((W + 31) // 32) * ((H + 31) // 32)
    for seed in range(4):
        depth, normals = scene.depth_planes(seed, W, H)
        keys = torch.zeros(T * 1024, dtype=torch.int32, device=cuda)
        kc = torch.zeros(1, dtype=torch.int32, device=cuda)
        refs = torch.zeros(W * H, dtype=torch.int32, device=cuda)
        finder(None, W, H, frame, to_dev(depth, cuda), to_dev(normals, cuda), keys, kc, refs)
        ekeys, erefs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0)
        U = int(u32(kc)[0])
        assert np.array_equal(u32(keys)[:U], ekeys) and np.array_equal(u32(refs), erefs)


def test_find_unique_clusters_capacity(cuda):
    W, H = 640, 360
    view = make_view(W, H)
    depth, normals = scene.depth_planes(5, W, H)
    ekeys, _ = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0)
    cap = len(ekeys) // 2
    _, keys, kc, refs = run_unique(cuda, depth, normals, W, H, view, key_cap=cap)
    torch.cuda.synchronize()
    assert vg.device_error(clear=True) == vg._lib.VREN_ERR_CAPACITY
    assert int(u32(kc)[0]) == cap
    assert np.array_equal(u32(keys)[:cap], ekeys[:cap])


# ------------------------------------------------------------------------------------------------
def run_assign(device, W, H, view, depth, normals, pos, li, L, spheres=True, index_cap=1 << 22):
    frame, keys, kc, refs = run_unique(device, depth, normals, W, H, view)
    _, vp, bvh, lidx, sph = run_light_bvh(device, pos, li, L, view, W, H)
    cap = keys.numel()
    counts = torch.zeros(cap, dtype=torch.int32, device=device)
    offsets = torch.zeros(cap, dtype=torch.int32, device=device)
    indices = torch.zeros(max(index_cap, 1), dtype=torch.int32, device=device)
    total = torch.zeros(1, dtype=torch.int32, device=device)
    cs.assign_lights()(None, keys, kc, frame, bvh, L, lidx, vp, counts, offsets, indices, total,
                       leaf_spheres=sph if spheres else None)
    torch.cuda.synchronize()
    return keys, kc, vp, bvh, lidx, counts, offsets, indices, total


@pytest.mark.parametrize("L", [1, 20, 32, 500, 1024, 5000, 16384, 40000])
@pytest.mark.parametrize("spheres", [True, False])
def test_assign_lights_dense(cuda, L, spheres):
    W, H = 640, 360
    view = make_view(W, H)
    depth, normals = scene.depth_planes(77, W, H)
    pos, li = dense_lights(L, L)
    keys, kc, vp, bvh, lidx, counts, offsets, indices, total = run_assign(cuda, W, H, view, depth, normals, pos, li, L,
                                                                          spheres)
    U = int(u32(kc)[0])
    evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, 15)
    ec, eo, ei, et = oracle.cs_assign_lights(u32(keys)[:U], W, H, view, ebvh, L, elidx, evp)
    assert int(u32(total)[0]) == et
    assert np.array_equal(u32(counts)[:U], ec)
    assert np.array_equal(u32(offsets)[:U], eo)
    assert np.array_equal(u32(indices)[:et], ei)
    assert et > 0 or L == 1


@pytest.mark.parametrize("fused", [0, 1, 2])
@pytest.mark.parametrize("L,seed", [(20, 20), (5000, 5000), (40000, 40000)])
def test_assign_lights_fused_and_three_kernel_forms(cuda, fused, L, seed):
    """Count/scan/write, one kernel (cluster counts resolved by look-back), and the count kernel that
    writes the offsets followed by the write kernel give the oracle's counts, offsets and lists; three
    calls in a row reuse the scratch (epoch-tagged status words)."""
    lib = vg.lib()
    knob = vg._lib.TUNE["assign_fused"]
    assert lib.vren_tuning_set(knob, fused) == 0
    try:
        W, H = 640, 360
        view = make_view(W, H)
        depth, normals = scene.depth_planes(77, W, H)
        pos, li = dense_lights(seed, L)
        evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, 15)
        frame, keys, kc, refs = run_unique(cuda, depth, normals, W, H, view)
        _, vp, bvh, lidx, sph = run_light_bvh(cuda, pos, li, L, view, W, H)
        U = int(u32(kc)[0])
        ec, eo, ei, et = oracle.cs_assign_lights(u32(keys)[:U], W, H, view, ebvh, L, elidx, evp)
        assert et > 0
        stage = cs.assign_lights()  # one scratch for all calls
        cap = keys.numel()
        for spheres in (True, False, True):
            counts = torch.zeros(cap, dtype=torch.int32, device=cuda)
            offsets = torch.zeros(cap, dtype=torch.int32, device=cuda)
            indices = torch.zeros(1 << 22, dtype=torch.int32, device=cuda)
            total = torch.zeros(1, dtype=torch.int32, device=cuda)
            stage(None, keys, kc, frame, bvh, L, lidx, vp, counts, offsets, indices, total,
                  leaf_spheres=sph if spheres else None)
            assert int(u32(total)[0]) == et
            assert np.array_equal(u32(counts)[:U], ec) and np.array_equal(u32(offsets)[:U], eo)
            assert np.array_equal(u32(indices)[:et], ei)
        assert vg.device_error() == 0
    finally:
        lib.vren_tuning_set(knob, 0)


@pytest.mark.parametrize("W,H,L,slicing", [(1920, 1080, 16384, "ref"), (1920, 1080, 16384, "fixed32"),
                                           (1280, 720, 65536, "ref"), (640, 360, 1024, "ref")])
def test_assign_lights_baseline_scene(cuda, W, H, L, slicing):
    """The benchmark scenes (seeded planes, lights uniform in the frustum box), including the 1080p /
    16,384-light frame with 32 exponential depth slices (FIXED32) as well as the reference's slicing."""
    view = make_view(W, H, slicing)
    depth, normals = scene.depth_planes(W + L, W, H)
    pos, li = scene.lights(L, L, W, H)
    keys, kc, vp, bvh, lidx, counts, offsets, indices, total = run_assign(cuda, W, H, view, depth, normals, pos, li, L)
    U = int(u32(kc)[0])
    evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, 15)
    ec, eo, ei, et = oracle.cs_assign_lights(u32(keys)[:U], W, H, view, ebvh, L, elidx, evp)
    assert int(u32(total)[0]) == et
    assert np.array_equal(u32(counts)[:U], ec) and np.array_equal(u32(offsets)[:U], eo)
    assert np.array_equal(u32(indices)[:et], ei)


def test_assign_lights_no_lights(cuda):
    W, H = 320, 200
    view = make_view(W, H)
    depth, normals = scene.depth_planes(1, W, H)
    frame, keys, kc, refs = run_unique(cuda, depth, normals, W, H, view)
    cap = keys.numel()
    counts = torch.full((cap,), 7, dtype=torch.int32, device=cuda)
    offsets = torch.full((cap,), 7, dtype=torch.int32, device=cuda)
    total = torch.full((1,), 7, dtype=torch.int32, device=cuda)
    cs.assign_lights()(None, keys, kc, frame, None, 0, None, None, counts, offsets, None, total)
    U = int(u32(kc)[0])
    assert np.all(u32(counts)[:U] == 0) and np.all(u32(offsets)[:U] == 0) and u32(total)[0] == 0


def test_assign_lights_index_capacity(cuda):
    W, H = 640, 360
    view = make_view(W, H)
    depth, normals = scene.depth_planes(77, W, H)
    pos, li = dense_lights(9, 5000)
    res = run_assign(cuda, W, H, view, depth, normals, pos, li, 5000, index_cap=100)
    assert vg.device_error(clear=True) == vg._lib.VREN_ERR_CAPACITY
    assert int(u32(res[-1])[0]) > 100


# ------------------------------------------------------------------------------------------------
def check_context_outputs(ctx, W, H, view, depth, normals, pos, li, L):
    o = ctx.outputs()
    U = int(cs.read_device(o.key_count, 1)[0])
    keys = cs.read_device(o.cluster_keys, U)
    refs = cs.read_device(o.cluster_refs, W * H)
    ekeys, erefs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0)
    assert np.array_equal(keys, ekeys) and np.array_equal(refs, erefs)
    evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, 15)
    ec, eo, ei, et = oracle.cs_assign_lights(ekeys, W, H, view, ebvh, L, elidx, evp)
    assert int(cs.read_device(o.total, 1)[0]) == et
    assert np.array_equal(cs.read_device(o.counts, U), ec)
    assert np.array_equal(cs.read_device(o.offsets, U), eo)
    assert np.array_equal(cs.read_device(o.indices, et), ei)


@pytest.mark.parametrize("fuc_form", [0, 1, 2])  # unique clusters: self-offset fix-up / scan + fix-up / one kernel
@pytest.mark.parametrize("slicing", ["ref", "fixed32"])
def test_cluster_and_shade_context_1080p(cuda, slicing, fuc_form):
    """The benchmark frame through the context (graph replay): 1920x1080, 16,384 lights, both slicings,
    both forms of the unique-cluster stage; a dense frame follows on the same context."""
    lib = vg.lib()
    knob = vg._lib.TUNE["fuc_fused"]
    assert lib.vren_tuning_set(knob, fuc_form) == 0
    try:
        W, H, L = 1920, 1080, 16384
        view = make_view(W, H, slicing)
        depth, normals = scene.depth_planes(W + L, W, H)
        pos, li = scene.lights(L, L, W, H)
        ctx = cs.cluster_and_shade(W, H, L, 1 << 22)
        stream = torch.cuda.Stream()
        bufs = [to_dev(x, cuda) for x in (depth, normals, pos, li)]
        torch.cuda.synchronize()
        for _ in range(2):
            with torch.cuda.stream(stream):
                ctx.cluster(stream, view, W, H, *bufs, L)
            stream.synchronize()
            check_context_outputs(ctx, W, H, view, depth, normals, pos, li, L)
        dpos, dli = dense_lights(5, L)
        dbufs = bufs[:2] + [to_dev(x, cuda) for x in (dpos, dli)]
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ctx.cluster(stream, view, W, H, *dbufs, L)
        stream.synchronize()
        check_context_outputs(ctx, W, H, view, depth, normals, dpos, dli, L)
    finally:
        lib.vren_tuning_set(knob, 0)


@pytest.mark.parametrize("radius_scale", [1.0, 2.0])
def test_cluster_and_shade_context_long_lists(cuda, radius_scale):
    """Lists around and far above the 128 lights that the count pass keeps for the write pass to copy
    (1.0: up to 142 lights, most clusters between 65 and 128; 2.0: up to 670): the copied and the
    re-traversed lists equal the oracle's."""
    W, H, L = 640, 360, 20000
    view = make_view(W, H)
    depth, normals = scene.depth_planes(77, W, H)
    pos, li = dense_lights(78, L)
    li = li.reshape(-1, 4).copy()
    li[:, 3] *= np.float32(radius_scale)
    li = li.reshape(-1)
    ctx = cs.cluster_and_shade(W, H, L, 1 << 22)
    stream = torch.cuda.Stream()
    bufs = [to_dev(x, cuda) for x in (depth, normals, pos, li)]
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        ctx.cluster(stream, view, W, H, *bufs, L)
    stream.synchronize()
    check_context_outputs(ctx, W, H, view, depth, normals, pos, li, L)
    o = ctx.outputs()
    counts = cs.read_device(o.counts, int(cs.read_device(o.key_count, 1)[0]))
    assert counts.max() > 128 and ((counts > 64) & (counts <= 128)).any()


@pytest.mark.parametrize("use_graph", [False, True])
def test_cluster_and_shade_context(cuda, use_graph):
    W, H, L = 1280, 720, 5000
    ctx = cs.cluster_and_shade(1920, 1080, 65536, 1 << 22, use_graph=use_graph)
    stream = torch.cuda.Stream()
    for seed in (1, 2):  # a second frame with new inputs (same buffers) replays the graph
        view = make_view(W, H, moved=(seed == 2))
        depth, normals = scene.depth_planes(seed, W, H)
        pos, li = dense_lights(seed, L)
        d, n, p, l = (to_dev(x, cuda) for x in (depth, normals, pos, li))
        if seed == 1:
            bufs = (d, n, p, l)
        else:
            for dst, src in zip(bufs, (d, n, p, l)):
                dst.copy_(src)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ctx.cluster(stream, view, W, H, *bufs, L)
        stream.synchronize()
        check_context_outputs(ctx, W, H, view, depth, normals, pos, li, L)


@pytest.fixture
def host_zero_copy():
    lib = vg.lib()
    knob = vg._lib.TUNE["host_zero_copy"]
    saved = lib.vren_tuning_get(knob)
    yield lambda v: lib.vren_tuning_set(knob, v)
    lib.vren_tuning_set(knob, saved)


@pytest.mark.parametrize("use_graph", [True, False])
@pytest.mark.parametrize("zero_copy,W,H", [(0, 640, 360), (1, 640, 360), (1, 601, 333)])
def test_cluster_host_matches_device_path(cuda, host_zero_copy, use_graph, zero_copy, W, H):
    """vren_cs_cluster_host (page-locked host inputs; the G-buffer copied up in bands with the
    reference download overlapped, or read and written over the link by the unique-cluster kernel
    itself) gives the same outputs as vren_cs_cluster on the same data; a width that is not a multiple
    of 4 takes the kernels' scalar loads."""
    assert host_zero_copy(zero_copy) == 0
    L = 3000
    view = make_view(W, H)
    depth, normals = scene.depth_planes(41, W, H)
    pos, li = dense_lights(42, L)
    stream = torch.cuda.Stream(device=cuda)
    a = cs.cluster_and_shade(W, H, L, 1 << 22, use_graph=use_graph)
    b = cs.cluster_and_shade(W, H, L, 1 << 22, use_graph=use_graph)
    with torch.cuda.stream(stream):
        a.cluster(stream, view, W, H, to_dev(depth, cuda), to_dev(normals, cuda), to_dev(pos, cuda), to_dev(li, cuda),
                  L)
    stream.synchronize()
    hp = lambda x: torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
    h_refs = torch.zeros(W * H, dtype=torch.int32).pin_memory()
    h_lists = torch.zeros(1 << 22, dtype=torch.int32).pin_memory()
    ins = (hp(depth), hp(normals), hp(pos), hp(li))
    for _ in range(2):  # second call replays the captured graph
        h_refs.zero_()
        h_lists.zero_()
        with torch.cuda.stream(stream):
            b.cluster_host(stream, view, W, H, *ins, L, h_refs, h_lists)
        stream.synchronize()
        oa, ob = a.outputs(), b.outputs()
        U = int(cs.read_device(oa.key_count, 1)[0])
        tot = int(cs.read_device(oa.total, 1)[0])
        assert U > 0 and tot > 0
        assert int(cs.read_device(ob.key_count, 1)[0]) == U and int(cs.read_device(ob.total, 1)[0]) == tot
        for name, n in (("cluster_keys", U), ("counts", U), ("offsets", U), ("indices", tot), ("cluster_refs", W * H)):
            assert np.array_equal(cs.read_device(getattr(oa, name), n), cs.read_device(getattr(ob, name), n)), name
        assert np.array_equal(h_refs.numpy().view(np.uint32), cs.read_device(oa.cluster_refs, W * H))
        hl = h_lists.numpy().view(np.uint32)
        assert hl[0] == U and hl[1] == tot
        for k, (name, n) in enumerate((("cluster_keys", U), ("counts", U), ("offsets", U))):
            assert np.array_equal(hl[2 + k * U: 2 + (k + 1) * U], cs.read_device(getattr(oa, name), n)), name
        assert np.array_equal(hl[2 + 3 * U: 2 + 3 * U + tot], cs.read_device(oa.indices, tot))
