"""The oracle against the reference's own shader source (oracle/_ref: the reference's GLSL compute
shaders rewritten mechanically into C++ by oracle/ref_shaders.py and run on the CPU).

Two variants of the reference are compared:
  - canonical: the shaders with the canonical decisions substituted at their five places (slice from
    the host-built table, slice bounds from the same table, host-built inverse(projection) and
    inverse(view), integer texel).  It must equal the oracle bit for bit, stage by stage, on seeded
    and adversarial inputs.
  - glsl: the shaders as written (C library log / pow, single-precision inverse, NEAREST + REPEAT
    sampling at gid / size).  Where it departs from the oracle, the departure must lie in one of the
    classes the canonical decisions cover, and each class is counted: a depth slice off by one at a
    slice boundary, a neighbouring texel picked by the float sampler coordinate, cluster boxes a few
    hundred ulps apart (float inverse and pow).

Runs where the reference checkout is present (this builds oracle/_ref if needed); skips elsewhere.
"""
import numpy as np
import pytest

import oracle
import shade_scene
import vren_gb300.clustered_shading as cs
import vren_gb300.scene as scene
from oracle import ref, ref_shaders


@pytest.fixture(scope="module")
def refs():
    if ref_shaders.build() is None and not ref.available():
        pytest.skip("reference checkout not present: oracle/_ref not built")
    return ref.Ref("glsl"), ref.Ref("canonical")


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same_floats(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return (bits(a) == bits(b)) | (np.isnan(a) & np.isnan(b))


def frame(W, H, seed, moved=False):
    if moved:
        cam = cs.scene_camera(W, H, position=(3.0, -2.0, 1.5), yaw=0.3, pitch=-0.2)
    else:
        cam = cs.scene_camera(W, H)
    view = cs.view_from_camera(cam, "ref")
    depth, normals = scene.depth_planes(seed, W, H)
    return view, depth, normals


def install_canonical(R, view, H):
    near, far = oracle.cs_slice_table(view, (H + 31) // 32)
    R.set_canonical(view, near, far, 1023)


def projection(view, W, H):
    return ref.reference_projection(W, H, view.near_plane, view.far_plane, 2.0 * view.half_fov_y)


def adversarial_normals():
    vals = np.array([0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 1e-40, -1e-40, 3e38, -3e38, np.inf, -np.inf, np.nan,
                     0.57735026, -0.57735026, 2.0 / 3.0, 1.0 / 3.0], np.float32)
    g = np.stack(np.meshgrid(vals, vals, vals, indexing="ij"), -1).reshape(-1, 3)
    return g


# ------------------------------------------------------------------------------------------------
def test_normal_bin(refs):
    """clustered_shading_discretize_normal (clustered_shading.glsl:7-43): 10^6 seeded normals, the
    adversarial grid (signed zeros, subnormals, infinities, NaN, exact ties between axes) and normals
    on the cube's bin edges; no canonical substitution applies, so both variants must agree."""
    rng = np.random.default_rng(11)
    n = np.concatenate([rng.standard_normal((1_000_000, 3)).astype(np.float32), adversarial_normals(),
                        rng.integers(-3, 4, (100_000, 3)).astype(np.float32) / np.float32(3.0)])
    want = oracle.cs_normal_bins(n)
    for R in refs:
        assert np.array_equal(R.normal_bin(n), want), R.variant


def test_decode_cluster_key(refs):
    keys = np.random.default_rng(12).integers(0, 2**32, 1_000_000, dtype=np.uint64).astype(np.uint32)
    got = refs[1].decode_cluster_key(keys)
    want = np.stack([keys & 0xFF, (keys >> 8) & 0xFF, (keys >> 16) & 0x3FF, keys >> 26], 1)
    assert np.array_equal(got, want)


def test_overlap_tests(refs):
    """test_aabb_aabb and test_sphere_aabb (assign_lights.comp:84-102) on 10^6 seeded cases each,
    with touching faces, invalid nodes (+inf / -inf boxes, radius -inf) and inverted cluster boxes."""
    rng = np.random.default_rng(13)
    N = 1_000_000
    t = rng.uniform(-10, 10, (N, 12)).astype(np.float32)
    t[::7, 6:9] = t[::7, 3:6]
    t[::11, 6:9] = np.inf
    t[::11, 9:12] = -np.inf
    t[::13, 0:3], t[::13, 3:6] = t[::13, 3:6].copy(), t[::13, 0:3].copy()
    s = rng.uniform(-10, 10, (N, 10)).astype(np.float32)
    s[:, 3] = np.abs(s[:, 3])
    s[::9, 3] = -np.inf
    s[::5, 4:7], s[::5, 7:10] = s[::5, 7:10].copy(), s[::5, 4:7].copy()
    s[::17, 0:3] = s[::17, 4:7]
    wa, ws = oracle.cs_test_aabb_aabb(t), oracle.cs_test_sphere_aabb(s)
    assert 0 < wa.sum() < N and 0 < ws.sum() < N
    for R in refs:
        assert np.array_equal(R.test_aabb_aabb(t), wa), R.variant
        assert np.array_equal(R.test_sphere_aabb(s), ws), R.variant


def slice_boundary_depths(view, W, H, count):
    """NDC depths whose view depth lands on, or one ulp either side of, REF slice boundaries."""
    near, _ = oracle.cs_slice_table(view, (H + 31) // 32)
    z = near[(near > view.near_plane) & (near < view.far_plane)].astype(np.float32)
    z = np.concatenate([z, np.nextafter(z, np.float32(0)), np.nextafter(z, np.float32(np.inf))])
    n, f = np.float64(view.near_plane), np.float64(view.far_plane)
    d = (f / (f - n) - f * n / ((f - n) * z.astype(np.float64))).astype(np.float32)
    return np.resize(d, count)


@pytest.mark.parametrize("W,H,seed,moved,boundary", [(1920, 1080, 7, False, False), (333, 197, 3, True, False),
                                                     (640, 360, 9, False, True)])
def test_cluster_key_of_every_invocation(refs, W, H, seed, moved, boundary):
    """find_unique_clusters.comp:46-76: the key of every invocation of the dispatch (the 32x32
    overhang included, its texels wrapped).  Canonical: equal everywhere.  GLSL as written: every
    difference is either an invocation whose float sampler coordinate picks another texel, or a depth
    slice off by one (log against the boundary table), nothing else."""
    G, C = refs
    view, depth, normals = frame(W, H, seed, moved)
    if boundary:
        depth = slice_boundary_depths(view, W, H, W * H)
    install_canonical(C, view, H)
    proj = projection(view, W, H)
    want = oracle.cs_pixel_keys(depth, normals, W, H, view)
    assert np.array_equal(C.pixel_keys(W, H, depth, normals, view.near_plane, view.half_fov_y, proj), want)
    got = G.pixel_keys(W, H, depth, normals, view.near_plane, view.half_fov_y, proj)
    TY, TX = want.shape
    gy, gx = np.mgrid[0:TY, 0:TX]
    sx = np.floor((gx.astype(np.float32) / np.float32(W)) * np.float32(W)).astype(np.int64) % W
    sy = np.floor((gy.astype(np.float32) / np.float32(H)) * np.float32(H)).astype(np.int64) % H
    texel_moved = (sx != gx % W) | (sy != gy % H)
    diff = got != want
    rest = diff & ~texel_moved
    kdelta = ((got[rest] >> 16) & 0x3FF).astype(np.int64) - ((want[rest] >> 16) & 0x3FF).astype(np.int64)
    assert np.all(np.abs(kdelta) == 1), np.unique(kdelta)
    assert np.all(((got[rest] ^ want[rest]) & ~np.uint32(0x3FF << 16)) == 0)
    assert diff.sum() < 0.01 * diff.size or boundary


def test_cluster_boxes(refs):
    """calc_cluster_aabb (clustered_shading.glsl:72-110) for every key of the 1080p frame (60 x 34 tiles,
    1024 slices): canonical equal; GLSL as written within a bounded number of ulps."""
    G, C = refs
    W, H = 1920, 1080
    view, _, _ = frame(W, H, 1)
    install_canonical(C, view, H)
    proj = projection(view, W, H)
    TX, TY = (W + 31) // 32, (H + 31) // 32
    i, j, k = np.meshgrid(np.arange(TX), np.arange(TY), np.arange(1024), indexing="ij")
    keys = (i | (j << 8) | (k << 16)).astype(np.uint32).reshape(-1)
    mn, mx = oracle.cs_cluster_boxes(keys, W, H, view)
    cmn, cmx = C.cluster_boxes(keys, TX, TY, view.near_plane, view.half_fov_y, proj)
    assert np.array_equal(bits(cmn[:, :3]), bits(mn)) and np.array_equal(bits(cmx[:, :3]), bits(mx))
    gmn, gmx = G.cluster_boxes(keys, TX, TY, view.near_plane, view.half_fov_y, proj)
    ulps = np.abs(bits(gmn[:, :3]).view(np.int32).astype(np.int64) - bits(mn).view(np.int32).astype(np.int64))
    assert ulps.max() < 4096


@pytest.mark.parametrize("W,H,L,kind,moved", [(1920, 1080, 16384, "uniform", False), (640, 360, 3000, "dense", True),
                                             (320, 180, 40000, "dense", False), (320, 180, 2000, "same_z", False)])
def test_light_bvh_and_assignment(refs, W, H, L, kind, moved):
    """construct_point_light_bvh's shaders (view transform, Morton codes, leaves) and assign_lights.comp
    (count and write dispatches, its 32 invocations run in lockstep with their ballots) against the
    oracle's stages: equal in both variants for the light stages, equal in the canonical variant for
    the assignment (counts, offsets and every list in order)."""
    G, C = refs
    view, depth, normals = frame(W, H, W + L, moved)
    if kind == "uniform":
        pos, li = scene.lights(L, L, W, H)
    else:
        rng = np.random.default_rng(L)
        p = np.zeros((L, 4), np.float32)
        p[:, 0] = rng.uniform(-8, 8, L)
        p[:, 1] = rng.uniform(-5, 5, L)
        p[:, 2] = rng.uniform(0.5, 25, L) if kind == "dense" else 10.0
        p[:, 3] = 1
        q = np.zeros((L, 4), np.float32)
        q[:, :3] = rng.uniform(0, 1, (L, 3))
        q[:, 3] = np.exp(np.log(2.0) + 0.5 * rng.standard_normal(L)).astype(np.float32) * 0.5
        pos, li = p.reshape(-1), q.reshape(-1)
    vp, mn, mx, codes = oracle.cs_light_codes(pos, L, view, 15)
    evp, ebvh, elidx = oracle.cs_light_bvh(pos, li, L, view, 15)
    sizes = oracle.size_helpers(L)
    P = sizes["padded"]
    valid = ebvh[:P, 3] != 0xFFFFFFFE
    for R in refs:
        assert np.all(same_floats(R.view_space(view.view, pos, L), vp)), R.variant
        assert np.array_equal(R.morton(vp, L, mn, mx), codes), R.variant
        leaves = R.leaves(evp, li, elidx, L, P)
        assert np.array_equal(leaves[:P][valid], ebvh[:P][valid]) and np.all(leaves[:P][~valid][:, 3] == 0xFFFFFFFE)
    keys, _ = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0)
    ec, eo, ei, et = oracle.cs_assign_lights(keys, W, H, view, ebvh, L, elidx, evp)
    assert et > 0 or kind == "uniform"
    install_canonical(C, view, H)
    proj = projection(view, W, H)
    lidx = np.zeros((P, 2), np.uint32)  # the reference's index buffer covers the padded leaves
    lidx[:L] = elidx.reshape(L, 2)
    TX, TY = (W + 31) // 32, (H + 31) // 32
    args = (keys, TX, TY, view.near_plane, view.half_fov_y, proj, ebvh, sizes["root"], sizes["levels"], lidx, evp, L)
    c, o, i = C.assign_lights(*args)
    assert np.array_equal(c, ec) and np.array_equal(o, eo) and np.array_equal(i, ei)
    assert C.oob() == 0
    gc, _, _ = G.assign_lights(*args)
    assert np.count_nonzero(gc != ec) <= max(2, len(keys) // 100)  # boxes a few hundred ulps apart


def test_shade(refs):
    """shade.comp:69-141 with pbr.glsl (the reference falloff, colour output with ambient and gamma),
    run through the reference's material model, against the oracle's FP64 evaluation: the same pixels
    shaded, and the single-precision shader within 1e-4 of FP64 normwise."""
    _, C = refs
    s = shade_scene.make(320, 180, 700, seed=5)
    W, H, view = s["W"], s["H"], s["view"]
    install_canonical(C, view, H)
    img = C.shade(W, H, shade_scene.gb(s), shade_scene.lists(s), s["pos"], s["lights"], s["L"], view.eye,
                  view.far_plane, view.view, projection(view, W, H))
    want, shaded = oracle.cs_shade_f64(view, W, H, shade_scene.gb(s), shade_scene.lists(s), s["pos"], s["lights"],
                                       s["L"], 0, 0)
    written = ~np.isnan(img[..., 0].reshape(-1))
    assert np.array_equal(written, shaded) and shaded.sum() > 1000
    got = img[..., :3].reshape(-1, 3).astype(np.float64)[shaded]
    want = want.reshape(-1, 3)[shaded]
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-4


def test_bouncer(refs):
    """vren_demo's bounce_point_lights.comp:33-73 on 10^6 lights (a thousand with a zero direction),
    bit for bit (NaN as NaN)."""
    rng = np.random.default_rng(14)
    L = 1_000_000
    pos = np.zeros((L, 4), np.float32)
    pos[:, :3] = rng.uniform(-12, 12, (L, 3))
    pos[:, 3] = 1
    d = rng.standard_normal((L, 4)).astype(np.float32)
    d[:, 3] = 0
    d[::1000, :3] = 0
    lo, hi = np.array([-10, -5, -8], np.float32), np.array([10, 5, 8], np.float32)
    wp, wd = oracle.bounce_point_lights(pos.reshape(-1), d.reshape(-1), L, lo, hi, 3.0, 0.7)
    for R in refs:
        gp, gd = R.bounce(pos.reshape(-1), d.reshape(-1), L, lo, hi, 3.0, 0.7)
        assert np.all(same_floats(gp, wp)) and np.all(same_floats(gd, wd)), R.variant


@pytest.mark.parametrize("W,H", [(5, 3), (37, 1000), (1920, 1080), (1, 1)])
def test_depth_pyramid(refs, W, H):
    """depth_buffer_copy.comp and one depth_buffer_reduce.comp dispatch per level (NaN, -0 and +inf
    depths included), bit for bit."""
    rng = np.random.default_rng(W * H)
    depth = rng.uniform(0, 1, W * H).astype(np.float32)
    depth[::97] = np.nan
    depth[::101] = -0.0
    depth[::103] = np.inf
    want = oracle.depth_pyramid(depth, W, H)
    for R in refs:
        got = R.depth_pyramid(depth, W, H, len(want))
        for lvl, (a, b) in enumerate(zip(got, want)):
            assert np.array_equal(a.view(np.uint32), b.reshape(-1).view(np.uint32)), (R.variant, lvl)


@pytest.mark.parametrize("mode", list(range(7)))
def test_show_clusters(refs, mode):
    """vren_demo's show_clusters.comp:68-125 in every mode (6 = an unknown mode, drawn red), bit for bit."""
    s = shade_scene.make(320, 180, 700, seed=5)
    want = oracle.cs_show_clusters(mode, s["W"], s["H"], s["refs"], s["keys"], s["counts"], s["offsets"], s["indices"])
    got = refs[1].show_clusters(mode, s["W"], s["H"], s["refs"], s["keys"], s["counts"], s["offsets"], s["indices"])
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
