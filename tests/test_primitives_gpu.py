"""GPU parity tests of the primitives against the CPU oracle, through the C ABI.

Modelled on the reference's tests (vren_test/vren_test/primitives/*.cpp): the same inputs
(seeded instead of std::rand), the same comparisons (whole reduce tree, whole scan, sorted keys,
BVH point queries vs a linear scan), plus edge cases: empty and ragged lengths, segments, in-place
forms, maximum-digit keys, duplicate keys (stability) and the reference's argument errors.
"""
import numpy as np
import pytest
import torch

import oracle
import vren_gb300 as vg

pytestmark = pytest.mark.gpu


def dev_u32(a: np.ndarray, device) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32)).to(device)


def host_u32(t: torch.Tensor) -> np.ndarray:
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint32)


# ------------------------------------------------------------------------------------------------
# Reduce
# ------------------------------------------------------------------------------------------------
@pytest.mark.parametrize("op", ["add", "min", "max"])
@pytest.mark.parametrize("n", [1, 2, 3, 31, 1000, 4096, 4097, 10000, 100000, 1 << 20, (1 << 20) + 5])
def test_reduce_tree_u32(cuda, op, n):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 100 if op != "add" else 1 << 20, n).astype(np.uint32)
    P = vg.calc_reduce_output_buffer_length(n)
    inp = dev_u32(x, cuda)
    out = torch.full((P,), -1, dtype=torch.int32, device=cuda)
    vg.reduce("uint", op)(None, inp, n, 0, out, 0, 1)
    assert np.array_equal(host_u32(out), oracle.reduce_tree_u32(op, x))


@pytest.mark.parametrize("n", [10000, (1 << 24) + 3])
def test_reduce_tree_u32_in_place_all_ones(cuda, n):
    P = vg.calc_reduce_output_buffer_length(n)
    buf = torch.zeros(P, dtype=torch.int32, device=cuda)
    buf[:n] = 1
    vg.reduce("uint", "add")(None, buf, n, 0, blocks_num=1)
    expect = oracle.reduce_tree_u32("add", np.ones(n, np.uint32))
    assert np.array_equal(host_u32(buf), expect)
    assert expect[-1] == n


def test_reduce_tree_u32_segments(cuda):
    rng = np.random.default_rng(9)
    n, blocks = 1000, 16
    x = rng.integers(0, 1 << 16, n * blocks).astype(np.uint32)
    P = vg.calc_reduce_output_buffer_length(n)
    out = torch.zeros(P * blocks, dtype=torch.int32, device=cuda)
    vg.reduce("uint", "add")(None, dev_u32(x, cuda), n, 0, out, 0, blocks)
    got = host_u32(out).reshape(blocks, P)
    for b in range(blocks):
        assert np.array_equal(got[b], oracle.reduce_tree_u32("add", x[b * n:(b + 1) * n]))


@pytest.mark.parametrize("op", ["add", "min", "max"])
@pytest.mark.parametrize("n", [1, 7, 1000, 10000, 300000])
def test_reduce_tree_vec4(cuda, op, n):
    rng = np.random.default_rng(100 + n)
    x = (rng.integers(0, 100, (n, 4)) if op != "add" else rng.standard_normal((n, 4))).astype(np.float32)
    P = vg.calc_reduce_output_buffer_length(n)
    out = torch.zeros((P, 4), dtype=torch.float32, device=cuda)
    vg.reduce("vec4", op)(None, torch.from_numpy(x).to(cuda), n, 0, out, 0, 1)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    expect = oracle.reduce_tree_vec4(op, x)
    assert np.array_equal(got.view(np.uint32), expect.view(np.uint32)), "float tree must be bit-identical"


@pytest.mark.parametrize("op", ["add", "min", "max"])
@pytest.mark.parametrize("n", [0, 1, 5, 1 << 16, (1 << 20) + 3, 1 << 24])
def test_reduce_scalar_u32(cuda, op, n):
    rng = np.random.default_rng(n + 1)
    x = rng.integers(0, 256, n).astype(np.uint32)
    out = torch.zeros(1, dtype=torch.int32, device=cuda)
    sc = vg.primitives.alloc_scratch(vg.primitives.reduce_scratch_bytes(n), cuda)
    for _ in range(2):  # the scratch is reusable across calls
        vg.reduce_scalar(None, op, dev_u32(x, cuda) if n else torch.zeros(4, dtype=torch.int32, device=cuda)[:0],
                         out, sc)
        assert host_u32(out)[0] == oracle.reduce_u32(op, x)


@pytest.mark.parametrize("n", [(1 << 22) + 4099, 305 * 4096, 1 << 20, 4099])
@pytest.mark.parametrize("form", [0, 1, 2, 3, 4, 5])
def test_reduce_scalar_streaming_edges(cuda, restore_tuning, n, form):
    """Every scalar reduce form (grid-stride loop, streaming stage shapes, automatic): extremes
    planted in the last partial stage, the scalar tail (n mod 4) and the first element; more stages
    than CTAs and CTAs with no stage."""
    assert restore_tuning.vren_tuning_set(vg._lib.TUNE["reduce_form"], form) == 0
    rng = np.random.default_rng(n)
    x = rng.integers(100, 200, n).astype(np.uint32)
    x[-1] = 3                     # tail element (n mod 4 != 0) or the last element of the last stage
    x[max((n // 4096) * 4096 - 5, 1)] = 900
    x[0] = 7
    sc = vg.primitives.alloc_scratch(vg.primitives.reduce_scratch_bytes(n), cuda)
    d = dev_u32(x, cuda)
    for op in ("add", "min", "max"):
        out = torch.zeros(1, dtype=torch.int32, device=cuda)
        vg.reduce_scalar(None, op, d, out, sc)
        assert host_u32(out)[0] == oracle.reduce_u32(op, x), op


def test_reduce_scalar_u32_sum_wraps(cuda):
    n = 1 << 26
    x = torch.full((n,), 255, dtype=torch.int32, device=cuda)
    out = torch.zeros(1, dtype=torch.int32, device=cuda)
    sc = vg.primitives.alloc_scratch(vg.primitives.reduce_scratch_bytes(n), cuda)
    vg.reduce_scalar(None, "add", x, out, sc)
    assert host_u32(out)[0] == (n * 255) & 0xFFFFFFFF


@pytest.mark.parametrize("op", ["min", "max"])
def test_reduce_scalar_f32_total_order(cuda, op):
    rng = np.random.default_rng(4)
    x = rng.integers(0, 256, (1 << 20) + 7).astype(np.float32)
    x[123] = -0.0
    x[456] = 0.0
    out = torch.zeros(1, dtype=torch.float32, device=cuda)
    sc = vg.primitives.alloc_scratch(vg.primitives.reduce_scratch_bytes(len(x)), cuda)
    vg.reduce_scalar(None, op, torch.from_numpy(x).to(cuda), out, sc)
    torch.cuda.synchronize()
    assert out.cpu().numpy().view(np.uint32)[0] == np.array([oracle.reduce_f32(op, x)], np.float32).view(np.uint32)[0]


# ------------------------------------------------------------------------------------------------
# Scan
# ------------------------------------------------------------------------------------------------
def test_scan_all_ones_reference_lengths(cuda):
    # vren_test/primitives/blelloch_scan.cpp:166-176: lengths 2^0 .. 2^19, all ones
    scan = vg.blelloch_scan()
    for e in range(0, 20):
        n = 1 << e
        buf = torch.ones(n, dtype=torch.int32, device=cuda)
        scan(None, buf, n)
        assert np.array_equal(host_u32(buf), np.arange(n, dtype=np.uint32)), n


@pytest.mark.parametrize("n", [1, 3, 4095, 4096, 4097, 100003, 1 << 22, (1 << 26)])
def test_scan_random(cuda, n):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 256, n).astype(np.uint32)
    buf = dev_u32(x, cuda)
    scan = vg.blelloch_scan()
    scan(None, buf, n)
    assert np.array_equal(host_u32(buf), oracle.exclusive_scan_u32(x))
    # a second call reuses the scratch (epoch-tagged status words)
    buf2 = dev_u32(x[::-1].copy(), cuda)
    scan(None, buf2, n)
    assert np.array_equal(host_u32(buf2), oracle.exclusive_scan_u32(x[::-1].copy()))


def test_scan_wraps_mod_2_32(cuda):
    n = 1 << 20
    x = np.full(n, 0xFFFFFFF0, np.uint32)
    buf = dev_u32(x, cuda)
    vg.blelloch_scan()(None, buf, n)
    assert np.array_equal(host_u32(buf), oracle.exclusive_scan_u32(x))


def test_scan_segments(cuda):
    rng = np.random.default_rng(77)
    n, blocks = 10000, 7
    x = rng.integers(0, 1000, n * blocks).astype(np.uint32)
    buf = dev_u32(x, cuda)
    vg.blelloch_scan()(None, buf, n, 0, blocks)
    got = host_u32(buf).reshape(blocks, n)
    for b in range(blocks):
        assert np.array_equal(got[b], oracle.exclusive_scan_u32(x[b * n:(b + 1) * n]))


@pytest.mark.parametrize("n", [1, 2, 16, 512, 1024, 2048, 4096, 8192, 1 << 17, 1 << 20])
@pytest.mark.parametrize("clear_last", [True, False])
def test_downsweep_matches_reference_dispatches(cuda, n, clear_last):
    rng = np.random.default_rng(n * 2 + int(clear_last))
    x = rng.integers(0, 1 << 30, n).astype(np.uint32)  # arbitrary buffer, not necessarily a tree
    buf = dev_u32(x, cuda)
    vg.blelloch_scan().downsweep(None, buf, n, 0, 1, clear_last)
    assert np.array_equal(host_u32(buf), oracle.downsweep_u32(x, clear_last))


def test_downsweep_segments(cuda):
    rng = np.random.default_rng(5)
    n, blocks = 4096, 16
    x = rng.integers(0, 1 << 30, n * blocks).astype(np.uint32)
    buf = dev_u32(x, cuda)
    vg.blelloch_scan().downsweep(None, buf, n, 0, blocks, True)
    got = host_u32(buf).reshape(blocks, n)
    for b in range(blocks):
        assert np.array_equal(got[b], oracle.downsweep_u32(x[b * n:(b + 1) * n], True))


# ------------------------------------------------------------------------------------------------
# Radix sort
# ------------------------------------------------------------------------------------------------
def test_radix_sort_reversed_iota_1024(cuda):
    # vren_test/primitives/radix_sort.cpp:68-132
    n = 1024
    rs = vg.radix_sort()
    buf = dev_u32(np.arange(n, dtype=np.uint32)[::-1].copy(), cuda)
    rs(None, buf, n, rs.create_scratch_buffer_1(n, cuda), rs.create_scratch_buffer_2(n, cuda))
    assert np.array_equal(host_u32(buf), np.arange(n, dtype=np.uint32))


def test_radix_sort_precondition(cuda):
    rs = vg.radix_sort()
    buf = torch.zeros(2000, dtype=torch.int32, device=cuda)
    for n in (1000, 512, 1536):
        with pytest.raises(ValueError, match="power of 2"):
            rs(None, buf, n, rs.create_scratch_buffer_1(2000, cuda), rs.create_scratch_buffer_2(2000, cuda))


@pytest.mark.parametrize("n", [1 << 10, 1 << 16, 1 << 20, 1 << 24])
def test_radix_sort_keys_dropin(cuda, n):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    rs = vg.radix_sort()
    buf = dev_u32(x, cuda)
    rs(None, buf, n, rs.create_scratch_buffer_1(n, cuda), rs.create_scratch_buffer_2(n, cuda))
    assert np.array_equal(host_u32(buf), np.sort(x))


@pytest.mark.parametrize("bits", [4, 6, 8])
@pytest.mark.parametrize("n", [2, 1000, 3839, 3840, 3841, 65537, 1 << 20, 3_000_017])
def test_radix_sort_pairs_stable(cuda, bits, n):
    rng = np.random.default_rng(n + bits)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 3] = keys[n // 3: 2 * (n // 3)]  # duplicates exercise stability
    keys[0] = 0xFFFFFFFF
    vals = np.arange(n, dtype=np.uint32)
    rs = vg.radix_sort(bits)
    k, v = dev_u32(keys, cuda), dev_u32(vals, cuda)
    s1 = rs.create_scratch_buffer_1(n, cuda)
    tk, tv = torch.empty_like(k), torch.empty_like(v)
    for rep in range(2):  # scratch reuse
        k, v = dev_u32(keys, cuda), dev_u32(vals, cuda)
        rs.sort(None, k, v, n, s1, tk, tv)
        ek, ev = oracle.stable_sort_u32(keys, vals)
        assert np.array_equal(host_u32(k), ek)
        assert np.array_equal(host_u32(v), ev)


@pytest.mark.parametrize("bits", [4, 6, 8])
@pytest.mark.parametrize("n", [2, 1000, 3839, 3840, 3841, 100003, 1 << 20, 3_000_017])
@pytest.mark.parametrize("values", [True, False])
def test_radix_sort_persistent_pass(cuda, restore_tuning, bits, n, values):
    """The persistent pass (bulk-copied tiles, digit counts published on arrival) sorts pairs and keys
    exactly as the stable oracle: partial last tiles whose length is not a multiple of 4, one tile,
    many tiles, equal keys; two sorts in a row on one scratch."""
    assert restore_tuning.vren_tuning_set(vg._lib.TUNE["radix_persistent"], 1) == 0
    rng = np.random.default_rng(7 * n + bits)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 3] = keys[n // 3: 2 * (n // 3)]
    keys[0] = 0xFFFFFFFF
    vals = np.arange(n, dtype=np.uint32)
    rs = vg.radix_sort(bits)
    s1 = rs.create_scratch_buffer_1(n, cuda)
    ek, ev = oracle.stable_sort_u32(keys, vals)
    for _ in range(2):
        k = dev_u32(keys, cuda)
        v = dev_u32(vals, cuda) if values else None
        tk = torch.empty_like(k)
        tv = torch.empty_like(v) if values else None
        rs.sort(None, k, v, n, s1, tk, tv)
        assert np.array_equal(host_u32(k), ek)
        if values:
            assert np.array_equal(host_u32(v), ev)
    assert vg.device_error() == 0


def test_radix_sort_pairs_2e20_config(cuda):
    """The benchmark configuration: 2^20 pairs, keys = PCG32 full range, values = index."""
    import ctypes

    from vren_gb300 import _build

    scene = ctypes.CDLL(str(_build.SCENE_LIB))
    n = 1 << 20
    keys = np.empty(n, np.uint32)
    scene.vren_gen_u32(ctypes.c_uint64(42), ctypes.c_uint64(1), keys.ctypes.data_as(ctypes.c_void_p),
                       ctypes.c_uint64(n), 0)
    vals = np.arange(n, dtype=np.uint32)
    rs = vg.radix_sort(8)
    k, v = dev_u32(keys, cuda), dev_u32(vals, cuda)
    rs.sort(None, k, v, n, rs.create_scratch_buffer_1(n, cuda), torch.empty_like(k), torch.empty_like(v))
    ek, ev = oracle.stable_sort_u32(keys, vals)
    assert np.array_equal(host_u32(k), ek) and np.array_equal(host_u32(v), ev)


# ------------------------------------------------------------------------------------------------
# Bucket sort
# ------------------------------------------------------------------------------------------------
@pytest.mark.parametrize("key_bits", [16, 10, 8, 3])
@pytest.mark.parametrize("n", [0, 1, 5, 30, 900, 5000, 123457, 1 << 24])
def test_bucket_sort(cuda, key_bits, n):
    if n == 1 << 24 and key_bits not in (16, 10):
        pytest.skip("large case only for the reference and benchmark widths")
    rng = np.random.default_rng(n * 31 + key_bits)
    pairs = np.stack([rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32),
                      np.arange(n, dtype=np.uint32)], 1).reshape(-1)
    bs = vg.bucket_sort(key_bits)
    out = torch.zeros(bs.get_required_output_buffer_size(n) // 4, dtype=torch.int32, device=cuda)
    inp = dev_u32(pairs, cuda) if n else torch.zeros(4, dtype=torch.int32, device=cuda)
    bs(None, inp, n, 0, out, 0)
    got = host_u32(out)
    exp_pairs, exp_ends = oracle.bucket_sort_u32x2(pairs.reshape(-1, 2), key_bits)
    assert np.array_equal(got[: 2 * n].reshape(-1, 2), exp_pairs)
    off = ((8 * n + 255) // 256 * 256) // 4
    assert np.array_equal(got[off: off + (1 << key_bits)], exp_ends)


@pytest.fixture
def bucket_form():
    lib = vg.lib()
    knobs = (vg._lib.TUNE["bucket_form"], vg._lib.TUNE["radix_rank"])
    saved = [lib.vren_tuning_get(k) for k in knobs]
    yield lambda form, rank: [lib.vren_tuning_set(k, v) for k, v in zip(knobs, (form, rank))]
    for k, v in zip(knobs, saved):
        lib.vren_tuning_set(k, v)


@pytest.mark.parametrize("form,rank", [(0, 0), (0, 1), (0, 2), (1, 0), (1, 2)])
@pytest.mark.parametrize("keys", ["uniform", "one_bucket", "two_buckets", "runs", "descending"])
@pytest.mark.parametrize("key_bits,n", [(10, 4096), (10, 4097), (10, 8192), (10, 8193), (10, 3 * 4096 - 5),
                                        (10, 3 * 4096), (10, 16384), (10, 16385), (10, 2 * 16384 + 3 * 4096 + 7),
                                        (10, 300001), (7, 123457), (1, 65537), (10, 1 << 22)])
def test_bucket_sort_forms(cuda, bucket_form, form, rank, keys, key_bits, n):
    """Both forms of the bucket sort of up to 10 key bits (one scatter pass over rows of two
    4096-element tiles, and radix passes) against the stable oracle: rows and tiles full, ragged and
    empty, and key sets that put every element in one bucket, in two, in long runs or in descending
    order."""
    bucket_form(form, rank)
    rng = np.random.default_rng(n * 7 + key_bits)
    if keys == "uniform":
        k = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    elif keys == "one_bucket":
        k = (rng.integers(0, 2**20, n, dtype=np.uint64).astype(np.uint32) << 10) | 5
    elif keys == "two_buckets":
        k = rng.integers(0, 2, n).astype(np.uint32) * 0x3FF
    elif keys == "runs":
        k = (np.arange(n, dtype=np.uint64) // 5000).astype(np.uint32) * 0x9E3779B1
    else:
        k = (n - np.arange(n, dtype=np.uint64)).astype(np.uint32)
    pairs = np.stack([k, np.arange(n, dtype=np.uint32)], 1).reshape(-1)
    bs = vg.bucket_sort(key_bits)
    out = torch.zeros(bs.get_required_output_buffer_size(n) // 4, dtype=torch.int32, device=cuda)
    inp = dev_u32(pairs, cuda)
    exp_pairs, exp_ends = oracle.bucket_sort_u32x2(pairs.reshape(-1, 2), key_bits)
    off = ((8 * n + 255) // 256 * 256) // 4
    for _ in range(2):  # a second call on the same scratch
        out.zero_()
        bs(None, inp, n, 0, out, 0)
        got = host_u32(out)
        assert np.array_equal(got[: 2 * n].reshape(-1, 2), exp_pairs)
        assert np.array_equal(got[off: off + (1 << key_bits)], exp_ends)
    assert vg.lib().vren_device_error(1) == 0


@pytest.mark.parametrize("n", [(1 << 26) + 12345])
def test_bucket_sort_many_row_blocks(cuda, n):
    """The one-scatter form past one wave of column-scan CTAs: 16,388 tile rows in 65 blocks of 256
    rows (the last one 4 rows, its last tile ragged), so blocks look back over blocks whose CTAs
    started in earlier waves.  Checked by properties: buckets ascending, values (the input indices)
    ascending within a bucket, a permutation, and the end offsets equal to the bucket counts' prefix."""
    key_bits = 10
    rng = np.random.default_rng(2026)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    pairs = np.stack([keys, np.arange(n, dtype=np.uint32)], 1).reshape(-1)
    bs = vg.bucket_sort(key_bits)
    out = torch.empty(bs.get_required_output_buffer_size(n) // 4, dtype=torch.int32, device=cuda)
    bs(None, dev_u32(pairs, cuda), n, 0, out, 0)
    got = host_u32(out)
    k, v = got[0: 2 * n: 2], got[1: 2 * n: 2]
    b = k & ((1 << key_bits) - 1)
    assert np.all(np.diff(b.astype(np.int64)) >= 0)
    assert np.all((np.diff(b.astype(np.int64)) > 0) | (np.diff(v.astype(np.int64)) > 0))
    assert np.array_equal(k, keys[v])
    assert np.array_equal(np.bincount(v, minlength=n), np.ones(n, np.int64))
    off = ((8 * n + 255) // 256 * 256) // 4
    ends = np.cumsum(np.bincount(keys & ((1 << key_bits) - 1), minlength=1 << key_bits))
    assert np.array_equal(got[off: off + (1 << key_bits)], ends.astype(np.uint32))
    assert vg.lib().vren_device_error(1) == 0


# ------------------------------------------------------------------------------------------------
# BVH
# ------------------------------------------------------------------------------------------------
def make_leaves(leaf_count: int, rng):
    P = vg.calc_bvh_padded_leaf_count(leaf_count)
    L = vg.calc_bvh_buffer_length(P)
    nodes = np.zeros((L, 8), np.uint32)
    f = nodes.view(np.float32)
    pos = rng.uniform(0, 100, (leaf_count, 3)).astype(np.float32)
    ext = rng.uniform(0, 100, (leaf_count, 3)).astype(np.float32)
    f[:leaf_count, 0:3] = pos - ext
    f[:leaf_count, 4:7] = pos + ext
    nodes[:leaf_count, 3] = 0xFFFFFFFF
    nodes[leaf_count:P, 3] = 0xFFFFFFFE
    return nodes, P


@pytest.mark.parametrize("leaf_count,queries", [(0, 16), (1, 16), (10, 16), (100, 8), (1000, 4), (10000, 2),
                                                (40000, 2), (1 << 20, 1)])
def test_build_bvh(cuda, leaf_count, queries):
    rng = np.random.default_rng(leaf_count + 1)
    nodes, P = make_leaves(leaf_count, rng)
    buf = torch.from_numpy(nodes.view(np.int32)).to(cuda)
    vg.build_bvh()(None, buf, P)
    got = host_u32(buf).reshape(-1, 8)
    expect = oracle.build_bvh(nodes, P)
    # invalid nodes: only next must agree (their AABB is +inf/-inf on both sides anyway)
    assert np.array_equal(got, expect)
    # the reference's own check: point queries vs a linear scan (vren_test/primitives/build_bvh.cpp:174-210)
    root = vg.calc_bvh_root_index(P)
    f = got.view(np.float32)
    for _ in range(queries):
        p = rng.uniform(0, 100, 3).astype(np.float32)
        lin = np.nonzero(np.all(p >= f[:leaf_count, 0:3], 1) & np.all(p <= f[:leaf_count, 4:7], 1))[0].tolist()
        assert sorted(oracle.bvh_point_query(got, root, p)) == lin


def test_build_bvh_bad_length(cuda):
    buf = torch.zeros(64 * 8, dtype=torch.int32, device=cuda)
    with pytest.raises(ValueError):
        vg.build_bvh()(None, buf, 64)


# ------------------------------------------------------------------------------------------------
# Tuning variants give identical results
# ------------------------------------------------------------------------------------------------
@pytest.fixture
def restore_tuning(native):
    saved = {k: native.vren_tuning_get(v) for k, v in vg._lib.TUNE.items()}
    yield native
    for k, v in saved.items():
        native.vren_tuning_set(vg._lib.TUNE[k], v)


@pytest.mark.parametrize("rank", [0, 1, 2])
@pytest.mark.parametrize("items", [0, 1])
@pytest.mark.parametrize("spin", [0, 64])
def test_radix_variants_identical(cuda, restore_tuning, rank, items, spin):
    lib = restore_tuning
    assert lib.vren_tuning_set(vg._lib.TUNE["radix_rank"], rank) == 0
    assert lib.vren_tuning_set(vg._lib.TUNE["radix_items"], items) == 0
    assert lib.vren_tuning_set(vg._lib.TUNE["spin_polls"], spin) == 0
    rng = np.random.default_rng(rank * 4 + items)
    n = (1 << 20) + 13
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    keys[::3] = keys[1::3][: len(keys[::3])]
    vals = np.arange(n, dtype=np.uint32)
    for bits in (8, 6, 4):
        rs = vg.radix_sort(bits)
        k, v = dev_u32(keys, cuda), dev_u32(vals, cuda)
        rs.sort(None, k, v, n, rs.create_scratch_buffer_1(n, cuda), torch.empty_like(k), torch.empty_like(v))
        ek, ev = oracle.stable_sort_u32(keys, vals)
        assert np.array_equal(host_u32(k), ek) and np.array_equal(host_u32(v), ev), bits
    pairs = np.stack([keys[:200000], vals[:200000]], 1).reshape(-1)
    for kb in (16, 10):
        bs = vg.bucket_sort(kb)
        out = torch.zeros(bs.get_required_output_buffer_size(200000) // 4, dtype=torch.int32, device=cuda)
        bs(None, dev_u32(pairs, cuda), 200000, 0, out, 0)
        ep, ee = oracle.bucket_sort_u32x2(pairs.reshape(-1, 2), kb)
        got = host_u32(out)
        assert np.array_equal(got[: 400000].reshape(-1, 2), ep)


@pytest.mark.parametrize("slices", [4, 8])
@pytest.mark.parametrize("spin", [0, 64, 4096])
@pytest.mark.parametrize("staged", [0, 1, 2, 3])
def test_scan_variants_identical(cuda, restore_tuning, slices, spin, staged):
    """Tiles in registers, tiles staged in shared memory by bulk copies (forced with staged=2,
    automatic from 2^20 elements with staged=0) and the persistent warp-specialised grid (staged=3)
    give the same sums: partial last tiles, aligned and unaligned segments, more tiles than resident
    CTAs, calls alternating between the forms on one scratch."""
    lib = restore_tuning
    assert lib.vren_tuning_set(vg._lib.TUNE["scan_slices"], slices) == 0
    assert lib.vren_tuning_set(vg._lib.TUNE["spin_polls"], spin) == 0
    assert lib.vren_tuning_set(vg._lib.TUNE["scan_staged"], staged) == 0
    rng = np.random.default_rng(slices + spin + 7 * staged)
    scan = vg.blelloch_scan()
    for n, blocks in ((1, 1), (8191, 1), (8193, 3), (8196, 3), (3 * 8192, 5), ((1 << 22) + 5, 1),
                      ((1 << 20) + 4, 3), (1 << 24, 1)):
        x = rng.integers(0, 256, n * blocks).astype(np.uint32)
        buf = dev_u32(x, cuda)
        scan(None, buf, n, 0, blocks)
        got = host_u32(buf).reshape(blocks, n)
        for b in range(blocks):
            assert np.array_equal(got[b], oracle.exclusive_scan_u32(x[b * n:(b + 1) * n]))


def test_tuning_rejects_unknown_values(native):
    assert native.vren_tuning_set(vg._lib.TUNE["scan_slices"], 5) == vg._lib.VREN_ERR_ARG
    assert native.vren_tuning_set(99, 1) == vg._lib.VREN_ERR_ARG
