"""CPU tests that pin the oracle to the reference's own known-answer tests (and to independent
numpy restatements where the reference test only checks properties)."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = json.loads((ROOT / "tests/golden/known_answers.json").read_text())


def test_bvh_size_helpers():
    kn = GOLDEN["bvh_size_helpers"]
    for n, v in kn["padded_leaf_count"].items():
        assert oracle.size_helpers(int(n))["padded"] == v
    for n, v in kn["buffer_length"].items():
        assert oracle.size_helpers(int(n))["length"] == v
    for n, v in kn["root_index"].items():
        assert oracle.size_helpers(int(n))["root"] == v
    for n, v in kn["level_count"].items():
        assert oracle.size_helpers(int(n))["levels"] == v


def test_scan_all_ones():
    lo, hi = GOLDEN["scan_all_ones"]["log2_lengths"]
    for e in range(lo, hi + 1):
        n = 1 << e
        out = oracle.exclusive_scan_u32(np.ones(n, np.uint32))
        assert np.array_equal(out, np.arange(n, dtype=np.uint32))


def numpy_tree(x: np.ndarray, op) -> np.ndarray:
    """Independent restatement: out[i] = op over x[i - 2^t + 1 .. i], t = trailing ones of i."""
    P = 1
    while P < len(x):
        P *= 2
    out = np.empty(P, dtype=x.dtype)
    for i in range(P):
        t = 0
        while (i >> t) & 1 and (1 << (t + 1)) <= P:
            t += 1
        lo = i - (1 << t) + 1
        out[i] = op(x[lo:i + 1])
    return out


@pytest.mark.parametrize("n", [1, 2, 5, 10, 100, 1000])
def test_reduce_tree_restatements(n):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 100, n).astype(np.uint32)
    P = 1
    while P < n:
        P *= 2
    pad = lambda fill: np.concatenate([x, np.full(P - n, fill, np.uint32)])
    assert np.array_equal(oracle.reduce_tree_u32("add", x), numpy_tree(pad(0), lambda s: np.uint32(s.sum(dtype=np.uint64) & 0xFFFFFFFF)))
    assert np.array_equal(oracle.reduce_tree_u32("min", x), numpy_tree(pad(0xFFFFFFFF), np.min))
    assert np.array_equal(oracle.reduce_tree_u32("max", x), numpy_tree(pad(0), np.max))


def test_reduce_all_ones_totals():
    for n in GOLDEN["reduce"]["lengths_add_ones"]:
        t = oracle.reduce_tree_u32("add", np.ones(n, np.uint32))
        assert t[-1] == n


def test_downsweep_of_upsweep_is_exclusive_scan():
    rng = np.random.default_rng(3)
    for e in range(0, 15):
        n = 1 << e
        x = rng.integers(0, 1 << 20, n).astype(np.uint32)
        tree = oracle.reduce_tree_u32("add", x)
        expect = oracle.exclusive_scan_u32(x)
        assert np.array_equal(oracle.downsweep_u32(tree, True), expect)
        kept = oracle.downsweep_u32(tree, False)
        if n >= 1024:  # the root value is added to every element
            assert np.array_equal(kept, expect + tree[-1])
        else:  # a single work-group always propagates zero into the root
            assert np.array_equal(kept, expect)


def test_stable_sort():
    rng = np.random.default_rng(5)
    keys = rng.integers(0, 1000, 5000).astype(np.uint32)
    vals = np.arange(5000, dtype=np.uint32)
    k, v = oracle.stable_sort_u32(keys, vals)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, vals[order])
    n = GOLDEN["radix_reversed_iota"]["length"]
    assert np.array_equal(oracle.stable_sort_u32(np.arange(n, dtype=np.uint32)[::-1].copy()), np.arange(n))


@pytest.mark.parametrize("key_bits", [16, 10])
def test_bucket_sort(key_bits):
    rng = np.random.default_rng(key_bits)
    n = 20000
    pairs = np.stack([rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32), np.arange(n, dtype=np.uint32)], 1)
    out, ends = oracle.bucket_sort_u32x2(pairs, key_bits)
    mask = (1 << key_bits) - 1
    order = np.argsort(pairs[:, 0] & mask, kind="stable")
    assert np.array_equal(out, pairs[order])
    assert np.array_equal(ends, np.cumsum(np.bincount(pairs[:, 0] & mask, minlength=1 << key_bits)).astype(np.uint32))


def make_leaves(leaf_count: int, rng) -> np.ndarray:
    """The reference test's leaves (vren_test/primitives/build_bvh.cpp:114-130): pos, ext uniform [0, 100)."""
    P = oracle.size_helpers(leaf_count)["padded"]
    L = oracle.size_helpers(P)["length"]
    nodes = np.zeros((L, 8), np.uint32)
    f = nodes.view(np.float32)
    pos = rng.uniform(0, 100, (leaf_count, 3)).astype(np.float32)
    ext = rng.uniform(0, 100, (leaf_count, 3)).astype(np.float32)
    f[:leaf_count, 0:3] = pos - ext
    f[:leaf_count, 4:7] = pos + ext
    nodes[:leaf_count, 3] = 0xFFFFFFFF
    nodes[leaf_count:P, 3] = 0xFFFFFFFE
    return nodes, P


def test_bvh_point_queries_match_linear_scan():
    rng = np.random.default_rng(11)
    for leaf_count, queries in GOLDEN["bvh_build_leaf_counts"]["cases"]:
        nodes, P = make_leaves(leaf_count, rng)
        built = oracle.build_bvh(nodes, P)
        root = oracle.size_helpers(P)["root"]
        f = built.view(np.float32)
        for _ in range(queries):
            p = rng.uniform(0, 100, 3).astype(np.float32)
            lin = [i for i in range(leaf_count) if np.all(p >= f[i, 0:3]) and np.all(p <= f[i, 4:7])]
            got = sorted(oracle.bvh_point_query(built, root, p))
            assert got == lin


def test_depth_pyramid_level_counts():
    """depth_buffer_pyramid.cpp:18: glm::log2 of an unsigned integer (glm/gtc/integer.hpp) is the
    floor of log2, so the level count is floor(log2(max(w, h))) + 1."""
    for (w, h), n in {(1, 1): 1, (2, 1): 2, (1, 3): 2, (4, 4): 3, (5, 7): 3, (1920, 1080): 11,
                      (2560, 1440): 12, (3840, 2160): 12, (4096, 1): 13, (65535, 3): 16}.items():
        assert oracle.depth_pyramid_level_count(w, h) == n


def _pyramid_closed_form(d0, w, h):
    """Each level-l texel is max(+0, the non-NaN values of its level-0 block): the block is 2^l wide
    on an axis until that axis reaches size 1 (at level floor(log2(size))), then stays at that width
    (the odd last row or column of a level is never read)."""
    pos = np.where(d0 > 0, d0, np.float32(0.0)).astype(np.float32)   # NaN, -0 and negatives -> +0
    kx, ky = int(w).bit_length() - 1, int(h).bit_length() - 1
    out = [d0]
    for l in range(1, oracle.depth_pyramid_level_count(w, h)):
        wl, hl = max(w >> l, 1), max(h >> l, 1)
        bx, by = 1 << min(l, kx), 1 << min(l, ky)
        out.append(pos[:hl * by, :wl * bx].reshape(hl, by, wl, bx).max(axis=(1, 3)))
    return out


@pytest.mark.parametrize("w,h", [(1, 1), (1, 9), (9, 1), (2, 2), (3, 5), (37, 64), (64, 64), (65, 127),
                                 (128, 1), (200, 77), (333, 257), (1023, 17)])
def test_depth_pyramid_restatement_against_closed_form(w, h):
    rng = np.random.default_rng(w * 1000 + h)
    d = rng.uniform(-0.2, 1.0, (h, w)).astype(np.float32)
    flat = d.reshape(-1)
    flat[rng.integers(0, flat.size, max(flat.size // 50, 1))] = np.nan
    flat[rng.integers(0, flat.size, max(flat.size // 60, 1))] = -0.0
    flat[rng.integers(0, flat.size, max(flat.size // 500, 1))] = np.inf
    got = oracle.depth_pyramid(d, w, h)
    want = _pyramid_closed_form(d, w, h)
    assert len(got) == len(want)
    assert np.array_equal(got[0].view(np.uint32), d.view(np.uint32))    # exact copy, NaN payloads kept
    for g, e in zip(got[1:], want[1:]):
        assert g.shape == e.shape and np.array_equal(g.view(np.uint32), e.view(np.uint32))
