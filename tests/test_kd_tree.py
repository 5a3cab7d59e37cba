"""k-d tree on the host (vren/vren/base/kd_tree.cpp): the library's build gives the oracle's node array
bit for bit (the reference's recursion restated literally), its search the oracle's results, and the
oracle's k-d search equals the linear search (the reference's own test, vren_test/kd_tree.cpp:29-112)."""
import numpy as np
import pytest

import oracle
from vren_gb300 import kd_tree as kd


def uniform(n, seed, lo=0.0, hi=100.0):
    return np.random.default_rng(seed).uniform(lo, hi, (n, 3)).astype(np.float32)


@pytest.mark.parametrize("n,max_leaf", [(1, 8), (8, 8), (9, 8), (100, 1), (1000, 8), (20000, 8), (5000, 32)])
def test_build_matches_oracle(native, n, max_leaf):
    pts = uniform(n, n + max_leaf)
    nodes, idx = kd.kd_tree_build(pts, 3, None, max_leaf)
    en, eidx = oracle.kd_tree_build(pts, 3, max_leaf)
    assert np.array_equal(nodes, en) and np.array_equal(idx, eidx)
    assert len(nodes) <= 2 * n


def test_build_degenerate_points(native):
    """Duplicates (where the reference's split separates nothing), NaN, a point stride of 4."""
    rng = np.random.default_rng(4)
    pts = np.zeros((3000, 4), np.float32)
    pts[:, :3] = rng.integers(0, 4, (3000, 3))          # many exact duplicates
    pts[::97, 1] = np.nan
    pts[:50, :3] = 7.0                                   # 50 identical points > max_leaf
    nodes, idx = kd.kd_tree_build(pts, 4, None, 8)
    en, eidx = oracle.kd_tree_build(pts, 4, 8)
    assert np.array_equal(nodes, en) and np.array_equal(idx, eidx)
    leaf_runs = nodes[(nodes[:, 1] == 3) & (nodes[:, 2] != 0x3FFFFFFF)]
    assert leaf_runs[:, 2].sum() == 3000 and leaf_runs[:, 2].max() >= 50
    assert kd.kd_tree_depth(nodes) >= 1


def test_reference_test_linear_vs_kd(native):
    """kd_tree.cpp test: 1M uniform points in [0, 100)^3, max 8 per leaf, 100 samples: the k-d search
    equals the linear search (point and squared distance)."""
    pts = uniform(1_000_000, 11)
    smp = uniform(100, 12)
    nodes, _ = kd.kd_tree_build(pts)
    lp, ld = oracle.linear_nn_search(pts, smp)
    kp, kdist = oracle.kd_tree_search(pts, nodes, smp)
    assert np.array_equal(lp, kp) and np.array_equal(ld.view(np.uint32), kdist.view(np.uint32))
    for q in range(0, 100, 9):
        p, dist = kd.kd_tree_search(pts, nodes, smp[q])
        assert p == lp[q] and np.float32(dist) == ld[q]


def test_host_search_filter_and_ties(native):
    """Integer grid points (many equal distances): the library's host search equals the oracle's
    recursion, ties included, with and without a filter."""
    rng = np.random.default_rng(5)
    pts = rng.integers(0, 20, (4000, 3)).astype(np.float32)
    smp = rng.integers(-2, 22, (300, 3)).astype(np.float32)
    nodes, _ = kd.kd_tree_build(pts)
    ex = (rng.uniform(0, 1, 4000) < 0.5).astype(np.uint8)
    ep, ed = oracle.kd_tree_search(pts, nodes, smp)
    fp, fd = oracle.kd_tree_search(pts, nodes, smp, excluded=ex)
    for q in range(300):
        assert kd.kd_tree_search(pts, nodes, smp[q]) == (int(ep[q]), float(ed[q]))
        assert kd.kd_tree_search(pts, nodes, smp[q], filter_predicate=lambda p: ex[p] == 0) == (int(fp[q]), float(fd[q]))
