"""GPU: batched nearest-neighbour search over vren's k-d tree against the oracle's recursive search,
bit for bit (points, squared distances, ties, the filter), on the reference test's workload and larger."""
import numpy as np
import pytest
import torch

import oracle
import vren_gb300 as vg
from vren_gb300 import kd_tree as kd

pytestmark = pytest.mark.gpu


def run(cuda, pts, nodes, smp, stride=3, excluded=None):
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dt).reshape(-1)).to(cuda)
    bp, bd = kd.kd_tree_search_batch(None, t(pts, np.float32), t(nodes.view(np.int32), np.int32),
                                     t(smp, np.float32), kd.kd_tree_depth(nodes), point_stride=stride,
                                     excluded=None if excluded is None else t(excluded, np.uint8))
    torch.cuda.synchronize()
    return bp.cpu().numpy().view(np.uint32), bd.cpu().numpy()


@pytest.mark.parametrize("n,q,max_leaf", [(1, 10, 8), (9, 100, 8), (1000, 5000, 8), (1_000_000, 100, 8),
                                          (1_000_000, 200_000, 8), (300_000, 50_000, 1), (100_000, 10_000, 64)])
def test_batch_matches_oracle(cuda, n, q, max_leaf):
    rng = np.random.default_rng(n + q)
    pts = rng.uniform(0, 100, (n, 3)).astype(np.float32)
    smp = rng.uniform(-5, 105, (q, 3)).astype(np.float32)
    nodes, _ = kd.kd_tree_build(pts, 3, None, max_leaf)
    gp, gd = run(cuda, pts, nodes, smp)
    ep, ed = oracle.kd_tree_search(pts, nodes, smp)
    assert np.array_equal(gp, ep) and np.array_equal(gd.view(np.uint32), ed.view(np.uint32))
    assert vg.device_error() == 0


def test_batch_ties_filter_and_stride(cuda):
    rng = np.random.default_rng(6)
    pts = np.zeros((50_000, 4), np.float32)
    pts[:, :3] = rng.integers(0, 30, (50_000, 3))
    pts[:100, :3] = 3.0
    smp = rng.integers(-3, 33, (20_000, 3)).astype(np.float32)
    nodes, _ = kd.kd_tree_build(pts, 4, None, 8)
    ex = (rng.uniform(0, 1, 50_000) < 0.3).astype(np.uint8)
    for excluded in (None, ex):
        gp, gd = run(cuda, pts, nodes, smp, 4, excluded)
        ep, ed = oracle.kd_tree_search(pts, nodes, smp, stride=4, excluded=excluded)
        assert np.array_equal(gp, ep) and np.array_equal(gd.view(np.uint32), ed.view(np.uint32))
    all_ex = np.ones(50_000, np.uint8)
    gp, gd = run(cuda, pts, nodes, smp[:10], 4, all_ex)
    assert (gp == 0xFFFFFFFF).all() and np.isinf(gd).all()


def test_batch_arguments(cuda):
    pts = np.random.default_rng(1).uniform(0, 1, (100, 3)).astype(np.float32)
    nodes, _ = kd.kd_tree_build(pts)
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dt).reshape(-1)).to(cuda)
    with pytest.raises(vg.VrenError):
        kd.kd_tree_search_batch(None, t(pts, np.float32), t(nodes.view(np.int32), np.int32), t(pts, np.float32), 129)
    with pytest.raises(ValueError):
        kd.kd_tree_search_batch(None, t(pts, np.float32), t(nodes.view(np.int32), np.int32), t(pts, np.float32), 8,
                                point_stride=2)
