"""Device similarity graph (CSR) and connected components against the scipy
restatement of clustkit/graph.py:7-39 and clustkit/cluster.py:43-55."""
import numpy as np
import pytest

import oracle.graph_oracle as go
from clustkit_gb300 import graph

pytestmark = pytest.mark.gpu


def _canon(m):
    m = m.tocsr()
    m.sum_duplicates()
    m.sort_indices()
    return m


def _same_csr(a, b):
    a, b = _canon(a), _canon(b)
    assert a.shape == b.shape
    assert np.array_equal(a.indptr.astype(np.int64), b.indptr.astype(np.int64))
    assert np.array_equal(a.indices.astype(np.int32), b.indices.astype(np.int32))
    assert np.array_equal(a.data.astype(np.float32), b.data.astype(np.float32))


@pytest.mark.parametrize("t", ["t0p5", "t0p3"])
def test_graph_and_components_on_pipeline_golden(ck, golden, t):
    g = golden("pipeline_golden.npz")
    pairs, sims, n = g[f"{t}_pairs"].astype(np.int32), g[f"{t}_sims"].astype(np.float32), len(g["lengths"])
    got = graph.build_similarity_graph(n, pairs, sims)
    ref = go.build_similarity_graph(n, pairs, sims)
    _same_csr(got, ref)
    assert np.array_equal(graph.cluster_connected_components(got), go.cluster_connected_components(ref))


def test_graph_duplicates_and_self_loops(ck):
    rng = np.random.default_rng(1)
    n = 3000
    base = np.unique(np.sort(rng.integers(0, n, size=(20000, 2)), 1), axis=0).astype(np.int32)
    base = base[base[:, 0] != base[:, 1]]
    sims = rng.random(len(base)).astype(np.float32)
    dup = base[:500]                       # repeated pairs: each entry summed from two copies
    rev = base[500:1000][:, ::-1].copy()   # reversed pairs: (j, i) on top of (i, j)
    loops = np.stack([np.arange(10), np.arange(10)], 1).astype(np.int32) * 7
    pairs = np.concatenate([base, dup, rev, loops]).astype(np.int32)
    w = np.concatenate([sims, rng.random(500).astype(np.float32), rng.random(500).astype(np.float32),
                        rng.random(10).astype(np.float32)])
    _same_csr(graph.build_similarity_graph(n, pairs, w), go.build_similarity_graph(n, pairs, w))


@pytest.mark.parametrize("kind", ["random_sparse", "random_dense", "path_shuffled", "star", "isolated", "empty",
                                  "one_node", "many_small"])
def test_components_match_scipy(ck, kind):
    rng = np.random.default_rng(7)
    if kind == "random_sparse":
        n = 200000
        pairs = rng.integers(0, n, size=(120000, 2))
    elif kind == "random_dense":
        n = 5000
        pairs = rng.integers(0, n, size=(200000, 2))
    elif kind == "path_shuffled":
        n = 300000
        perm = rng.permutation(n)
        pairs = np.stack([perm[:-1], perm[1:]], 1)
    elif kind == "star":
        n = 50000
        pairs = np.stack([np.full(n - 1, n - 1), np.arange(n - 1)], 1)
    elif kind == "isolated":
        n = 1000
        pairs = np.array([[5, 9], [9, 700]])
    elif kind == "empty":
        n = 50
        pairs = np.zeros((0, 2), np.int64)
    elif kind == "one_node":
        n = 1
        pairs = np.array([[0, 0]])
    else:
        n = 100000
        a = rng.integers(0, n, 60000)
        pairs = np.stack([a, np.minimum(a + rng.integers(1, 4, a.size), n - 1)], 1)
    pairs = pairs.astype(np.int32)
    ref = go.cluster_connected_components(go.build_similarity_graph(n, pairs, np.ones(len(pairs), np.float32)))
    k, labels, rounds = graph.connected_components_device(pairs, n)
    assert np.array_equal(labels.cpu().numpy(), ref)
    assert k == (int(ref.max()) + 1 if n else 0)
    assert rounds <= 64
