"""End-to-end drop-in parity: the reference's compute_pairwise_alignment output
(recorded in tests/golden/pipeline_golden.npz on a 2,000-sequence, 200-family
set: k=5, s=128 sketches, LSH at t=0.5 medium sensitivity, band width 100,
C Smith-Waterman path) reproduced pair for pair by this library."""
import numpy as np
import pytest

from clustkit_gb300.pairwise import compute_pairwise_alignment
from clustkit_gb300.sketch import sketch_flat

pytestmark = pytest.mark.gpu


def test_sketches_reproduce_reference_pipeline(ck, golden):
    g = golden("pipeline_golden.npz")
    sk = sketch_flat(g["flat"], g["offsets"], g["lengths"], 5, 128)
    assert np.array_equal(sk, g["sketches"])


@pytest.mark.parametrize("t,tag", [(0.5, "0p5"), (0.3, "0p3")])
def test_compute_pairwise_alignment_matches_reference(ck, golden, t, tag):
    g = golden("pipeline_golden.npz")
    fp, fs = compute_pairwise_alignment(
        g["candidates"], None, g["lengths"], t, band_width=100, device="cpu", sketches=g["sketches"],
        flat_sequences=g["flat"], offsets=g["offsets"], use_sw=True, use_c_sw=True)
    assert np.array_equal(fp, g[f"t{tag}_pairs"])
    assert np.array_equal(fs.view(np.uint32), g[f"t{tag}_sims"].view(np.uint32))


def test_connected_components_identical(ck, golden):
    """Downstream graph + connected components (clustkit/graph.py:7-39,
    clustkit/cluster.py:43-55) give identical clusters from both edge lists."""
    sp = pytest.importorskip("scipy.sparse")
    from scipy.sparse.csgraph import connected_components
    g = golden("pipeline_golden.npz")
    fp, fs = compute_pairwise_alignment(
        g["candidates"], None, g["lengths"], 0.5, band_width=100, device="cpu",
        sketches=g["sketches"], flat_sequences=g["flat"], offsets=g["offsets"], use_sw=True,
        use_c_sw=True)
    n = len(g["lengths"])

    def labels(p, w):
        a = sp.coo_matrix((w, (p[:, 0], p[:, 1])), shape=(n, n))
        return connected_components(a + a.T, directed=False)[1]

    assert np.array_equal(labels(fp, fs), labels(g["t0p5_pairs"], g["t0p5_sims"]))


@pytest.mark.parametrize("t,tag", [(0.5, "0p5"), (0.3, "0p3")])
def test_whole_chain_on_device_matches_reference(ck, golden, t, tag):
    """Sketches, LSH, Jaccard pre-filter, SW, similarity graph and connected
    components, every stage on the GPU from the sequences alone, against the
    reference pipeline's recorded candidates and passing pairs and the clusters
    scipy gives for them (clustkit/pipeline.py:600-700's order of stages)."""
    import oracle.graph_oracle as go
    from clustkit_gb300 import graph
    from clustkit_gb300.lsh import lsh_candidates_device
    g = golden("pipeline_golden.npz")
    n = len(g["lengths"])
    sk = sketch_flat(g["flat"], g["offsets"], g["lengths"], 5, 128)
    cand = lsh_candidates_device(sk, int(g["num_tables"]), int(g["num_bands"]), 42).cpu().numpy()
    assert np.array_equal(cand, g["candidates"].astype(np.int32))
    fp, fs = compute_pairwise_alignment(
        cand, None, g["lengths"], t, band_width=100, device="cpu", sketches=sk,
        flat_sequences=g["flat"], offsets=g["offsets"], use_sw=True, use_c_sw=True)
    assert np.array_equal(fp, g[f"t{tag}_pairs"])
    gr = graph.build_similarity_graph(n, fp, fs)
    labels = graph.cluster_connected_components(gr)
    ref = go.cluster_connected_components(go.build_similarity_graph(n, g[f"t{tag}_pairs"], g[f"t{tag}_sims"]))
    assert np.array_equal(labels, ref)
