"""Device LSH (csrc/lsh.cu) against the reference's lsh_candidates golden
vectors and the host restatement."""
import numpy as np
import pytest

from clustkit_gb300 import synth
from clustkit_gb300.lsh import auto_lsh_params, lsh_candidates, lsh_candidates_device
from clustkit_gb300.sketch import compute_sketches

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tables,bands,seed,key", [(32, 2, 42, "pairs_t32_b2"), (16, 1, 7, "pairs_t16_b1")])
def test_device_lsh_matches_reference_golden(ck, golden, tables, bands, seed, key):
    g = golden("lsh_golden.npz")
    got = lsh_candidates_device(g["sketches"], tables, bands, seed).cpu().numpy()
    assert np.array_equal(got, g[key].astype(np.int32))


def test_device_lsh_config1_pairs(ck, golden):
    """The 2,000-sequence pipeline golden: its LSH candidate list, from the
    reference, on the reference's own sketches."""
    g = golden("pipeline_golden.npz")
    got = lsh_candidates_device(g["sketches"], int(g["num_tables"]), int(g["num_bands"]), 42).cpu().numpy()
    assert np.array_equal(got, g["candidates"].astype(np.int32))


@pytest.mark.parametrize("t,sens", [(0.3, "high"), (0.4, "medium"), (0.7, "low")])
def test_device_lsh_matches_host_on_families(ck, t, sens):
    s = synth.generate_families(400, 10, median=300, lo=30, hi=1500, seed=int(t * 10))
    sk = compute_sketches(None, s.lengths, 5, 128, "protein", flat_sequences=s.flat, offsets=s.offsets)
    lp = auto_lsh_params(t, sens, 5)
    host = lsh_candidates(sk, lp["num_tables"], lp["num_bands"], 42)
    dev = lsh_candidates_device(sk, lp["num_tables"], lp["num_bands"], 42).cpu().numpy()
    assert np.array_equal(dev, host)


def test_device_lsh_large_bucket_keeps_lowest_ids(ck):
    """A bucket above 1000 members: the 1000 lowest ids make all its pairs."""
    n, s = 1500, 16
    sk = np.arange(n * s, dtype=np.uint64).reshape(n, s) * np.uint64(7919) + np.uint64(11)
    sk[:1200, 3] = np.uint64(5)  # 1200 sequences share sketch slot 3
    from clustkit_gb300.lsh import band_parameters
    idx, _ = band_parameters(s, 1, 1, 1)
    assert int(idx[0, 0]) == 3  # seed 1 draws slot 3 for the one table
    got = lsh_candidates_device(sk, 1, 1, 1).cpu().numpy()
    a, b = np.triu_indices(1000, 1)
    assert np.array_equal(got, np.stack([a, b], 1).astype(np.int32))


def test_device_lsh_edges(ck):
    assert lsh_candidates_device(np.zeros((1, 8), np.uint64), 4, 1).shape == (0, 2)
    same = np.tile(np.arange(8, dtype=np.uint64), (5, 1))
    got = lsh_candidates_device(same, 3, 2).cpu().numpy()
    a, b = np.triu_indices(5, 1)
    assert np.array_equal(got, np.stack([a, b], 1).astype(np.int32))
