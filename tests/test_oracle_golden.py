"""The CPU oracle against the golden fixtures made from the reference itself.

The fixtures (tests/golden/make_golden.py) hold clustkit's own outputs: its C
Smith-Waterman compiled from source, its Numba kernels run as Python, its
BLOSUM62 table.  Passing here pins the oracle that every GPU parity test uses.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from clustkit_gb300.blosum import BLOSUM62


def test_blosum62_matches_reference(golden):
    ref = np.load(Path(__file__).parent / "golden" / "blosum62_ref.npy")
    assert ref.shape == (20, 20)
    assert np.array_equal(ref, BLOSUM62)
    # the reference table is not symmetric in one cell; keep it that way
    assert not np.array_equal(BLOSUM62, BLOSUM62.T)


@pytest.mark.parametrize("bw", [0, 1, 2, 3, 8, 16, 32, 50, 64, 100, 128, 1000])
def test_oracle_sw_matches_reference_c(golden, bw):
    g = golden("sw_golden.npz")
    r = oracle.sw_batch(g["pairs"], g["flat"], g["offsets"], g["lengths"], bw, BLOSUM62)
    assert np.array_equal(r["scores"], g[f"bw{bw}_scores"])
    assert np.array_equal(r["sims"].view(np.uint32), g[f"bw{bw}_sims"].view(np.uint32))
    assert np.array_equal(r["mask"], g[f"bw{bw}_mask"])
    # identity is matches / shorter exactly
    pos = r["scores"] > 0
    sh = r["shorter"][pos].astype(np.float32)
    assert np.array_equal(r["sims"][pos], r["matches"][pos].astype(np.float32) / sh)


@pytest.mark.parametrize("bw", [8, 32, 100])
def test_oracle_sw_diagonal_hints(golden, bw):
    g = golden("sw_golden.npz")
    r = oracle.sw_batch(g["pairs"], g["flat"], g["offsets"], g["lengths"], bw, BLOSUM62,
                        diag_hints=g["hints"])
    assert np.array_equal(r["scores"], g[f"hint_bw{bw}_scores"])
    assert np.array_equal(r["sims"], g[f"hint_bw{bw}_sims"])


def test_oracle_sw_matches_numba_twin(golden):
    g = golden("sw_golden.npz")
    idx = g["twin_idx"]
    r = oracle.sw_batch(g["pairs"][idx], g["flat"], g["offsets"], g["lengths"], int(g["twin_bw"]),
                        BLOSUM62)
    assert np.array_equal(r["scores"], g["twin_scores"])
    assert np.array_equal(r["sims"], g["twin_sims"])
    assert np.array_equal(r["scores"] > 0, g["twin_mask"])


def test_oracle_sketches_match_reference(golden):
    g = golden("sketch_golden.npz")
    for k, s, a in g["cases"]:
        out = oracle.sketches(g["flat"], g["offsets"], g["lengths"], k, s, a)
        assert np.array_equal(out, g[f"k{k}_s{s}_a{a}"]), (k, s, a)
    out = oracle.sketches(g["nuc_flat"], g["nuc_offsets"], g["nuc_lengths"], 11, 16, 4)
    assert np.array_equal(out, g["nuc_k11_s16"])


def test_oracle_sketch_edge_semantics(golden):
    g = golden("sketch_golden.npz")
    sk = g["k5_s128_a20"]
    L = g["lengths"]
    assert np.all(sk[L < 5] == 0)                       # shorter than k -> zeros
    few = (L >= 5) & (L - 5 + 1 < 128)
    assert np.all(sk[few, -1] == np.iinfo(np.uint64).max)  # padding
    assert np.all(sk[:, 1:] >= sk[:, :-1])                # sorted


def test_oracle_fmix_known_values():
    # fmix64(0 ^ 42) and a chained value computed with Python integers
    def fmix(x):
        m = (1 << 64) - 1
        x ^= x >> 33
        x = (x * 0xFF51AFD7ED558CCD) & m
        x ^= x >> 33
        x = (x * 0xC4CEB9FE1A85EC53) & m
        x ^= x >> 33
        return x
    for key in (0, 1, 12345, 3199999, 2**63 + 5):
        assert oracle.fmix64(key, 42) == fmix(key ^ 42)


def test_oracle_jaccard_matches_reference(golden):
    g = golden("jaccard_golden.npz")
    assert np.array_equal(oracle.jaccard(g["pairs"], g["sketches"]), g["sims"])
    assert np.array_equal(oracle.jaccard(g["hand_pairs"], g["hand_sketches"]), g["hand_sims"])


def test_oracle_reference_tests_known_answers():
    # the values clustkit's own tests pin (tests/test_pairwise.py:14-34)
    a = np.array([1, 2, 3, 4, 5], np.uint64)
    b = np.array([6, 7, 8, 9, 10], np.uint64)
    sk = np.stack([a, a, b])
    j = oracle.jaccard(np.array([[0, 1], [0, 2]], np.int32), sk)
    assert j[0] == 1.0 and j[1] == 0.0


@pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not mounted")
def test_oracle_matches_compiled_reference_random():
    from clustkit_gb300 import synth
    s = synth.generate_families(15, 8, median=250, lo=20, hi=700, seed=5)
    pairs = synth.mixed_pairs(s, 3000, seed=3)
    for bw in (0, 10, 48, 100):
        a = oracle.sw_batch(pairs, s.flat, s.offsets, s.lengths, bw, BLOSUM62)
        r = oracle.ref_sw_batch(pairs, s.flat, s.offsets, s.lengths, bw, BLOSUM62, n_threads=4)
        assert np.array_equal(a["scores"], r["scores"])
        assert np.array_equal(a["sims"], r["sims"])
