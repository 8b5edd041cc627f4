"""GPU sketches and Jaccard against the reference's outputs and the oracle (bit-exact)."""
import numpy as np
import pytest

import oracle
from clustkit_gb300 import synth
from clustkit_gb300.pairwise import _jaccard_prefilter, batch_jaccard, compute_pairwise_jaccard, \
    jaccard_from_sketches
from clustkit_gb300.sketch import compute_sketches, sketch_flat, sketch_sequence

pytestmark = pytest.mark.gpu


def test_sketch_golden(ck, golden):
    g = golden("sketch_golden.npz")
    for k, s, a in g["cases"]:
        out = sketch_flat(g["flat"], g["offsets"], g["lengths"], k, s, a)
        assert np.array_equal(out, g[f"k{k}_s{s}_a{a}"]), (k, s, a)
    out = sketch_flat(g["nuc_flat"], g["nuc_offsets"], g["nuc_lengths"], 11, 16, 4)
    assert np.array_equal(out, g["nuc_k11_s16"])


@pytest.mark.parametrize("k,s", [(5, 128), (3, 32), (7, 1), (5, 1000), (12, 64)])
def test_sketch_vs_oracle(ck, k, s):
    ss = synth.generate_families(40, 5, median=400, lo=1, hi=3000, seed=k * 7 + s,
                                 length_dist="pareto")
    out = sketch_flat(ss.flat, ss.offsets, ss.lengths, k, s)
    assert np.array_equal(out, oracle.sketches(ss.flat, ss.offsets, ss.lengths, k, s))


def test_sketch_api_shapes(ck):
    seq = np.array([0, 1, 2, 3, 4, 0, 1, 2, 3, 4], np.uint8)
    sk = sketch_sequence(seq, len(seq), k=3, sketch_size=4, alphabet_size=20)
    assert sk.dtype == np.uint64 and len(sk) == 4 and np.all(sk[:-1] <= sk[1:])
    assert np.all(sketch_sequence(np.array([0, 1], np.uint8), 2, 5, 4, 20) == 0)
    sk = sketch_sequence(np.array([0, 1, 2, 3, 4], np.uint8), 5, 3, 8, 20)
    assert sk[-1] == np.iinfo(np.uint64).max
    pad = np.full((2, 10), 20, np.uint8)
    pad[0, :6] = [1, 2, 3, 4, 5, 6]
    pad[1, :10] = np.arange(10)
    out = compute_sketches(pad, np.array([6, 10], np.int32), 5, 16, "protein")
    ref = oracle.sketches(np.concatenate([pad[0, :6], pad[1]]), np.array([0, 6]),
                          np.array([6, 10]), 5, 16)
    assert np.array_equal(out, ref)


def test_jaccard_golden(ck, golden):
    g = golden("jaccard_golden.npz")
    sims, _ = batch_jaccard(g["pairs"], g["sketches"])
    assert np.array_equal(sims, g["sims"])
    sims, _ = batch_jaccard(g["hand_pairs"], g["hand_sketches"])
    assert np.array_equal(sims, g["hand_sims"])


def test_jaccard_random_vs_oracle(ck):
    ss = synth.generate_families(100, 10, median=300, lo=20, hi=900, seed=77)
    sk = sketch_flat(ss.flat, ss.offsets, ss.lengths, 5, 128)
    # low-complexity rows with heavy duplication inside one sketch
    sk[:20] = np.sort(np.random.default_rng(0).integers(0, 40, size=(20, 128)).astype(np.uint64), 1)
    pairs = synth.mixed_pairs(ss, 30000, seed=1)
    sims, mask = batch_jaccard(pairs, sk, 0.01)
    ref = oracle.jaccard(pairs, sk)
    assert np.array_equal(sims, ref)
    assert np.array_equal(mask, ref >= np.float32(0.01))


def test_jaccard_reference_known_answers(ck):
    a = np.array([1, 2, 3, 4, 5], np.uint64)
    assert jaccard_from_sketches(a, a) == 1.0
    assert jaccard_from_sketches(a, np.array([6, 7, 8, 9, 10], np.uint64)) == 0.0
    mx = np.iinfo(np.uint64).max
    s = jaccard_from_sketches(np.array([1, 2, 3, mx, mx], np.uint64), np.array([1, 2, 4, mx, mx], np.uint64))
    assert 0.0 < s < 1.0
    sk = np.array([[1, 2, 3, 4, 5], [1, 2, 3, 4, 5], [6, 7, 8, 9, 10]], np.uint64)
    fp, fs = compute_pairwise_jaccard(np.array([[0, 1], [0, 2]], np.int32), sk, 0.5)
    assert fp.tolist() == [[0, 1]] and fs.tolist() == [1.0]


def test_prefilter_golden(ck, golden):
    g = golden("pipeline_golden.npz")
    for t, tag in ((0.5, "0p5"), (0.3, "0p3")):
        m = _jaccard_prefilter(g["candidates"], g["sketches"], t)
        if bool(g[f"t{tag}_jskipped"]):
            assert m is None
        else:
            assert np.array_equal(m, g[f"t{tag}_jmask"])


@pytest.mark.parametrize("s", [32, 64, 96, 128, 200, 256])
def test_jaccard_sizes_duplicates_padding_vs_oracle(ck, s):
    """Both Jaccard kernels (chunked for s a multiple of 32 up to 256, general
    otherwise) on sketches with duplicate runs, MAX padding and shared parts."""
    rng = np.random.default_rng(s)
    mx = np.uint64(np.iinfo(np.uint64).max)
    rows = []
    for r in range(300):
        hi = [20, 300, 10 ** 6, 2 ** 62][r % 4]
        n_real = int(rng.integers(0, s + 1))
        x = np.sort(rng.integers(0, hi, n_real).astype(np.uint64))
        rows.append(np.concatenate([x, np.full(s - n_real, mx, np.uint64)]))
    sk = np.stack(rows)
    sk[150:] = np.sort(np.where(rng.random((150, s)) < 0.5, sk[:150], sk[150:]), 1)
    pairs = rng.integers(0, 300, size=(20000, 2)).astype(np.int32)
    pairs[:300, 1] = (pairs[:300, 0] + 150) % 300
    sims, _ = batch_jaccard(pairs, sk)
    assert np.array_equal(sims, oracle.jaccard(pairs, sk))
