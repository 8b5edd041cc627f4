"""bench.py's parity helpers on CPU: the comparison every GPU output of a bench
run goes through, against the oracle on the same pairs.  Mistakes are planted
in a copy of the oracle's own outputs."""
import numpy as np

import bench
import oracle
from clustkit_gb300 import synth
from clustkit_gb300.blosum import BLOSUM62


def _workload():
    s = synth.generate_families(6, 5, median=120, lo=30, hi=300, seed=3)
    return s, synth.mixed_pairs(s, 300, seed=4)


def test_same_as_oracle_accepts_equal_and_flags_each_field():
    s, pairs = _workload()
    ref = oracle.sw_batch(pairs, s.flat, s.offsets, s.lengths, 100, BLOSUM62)
    res = {k: v.copy() for k, v in ref.items()}
    res["mask"] = (ref["sims"] >= np.float32(0.3)).astype(np.uint8)
    assert bench.same_as_oracle(res, ref, 0.3)
    for key in ("scores", "matches", "shorter"):
        bad = {k: v.copy() for k, v in res.items()}
        bad[key][7] += 1
        assert not bench.same_as_oracle(bad, ref, 0.3), key
    bad = {k: v.copy() for k, v in res.items()}
    bad["sims"][11] = np.nextafter(bad["sims"][11], np.float32(2))  # one ulp
    assert not bench.same_as_oracle(bad, ref)
    bad = {k: v.copy() for k, v in res.items()}
    bad["mask"][5] ^= 1
    assert bench.same_as_oracle(bad, ref) and not bench.same_as_oracle(bad, ref, 0.3)


def test_oracle_on_sample_indexes_the_full_result_arrays():
    s, pairs = _workload()
    full = oracle.sw_batch(pairs, s.flat, s.offsets, s.lengths, 32, BLOSUM62)
    chk, idx, ref = bench.oracle_on_sample(s, pairs, 32, 100, 9, full)
    assert chk["bit_exact"] and chk["pairs"] == 100 == len(idx) and np.all(np.diff(idx) > 0)
    assert np.array_equal(ref["scores"], full["scores"][idx])
    planted = {k: v.copy() for k, v in full.items()}
    planted["matches"][idx[50]] += 1
    assert not bench.oracle_on_sample(s, pairs, 32, 100, 9, planted)[0]["bit_exact"]
