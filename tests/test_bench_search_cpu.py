"""Host-side pieces of bench.py's search leg, on CPU: the similar-k-mer chain
timed on the host cores (scorer restatement -> oracle SW -> rank) gives the
same candidates as the numpy restatement, and the per-mode summary carries
the host-core ratio only where a baseline was measured."""
import numpy as np

from oracle import search_oracle as so
from clustkit_gb300 import synth
from clustkit_gb300.blosum import BLOSUM62


def test_similar_chain_runs_and_matches_restatement():
    import bench
    import oracle
    s = synth.generate_families(60, 5, median=150, lo=40, hi=300, seed=31)
    off, ent, fr = so.build_kmer_index(s.flat, s.offsets, s.lengths, 5)
    ft = int(fr.max())
    qs = [s.seq(i).copy() for i in (0, 7, 55)]
    tot, ts, tsw, trank, npairs = bench._similar_chain(off, ent, fr, ft, s, qs, 40, max_cands=50)
    assert tot >= ts + tsw and npairs > 0
    lens = np.array([len(q) for q in qs], np.int32)
    got = oracle.similar_candidates_batch(np.concatenate(qs), np.concatenate([[0], np.cumsum(lens[:-1])]), lens,
                                          BLOSUM62, 13, off, ent, fr, ft, s.n, 2, 50)
    assert npairs == sum(len(c[0]) for c in got)
    for q, (ids, sc) in zip(qs, got):
        want = so.phase_a_similar(q, off, ent, fr, ft, s.n, 2, 50, BLOSUM62, 13)
        assert np.array_equal(ids, want[0]) and np.array_equal(sc, want[1])


def test_search_summary_ratios():
    import bench
    sweep = [{"offered_qps": 100, "achieved_qps": 95.0, "p50_ms": 1.0, "p99_ms": 2.0},
             {"offered_qps": 900, "achieved_qps": 880.0, "p50_ms": 3.0, "p99_ms": 9.0}]
    plain = {"p50_ms": 1.5}
    out = {"plain_loop": plain, "continuous_batching": sweep,
           "similar_kmers_thresh13": {"plain_loop": plain, "continuous_batching": sweep,
                                      "cpu_baseline": {"value": 44.0}},
           "c_path_phase_b_hinted_sw": {"plain_loop": plain, "continuous_batching": sweep,
                                        "cpu_baseline_error": "RuntimeError()"}}
    summ = bench.search_summary(out)
    assert summ["exact"]["server_max_achieved_qps"] == 880.0 and "host_cores_qps" not in summ["exact"]
    assert summ["similar"]["server_vs_host_cores"] == 880.0 / 44.0
    assert "host_cores_qps" not in summ["c_path"]
    assert summ["c_path"]["server_low_rate"]["p99_ms"] == 2.0


def test_exact_mode_host_chain_is_phase_a_then_unhinted_sw():
    """The exact-5-mer host baseline's scorer call (the C scorer with Phase B
    off) gives clustkit's Phase A survivors, and the chain runs end to end."""
    import types

    import bench
    import oracle
    s = synth.generate_families(60, 5, median=150, lo=40, hi=300, seed=32)
    off, ent, fr = so.build_kmer_index(s.flat, s.offsets, s.lengths, 5)
    ft = so.compute_freq_threshold(fr, s.n, 99.5)
    qs = [s.seq(i).copy() for i in (1, 9, 44, 120)]
    lens = np.array([len(q) for q in qs], np.int32)
    got = oracle.kmer_candidates_batch(np.concatenate(qs), np.concatenate([[0], np.cumsum(lens[:-1])]), lens,
                                       5, 20, off, ent, fr, ft, s.n, 2, 0, 10, 20, 10000)
    for q, (ids, sc, dg) in zip(qs, got):
        want = so.phase_a(q, 5, 20, off, ent, fr, ft, s.n, 2, 20)
        assert np.array_equal(ids, want[0]) and np.array_equal(sc, want[1]) and not dg.any()
    db = types.SimpleNamespace(index_arrays=lambda: (off, ent, fr), freq_thresh=ft, band_width=40)
    base = bench.search_cpu_baseline(db, s, qs * 8, target_s=0.01, mode="exact")
    assert base["value"] > 0 and base["unit"] == "queries/s" and "470-534" in base["source"]
