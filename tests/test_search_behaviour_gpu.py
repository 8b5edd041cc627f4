"""Behaviour of the drop-in search_kmer_index, case for case as clustkit's own
search tests state it (tests/test_search.py in the reference: exact matches
found, the top-k limit, hits in rank order, empty queries), in every scoring
mode the GPU builds; the exact hits against the reference are pinned
elsewhere by golden vectors."""
import types

import numpy as np
import pytest

from clustkit_gb300 import synth

MODES = {"similar": {}, "exact": {"kmer_score_thresh": 0, "min_diag_hits": 1},
         "phase_b": {"kmer_score_thresh": 0, "min_diag_hits": 2},
         "c_path": {"kmer_score_thresh": 0, "min_diag_hits": 2, "use_c_scoring": True, "use_c_sw": True}}


def _dataset(seqs, prefix):
    lens = np.array([len(x) for x in seqs], np.int32)
    offs = np.zeros(len(seqs), np.int64)
    if len(seqs) > 1:
        offs[1:] = np.cumsum(lens[:-1])
    flat = np.concatenate(seqs).astype(np.uint8) if len(seqs) and lens.sum() else np.zeros(0, np.uint8)
    return types.SimpleNamespace(flat_sequences=flat, offsets=offs, lengths=lens,
                                 ids=[f"{prefix}{i}" for i in range(len(seqs))])


@pytest.fixture(scope="module")
def db():
    s = synth.generate_families(60, 5, median=220, lo=60, hi=600, seed=41)
    ds = _dataset([s.seq(i).copy() for i in range(s.n)], "t")
    return s, types.SimpleNamespace(dataset=ds, params={"mode": "protein", "kmer_size": 5})


@pytest.mark.gpu
@pytest.mark.parametrize("mode", list(MODES))
def test_finds_exact_matches(ck, db, mode):
    """A query identical to a database sequence finds it first, at identity 1."""
    from clustkit_gb300.search import search_kmer_index
    s, idx = db
    picks = [3, 77, 150, 299]
    res = search_kmer_index(idx, _dataset([s.seq(i).copy() for i in picks], "q"), top_k=5, **MODES[mode])
    for qi, i in enumerate(picks):
        hits = res.hits[qi]
        assert hits, (mode, qi)
        assert hits[0].target_id == f"t{i}" and hits[0].identity == 1.0, (mode, qi, hits[0])
        assert hits[0].query_length == hits[0].target_length == len(s.seq(i))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("top_k", [1, 3, 10])
def test_top_k_and_rank_order(ck, db, mode, top_k):
    """At most top_k hits per query, in non-increasing rank order; a member
    of a family of five finds its relatives."""
    from clustkit_gb300.search import search_kmer_index
    s, idx = db
    qs = [s.seq(i).copy() for i in range(0, s.n, 37)]
    res = search_kmer_index(idx, _dataset(qs, "q"), top_k=top_k, **MODES[mode])
    assert res.num_queries == len(qs) and res.num_targets == s.n
    for hl in res.hits:
        assert len(hl) <= top_k
        ranks = [h.score for h in hl]
        assert ranks == sorted(ranks, reverse=True)
    if top_k >= 3:
        assert sum(len(hl) >= 2 for hl in res.hits) >= len(qs) // 2


@pytest.mark.gpu
@pytest.mark.parametrize("mode", list(MODES))
def test_empty_queries(ck, db, mode):
    """No queries: empty results; an empty or sub-k query: no hits, and the
    other queries of its batch are unaffected."""
    from clustkit_gb300.search import search_kmer_index
    s, idx = db
    none = search_kmer_index(idx, _dataset([], "q"), **MODES[mode])
    assert none.hits == [] and none.num_queries == 0
    mixed = [np.zeros(0, np.uint8), s.seq(5).copy(), np.array([1, 2, 3], np.uint8)]
    # one band for both calls (by default it follows the call's query lengths)
    res = search_kmer_index(idx, _dataset(mixed, "q"), top_k=5, band_width=100, **MODES[mode])
    alone = search_kmer_index(idx, _dataset([s.seq(5).copy()], "q"), top_k=5, band_width=100, **MODES[mode])
    assert res.hits[0] == [] and res.hits[2] == []
    assert [(h.target_id, h.identity, h.score) for h in res.hits[1]] == \
        [(h.target_id, h.identity, h.score) for h in alone.hits[0]]
