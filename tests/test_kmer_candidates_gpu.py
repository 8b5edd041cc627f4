"""The device twin of clustkit's C k-mer scorer (batch_score_queries_c,
clustkit/csrc/kmer_score.c:420-470) through ck_search_kmer_candidates_device:
against golden vectors recorded from the compiled reference scorer, against the
oracle on caps, ties, long queries and the select's list overflow, and the
searches built on it (C scoring + C SW with diagonal hints, the Numba
two-stage scorer's path) against the oracle chain."""
import numpy as np
import pytest

import oracle
from oracle import search_oracle as so
from clustkit_gb300 import synth
from clustkit_gb300.blosum import BLOSUM62


def _queries(g):
    return [g["q_flat"][o:o + L] for o, L in zip(g["q_offsets"], g["q_lengths"])]


def _bins_bound(db, qs, width, topk):
    """The caller's bound on the Phase-B bins (no host synchronisation)."""
    return min(topk, db.n) * ((sum(len(q) for q in qs) + len(qs) * db.max_len) // width + len(qs))


def _device_candidates(db, qs, mth, mdh, width, mc, topk, with_diags=True, with_scores=True, bins_capacity=-1,
                       expect=0, ctx=None):
    """Per query (ids, scores, diags) from one call of the C-ABI entry point
    (``expect``: the status ck_ctx_status should report; ``ctx``: a library
    context to reuse, else a fresh one)."""
    import torch
    from clustkit_gb300 import _lib
    lib, dev = db.lib, db.dev
    nq = len(qs)
    lens = np.array([len(q) for q in qs], np.int32)
    offs = np.zeros(nq, np.int64)
    if nq > 1:
        offs[1:] = np.cumsum(lens[:-1])
    flat = np.concatenate(qs).astype(np.uint8) if int(lens.sum()) else np.zeros(1, np.uint8)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_q, d_off, d_len = T(flat), T(offs), T(lens)
    fill = lambda n: torch.full((max(n, 1),), -7, dtype=torch.int32, device=dev)
    out_t, out_s, out_d, out_n = fill(nq * mc), fill(nq * mc), fill(nq * mc), fill(nq)
    own = ctx is None
    if own:
        h = np.zeros(1, np.int32)
        _lib.check(lib.ck_ctx_create(h.ctypes.data))
        ctx = int(h[0])
    st = torch.cuda.current_stream(dev).cuda_stream
    try:
        _lib.check(lib.ck_search_kmer_candidates_device(
            ctx, d_q.data_ptr(), int(lens.sum()), d_off.data_ptr(), d_len.data_ptr(), nq,
            int(lens.max()) if nq else 0, db.k, db.alpha, db.d_kmer_offsets.data_ptr(),
            db.d_kmer_entries.data_ptr(), db.kmer_targets_ptr, db.d_kmer_freqs.data_ptr(), db.freq_thresh, db.n,
            db.d_lengths.data_ptr(), int(mth), int(mdh), int(width), int(mc), int(topk), out_t.data_ptr(),
            out_s.data_ptr() if with_scores else None, out_d.data_ptr() if with_diags else None,
            out_n.data_ptr(), int(bins_capacity), st))
        assert lib.ck_ctx_status(ctx, st) == expect
    finally:
        if own:
            lib.ck_ctx_destroy(ctx)
    n = out_n.cpu().numpy()[:nq]
    t = out_t.cpu().numpy()[: nq * mc].reshape(nq, mc) if nq else np.zeros((0, mc), np.int32)
    s = out_s.cpu().numpy()[: nq * mc].reshape(nq, mc) if nq else t
    d = out_d.cpu().numpy()[: nq * mc].reshape(nq, mc) if nq else t
    return [(t[i, :n[i]], s[i, :n[i]], d[i, :n[i]]) for i in range(nq)]


@pytest.mark.gpu
@pytest.mark.parametrize("compact", [True, False])
def test_device_kmer_candidates_match_reference_c_scorer(ck, golden, compact):
    """Every configuration of the golden set: targets, scores (Phase-A hits or
    Phase-B runs) in the scorer's order, and the diagonal hints; Phase A
    reading the compact target index or the full entries."""
    from clustkit_gb300.search import DeviceDatabase
    g = golden("kmer_scorer_golden.npz")
    db = DeviceDatabase(g["db_flat"], g["db_offsets"], g["db_lengths"], arena_queries=4, arena_residues=4 * 600,
                        compact_index=compact)
    assert (db.kmer_targets_ptr is not None) == compact
    assert db.freq_thresh == int(g["freq_thresh"])
    qs = _queries(g)
    for ci, (mth, mdh, width, mc, topk) in enumerate(g["configs"]):
        # bins sized on the host from the device count, or under the caller's bound
        got = _device_candidates(db, qs, mth, mdh, width, mc, topk,
                                 bins_capacity=_bins_bound(db, qs, width, topk) if compact else -1)
        for qi, (ids, sc, dg) in enumerate(got):
            assert np.array_equal(ids, g[f"c{ci}_q{qi}_targets"]), (ci, qi)
            assert np.array_equal(sc, g[f"c{ci}_q{qi}_scores"]), (ci, qi)
            if mdh >= 2:
                assert np.array_equal(dg, g[f"c{ci}_q{qi}_diags"]), (ci, qi)
            else:
                assert not dg.any()


@pytest.mark.gpu
def test_device_kmer_candidates_vs_oracle_edges(ck):
    """Empty and sub-k queries, unknown residues, Phase-A top-K and final caps
    with ties, bin widths 1..100000, and queries whose kept targets overflow
    the select's candidate list (more than 4,096: the row scan)."""
    from clustkit_gb300.search import DeviceDatabase
    db_set = synth.generate_families(5000, 8, median=300, lo=40, hi=800, seed=12)
    db = DeviceDatabase(db_set.flat, db_set.offsets, db_set.lengths, arena_queries=4, arena_residues=4 * 7000)
    off, ent, fr = db.index_arrays()
    rng = np.random.default_rng(21)
    qs = [db_set.seq(int(i)).copy() for i in rng.choice(db_set.n, 6, replace=False)]
    bg = synth.random_sequences(2, median=6000, lo=5800, hi=6200, seed=13)
    qs += [bg.seq(0).copy(), bg.seq(1).copy()]
    x = db_set.seq(3).copy()
    x[::7] = 20  # unknown residues break k-mers
    qs += [x, np.zeros(0, np.uint8), np.array([1, 2, 3], np.uint8), np.tile(np.arange(5, dtype=np.uint8), 40)]
    configs = [(2, 2, 10, 2000, 10000), (1, 2, 100000, 20000, 10 ** 6), (1, 2, 10, 5000, 10 ** 6),
               (2, 3, 1, 40, 300), (1, 2, 25, 7, 12), (3, 4, 10, 100, 50), (2, 1, 10, 30, 10000),
               (1, 2, 100000, 5000, 10 ** 6), (1, 1, 10, 6000, 10000)]
    over = capped_big = 0
    for mth, mdh, width, mc, topk in configs:
        got = _device_candidates(db, qs, mth, mdh, width, mc, topk)
        for qi, q in enumerate(qs):
            ids, sc, dg = so.kmer_candidates(q, 5, 20, off, ent, fr, db.freq_thresh, db_set.n, mth, mdh, width,
                                             mc, topk)
            assert np.array_equal(got[qi][0], ids), (mth, mdh, width, mc, topk, qi)
            assert np.array_equal(got[qi][1], sc), (mth, mdh, width, mc, topk, qi)
            assert np.array_equal(got[qi][2], dg), (mth, mdh, width, mc, topk, qi)
            over += len(ids) > 4096
            if mc > 4096 and len(ids) == mc:
                full, _, _ = so.kmer_candidates(q, 5, 20, off, ent, fr, db.freq_thresh, db_set.n, mth, mdh, width,
                                                10 ** 7, topk)
                capped_big += len(full) > mc
    assert over >= 2  # the long background queries at one bin per target
    assert capped_big >= 2  # rows capped above 4,096 (the segmented sort)
    # the same order when the caller takes no scores (nor hints)
    for mth, mdh, width, mc, topk in [(1, 2, 100000, 5000, 10 ** 6), (1, 1, 10, 6000, 10000)]:
        a = _device_candidates(db, qs, mth, mdh, width, mc, topk)
        b = _device_candidates(db, qs, mth, mdh, width, mc, topk, with_diags=False, with_scores=False)
        for qi in range(len(qs)):
            assert np.array_equal(a[qi][0], b[qi][0]), (mth, mdh, width, mc, topk, qi)


def _oracle_search(db_set, qs, top_k, mth, mdh, width, mc, topk, band, hints):
    off, ent, fr = so.build_kmer_index(db_set.flat, db_set.offsets, db_set.lengths, 5)
    thr = so.compute_freq_threshold(fr, db_set.n, 95.0)
    nq = len(qs)
    pairs, diags = [], []
    for qi, q in enumerate(qs):
        ids, _, dg = so.kmer_candidates(q, 5, 20, off, ent, fr, thr, db_set.n, mth, mdh, width, mc, topk)
        pairs += [(qi, int(t)) for t in ids]
        diags += list(dg)
    pairs = np.array(pairs, np.int32).reshape(-1, 2)
    q_lens = np.array([len(q) for q in qs], np.int32)
    q_offs = np.zeros(nq, np.int64)
    q_offs[1:] = np.cumsum(q_lens[:-1])
    flat = np.concatenate(list(qs) + [db_set.flat]).astype(np.uint8)
    offs = np.concatenate([q_offs, db_set.offsets + int(q_lens.sum())])
    lens = np.concatenate([q_lens, db_set.lengths])
    merged = pairs.copy()
    merged[:, 1] += nq
    r = oracle.sw_batch(merged, flat, offs, lens, band, BLOSUM62,
                        diag_hints=np.array(diags, np.int32) if hints else None)
    keep = r["scores"] > 0
    return so.rank_hits(pairs[keep], r["sims"][keep], r["scores"][keep], q_lens, db_set.lengths, nq, top_k)


@pytest.mark.gpu
@pytest.mark.parametrize("c_path", [True, False])
def test_search_with_diagonal_scoring_vs_oracle(ck, c_path):
    """clustkit's C path (C scoring, C SW at band 50 centred on the Phase-B
    hints) and its Numba two-stage path (Phase B, the database band, no hints):
    the hits of search_batch against the oracle chain."""
    from clustkit_gb300.search import DeviceDatabase, search_batch
    db_set = synth.generate_families(300, 8, median=220, lo=40, hi=900, seed=77)
    db = DeviceDatabase(db_set.flat, db_set.offsets, db_set.lengths, arena_queries=8, arena_residues=8 * 900)
    rng = np.random.default_rng(8)
    qs = [db_set.seq(int(i)).copy() for i in rng.choice(db_set.n, 14, replace=False)]
    bg = synth.random_sequences(4, median=250, lo=60, hi=700, seed=78)
    qs += [bg.seq(i).copy() for i in range(bg.n)]
    mth, mdh, width, mc, topk = 2, 2, 10, 40, 200
    kw = dict(min_diag_hits=mdh, diag_bin_width=width, phase_a_topk=topk)
    if c_path:
        kw.update(use_c_scoring=True, use_c_sw=True, c_sw_band_width=50)
    res = search_batch(db, qs, top_k=10, max_cands=mc, min_total_hits=mth, kmer_score_thresh=0, **kw)
    band = 50 if c_path else db.band_width
    want = _oracle_search(db_set, qs, 10, mth, mdh, width, mc, topk, band, c_path)
    for qi, (hits, w) in enumerate(zip(res, want)):
        assert [h.target for h in hits] == [x[0] for x in w], qi
        assert [np.float32(h.identity) for h in hits] == [np.float32(x[1]) for x in w], qi
        assert [np.float32(h.rank) for h in hits] == [np.float32(x[2]) for x in w], qi
    assert sum(len(h) for h in res) >= 14


@pytest.mark.gpu
def test_bounded_bins_reuse_and_overflow(ck):
    """Phase B under the caller's bin bound keeps its buffer zero between calls
    (repeated calls, shrinking and growing batches agree with the oracle); a
    bound too small is reported as CK_ERR_CAPACITY with nothing written
    out of range, and the next call is correct again."""
    from clustkit_gb300.search import DeviceDatabase
    db_set = synth.generate_families(400, 8, median=250, lo=40, hi=900, seed=31)
    db = DeviceDatabase(db_set.flat, db_set.offsets, db_set.lengths, arena_queries=4, arena_residues=4 * 1000)
    off, ent, fr = db.index_arrays()
    rng = np.random.default_rng(4)
    qs = [db_set.seq(int(i)).copy() for i in rng.choice(db_set.n, 12, replace=False)]
    cfg = (2, 2, 10, 50, 500)

    def check(sub_qs, got):
        for qi, q in enumerate(sub_qs):
            want = so.kmer_candidates(q, 5, 20, off, ent, fr, db.freq_thresh, db_set.n, *cfg)
            for a, b in zip(got[qi], want):
                assert np.array_equal(a, b), qi

    from clustkit_gb300 import _lib
    h = np.zeros(1, np.int32)
    _lib.check(db.lib.ck_ctx_create(h.ctypes.data))
    ctx = int(h[0])  # one context: its kept-zero bin buffer is reused call after call
    try:
        for sub_qs in (qs, qs[:3], qs[5:], qs, qs[:1]):
            check(sub_qs, _device_candidates(db, sub_qs, *cfg, bins_capacity=_bins_bound(db, sub_qs, 10, 500),
                                             ctx=ctx))
        _device_candidates(db, qs, *cfg, bins_capacity=1000, expect=_lib.CK_ERR_CAPACITY, ctx=ctx)
        check(qs, _device_candidates(db, qs, *cfg, bins_capacity=_bins_bound(db, qs, 10, 500), ctx=ctx))
    finally:
        db.lib.ck_ctx_destroy(ctx)
