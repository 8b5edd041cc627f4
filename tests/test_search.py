"""Search path: k-mer index, Phase-A scoring, SW + rank, continuous batching.

CPU tests pin the numpy restatement (oracle/search_oracle.py) against the
reference's own outputs (tests/golden/search_golden.npz); GPU tests compare
the device index, Phase A and the full search with both, and check that a
query's result is the same alone and inside a concurrent mix.
"""
import numpy as np
import pytest

import oracle
from oracle import search_oracle as so
from clustkit_gb300 import synth
from clustkit_gb300.blosum import BLOSUM62


def _queries(g):
    return [g["q_flat"][o:o + L] for o, L in zip(g["q_offsets"], g["q_lengths"])]


def _ref_index(g):
    return so.build_kmer_index(g["db_flat"], g["db_offsets"], g["db_lengths"], int(g["k"]))


def test_oracle_index_and_phase_a_match_reference(golden):
    g = golden("search_golden.npz")
    k = int(g["k"])
    off, ent, fr = so.build_kmer_index(g["db_flat"], g["db_offsets"], g["db_lengths"], k)
    assert np.array_equal(ent, g["kmer_entries"])
    nz = np.nonzero(fr)[0]
    assert np.array_equal(nz, g["freq_nonzero_idx"]) and np.array_equal(fr[nz], g["freq_nonzero_val"])
    assert off[-1] == g["offsets_total"]
    thr = so.compute_freq_threshold(fr, len(g["db_lengths"]), 95.0)
    assert thr == int(g["freq_thresh"])
    for qi, q in enumerate(_queries(g)):
        ids, c = so.phase_a(q, k, 20, off, ent, fr, thr, len(g["db_lengths"]), 2, 10**9)
        assert np.array_equal(ids, g[f"q{qi}_ids"]) and np.array_equal(c, g[f"q{qi}_counts"])


def _oracle_search(g, top_k):
    k = int(g["k"])
    off, ent, fr = so.build_kmer_index(g["db_flat"], g["db_offsets"], g["db_lengths"], k)
    thr = so.compute_freq_threshold(fr, len(g["db_lengths"]), 95.0)
    qs = _queries(g)
    nq, nd = len(qs), len(g["db_lengths"])
    pairs = []
    for qi, q in enumerate(qs):
        ids, _ = so.phase_a(q, k, 20, off, ent, fr, thr, nd, 2, 10**9)
        pairs += [(qi, t) for t in ids]
    pairs = np.array(pairs, np.int32).reshape(-1, 2)
    flat = np.concatenate([g["q_flat"], g["db_flat"]])
    offs = np.concatenate([g["q_offsets"], g["db_offsets"] + len(g["q_flat"])])
    lens = np.concatenate([g["q_lengths"], g["db_lengths"]])
    merged = pairs.copy()
    merged[:, 1] += nq
    r = oracle.sw_batch(merged, flat, offs, lens, int(g["band_width"]), BLOSUM62)
    keep = r["scores"] > 0
    return so.rank_hits(pairs[keep], r["sims"][keep], r["scores"][keep], g["q_lengths"],
                        g["db_lengths"], nq, top_k)


def _golden_hits(g):
    hits = [[] for _ in range(len(g["q_lengths"]))]
    for q, t, i, s in zip(g["hit_query"], g["hit_target"], g["hit_identity"], g["hit_score"]):
        hits[int(q)].append((int(t), float(i), float(s)))
    return hits


def test_oracle_search_matches_reference(golden):
    g = golden("search_golden.npz")
    got = _oracle_search(g, int(g["top_k"]))
    want = _golden_hits(g)
    for a, b in zip(got, want):
        assert [x[0] for x in a] == [x[0] for x in b]
        assert np.allclose([x[1] for x in a], [x[1] for x in b], rtol=0, atol=0)
        assert np.allclose([x[2] for x in a], [x[2] for x in b], rtol=0, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("compact", [True, False])
def test_device_index_and_phase_a(ck, golden, compact):
    torch = pytest.importorskip("torch")
    from clustkit_gb300.search import DeviceDatabase, _Slot
    g = golden("search_golden.npz")
    db = DeviceDatabase(g["db_flat"], g["db_offsets"], g["db_lengths"], band_width=int(g["band_width"]),
                        arena_queries=32, arena_residues=32 * 400, compact_index=compact)
    off, ent, fr = db.index_arrays()
    assert np.array_equal(ent, g["kmer_entries"])
    if compact:  # clustkit's compact Phase-A index: the entries' sequence ids
        assert np.array_equal(db.d_kmer_targets[: db.n_entries].cpu().numpy(), (ent >> 32).astype(np.int32))
    nz = np.nonzero(fr)[0]
    assert np.array_equal(nz, g["freq_nonzero_idx"]) and np.array_equal(fr[nz], g["freq_nonzero_val"])
    assert off[-1] == g["offsets_total"] and db.freq_thresh == int(g["freq_thresh"])
    slot = _Slot(db, 0, 1000)
    try:
        qs = _queries(g)
        slot.launch(qs, 2)
        slot.event.synchronize()
        n = slot.h_n.numpy()[:len(qs)]
        tg = slot.h_targets.numpy().reshape(-1, 1000)
        for qi in range(len(qs)):
            assert np.array_equal(tg[qi, :n[qi]], g[f"q{qi}_ids"]), qi
        slot.results(5)
    finally:
        slot.close()


@pytest.mark.gpu
def test_search_batch_matches_reference(ck, golden):
    from clustkit_gb300.search import DeviceDatabase, search_batch
    g = golden("search_golden.npz")
    db = DeviceDatabase(g["db_flat"], g["db_offsets"], g["db_lengths"], band_width=int(g["band_width"]),
                        arena_queries=8, arena_residues=8 * 400)
    res = search_batch(db, _queries(g), top_k=int(g["top_k"]), max_cands=1000, kmer_score_thresh=0)
    want = _golden_hits(g)
    for hits, w in zip(res, want):
        assert [h.target for h in hits] == [x[0] for x in w]
        assert [h.identity for h in hits] == [x[1] for x in w]
        assert [np.float32(h.rank) for h in hits] == [np.float32(x[2]) for x in w]


@pytest.mark.gpu
@pytest.mark.parametrize("min_hits", [1, 2])
def test_phase_a_candidate_list_overflow(ck, min_hits):
    """Queries whose targets at >= min_hits outnumber the select's candidate
    list (4,096) take the full-row path; the result is the same."""
    from clustkit_gb300.search import DeviceDatabase, _Slot
    db_set = synth.generate_families(5000, 8, median=300, lo=40, hi=800, seed=12)
    db = DeviceDatabase(db_set.flat, db_set.offsets, db_set.lengths, arena_queries=4,
                        arena_residues=4 * 3000)
    off, ent, fr = db.index_arrays()
    bg = synth.random_sequences(2, median=2500, lo=2400, hi=2600, seed=13)
    qs = [bg.seq(0).copy(), bg.seq(1).copy(), db_set.seq(7).copy()]
    cap = 500
    slot = _Slot(db, 0, cap)
    try:
        slot.launch(qs, min_hits)
        slot.event.synchronize()
        n = slot.h_n.numpy()[:len(qs)]
        tg = slot.h_targets.numpy().reshape(-1, cap)
        over = 0
        for qi, q in enumerate(qs):
            ids, _ = so.phase_a(q, 5, 20, off, ent, fr, db.freq_thresh, db_set.n, min_hits, cap)
            assert np.array_equal(tg[qi, :n[qi]], ids), qi
            allc, _ = so.phase_a(q, 5, 20, off, ent, fr, db.freq_thresh, db_set.n, min_hits, 10 ** 9)
            over += len(allc) > 4096
        slot.results(3)
        if min_hits == 1:
            assert over >= 1  # the long background queries overflow the list
    finally:
        slot.close()


@pytest.mark.gpu
def test_phase_a_cap_and_ties_vs_oracle(ck):
    from clustkit_gb300.search import DeviceDatabase, _Slot
    db_set = synth.generate_families(300, 8, median=150, lo=40, hi=400, seed=91)
    db = DeviceDatabase(db_set.flat, db_set.offsets, db_set.lengths, arena_queries=16,
                        arena_residues=16 * 500)
    off, ent, fr = db.index_arrays()
    rng = np.random.default_rng(3)
    qs = [db_set.seq(int(i)).copy() for i in rng.choice(db_set.n, 12, replace=False)]
    qs += [np.tile(np.array([1, 2, 3, 4, 5, 6], np.uint8), 30), np.arange(60, dtype=np.uint8) % 20]
    for cap in (3, 17, 500):
        slot = _Slot(db, 0, cap)
        try:
            slot.launch(qs, 1)
            slot.event.synchronize()
            n = slot.h_n.numpy()[:len(qs)]
            tg = slot.h_targets.numpy().reshape(-1, cap)
            for qi, q in enumerate(qs):
                ids, _ = so.phase_a(q, 5, 20, off, ent, fr, db.freq_thresh, db_set.n, 1, cap)
                assert np.array_equal(tg[qi, :n[qi]], ids), (cap, qi)
            slot.results(3)
        finally:
            slot.close()


_C_PATH = {"min_diag_hits": 2, "use_c_scoring": True, "use_c_sw": True}


@pytest.mark.gpu
@pytest.mark.parametrize("use_graphs,thresh,scoring,list_rate",
                         [(True, 0, {}, None), (False, 0, {}, None), (False, 13, {}, None), (True, 13, {}, None),
                          (True, 13, {}, 1), (True, 0, _C_PATH, None)])
def test_server_results_same_alone_and_in_mix(ck, monkeypatch, use_graphs, thresh, scoring, list_rate):
    """Each query's hits are identical whether it is searched alone or lands
    in concurrent batches of the continuous-batching server (slots replaying
    captured CUDA graphs, or launching the pipeline call by call; exact,
    similar-k-mer and Phase-B + hinted-SW scoring).  ``list_rate`` 1: a
    similar-k-mer list bound so small that every replayed batch overflows it
    and is run again call by call in the slot's spare context."""
    from clustkit_gb300 import search as search_mod
    from clustkit_gb300.search import DeviceDatabase, SearchServer, search_batch
    if list_rate is not None:
        monkeypatch.setattr(search_mod, "LIST_RATE", list_rate)
    db_set = synth.generate_families(400, 10, median=200, lo=40, hi=600, seed=92)
    db = DeviceDatabase(db_set.flat, db_set.offsets, db_set.lengths, arena_slots=3, arena_queries=16,
                        arena_residues=16 * 600)
    rng = np.random.default_rng(5)
    qs = [db_set.seq(int(i)).copy() for i in rng.choice(db_set.n, 40, replace=False)]
    bg = synth.random_sequences(20, median=200, lo=40, hi=600, seed=93)
    qs += [bg.seq(i).copy() for i in range(bg.n)]
    alone = [search_batch(db, [q], top_k=10, kmer_score_thresh=thresh, **scoring)[0] for q in qs]
    server = SearchServer(db, top_k=10, max_batch=7, use_graphs=use_graphs, kmer_score_thresh=thresh,
                          **scoring).start()
    try:
        futs = [server.submit(q) for q in qs]
        mixed = [f.result(timeout=120) for f in futs]
        replaying = [bool(s.graphs) for s in server.slots]
        spare = [s.ctx_spare for s in server.slots]
    finally:
        server.stop()
    assert len(server.slots) >= 2
    if use_graphs:
        assert all(replaying)
    if list_rate is not None:  # every slot's warm-up batch already overflowed
        assert all(spare)
    for a, b in zip(alone, mixed):
        assert [(h.target, h.identity, h.score, h.rank) for h in a] == \
            [(h.target, h.identity, h.score, h.rank) for h in b]
    assert any(len(h) for h in mixed)
    lat = server.latency_percentiles()
    assert lat["n"] == len(qs)


@pytest.mark.gpu
def test_server_memory_budget_defers_and_keeps_results(ck):
    """A device-memory budget smaller than two full batches: the server never
    holds more than the budget in flight, defers requests until running
    batches return their bytes, and every query's hits are the same as when
    it is searched alone."""
    from clustkit_gb300.search import DeviceDatabase, SearchServer, batch_bytes, search_batch
    db_set = synth.generate_families(400, 10, median=200, lo=40, hi=600, seed=94)
    db = DeviceDatabase(db_set.flat, db_set.offsets, db_set.lengths, arena_slots=3, arena_queries=16,
                        arena_residues=16 * 600)
    rng = np.random.default_rng(7)
    qs = [db_set.seq(int(i)).copy() for i in rng.choice(db_set.n, 48, replace=False)]
    alone = [search_batch(db, [q], top_k=10, kmer_score_thresh=0)[0] for q in qs]
    budget = int(1.5 * batch_bytes(db, qs[:8], 500))  # room for one full batch, not two
    server = SearchServer(db, top_k=10, max_batch=8, use_graphs=False, kmer_score_thresh=0,
                          mem_budget=budget).start()
    try:
        futs = [server.submit(q) for q in qs]
        mixed = [f.result(timeout=120) for f in futs]
    finally:
        server.stop()
    assert len(server.slots) >= 2  # slots alone would let batches overlap
    assert server.deferrals > 0
    assert 0 < server.peak_in_flight_bytes <= budget
    assert server.in_flight_bytes == 0
    for a, b in zip(alone, mixed):
        assert [(h.target, h.identity, h.score, h.rank) for h in a] == \
            [(h.target, h.identity, h.score, h.rank) for h in b]


@pytest.mark.gpu
def test_frozen_context_refuses_to_grow(ck):
    """A frozen context (its buffers may sit in a captured graph) keeps
    working at the sizes it has and fails, instead of reallocating, beyond."""
    import torch
    from clustkit_gb300 import _lib
    from clustkit_gb300.blosum import BLOSUM62
    lib = _lib.load()
    s = synth.generate_families(50, 10, median=200, lo=40, hi=600, seed=4)
    pairs = synth.mixed_pairs(s, 60000, seed=1)
    dev = torch.device("cuda", 0)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_pairs, d_flat, d_off, d_len = T(pairs), T(s.flat), T(s.offsets), T(s.lengths)
    outs = [torch.empty(len(pairs), dtype=dt, device=dev) for dt in (torch.float32, torch.int32, torch.uint8)]
    sub = np.ascontiguousarray(BLOSUM62, np.int8)
    h = np.zeros(1, np.int32)
    _lib.check(lib.ck_ctx_create(h.ctypes.data))
    ctx = int(h[0])
    st = torch.cuda.current_stream(dev).cuda_stream

    def call(m):
        return lib.ck_sw_batch_device_ctx(ctx, d_pairs.data_ptr(), m, d_flat.data_ptr(), len(s.flat),
                                          d_off.data_ptr(), d_len.data_ptr(), s.n, 100, sub.ctypes.data,
                                          0.0, None, _lib.PASS_SCORE, 0, outs[0].data_ptr(),
                                          outs[1].data_ptr(), None, None, outs[2].data_ptr(), st)
    try:
        assert call(1000) == 0
        _lib.check(lib.ck_ctx_status(ctx, st))
        _lib.check(lib.ck_ctx_freeze(ctx, 1))
        assert call(1000) == 0
        assert call(len(pairs)) == 5  # CK_ERR_UNSUPPORTED: would have to grow
        _lib.check(lib.ck_ctx_freeze(ctx, 0))
        assert call(len(pairs)) == 0
        _lib.check(lib.ck_ctx_status(ctx, st))
        ref = oracle.sw_batch(pairs, s.flat, s.offsets, s.lengths, 100, BLOSUM62)
        assert np.array_equal(outs[1].cpu().numpy(), ref["scores"])
    finally:
        lib.ck_ctx_destroy(ctx)


def test_oracle_similar_phase_a_matches_reference(golden):
    """The numpy restatement of the BLOSUM62 similar-k-mer scoring against the
    reference's own _score_query_similar_k5 (golden)."""
    g = golden("search_golden.npz")
    off, ent, fr = _ref_index(g)
    qs = _queries(g)
    for qi in g["sim_queries"]:
        ids, sc = so.phase_a_similar(qs[qi], off, ent, fr, int(g["freq_thresh"]), len(g["db_lengths"]), 2,
                                     10 ** 9, BLOSUM62, 13)
        assert np.array_equal(ids, g[f"q{qi}_sim_ids"]), qi
        assert np.array_equal(sc, g[f"q{qi}_sim_scores"]), qi


def test_c_oracle_similar_matches_reference_and_numpy(golden):
    """The C restatement of the similar-5-mer scorer (the host-core baseline
    of that search mode) against the reference's own _score_query_similar_k5
    (golden), and against the numpy restatement with binding caps at
    thresholds 11/13/15."""
    import oracle
    g = golden("search_golden.npz")
    off, ent, fr = _ref_index(g)
    qs = _queries(g)
    sq = [qs[i] for i in g["sim_queries"]]
    nd = len(g["db_lengths"])

    def flat(queries):
        lens = np.array([len(q) for q in queries], np.int32)
        return np.concatenate(queries).astype(np.uint8), np.concatenate([[0], np.cumsum(lens[:-1])]), lens

    got = oracle.similar_candidates_batch(*flat(sq), BLOSUM62, 13, off, ent, fr, int(g["freq_thresh"]), nd, 2, nd)
    for (ids, sc), qi in zip(got, g["sim_queries"]):
        assert np.array_equal(ids, g[f"q{qi}_sim_ids"]), qi
        assert np.array_equal(sc, g[f"q{qi}_sim_scores"]), qi
    db_set = synth.generate_families(120, 6, median=150, lo=40, hi=400, seed=21)
    off, ent, fr = so.build_kmer_index(db_set.flat, db_set.offsets, db_set.lengths, 5)
    rng = np.random.default_rng(22)
    qs = [db_set.seq(int(i)).copy() for i in rng.choice(db_set.n, 4, replace=False)]
    qs += [synth.random_sequences(1, median=100, lo=60, hi=160, seed=23).seq(0).copy()]
    freq_thresh = int(fr.max())
    for thresh, cap in ((11, 40), (13, 7), (15, 300)):
        got = oracle.similar_candidates_batch(*flat(qs), BLOSUM62, thresh, off, ent, fr, freq_thresh, db_set.n, 2,
                                              cap)
        for q, (ids, sc) in zip(qs, got):
            want = so.phase_a_similar(q, off, ent, fr, freq_thresh, db_set.n, 2, cap, BLOSUM62, thresh)
            assert np.array_equal(ids, want[0]) and np.array_equal(sc, want[1]), (thresh, cap)


@pytest.mark.gpu
@pytest.mark.parametrize("compact", [True, False])
def test_similar_phase_a_and_search_match_reference(ck, golden, compact):
    """Golden similar-k-mer Phase A and search (compact and full index)."""
    from clustkit_gb300.search import DeviceDatabase, _Slot, search_batch
    g = golden("search_golden.npz")
    db = DeviceDatabase(g["db_flat"], g["db_offsets"], g["db_lengths"], band_width=int(g["sim_band_width"]),
                        arena_queries=16, arena_residues=16 * 400, compact_index=compact)
    qs = _queries(g)
    sq = [qs[i] for i in g["sim_queries"]]
    slot = _Slot(db, 0, 1000)
    try:
        slot.launch(sq, 2, 13)
        slot.event.synchronize()
        n = slot.h_n.numpy()[:len(sq)]
        tg = slot.h_targets.numpy().reshape(-1, 1000)
        for k, qi in enumerate(g["sim_queries"]):
            assert np.array_equal(tg[k, :n[k]], g[f"q{qi}_sim_ids"]), qi
        slot.results(5)
    finally:
        slot.close()
    res = search_batch(db, sq, top_k=int(g["top_k"]), max_cands=1000, kmer_score_thresh=13)
    got = [(int(g["sim_queries"][q]), h.target, h.identity, h.rank) for q, hl in enumerate(res) for h in hl]
    exp = list(zip(g["sim_hit_query"].tolist(), g["sim_hit_target"].tolist(), g["sim_hit_identity"].tolist(),
                   g["sim_hit_score"].tolist()))
    assert len(got) == len(exp)
    for a, b in zip(got, exp):
        assert a[0] == b[0] and a[1] == b[1]
        assert np.float32(a[2]) == np.float32(b[2]) and np.float32(a[3]) == np.float32(b[3])


@pytest.mark.gpu
@pytest.mark.parametrize("thresh", [11, 13, 15])
def test_similar_phase_a_cap_vs_oracle(ck, thresh):
    """Capped and uncapped outputs of the neighbour scoring against the oracle,
    on a database large enough that most queries hit the cap."""
    from clustkit_gb300.search import DeviceDatabase, _Slot
    db_set = synth.generate_families(200, 8, median=150, lo=40, hi=400, seed=thresh)
    db = DeviceDatabase(db_set.flat, db_set.offsets, db_set.lengths, arena_queries=8, arena_residues=8 * 500)
    off, ent, fr = db.index_arrays()
    rng = np.random.default_rng(thresh)
    qs = [db_set.seq(int(i)).copy() for i in rng.choice(db_set.n, 5, replace=False)]
    qs += [synth.random_sequences(1, median=120, lo=60, hi=200, seed=thresh + 1).seq(0).copy()]
    for cap in (7, 300, 5000):
        slot = _Slot(db, 0, cap)
        try:
            slot.launch(qs, 2, thresh)
            slot.event.synchronize()
            n = slot.h_n.numpy()[:len(qs)]
            tg = slot.h_targets.numpy().reshape(-1, cap)
            for qi, q in enumerate(qs):
                ids, _ = so.phase_a_similar(q, off, ent, fr, db.freq_thresh, db_set.n, 2, cap, BLOSUM62, thresh)
                assert np.array_equal(tg[qi, :n[qi]], ids), (cap, qi)
            slot.results(3)
        finally:
            slot.close()


def _similar_call(db, qs, top_k, list_capacity, ctx, expect=0, thresh=13):
    """(ids, scores) rows from one ck_search_phase_a_similar_device call in
    library context ``ctx`` (``expect``: the status ck_ctx_status reports)."""
    import torch
    from clustkit_gb300 import _lib
    from clustkit_gb300.search import _SUB
    lib, dev = db.lib, db.dev
    nq = len(qs)
    lens = np.array([len(q) for q in qs], np.int32)
    offs = np.concatenate([[0], np.cumsum(lens[:-1])]).astype(np.int64)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_q, d_off, d_len = T(np.concatenate(qs).astype(np.uint8)), T(offs), T(lens)
    out_t = torch.full((nq * top_k,), -7, dtype=torch.int32, device=dev)
    out_s = torch.full_like(out_t, -7)
    out_n = torch.full((nq,), -7, dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(lib.ck_search_phase_a_similar_device(
        ctx, d_q.data_ptr(), int(lens.sum()), d_off.data_ptr(), d_len.data_ptr(), nq, int(lens.max()),
        _SUB.ctypes.data, thresh, db.d_kmer_offsets.data_ptr(), db.d_kmer_entries.data_ptr(), db.kmer_targets_ptr,
        db.d_kmer_freqs.data_ptr(), db.freq_thresh, db.n, 2, top_k, out_t.data_ptr(), out_s.data_ptr(),
        out_n.data_ptr(), int(list_capacity), st))
    assert lib.ck_ctx_status(ctx, st) == expect
    n = out_n.cpu().numpy()
    t = out_t.cpu().numpy().reshape(nq, top_k)
    s = out_s.cpu().numpy().reshape(nq, top_k)
    return [(t[i, :n[i]], s[i, :n[i]]) for i in range(nq)]


@pytest.mark.gpu
def test_similar_neighbour_list_bounds(ck):
    """The neighbour list three ways on one batch: sized by the library in a
    fresh context (more triples than its first list holds, so it grows and
    lists again), under an ample caller bound (no host synchronisation), and
    under a bound too small (CK_ERR_CAPACITY, after which the context is
    usable again) -- the first two identical, and one query of them against
    the oracle."""
    from clustkit_gb300 import _lib
    from clustkit_gb300.search import DeviceDatabase
    db_set = synth.generate_families(600, 8, median=350, lo=60, hi=1200, seed=5)
    db = DeviceDatabase(db_set.flat, db_set.offsets, db_set.lengths, arena_queries=8, arena_residues=8 * 2500)
    rng = np.random.default_rng(6)
    qs = [db_set.seq(int(i)).copy() for i in rng.choice(db_set.n, 5, replace=False)]
    qs += [synth.random_sequences(1, median=2000, lo=1800, hi=2200, seed=9).seq(0).copy()]
    top_k = 400
    h = np.zeros(1, np.int32)
    ctxs = []
    try:
        for _ in range(2):
            _lib.check(db.lib.ck_ctx_create(h.ctypes.data))
            ctxs.append(int(h[0]))
        sized = _similar_call(db, qs, top_k, -1, ctxs[0])
        bounded = _similar_call(db, qs, top_k, 1 << 26, ctxs[1])
        for a, b in zip(sized, bounded):
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        _similar_call(db, qs, top_k, 1000, ctxs[1], expect=_lib.CK_ERR_CAPACITY)
        again = _similar_call(db, qs, top_k, 1 << 26, ctxs[1])
        for a, b in zip(sized, again):
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        off, ent, fr = db.index_arrays()
        ids, sc = so.phase_a_similar(qs[0], off, ent, fr, db.freq_thresh, db_set.n, 2, top_k, BLOSUM62, 13)
        assert np.array_equal(sized[0][0], ids) and np.array_equal(sized[0][1], sc)
    finally:
        for c in ctxs:
            db.lib.ck_ctx_destroy(c)


def test_oracle_kmer_candidates_match_reference_c_scorer(golden):
    """The numpy restatement of clustkit's C k-mer scorer (Phase A, top-K,
    Phase B, diagonal hints, caps) against the compiled reference scorer, and
    the reference's Numba two-stage scorer where no cap binds."""
    g = golden("kmer_scorer_golden.npz")
    off, ent, fr = so.build_kmer_index(g["db_flat"], g["db_offsets"], g["db_lengths"], 5)
    qs = _queries(g)
    nd = len(g["db_lengths"])
    for ci, (mth, mdh, dbw, mc, topk) in enumerate(g["configs"]):
        for qi, q in enumerate(qs):
            ids, sc, dg = so.kmer_candidates(q, 5, 20, off, ent, fr, int(g["freq_thresh"]), nd, int(mth), int(mdh),
                                             int(dbw), int(mc), int(topk))
            assert np.array_equal(ids, g[f"c{ci}_q{qi}_targets"]), (ci, qi)
            assert np.array_equal(sc, g[f"c{ci}_q{qi}_scores"]), (ci, qi)
            if mdh >= 2:
                assert np.array_equal(dg, g[f"c{ci}_q{qi}_diags"]), (ci, qi)
    for qi in range(len(qs)):
        assert np.array_equal(g[f"numba_q{qi}_ids"], g[f"c2_q{qi}_targets"])
        assert np.array_equal(g[f"numba_q{qi}_scores"], g[f"c2_q{qi}_scores"])


def test_c_oracle_kmer_candidates_match_reference_and_numpy(golden):
    """The C restatement of the k-mer scorer (the search path's CPU baseline)
    against the reference scorer's golden vectors and the numpy restatement."""
    g = golden("kmer_scorer_golden.npz")
    off, ent, fr = so.build_kmer_index(g["db_flat"], g["db_offsets"], g["db_lengths"], 5)
    nd = len(g["db_lengths"])
    for ci, (mth, mdh, dbw, mc, topk) in enumerate(g["configs"]):
        got = oracle.kmer_candidates_batch(g["q_flat"], g["q_offsets"], g["q_lengths"], 5, 20, off, ent, fr,
                                           int(g["freq_thresh"]), nd, int(mth), int(mdh), int(dbw), int(mc),
                                           int(topk))
        for qi, (ids, sc, dg) in enumerate(got):
            assert np.array_equal(ids, g[f"c{ci}_q{qi}_targets"]), (ci, qi)
            assert np.array_equal(sc, g[f"c{ci}_q{qi}_scores"]), (ci, qi)
            if mdh >= 2:
                assert np.array_equal(dg, g[f"c{ci}_q{qi}_diags"]), (ci, qi)
    db_set = synth.generate_families(300, 8, median=200, lo=40, hi=700, seed=33)
    off, ent, fr = so.build_kmer_index(db_set.flat, db_set.offsets, db_set.lengths, 5)
    thr = so.compute_freq_threshold(fr, db_set.n, 95.0)
    rng = np.random.default_rng(2)
    qs = [db_set.seq(int(i)).copy() for i in rng.choice(db_set.n, 10, replace=False)]
    qs += [np.zeros(0, np.uint8), np.array([1, 2], np.uint8), np.full(50, 20, np.uint8)]
    lens = np.array([len(q) for q in qs], np.int32)
    offs = np.concatenate([[0], np.cumsum(lens[:-1])]).astype(np.int64)
    flat = np.concatenate(qs).astype(np.uint8)
    for cfg in [(2, 2, 10, 2000, 10000), (1, 3, 1, 9, 40), (2, 1, 10, 5, 100), (0, 2, 30, 50, 200)]:
        got = oracle.kmer_candidates_batch(flat, offs, lens, 5, 20, off, ent, fr, thr, db_set.n, *cfg)
        for qi, q in enumerate(qs):
            want = so.kmer_candidates(q, 5, 20, off, ent, fr, thr, db_set.n, *cfg)
            for a, b in zip(got[qi], want):
                assert np.array_equal(a, b), (cfg, qi)


def _ref_like_index(g):
    """The database and queries of a golden file in the shape of clustkit's
    DatabaseIndex / SequenceDataset (the fields search_kmer_index reads)."""
    import types
    db = types.SimpleNamespace(flat_sequences=g["db_flat"], offsets=g["db_offsets"], lengths=g["db_lengths"],
                               ids=[f"d{i}" for i in range(len(g["db_lengths"]))])
    idx = types.SimpleNamespace(dataset=db, params={"mode": "protein", "kmer_size": int(g["k"])})
    return idx


def _ref_like_queries(flat, offs, lens, names):
    import types
    return types.SimpleNamespace(flat_sequences=flat, offsets=offs, lengths=lens, ids=list(names))


@pytest.mark.gpu
def test_search_kmer_index_dropin_matches_reference(ck, golden):
    """The drop-in search_kmer_index, called with the arguments the golden run of
    clustkit's own search_kmer_index used (exact Phase A; BLOSUM62 similar 5-mers
    on a query subset), returns the same hits: target ids, identities and rank
    scores, in order, with clustkit's per-call band width."""
    from clustkit_gb300.search import search_kmer_index
    g = golden("search_golden.npz")
    idx = _ref_like_index(g)
    qs = _ref_like_queries(g["q_flat"], g["q_offsets"], g["q_lengths"], [f"q{i}" for i in range(len(g["q_lengths"]))])
    res = search_kmer_index(idx, qs, threshold=0.0, top_k=5, band_width=None, min_total_hits=2, min_diag_hits=1,
                            max_cands_per_query=100000, freq_percentile=95.0, kmer_score_thresh=0,
                            local_alignment=True, evalue_normalize=True)
    want = _golden_hits(g)
    assert res.num_queries == len(want) and res.num_targets == len(g["db_lengths"])
    for qi, (hl, w) in enumerate(zip(res.hits, want)):
        assert [int(h.target_id[1:]) for h in hl] == [x[0] for x in w], qi
        assert [np.float32(h.identity) for h in hl] == [np.float32(x[1]) for x in w], qi
        assert [np.float32(h.score) for h in hl] == [np.float32(x[2]) for x in w], qi
        assert all(h.query_id == f"q{qi}" and h.query_length == g["q_lengths"][qi] for h in hl)
        assert all(h.target_length == g["db_lengths"][int(h.target_id[1:])] for h in hl)
    # similar 5-mers, clustkit's default scoring, on the golden query subset
    sq = [int(i) for i in g["sim_queries"]]
    lens = g["q_lengths"][sq]
    flat = np.concatenate([g["q_flat"][g["q_offsets"][i]:g["q_offsets"][i] + g["q_lengths"][i]] for i in sq])
    offs = np.concatenate([[0], np.cumsum(lens[:-1])]).astype(np.int64)
    res2 = search_kmer_index(idx, _ref_like_queries(flat, offs, lens, [f"q{i}" for i in sq]), threshold=0.0,
                             top_k=5, band_width=None, min_total_hits=2, min_diag_hits=1,
                             max_cands_per_query=100000, freq_percentile=95.0, kmer_score_thresh=13)
    want2 = {}
    for q, t, i, s in zip(g["sim_hit_query"], g["sim_hit_target"], g["sim_hit_identity"], g["sim_hit_score"]):
        want2.setdefault(int(q), []).append((int(t), float(i), float(s)))
    for k, qi in enumerate(sq):
        hl, w = res2.hits[k], want2.get(qi, [])
        assert [int(h.target_id[1:]) for h in hl] == [x[0] for x in w], qi
        assert [np.float32(h.identity) for h in hl] == [np.float32(x[1]) for x in w], qi
        assert [np.float32(h.score) for h in hl] == [np.float32(x[2]) for x in w], qi


def test_search_kmer_index_refuses_unbuilt_variants():
    """Options for the search variants not built on the GPU fail loudly."""
    import types
    from clustkit_gb300.search import search_kmer_index
    idx = types.SimpleNamespace(dataset=None, params={"mode": "protein", "kmer_size": 5})
    for kw in ({"reduced_alphabet": True}, {"use_idf": True}, {"spaced_seeds": ["11011"]},
               {"min_ungapped_score": 5}, {"local_alignment": False}):
        with pytest.raises(NotImplementedError):
            search_kmer_index(idx, None, **kw)
