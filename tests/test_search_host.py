"""Host logic of the search slot: the ranking pass of a batch (rank, per-query
pre-selection, packed-key stable sort) equals the two-key lexsort
formulation, clustkit's stable descending-rank order (kmer_index.py:2318-2323,
clustkit/search.py:727-800), on random batches full of equal ranks."""
import types

import numpy as np

from clustkit_gb300 import search as S


def _lexsort_hits(nq, K, n, tg, sims, scores, mask, lens, lh, top_k):
    col = np.arange(K)[None, :]
    keep = (col < n[:, None]) & mask.astype(bool)
    qi, ci = np.nonzero(keep)
    t, sc, si = tg[qi, ci], scores[qi, ci], sims[qi, ci]
    rank = S.LAMBDA * sc.astype(np.float32) - np.log(lens[qi].astype(np.float32) * lh[t].astype(np.float32))
    out = [[] for _ in range(nq)]
    for o in np.lexsort((-rank, qi)):
        q = qi[o]
        if len(out[q]) < top_k:
            out[q].append((int(t[o]), float(si[o]), int(sc[o]), float(rank[o])))
    return out


def test_ranking_pass_matches_lexsort(monkeypatch):
    import torch
    monkeypatch.setattr(S._lib, "check", lambda rc: None)
    rng = np.random.default_rng(1)
    for trial in range(60):
        nq, K, top_k = int(rng.integers(1, 40)), int(rng.integers(1, 60)), int(rng.integers(1, 15))
        n = rng.integers(0, K + 1, nq).astype(np.int32)
        tg = rng.integers(0, 50, nq * K).astype(np.int32)  # few targets and scores: many equal ranks
        sims = rng.random(nq * K).astype(np.float32)
        scores = rng.integers(0, 6, nq * K).astype(np.int32)
        mask = (rng.random(nq * K) < 0.7).astype(np.uint8)
        lens = rng.integers(1, 5, nq).astype(np.int32)
        lh = rng.integers(1, 5, 50).astype(np.int32)
        slot = types.SimpleNamespace(
            db=types.SimpleNamespace(lib=types.SimpleNamespace(ck_ctx_status=lambda *a: 0), lengths_host=lh),
            ctx=0, stream=types.SimpleNamespace(cuda_stream=0), max_cands=K, h_n=torch.from_numpy(n),
            h_targets=torch.from_numpy(tg), h_sims=torch.from_numpy(sims), h_scores=torch.from_numpy(scores),
            h_mask=torch.from_numpy(mask), batch=(nq, lens))
        got = S._Slot.results(slot, top_k)
        want = _lexsort_hits(nq, K, n, tg.reshape(nq, K), sims.reshape(nq, K), scores.reshape(nq, K),
                             mask.reshape(nq, K), lens, lh, top_k)
        assert [[(h.target, h.identity, h.score, h.rank) for h in g] for g in got] == want, trial


def test_batch_bytes_grows_with_queries_residues_and_candidates():
    from clustkit_gb300.search import batch_bytes
    db = types.SimpleNamespace(n=1000)
    q = [np.zeros(300, np.uint8)] * 4
    b4 = batch_bytes(db, q, 500)
    assert batch_bytes(db, q * 2, 500) == 2 * b4
    assert batch_bytes(db, q, 500) < batch_bytes(db, q, 600)
    assert batch_bytes(db, [np.zeros(301, np.uint8)] + q[1:], 500) == b4 + 1
    assert batch_bytes(db, [], 500) == 0
