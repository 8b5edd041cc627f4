"""CPU restatement of clustkit's k-mer search path (numpy).

TEST INFRASTRUCTURE ONLY -- the checker for clustkit_gb300.search, never the
thing measured or shipped.  Reference paths are relative to the clustkit
project root.

* ``build_kmer_index``      -- clustkit/kmer_index.py:77-166
* ``compute_freq_threshold`` -- clustkit/kmer_index.py:451-463
* ``phase_a``               -- clustkit/kmer_index.py:470-534 (Phase A only,
  the path taken when min_diag_hits <= 1, :832-850) with the per-query cap of
  :893-902: above the cap the top targets in score order, ties to the lower
  target id (clustkit's ``np.argsort(-scores)`` leaves tie order to numpy's
  unstable quicksort)
* ``phase_a_similar``       -- the k = 5 BLOSUM62-neighbour scoring of
  clustkit/kmer_index.py:1187-1291 (every 5-mer whose column-sum score against
  the query 5-mer is >= the threshold adds that score per posting) with the
  cap of :1320-1328
* ``kmer_candidates``       -- the C scorer's per-query candidates
  (clustkit/csrc/kmer_score.c:195-415, ``score_query_full``): Phase A, the
  top ``phase_a_topk`` by (count desc, id asc), Phase B -- per target the
  longest run of hits on one diagonal bin ``(tpos - qpos + qlen) //
  diag_bin_width``, first bin on ties -- kept at >= ``min_diag_hits``, the
  diagonal hint ``bin * width - qlen + width // 2``, and the ``max_cands``
  cap by (score desc, id asc)
* ``rank_hits``             -- the E-value-style rank of
  clustkit/kmer_index.py:2318-2323 and the top-k collection of
  clustkit/search.py:727-800
"""
from __future__ import annotations

import numpy as np


def kmer_values(seq: np.ndarray, k: int, alpha: int):
    """(values, valid) for every k-mer start of one sequence."""
    L = len(seq)
    if L < k:
        return np.empty(0, np.int64), np.empty(0, bool)
    s = seq.astype(np.int64)
    n = L - k + 1
    v = np.zeros(n, np.int64)
    ok = np.ones(n, bool)
    for m in range(k):
        c = s[m:m + n]
        ok &= c < alpha
        v = v * alpha + c
    return v, ok


def build_kmer_index(flat, offsets, lengths, k: int, alpha: int = 20):
    """(kmer_offsets int64[alpha^k+1], kmer_entries int64[total], kmer_freqs int32[alpha^k])."""
    nk = alpha ** k
    keys, vals = [], []
    for i in range(len(lengths)):
        L = int(lengths[i])
        o = int(offsets[i])
        v, ok = kmer_values(flat[o:o + L], k, alpha)
        pos = np.nonzero(ok)[0]
        keys.append(v[ok])
        vals.append((np.int64(i) << 32) | pos.astype(np.int64))
    keys = np.concatenate(keys) if keys else np.empty(0, np.int64)
    vals = np.concatenate(vals) if vals else np.empty(0, np.int64)
    order = np.argsort(keys, kind="stable")  # (sequence, position) order kept inside a k-mer
    freqs = np.bincount(keys, minlength=nk).astype(np.int32)
    offs = np.zeros(nk + 1, np.int64)
    np.cumsum(freqs, out=offs[1:])
    return offs, vals[order], freqs


def compute_freq_threshold(kmer_freqs, num_sequences: int, percentile: float = 99.5) -> int:
    nonzero = kmer_freqs[kmer_freqs > 0]
    if len(nonzero) == 0:
        return int(num_sequences)
    pctl = int(np.percentile(nonzero, percentile))
    return int(max(pctl, max(100, num_sequences // 200)))


def phase_a(query, k, alpha, kmer_offsets, kmer_entries, kmer_freqs, freq_thresh, num_db,
            min_total_hits, top_k):
    """Surviving target ids (ascending) and their hit counts, at most top_k."""
    v, ok = kmer_values(np.asarray(query), k, alpha)
    counts = np.zeros(num_db, np.int64)
    for val in v[ok]:
        if kmer_freqs[val] > freq_thresh:
            continue
        t = (kmer_entries[kmer_offsets[val]:kmer_offsets[val + 1]] >> 32).astype(np.int64)
        np.add.at(counts, t, 1)
    counts = np.minimum(counts, 32767)
    ids = np.nonzero(counts >= min_total_hits)[0]
    sc = counts[ids]
    return _cap(ids, sc, top_k)


def _cap(ids, sc, top_k):
    """Survivors in id order; above top_k the top_k by score in score order
    (clustkit's argsort(-scores), kmer_index.py:893-899), ties by id."""
    if len(ids) > top_k:
        order = np.lexsort((ids, -sc))[:top_k]
        return ids[order].astype(np.int32), sc[order].astype(np.int32)
    return ids.astype(np.int32), sc.astype(np.int32)


def neighbours_k5(q5, sub, T):
    """(values, scores) of every 5-mer with sum_i sub[q_i, a_i] >= T."""
    S = np.asarray(sub, np.int64)
    s = (S[q5[0]][:, None, None, None, None] + S[q5[1]][None, :, None, None, None]
         + S[q5[2]][None, None, :, None, None] + S[q5[3]][None, None, None, :, None]
         + S[q5[4]][None, None, None, None, :])
    idx = np.nonzero(s.reshape(-1) >= T)[0]
    return idx.astype(np.int64), s.reshape(-1)[idx]


def phase_a_similar(query, kmer_offsets, kmer_entries, kmer_freqs, freq_thresh, num_db, min_total_hits,
                    top_k, sub, T):
    """Survivors (ids, score-weighted counts) of the neighbour scoring, capped as above."""
    q = np.asarray(query)
    counts = np.zeros(num_db, np.int64)
    for p in range(len(q) - 4):
        q5 = q[p:p + 5].astype(np.int64)
        if (q5 >= 20).any():
            continue
        vals, sc = neighbours_k5(q5, sub, T)
        f = kmer_freqs[vals]
        ok = (f > 0) & (f <= freq_thresh)
        for v, w in zip(vals[ok], sc[ok]):
            t = (kmer_entries[kmer_offsets[v]:kmer_offsets[v + 1]] >> 32).astype(np.int64)
            np.add.at(counts, t, int(w))
    ids = np.nonzero(counts >= min_total_hits)[0]
    return _cap(ids, counts[ids], top_k)


def rank_hits(pairs, sims, scores, q_lengths, t_lengths, nq, top_k):
    """Top-k hits per query: list of lists of (target, identity, rank score).

    rank = float32(0.267) * score - log(qlen * tlen) in float32; ordering is
    numpy's stable lexsort on (-rank, query), as clustkit does."""
    hits = [[] for _ in range(nq)]
    if len(pairs) == 0:
        return hits
    lam = np.float32(0.267)
    ql = q_lengths[pairs[:, 0]].astype(np.float32)
    tl = t_lengths[pairs[:, 1]].astype(np.float32)
    rank = lam * scores.astype(np.float32) - np.log(ql * tl)
    order = np.lexsort((-rank, pairs[:, 0]))
    for idx in order:
        q = int(pairs[idx, 0])
        if len(hits[q]) < top_k:
            hits[q].append((int(pairs[idx, 1]), float(sims[idx]), float(rank[idx])))
    return hits


def _top_by_score(ids, sc, k):
    """kmer_score.c:148-193: all in the given order when n <= k, else the top k by
    (score desc, id asc) in that order."""
    if len(ids) <= k:
        return np.arange(len(ids))
    return np.lexsort((ids, -sc))[:k]


def kmer_candidates(query, k, alpha, kmer_offsets, kmer_entries, kmer_freqs, freq_thresh, num_db,
                    min_total_hits, min_diag_hits, diag_bin_width, max_cands, phase_a_topk):
    """(ids, scores, diags); diags are 0 when min_diag_hits <= 1 (the C scorer leaves them unset)."""
    q = np.asarray(query)
    v, ok = kmer_values(q, k, alpha)
    counts = np.zeros(num_db, np.int64)
    post = []  # (qpos, entries) of the valid, frequency-capped k-mers
    for p in np.nonzero(ok)[0]:
        val = v[p]
        if kmer_freqs[val] > freq_thresh:
            continue
        e = kmer_entries[kmer_offsets[val]:kmer_offsets[val + 1]]
        np.add.at(counts, (e >> 32).astype(np.int64), 1)
        post.append((int(p), e))
    counts = np.minimum(counts, 32767)
    ids = np.nonzero(counts >= min_total_hits)[0]
    sc = counts[ids]
    empty = np.empty(0, np.int32)
    if len(ids) == 0:
        return empty, empty, empty
    if min_diag_hits <= 1:
        o = _top_by_score(ids, sc, max_cands)
        return ids[o].astype(np.int32), sc[o].astype(np.int32), np.zeros(len(o), np.int32)
    sel = ids[_top_by_score(ids, sc, phase_a_topk)]
    in_sel = np.zeros(num_db, bool)
    in_sel[sel] = True
    qlen = len(q)
    runs = {}
    for p, e in post:
        t = (e >> 32).astype(np.int64)
        m = in_sel[t]
        tpos = (e[m] & 0xFFFFFFFF).astype(np.int64)
        for tid, b in zip(t[m], (tpos - p + qlen) // diag_bin_width):
            runs[(int(tid), int(b))] = runs.get((int(tid), int(b)), 0) + 1
    best = {}
    for (tid, b) in sorted(runs):
        c = runs[(tid, b)]
        if tid not in best or c > best[tid][0]:
            best[tid] = (c, b)
    fid = np.array([t for t in sorted(best) if best[t][0] >= min_diag_hits], np.int64)
    if len(fid) == 0:
        return empty, empty, empty
    fsc = np.array([best[t][0] for t in fid], np.int64)
    fdg = np.array([best[t][1] * diag_bin_width - qlen + diag_bin_width // 2 for t in fid], np.int64)
    o = _top_by_score(fid, fsc, max_cands)
    return fid[o].astype(np.int32), fsc[o].astype(np.int32), fdg[o].astype(np.int32)
