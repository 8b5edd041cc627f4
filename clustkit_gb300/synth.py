"""Seeded synthetic protein families for tests and benchmarks.

No public dataset is used.  Sequences come from a family model built from
BLOSUM62 alone:

* background residue frequencies ``p`` and the scale ``lam`` are the ones the
  matrix itself implies: ``sum_b p_b exp(lam * S_ab) = 1`` for every residue
  ``a`` with ``sum_a p_a = 1`` (solved numerically below);
* substitution probabilities are the implied target frequencies
  ``P(b | a) = p_b exp(lam * S_ab)``;
* ancestors have lognormal lengths (median ``m``, sigma 0.5, clipped) or Pareto
  lengths, residues i.i.d. from ``p``;
* each descendant mutates every residue with its family's divergence
  (uniform in a range), drawing the new residue from ``P(b | a)``, and has
  indels at ``indel_rate`` per residue (half insertions of background
  residues, half deletions), each of geometric length with mean 3.

The output layout is clustkit's compact storage: ``flat`` uint8 codes 0..19,
``offsets`` int64, ``lengths`` int32 (clustkit/io.py:35-131).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .blosum import BLOSUM62


def _symmetric_blosum() -> np.ndarray:
    s = BLOSUM62.astype(np.float64)
    return np.round((s + s.T) / 2.0)


def implied_background() -> tuple[np.ndarray, float]:
    """Background frequencies and lambda implied by BLOSUM62."""
    S = _symmetric_blosum()
    ones = np.ones(S.shape[0])

    def p_of(lam: float) -> np.ndarray:
        return np.linalg.solve(np.exp(lam * S), ones)

    lo, hi = 0.2, 0.5  # sum(p) - 1 changes sign between these for BLOSUM62
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if (p_of(mid).sum() - 1.0) * (p_of(lo).sum() - 1.0) <= 0:
            hi = mid
        else:
            lo = mid
    lam = 0.5 * (lo + hi)
    p = p_of(lam)
    p = np.clip(p, 1e-6, None)
    return p / p.sum(), lam


def substitution_cdf() -> tuple[np.ndarray, np.ndarray]:
    p, lam = implied_background()
    S = _symmetric_blosum()
    cond = p[None, :] * np.exp(lam * S)
    cond /= cond.sum(axis=1, keepdims=True)
    return np.cumsum(p), np.cumsum(cond, axis=1)


@dataclass
class SequenceSet:
    flat: np.ndarray      # uint8 codes
    offsets: np.ndarray   # int64
    lengths: np.ndarray   # int32
    family: np.ndarray    # int32 family id per sequence

    @property
    def n(self) -> int:
        return int(self.lengths.shape[0])

    def seq(self, i: int) -> np.ndarray:
        o = int(self.offsets[i])
        return self.flat[o:o + int(self.lengths[i])]


def _draw(cdf: np.ndarray, u: np.ndarray) -> np.ndarray:
    return np.minimum(np.searchsorted(cdf, u, side="right"), cdf.shape[-1] - 1).astype(np.uint8)


def _lengths(rng, n, median, lo, hi, dist, sigma, pareto_alpha):
    if dist == "pareto":
        x = lo * (1.0 + rng.pareto(pareto_alpha, size=n))
    else:
        x = np.exp(np.log(median) + sigma * rng.standard_normal(n))
    return np.clip(np.rint(x), lo, hi).astype(np.int64)


def _gen_chunk(rng, n_fam, per_family, anc_len, div, bg_cdf, cond_cdf, indel_rate, indel_mean,
               lo, hi):
    """Descendants of ``n_fam`` families, vectorised over the whole chunk."""
    # ancestors, then per_family copies of each
    anc = _draw(bg_cdf, rng.random(int(anc_len.sum())))
    anc_off = np.concatenate([[0], np.cumsum(anc_len)])
    seq_anc = np.repeat(np.arange(n_fam), per_family)
    L = anc_len[seq_anc]
    starts = np.concatenate([[0], np.cumsum(L)[:-1]])
    idx = np.repeat(anc_off[seq_anc] - starts, L) + np.arange(int(L.sum()))
    res = anc[idx].copy()
    seq_of = np.repeat(np.arange(seq_anc.size), L)
    # substitutions: each residue mutates with its family's divergence
    mut = rng.random(res.size) < div[seq_anc][seq_of]
    if mut.any():
        a = res[mut]
        u = rng.random(a.size)
        res[mut] = np.minimum((cond_cdf[a] < u[:, None]).sum(1), 19).astype(np.uint8)
    # indels: events at rate indel_rate, geometric lengths; half delete the
    # residues from the event on, half insert background residues before it
    ev = np.nonzero(rng.random(res.size) < indel_rate)[0]
    ln = rng.geometric(1.0 / indel_mean, size=ev.size)
    is_del = rng.random(ev.size) < 0.5
    keep = np.ones(res.size, bool)
    if is_del.any():
        d0 = ev[is_del]
        d1 = np.minimum(d0 + ln[is_del], (starts + L)[seq_of[d0]])
        diff = np.zeros(res.size + 1, np.int64)
        np.add.at(diff, d0, 1)
        np.add.at(diff, d1, -1)
        keep = np.cumsum(diff[:-1]) == 0
    ins_at = np.repeat(ev[~is_del], ln[~is_del])
    ins_val = _draw(bg_cdf, rng.random(ins_at.size))
    seq_keep = seq_of[keep]
    out = np.insert(res[keep], np.searchsorted(np.nonzero(keep)[0], ins_at), ins_val)
    out_seq = np.insert(seq_keep, np.searchsorted(np.nonzero(keep)[0], ins_at), seq_of[ins_at])
    newL = np.bincount(out_seq, minlength=seq_anc.size)
    # clip to [lo, hi]: truncate long ones, pad short ones with background
    o_starts = np.concatenate([[0], np.cumsum(newL)[:-1]])
    pos_in = np.arange(out.size) - np.repeat(o_starts, newL)
    trunc = pos_in < hi
    out = out[trunc]
    newL = np.minimum(newL, hi)
    seqs_short = np.nonzero(newL < lo)[0]
    if seqs_short.size:
        pieces = np.split(out, np.cumsum(newL)[:-1])
        for i in seqs_short:
            pieces[i] = np.concatenate([pieces[i], _draw(bg_cdf, rng.random(lo - newL[i]))])
        newL = np.array([p.size for p in pieces])
        out = np.concatenate(pieces)
    return out.astype(np.uint8), newL.astype(np.int32)


def generate_families(n_families: int, per_family: int = 10, median: int = 300,
                      lo: int = 50, hi: int = 800, seed: int = 0, *,
                      length_dist: str = "lognormal", sigma: float = 0.5,
                      pareto_alpha: float = 1.5, divergence=(0.10, 0.70),
                      indel_rate: float = 0.05, indel_mean: float = 3.0,
                      chunk: int = 5000) -> SequenceSet:
    """``n_families`` ancestors, each replaced by ``per_family`` descendants."""
    rng = np.random.default_rng(seed)
    bg_cdf, cond_cdf = substitution_cdf()
    anc_len = _lengths(rng, n_families, median, lo, hi, length_dist, sigma, pareto_alpha)
    div = rng.uniform(*divergence, size=n_families)
    flats, lens = [], []
    for f0 in range(0, n_families, chunk):
        f1 = min(n_families, f0 + chunk)
        fl, ln = _gen_chunk(rng, f1 - f0, per_family, anc_len[f0:f1], div[f0:f1], bg_cdf, cond_cdf,
                            indel_rate, indel_mean, lo, hi)
        flats.append(fl)
        lens.append(ln)
    lengths = np.concatenate(lens) if lens else np.zeros(0, np.int32)
    flat = np.concatenate(flats) if flats else np.zeros(0, np.uint8)
    offsets = np.zeros(lengths.size, dtype=np.int64)
    if lengths.size > 1:
        offsets[1:] = np.cumsum(lengths[:-1], dtype=np.int64)
    fam = np.repeat(np.arange(n_families, dtype=np.int32), per_family)
    return SequenceSet(flat=flat, offsets=offsets, lengths=lengths, family=fam)


def random_sequences(n: int, median: int = 300, lo: int = 50, hi: int = 800, seed: int = 0,
                     length_dist: str = "lognormal") -> SequenceSet:
    """Unrelated background sequences (one per family)."""
    return generate_families(n, 1, median, lo, hi, seed, length_dist=length_dist,
                             divergence=(0.0, 0.0), indel_rate=0.0)


def mixed_pairs(seqs: SequenceSet, n_pairs: int, seed: int = 0, within_frac: float = 0.5,
                min_ratio: float = 0.0) -> np.ndarray:
    """Candidate pairs, ``within_frac`` of them inside a family, the rest random,
    keeping only pairs whose length ratio (shorter/longer) is >= ``min_ratio``."""
    rng = np.random.default_rng(seed)
    fam = seqs.family
    L = seqs.lengths
    n = seqs.n
    order = np.argsort(fam, kind="stable")
    fam_sorted = fam[order]
    starts = np.searchsorted(fam_sorted, fam_sorted, side="left")
    ends = np.searchsorted(fam_sorted, fam_sorted, side="right")
    out = []
    need_w = int(round(n_pairs * within_frac))
    need_r = n_pairs - need_w
    got_w = got_r = 0
    while got_w < need_w or got_r < need_r:
        batch = max(1024, 2 * (need_w + need_r - got_w - got_r))
        if got_w < need_w:
            k = rng.integers(0, n, size=batch)
            s, e = starts[k], ends[k]
            ok = (e - s) > 1
            k, s, e = k[ok], s[ok], e[ok]
            j = order[s + rng.integers(0, np.maximum(e - s, 1))]
            i = order[k]
            p = np.stack([i, j], axis=1)
            p = p[p[:, 0] != p[:, 1]]
            r = np.minimum(L[p[:, 0]], L[p[:, 1]]) / np.maximum(L[p[:, 0]], L[p[:, 1]])
            p = p[r >= min_ratio][: need_w - got_w]
            out.append(p)
            got_w += p.shape[0]
        if got_r < need_r:
            p = rng.integers(0, n, size=(batch, 2))
            p = p[p[:, 0] != p[:, 1]]
            r = np.minimum(L[p[:, 0]], L[p[:, 1]]) / np.maximum(L[p[:, 0]], L[p[:, 1]])
            p = p[r >= min_ratio][: need_r - got_r]
            out.append(p)
            got_r += p.shape[0]
    pairs = np.concatenate(out).astype(np.int32)
    return pairs[rng.permutation(pairs.shape[0])]
