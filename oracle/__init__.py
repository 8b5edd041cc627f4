"""CPU oracle for the Align-phase / sketch path.

TEST INFRASTRUCTURE ONLY.  Import this from tests/, __graft_entry__.smoke() or
bench.py's cpu_baseline / reference legs -- never from the product package.
It is the checker the CUDA path is compared against, not a fallback.

``liboracle.so`` (built from ``oracle/oracle.c``) restates, function by
function (reference paths relative to the clustkit project root):

* ``sw_batch``  -- clustkit/csrc/sw_align.c:25-266 (banded Smith-Waterman,
  BLOSUM62, gaps -11/-1, match-count provenance, first-max tie rule);
* ``sketches``  -- clustkit/sketch.py:17-109 (fmix64 bottom-s MinHash);
* ``jaccard``   -- clustkit/pairwise.py:1564-1612 (merge-walk Jaccard);
* ``kmer_candidates_batch`` -- clustkit/csrc/kmer_score.c:195-470 (the C
  k-mer scorer: Phase A, top-K, Phase B diagonal runs and hints), from
  ``oracle/kmer_oracle.c``;
* ``similar_candidates_batch`` -- clustkit/kmer_index.py:1187-1328 (the
  BLOSUM62 similar-5-mer scorer, clustkit's default search scoring), from
  ``oracle/kmer_oracle.c``.

``ref_sw_batch`` calls the reference's own sw_align.c, compiled from source
into ``oracle/_ref/`` by ``oracle/build.py`` (only where the reference
checkout is mounted).  Parity of the restatement is pinned against it and
against the committed golden fixtures in ``tests/golden/``.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build as _build

_lib = None
_ref = None

_P = ctypes.c_void_p


def _load():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        lib = ctypes.CDLL(str(path))
        lib.or_sw_batch.restype = None
        lib.or_sw_batch.argtypes = [_P, _P, _P, _P, ctypes.c_int64, ctypes.c_int32, _P, _P,
                                    _P, _P, _P, _P, _P]
        lib.or_sketch.restype = None
        lib.or_sketch.argtypes = [_P, _P, _P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_int32, ctypes.c_uint64, _P]
        lib.or_jaccard.restype = None
        lib.or_jaccard.argtypes = [_P, _P, ctypes.c_int64, ctypes.c_int32, _P]
        lib.or_kmer_candidates.restype = None
        lib.or_kmer_candidates.argtypes = [_P, _P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P, _P, _P,
                                           ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P, _P, _P, _P]
        lib.or_set_num_threads.restype = None
        lib.or_similar_candidates.restype = None
        lib.or_similar_candidates.argtypes = [_P, _P, _P, ctypes.c_int32, _P, ctypes.c_int32, _P, _P, _P,
                                              ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                              _P, _P, _P]
        lib.or_set_num_threads.argtypes = [ctypes.c_int32]
        lib.or_max_threads.restype = ctypes.c_int32
        lib.or_fmix64_export.restype = ctypes.c_uint64
        lib.or_fmix64_export.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        _lib = lib
    return _lib


def set_num_threads(n: int) -> None:
    _load().or_set_num_threads(int(n))


def max_threads() -> int:
    return int(_load().or_max_threads())


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def sw_batch(pairs, flat, offsets, lengths, band_width, sub_matrix, diag_hints=None):
    """Returns dict(sims float32, scores int32, matches int32, shorter int32, mask uint8)."""
    lib = _load()
    pairs = _c(pairs, np.int32).reshape(-1, 2)
    flat = _c(flat, np.uint8)
    offsets = _c(offsets, np.int64)
    lengths = _c(lengths, np.int32)
    sub = _c(sub_matrix, np.int8).reshape(-1)
    M = pairs.shape[0]
    out = {
        "sims": np.empty(M, np.float32),
        "scores": np.empty(M, np.int32),
        "matches": np.empty(M, np.int32),
        "shorter": np.empty(M, np.int32),
        "mask": np.empty(M, np.uint8),
    }
    hints = None if diag_hints is None else _c(diag_hints, np.int32)
    lib.or_sw_batch(pairs.ctypes.data, flat.ctypes.data, offsets.ctypes.data, lengths.ctypes.data,
                    M, int(band_width), sub.ctypes.data,
                    None if hints is None else hints.ctypes.data,
                    out["sims"].ctypes.data, out["scores"].ctypes.data, out["matches"].ctypes.data,
                    out["shorter"].ctypes.data, out["mask"].ctypes.data)
    return out


def kmer_candidates_batch(q_flat, q_offsets, q_lengths, k, alpha, kmer_offsets, kmer_entries, kmer_freqs,
                          freq_thresh, num_db, min_total_hits, min_diag_hits, diag_bin_width, max_cands,
                          phase_a_topk):
    """Per query (ids, scores, diags) of the C k-mer scorer's restatement,
    all queries in one OpenMP call."""
    lib = _load()
    q_flat = _c(q_flat if len(q_flat) else np.zeros(1, np.uint8), np.uint8)
    q_offsets, q_lengths = _c(q_offsets, np.int64), _c(q_lengths, np.int32)
    off, ent, fr = _c(kmer_offsets, np.int64), _c(kmer_entries, np.int64), _c(kmer_freqs, np.int32)
    nq = len(q_lengths)
    mc = int(max_cands)
    t = np.zeros((max(nq, 1), mc), np.int32)
    s = np.zeros_like(t)
    d = np.zeros_like(t)
    n = np.zeros(max(nq, 1), np.int32)
    lib.or_kmer_candidates(q_flat.ctypes.data, q_offsets.ctypes.data, q_lengths.ctypes.data, nq, int(k), int(alpha),
                           off.ctypes.data, ent.ctypes.data, fr.ctypes.data, int(freq_thresh), int(num_db),
                           int(min_total_hits), int(min_diag_hits), int(diag_bin_width), mc, int(phase_a_topk),
                           t.ctypes.data, s.ctypes.data, d.ctypes.data, n.ctypes.data)
    return [(t[i, :n[i]].copy(), s[i, :n[i]].copy(), d[i, :n[i]].copy()) for i in range(nq)]


def similar_candidates_batch(q_flat, q_offsets, q_lengths, sub, thresh, kmer_offsets, kmer_entries, kmer_freqs,
                             freq_thresh, num_db, min_total_hits, max_cands):
    """Per query (ids, scores) of the similar-5-mer scorer's restatement
    (k = 5 index over 20 codes), all queries in one OpenMP call."""
    lib = _load()
    q_flat = _c(q_flat if len(q_flat) else np.zeros(1, np.uint8), np.uint8)
    q_offsets, q_lengths = _c(q_offsets, np.int64), _c(q_lengths, np.int32)
    off, ent, fr = _c(kmer_offsets, np.int64), _c(kmer_entries, np.int64), _c(kmer_freqs, np.int32)
    S = _c(np.asarray(sub).reshape(-1), np.int8)
    if int(thresh) < 1:
        raise ValueError("the similar-k-mer threshold must be >= 1")
    nq = len(q_lengths)
    mc = int(max_cands)
    t = np.zeros((max(nq, 1), mc), np.int32)
    s = np.zeros_like(t)
    n = np.zeros(max(nq, 1), np.int32)
    lib.or_similar_candidates(q_flat.ctypes.data, q_offsets.ctypes.data, q_lengths.ctypes.data, nq, S.ctypes.data,
                              int(thresh), off.ctypes.data, ent.ctypes.data, fr.ctypes.data, int(freq_thresh),
                              int(num_db), int(min_total_hits), mc, t.ctypes.data, s.ctypes.data, n.ctypes.data)
    return [(t[i, :n[i]].copy(), s[i, :n[i]].copy()) for i in range(nq)]


def sketches(flat, offsets, lengths, k, s, alphabet=20, seed=42):
    lib = _load()
    flat = _c(flat, np.uint8)
    offsets = _c(offsets, np.int64)
    lengths = _c(lengths, np.int32)
    N = lengths.shape[0]
    out = np.empty((N, s), np.uint64)
    lib.or_sketch(flat.ctypes.data, offsets.ctypes.data, lengths.ctypes.data, N, int(k), int(s),
                  int(alphabet), int(seed), out.ctypes.data)
    return out


def jaccard(pairs, sketch_matrix):
    lib = _load()
    pairs = _c(pairs, np.int32).reshape(-1, 2)
    sk = _c(sketch_matrix, np.uint64)
    M = pairs.shape[0]
    out = np.empty(M, np.float32)
    lib.or_jaccard(pairs.ctypes.data, sk.ctypes.data, M, int(sk.shape[1]), out.ctypes.data)
    return out


def fmix64(key: int, seed: int = 42) -> int:
    return int(_load().or_fmix64_export(int(key), int(seed)))


def ref_available() -> bool:
    return _load_ref() is not None


def _load_ref():
    global _ref
    if _ref is None:
        path = _build.build_reference()
        if path is None:
            return None
        lib = ctypes.CDLL(str(path))
        # argtypes as clustkit/pairwise.py:50-58 binds them
        lib.batch_sw_align_c.restype = None
        lib.batch_sw_align_c.argtypes = [_P, _P, _P, _P, ctypes.c_int32, ctypes.c_int32, _P,
                                         ctypes.c_float, _P, _P, _P, _P]
        lib.sw_set_num_threads.restype = None
        lib.sw_set_num_threads.argtypes = [ctypes.c_int32]
        _ref = lib
    return _ref


def ref_sw_batch(pairs, flat, offsets, lengths, band_width, sub_matrix, threshold=0.0,
                 diag_hints=None, n_threads=None):
    """The reference's batch_sw_align_c itself.  Returns dict(sims, scores, mask)."""
    lib = _load_ref()
    if lib is None:
        raise RuntimeError("reference sources not mounted; oracle/_ref unavailable")
    if n_threads:
        lib.sw_set_num_threads(int(n_threads))
    pairs = _c(pairs, np.int32).reshape(-1)
    flat = _c(flat, np.uint8)
    offsets = _c(offsets, np.int64)
    lengths = _c(lengths, np.int32)
    sub = _c(sub_matrix, np.int8).reshape(-1)
    M = pairs.shape[0] // 2
    sims = np.empty(M, np.float32)
    scores = np.empty(M, np.int32)
    mask = np.empty(M, np.uint8)
    hints = None if diag_hints is None else _c(diag_hints, np.int32)
    lib.batch_sw_align_c(pairs.ctypes.data, flat.ctypes.data, offsets.ctypes.data,
                         lengths.ctypes.data, M, int(band_width), sub.ctypes.data,
                         np.float32(threshold), None if hints is None else hints.ctypes.data,
                         sims.ctypes.data, scores.ctypes.data, mask.ctypes.data)
    return {"sims": sims, "scores": scores, "mask": mask}
