"""Align-phase entry points, drop-in for clustkit's ``clustkit.pairwise``.

Same names, arguments, return types and pass/fail rules as clustkit
(clustkit/pairwise.py); the arithmetic runs in libckgpu.so on the GPU:

* ``compute_pairwise_alignment``  -- clustkit/pairwise.py:1047-1208
* ``_batch_sw_c``                 -- clustkit/pairwise.py:69-108
* ``_jaccard_prefilter``          -- clustkit/pairwise.py:949-1001
* ``compute_pairwise_jaccard``    -- clustkit/pairwise.py:1623-1654
* ``jaccard_from_sketches``       -- clustkit/pairwise.py:1615-1620
* ``batch_sw``                    -- the full per-pair output (score, identity
  numerator and denominator, pass/fail) under any of clustkit's three rules.

clustkit decides pass/fail differently on its three Smith-Waterman paths, and
``compute_pairwise_alignment`` reproduces whichever one the arguments select:
``device="cpu"`` with ``use_c_sw=True`` is the C path (identity >= t), with
``use_c_sw=False`` the Numba path (score > 0 and identity >= t); a GPU device
string is clustkit's CuPy path (length-ratio filter, identity >= t, result
ordered by the longer length).  The global-alignment (NW) branches are not
part of this library.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from ._lib import ENGINE_BATCHED, ENGINE_PLAIN, PASS_CPU, PASS_CUPY, PASS_NUMBA, PASS_SCORE
from .blosum import BLOSUM62

__all__ = [
    "batch_sw", "compute_pairwise_alignment", "_batch_sw_c", "_jaccard_prefilter",
    "compute_pairwise_jaccard", "jaccard_from_sketches", "batch_jaccard", "BLOSUM62",
    "PASS_CPU", "PASS_NUMBA", "PASS_CUPY", "PASS_SCORE", "ENGINE_BATCHED", "ENGINE_PLAIN",
]


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def batch_sw(pairs, flat_sequences, offsets, lengths, band_width: int = 100,
             sub_matrix=BLOSUM62, threshold: float = 0.0, diag_hints=None,
             pass_rule: int = PASS_CPU, engine: int = ENGINE_BATCHED) -> dict:
    """Banded SW over every pair (clustkit/csrc/sw_align.c:182-266 semantics).

    Returns dict of numpy arrays: ``sims`` float32 identity, ``scores`` int32,
    ``matches`` int32 (identity numerator), ``shorter`` int32 (denominator),
    ``mask`` bool pass/fail under ``pass_rule``.
    """
    lib = _lib.load()
    _lib.require_gpu()
    pairs = _c(pairs, np.int32).reshape(-1, 2)
    flat = _c(flat_sequences, np.uint8).reshape(-1)
    offsets = _c(offsets, np.int64).reshape(-1)
    lengths = _c(lengths, np.int32).reshape(-1)
    if offsets.shape[0] != lengths.shape[0]:
        raise ValueError("offsets and lengths differ in length")
    sub = _c(sub_matrix, np.int8).reshape(-1)
    if sub.shape[0] != 400:
        raise ValueError("sub_matrix must be 20x20")
    hints = None if diag_hints is None else _c(diag_hints, np.int32).reshape(-1)
    if hints is not None and hints.shape[0] != pairs.shape[0]:
        raise ValueError("diag_hints must have one entry per pair")
    M = pairs.shape[0]
    sims = np.empty(M, np.float32)
    scores = np.empty(M, np.int32)
    matches = np.empty(M, np.int32)
    shorter = np.empty(M, np.int32)
    mask = np.empty(M, np.uint8)
    _lib.check(lib.ck_sw_batch(
        _lib.ptr(pairs), M, _lib.ptr(flat), flat.shape[0], _lib.ptr(offsets), _lib.ptr(lengths),
        lengths.shape[0], int(band_width), _lib.ptr(sub), float(np.float32(threshold)),
        _lib.ptr(hints), int(pass_rule), int(engine),
        _lib.ptr(sims), _lib.ptr(scores), _lib.ptr(matches), _lib.ptr(shorter), _lib.ptr(mask)))
    return {"sims": sims, "scores": scores, "matches": matches, "shorter": shorter,
            "mask": mask.astype(bool)}


def _batch_sw_c(pairs, flat_sequences, offsets, lengths, threshold, band_width, sub_matrix,
                n_threads=4):
    """clustkit/pairwise.py:69-108: returns ``(sims, mask)`` with
    ``mask = sims >= threshold`` (float32 comparison)."""
    r = batch_sw(pairs, flat_sequences, offsets, lengths, band_width, sub_matrix, threshold,
                 pass_rule=PASS_CPU)
    return r["sims"], r["mask"]


def batch_jaccard(pairs, sketches, floor: float = 0.0):
    """Per-pair merge-walk Jaccard (clustkit/pairwise.py:1598-1612): ``(sims, mask)``."""
    lib = _lib.load()
    _lib.require_gpu()
    pairs = _c(pairs, np.int32).reshape(-1, 2)
    sk = _c(sketches, np.uint64)
    if sk.ndim != 2:
        raise ValueError("sketches must be (N, s)")
    M = pairs.shape[0]
    sims = np.empty(M, np.float32)
    mask = np.empty(M, np.uint8)
    _lib.check(lib.ck_jaccard(_lib.ptr(pairs), M, _lib.ptr(sk), sk.shape[0], sk.shape[1],
                              float(np.float32(floor)), _lib.ptr(sims), _lib.ptr(mask)))
    return sims, mask.astype(bool)


def jaccard_from_sketches(sketch_a: np.ndarray, sketch_b: np.ndarray) -> float:
    sk = np.stack([_c(sketch_a, np.uint64), _c(sketch_b, np.uint64)])
    sims, _ = batch_jaccard(np.array([[0, 1]], np.int32), sk)
    return float(sims[0])


def _jaccard_prefilter(candidate_pairs, sketches, threshold, min_filter_rate: float = 0.05):
    """clustkit/pairwise.py:949-1001, including its 2000-pair cost check
    drawn with ``np.random.RandomState(0)``."""
    m = len(candidate_pairs)
    if m == 0:
        return np.ones(0, dtype=np.bool_)
    jaccard_floor = max(0.001, 0.3 * threshold ** 5)
    sample_size = min(2000, m)
    if sample_size < m:
        rng = np.random.RandomState(0)
        sample_idx = rng.choice(m, size=sample_size, replace=False)
        sample_sims, _ = batch_jaccard(np.asarray(candidate_pairs)[sample_idx], sketches)
        est_filter_rate = float(np.mean(sample_sims < jaccard_floor))
        if est_filter_rate < min_filter_rate:
            return None
    sims, _ = batch_jaccard(candidate_pairs, sketches)
    return sims >= jaccard_floor


def compute_pairwise_jaccard(candidate_pairs, sketches, threshold, device: str = "0"):
    """clustkit/pairwise.py:1623-1654."""
    if len(candidate_pairs) == 0:
        return np.empty((0, 2), dtype=np.int32), np.empty(0, dtype=np.float32)
    sims, mask = batch_jaccard(candidate_pairs, sketches, threshold)
    pairs = np.asarray(candidate_pairs)
    return pairs[mask], sims[mask]


def _flat_from_padded(encoded_sequences, lengths):
    n = len(lengths)
    offsets = np.zeros(n, dtype=np.int64)
    if n > 1:
        offsets[1:] = np.cumsum(np.asarray(lengths[:-1], dtype=np.int64))
    flat = np.empty(int(np.sum(lengths)), dtype=np.uint8)
    for k in range(n):
        ln = int(lengths[k])
        flat[offsets[k]:offsets[k] + ln] = encoded_sequences[k, :ln]
    return flat, offsets


def _gpu_semantics_run(pairs, flat, offsets, lengths, threshold, band_width):
    """clustkit's CuPy path (pairwise.py:1458-1557): pairs stably sorted by the
    longer length, length-ratio filter, identity >= t, kept pairs in that order."""
    max_lens = np.maximum(lengths[pairs[:, 0]], lengths[pairs[:, 1]])
    order = np.argsort(max_lens, kind="mergesort")
    sp = pairs[order]
    r = batch_sw(sp, flat, offsets, lengths, band_width, BLOSUM62, threshold, pass_rule=PASS_CUPY)
    return sp[r["mask"]], r["sims"][r["mask"]]


def compute_pairwise_alignment(candidate_pairs, encoded_sequences, lengths, threshold,
                               band_width: int = 50, device: str = "cpu", mode: str = "protein",
                               sketches=None, flat_sequences=None, offsets=None,
                               use_sw: bool = False, use_c_sw: bool = False, n_threads: int = 4,
                               refine_global_margin: float = 0.0):
    """clustkit/pairwise.py:1047-1208.  Returns ``(filtered_pairs (K,2) int32,
    identities (K,) float32)`` in clustkit's order."""
    if len(candidate_pairs) == 0:
        return np.empty((0, 2), dtype=np.int32), np.empty(0, dtype=np.float32)
    candidate_pairs = np.asarray(candidate_pairs)
    lengths = np.asarray(lengths)

    if sketches is not None:
        jaccard_mask = _jaccard_prefilter(candidate_pairs, sketches, threshold)
        if jaccard_mask is not None:
            candidate_pairs = candidate_pairs[jaccard_mask]
            if len(candidate_pairs) == 0:
                return np.empty((0, 2), dtype=np.int32), np.empty(0, dtype=np.float32)

    sort_key = np.minimum(candidate_pairs[:, 0], candidate_pairs[:, 1])
    candidate_pairs = candidate_pairs[np.argsort(sort_key, kind="mergesort")]

    if flat_sequences is None or offsets is None:
        if encoded_sequences is None:
            raise ValueError("need flat_sequences+offsets or encoded_sequences")
        flat_sequences, offsets = _flat_from_padded(encoded_sequences, lengths)

    if refine_global_margin and refine_global_margin > 0:
        raise NotImplementedError("refine_global_margin uses global (NW) alignment, which this "
                                  "library does not implement")

    if device != "cpu":
        # clustkit's GPU branch (single device, "auto" or "0,1"): CuPy semantics.
        # clustkit's "auto" times one CPU thread against its GPU path and, with
        # CuPy present, lands on the GPU (pairwise.py:853-946); this library
        # takes that outcome without timing anything.
        if "," in str(device):
            n_dev = len(str(device).split(","))
            m = len(candidate_pairs)
            chunk = (m + n_dev - 1) // n_dev
            parts = [_gpu_semantics_run(candidate_pairs[s:s + chunk], flat_sequences, offsets,
                                        lengths, threshold, band_width)
                     for s in range(0, m, chunk)]
            parts = [p for p in parts if len(p[0]) > 0]
            if not parts:
                return np.empty((0, 2), dtype=np.int32), np.empty(0, dtype=np.float32)
            return (np.concatenate([p[0] for p in parts], axis=0),
                    np.concatenate([p[1] for p in parts]))
        return _gpu_semantics_run(candidate_pairs, flat_sequences, offsets, lengths, threshold,
                                  band_width)

    if not use_sw:
        raise NotImplementedError("global (NW) alignment is not part of this library; "
                                  "call with use_sw=True")
    rule = PASS_CPU if use_c_sw else PASS_NUMBA
    r = batch_sw(candidate_pairs, flat_sequences, offsets, lengths, band_width, BLOSUM62,
                 threshold, pass_rule=rule)
    mask = r["mask"]
    return candidate_pairs[mask], r["sims"][mask]
