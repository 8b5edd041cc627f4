"""Query-vs-database search on the GPU, batch and continuous-batching serving.

Mirrors the k-mer search of clustkit (clustkit/kmer_index.py:1475-2349).
With ``min_diag_hits <= 1``: k-mer inverted index
(k = 5, clustkit's CSR layout, kmer_index.py:117-166); either BLOSUM62
similar-k-mer scoring (``kmer_score_thresh > 0``, clustkit's default 13:
every 5-mer scoring >= the threshold against a query 5-mer adds its score,
:1187-1328) or exact Phase-A hit counting (``kmer_score_thresh = 0``,
:451-534), both with the frequency cap; at most ``max_cands`` candidates per
query (:893-902, :1320-1328); banded Smith-Waterman with a positive score as
pass (:2271-2280, pairwise.py:636-681); rank ``0.267 * score - ln(qlen *
tlen)`` (:2318-2323) and the top-k hits per query (clustkit/search.py:727-800).

With ``min_diag_hits >= 2`` (exact k-mers) or ``use_c_scoring`` the
candidates come from the device twin of clustkit's C k-mer scorer
(clustkit/csrc/kmer_score.c:195-470; its Numba two-stage scorer,
kmer_index.py:262-410, selects the same targets): Phase A, the top
``phase_a_topk`` by hits, Phase B's longest diagonal-bin run per target and
its diagonal hint.  ``use_c_sw`` aligns with clustkit's C SW settings
(kmer_index.py:2230-2266): band ``c_sw_band_width`` and, with
``use_c_scoring``, the Phase-B hints as band centres.

Differences, by design:
* candidates above the cap are the top ones by score, in score order as
  clustkit gives them, with ties to the lower target id (clustkit's order
  among equal scores is numpy's unstable quicksort);
* the band width is fixed when the database is loaded
  (``max(20, 0.3 * p95(database lengths))``) instead of being recomputed per
  query batch, so a query's result does not depend on which other queries
  share its batch.

Everything heavy runs in libckgpu.so: the index is built on the GPU and stays
resident with the sequences; a batch's queries are copied into a per-slot
arena behind the database sequences so that query/target pairs address one
sequence space.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass

import numpy as np

from . import _lib
from .blosum import BLOSUM62
from .pairwise import ENGINE_BATCHED, PASS_SCORE

LAMBDA = np.float32(0.267)
_SUB = np.ascontiguousarray(BLOSUM62, np.int8)
GRAPH_BUCKETS = (1, 2, 4, 8, 16, 32, 64, 128, 256)


def compute_freq_threshold(kmer_freqs, num_sequences: int, percentile: float = 99.5) -> int:
    """clustkit/kmer_index.py:451-463."""
    nonzero = kmer_freqs[kmer_freqs > 0]
    if len(nonzero) == 0:
        return int(num_sequences)
    pctl = int(np.percentile(nonzero, percentile))
    return int(max(pctl, max(100, num_sequences // 200)))


@dataclass(frozen=True)
class Scoring:
    """k-mer scoring and alignment settings of a search, with the meaning of
    clustkit's search_kmer_index keywords (clustkit/kmer_index.py:1475-1501)."""
    min_total_hits: int = 2
    kmer_score_thresh: int = 0
    min_diag_hits: int = 1
    diag_bin_width: int = 10
    phase_a_topk: int = 10000
    use_c_scoring: bool = False
    use_c_sw: bool = False
    c_sw_band_width: int = 50
    band_width: int | None = None  # SW band without use_c_sw; None: the database's

    @property
    def similar(self) -> bool:
        return self.kmer_score_thresh > 0

    @property
    def diagonal(self) -> bool:
        """Candidates from the C-scorer twin (Phase B when min_diag_hits >= 2)."""
        return not self.similar and (self.min_diag_hits >= 2 or self.use_c_scoring)

    @property
    def hints(self) -> bool:
        """Phase-B diagonal hints centre the alignment bands."""
        return self.use_c_sw and self.use_c_scoring and not self.similar

    @property
    def graphable(self) -> bool:
        """The pipeline can run without host synchronisation: every mode, under
        a caller bound where the library would otherwise read a device count
        (the Phase-B bins, _Slot.bins_bound; the similar-k-mer neighbour list,
        _Slot.list_bound)."""
        return True


# largest Phase-B bin buffer a slot keeps resident (int32 counters); beyond it
# the bins are sized per call from a device count (one host synchronisation)
BINS_CAP = 1 << 29
# Graph-replayed similar-k-mer batches list at most LIST_RATE neighbour triples
# per arena residue (~5,000 per residue is typical at threshold 13 on a 500k
# database, and arenas hold ~5x the residues of a typical batch); a batch that
# lists more is run again call by call.  LIST_CAP bounds the list (8 bytes a
# triple).
LIST_RATE = 2048
LIST_CAP = 1 << 28


def _torch():
    import torch
    return torch


@dataclass
class SearchHit:
    query: int
    target: int
    identity: float
    score: int
    rank: float


class DeviceDatabase:
    """Sequences, k-mer index and sketches resident on one GPU.

    ``arena_slots`` x ``arena_queries`` query entries and ``arena_slots`` x
    ``arena_residues`` residues are reserved behind the database sequences
    for query batches (one region per serving slot)."""

    def __init__(self, flat, offsets, lengths, k: int = 5, freq_percentile: float = 95.0,
                 band_width: int | None = None, arena_slots: int = 1, arena_queries: int = 64,
                 arena_residues: int = 64 * 2000, sketch_size: int = 128, sketch_k: int = 5,
                 device: str = "cuda:0", compact_index: bool = True):
        torch = _torch()
        self.lib = _lib.load()
        _lib.require_gpu()
        self.dev = torch.device(device)
        flat = np.ascontiguousarray(flat, np.uint8)
        offsets = np.ascontiguousarray(offsets, np.int64)
        lengths = np.ascontiguousarray(lengths, np.int32)
        if flat.size and flat.max() > 20:
            raise ValueError("database residue codes must be 0..20")
        self.n = int(lengths.shape[0])
        self.k = int(k)
        self.alpha = 20
        self.lengths_host = lengths
        self.max_len = int(self.lengths_host[: self.n].max()) if self.n else 0
        self.slots = int(arena_slots)
        self.arena_queries = int(arena_queries)
        self.arena_residues = int(arena_residues)
        # merged sequence space: database, one empty sequence, then the arenas
        self.empty_idx = self.n
        self.arena_seq0 = self.n + 1
        n_all = self.n + 1 + self.slots * self.arena_queries
        self.flat_len = int(flat.size) + self.slots * self.arena_residues
        self.arena_res0 = int(flat.size)
        self.d_flat = torch.zeros(max(self.flat_len, 1), dtype=torch.uint8, device=self.dev)
        self.d_flat[: flat.size].copy_(torch.from_numpy(flat))
        off_all = np.zeros(n_all, np.int64)
        len_all = np.zeros(n_all, np.int32)
        off_all[: self.n] = offsets
        len_all[: self.n] = lengths
        self.d_offsets = torch.from_numpy(off_all).to(self.dev)
        self.d_lengths = torch.from_numpy(len_all).to(self.dev)
        self.n_all = n_all
        # k-mer index
        nk = self.alpha ** self.k
        positions = int(np.maximum(lengths.astype(np.int64) - self.k + 1, 0).sum())
        self.d_kmer_offsets = torch.empty(nk + 1, dtype=torch.int64, device=self.dev)
        self.d_kmer_freqs = torch.empty(nk, dtype=torch.int32, device=self.dev)
        self.d_kmer_entries = torch.empty(max(positions, 1), dtype=torch.int64, device=self.dev)
        total = np.zeros(1, np.int64)
        stream = torch.cuda.current_stream(self.dev).cuda_stream
        _lib.check(self.lib.ck_kmer_index_build_device(
            0, self.d_flat.data_ptr(), self.flat_len, self.d_offsets.data_ptr(),
            self.d_lengths.data_ptr(), self.n, self.k, self.alpha, self.d_kmer_offsets.data_ptr(),
            self.d_kmer_entries.data_ptr(), positions, self.d_kmer_freqs.data_ptr(),
            total.ctypes.data, stream))
        self.n_entries = int(total[0])
        # the compact Phase-A index (target ids only), read by the Phase-A walks
        self.d_kmer_targets = None
        if compact_index:
            self.d_kmer_targets = torch.empty(max(self.n_entries, 1), dtype=torch.int32, device=self.dev)
            _lib.check(self.lib.ck_kmer_targets_device(0, self.d_kmer_entries.data_ptr(), self.n_entries,
                                                       self.d_kmer_targets.data_ptr(), stream))
        self.kmer_targets_ptr = self.d_kmer_targets.data_ptr() if self.d_kmer_targets is not None else None
        freqs = self.d_kmer_freqs.cpu().numpy()
        self.freq_thresh = compute_freq_threshold(freqs, self.n, freq_percentile)
        if band_width is None:
            band_width = max(20, int(int(np.percentile(lengths, 95)) * 0.3)) if self.n else 20
        self.band_width = int(band_width)
        # MinHash sketches of the database, resident beside the index
        self.d_sketches = torch.empty((self.n, sketch_size), dtype=torch.int64, device=self.dev)
        if self.n:
            _lib.check(self.lib.ck_sketch_device(
                self.d_flat.data_ptr(), self.flat_len, self.d_offsets.data_ptr(),
                self.d_lengths.data_ptr(), self.n, sketch_k, sketch_size, 20, 42,
                self.d_sketches.data_ptr(), stream))
        torch.cuda.synchronize(self.dev)

    def index_arrays(self):
        """(kmer_offsets, kmer_entries, kmer_freqs) as numpy, clustkit's layout."""
        return (self.d_kmer_offsets.cpu().numpy(),
                self.d_kmer_entries[: self.n_entries].cpu().numpy(),
                self.d_kmer_freqs.cpu().numpy())


class _Slot:
    """Buffers, stream and library context for one batch in flight."""

    def __init__(self, db: DeviceDatabase, index: int, max_cands: int):
        torch = _torch()
        self.db = db
        self.index = index
        self.max_cands = max_cands
        self.stream = torch.cuda.Stream(db.dev)
        h = np.zeros(1, np.int32)
        _lib.check(db.lib.ck_ctx_create(h.ctypes.data))
        self.ctx = int(h[0])
        self.ctx_spare = 0  # an unfrozen context for reruns of replayed batches, made on first use
        self._batch_info = None  # (scoring, max_qlen, residues, replayed) of the batch in flight
        Q, K = db.arena_queries, max_cands
        self.seq0 = db.arena_seq0 + index * Q
        self.res0 = db.arena_res0 + index * db.arena_residues
        dev = db.dev
        self.d_targets = torch.empty(Q * K, dtype=torch.int32, device=dev)
        self.d_counts = torch.empty(Q * K, dtype=torch.int32, device=dev)
        self.d_diags = torch.zeros(Q * K, dtype=torch.int32, device=dev)
        self.d_n = torch.empty(Q, dtype=torch.int32, device=dev)
        self.d_pairs = torch.empty((Q * K, 2), dtype=torch.int32, device=dev)
        self.d_sims = torch.empty(Q * K, dtype=torch.float32, device=dev)
        self.d_scores = torch.empty(Q * K, dtype=torch.int32, device=dev)
        self.d_mask = torch.empty(Q * K, dtype=torch.uint8, device=dev)
        pin = lambda n, dt: torch.zeros(n, dtype=dt).pin_memory()
        self.h_res = pin(db.arena_residues, torch.uint8)
        self.h_off = pin(Q, torch.int64)
        self.h_len = pin(Q, torch.int32)
        self.h_n = pin(Q, torch.int32)
        self.h_targets = pin(Q * K, torch.int32)
        self.h_sims = pin(Q * K, torch.float32)
        self.h_scores = pin(Q * K, torch.int32)
        self.h_mask = pin(Q * K, torch.uint8)
        self.event = torch.cuda.Event()
        self.batch = None
        # optional stage events: start, after the H2D copy, after Phase A, after SW, end
        self.stage_events = None
        self.graphs: dict = {}  # batch-size bucket -> captured pipeline
        self.graph_scoring = None
        self.last_band = db.band_width  # band of the last enqueued batch

    def close(self):
        self.graphs.clear()
        for name in ("ctx", "ctx_spare"):
            if getattr(self, name):
                self.db.lib.ck_ctx_destroy(getattr(self, name))
                setattr(self, name, 0)

    def enable_stage_timing(self):
        torch = _torch()
        self.stage_events = [torch.cuda.Event(enable_timing=True) for _ in range(5)]

    def last_cells(self) -> int:
        """Banded DP cells of the last batch's query/candidate pairs (after its event)."""
        from .cells import band_cells, effective_band
        nq, lens = self.batch if self.batch is not None else self._last_batch
        K = self.max_cands
        n = self.h_n.numpy()[:nq]
        tg = self.h_targets.numpy()[: nq * K].reshape(nq, K)
        keep = np.arange(K)[None, :] < n[:, None]
        qi, ci = np.nonzero(keep)
        ql = lens[qi].astype(np.int64)
        tl = self.db.lengths_host[tg[qi, ci]].astype(np.int64)
        la, lb = np.minimum(ql, tl), np.maximum(ql, tl)
        return int(band_cells(la, lb, effective_band(la, lb, self.last_band)).sum())

    def stage_ms(self):
        """(h2d, phase_a, sw, d2h) milliseconds of the last batch (after its event)."""
        ev = self.stage_events
        return tuple(ev[i].elapsed_time(ev[i + 1]) for i in range(4))

    def _mark(self, i):
        if self.stage_events is not None:
            self.stage_events[i].record(self.stream)

    def _fill_host(self, queries, pad_to=None):
        """Queries into the pinned staging buffers; (nq, lengths, residues)."""
        db = self.db
        nq = len(queries)
        lens = np.array([len(q) for q in queries], np.int32)
        offs = np.zeros(nq, np.int64)
        if nq > 1:
            offs[1:] = np.cumsum(lens[:-1])
        tot = int(lens.sum())
        if nq > db.arena_queries or tot > db.arena_residues:
            raise ValueError("batch exceeds the slot arena")
        hres = self.h_res.numpy()
        if tot:
            hres[:tot] = np.concatenate(queries)
        n_all = nq if pad_to is None else pad_to
        ho, hl = self.h_off.numpy(), self.h_len.numpy()
        ho[:nq] = offs + self.res0
        hl[:nq] = lens
        ho[nq:n_all] = self.res0  # padding queries: empty
        hl[nq:n_all] = 0
        return nq, lens, tot

    def bins_bound(self, nq: int, res_bytes: int, sc: Scoring) -> int:
        """Upper bound on the Phase-B bin counters of a batch of nq queries with
        res_bytes residues in all: each of at most phase_a_topk selected targets
        per query has (qlen + tlen) / width + 1 bins; -1 when above BINS_CAP."""
        db = self.db
        topk = min(int(sc.phase_a_topk), db.n)
        w = max(1, int(sc.diag_bin_width))
        bound = topk * ((int(res_bytes) + nq * db.max_len) // w + nq)
        return bound if bound <= BINS_CAP else -1

    def list_bound(self, res_bytes: int) -> int:
        """The caller bound on a similar-k-mer batch's neighbour triples
        (LIST_RATE per residue of the slot arena); -1 when above LIST_CAP."""
        bound = int(res_bytes) * LIST_RATE
        return bound if bound <= LIST_CAP else -1

    def can_capture(self, sc: Scoring) -> bool:
        """Whether the pipeline for ``sc`` can be captured in graphs on this slot."""
        if not sc.graphable:
            return False
        if sc.similar:
            return self.list_bound(self.db.arena_residues) >= 0
        return not sc.diagonal or self.bins_bound(self.db.arena_queries, self.db.arena_residues, sc) >= 0

    def _enqueue(self, nq: int, max_qlen: int, res_bytes: int, sc: Scoring, bounded: bool = False,
                 ctx: int | None = None):
        """The device pipeline of a batch of nq queries on this slot's stream:
        H2D, k-mer scoring, pair list, SW, D2H.  ``bounded``: the similar-k-mer
        neighbour list under the slot's list bound, so that no step reads a
        device count on the host and the pipeline can be captured in a CUDA
        graph.  ``ctx``: a library context other than the slot's."""
        torch = _torch()
        db = self.db
        K = self.max_cands
        M = nq * K
        lib = db.lib
        ctx = self.ctx if ctx is None else ctx
        st = self.stream.cuda_stream
        self._mark(0)
        db.d_flat[self.res0:self.res0 + res_bytes].copy_(self.h_res[:res_bytes], non_blocking=True)
        db.d_offsets[self.seq0:self.seq0 + nq].copy_(self.h_off[:nq], non_blocking=True)
        db.d_lengths[self.seq0:self.seq0 + nq].copy_(self.h_len[:nq], non_blocking=True)
        qoff_ptr = db.d_offsets.data_ptr() + self.seq0 * 8
        qlen_ptr = db.d_lengths.data_ptr() + self.seq0 * 4
        self._mark(1)
        min_total_hits = int(sc.min_total_hits)
        if sc.similar:  # BLOSUM62 similar k-mers (k = 5), clustkit's default scoring
            _lib.check(lib.ck_search_phase_a_similar_device(
                ctx, db.d_flat.data_ptr(), db.flat_len, qoff_ptr, qlen_ptr, nq, max_qlen, _SUB.ctypes.data,
                int(sc.kmer_score_thresh), db.d_kmer_offsets.data_ptr(), db.d_kmer_entries.data_ptr(),
                db.kmer_targets_ptr, db.d_kmer_freqs.data_ptr(), db.freq_thresh, db.n, min_total_hits, K,
                self.d_targets.data_ptr(), self.d_counts.data_ptr(), self.d_n.data_ptr(),
                self.list_bound(db.arena_residues) if bounded else -1, st))
        elif sc.diagonal:  # the C scorer's Phase A + Phase B, with diagonal hints
            _lib.check(lib.ck_search_kmer_candidates_device(
                ctx, db.d_flat.data_ptr(), db.flat_len, qoff_ptr, qlen_ptr, nq, max_qlen,
                db.k, db.alpha, db.d_kmer_offsets.data_ptr(), db.d_kmer_entries.data_ptr(), db.kmer_targets_ptr,
                db.d_kmer_freqs.data_ptr(), db.freq_thresh, db.n, db.d_lengths.data_ptr(), min_total_hits,
                int(sc.min_diag_hits), int(sc.diag_bin_width), K, int(sc.phase_a_topk),
                self.d_targets.data_ptr(), self.d_counts.data_ptr(), self.d_diags.data_ptr(),
                self.d_n.data_ptr(), self.bins_bound(nq, res_bytes, sc), st))
        else:
            _lib.check(lib.ck_search_phase_a_device(
                ctx, db.d_flat.data_ptr(), db.flat_len, qoff_ptr, qlen_ptr, nq, max_qlen,
                db.k, db.alpha, db.d_kmer_offsets.data_ptr(), db.d_kmer_entries.data_ptr(), db.kmer_targets_ptr,
                db.d_kmer_freqs.data_ptr(), db.freq_thresh, db.n, min_total_hits, K,
                self.d_targets.data_ptr(), self.d_counts.data_ptr(), self.d_n.data_ptr(), st))
        self._mark(2)
        self.last_band = (int(sc.c_sw_band_width) if sc.use_c_sw else
                          int(sc.band_width) if sc.band_width is not None else db.band_width)
        # dense pair list: (query, target) or (empty, empty) past a query's candidates
        _lib.check(lib.ck_search_pairs_device(nq, K, self.seq0, db.empty_idx, self.d_n.data_ptr(),
                                              self.d_targets.data_ptr(), self.d_pairs.data_ptr(), st))
        _lib.check(lib.ck_sw_batch_device_ctx(
            ctx, self.d_pairs.data_ptr(), M, db.d_flat.data_ptr(), db.flat_len,
            db.d_offsets.data_ptr(), db.d_lengths.data_ptr(), db.n_all, self.last_band,
            _SUB.ctypes.data, 0.0, self.d_diags.data_ptr() if sc.hints else None, PASS_SCORE, ENGINE_BATCHED,
            self.d_sims.data_ptr(), self.d_scores.data_ptr(), None, None, self.d_mask.data_ptr(), st))
        self._mark(3)
        self.h_n[:nq].copy_(self.d_n[:nq], non_blocking=True)
        self.h_targets[:M].copy_(self.d_targets[:M], non_blocking=True)
        self.h_sims[:M].copy_(self.d_sims[:M], non_blocking=True)
        self.h_scores[:M].copy_(self.d_scores[:M], non_blocking=True)
        self.h_mask[:M].copy_(self.d_mask[:M], non_blocking=True)
        self._mark(4)

    def capture_graphs(self, sc: Scoring | int, buckets=GRAPH_BUCKETS):
        """Capture the pipeline once per batch-size bucket in CUDA graphs.

        Every buffer is sized first by an uncaptured run of the largest
        bucket; the slot's library context is then frozen so no scratch buffer
        a graph points at is ever reallocated.  A batch then costs one graph
        replay (queries padded with empty ones up to the bucket)."""
        torch = _torch()
        db = self.db
        buckets = sorted({b for b in buckets if b <= db.arena_queries} | {db.arena_queries})
        self.stage_events = None
        self._fill_host([], pad_to=buckets[-1])  # every query slot an empty query
        if not isinstance(sc, Scoring):  # a minimum hit count: exact Phase A
            sc = Scoring(int(sc), 0)
        if not self.can_capture(sc):
            raise ValueError("this scoring cannot run without host synchronisation on this slot")
        with torch.cuda.stream(self.stream):
            self._enqueue(buckets[-1], db.arena_residues, db.arena_residues, sc, bounded=True)
        self.stream.synchronize()
        _lib.check(db.lib.ck_ctx_status(self.ctx, self.stream.cuda_stream))
        _lib.check(db.lib.ck_ctx_freeze(self.ctx, 1))
        for b in buckets:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=self.stream, capture_error_mode="thread_local"):
                self._enqueue(b, db.arena_residues, db.arena_residues, sc, bounded=True)
            self.graphs[b] = g
        # one replay of each (empty queries) so no graph's first upload falls
        # on a request
        with torch.cuda.stream(self.stream):
            for b in buckets:
                self.graphs[b].replay()
        self.graph_scoring = sc
        self.stream.synchronize()

    def launch(self, queries: list[np.ndarray], min_total_hits: int, kmer_score_thresh: int = 0, **scoring):
        """Enqueue the whole pipeline for a batch on this slot's stream
        (``scoring``: the other fields of Scoring).  Batches with the scoring the
        slot's graphs were captured for replay them; others run call by call."""
        torch = _torch()
        db = self.db
        sc = Scoring(int(min_total_hits), int(kmer_score_thresh), **scoring)
        bucket = None
        if self.graphs and sc == self.graph_scoring:
            bucket = next((b for b in sorted(self.graphs) if b >= len(queries)), None)
        if bucket is not None:
            nq, lens, tot = self._fill_host(queries, pad_to=bucket)
            with torch.cuda.stream(self.stream):
                self.graphs[bucket].replay()
                self.event.record(self.stream)
        else:
            nq, lens, tot = self._fill_host(queries)
            with torch.cuda.stream(self.stream):
                self._enqueue(nq, int(lens.max() if nq else 0), tot, sc)
                self.event.record(self.stream)
        self.batch = (nq, lens)
        self._batch_info = (sc, int(lens.max() if nq else 0), tot, bucket is not None)

    def _rerun_unbounded(self):
        """The batch in flight again, call by call in the slot's spare context
        (unfrozen, so its neighbour list can grow): a replayed batch whose
        listing passed the slot's list bound.  The pinned inputs still hold
        the batch; the outputs land in the same buffers."""
        torch = _torch()
        if not self.ctx_spare:
            h = np.zeros(1, np.int32)
            _lib.check(self.db.lib.ck_ctx_create(h.ctypes.data))
            self.ctx_spare = int(h[0])
        sc, max_qlen, tot, _ = self._batch_info
        nq = self.batch[0]
        with torch.cuda.stream(self.stream):
            self._enqueue(nq, max_qlen, tot, sc, ctx=self.ctx_spare)
            self.event.record(self.stream)
        self.event.synchronize()
        _lib.check(self.db.lib.ck_ctx_status(self.ctx_spare, self.stream.cuda_stream))

    def results(self, top_k: int, evalue_normalize: bool = True) -> list[list[SearchHit]]:
        """Hits of the batch (after the slot's event): top_k per query, ranked
        by 0.267 * score - ln(qlen * tlen), or by the raw score when
        evalue_normalize is off (clustkit/kmer_index.py:2315-2323)."""
        db = self.db
        status = db.lib.ck_ctx_status(self.ctx, self.stream.cuda_stream)
        if status == _lib.CK_ERR_CAPACITY and self._batch_info and self._batch_info[3] and self._batch_info[0].similar:
            self._rerun_unbounded()
        else:
            _lib.check(status)
        nq, lens = self.batch
        K = self.max_cands
        n = self.h_n.numpy()[:nq]
        tg = self.h_targets.numpy()[: nq * K].reshape(nq, K)
        sims = self.h_sims.numpy()[: nq * K].reshape(nq, K)
        scores = self.h_scores.numpy()[: nq * K].reshape(nq, K)
        mask = self.h_mask.numpy()[: nq * K].reshape(nq, K)
        # one vectorised pass over the batch: candidates that passed and their
        # rank; per query only those ranked at least its top_k-th best can be
        # hits (ties included); then a stable sort by (query, -rank) -- per
        # query the stable descending-rank order.  The sort key packs the query
        # above the order-preserving integer image of -rank (one int64 argsort
        # instead of a two-key lexsort; the same order, ties to the earlier
        # candidate).
        col = np.arange(K)[None, :]
        keep = (col < n[:, None]) & mask.astype(bool)
        qi, ci = np.nonzero(keep)
        t = tg[qi, ci]
        if evalue_normalize:
            rank = LAMBDA * scores[qi, ci].astype(np.float32) - np.log(
                lens[qi].astype(np.float32) * db.lengths_host[t].astype(np.float32))
        else:
            rank = scores[qi, ci].astype(np.float32)
        if top_k < K and len(qi):
            r2 = np.full((nq, K), -np.inf, np.float32)
            r2[qi, ci] = rank
            kth = np.partition(r2, K - top_k, axis=1)[:, K - top_k]  # each query's top_k-th largest
            near = rank >= kth[qi]
            qi, ci, t, rank = qi[near], ci[near], t[near], rank[near]
        sc = scores[qi, ci]
        si = sims[qi, ci]
        neg = (-rank + np.float32(0)).view(np.int32)  # + 0 folds -0.0 into +0.0
        ordered = np.where(neg < 0, neg ^ np.int32(0x7FFFFFFF), neg).astype(np.int64) + (1 << 31)
        order = np.argsort((qi.astype(np.int64) << 32) | ordered, kind="stable")
        qs = qi[order]
        first = np.searchsorted(qs, np.arange(nq + 1))
        out = []
        for q in range(nq):
            sel = order[first[q]:min(first[q + 1], first[q] + top_k)]
            out.append([SearchHit(q, int(t[o]), float(si[o]), int(sc[o]), float(rank[o])) for o in sel])
        self._last_batch = self.batch
        self.batch = None
        return out


def search_batch(db: DeviceDatabase, queries: list[np.ndarray], top_k: int = 10,
                 max_cands: int = 500, min_total_hits: int = 2, slot: _Slot | None = None,
                 kmer_score_thresh: int = 13, **scoring):
    """Synchronous search of a list of encoded queries; list of hit lists.
    ``scoring``: min_diag_hits, diag_bin_width, phase_a_topk, use_c_scoring,
    use_c_sw, c_sw_band_width (Scoring)."""
    own = slot is None
    if own:
        slot = _Slot(db, 0, max_cands)
    try:
        res = []
        for s in range(0, len(queries), db.arena_queries):
            chunk = queries[s:s + db.arena_queries]
            slot.launch(chunk, min_total_hits, kmer_score_thresh, **scoring)
            slot.event.synchronize()
            for qi, hits in enumerate(slot.results(top_k)):
                for h in hits:
                    h.query = s + qi
                res.append(hits)
        return res
    finally:
        if own:
            slot.close()


@dataclass
class KmerSearchHit:
    """One hit, with the fields of clustkit's SearchHit (clustkit/search.py:40-48)."""
    query_id: str
    target_id: str
    identity: float
    query_length: int
    target_length: int
    score: float = 0.0  # the rank value: E-value-normalised score, or the raw score


@dataclass
class SearchResults:
    """Results for all queries, with the fields of clustkit's SearchResults
    (clustkit/search.py:51-60)."""
    hits: list[list[KmerSearchHit]]
    num_queries: int
    num_targets: int
    num_candidates: int
    num_aligned: int
    runtime_seconds: float


_DB_CACHE: dict = {}  # id(db_index) -> (db_index, k, freq_percentile, arena_residues, DeviceDatabase)

_UNSUPPORTED = ("reduced_alphabet", "use_idf", "spaced_seeds", "extra_alphabets", "ml_prefilter_model")


def _device_db(db_index, k: int, freq_percentile: float, residues: int, device) -> DeviceDatabase:
    """The database resident on the GPU, built once per index object (and again
    only when a call's queries need a larger staging arena)."""
    hit = _DB_CACHE.get(id(db_index))
    same = hit is not None and hit[0] is db_index and hit[1] == k and hit[2] == freq_percentile
    if same and hit[3] >= residues:
        return hit[4]
    ds = db_index.dataset
    arena = max(residues, hit[3] if same else 0, 64 * 400)
    db = DeviceDatabase(ds.flat_sequences, ds.offsets, ds.lengths, k=k, freq_percentile=freq_percentile,
                        arena_slots=1, arena_queries=64, arena_residues=arena, device=device)
    _DB_CACHE.clear()  # one resident database at a time
    _DB_CACHE[id(db_index)] = (db_index, k, freq_percentile, arena, db)
    return db


def search_kmer_index(db_index, query_dataset, threshold: float = 0.5, top_k: int = 10,
                      band_width: int | None = None, device="cpu", min_total_hits: int = 2,
                      min_diag_hits: int = 2, diag_bin_width: int = 10, max_cands_per_query: int = 2000,
                      phase_a_topk: int = 10000, freq_percentile: float = 95.0, min_ungapped_score: int = 0,
                      kmer_score_thresh: int = 13, local_alignment: bool = True, evalue_normalize: bool = True,
                      reduced_alphabet: bool = False, reduced_k=5, use_idf: bool = False, spaced_seeds=None,
                      extra_alphabets=None, ml_prefilter_model=None, use_c_sw: bool = False,
                      c_sw_band_width: int = 50, use_c_scoring: bool = False) -> SearchResults:
    """Drop-in for clustkit's search_kmer_index (clustkit/kmer_index.py:1475-2349)
    on the GPU: the same arguments, defaults and results for its protein k-mer
    paths -- exact Phase A, Phase B (min_diag_hits >= 2), BLOSUM62 similar
    5-mers (kmer_score_thresh > 0, the default), the C scorer and C SW
    settings -- with banded SW (score > 0 passes; ``threshold`` plays no part
    there, as in clustkit), the E-value-style rank and the top_k hits per query.
    ``db_index`` needs ``dataset`` (flat_sequences, offsets, lengths, ids) and
    ``params`` (mode, kmer_size or kmer_index_k); ``query_dataset`` the same
    compact fields.  The index is rebuilt on the device from the database
    sequences (clustkit's layout) and kept resident between calls on the same
    index object.  The band width, when not given, is clustkit's per-call
    ``max(20, 0.3 * p95(query and database lengths))``.  ``device`` is the
    GPU ("cpu" means the default GPU: there is no CPU path).  Options for the
    search variants not built here raise NotImplementedError."""
    start = time.perf_counter()
    opts = {"reduced_alphabet": reduced_alphabet, "use_idf": use_idf, "spaced_seeds": spaced_seeds,
            "extra_alphabets": extra_alphabets, "ml_prefilter_model": ml_prefilter_model}
    for name in _UNSUPPORTED:
        if opts[name]:
            raise NotImplementedError(f"search_kmer_index: {name} is not built on the GPU")
    if min_ungapped_score > 0:
        raise NotImplementedError("search_kmer_index: the ungapped pre-filter is not built on the GPU")
    if not local_alignment:
        raise NotImplementedError("search_kmer_index: global (NW) alignment is not built on the GPU")
    params = db_index.params
    if params.get("mode", "protein") != "protein":
        raise NotImplementedError("search_kmer_index: only the protein path is built on the GPU")
    k = int(params.get("kmer_index_k", params.get("kmer_size", 5)))
    if kmer_score_thresh > 0 and k != 5:
        raise NotImplementedError("search_kmer_index: similar k-mer scoring is built for k = 5")
    nq = len(query_dataset.lengths)
    nd = len(db_index.dataset.lengths)
    if nq == 0 or nd == 0:
        return SearchResults([[] for _ in range(nq)], nq, nd, 0, 0, time.perf_counter() - start)
    q_flat = np.asarray(query_dataset.flat_sequences, np.uint8)
    q_off = np.asarray(query_dataset.offsets, np.int64)
    q_len = np.asarray(query_dataset.lengths, np.int64)
    queries = [q_flat[o:o + L] for o, L in zip(q_off, q_len)]
    if band_width is None:
        p95 = int(np.percentile(np.concatenate([q_len, np.asarray(db_index.dataset.lengths, np.int64)]), 95))
        band_width = max(20, int(p95 * 0.3))
    dev = "cuda:0" if device in (None, "cpu", "gpu", "cuda") else (
        f"cuda:{device}" if isinstance(device, int) or str(device).isdigit() else str(device))
    db = _device_db(db_index, k, float(freq_percentile), int(q_len.max(initial=1)) * 64, dev)
    scoring = dict(min_diag_hits=int(min_diag_hits), diag_bin_width=int(diag_bin_width),
                   phase_a_topk=int(phase_a_topk), use_c_scoring=bool(use_c_scoring), use_c_sw=bool(use_c_sw),
                   c_sw_band_width=int(c_sw_band_width), band_width=int(band_width))
    slot = _Slot(db, 0, int(max_cands_per_query))
    hits: list[list[KmerSearchHit]] = []
    n_cands = 0
    q_ids, t_ids = query_dataset.ids, db_index.dataset.ids
    t_len = db.lengths_host
    try:
        i = 0
        while i < nq:  # chunks within the slot's query and residue capacity
            j, res = i, 0
            while j < nq and j - i < db.arena_queries and res + len(queries[j]) <= db.arena_residues:
                res += len(queries[j])
                j += 1
            slot.launch(queries[i:j], int(min_total_hits), int(kmer_score_thresh), **scoring)
            slot.event.synchronize()
            n_cands += int(slot.h_n.numpy()[: j - i].sum())
            for qi, hl in enumerate(slot.results(int(top_k), evalue_normalize=evalue_normalize)):
                q = i + qi
                hits.append([KmerSearchHit(q_ids[q], t_ids[h.target], h.identity, int(q_len[q]),
                                           int(t_len[h.target]), h.rank) for h in hl])
            i = j
    finally:
        slot.close()
    return SearchResults(hits, nq, nd, n_cands, n_cands, time.perf_counter() - start)


def batch_bytes(db, queries, max_cands: int) -> int:
    """Device bytes a search batch of these queries occupies while it runs:
    its residues and query table, the Phase-A hit counts (one int32 per
    database sequence per query), the candidate list with its scores and
    diagonals, the dense pair list and the SW outputs, and the batched SW
    engine's per-pair sort and fallback scratch."""
    nq = len(queries)
    res = int(sum(int(np.asarray(q).size) for q in queries))
    M = nq * int(max_cands)
    return (res + nq * 12 + nq * db.n * 4 + M * (4 + 4 + 4) + M * 8 + M * (4 + 4 + 1)
            + M * (4 * 4 + 4))


@dataclass
class _Request:
    query: np.ndarray
    future: Future
    t_arrival: float


class SearchServer:
    """Continuous-batching search server on one GPU.

    Requests (encoded protein queries) are queued on arrival.  A scheduler
    thread admits queued requests into a batch whenever a slot -- a stream, a
    library context and a pre-sized region of device memory -- is free, up to
    the slot's query and residue capacity; batches in different slots overlap
    on the device.  The number of slots is bounded by free device memory at
    start-up.

    Admission is also by device memory: a batch's footprint (``batch_bytes``:
    its residues, its per-query Phase-A counts over the database, its
    candidate and pair lists and the SW engine's per-pair scratch) is taken
    from a byte budget while it runs and returned when it completes.  A batch
    is formed only from queued requests that fit both the slot and what is
    left of the budget; a request that does not fit waits (a deferral) until
    running batches return their bytes, and one that cannot fit beside any
    other runs alone.  ``mem_budget`` defaults to the device memory that is
    free once the slots are allocated plus what the slots hold -- the slots
    are then the binding limit -- and a smaller budget caps the concurrent
    work by bytes.  Each request's future resolves to its list of SearchHit
    (query index 0) when its batch completes; latency is recorded per request.
    """

    def __init__(self, db: DeviceDatabase, top_k: int = 10, max_cands: int = 500,
                 min_total_hits: int = 2, max_batch: int | None = None, use_graphs: bool = True,
                 kmer_score_thresh: int = 13, mem_budget: int | None = None, **scoring):
        torch = _torch()
        self.db = db
        self.top_k = top_k
        self.max_cands = max_cands
        self.min_total_hits = min_total_hits
        self.kmer_score_thresh = int(kmer_score_thresh)
        self.scoring = dict(scoring)
        self.max_batch = min(max_batch or db.arena_queries, db.arena_queries)
        free, _ = torch.cuda.mem_get_info(db.dev)
        # per slot: counts scratch + pair/SW buffers + the SW kernel's window scratch
        per_slot = (db.arena_queries * db.n * 4 + db.arena_queries * max_cands * 64 + (256 << 20))
        sc = Scoring(int(min_total_hits), self.kmer_score_thresh, **scoring)
        if sc.diagonal:  # Phase B: target -> selection row, selection and bin offsets
            per_slot += db.arena_queries * (db.n * 4 + min(sc.phase_a_topk, db.n) * 16)
        if sc.similar and use_graphs:  # the bounded neighbour list (8 bytes a triple)
            per_slot += max(0, db.arena_residues * LIST_RATE) * 8
        n_slots = int(max(1, min(db.slots, (free // 2) // max(per_slot, 1))))
        self.slots = [_Slot(db, i, max_cands) for i in range(n_slots)]
        self.free = list(self.slots)
        self.busy: list[tuple[_Slot, list[_Request], int]] = []  # slot, requests, bytes held
        self.queue: collections.deque[_Request] = collections.deque()
        self.cv = threading.Condition()
        self.running = False
        self.latencies: list[float] = []
        self.thread = None
        # allocate every slot's scratch before serving: capture its pipeline in
        # CUDA graphs (one replay per batch), or warm it with a full batch of
        # typical queries (random residues, 400 long) so that serving rarely
        # grows a buffer (a growth synchronises the device)
        rng = np.random.default_rng(0)
        wl = max(1, min(400, db.arena_residues // self.max_batch))
        warm = [rng.integers(0, 20, wl).astype(np.uint8) for _ in range(self.max_batch)]
        for s in self.slots:
            if use_graphs and s.can_capture(sc):
                s.capture_graphs(sc)
            s.launch(warm, min_total_hits, self.kmer_score_thresh, **self.scoring)
            s.event.synchronize()
            s.results(1)
        self.per_slot_bytes = per_slot
        if mem_budget is None:
            mem_budget = int(torch.cuda.mem_get_info(db.dev)[0]) + n_slots * per_slot
        self.mem_budget = int(mem_budget)
        self.in_flight_bytes = 0
        self.peak_in_flight_bytes = 0
        self.deferrals = 0

    def batch_bytes(self, queries) -> int:
        return batch_bytes(self.db, queries, self.max_cands)

    def start(self):
        self.running = True
        self.thread = threading.Thread(target=self._loop, name="ck-search-scheduler", daemon=True)
        self.thread.start()
        return self

    def stop(self):
        with self.cv:
            self.running = False
            self.cv.notify_all()
        if self.thread:
            self.thread.join()
        for s in self.slots:
            s.close()

    def submit(self, query, t_arrival: float | None = None) -> Future:
        """Queue a query; ``t_arrival`` (perf_counter time) defaults to now and
        is where its latency is measured from."""
        q = np.ascontiguousarray(query, np.uint8)
        if q.size and q.max() > 20:
            raise ValueError("query residue codes must be 0..20")
        if q.size > self.db.arena_residues:
            raise ValueError("query longer than a slot arena")
        fut: Future = Future()
        with self.cv:
            self.queue.append(_Request(q, fut, time.perf_counter() if t_arrival is None else t_arrival))
            self.cv.notify()
        return fut

    def _finish(self, slot: _Slot, reqs: list[_Request]):
        try:
            res = slot.results(self.top_k)
            now = time.perf_counter()
            for r, hits in zip(reqs, res):
                for h in hits:
                    h.query = 0
                self.latencies.append(now - r.t_arrival)
                r.future.set_result(hits)
        except Exception as e:  # surface device errors to every waiting request
            for r in reqs:
                r.future.set_exception(e)

    def _loop(self):
        while True:
            with self.cv:
                if not self.running and not self.queue and not self.busy:
                    return
            progressed = False
            still = []
            for slot, reqs, nbytes in self.busy:
                if slot.event.query():
                    self._finish(slot, reqs)
                    self.free.append(slot)
                    self.in_flight_bytes -= nbytes
                    progressed = True
                else:
                    still.append((slot, reqs, nbytes))
            self.busy = still
            batch: list[_Request] = []
            need = 0
            with self.cv:
                if self.free and self.queue:
                    res = 0
                    left = self.mem_budget - self.in_flight_bytes
                    while self.queue and len(batch) < self.max_batch:
                        q = self.queue[0].query
                        if res + q.size > self.db.arena_residues:
                            break
                        grown = self.batch_bytes([r.query for r in batch] + [q])
                        if grown > left and (batch or self.busy):
                            self.deferrals += 1  # waits for running batches to return their bytes
                            break
                        r = self.queue.popleft()
                        res += q.size
                        need = grown
                        batch.append(r)
            if batch:
                slot = self.free.pop()
                try:
                    slot.launch([r.query for r in batch], self.min_total_hits, self.kmer_score_thresh,
                                **self.scoring)
                    self.busy.append((slot, batch, need))
                    self.in_flight_bytes += need
                    self.peak_in_flight_bytes = max(self.peak_in_flight_bytes, self.in_flight_bytes)
                except Exception as e:
                    for r in batch:
                        r.future.set_exception(e)
                    self.free.append(slot)
                progressed = True
            if not progressed:
                with self.cv:
                    self.cv.wait(timeout=0.0002)

    def latency_percentiles(self):
        a = np.array(self.latencies)
        if not a.size:
            return {}
        return {"p50_ms": float(np.percentile(a, 50) * 1e3), "p99_ms": float(np.percentile(a, 99) * 1e3),
                "mean_ms": float(a.mean() * 1e3), "n": int(a.size)}
