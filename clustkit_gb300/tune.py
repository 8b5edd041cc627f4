"""Autotuner for the batched Smith-Waterman engine.

The batched engine (csrc/sw_batched.cu) has three kinds of tunables, the
GB300 counterparts of "bin edges, band tiling and CTA shape":

* bin edge -- which pairs run one warp per pair instead of one lane per pair:
  every pair of a call with at most ``wave_all_below`` pairs, and in larger
  calls the pairs with at least ``wave_min_rows`` rows, raised (when
  ``wave_adaptive``) to where a pair's one-lane time would pass the call's
  expected time;
* band tiling -- rows a lane keeps in registers per strip (8, 16, 24, 32;
  the library's default 0 picks 8 for half-widths up to 64, else 16);
* strip variant -- interior columns in groups of 2 or 4 (one first-maximum
  vote per group), aligned with base-pointer addressing and a 4-column
  prefetch or not, i.e. the shape of a lane's inner loop (the library's
  default -1 takes groups of 4 at 8 rows per strip, else 2);
* CTA shape -- resident 256-thread CTAs per SM for strips of up to 16 rows
  (2 at <= 128 registers a thread, or 1 with up to 255; taller strips run 1),
  which sets the warps per SM and the lanes' scratch windows in flight.

``autotune`` times candidates on the caller's own pairs (device-resident,
CUDA events around the whole call, L2 flushed between runs, the median of
``repeats`` runs) by coordinate descent -- bin edge, then tiling x variant x
CTA shape, then the bin edge again.  The fastest candidate is then timed
again against the default, alternating the two, and replaces the default only
when it is at least ``min_gain`` (2 %) faster there, so a noisy trial never
leaves a slower setting in place.  Settings are process-wide (``apply``);
every setting gives identical results, only the time changes.  Results are
cached per (band width, length profile).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .blosum import BLOSUM62
from .cells import band_cells, effective_band

KEYS = {
    "rows_per_strip": _lib.CFG_ROWS_PER_STRIP,
    "strip_variant": _lib.CFG_STRIP_VARIANT,
    "strip_threads": _lib.CFG_STRIP_THREADS,
    "wave_min_rows": _lib.CFG_WAVE_MIN_ROWS,
    "wave_all_below": _lib.CFG_WAVE_ALL_BELOW,
    "wave_adaptive": _lib.CFG_WAVE_ADAPTIVE,
}

DEFAULT = {"rows_per_strip": 0, "strip_variant": -1, "strip_threads": 0, "wave_min_rows": 512,
           "wave_all_below": 40960, "wave_adaptive": 1}

# bin-edge candidates: (wave_min_rows, wave_adaptive); 1 << 30 = never by length
BIN_EDGES = [(512, 1), (256, 1), (512, 0), (1024, 0), (2048, 0), (4096, 0), (1 << 30, 0)]
# (rows per strip, strip variant, threads of the strip kernel's CTA); 0 = the
# library's choice (the only one for 16, 24 and 32 rows)
TILINGS = ([(8, v, t) for v in (0, 1, 2, 3) for t in (512, 640, 768)] +
           [(16, v, 0) for v in (0, 1, 2, 3)] +
           [(r, v, 0) for r in (24, 32) for v in (0, 1)])

_cache: dict = {}


def current() -> dict:
    return {k: _lib.get_config(v) for k, v in KEYS.items()}


def apply(config: dict) -> None:
    for k, v in config.items():
        _lib.set_config(KEYS[k], int(v))


@dataclass
class TuneResult:
    config: dict
    ms: float
    gcups: float
    cells: int
    trials: list = field(default_factory=list)  # (config, ms)
    confirm: dict = field(default_factory=dict)  # the winner re-timed against the default


class _DeviceCall:
    """One pair set resident on the device, timed through ck_sw_batch_device."""

    def __init__(self, pairs, flat, offsets, lengths, band_width):
        import torch
        self.torch = torch
        self.lib = _lib.load()
        _lib.require_gpu()
        dev = torch.device("cuda", torch.cuda.current_device())
        T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        self.pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        self.M = int(self.pairs.shape[0])
        self.d_pairs, self.d_flat = T(self.pairs), T(np.asarray(flat, np.uint8))
        self.d_off, self.d_len = T(np.asarray(offsets, np.int64)), T(np.asarray(lengths, np.int32))
        self.n = int(len(lengths))
        self.flat_len = int(len(flat))
        self.bw = int(band_width)
        self.sub = np.ascontiguousarray(BLOSUM62)
        self.out = [torch.empty(self.M, dtype=dt, device=dev) for dt in
                    (torch.float32, torch.int32, torch.int32, torch.int32, torch.uint8)]
        self.stream = torch.cuda.current_stream(dev)
        self.flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def run(self, engine=0):
        o = self.out
        _lib.check(self.lib.ck_sw_batch_device(
            self.d_pairs.data_ptr(), self.M, self.d_flat.data_ptr(), self.flat_len, self.d_off.data_ptr(),
            self.d_len.data_ptr(), self.n, self.bw, self.sub.ctypes.data, 0.0, None, _lib.PASS_SCORE, engine,
            o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(), o[3].data_ptr(), o[4].data_ptr(),
            self.stream.cuda_stream))

    def time_ms(self, repeats=5, warmup=1, engine=0) -> float:
        """Median of `repeats` timed calls after `warmup` untimed ones."""
        torch = self.torch
        for _ in range(warmup):
            self.run(engine)
        times = []
        for k in range(repeats):
            self.flush.fill_(k & 0xFF)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(self.stream)
            self.run(engine)
            b.record(self.stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        _lib.check(self.lib.ck_sw_status_device(self.stream.cuda_stream))
        return float(np.median(times))

    def results(self):
        return {k: t.cpu().numpy() for k, t in zip(("sims", "scores", "matches", "shorter", "mask"), self.out)}


def profile_key(lengths, pairs, band_width):
    """Cache key: band width and the log2 buckets of the rows' 50/90/99/99.9 percentiles."""
    L = np.asarray(lengths)
    p = np.asarray(pairs).reshape(-1, 2)
    rows = np.minimum(L[p[:, 0]], L[p[:, 1]]) if len(p) else np.zeros(1)
    q = np.percentile(rows, [50, 90, 99, 99.9]) if len(p) else np.zeros(4)
    return (int(band_width), tuple(int(np.log2(max(x, 1))) for x in q), int(np.log2(max(len(p), 1))))


def confirm(call, candidate: dict, base: dict, rounds: int = 3, repeats: int = 5) -> dict:
    """Time the candidate and the base setting alternately (rounds x repeats
    runs each, medians of the per-round medians) on the same call."""
    t_c, t_b = [], []
    for _ in range(rounds):
        apply(base)
        t_b.append(call.time_ms(repeats))
        apply(candidate)
        t_c.append(call.time_ms(repeats))
    return {"candidate_ms": float(np.median(t_c)), "default_ms": float(np.median(t_b))}


def autotune(pairs, flat, offsets, lengths, band_width: int, repeats: int = 5,
             use_cache: bool = True, apply_best: bool = True, min_gain: float = 0.02) -> TuneResult:
    """Time the engine's settings on these pairs and return (and apply) the
    fastest, which must beat the default by ``min_gain`` on a re-time."""
    key = profile_key(lengths, pairs, band_width)
    if use_cache and key in _cache:
        res = _cache[key]
        if apply_best:
            apply(res.config)
        return res
    call = _DeviceCall(pairs, flat, offsets, lengths, band_width)
    L = np.asarray(lengths, np.int64)
    p = call.pairs
    la = np.minimum(L[p[:, 0]], L[p[:, 1]])
    lb = np.maximum(L[p[:, 0]], L[p[:, 1]])
    cells = int(band_cells(la, lb, effective_band(la, lb, band_width)).sum())
    keep = current()
    trials = []
    best = dict(DEFAULT)
    best_ms = None
    chk = {}

    def trial(cfg):
        nonlocal best, best_ms
        apply(cfg)
        ms = call.time_ms(repeats)
        trials.append((dict(cfg), ms))
        if best_ms is None or ms < best_ms:
            best, best_ms = dict(cfg), ms

    try:
        base = dict(DEFAULT)
        for mr, ad in BIN_EDGES:
            trial({**base, "wave_min_rows": mr, "wave_adaptive": ad})
        edge = {k: best[k] for k in ("wave_min_rows", "wave_adaptive")}
        for r, v, c in TILINGS:
            trial({**base, **edge, "rows_per_strip": r, "strip_variant": v, "strip_threads": c})
        tiling = {k: best[k] for k in ("rows_per_strip", "strip_variant", "strip_threads")}
        for mr, ad in BIN_EDGES:
            cfg = {**base, **tiling, "wave_min_rows": mr, "wave_adaptive": ad}
            if not any(c == cfg for c, _ in trials):
                trial(cfg)
        if best != DEFAULT:
            chk = confirm(call, best, DEFAULT)
            if chk["candidate_ms"] > (1.0 - min_gain) * chk["default_ms"]:
                best, best_ms = dict(DEFAULT), chk["default_ms"]
                chk["kept"] = "default"
            else:
                best_ms = chk["candidate_ms"]
                chk["kept"] = "candidate"
    finally:
        apply(keep)
    res = TuneResult(best, best_ms, cells / (best_ms * 1e-3) / 1e9 if best_ms else 0.0, cells, trials, chk)
    _cache[key] = res
    if apply_best:
        apply(best)
    return res
