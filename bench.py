"""Benchmark: banded Smith-Waterman over clustkit's Align-phase candidate pairs.

Workload (one "step"): the Align phase of the 50,000-sequence clustering set --
5,000 synthetic families x 10 (median length 350, clipped 30..2000), k=5 /
s=128 MinHash sketches, LSH with clustkit's high-sensitivity parameters at
t=0.3 (b=1, L=512), clustkit's Jaccard pre-filter, pairs ordered by min(i,j)
as compute_pairwise_alignment orders them, then banded SW (band width 100,
BLOSUM62, gaps -11/-1) over every remaining pair with per-pair score, identity
numerator/denominator and pass/fail.  Data are seeded synthetic (no public
dataset); the sequences and pair list are built once, before timing.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm prints one JSON line: value = GCUPS of the batched engine with inputs
resident in HBM (device pointers, CUDA events per step on the launching
stream, L2 flushed between steps outside the timed events); e2e = the same
through the host-buffer C entry point ck_sw_batch (H2D of the step's inputs
from pinned memory and D2H of its outputs inside the timed region).  The
plain engine (one unbinned launch) is timed beside it.  The reference arm
times clustkit's CPU implementation (its own C compiled from source when that
library was built in this checkout, else this repo's C restatement) on the
host cores, on a bounded sample of the same pairs.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

BAND_WIDTH = 100
THRESHOLD = 0.3
THRESHOLD_MILLION = 0.4
WORKLOAD = {"workload": "align-50k: 5000 families x 10, median 350 [30,2000], k=5 s=128, "
                        "LSH b=1 L=512 (t=0.3 high), Jaccard pre-filter, SW bw=100 BLOSUM62 -11/-1",
            "n_sequences": 50000, "threshold": THRESHOLD, "band_width": BAND_WIDTH,
            "l2": "flushed between timed steps (256 MiB write, outside the step events)"}
OPS_PER_CELL = 6  # max-plus lane ops of the score recurrence: E, F: viaddmax+add; H: vimax3+add
# DRAM traffic of the strip kernel: dram__bytes_read.sum + dram__bytes_write.sum of
# one launch on this workload from an ncu capture (the profile named here), per DP
# cell of that launch; a run reports it scaled to its own cells and says so
STRIP_PROFILE = "profiles/sw_strip_kernel_align50k.md"
STRIP_PROFILE_CELLS = 46_229_358_568
STRIP_DRAM_BYTES_PER_CELL = (25.128211e9 + 27.463094e9) / STRIP_PROFILE_CELLS


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------- workload
def build_workload(use_gpu: bool, quick: bool = False):
    from clustkit_gb300 import synth
    from clustkit_gb300.lsh import auto_lsh_params, lsh_candidates
    n_fam = 500 if quick else 5000
    t0 = time.time()
    s = synth.generate_families(n_fam, 10, median=350, lo=30, hi=2000, seed=2)
    t1 = time.time()
    if use_gpu:
        from clustkit_gb300.sketch import sketch_flat
        sk = sketch_flat(s.flat, s.offsets, s.lengths, 5, 128)
    else:
        import oracle
        sk = oracle.sketches(s.flat, s.offsets, s.lengths, 5, 128)
    lp = auto_lsh_params(THRESHOLD, "high", 5)
    # the host restatement, not the device LSH: with b = 1 this set has buckets
    # of more than 1,000 members, where clustkit keeps the first 1,000 of numpy's
    # unstable argsort (reproduced on the host) and the device the 1,000 lowest
    # ids -- the workload must be clustkit's own
    cand = lsh_candidates(sk, lp["num_tables"], lp["num_bands"], 42)
    t2 = time.time()
    floor = max(0.001, 0.3 * THRESHOLD ** 5)
    if use_gpu:
        from clustkit_gb300.pairwise import _jaccard_prefilter
        keep = _jaccard_prefilter(cand, sk, THRESHOLD)
    else:
        import oracle
        m = len(cand)
        keep = None
        rng = np.random.RandomState(0)
        idx = rng.choice(m, size=min(2000, m), replace=False)
        if float(np.mean(oracle.jaccard(cand[idx], sk) < floor)) >= 0.05:
            keep = oracle.jaccard(cand, sk) >= floor
    pairs = cand if keep is None else cand[keep]
    pairs = pairs[np.argsort(np.minimum(pairs[:, 0], pairs[:, 1]), kind="mergesort")]
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    log(f"workload: {s.n} seqs ({t1 - t0:.1f}s), {len(cand)} LSH candidates ({t2 - t1:.1f}s), "
        f"{len(pairs)} after Jaccard pre-filter")
    return s, pairs, len(cand)


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
            os.unlink(self.path)
        except OSError:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        busy = [v for v in sm if mx and v > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------------------- dist
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def shard(pairs: np.ndarray, world: int, rank: int) -> np.ndarray:
    """Weak scaling: every rank aligns its own full-size replica of the pair
    list (the path has no exchange step, so ranks never communicate data)."""
    return pairs


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ----------------------------------------------------------------------------- CPU baselines
def reference_gpu_baseline(s, pairs, d_flat, d_off, d_len, stream, n_sample: int = 150_000):
    """The reference's CuPy GPU path (its own kernel source, compiled from the
    reference checkout into oracle/_ref/, with its host batching restated in
    oracle/cupy_ref.py) on a random sample of the workload's pairs, device-resident
    inputs, CUDA events around its launches; plus whether its identities and
    pass/fail equal this engine's under the same (CuPy) pass rule."""
    import torch
    from oracle import cupy_ref
    from clustkit_gb300.blosum import BLOSUM62
    from clustkit_gb300.cells import pair_cells
    from clustkit_gb300.pairwise import PASS_CUPY, batch_sw
    if not cupy_ref.available():
        return {"unavailable": "oracle/_ref/sw_cupy_ref.cubin is built from the reference checkout, absent here"}
    rng = np.random.default_rng(0)
    idx = np.sort(rng.choice(len(pairs), size=min(n_sample, len(pairs)), replace=False))
    sp = pairs[idx]
    k = cupy_ref.CupyPathKernel()
    plan = k.prepare(sp, s.lengths, BAND_WIDTH, BLOSUM62)
    k.launch(plan, d_flat, d_off, d_len, THRESHOLD, stream.cuda_stream)  # warm-up
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    k.launch(plan, d_flat, d_off, d_len, THRESHOLD, stream.cuda_stream)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b)
    sims, mask = k.results(plan)
    ours = batch_sw(sp, s.flat, s.offsets, s.lengths, BAND_WIDTH, BLOSUM62, THRESHOLD, pass_rule=PASS_CUPY)
    cells = int(pair_cells(sp, s.lengths, BAND_WIDTH).sum())
    return {"value": cells / (ms * 1e-3) / 1e9, "unit": "GCUPS", "pairs_per_s": len(sp) / (ms * 1e-3),
            "kernel_ms": ms, "sample": f"{len(sp)} random pairs of the workload ({cells} cells)",
            "threads_per_block": [t for (_, _, _, t) in plan["batches"]], "launches": len(plan["batches"]),
            "agrees_with_this_engine_pass_cupy": bool(np.array_equal(sims, ours["sims"]) and
                                                      np.array_equal(mask, ours["mask"])),
            "source": "clustkit/pairwise.py:1215-1402 kernel + :1480-1547 batching (CuPy not installed)"}


def hbm_check(s, pairs, kernel_s, cells):
    """Why the bound is integer issue and not HBM: the strip kernel's
    algorithmic bytes (both sequences, the pair, two offsets, two lengths and
    the 17 output bytes per pair) and its measured DRAM traffic (ncu, the
    window spilling from L2) against the measured copy bandwidth."""
    L = s.lengths.astype(np.int64)
    alg = int((L[pairs[:, 0]] + L[pairs[:, 1]]).sum()) + len(pairs) * (8 + 16 + 8 + 17)
    peak = None
    try:
        peak = float(json.loads((Path(__file__).resolve().parent / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
        basis = "of measured"
    except (OSError, ValueError, KeyError):
        peak, basis = 6800.0, "of fallback"
    alg_gbs = alg / kernel_s / 1e9
    dram_gbs = STRIP_DRAM_BYTES_PER_CELL * cells / kernel_s / 1e9
    return {"algorithmic_bytes": alg, "algorithmic_gbs": alg_gbs, "dram_gbs_from_profile": dram_gbs,
            "peak_gbs": peak, "frac_algorithmic": alg_gbs / peak, "frac_dram": dram_gbs / peak, "peak_basis": basis,
            "dram_source": f"ncu DRAM bytes per cell from {STRIP_PROFILE} x this run's cells / this run's "
                           f"kernel time"}


def same_as_oracle(res, ref, threshold=None) -> bool:
    """Every pair's score, identity numerator and denominator and float32
    identity (bit pattern) equal the oracle's; with a threshold, also the
    pass/fail mask under the C path's rule (sims >= t, clustkit/pairwise.py:107)."""
    ok = all(np.array_equal(np.asarray(res[k]), ref[k]) for k in ("scores", "matches", "shorter"))
    ok = ok and np.array_equal(np.asarray(res["sims"]).view(np.uint32), ref["sims"].view(np.uint32))
    if threshold is not None:
        ok = ok and np.array_equal(np.asarray(res["mask"]).astype(bool), ref["sims"] >= np.float32(threshold))
    return bool(ok)


def cpu_baseline(s, pairs, use_ref: bool = True):
    """clustkit's CPU algorithm on every pair of the workload, on all host
    cores: the host-core baseline (GCUPS over the whole pair list, ~15 s on
    16 cores) and, from the same run, the oracle outputs that every GPU result
    of the step is checked against.  Plus one thread on a ~3 s slice."""
    import oracle
    from clustkit_gb300.blosum import BLOSUM62
    from clustkit_gb300.cells import pair_cells
    threads = os.cpu_count() or 1
    kind = "reference" if (use_ref and oracle.ref_available()) else "port"
    oracle.set_num_threads(threads)
    t = time.perf_counter()
    ref = oracle.sw_batch(pairs, s.flat, s.offsets, s.lengths, BAND_WIDTH, BLOSUM62)
    dt_port = time.perf_counter() - t
    cells = int(pair_cells(pairs, s.lengths, BAND_WIDTH).sum())
    dt = dt_port
    if kind == "reference":
        t = time.perf_counter()
        oracle.ref_sw_batch(pairs, s.flat, s.offsets, s.lengths, BAND_WIDTH, BLOSUM62, n_threads=threads)
        dt = time.perf_counter() - t
    rng = np.random.default_rng(0)
    sample = pairs[rng.permutation(len(pairs))]
    # one thread, on a ~3 s slice of the pairs in random order
    n1 = int(min(len(pairs), max(50, len(pairs) * 3.0 / max(dt_port * threads, 1e-3))))
    p1 = sample[:n1]
    oracle.set_num_threads(1)
    t = time.perf_counter()
    if kind == "reference":
        oracle.ref_sw_batch(p1, s.flat, s.offsets, s.lengths, BAND_WIDTH, BLOSUM62, n_threads=1)
    else:
        oracle.sw_batch(p1, s.flat, s.offsets, s.lengths, BAND_WIDTH, BLOSUM62)
    dt1 = time.perf_counter() - t
    cells1 = int(pair_cells(p1, s.lengths, BAND_WIDTH).sum())
    oracle.set_num_threads(threads)
    base = {"value": cells / dt / 1e9, "unit": "GCUPS", "cores": threads, "kind": kind,
            "pairs_per_s": len(pairs) / dt,
            "sample": f"every pair of the workload ({len(pairs)} pairs, {cells} cells), {threads} threads, "
                      f"{dt:.1f}s",
            "single_thread": {"value": cells1 / dt1 / 1e9, "unit": "GCUPS", "pairs_per_s": n1 / dt1,
                              "sample": f"{n1} random pairs ({cells1} cells), 1 thread, {dt1:.1f}s"}}
    return base, ref


def oracle_on_sample(s, pairs, band_width, n, seed, results=None, hints=None):
    """The oracle (all host threads) on a random sample of n pairs; with
    results (this engine's outputs for every pair), whether they agree."""
    import oracle
    from clustkit_gb300.blosum import BLOSUM62
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(len(pairs), size=min(n, len(pairs)), replace=False))
    oracle.set_num_threads(os.cpu_count() or 1)
    t = time.perf_counter()
    ref = oracle.sw_batch(pairs[idx], s.flat, s.offsets, s.lengths, band_width, BLOSUM62,
                          diag_hints=None if hints is None else hints[idx])
    dt = time.perf_counter() - t
    out = {"pairs": int(len(idx)), "oracle_s": round(dt, 2)}
    if results is not None:
        out["bit_exact"] = same_as_oracle({k: np.asarray(v)[idx] for k, v in results.items()}, ref)
    return out, idx, ref


# ----------------------------------------------------------------------------- arms
def run_reference(args, world, rank):
    if rank != 0:
        return
    from clustkit_gb300.cells import pair_cells
    s, pairs, n_cand = build_workload(use_gpu=False, quick=args.quick)
    import oracle
    from clustkit_gb300.blosum import BLOSUM62
    threads = os.cpu_count() or 1
    kind = "reference" if oracle.ref_available() else "port"
    rng = np.random.default_rng(1)
    order = rng.permutation(len(pairs))
    # size one step to ~4 s of host work
    probe = pairs[order[:1000]]
    t = time.perf_counter()
    oracle.set_num_threads(threads)
    oracle.sw_batch(probe, s.flat, s.offsets, s.lengths, BAND_WIDTH, BLOSUM62)
    dt = time.perf_counter() - t
    per_step = int(min(len(pairs), max(1000, 1000 * 4.0 / max(dt, 1e-3))))

    def step(k):
        sel = order[(k * per_step) % len(pairs):][:per_step]
        p = pairs[sel] if len(sel) == per_step else pairs[order[:per_step]]
        t0 = time.perf_counter()
        if kind == "reference":
            oracle.ref_sw_batch(p, s.flat, s.offsets, s.lengths, BAND_WIDTH, BLOSUM62, n_threads=threads)
        else:
            oracle.sw_batch(p, s.flat, s.offsets, s.lengths, BAND_WIDTH, BLOSUM62)
        return time.perf_counter() - t0, int(pair_cells(p, s.lengths, BAND_WIDTH).sum()), len(p)

    for k in range(args.warmup):
        step(k)
    tt = cc = pp = 0
    for k in range(args.steps):
        dt, c, n = step(args.warmup + k)
        tt += dt; cc += c; pp += n
    gcups = cc / tt / 1e9
    line = {"metric": "banded-SW GCUPS (Align phase, 50k-sequence clustering set)", "value": gcups,
            "unit": "GCUPS", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": tt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)",
            "config": dict(WORKLOAD, sample=f"{per_step} random pairs per step"),
            "impl": "reference", "pairs_per_s": pp / tt,
            "cpu_baseline": {"value": gcups, "unit": "GCUPS", "cores": threads, "kind": kind,
                             "sample": f"{per_step} pairs per step of {len(pairs)}"},
            "e2e": {"value": gcups, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch
    from clustkit_gb300 import _lib
    from clustkit_gb300.blosum import BLOSUM62
    from clustkit_gb300.cells import pair_cells
    from clustkit_gb300.pairwise import ENGINE_BATCHED, ENGINE_PLAIN, PASS_CPU

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    lib = _lib.load()
    _lib.require_gpu()
    if args.rows:
        _lib.set_config(_lib.CFG_ROWS_PER_STRIP, args.rows)
    if args.variant >= 0:
        _lib.set_config(_lib.CFG_STRIP_VARIANT, args.variant)
    if args.threads:
        _lib.set_config(_lib.CFG_STRIP_THREADS, args.threads)
    if args.strip_key:
        _lib.set_config(_lib.CFG_STRIP_KEY, args.strip_key)
    s, pairs, n_cand = build_workload(use_gpu=True, quick=args.quick)
    pairs = shard(pairs, world, rank)
    M = len(pairs)
    cells = int(pair_cells(pairs, s.lengths, BAND_WIDTH).sum())
    dev = torch.device("cuda", local)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_pairs, d_flat, d_off, d_len = T(pairs), T(s.flat), T(s.offsets), T(s.lengths)
    out = {k: torch.empty(M, dtype=dt, device=dev) for k, dt in
           (("sims", torch.float32), ("scores", torch.int32), ("matches", torch.int32),
            ("shorter", torch.int32), ("mask", torch.uint8))}
    sub = np.ascontiguousarray(BLOSUM62)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def launch(engine):
        st = lib.ck_sw_batch_device(
            d_pairs.data_ptr(), M, d_flat.data_ptr(), len(s.flat), d_off.data_ptr(), d_len.data_ptr(),
            s.n, BAND_WIDTH, sub.ctypes.data, THRESHOLD, None, PASS_CPU, engine,
            out["sims"].data_ptr(), out["scores"].data_ptr(), out["matches"].data_ptr(),
            out["shorter"].data_ptr(), out["mask"].data_ptr(), stream.cuda_stream)
        _lib.check(st)

    def timed(engine, steps, warmup, kernel_times=None):
        for _ in range(warmup):
            launch(engine)
        _lib.check(lib.ck_sw_status_device(stream.cuda_stream))
        torch.cuda.synchronize()
        barrier(world)
        total = 0.0
        launches = 0
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        for k in range(steps):
            flush.fill_(k & 0xFF)  # evict L2 between steps (outside the step events)
            ev[k][0].record(stream)
            launch(engine)
            ev[k][1].record(stream)
            launches += _lib.sw_counters()["launches"]
            if kernel_times is not None:
                ms = np.zeros(1, np.float32)
                _lib.check(lib.ck_sw_last_kernel_ms(ms.ctypes.data))
                kernel_times.append(float(ms[0]))
        torch.cuda.synchronize()
        barrier(world)
        total = sum(a.elapsed_time(b) for a, b in ev) / 1e3
        _lib.check(lib.ck_sw_status_device(stream.cuda_stream))
        return max_over_ranks(total, world), launches

    # ---- batched engine, device-resident inputs (value)
    clocks = ClockSampler(local)
    lib.ck_sw_profile(1)
    kt = []
    clocks.start()
    t_batched, launches = timed(ENGINE_BATCHED, args.steps, args.warmup, kt)
    clk = clocks.stop()
    lib.ck_sw_profile(0)
    res_b = {k: v.cpu().numpy() for k, v in out.items()}
    # the same step with the other key form of the strip kernel (compact key for
    # pairs of <= 2047 rows, or the wide key for every pair): speed and results
    key_now = _lib.get_config(_lib.CFG_STRIP_KEY)
    _lib.set_config(_lib.CFG_STRIP_KEY, 1 - key_now)
    t_other, _ = timed(ENGINE_BATCHED, 3, 1)
    other_same = all(np.array_equal(res_b[k], v.cpu().numpy()) for k, v in out.items())
    _lib.set_config(_lib.CFG_STRIP_KEY, key_now)
    gc_this = cells / (t_batched / args.steps) / 1e9
    gc_other = cells / (t_other / 3) / 1e9
    key_forms = {"compact_gcups": round(gc_other if key_now else gc_this, 1),
                 "wide_gcups": round(gc_this if key_now else gc_other, 1),
                 "results_identical": bool(other_same), "in_use": "wide" if key_now else "compact"}
    sweep = {}
    if args.sweep:
        keys = (_lib.CFG_ROWS_PER_STRIP, _lib.CFG_STRIP_VARIANT, _lib.CFG_STRIP_THREADS)
        keep = [_lib.get_config(k) for k in keys]
        for rows in (8, 16, 24, 32):
            for nt in ((512, 640, 768) if rows == 8 else (0,)):
                for var in range(4):
                    for k, v in zip(keys, (rows, var, nt)):
                        _lib.set_config(k, v)
                    t_r, _ = timed(ENGINE_BATCHED, 3, 1)
                    sweep[f"R{rows}_V{var}_T{nt or (512 if rows == 16 else 256)}"] = round(cells / (t_r / 3) / 1e9, 1)
        for k, v in zip(keys, keep):
            _lib.set_config(k, v)
    # ---- plain engine (the plain GPU form), same pairs
    plain_steps = max(1, min(args.steps, 3))
    lib.ck_sw_profile(1)
    kt_plain = []
    t_plain, _ = timed(ENGINE_PLAIN, plain_steps, 1, kt_plain)
    lib.ck_sw_profile(0)
    res_p = {k: v.cpu().numpy() for k, v in out.items()}
    engines_agree = all(np.array_equal(res_b[k], res_p[k]) for k in res_b)


    # ---- e2e through the host-buffer C entry point, pinned host memory
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    h_pairs, h_flat, h_off, h_len = pin(pairs), pin(s.flat), pin(s.offsets), pin(s.lengths)
    h_out = {k: pin(np.empty(M, dt)) for k, dt in (("sims", np.float32), ("scores", np.int32),
                                                   ("matches", np.int32), ("shorter", np.int32),
                                                   ("mask", np.uint8))}

    def host_call():
        _lib.check(lib.ck_sw_batch(
            h_pairs.ctypes.data, M, h_flat.ctypes.data, len(h_flat), h_off.ctypes.data, h_len.ctypes.data,
            s.n, BAND_WIDTH, sub.ctypes.data, THRESHOLD, None, PASS_CPU, ENGINE_BATCHED,
            h_out["sims"].ctypes.data, h_out["scores"].ctypes.data, h_out["matches"].ctypes.data,
            h_out["shorter"].ctypes.data, h_out["mask"].ctypes.data))

    for _ in range(max(1, args.warmup)):
        host_call()
    barrier(world)
    e2e_t = 0.0
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_call()
        e2e_t += time.perf_counter() - t0
    e2e_t = max_over_ranks(e2e_t, world)
    e2e_ok = all(np.array_equal(h_out[k], res_b[k]) for k in res_b)
    h2d = pairs.nbytes + s.flat.nbytes + s.offsets.nbytes + s.lengths.nbytes
    d2h = M * (4 + 4 + 4 + 4 + 1)

    # ---- roofline (integer issue bound) and CPU baseline
    peak = np.zeros(1, np.float64)
    rates = {}
    for which, name in ((0, "viaddmax_s32"), (1, "vimax3_s32"), (2, "iadd3_s32"), (3, "viaddmax_s16x2"),
                        (4, "lop3_b32"), (5, "imad_s32")):
        _lib.check(lib.ck_probe_int_rate(which, peak.ctypes.data))
        rates[name] = float(peak[0])
    # the recurrence's max-plus ops are DPX instructions: their measured rate is the roof
    p_int32 = rates["viaddmax_s32"]
    # cell arithmetic alone, in the exact int32 form and two int16x2 forms
    cell_forms = {}
    for form, name in ((0, "int32_exact_key"), (1, "int16x2_score_only"), (2, "int16x2_match_select"),
                       (3, "int32_exact_key_skewed_halves"), (4, "int32_compact_key_ext_counter")):
        _lib.check(lib.ck_probe_cell_rate(form, peak.ctypes.data))
        cell_forms[name] = float(peak[0]) / 1e9
    kernel_s = float(np.mean(kt)) / 1e3 if kt and min(kt) > 0 else t_batched / args.steps
    gcups_kernel = cells / kernel_s / 1e9
    achieved = gcups_kernel * OPS_PER_CELL  # Gop/s
    # ---- clustkit's CPU algorithm on every pair: the host-core baseline and the
    # oracle every GPU output of the step is compared with (--no-cpu: a 3,000-pair
    # sample instead, for quick runs)
    if rank == 0 and not args.no_cpu:
        cpu, ref_all = cpu_baseline(s, pairs)
        parity = {"vs_oracle_all_pairs": same_as_oracle(res_b, ref_all, THRESHOLD), "oracle_pairs": int(M)}
        del ref_all
    else:
        cpu = None
        chk, _, _ = oracle_on_sample(s, pairs, BAND_WIDTH, 3000, 7, res_b)
        parity = {"vs_oracle_sample": chk["bit_exact"], "oracle_pairs": chk["pairs"]}
    gpu_ref = (reference_gpu_baseline(s, pairs, d_flat, d_off, d_len, stream)
               if (rank == 0 and not args.no_cpu) else None)

    gcups = world * cells / t_batched * args.steps / 1e9
    line = {
        "metric": "banded-SW GCUPS (Align phase, 50k-sequence clustering set)",
        "value": gcups, "unit": "GCUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_batched / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded families; no public dataset)",
        "config": dict(WORKLOAD, pairs=M, lsh_candidates=n_cand, cells_per_step=cells,
                       engine="batched (length-sorted persistent strip kernel)"),
        "pairs_per_s": world * M / t_batched * args.steps,
        "plain": {"value": world * cells / t_plain * plain_steps / 1e9, "unit": "GCUPS",
                  "pairs_per_s": world * M / t_plain * plain_steps,
                  "kernel_ms": float(np.mean(kt_plain)) if kt_plain else None, "steps": plain_steps},
        "speedup_vs_plain": (cells / (t_batched / args.steps)) / (cells / (t_plain / plain_steps)),
        "bit_exact": {"batched_vs_plain_all_pairs": bool(engines_agree), "e2e_vs_device": bool(e2e_ok),
                      **parity},
        "e2e": {"value": world * cells / e2e_t * args.steps / 1e9, "unit": "GCUPS",
                "pairs_per_s": world * M / e2e_t * args.steps,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "api": "ck_sw_batch (host buffers, pinned)"},
        "roofline": {"bound": "int", "achieved": achieved, "peak": p_int32 / 1e9, "unit": "Gop/s",
                     "frac": achieved / (p_int32 / 1e9), "traffic": STRIP_DRAM_BYTES_PER_CELL * cells,
                     "traffic_source": f"not measured in this run: ncu DRAM bytes per cell from {STRIP_PROFILE} "
                                       f"x this run's {cells} cells (same workload, same kernel settings)",
                     "basis": f"{OPS_PER_CELL} int32 max-plus lane-ops per cell x cells / strip-kernel "
                              f"event time; peak = measured int32 DPX/ALU lane-op rate (in-repo probe)",
                     "kernel": "sw_strip_kernel", "kernel_ms": kernel_s * 1e3,
                     "gcups_kernel": gcups_kernel, "gcups_roof": p_int32 / 1e9 / OPS_PER_CELL,
                     "probe_gops": {k: v / 1e9 for k, v in rates.items()},
                     "frac_of_int16x2_roof": gcups_kernel / (rates["viaddmax_s16x2"] / 1e9 / OPS_PER_CELL),
                     "cell_form_probe_gcups": cell_forms,
                     "hbm_check": hbm_check(s, pairs, kernel_s, cells)},
        "cpu_baseline": cpu,
        "reference_cupy_path": gpu_ref,
        "rows_per_strip": _lib.get_config(_lib.CFG_ROWS_PER_STRIP),
        "strip_variant": _lib.get_config(_lib.CFG_STRIP_VARIANT),
        "strip_key_forms": key_forms,
        "sweep_gcups": sweep or None,
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    if rank == 0 and (args.million == "on" or (args.million == "auto" and not args.quick)):
        try:
            line["million"] = run_million(args, p_int32)
        except Exception as e:
            line["million"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and (args.uneven == "on" or (args.uneven == "auto" and not args.quick)):
        try:
            line["uneven"] = run_uneven(args)
        except Exception as e:  # the SW line stands; the failure is reported in it
            line["uneven"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and (args.search == "on" or (args.search == "auto" and not args.quick)):
        try:
            line["search"] = run_search(args)
        except Exception as e:  # the SW line stands; the failure is reported in it
            line["search"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ----------------------------------------------------------------------------- uneven lengths / autotuner
def run_uneven(args):
    """Heavy-tailed lengths (Pareto alpha 1.5, 30..8000), 2M pairs (half within
    family, half random, length ratio >= 0.5); per band width the default
    setting, the autotuned one and the plain kernel, all pairs compared."""
    from clustkit_gb300 import _lib, synth, tune
    n_fam, n_pairs = (200, 200_000) if args.quick else (2000, 2_000_000)
    s = synth.generate_families(n_fam, 10, median=0, lo=30, hi=8000, seed=17, length_dist="pareto")
    pairs = synth.mixed_pairs(s, n_pairs, seed=5, within_frac=0.5, min_ratio=0.5)
    out = {"workload": f"uneven: {s.n} seqs Pareto(1.5) 30..8000, {len(pairs)} pairs (50% within family, "
                       f"ratio >= 0.5)", "by_band": {}}
    for bw in (16, 32, 64, 128):
        call = tune._DeviceCall(pairs, s.flat, s.offsets, s.lengths, bw)
        tune.apply(tune.DEFAULT)
        ms_default = call.time_ms(3)
        res = tune.autotune(pairs, s.flat, s.offsets, s.lengths, bw, use_cache=False)
        ms_tuned = call.time_ms(3)
        tuned = call.results()
        from clustkit_gb300.pairwise import batch_sw  # host entry point: reads the routing counters
        batch_sw(pairs, s.flat, s.offsets, s.lengths, bw)
        wave = _lib.sw_counters()["wave"]
        ms_plain = call.time_ms(1, warmup=0, engine=1)
        plain = call.results()
        tune.apply(tune.DEFAULT)
        same = all(np.array_equal(tuned[k], plain[k]) for k in ("scores", "matches", "shorter", "mask"))
        g = lambda ms: res.cells / (ms * 1e-3) / 1e9
        # the tuned engine's outputs against the oracle on a random sample of the pairs
        vs_oracle = None
        if not args.no_cpu:
            vs_oracle, _, _ = oracle_on_sample(s, pairs, bw, 250_000 if not args.quick else 20_000, bw, tuned)
        out["by_band"][str(bw)] = {"cells": res.cells, "gcups_default": g(ms_default), "gcups_tuned": g(ms_tuned),
                                   "gcups_plain": g(ms_plain), "tuned_vs_plain": ms_plain / ms_tuned,
                                   "config": res.config, "confirm": res.confirm, "wave_pairs": wave,
                                   "trials": len(res.trials), "bit_exact_vs_plain": bool(same),
                                   "vs_oracle_sample": vs_oracle}
        log(f"uneven bw={bw}: {out['by_band'][str(bw)]}")
        del call
    return out


# ----------------------------------------------------------------------------- 1M-sequence streaming
def run_million(args, int_peak=None):
    """1,000,000 sequences (100,000 families x 10, median 300, 30..1500), t = 0.4:
    sketches on the GPU, LSH on the GPU, the Jaccard pre-filter on the GPU, then
    every surviving pair through the batched SW engine in device-resident
    chunks.  Reports each stage's time, GCUPS and pairs/s of the SW stream."""
    import torch
    from clustkit_gb300 import _lib, synth
    from clustkit_gb300.blosum import BLOSUM62
    from clustkit_gb300.cells import band_cells, effective_band
    from clustkit_gb300.lsh import auto_lsh_params, lsh_candidates_device
    from clustkit_gb300.pairwise import ENGINE_BATCHED, PASS_CPU
    lib = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    n_fam = 10_000 if args.quick else 100_000
    t0 = time.time()
    s = synth.generate_families(n_fam, 10, median=300, lo=30, hi=1500, seed=31)
    t_gen = time.time() - t0
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_flat, d_off, d_len = T(s.flat), T(s.offsets), T(s.lengths)
    stream = torch.cuda.current_stream(dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    e0, e1, e2, e3 = ev(), ev(), ev(), ev()
    sk = torch.empty((s.n, 128), dtype=torch.int64, device=dev)
    e0.record(stream)
    _lib.check(lib.ck_sketch_device(d_flat.data_ptr(), len(s.flat), d_off.data_ptr(), d_len.data_ptr(), s.n, 5,
                                    128, 20, 42, sk.data_ptr(), stream.cuda_stream))
    e1.record(stream)
    lp = auto_lsh_params(THRESHOLD_MILLION, "medium", 5)
    t1 = time.time()
    cand = lsh_candidates_device(sk, lp["num_tables"], lp["num_bands"], 42)
    torch.cuda.synchronize()
    t_lsh = time.time() - t1
    n_cand = int(cand.shape[0])
    # Jaccard pre-filter (clustkit/pairwise.py:949-1001): the 2000-pair cost check
    # drawn with RandomState(0) on the host, the filter itself on the device
    floor = max(0.001, 0.3 * THRESHOLD_MILLION ** 5)
    sims = torch.empty(n_cand, dtype=torch.float32, device=dev)
    mask = torch.empty(n_cand, dtype=torch.uint8, device=dev)
    e2.record(stream)
    _lib.check(lib.ck_jaccard_device(cand.data_ptr(), n_cand, sk.data_ptr(), s.n, 128, float(np.float32(floor)),
                                     sims.data_ptr(), mask.data_ptr(), stream.cuda_stream))
    e3.record(stream)
    rng = np.random.RandomState(0)
    sample = rng.choice(n_cand, size=min(2000, n_cand), replace=False) if n_cand > 2000 else np.arange(n_cand)
    est = float((sims[T(sample)].cpu().numpy() < np.float32(floor)).mean()) if n_cand else 0.0
    pairs = cand[mask.bool()] if est >= 0.05 else cand
    del cand, sims, mask
    M = int(pairs.shape[0])
    L = s.lengths.astype(np.int64)
    ph = pairs.cpu().numpy()
    la = np.minimum(L[ph[:, 0]], L[ph[:, 1]])
    lb = np.maximum(L[ph[:, 0]], L[ph[:, 1]])
    cells = int(band_cells(la, lb, effective_band(la, lb, BAND_WIDTH)).sum())
    del ph, la, lb
    chunk = 20_000_000
    outs = [torch.empty(min(chunk, max(M, 1)), dtype=dt, device=dev)
            for dt in (torch.float32, torch.int32, torch.int32, torch.int32, torch.uint8)]
    sub = np.ascontiguousarray(BLOSUM62)

    def sw_stream():
        for c0 in range(0, M, chunk):
            m = min(chunk, M - c0)
            _lib.check(lib.ck_sw_batch_device(
                pairs[c0:].data_ptr(), m, d_flat.data_ptr(), len(s.flat), d_off.data_ptr(), d_len.data_ptr(),
                s.n, BAND_WIDTH, sub.ctypes.data, THRESHOLD_MILLION, None, PASS_CPU, ENGINE_BATCHED,
                outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr(), outs[3].data_ptr(), outs[4].data_ptr(),
                stream.cuda_stream))

    sw_stream()  # warm-up (scratch sized for the largest chunk)
    torch.cuda.synchronize()
    a, b = ev(), ev()
    a.record(stream)
    sw_stream()
    b.record(stream)
    b.synchronize()
    _lib.check(lib.ck_sw_status_device(stream.cuda_stream))
    sw_ms = a.elapsed_time(b)
    gcups = cells / (sw_ms * 1e-3) / 1e9
    # the same stream with every full chunk replayed from one captured CUDA graph:
    # the chunk's pairs are copied into a fixed buffer, the graph holds the whole
    # batched call (prep, sort, routing, alignment kernel, fallback) on a context
    # whose scratch is frozen after a sizing call; the last, partial chunk runs directly
    graph_ms = None
    if M >= chunk:
        h = np.zeros(1, np.int32)
        _lib.check(lib.ck_ctx_create(h.ctypes.data))
        ctx = int(h[0])
        buf = torch.empty((chunk, 2), dtype=torch.int32, device=dev)
        gstream = torch.cuda.Stream(dev)

        def ctx_call(p_ptr, m, st):
            _lib.check(lib.ck_sw_batch_device_ctx(
                ctx, p_ptr, m, d_flat.data_ptr(), len(s.flat), d_off.data_ptr(), d_len.data_ptr(), s.n, BAND_WIDTH,
                sub.ctypes.data, THRESHOLD_MILLION, None, PASS_CPU, ENGINE_BATCHED, outs[0].data_ptr(),
                outs[1].data_ptr(), outs[2].data_ptr(), outs[3].data_ptr(), outs[4].data_ptr(), st))

        with torch.cuda.stream(gstream):
            buf.copy_(pairs[:chunk])
            ctx_call(buf.data_ptr(), chunk, gstream.cuda_stream)
        gstream.synchronize()
        _lib.check(lib.ck_ctx_status(ctx, gstream.cuda_stream))
        _lib.check(lib.ck_ctx_freeze(ctx, 1))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=gstream, capture_error_mode="thread_local"):
            ctx_call(buf.data_ptr(), chunk, gstream.cuda_stream)
        ga, gb = ev(), ev()
        with torch.cuda.stream(gstream):
            ga.record(gstream)
            for c0 in range(0, M, chunk):
                m = min(chunk, M - c0)
                if m == chunk:
                    buf.copy_(pairs[c0:c0 + chunk], non_blocking=True)
                    g.replay()
                else:
                    ctx_call(pairs[c0:].data_ptr(), m, gstream.cuda_stream)
            gb.record(gstream)
        gb.synchronize()
        _lib.check(lib.ck_ctx_status(ctx, gstream.cuda_stream))
        graph_ms = ga.elapsed_time(gb)
        del g
        lib.ck_ctx_destroy(ctx)
    # every output of a random sample of the streamed pairs against the oracle: the
    # stream runs once more (untimed) and the sampled pairs' results are gathered
    # from each chunk's outputs
    vs_oracle = None
    if not args.no_cpu and M:
        import oracle
        rng = np.random.default_rng(4)
        idx = np.sort(rng.choice(M, size=min(M, 100_000 if args.quick else 2_000_000), replace=False))
        samp_pairs = pairs[T(idx)].cpu().numpy()
        got = {k: np.empty(len(idx), dt) for k, dt in (("sims", np.float32), ("scores", np.int32),
                                                       ("matches", np.int32), ("shorter", np.int32))}
        for c0 in range(0, M, chunk):
            m = min(chunk, M - c0)
            _lib.check(lib.ck_sw_batch_device(
                pairs[c0:].data_ptr(), m, d_flat.data_ptr(), len(s.flat), d_off.data_ptr(), d_len.data_ptr(),
                s.n, BAND_WIDTH, sub.ctypes.data, THRESHOLD_MILLION, None, PASS_CPU, ENGINE_BATCHED,
                outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr(), outs[3].data_ptr(), outs[4].data_ptr(),
                stream.cuda_stream))
            sel = (idx >= c0) & (idx < c0 + m)
            loc = T(idx[sel] - c0)
            for k, o in zip(("sims", "scores", "matches", "shorter"), outs):
                got[k][sel] = o[loc].cpu().numpy()
        oracle.set_num_threads(os.cpu_count() or 1)
        t_o = time.perf_counter()
        ref = oracle.sw_batch(samp_pairs, s.flat, s.offsets, s.lengths, BAND_WIDTH, BLOSUM62)
        vs_oracle = {"pairs": int(len(idx)), "bit_exact": same_as_oracle(got, ref),
                     "oracle_s": round(time.perf_counter() - t_o, 2)}
        del ref, got, samp_pairs
    peak = int_peak if int_peak else None
    out = {"workload": f"million: {s.n} seqs ({n_fam} families x 10, median 300, 30..1500), t={THRESHOLD_MILLION}, "
                       f"k=5 s=128, LSH b={lp['num_bands']} L={lp['num_tables']}, Jaccard floor {floor:.6f}, "
                       f"bw={BAND_WIDTH}",
           "generate_s": t_gen, "sketch_ms": e0.elapsed_time(e1), "lsh_s": t_lsh, "lsh_candidates": n_cand,
           "jaccard_ms": e2.elapsed_time(e3), "prefilter_applied": est >= 0.05, "pairs": M, "cells": cells,
           "sw_ms": sw_ms, "gcups": gcups, "pairs_per_s": M / (sw_ms * 1e-3), "chunk_pairs": chunk,
           "sw_ms_graph_replay": graph_ms,
           "gcups_graph_replay": cells / (graph_ms * 1e-3) / 1e9 if graph_ms else None,
           "roofline_frac": gcups * 1e9 * OPS_PER_CELL / peak if peak else None,
           "roofline_peak_gops": peak / 1e9 if peak else None,
           "roofline_basis": "SW-stream GCUPS x 6 ops per cell / the int32 DPX lane-op rate measured by the "
                             "in-library probe in this run",
           "hbm_gbs_est": gcups * STRIP_DRAM_BYTES_PER_CELL,
           "hbm_basis": f"not measured in this run: {STRIP_DRAM_BYTES_PER_CELL:.3f} DRAM bytes per cell from "
                        f"{STRIP_PROFILE} (ncu, the strip kernel on the 50k set) x this run's GCUPS",
           "vs_oracle_sample": vs_oracle}
    log(f"million: {out}")
    return out


# ----------------------------------------------------------------------------- search / serving
def make_queries(s, n, seed=11):
    """Half mutated database members (30-90% identity), half background;
    lengths lognormal, median 300, clipped 50..2000."""
    from clustkit_gb300 import synth
    rng = np.random.default_rng(seed)
    L = np.clip(np.rint(np.exp(np.log(300) + 0.5 * rng.standard_normal(n))), 50, 2000).astype(int)
    bg = synth.random_sequences(n, median=300, lo=50, hi=2000, seed=seed + 1)
    qs = []
    for i in range(n):
        if i % 2 == 0:
            m = s.seq(int(rng.integers(s.n))).copy()
            ln = min(int(L[i]), len(m))
            st = int(rng.integers(0, len(m) - ln + 1))
            q = m[st:st + ln]
            mut = rng.random(ln) < rng.uniform(0.1, 0.7)
            q[mut] = rng.integers(0, 20, int(mut.sum()))
            qs.append(q.astype(np.uint8))
        else:
            qs.append(bg.seq(i).copy())
    return qs


def run_search(args, n_db_fam=50000):
    """Resident 500k-sequence database; continuous-batching server under
    Poisson arrivals swept over rates, against a one-query-at-a-time loop."""
    import torch
    from clustkit_gb300 import synth
    from clustkit_gb300.search import DeviceDatabase, SearchServer, _Slot, search_batch
    t0 = time.time()
    s = synth.generate_families(n_db_fam, 10, median=350, lo=30, hi=2000, seed=7)
    t1 = time.time()
    B = int(args.search_batch)
    db = DeviceDatabase(s.flat, s.offsets, s.lengths, arena_slots=4, arena_queries=B,
                        arena_residues=B * 2000)
    t2 = time.time()
    log(f"search db: {s.n} seqs gen {t1 - t0:.1f}s, index+sketch {t2 - t1:.1f}s, "
        f"{db.n_entries} index entries, band {db.band_width}, freq cap {db.freq_thresh}")
    qs = make_queries(s, 6000)
    modes = set(args.search_modes.split(","))
    out = {"db_sequences": int(s.n), "db_residues": int(s.flat.size), "index_entries": db.n_entries,
           "band_width": db.band_width, "max_cands": 500, "top_k": 10}
    if "exact" in modes:
        exact = _measure_search_mode(db, qs, 0, (100, 1000, 3000, 10000, 20000), n_plain=300, n_stage=50,
                                     n_batch=5, batches_only=args.search_batches_only)
        if not args.no_cpu and not args.search_batches_only:
            try:
                exact["cpu_baseline"] = search_cpu_baseline(db, s, qs, mode="exact")
                log(f"search exact 5-mers on the host cores: {exact['cpu_baseline']}")
            except Exception as e:  # a baseline that fails leaves the GPU figures standing
                exact["cpu_baseline_error"] = repr(e)
        out.update({"slots": exact.pop("slots", None), "kmer_scoring": "exact 5-mers (kmer_score_thresh 0)",
                    **exact})
    if "similar" in modes:
        # clustkit's default scoring (BLOSUM62 similar 5-mers, threshold 13):
        # far more k-mer work per query, so the rates follow its batch rate
        similar = _measure_search_mode(db, qs[3000:], 13, None, n_plain=30, n_stage=10, n_batch=3,
                                       batches_only=args.search_batches_only)
        if not args.no_cpu and not args.search_batches_only:
            try:
                similar["cpu_baseline"] = search_cpu_baseline_similar(db, s, qs[3000:])
                log(f"search similar 5-mers on the host cores: {similar['cpu_baseline']}")
            except Exception as e:  # a baseline that fails leaves the GPU figures standing
                similar["cpu_baseline_error"] = repr(e)
        out["similar_kmers_thresh13"] = similar
    if "c_path" in modes:
        # clustkit's C path: exact 5-mers with Phase B (min_diag_hits 2, bin
        # 10, Phase-A top 10,000), SW at band 50 centred on the diagonal hints
        c_path = _measure_search_mode(db, qs[1500:], 0, None, n_plain=100, n_stage=20, n_batch=3,
                                      scoring={"min_diag_hits": 2, "diag_bin_width": 10, "phase_a_topk": 10000,
                                               "use_c_scoring": True, "use_c_sw": True, "c_sw_band_width": 50},
                                      batches_only=args.search_batches_only)
        if not args.no_cpu and not args.search_batches_only:
            c_path["cpu_baseline"] = search_cpu_baseline(db, s, qs[1500:])
            log(f"search C path on the host cores: {c_path['cpu_baseline']}")
        out["c_path_phase_b_hinted_sw"] = c_path
    if not args.search_batches_only:
        out["summary"] = search_summary(out)
    return out


def search_summary(out):
    """One line per scoring mode: the one-query loop, the server at its lowest
    offered rate and its highest achieved rate (p50/p99 in ms)."""
    modes = {"exact": out if "plain_loop" in out else None, "similar": out.get("similar_kmers_thresh13"),
             "c_path": out.get("c_path_phase_b_hinted_sw")}
    summ = {}
    for name, m in modes.items():
        if not m:
            continue
        sweep = m["continuous_batching"]
        low, top = sweep[0], max(sweep, key=lambda r: r["achieved_qps"])
        summ[name] = {"one_query_p50_ms": m["plain_loop"]["p50_ms"],
                      "server_low_rate": {"offered_qps": low["offered_qps"], "p50_ms": low["p50_ms"],
                                          "p99_ms": low["p99_ms"]},
                      "server_max_achieved_qps": top["achieved_qps"],
                      "at_max": {"offered_qps": top["offered_qps"], "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"]}}
        if "cpu_baseline" in m:
            summ[name]["host_cores_qps"] = m["cpu_baseline"]["value"]
            summ[name]["server_vs_host_cores"] = top["achieved_qps"] / m["cpu_baseline"]["value"]
    return summ


def search_cpu_baseline(db, s, qs, target_s: float = 10.0, mode: str = "c_path"):
    """A search chain of clustkit's on the host cores, as C restatements (the
    port), on a sample of the same queries; queries/s of the whole chain with
    the index resident in host memory.
      mode "c_path": the C k-mer scorer (kmer_score.c, Phase A + Phase B +
        hints, OpenMP over queries), the C SW at band 50 centred on the hints;
      mode "exact": the same scorer with Phase B off -- exact 5-mer hit
        counts, at least 2 hits, the top 500 (kmer_index.py:470-534) -- and
        the C SW at the database band, unhinted (kmer_index.py:2226-2311);
    both followed by the rank (sw_align.c over pairs, OpenMP)."""
    import oracle
    from oracle import search_oracle as so
    from clustkit_gb300.blosum import BLOSUM62
    threads = os.cpu_count() or 1
    oracle.set_num_threads(threads)
    off, ent, fr = db.index_arrays()
    mc, topk = 500, 10000
    exact = mode == "exact"
    min_diag, band = (0, db.band_width) if exact else (2, 50)

    def run(sample):
        lens = np.array([len(q) for q in sample], np.int32)
        q_off = np.zeros(len(sample), np.int64)
        q_off[1:] = np.cumsum(lens[:-1])
        q_flat = np.concatenate(sample).astype(np.uint8)
        flat = np.concatenate([s.flat, q_flat])
        offs = np.concatenate([s.offsets, q_off + len(s.flat)])
        all_lens = np.concatenate([s.lengths, lens])
        t0 = time.perf_counter()
        cands = oracle.kmer_candidates_batch(q_flat, q_off, lens, 5, 20, off, ent, fr, db.freq_thresh, s.n,
                                             2, min_diag, 10, mc, topk)
        t1 = time.perf_counter()
        qi = np.concatenate([np.full(len(c[0]), i, np.int32) for i, c in enumerate(cands)])
        tg = np.concatenate([c[0] for c in cands]).astype(np.int32)
        hints = None if exact else np.concatenate([c[2] for c in cands]).astype(np.int32)
        pairs = np.stack([qi + s.n, tg], axis=1)
        r = oracle.sw_batch(pairs, flat, offs, all_lens, band, BLOSUM62, diag_hints=hints)
        t2 = time.perf_counter()
        keep = r["scores"] > 0
        so.rank_hits(np.stack([qi, tg], axis=1)[keep], r["sims"][keep], r["scores"][keep], lens, s.lengths,
                     len(sample), 10)
        t3 = time.perf_counter()
        return t3 - t0, t1 - t0, t2 - t1, t3 - t2, len(pairs)

    n = 32
    dt = run(qs[:n])[0]
    n = int(min(len(qs), max(n, n * target_s / max(dt, 1e-3))))
    tot, ts, tsw, trank, npairs = run(qs[:n])
    src = ("restatements of clustkit/kmer_index.py:470-534 (Phase A via the C scorer with Phase B off) and "
           "csrc/sw_align.c:25-266" if exact else
           "restatements of clustkit/csrc/kmer_score.c:195-470 and sw_align.c:25-266")
    return {"value": n / tot, "unit": "queries/s", "cores": threads, "kind": "port",
            "stage_s": {"kmer_scorer": ts, "sw": tsw, "rank": trank},
            "sample": f"{n} queries of the stream, {npairs} candidate pairs, {threads} threads, {tot:.1f}s",
            "source": src}


def _similar_chain(off, ent, fr, freq_thresh, s, sample, band, thresh=13, max_cands=500, top_k=10):
    """One pass of the similar-5-mer search chain on the host cores: the
    scorer's C restatement (OpenMP over queries), the C SW at the database
    band (OpenMP over pairs), the rank; (total, scorer, sw, rank seconds,
    candidate pairs)."""
    import oracle
    from oracle import search_oracle as so
    from clustkit_gb300.blosum import BLOSUM62
    lens = np.array([len(q) for q in sample], np.int32)
    q_off = np.zeros(len(sample), np.int64)
    q_off[1:] = np.cumsum(lens[:-1])
    q_flat = np.concatenate(sample).astype(np.uint8)
    flat = np.concatenate([s.flat, q_flat])
    offs = np.concatenate([s.offsets, q_off + len(s.flat)])
    all_lens = np.concatenate([s.lengths, lens])
    t0 = time.perf_counter()
    cands = oracle.similar_candidates_batch(q_flat, q_off, lens, BLOSUM62, thresh, off, ent, fr, freq_thresh, s.n,
                                            2, max_cands)
    t1 = time.perf_counter()
    qi = np.concatenate([np.full(len(c[0]), i, np.int32) for i, c in enumerate(cands)])
    tg = np.concatenate([c[0] for c in cands]).astype(np.int32)
    pairs = np.stack([qi + s.n, tg], axis=1)
    r = oracle.sw_batch(pairs, flat, offs, all_lens, band, BLOSUM62)
    t2 = time.perf_counter()
    keep = r["scores"] > 0
    so.rank_hits(np.stack([qi, tg], axis=1)[keep], r["sims"][keep], r["scores"][keep], lens, s.lengths,
                 len(sample), top_k)
    t3 = time.perf_counter()
    return t3 - t0, t1 - t0, t2 - t1, t3 - t2, len(pairs)


def search_cpu_baseline_similar(db, s, qs, target_s: float = 10.0):
    """clustkit's default search scoring on the host cores, as C restatements
    (the port): the BLOSUM62 similar-5-mer scorer (kmer_index.py:1187-1328,
    OpenMP over queries; clustkit runs it in Numba, absent here), the C SW at
    the database band (sw_align.c, OpenMP over pairs) and the rank, on a sample
    of the same queries; queries/s of the whole chain."""
    import oracle
    threads = os.cpu_count() or 1
    oracle.set_num_threads(threads)
    off, ent, fr = db.index_arrays()
    n = 16
    dt = _similar_chain(off, ent, fr, db.freq_thresh, s, qs[:n], db.band_width)[0]
    n = int(min(len(qs), max(n, n * target_s / max(dt, 1e-3))))
    tot, ts, tsw, trank, npairs = _similar_chain(off, ent, fr, db.freq_thresh, s, qs[:n], db.band_width)
    return {"value": n / tot, "unit": "queries/s", "cores": threads, "kind": "port",
            "stage_s": {"kmer_scorer": ts, "sw": tsw, "rank": trank},
            "sample": f"{n} queries of the stream, {npairs} candidate pairs, {threads} threads, {tot:.1f}s",
            "source": "restatements of clustkit/kmer_index.py:1187-1328 and csrc/sw_align.c:25-266"}


def _batches_only(db, qs, thresh, n_batch, scoring):
    """One warm-up batch, then n_batch full batches and nothing else: the
    launch list of a profiler run then holds only batch pipelines."""
    from clustkit_gb300.search import _Slot, search_batch
    B = db.arena_queries
    slot = _Slot(db, 0, 500)
    slot.enable_stage_timing()
    search_batch(db, qs[:B], top_k=10, slot=slot, kmer_score_thresh=thresh, **scoring)
    stages = []
    for r in range(n_batch):
        search_batch(db, qs[B * (r + 1):B * (r + 2)], top_k=10, slot=slot, kmer_score_thresh=thresh, **scoring)
        stages.append(slot.stage_ms())
    slot.close()
    med = np.median(np.array(stages), axis=0)
    return {"batch_queries": B, "batches": n_batch,
            "device_stage_ms_median_batch": {"h2d": float(med[0]), "phase_a": float(med[1]), "sw": float(med[2]),
                                             "d2h": float(med[3])}}


def _measure_search_mode(db, qs, thresh, rates, n_plain, n_stage, n_batch, scoring=None, batches_only=False):
    from clustkit_gb300.search import SearchServer, _Slot, search_batch
    scoring = scoring or {}
    if batches_only:
        return _batches_only(db, qs, thresh, n_batch, scoring)
    B = db.arena_queries
    slot = _Slot(db, 0, 500)
    for q in qs[:min(20, n_plain)]:
        search_batch(db, [q], top_k=10, slot=slot, kmer_score_thresh=thresh, **scoring)
    lat = []
    tp0 = time.perf_counter()
    for q in qs[:n_plain]:
        a = time.perf_counter()
        search_batch(db, [q], top_k=10, slot=slot, kmer_score_thresh=thresh, **scoring)
        lat.append(time.perf_counter() - a)
    plain_qps = n_plain / (time.perf_counter() - tp0)
    # device time per stage of a one-query batch (separate pass: events add syncs)
    slot.enable_stage_timing()
    stages, cells1 = [], []
    for q in qs[:n_stage]:
        search_batch(db, [q], top_k=10, slot=slot, kmer_score_thresh=thresh, **scoring)
        stages.append(slot.stage_ms())
        cells1.append(slot.last_cells())
    # one untimed full batch first: the slot's buffers were sized by one-query
    # batches (the similar-k-mer neighbour list grows, and lists again, once)
    search_batch(db, qs[B * n_batch:B * (n_batch + 1)], top_k=10, slot=slot, kmer_score_thresh=thresh, **scoring)
    full, cells_b = [], []
    for r in range(n_batch):
        search_batch(db, qs[B * r:B * (r + 1)], top_k=10, slot=slot, kmer_score_thresh=thresh, **scoring)
        full.append(slot.stage_ms())
        cells_b.append(slot.last_cells())
    sw1 = np.array([x[2] for x in stages])
    sw_b = np.array([x[2] for x in full])
    slot.close()
    full_med = np.median(np.array(full), axis=0)
    st_med = np.median(np.array(stages), axis=0)
    plain = {"qps": plain_qps, "p50_ms": float(np.percentile(lat, 50) * 1e3),
             "p99_ms": float(np.percentile(lat, 99) * 1e3), "queries": n_plain,
             "device_stage_ms_median": {"h2d": float(st_med[0]), "phase_a": float(st_med[1]),
                                        "sw": float(st_med[2]), "d2h": float(st_med[3])},
             "batch_queries": B,
             "device_stage_ms_median_batch": {"h2d": float(full_med[0]), "phase_a": float(full_med[1]),
                                                "sw": float(full_med[2]), "d2h": float(full_med[3])},
             "sw_gcups_one_query": float(np.sum(cells1) / np.sum(sw1) / 1e6),
             "sw_gcups_batch": float(np.sum(cells_b) / np.sum(sw_b) / 1e6),
             "cells_per_query": float(np.mean(cells1))}
    if rates is None:
        batch_qps = B / (float(np.sum(full_med)) * 1e-3)
        rates = tuple(int(max(10, round(batch_qps * f, -1))) for f in (0.1, 0.3, 0.6, 0.9))
    server = SearchServer(db, top_k=10, max_cands=500, kmer_score_thresh=thresh, **scoring).start()
    # a serving process keeps its start-up objects (database arrays, query
    # set) out of the cyclic collector, whose full passes over them would
    # pause the scheduler thread for tens of milliseconds
    gc.collect()
    gc.freeze()
    sweep = []
    rng = np.random.default_rng(3)
    qi = 0
    try:
        for rate in rates:
            n = int(min(2000, max(200, rate * 2)))
            arr = np.cumsum(rng.exponential(1.0 / rate, n))
            server.latencies.clear()
            futs = []
            t_start = time.perf_counter()
            for i in range(n):
                target = t_start + arr[i]
                lag = target - time.perf_counter()
                if lag > 0:
                    time.sleep(lag)  # sleeping releases the GIL to the scheduler thread
                futs.append(server.submit(qs[qi % len(qs)], t_arrival=target))
                qi += 1
            for f in futs:
                f.result(timeout=600)
            t_end = time.perf_counter()
            p = server.latency_percentiles()
            sweep.append({"offered_qps": rate, "achieved_qps": n / (t_end - t_start), "queries": n,
                          "p50_ms": p["p50_ms"], "p99_ms": p["p99_ms"], "deferrals": server.deferrals,
                          "peak_in_flight_mb": server.peak_in_flight_bytes / 2 ** 20})
            log(f"search (kmer_score_thresh {thresh}{', C path' if scoring else ''}) rate {rate}/s: {sweep[-1]}")
    finally:
        server.stop()
        gc.unfreeze()
    return {"plain_loop": plain, "continuous_batching": sweep, "slots": len(server.slots),
            "mem_budget_mb": server.mem_budget / 2 ** 20, "batch_mb_full": server.per_slot_bytes / 2 ** 20}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--quick", action="store_true", help="10x smaller workload (smoke-testing the bench)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--search-batch", type=int, default=64,
                    help="most queries per search batch (the server's slot size)")
    ap.add_argument("--search-modes", default="exact,similar,c_path",
                    help="search leg scoring modes: exact, similar, c_path (comma list)")
    ap.add_argument("--search-batches-only", action="store_true",
                    help="search leg: only full batches per mode (a warm-up and a few), for profiler launch lists")
    ap.add_argument("--rows", type=int, default=0, help="rows per strip (8/16/24/32); 0 = library default")
    ap.add_argument("--threads", type=int, default=0,
                    help="strip kernel CTA threads for 8-row strips (512/640/768); 0 = library default")
    ap.add_argument("--strip-key", type=int, default=0, choices=[0, 1],
                    help="1: the strip kernel's wide key for every pair (default 0: compact where rows fit)")
    ap.add_argument("--variant", type=int, default=-1, help="strip kernel variant 0..3; -1 = library default (by strip height)")
    ap.add_argument("--sweep", action="store_true", help="also time every rows-per-strip x variant setting")
    ap.add_argument("--search", choices=["auto", "on", "off", "only"], default="auto",
                    help="search/serving leg (auto: on for the full workload, off with --quick)")
    ap.add_argument("--uneven", choices=["auto", "on", "off", "only"], default="auto",
                    help="heavy-tailed lengths + autotuner leg (auto: on for the full workload)")
    ap.add_argument("--million", choices=["auto", "off", "on", "only"], default="auto",
                    help="1M-sequence leg: GPU sketches, GPU LSH, pre-filter, SW in device-resident chunks "
                         "(auto: on for the full workload)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.million == "only":
        import torch
        from clustkit_gb300 import _lib
        torch.cuda.set_device(local)
        _lib.load()
        _lib.require_gpu()
        print(json.dumps({"metric": "banded-SW GCUPS streaming 1M sequences' LSH pairs in device-resident chunks",
                          "million": run_million(args)}), flush=True)
    elif args.uneven == "only":
        import torch
        from clustkit_gb300 import _lib
        torch.cuda.set_device(local)
        _lib.load()
        _lib.require_gpu()
        print(json.dumps({"metric": "banded-SW GCUPS, heavy-tailed lengths, autotuned vs default vs plain",
                          "uneven": run_uneven(args)}), flush=True)
    elif args.search == "only":
        import torch
        from clustkit_gb300 import _lib
        torch.cuda.set_device(local)
        _lib.load()
        _lib.require_gpu()
        print(json.dumps({"metric": "search queries/s and p50/p99 latency (500k-sequence resident DB)",
                          "search": run_search(args, 5000 if args.quick else 50000)}), flush=True)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
