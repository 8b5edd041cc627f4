"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where the clustkit reference checkout is available (its root is
oracle/build.py's REF_ROOT: the CLUSTKIT_REFERENCE environment variable, else
the build container's mount point):

    python tests/golden/make_golden.py

numba is not installed, so a tiny stand-in module (``njit`` -> identity,
``prange`` -> ``range``, numba scalar types -> numpy scalar types) is placed
in ``sys.modules`` before the reference modules are imported; the reference's
Numba kernels then run as plain Python with numpy scalar arithmetic.  The
reference's C Smith-Waterman (clustkit/csrc/sw_align.c) is compiled from its
source by oracle/build.py and loaded through ctypes, and the reference's
``compute_pairwise_alignment`` is pointed at it (its own loader looks for a
prebuilt .so next to pairwise.py, which the read-only checkout does not have).

Outputs (all small, compressed):
  blosum62_ref.npy      the reference's BLOSUM62 table
  sketch_golden.npz     sequences + reference sketches for several (k, s, alphabet)
  jaccard_golden.npz    sketch pairs + reference _batch_jaccard values
  kmer_scorer_golden.npz  the reference's C k-mer scorer (Phase A/B, caps, hints)
  sw_golden.npz         sequences, pairs, band widths + reference C SW outputs,
                        a diagonal-hint case, and a Numba-twin cross-check subset
  lsh_golden.npz        reference lsh_candidates on the sketches
  pipeline_golden.npz   config-1 sized run: sketches -> LSH -> the reference's
                        compute_pairwise_alignment(use_sw=True, use_c_sw=True)
  search_golden.npz     a 240-sequence database and 20 queries: the reference's
                        build_kmer_index (k = 5), compute_freq_threshold,
                        _score_query_phase_a and search_kmer_index (Phase A,
                        every survivor aligned with SW, E-value rank, top 5)
"""
from __future__ import annotations

import os
import sys
import time
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))
from oracle.build import REF_ROOT  # noqa: E402

if not (REF_ROOT / "clustkit" / "pairwise.py").exists():
    raise SystemExit(f"clustkit reference checkout not found at {REF_ROOT}; set CLUSTKIT_REFERENCE")


# --------------------------------------------------------------------------- numba stand-in
class _Ty:
    def __init__(self, np_type):
        self.np_type = np_type

    def __call__(self, *args):
        if args and all(isinstance(a, (_Ty, _ArrTy)) for a in args):
            return ("signature",)
        return self.np_type(*args)

    def __getitem__(self, item):
        return _ArrTy()


class _ArrTy:
    pass


def _njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not isinstance(args[0], _Ty) and not kwargs:
        return args[0]
    return lambda f: f


def install_numba_shim():
    mod = types.ModuleType("numba")
    mod.njit = _njit
    mod.jit = _njit
    mod.prange = range
    for name in ("uint64", "uint32", "uint8", "int64", "int32", "int16", "int8",
                 "float32", "float64", "boolean"):
        setattr(mod, name, _Ty(getattr(np, name if name != "boolean" else "bool_")))
    mod.get_num_threads = lambda: 1
    mod.set_num_threads = lambda n: None
    sys.modules["numba"] = mod


def logging_quiet():
    import logging
    logging.getLogger("clustkit").setLevel(logging.WARNING)


def import_reference():
    install_numba_shim()
    sys.path.insert(0, str(REF_ROOT))
    logging_quiet()
    import clustkit.lsh as rlsh
    import clustkit.pairwise as rpw
    import clustkit.sketch as rsk
    return rsk, rpw, rlsh


# --------------------------------------------------------------------------- inputs
def edge_sequences(rng) -> list[np.ndarray]:
    seqs = [
        np.zeros(0, np.uint8),                          # empty
        np.array([3], np.uint8),                        # length 1
        np.array([0, 1, 2, 3], np.uint8),               # shorter than k=5
        np.array([0, 1, 2, 3, 4], np.uint8),            # exactly k
        np.full(60, 9, np.uint8),                       # homopolymer: repeated k-mer
        np.tile(np.array([1, 2, 3], np.uint8), 40),     # low complexity
        np.array([20] * 30, np.uint8),                  # all unknown (X)
        np.concatenate([rng.integers(0, 20, 50), [20, 20], rng.integers(0, 20, 50)]).astype(np.uint8),
        rng.integers(0, 21, 49).astype(np.uint8),       # <= 50 with X
        rng.integers(0, 20, 51).astype(np.uint8),       # just over 50
        rng.integers(0, 20, 200).astype(np.uint8),
    ]
    return seqs


def pack(seqs):
    lengths = np.array([len(s) for s in seqs], np.int32)
    offsets = np.zeros(len(seqs), np.int64)
    if len(seqs) > 1:
        offsets[1:] = np.cumsum(lengths[:-1])
    flat = np.concatenate(seqs).astype(np.uint8) if len(seqs) else np.zeros(0, np.uint8)
    return flat, offsets, lengths


def main():
    sys.path.insert(0, str(REPO))
    from clustkit_gb300 import synth
    from clustkit_gb300.lsh import auto_lsh_params
    import oracle

    rsk, rpw, rlsh = import_reference()
    np.save(HERE / "blosum62_ref.npy", np.asarray(rpw.BLOSUM62, np.int8))
    rng = np.random.default_rng(12345)

    # ---------------------------------------------------------------- sketches
    fam = synth.generate_families(6, 8, median=150, lo=40, hi=400, seed=7)
    seqs = edge_sequences(rng) + [fam.seq(i).copy() for i in range(fam.n)]
    # mutated copies with X runs and a nucleotide-like block
    seqs.append(np.where(rng.random(len(seqs[-1])) < 0.1, 20, seqs[-1]).astype(np.uint8))
    flat, offsets, lengths = pack(seqs)
    cases = [(5, 128, 20), (3, 8, 20), (5, 16, 20), (4, 300, 20)]
    sk_out = {}
    t0 = time.time()
    with np.errstate(over="ignore"):
        for (k, s, alpha) in cases:
            sk_out[f"k{k}_s{s}_a{alpha}"] = rsk._compute_sketches_compact(
                flat, offsets, lengths, k, s, alpha, 42)
        nuc = [rng.integers(0, 4, int(L)).astype(np.uint8) for L in (5, 10, 11, 12, 64, 100, 257)]
        nflat, noff, nlen = pack(nuc)
        sk_nuc = rsk._compute_sketches_compact(nflat, noff, nlen, 11, 16, 4, 42)
    print(f"sketches {time.time()-t0:.1f}s")
    np.savez_compressed(HERE / "sketch_golden.npz", flat=flat, offsets=offsets, lengths=lengths,
                        cases=np.array(cases, np.int32), **sk_out,
                        nuc_flat=nflat, nuc_offsets=noff, nuc_lengths=nlen, nuc_k11_s16=sk_nuc)

    # ---------------------------------------------------------------- jaccard
    sk = sk_out["k5_s128_a20"]
    n = sk.shape[0]
    ii, jj = np.triu_indices(n, 1)
    jp = np.stack([ii, jj], 1).astype(np.int32)
    jp = np.concatenate([jp, np.array([[5, 5], [0, 0], [0, 1], [2, 3]], np.int32)])
    js, _ = rpw._batch_jaccard(jp, sk, np.float32(0.0))
    hand = np.array([[1, 2, 3, 4, 5], [1, 2, 3, 4, 5], [6, 7, 8, 9, 10], [1, 2, 6, 7, 8],
                     [1, 2, 3, 2**64 - 1, 2**64 - 1], [1, 2, 4, 2**64 - 1, 2**64 - 1],
                     [2**64 - 1] * 5, [1, 1, 1, 2, 3], [1, 1, 2, 2, 2]], dtype=np.uint64)
    hi_, hj_ = np.meshgrid(np.arange(len(hand)), np.arange(len(hand)), indexing="ij")
    hp = np.stack([hi_.ravel(), hj_.ravel()], 1).astype(np.int32)
    hs, _ = rpw._batch_jaccard(hp, hand, np.float32(0.0))
    np.savez_compressed(HERE / "jaccard_golden.npz", sketches=sk, pairs=jp, sims=js,
                        hand_sketches=hand, hand_pairs=hp, hand_sims=hs)

    # ---------------------------------------------------------------- SW
    fam2 = synth.generate_families(10, 6, median=180, lo=30, hi=420, seed=11)
    sw_seqs = edge_sequences(rng) + [fam2.seq(i).copy() for i in range(fam2.n)]
    x = fam2.seq(0).copy()
    x[::7] = 20
    sw_seqs.append(x)
    sw_seqs += [rng.integers(0, 20, L).astype(np.uint8) for L in (2, 3, 17, 48, 50, 52, 99, 101, 600)]
    sflat, soff, slen = pack(sw_seqs)
    ns = len(sw_seqs)
    pairs = []
    for a in range(ns):  # every sequence against a few others, both orientations
        for b in rng.choice(ns, size=6, replace=False):
            pairs.append((a, int(b)))
    pairs += [(0, 5), (5, 0), (1, 1), (3, 3), (6, 6), (6, 7), (7, 6)]
    pairs = np.array(pairs, np.int32)
    ref = oracle  # compiled reference lives behind oracle.ref_sw_batch
    bws = np.array([0, 1, 2, 3, 8, 16, 32, 50, 64, 100, 128, 1000], np.int32)
    sw = {}
    for bw in bws:
        r = ref.ref_sw_batch(pairs, sflat, soff, slen, int(bw), rpw.BLOSUM62, threshold=0.0, n_threads=4)
        sw[f"bw{bw}_sims"] = r["sims"]
        sw[f"bw{bw}_scores"] = r["scores"]
        sw[f"bw{bw}_mask"] = r["mask"]
    hints = rng.integers(-250, 250, size=pairs.shape[0]).astype(np.int32)
    hints[::5] = 0
    for bw in (8, 32, 100):
        r = ref.ref_sw_batch(pairs, sflat, soff, slen, bw, rpw.BLOSUM62, diag_hints=hints, n_threads=4)
        sw[f"hint_bw{bw}_sims"] = r["sims"]
        sw[f"hint_bw{bw}_scores"] = r["scores"]
    # Numba twin (run as Python) on short pairs: bit-equal to the C path
    short = np.nonzero(np.maximum(slen[pairs[:, 0]], slen[pairs[:, 1]]) <= 110)[0][:120]
    t0 = time.time()
    nb_sims, nb_scores, nb_mask = rpw._batch_sw_compact_scored(
        pairs[short], sflat, soff, slen, np.float32(0.5), np.int32(16), rpw.BLOSUM62)
    print(f"numba-twin SW {time.time()-t0:.1f}s on {len(short)} pairs")
    np.savez_compressed(HERE / "sw_golden.npz", flat=sflat, offsets=soff, lengths=slen,
                        pairs=pairs, band_widths=bws, hints=hints, **sw,
                        twin_idx=short.astype(np.int64), twin_bw=np.int32(16),
                        twin_sims=nb_sims, twin_scores=nb_scores, twin_mask=nb_mask)

    # ---------------------------------------------------------------- LSH
    t0 = time.time()
    lsh_a = rlsh.lsh_candidates(sk, num_tables=32, num_bands=2, seed=42)
    lsh_b = rlsh.lsh_candidates(sk, num_tables=16, num_bands=1, seed=7)
    print(f"lsh {time.time()-t0:.1f}s")
    np.savez_compressed(HERE / "lsh_golden.npz", sketches=sk, pairs_t32_b2=lsh_a, pairs_t16_b1=lsh_b)

    # ---------------------------------------------------------------- pipeline (config-1 sized)
    c1 = synth.generate_families(200, 10, median=300, lo=50, hi=800, seed=2024)
    t0 = time.time()
    with np.errstate(over="ignore"):
        c1_sk = rsk._compute_sketches_compact(c1.flat, c1.offsets, c1.lengths, 5, 128, 20, 42)
    print(f"config-1 sketches {time.time()-t0:.1f}s")
    lp = auto_lsh_params(0.5, "medium", 5)
    t0 = time.time()
    c1_pairs = rlsh.lsh_candidates(c1_sk, lp["num_tables"], lp["num_bands"], seed=42)
    print(f"config-1 lsh {time.time()-t0:.1f}s -> {len(c1_pairs)} pairs")
    # Point the reference dispatcher at the reference C library compiled from source.
    rpw._c_sw_lib = oracle._load_ref()
    rpw._c_sw_available = True
    results = {}
    for t in (0.5, 0.3):
        t0 = time.time()
        jm = rpw._jaccard_prefilter(c1_pairs, c1_sk, t)
        fp, fs = rpw.compute_pairwise_alignment(
            c1_pairs, None, c1.lengths, t, band_width=100, device="cpu", sketches=c1_sk,
            flat_sequences=c1.flat, offsets=c1.offsets, use_sw=True, use_c_sw=True, n_threads=4)
        print(f"config-1 align t={t} {time.time()-t0:.1f}s -> {len(fp)} kept")
        tag = str(t).replace(".", "p")
        results[f"t{tag}_pairs"] = fp
        results[f"t{tag}_sims"] = fs
        results[f"t{tag}_jmask"] = (np.ones(0, bool) if jm is None else jm)
        results[f"t{tag}_jskipped"] = np.bool_(jm is None)
    np.savez_compressed(HERE / "pipeline_golden.npz", flat=c1.flat, offsets=c1.offsets,
                        lengths=c1.lengths, family=c1.family, sketches=c1_sk,
                        candidates=c1_pairs, num_tables=lp["num_tables"],
                        num_bands=lp["num_bands"], **results)
    make_search_golden(rpw)
    print("done")


def _dataset(flat, offsets, lengths, prefix):
    from clustkit.io import SequenceDataset, SequenceRecord
    from clustkit_gb300.blosum import PROTEIN_ALPHABET
    letters = np.array(list(PROTEIN_ALPHABET + "X"))
    recs = []
    for i in range(len(lengths)):
        o, L = int(offsets[i]), int(lengths[i])
        recs.append(SequenceRecord(id=f"{prefix}{i}", description="",
                                   sequence="".join(letters[flat[o:o + L]])))
    return SequenceDataset(records=recs, mode="protein", lengths=lengths.astype(np.int32),
                           ids=[r.id for r in recs], flat_sequences=flat, offsets=offsets)


def make_search_golden(rpw):
    """clustkit's k-mer search in the configuration the serving path mirrors:
    k = 5 index, Phase A only (min_diag_hits = 1, no similar-k-mer scoring),
    every survivor aligned (cap above the survivor count), SW + E-value rank."""
    import clustkit.kmer_index as rki
    from clustkit.database import DatabaseIndex
    sys.path.insert(0, str(REPO))
    from clustkit_gb300 import synth
    db = synth.generate_families(40, 6, median=90, lo=30, hi=180, seed=404)
    rng = np.random.default_rng(405)
    qs = []
    for i in rng.choice(db.n, 10, replace=False):  # mutated members
        q = db.seq(int(i)).copy()
        m = rng.random(len(q)) < rng.uniform(0.1, 0.5)
        q[m] = rng.integers(0, 20, int(m.sum()))
        qs.append(q.astype(np.uint8))
    bg = synth.random_sequences(8, median=90, lo=30, hi=180, seed=406)
    qs += [bg.seq(i).copy() for i in range(bg.n)]
    qs.append(np.array([1, 2, 20, 3, 4, 5, 6, 7, 8, 9, 20, 20, 1, 2, 3], np.uint8))  # X codes
    qs.append(np.array([5, 6, 7], np.uint8))                                        # shorter than k
    qflat, qoff, qlen = pack(qs)
    k = 5
    t0 = time.time()
    koff, kent, kfreq = rki.build_kmer_index(db.flat, db.offsets, db.lengths, k, "protein")
    thr = int(rki.compute_freq_threshold(kfreq, db.n, 95.0))
    phase = {}
    for qi in range(len(qs)):
        ids, sc = rki._score_query_phase_a(qs[qi], np.int32(len(qs[qi])), np.int32(k), np.int32(20),
                                           koff, kent, kfreq, np.int32(thr), np.int32(db.n), np.int32(2))
        phase[f"q{qi}_ids"] = np.asarray(ids, np.int32)
        phase[f"q{qi}_counts"] = np.asarray(sc, np.int32)
    print(f"search index + phase A {time.time()-t0:.1f}s")
    db_ds = _dataset(db.flat, db.offsets, db.lengths, "d")
    q_ds = _dataset(qflat, qoff, qlen, "q")
    idx = DatabaseIndex(dataset=db_ds, sketches=None, lsh_bucket_ids=None, lsh_band_indices=None,
                        lsh_seeds=None, params={"mode": "protein", "kmer_size": k},
                        kmer_offsets=koff, kmer_entries=kent, kmer_freqs=kfreq)
    t0 = time.time()
    res = rki.search_kmer_index(idx, q_ds, threshold=0.0, top_k=5, band_width=None,
                                min_total_hits=2, min_diag_hits=1, max_cands_per_query=100000,
                                freq_percentile=95.0, kmer_score_thresh=0, local_alignment=True,
                                evalue_normalize=True)
    print(f"search_kmer_index {time.time()-t0:.1f}s, {sum(len(h) for h in res.hits)} hits")
    hq, ht, hid, hsc = [], [], [], []
    for qi, hl in enumerate(res.hits):
        for h in hl:
            hq.append(qi)
            ht.append(int(h.target_id[1:]))
            hid.append(h.identity)
            hsc.append(h.score)
    # BLOSUM62-neighbour scoring (clustkit's default search mode, kmer_score_thresh = 13)
    # on a subset of the queries: the pure-Python run of the neighbour loops is slow
    sim_q = [0, 1, 2, 3, 10, 11, 18, 19]
    sim = {"sim_queries": np.array(sim_q, np.int32)}
    t0 = time.time()
    for qi in sim_q:
        ids, sc = rki._score_query_similar_k5(qs[qi], np.int32(len(qs[qi])), koff, kent, kfreq, np.int32(thr),
                                              np.int32(db.n), np.int32(2), rpw.BLOSUM62, np.int32(13))
        sim[f"q{qi}_sim_ids"] = np.asarray(ids, np.int32)
        sim[f"q{qi}_sim_scores"] = np.asarray(sc, np.int32)
    print(f"similar-k-mer phase A {time.time()-t0:.1f}s")
    sq_flat, sq_off, sq_len = pack([qs[i] for i in sim_q])
    t0 = time.time()
    res2 = rki.search_kmer_index(idx, _dataset(sq_flat, sq_off, sq_len, "q"), threshold=0.0, top_k=5,
                                 band_width=None, min_total_hits=2, min_diag_hits=1, max_cands_per_query=100000,
                                 freq_percentile=95.0, kmer_score_thresh=13, local_alignment=True,
                                 evalue_normalize=True)
    print(f"search_kmer_index (similar k-mers) {time.time()-t0:.1f}s, {sum(len(h) for h in res2.hits)} hits")
    sq, st_, sid, ssc = [], [], [], []
    for qi, hl in enumerate(res2.hits):
        for h in hl:
            sq.append(sim_q[qi])
            st_.append(int(h.target_id[1:]))
            sid.append(h.identity)
            ssc.append(h.score)
    sim.update(sim_hit_query=np.array(sq, np.int32), sim_hit_target=np.array(st_, np.int32),
               sim_hit_identity=np.array(sid, np.float64), sim_hit_score=np.array(ssc, np.float64),
               sim_band_width=np.int32(max(20, int(int(np.percentile(np.concatenate([sq_len, db.lengths]), 95))
                                                   * 0.3))))
    nz = np.nonzero(kfreq)[0]
    all_len = np.concatenate([qlen, db.lengths])
    np.savez_compressed(HERE / "search_golden.npz", db_flat=db.flat, db_offsets=db.offsets,
                        db_lengths=db.lengths, q_flat=qflat, q_offsets=qoff, q_lengths=qlen,
                        k=np.int32(k), kmer_entries=kent, freq_nonzero_idx=nz.astype(np.int64),
                        freq_nonzero_val=kfreq[nz], offsets_total=np.int64(koff[-1]), freq_thresh=np.int32(thr),
                        band_width=np.int32(max(20, int(int(np.percentile(all_len, 95)) * 0.3))),
                        hit_query=np.array(hq, np.int32), hit_target=np.array(ht, np.int32),
                        hit_identity=np.array(hid, np.float64), hit_score=np.array(hsc, np.float64),
                        top_k=np.int32(5), **phase, **sim)


def make_kmer_scorer_golden(rpw):
    """clustkit's C k-mer scorer (csrc/kmer_score.c, batch_score_queries_c --
    Phase A, top-K, Phase B diagonal scoring, diagonal hints) compiled from the
    checkout into oracle/_ref/, on a family database large enough for every cap
    to bind; plus the Numba two-stage scorer (kmer_index.py:654-829) where no
    cap binds."""
    import ctypes
    import clustkit.kmer_index as rki
    sys.path.insert(0, str(REPO))
    import oracle.build as obuild
    from clustkit_gb300 import synth
    lib = ctypes.CDLL(str(obuild.build_reference_kmer_scorer()))
    db = synth.generate_families(600, 8, median=150, lo=30, hi=400, seed=707)
    rng = np.random.default_rng(708)
    qs = []
    for i in rng.choice(db.n, 8, replace=False):
        q = db.seq(int(i)).copy()
        m = rng.random(len(q)) < rng.uniform(0.05, 0.4)
        q[m] = rng.integers(0, 20, int(m.sum()))
        qs.append(q.astype(np.uint8))
    bg = synth.random_sequences(4, median=200, lo=60, hi=400, seed=709)
    qs += [bg.seq(i).copy() for i in range(bg.n)]
    qs.append(np.concatenate([db.seq(3)[:60], np.full(3, 20, np.uint8), db.seq(3)[60:]]).astype(np.uint8))
    qs.append(np.array([5, 6, 7], np.uint8))
    qflat, qoff, qlen = pack(qs)
    k = 5
    koff, kent, kfreq = rki.build_kmer_index(db.flat, db.offsets, db.lengths, k, "protein")
    thr = int(rki.compute_freq_threshold(kfreq, db.n, 95.0))
    # (min_total_hits, min_diag_hits, diag_bin_width, max_cands, phase_a_topk)
    configs = [(2, 1, 10, 100000, 10000), (2, 1, 10, 17, 10000), (2, 2, 10, 100000, 10000),
               (2, 2, 10, 11, 40), (1, 3, 7, 25, 200), (3, 2, 16, 6, 9)]
    P, I32 = ctypes.c_void_p, ctypes.c_int32
    lib.batch_score_queries_c.restype = None
    lib.batch_score_queries_c.argtypes = [P, P, P, I32, I32, I32, P, P, P, P, I32, I32, I32, I32, I32, I32, I32,
                                          P, P, P, P]
    out = {}
    nq = len(qs)
    qoff64 = qoff.astype(np.int64)
    qlen32 = qlen.astype(np.int32)
    for ci, (mth, mdh, dbw, mc, topk) in enumerate(configs):
        tg = np.full((nq, mc), -1, np.int32)
        cnt = np.zeros(nq, np.int32)
        sc = np.zeros((nq, mc), np.int32)
        dg = np.zeros((nq, mc), np.int32)
        lib.batch_score_queries_c(qflat.ctypes.data, qoff64.ctypes.data, qlen32.ctypes.data, nq, k, 20,
                                  koff.ctypes.data, kent.ctypes.data, None, kfreq.ctypes.data, thr, db.n, mth, mdh,
                                  dbw, mc, topk, tg.ctypes.data, cnt.ctypes.data, sc.ctypes.data, dg.ctypes.data)
        for qi in range(nq):
            n = int(cnt[qi])
            out[f"c{ci}_q{qi}_targets"] = tg[qi, :n].copy()
            out[f"c{ci}_q{qi}_scores"] = sc[qi, :n].copy()
            out[f"c{ci}_q{qi}_diags"] = dg[qi, :n].copy()
    for qi in range(nq):  # Numba two-stage, config 2 (no cap binds)
        ids, sc = rki._score_query_two_stage(qs[qi], np.int32(len(qs[qi])), np.int32(k), np.int32(20), koff, kent,
                                             kfreq, np.int32(thr), np.int32(db.n), np.int32(2), np.int32(2),
                                             np.int32(10), np.int32(10000))
        out[f"numba_q{qi}_ids"] = np.asarray(ids, np.int32)
        out[f"numba_q{qi}_scores"] = np.asarray(sc, np.int32)
    np.savez_compressed(HERE / "kmer_scorer_golden.npz", db_flat=db.flat, db_offsets=db.offsets,
                        db_lengths=db.lengths, q_flat=qflat, q_offsets=qoff, q_lengths=qlen,
                        configs=np.array(configs, np.int32), freq_thresh=np.int32(thr), **out)
    print("kmer scorer golden:", {f"c{ci}": int(sum(len(out[f'c{ci}_q{q}_targets']) for q in range(nq)))
                                  for ci in range(len(configs))})


if __name__ == "__main__":
    main()
