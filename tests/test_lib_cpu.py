"""CPU-only checks of the native library and the host logic (no GPU needed).

* libckgpu.so builds for sm_103a, loads, and exports every function that
  include/clustkit_gb300.h declares, with the ctypes signatures bound.
* Without a GPU the product path refuses to run (no CPU fallback).
* Host-side logic: closed-form band cell counts, the LSH restatement against
  the reference's own pairs, the synthetic generator, the adapter's ordering
  and pre-filter rules.
"""
import re
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]


def header_functions():
    text = (REPO / "include" / "clustkit_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*\b([a-z_][a-z_0-9]*)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_expected_surface():
    names = header_functions()
    for n in ("batch_sw_align_c", "sw_set_num_threads", "ck_sw_batch", "ck_sw_batch_device",
              "ck_sketch", "ck_sketch_device", "ck_jaccard", "ck_jaccard_device", "ck_last_error",
              "ck_probe_int_rate"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from clustkit_gb300 import _lib
    lib = _lib.load()
    for name in header_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"
    assert lib.ck_version() >= 100


def test_header_constants_match_bindings():
    """Every CK_OK / CK_ERR_* status and CK_CFG_* key the header defines has
    the same value in the Python bindings."""
    from clustkit_gb300 import _lib
    text = (REPO / "include" / "clustkit_gb300.h").read_text()
    defs = dict((n, int(v)) for n, v in re.findall(r"^#define\s+(CK_(?:OK|ERR_[A-Z_]+|CFG_[A-Z_]+))\s+(\d+)",
                                                  text, flags=re.M))
    assert "CK_ERR_CAPACITY" in defs and "CK_CFG_WAVE_ROWS" in defs
    for name, value in defs.items():
        py = name if not name.startswith("CK_CFG_") else "CFG_" + name[len("CK_CFG_"):]
        assert getattr(_lib, py) == value, name


def test_search_scoring_modes():
    """Scoring's modes as search_kmer_index's keywords select them, and every
    mode can be captured in CUDA graphs (under a caller bound where one is
    needed)."""
    from clustkit_gb300.search import Scoring
    exact = Scoring(2, 0)
    similar = Scoring(2, 13)
    phase_b = Scoring(2, 0, min_diag_hits=2)
    c_path = Scoring(2, 0, min_diag_hits=2, use_c_scoring=True, use_c_sw=True)
    assert not exact.similar and not exact.diagonal and not exact.hints
    assert similar.similar and not similar.diagonal and not similar.hints
    assert phase_b.diagonal and not phase_b.hints
    assert c_path.diagonal and c_path.hints
    # similar k-mers take precedence over the C scorer's settings
    assert not Scoring(2, 13, use_c_scoring=True, use_c_sw=True).hints
    assert all(s.graphable for s in (exact, similar, phase_b, c_path))
    assert exact == Scoring(2, 0) and exact != similar


def test_library_is_built_for_sm103a():
    from clustkit_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)
    assert build.LIB.exists()


def test_no_cpu_fallback_without_gpu():
    from clustkit_gb300 import _lib
    from clustkit_gb300.pairwise import batch_sw
    if _lib.load().ck_device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(_lib.CkError):
        batch_sw(np.array([[0, 1]], np.int32), np.zeros(4, np.uint8), np.array([0, 2]),
                 np.array([2, 2], np.int32))


def test_config_keys_validate_and_round_trip():
    """The batched engine's settings (host-only setters, no GPU needed): each
    key takes its documented values and reads them back, rejects others
    without changing the setting, and the retired CTAs-per-SM key 8 is gone."""
    from clustkit_gb300 import _lib
    cases = {
        _lib.CFG_ROWS_PER_STRIP: ([0, 8, 16, 24, 32], [4, 12, -1]),
        _lib.CFG_STRIP_VARIANT: ([-1, 0, 1, 2, 3], [4, -2]),
        _lib.CFG_STRIP_THREADS: ([0, 512, 640, 768], [256, 576, 1024, -1]),
        _lib.CFG_STRIP_KEY: ([0, 1], [2, -1]),
        _lib.CFG_WAVE_ROWS: ([0, 4, 8, 16], [2, 32]),
    }
    for key, (good, bad) in cases.items():
        keep = _lib.get_config(key)
        try:
            for v in good:
                _lib.set_config(key, v)
                assert _lib.get_config(key) == v
            for v in bad:
                with pytest.raises(_lib.CkError):
                    _lib.set_config(key, v)
                assert _lib.get_config(key) == good[-1]
        finally:
            _lib.set_config(key, keep)
    with pytest.raises(_lib.CkError):
        _lib.set_config(8, 2)
    with pytest.raises(_lib.CkError):
        _lib.get_config(8)


def test_band_cells_closed_form():
    from clustkit_gb300.cells import band_cells, band_cells_loop
    rng = np.random.default_rng(0)
    for _ in range(400):
        la = int(rng.integers(0, 300))
        lb = la + int(rng.integers(0, 300))
        w = int(rng.integers(1, 400))
        h = int(rng.integers(-la, la + 1)) if la > 0 and rng.random() < 0.5 else 0
        assert band_cells(np.array([la]), np.array([lb]), np.array([w]), np.array([h]))[0] == \
            band_cells_loop(la, lb, w, h)


def test_lsh_restatement_matches_reference(golden):
    from clustkit_gb300.lsh import lsh_candidates
    g = golden("lsh_golden.npz")
    assert np.array_equal(lsh_candidates(g["sketches"], 32, 2, 42), g["pairs_t32_b2"])
    assert np.array_equal(lsh_candidates(g["sketches"], 16, 1, 7), g["pairs_t16_b1"])
    p = golden("pipeline_golden.npz")
    c = lsh_candidates(p["sketches"], int(p["num_tables"]), int(p["num_bands"]), 42)
    assert np.array_equal(c, p["candidates"])


def test_lsh_reference_properties():
    from clustkit_gb300.lsh import lsh_candidates
    sk = np.array([[1, 2, 3, 4, 5, 6, 7, 8], [1, 2, 3, 4, 5, 6, 7, 8]], np.uint64)
    assert (0, 1) in [tuple(x) for x in lsh_candidates(sk, 8, 2)]
    sk = np.tile(np.arange(16, dtype=np.uint64), (5, 1))
    p = lsh_candidates(sk, 4, 2)
    assert np.all(p[:, 0] < p[:, 1]) and len(set(map(tuple, p))) == len(p)
    assert len(lsh_candidates(np.empty((0, 16), np.uint64), 4, 2)) == 0


def test_auto_lsh_params():
    from clustkit_gb300.lsh import auto_lsh_params
    assert auto_lsh_params(0.5, "medium", 5) == {"num_tables": 146, "num_bands": 1}
    assert auto_lsh_params(0.3, "high", 5) == {"num_tables": 512, "num_bands": 1}


def test_synthetic_generator_shape_and_determinism():
    from clustkit_gb300 import synth
    a = synth.generate_families(20, 10, median=300, lo=50, hi=800, seed=3)
    b = synth.generate_families(20, 10, median=300, lo=50, hi=800, seed=3)
    assert a.n == 200 and np.array_equal(a.flat, b.flat)
    assert a.lengths.min() >= 50 and a.lengths.max() <= 800
    assert a.flat.max() < 20
    assert a.offsets[-1] + a.lengths[-1] == len(a.flat)
    p, lam = synth.implied_background()
    assert abs(p.sum() - 1) < 1e-9 and 0.25 < lam < 0.4
    pairs = synth.mixed_pairs(a, 500, seed=1, min_ratio=0.5)
    r = np.minimum(a.lengths[pairs[:, 0]], a.lengths[pairs[:, 1]]) / \
        np.maximum(a.lengths[pairs[:, 0]], a.lengths[pairs[:, 1]])
    assert len(pairs) == 500 and r.min() >= 0.5


def test_adapter_host_logic_with_oracle_stub(golden, monkeypatch):
    """Ordering, pre-filter and pass rules of compute_pairwise_alignment, with
    the GPU calls replaced by the oracle (this tests the host logic only)."""
    import oracle
    from clustkit_gb300 import pairwise as pw

    def fake_batch_sw(pairs, flat, offsets, lengths, band_width=100, sub_matrix=None,
                      threshold=0.0, diag_hints=None, pass_rule=0, engine=0):
        r = oracle.sw_batch(pairs, flat, offsets, lengths, band_width, pw.BLOSUM62)
        t = np.float32(threshold)
        if pass_rule == pw.PASS_CPU:
            r["mask"] = r["sims"] >= t
        elif pass_rule == pw.PASS_NUMBA:
            r["mask"] = (r["scores"] > 0) & (r["sims"] >= t)
        return r

    monkeypatch.setattr(pw, "batch_sw", fake_batch_sw)
    monkeypatch.setattr(pw, "batch_jaccard", lambda pairs, sk, floor=0.0: (oracle.jaccard(pairs, sk), None))
    g = golden("pipeline_golden.npz")
    for t, tag in ((0.5, "0p5"), (0.3, "0p3")):
        fp, fs = pw.compute_pairwise_alignment(
            g["candidates"], None, g["lengths"], t, band_width=100, sketches=g["sketches"],
            flat_sequences=g["flat"], offsets=g["offsets"], use_sw=True, use_c_sw=True)
        assert np.array_equal(fp, g[f"t{tag}_pairs"])
        assert np.array_equal(fs, g[f"t{tag}_sims"])
    with pytest.raises(NotImplementedError):
        pw.compute_pairwise_alignment(g["candidates"], None, g["lengths"], 0.5,
                                      flat_sequences=g["flat"], offsets=g["offsets"], use_sw=False)


def test_search_entry_points_reject_bad_arguments():
    """The search entry points validate their arguments before touching the
    device: NULL outputs, a missing index or bad sizes give
    CK_ERR_INVALID_ARGUMENT (no GPU needed to see it)."""
    from clustkit_gb300 import _lib
    lib = _lib.load()
    INVALID = 1
    z = np.zeros(16, np.int64)
    p = z.ctypes.data
    # compact targets: negative count, NULL buffers
    assert lib.ck_kmer_targets_device(0, p, -1, p, None) == INVALID
    assert lib.ck_kmer_targets_device(0, None, 10, p, None) == INVALID
    # Phase A with neither entries nor compact targets
    assert lib.ck_search_phase_a_device(0, p, 4, p, p, 1, 4, 5, 20, p, None, None, p, 10, 1, 2, 5,
                                        p, p, p, None) == INVALID
    # C-scorer twin: Phase B needs the full entries and the database lengths
    assert lib.ck_search_kmer_candidates_device(0, p, 4, p, p, 1, 4, 5, 20, p, None, p, p, 10, 1, None, 2, 2, 10,
                                                5, 100, p, p, p, p, -1, None) == INVALID
    assert lib.ck_search_kmer_candidates_device(0, p, 4, p, p, 1, 4, 5, 20, p, p, None, p, 10, 1, None, 2, 2, 10,
                                                5, 100, p, p, p, p, -1, None) == INVALID
    # no output buffers / zero cap
    assert lib.ck_search_kmer_candidates_device(0, p, 4, p, p, 1, 4, 5, 20, p, p, None, p, 10, 1, p, 2, 1, 10,
                                                0, 100, p, p, p, p, -1, None) == INVALID
    assert lib.ck_search_phase_a_similar_device(0, p, 4, p, p, 1, 4, None, 13, p, p, None, p, 10, 1, 2, 5,
                                                p, p, p, -1, None) == INVALID
