"""CPU model of the strip kernel's packed DP keys, both forms, against the oracle.

The strip kernel (clustkit_gb300/csrc/sw_batched.cu) computes every cell of
clustkit's banded Smith-Waterman (clustkit/csrc/sw_align.c:25-177) as signed
int32 max operations over packed keys

    key = score * 2^16 + priority * 2^14 + (tie mark) + matches

so that one max picks the candidate clustkit's comparisons pick (score first,
then H's zero > diagonal > E > F order, then gap extension over gap opening on
ties) and carries the winner's match count.  Two forms of the tie mark:

* wide: 13-bit match count and a tie bit (2^13) set on every stored E and F;
* compact (pairs of <= 2047 rows): 11-bit match count and a 3-bit counter at
  bits 11..13 that every gap extension increments; E's counter is cleared at
  strip rows 5, 11, 17, ... and each strip's last row (strips of R rows), F's
  every (at most) 4 columns.

This restates that arithmetic in numpy, row by row over many pairs of one
shape at once, and checks score and first-maximum match count against the
oracle on pairs built to tie (two-letter sequences) and to open long gaps
(runs of up to 40 inserted residues), with the counters' bound asserted.  A
control with the tie mark left out must disagree with the oracle, so the
pairs do exercise the tie rule.
"""
import numpy as np
import pytest

import oracle
from clustkit_gb300.blosum import BLOSUM62

KU, PU, TBIT = 1 << 16, 1 << 14, 1 << 13
ZKEY = 3 * PU
OPEN_E = -11 * KU + PU
OPEN_F = -11 * KU
EXT = -1 * KU
CTR = 7 << 11

FORMS = {
    "wide": dict(ext=EXT, neg_e=-16 * KU + PU + TBIT, neg_f=-16 * KU + TBIT, clean=~(TBIT | 3 * PU),
                 mmask=(1 << 13) - 1, tie_bit=True, counter=False),
    "compact": dict(ext=EXT + (1 << 11), neg_e=-16 * KU + PU, neg_f=-16 * KU, clean=~(CTR | 3 * PU),
                    mmask=(1 << 11) - 1, tie_bit=False, counter=True),
    # planted mistake: neither a tie bit nor a counter (ties then go to the
    # larger match count instead of to the extension)
    "no_tie_mark": dict(ext=EXT, neg_e=-16 * KU + PU, neg_f=-16 * KU, clean=~(3 * PU),
                        mmask=(1 << 13) - 1, tie_bit=False, counter=False),
}


def _inc_table():
    t = np.zeros((20, 20), np.int64)
    for a in range(20):
        for b in range(20):
            t[a, b] = int(BLOSUM62[a, b]) * KU + 2 * PU + (1 if a == b else 0)
    return t


def model_keys(A, B, w, hint, form, R=16):
    """Best score and first-max match count of each pair (rows A[p] against
    columns B[p], all of one shape), by the kernel's key arithmetic with
    strips of R rows (the E counter clears)."""
    f_ = FORMS[form]
    P, la = A.shape
    lb = B.shape[1]
    inc_t = _inc_table()
    H = np.zeros((P, lb + 2), np.int64)
    E = np.full((P, lb + 2), f_["neg_e"], np.int64)
    best = np.zeros(P, np.int64)
    max_ctr = 0
    for i in range(1, la + 1):
        lo, hi = i + hint - w, i + hint + w
        js, je = max(1, lo), min(lb, hi)
        if hi < 1:
            continue
        if js > lb:
            break
        hd = H[:, js - 1].copy()
        hl = np.zeros(P, np.int64)
        f = np.full(P, f_["neg_f"], np.int64)
        for j in range(js, je + 1):
            inc = inc_t[A[:, i - 1], B[:, j - 1]]
            diag = np.maximum(hd + inc, ZKEY)
            hu, eu = H[:, j].copy(), E[:, j]
            e = np.maximum(hu + OPEN_E, eu + f_["ext"])
            f = np.maximum(f + f_["ext"], hl + OPEN_F)
            if f_["tie_bit"]:
                f |= TBIT
            h = np.maximum(np.maximum(diag, e), f) & f_["clean"]
            if f_["counter"]:
                max_ctr = max(max_ctr, int(((e >> 11) & 7).max()), int(((f >> 11) & 7).max()))
                r = (i - 1) % R  # the strip row
                e_st = e & ~CTR if (r % 6 == 5 or r == R - 1) else e
            else:
                e_st = e | TBIT if f_["tie_bit"] else e
            upd = (h >> 16) > (best >> 16)  # strict '>' in row-major order: the first maximum
            best = np.where(upd, h, best)
            H[:, j], E[:, j] = h, e_st
            hd, hl = hu, h
            if f_["counter"] and j % 4 == 3:
                f &= ~CTR
        if je + 1 <= lb:
            H[:, je + 1] = 0
            E[:, je + 1] = f_["neg_e"]
    return best >> 16, best & f_["mmask"], max_ctr


def _pairs(rng, P, la, lb):
    """Half two-letter sequences, half a random sequence against a copy with
    runs of 5..40 residues inserted and deleted (cut or padded to lb)."""
    A = np.empty((P, la), np.int64)
    B = np.empty((P, lb), np.int64)
    for p in range(P):
        if p % 2 == 0:
            A[p] = rng.choice([0, 7], la)
            B[p] = rng.choice([0, 7], lb)
        else:
            a = rng.integers(0, 20, la)
            b = list(a)
            for _ in range(3):
                at = int(rng.integers(0, max(1, len(b))))
                if rng.random() < 0.5:
                    b[at:at] = list(rng.integers(0, 20, int(rng.integers(5, 41))))
                else:
                    del b[at:at + int(rng.integers(5, 41))]
            b = (b + list(rng.integers(0, 20, lb)))[:lb]
            A[p], B[p] = a, b
    return A, B


def _oracle(A, B, bw, hint):
    P, la = A.shape
    lb = B.shape[1]
    flat = np.concatenate([np.concatenate([A[p], B[p]]) for p in range(P)]).astype(np.uint8)
    lengths = np.tile(np.array([la, lb], np.int32), P)
    offsets = np.zeros(2 * P, np.int64)
    offsets[1:] = np.cumsum(lengths[:-1])
    pairs = np.stack([np.arange(0, 2 * P, 2), np.arange(1, 2 * P, 2)], 1).astype(np.int32)
    hints = np.full(P, hint, np.int32) if hint else None
    r = oracle.sw_batch(pairs, flat, offsets, lengths, bw, BLOSUM62, diag_hints=hints)
    return r["scores"], r["matches"]


SHAPES = [(150, 170, 8, 0), (120, 120, 0, 0), (90, 200, 25, 0), (60, 61, 3, 0), (100, 160, 10, 30),
          (80, 140, 40, -20)]


@pytest.mark.parametrize("la,lb,bw,hint", SHAPES)
def test_key_forms_match_oracle(la, lb, bw, hint):
    rng = np.random.default_rng(la * 7 + lb + bw)
    A, B = _pairs(rng, 192, la, lb)
    ref_s, ref_m = _oracle(A, B, bw, hint)
    longer = max(la, lb)
    w = longer if (bw <= 0 or longer <= 50) else bw
    for form, R in (("wide", 16), ("compact", 8), ("compact", 16), ("compact", 24), ("compact", 32)):
        s, m, max_ctr = model_keys(A, B, w, hint, form, R)
        assert np.array_equal(s, ref_s), (form, R)
        assert np.array_equal(m, ref_m), (form, R)
        if form == "compact":
            assert 1 <= max_ctr <= 6  # extensions happened; never a carry into the priority bits


@pytest.mark.parametrize("R", [8, 16, 24, 32])
def test_e_counter_clears_bound_the_count(R):
    """At most 6 extensions between two E clears, counted across strip
    boundaries (the window carries the last row's E into the next strip)."""
    clears = [r for r in range(R) if r % 6 == 5 or r == R - 1]
    gaps = [b - a for a, b in zip(clears, clears[1:])] + [clears[0] + R - clears[-1]]
    assert max(gaps) <= 6 and clears[-1] == R - 1


def test_tie_mark_matters():
    """Leaving the tie mark out changes some first-max match counts."""
    rng = np.random.default_rng(5)
    A, B = _pairs(rng, 192, 150, 170)
    ref_s, ref_m = _oracle(A, B, 8, 0)
    s, m, _ = model_keys(A, B, 8, 0, "no_tie_mark")
    assert np.array_equal(s, ref_s)  # scores never depend on the tie rule
    assert not np.array_equal(m, ref_m)
