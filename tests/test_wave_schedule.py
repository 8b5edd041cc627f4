"""CPU model of the warp-per-pair SW kernel's schedule, checked against the oracle.

The kernel (clustkit_gb300/csrc/sw_batched.cu, sw_wave_kernel) cuts a pair's
rows into strips of R; lane l computes strips l, l + 32, ..., strip s working
on column j = T - s + 1 + h - w at step T and receiving the row above from
lane l - 1 by shuffle.  This model runs the same steps for 32 emulated lanes
in plain Python -- strip ownership, the hand-over, the out-of-band overrides
and the first-maximum merge -- and compares score and match count with the
oracle (clustkit/csrc/sw_align.c:25-177 restated), asserting every residue
index it touches.  It pins the schedule logic without a GPU; the kernel
itself is checked against the oracle by the GPU tests.
"""
import numpy as np
import pytest

import oracle
from clustkit_gb300.blosum import BLOSUM62

TBIT = 1 << 13; PU = 1 << 14; KU = 1 << 16
CLEAN = ~(TBIT | 3 * PU); ZKEY = 3 * PU
OPEN_E = -11 * KU + PU; OPEN_F = -11 * KU; EXT = -1 * KU
NEG_E = -16 * KU + PU + TBIT; NEG_F = -16 * KU + TBIT
MATCH = (1 << 13) - 1; INT_MAX = 2**31 - 1

def inc(a, b):
    s = int(BLOSUM62[a, b]) if a < 20 and b < 20 else -4
    return s * KU + 2 * PU + (1 if a == b else 0)

def wave_rows(la, w):
    if la <= 128 or 2 * w < 31 * 4 + 32: return 4
    if la <= 256 or 2 * w < 31 * 8 + 32: return 8
    if la <= 512 or 2 * w < 31 * 16 + 32: return 16
    return 0

def geometry(li, lj, bw, hint):
    shorter = min(li, lj)
    if hint > shorter or hint < -shorter: hint = 0
    swap = not (li <= lj)
    la, lb = (li, lj) if not swap else (lj, li)
    h = hint if not swap else -hint
    w = lb if (bw <= 0 or lb <= 50) else bw
    return swap, la, lb, w, h

def align_wave(A, B, la, lb, w, h):
    R = wave_rows(la, w); assert R
    D = R + 1; w2 = 2 * w; c0 = 1 + h - w
    n_strips = (la + R - 1) // R
    lim = lb - 1 - h + w
    s_lim = 0 if lim < 0 else lim // R + 1
    n_strips = min(n_strips, s_lim)
    lbest = [0] * 32; lrow = [INT_MAX] * 32
    if n_strips > 0:
        J0_0 = max(c0, 1); T_first = J0_0 - c0
        sl = n_strips - 1
        J1_l = min(sl * R + R + h + w, lb); T_last = J1_l + sl - c0
        rotate = n_strips > 32
        st = []
        for lane in range(32):
            s = lane
            if rotate and T_first >= lane * D:
                s = lane + 32 * ((T_first - lane * D) // (32 * D))
            L = dict(s=s, nsw=(s + 32) * D if rotate else INT_MAX)
            st.append(L)
        def setup(L):
            s = L['s']; i0 = s * R + 1; L['i0'] = i0; L['lo0'] = i0 + h - w
            L['J0'] = max(L['lo0'], 1); L['J1'] = min(i0 + R - 1 + h + w, lb)
            if s >= n_strips: L['J0'], L['J1'] = 1, 0
            alive = max(0, min(la - i0 + 1, R)); L['alive'] = alive
            L['hc'] = [0] * R; L['fT'] = [NEG_F] * R; L['best'] = [0] * R
            codes = []
            for r in range(R):
                if r < alive and s < n_strips:
                    idx = i0 + r - 1; assert 0 <= idx < la
                    codes.append(int(A[idx]))
                else: codes.append(0)
            L['code'] = codes
        def merge(L, lane):
            for r in range(R):
                b = L['best'][r]
                if r < L['alive'] and b > (lbest[lane] | (KU - 1)):
                    lbest[lane] = b; lrow[lane] = L['i0'] + r
        for L in st: setup(L)
        hout = [0] * 32; eout = [NEG_E] * 32; hprev = [0] * 32; gs = 1
        for T in range(T_first, T_last + 1):
            for lane, L in enumerate(st):
                if T == L['nsw']:
                    merge(L, lane); L['s'] += 32; L['nsw'] += 32 * D; setup(L)
            hin_all = [hout[(l + 31) & 31] for l in range(32)]
            ein_all = [eout[(l + 31) & 31] for l in range(32)]
            cms = [0] * 32
            for lane, L in enumerate(st):
                s = L['s']; j = T - s + c0
                hin, ein = hin_all[lane], ein_all[lane]
                top = s * R + h + w
                hdiag = 0 if (s == 0 or j - 1 > top) else hprev[lane]
                hprev[lane] = hin
                if s == 0 or j > top: hin, ein = 0, NEG_E
                if L['J0'] <= j <= L['J1']:
                    assert 1 <= j <= lb
                    bc = int(B[j - 1])
                    hu, eu = hin, ein
                    hc, fT = L['hc'], L['fT']
                    for r in range(R):
                        if r < L['alive'] and 0 <= j - r - L['lo0'] <= w2:
                            diagc = max(hdiag + inc(L['code'][r], bc), ZKEY)
                            eT = max(eu + EXT, hu + OPEN_E) | TBIT
                            fTn = max(fT[r] + EXT, hc[r] + OPEN_F) | TBIT
                            hn = max(diagc, eT, fTn) & CLEAN
                            hdiag = hc[r]; hc[r] = hn; fT[r] = fTn; hu = hn; eu = eT
                        else:
                            hdiag = hc[r]; hc[r] = 0; hu = 0; eu = NEG_E
                    hout[lane], eout[lane] = hu, eu
                    cms[lane] = max(hc)
                else:
                    hout[lane], eout[lane] = 0, NEG_E
            if any((cm >> 16) >= gs for cm in cms):
                for lane, L in enumerate(st):
                    for r in range(R):
                        b = L['best'][r]
                        if L['hc'][r] > (b | (KU - 1)): L['best'][r] = L['hc'][r]
                m = max(cm >> 16 for cm in cms)
                gs = max(gs, m)
        for lane, L in enumerate(st): merge(L, lane)
    best = max(b >> 16 for b in lbest)
    if best <= 0: return 0, 0
    row = min(lrow[l] for l in range(32) if (lbest[l] >> 16) == best)
    wl = [l for l in range(32) if (lbest[l] >> 16) == best and lrow[l] == row]
    assert len(wl) == 1
    return best, lbest[wl[0]] & MATCH

def run_case(rng, li, lj, bw, hint=0, related=False):
    """(model score, model matches, oracle score, oracle matches) for one pair."""
    a = rng.integers(0, 20, li).astype(np.uint8)
    if related:
        b = a.copy()[:lj] if lj <= li else np.concatenate([a, rng.integers(0, 20, lj - li)]).astype(np.uint8)
        mut = rng.random(lj) < 0.3
        b[mut] = rng.integers(0, 20, mut.sum())
    else:
        b = rng.integers(0, 20, lj).astype(np.uint8)
    if rng.random() < 0.1 and li > 3: a[rng.integers(li)] = 20
    swap, la, lb, w, h = geometry(li, lj, bw, hint)
    if not wave_rows(la, w): return None
    A, Bs = (a, b) if not swap else (b, a)
    sc, m = align_wave(A, Bs, la, lb, w, h)
    flat = np.concatenate([a, b]); offs = np.array([0, li], np.int64); lens = np.array([li, lj], np.int32)
    hints = np.array([hint], np.int32)
    r = oracle.sw_batch(np.array([[0, 1]], np.int32), flat, offs, lens, bw, BLOSUM62, diag_hints=hints)
    return sc, m, int(r['scores'][0]), int(r['matches'][0])



CASES = [(30, 40, 100, 0), (5, 5, 100, 0), (1, 7, 100, 0), (200, 260, 100, 0), (600, 650, 100, 0),
         (400, 420, 238, 0), (90, 95, 0, 0), (130, 500, 100, 7), (300, 310, 100, -40),
         (600, 620, 100, 600), (50, 52, 0, 0), (191, 355, 1, 0), (182, 600, 1, 0), (160, 170, 2, 0),
         (300, 330, 3, 5), (800, 810, 16, 3), (520, 530, 260, 0), (129, 131, 77, -5), (2, 3000, 100, 0)]


@pytest.mark.parametrize("li,lj,bw,hint", CASES)
def test_wave_schedule_matches_oracle(li, lj, bw, hint):
    rng = np.random.default_rng(li * 7 + lj + bw)
    for related in (False, True):
        res = run_case(rng, li, lj, bw, hint, related)
        assert res is not None
        assert res[0] == res[2] and res[1] == res[3], res
