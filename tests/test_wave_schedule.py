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


# ----------------------------------------------------------------------------
# The streamed schedule (sw_batched.cu, wave_stream): strips of consecutive
# pairs flow through one warp's lanes; strip s of a pair starting at T0 runs
# column j at step T0 + s + j - J0(strip 0); a pair is issued (one per step,
# after every strip of the previous one has started) at the smallest T0 that
# finds each of its first 32 strips' lanes free; per-pair slots hold the
# running best score and the packed best cell.
NSLOT = 16

def r_call(bw):
    wmax = max(bw, 50) if bw > 0 else 10**9
    if 2 * wmax < 31 * 4 + 32: return 4
    if 2 * wmax < 31 * 8 + 32: return 8
    return 16

def stream(pairs_geo, R):
    """pairs_geo: list of (A, B, la, lb, w, h).  Returns list of (score, matches)."""
    res = [None] * len(pairs_geo)
    slots = [None] * NSLOT
    lanes = [dict(cur=None, pend=None, F=-1, hout=0, eout=NEG_E, hprev=0) for _ in range(32)]
    T = 0; q = 0; g_next = 0; seq = 0; T_issue = -1
    def strip_geo(sl, s):
        i0 = s * R + 1; lo = s * R + sl['c0']
        J0 = max(1, lo); J1 = min(sl['lb'], lo + R - 1 + 2 * sl['w'])
        alive = max(0, min(R, sl['la'] - i0 + 1))
        return i0, lo, J0, J1, alive
    def t0(sl, s):
        return sl['T0'] + s + strip_geo(sl, s)[2] - sl['J00']
    def te(sl, s):
        # a strip whose band lies left of column 1 has no cells: it ends where it starts
        return max(t0(sl, s), sl['T0'] + s + strip_geo(sl, s)[3] - sl['J00'])
    while True:
        # issue
        if q < len(pairs_geo) and T > T_issue and slots[seq % NSLOT] is None:
            A, B, la, lb, w, h = pairs_geo[q]
            c0 = 1 + h - w
            n_strips = (la + R - 1) // R
            lim = lb - 1 - h + w
            s_lim = 0 if lim < 0 else lim // R + 1
            S = min(n_strips, s_lim)
            if S == 0:
                res[q] = (0, 0); q += 1   # written at issue; the next issue waits a step
            else:
                sl = dict(p=q, A=A, B=B, la=la, lb=lb, w=w, h=h, c0=c0, S=S, J00=max(1, c0), T0=0, acc=0, gs=1,
                          seq=seq)
                req = T
                for lane in range(32):
                    m = (lane - g_next) % 32
                    if m < min(S, 32):
                        J0m = max(1, m * R + c0)
                        req = max(req, lanes[lane]['F'] + 1 - m - (J0m - sl['J00']))
                sl['T0'] = req
                slots[seq % NSLOT] = sl
                for lane in range(32):
                    m = (lane - g_next) % 32
                    if m < min(S, 32):
                        assert lanes[lane]['pend'] is None
                        lanes[lane]['pend'] = (seq % NSLOT, m)
                        last = m + 32 * ((S - 1 - m) // 32)
                        lanes[lane]['F'] = te(sl, last)
                T_issue = t0(sl, S - 1)
                g_next += S; seq += 1; q += 1
        # activation
        for L in lanes:
            if L['pend'] is not None:
                slot_i, s = L['pend']
                sl = slots[slot_i]
                if T >= t0(sl, s):
                    assert T == t0(sl, s), 'strip started late'
                    assert L['cur'] is None
                    i0, lo, J0, J1, alive = strip_geo(sl, s)
                    codes = [int(sl['A'][i0 + r - 1]) if r < alive else 0 for r in range(R)]
                    L['cur'] = dict(slot=slot_i, s=s, i0=i0, lo=lo, J0=J0, J1=J1, alive=alive, codes=codes,
                                    hc=[0] * R, fT=[NEG_F] * R, best=[0] * R, Te=te(sl, s))
                    L['pend'] = None
        hin_all = [lanes[(l + 31) & 31]['hout'] for l in range(32)]
        ein_all = [lanes[(l + 31) & 31]['eout'] for l in range(32)]
        cms = [0] * 32
        for lane, L in enumerate(lanes):
            hin, ein = hin_all[lane], ein_all[lane]
            c = L['cur']
            if c is None:
                L['hprev'] = hin; L['hout'], L['eout'] = 0, NEG_E; continue
            sl = slots[c['slot']]; s = c['s']
            j = T - sl['T0'] - s + sl['J00']
            top = s * R + sl['h'] + sl['w']
            hdiag = 0 if (s == 0 or j - 1 > top or j - 1 < 1) else L['hprev']
            L['hprev'] = hin
            if s == 0 or j > top: hin, ein = 0, NEG_E
            assert c['J0'] <= j <= c['J1'] or j > c['J1'] or j < c['J0']
            if c['J0'] <= j <= c['J1']:
                bc = int(sl['B'][j - 1]); hu, eu = hin, ein; hc, fT = c['hc'], c['fT']
                for r in range(R):
                    if r < c['alive'] and 0 <= j - r - c['lo'] <= 2 * sl['w']:
                        diagc = max(hdiag + inc(c['codes'][r], bc), ZKEY)
                        eR = max(hu + OPEN_E, eu + EXT)
                        fTn = max(fT[r] + EXT, hc[r] + OPEN_F) | TBIT
                        hn = max(diagc, eR, fTn) & CLEAN
                        hdiag = hc[r]; hc[r] = hn; fT[r] = fTn; hu = hn; eu = eR | TBIT
                    else:
                        hdiag = hc[r]; hc[r] = 0; hu = 0; eu = NEG_E
                L['hout'], L['eout'] = hu, eu
                cms[lane] = max(hc)
            else:
                L['hout'], L['eout'] = 0, NEG_E
        # tracking: per-pair gs
        trig = any(lanes[l]['cur'] is not None and (cms[l] >> 16) >= slots[lanes[l]['cur']['slot']]['gs']
                   for l in range(32))
        if trig:
            for l, L in enumerate(lanes):
                c = L['cur']
                if c is None: continue
                for r in range(R):
                    if c['hc'][r] > (c['best'][r] | (KU - 1)): c['best'][r] = c['hc'][r]
                sl = slots[c['slot']]
                if cms[l] > 0:
                    sl['gs'] = max(sl['gs'], cms[l] >> 16)
        # strip ends
        for l, L in enumerate(lanes):
            c = L['cur']
            if c is None or T != c['Te']: continue
            sl = slots[c['slot']]
            lb_, lr = 0, INT_MAX
            for r in range(R):
                b = c['best'][r]
                if r < c['alive'] and b > (lb_ | (KU - 1)): lb_, lr = b, c['i0'] + r
            if lb_ > 0:
                packed = ((lb_ >> 16) << 27) | ((16383 - lr) << 13) | (lb_ & MATCH)
                sl['acc'] = max(sl['acc'], packed)
            L['cur'] = None
            s = c['s']
            if s == sl['S'] - 1:
                acc = sl['acc']
                res[sl['p']] = (acc >> 27, acc & MATCH) if acc else (0, 0)
                slots[c['slot']] = None
            elif s + 32 < sl['S']:
                L['pend'] = (c['slot'], s + 32)
        T += 1
        if q >= len(pairs_geo) and all(L['cur'] is None and L['pend'] is None for L in lanes):
            break
    return res, T

def run_stream(seed, n, bw, maxlen=400, hint_frac=0.3, rows=None):
    rng = np.random.default_rng(seed)
    seqs, pg, pairs = [], [], []
    for k in range(n):
        li = int(rng.integers(1, maxlen)); lj = int(rng.integers(1, maxlen))
        a = rng.integers(0, 20, li).astype(np.uint8); b = rng.integers(0, 20, lj).astype(np.uint8)
        if rng.random() < 0.5:
            b = a[:lj].copy() if lj <= li else np.concatenate([a, rng.integers(0, 20, lj - li)]).astype(np.uint8)
            m = rng.random(lj) < 0.3; b[m] = rng.integers(0, 20, m.sum())
        sh = min(li, lj)
        hint = int(rng.integers(-sh, sh + 1)) if rng.random() < hint_frac else 0
        swap, la, lb, w, h = geometry(li, lj, bw, hint)
        A, B = (a, b) if not swap else (b, a)
        pg.append((A, B, la, lb, w, h)); seqs.append((a, b, hint))
    R = max(r_call(bw), rows or 0)
    got, T = stream(pg, R)
    bad = 0
    for k, (a, b, hint) in enumerate(seqs):
        flat = np.concatenate([a, b]); offs = np.array([0, len(a)], np.int64); lens = np.array([len(a), len(b)], np.int32)
        r = oracle.sw_batch(np.array([[0, 1]], np.int32), flat, offs, lens, bw, BLOSUM62, diag_hints=np.array([hint], np.int32))
        exp = (int(r['scores'][0]), int(r['matches'][0]))
        if got[k] != exp:
            bad += 1
            if bad < 4: print('BAD', k, len(a), len(b), bw, hint, got[k], exp)
    cells = sum(la * min(2 * w + 1, lb) for (_, _, la, lb, w, h) in pg)
    return bad



@pytest.mark.parametrize("seed,n,bw,maxlen", [(1, 12, 238, 300), (2, 20, 100, 200), (3, 8, 16, 700),
                                              (4, 6, 60, 900), (5, 10, 0, 45), (6, 6, 1, 300),
                                              (7, 4, 238, 900), (8, 40, 238, 120)])
def test_streamed_schedule_matches_oracle(seed, n, bw, maxlen):
    assert run_stream(seed, n, bw, maxlen) == 0


@pytest.mark.parametrize("seed,n,bw,maxlen,rows", [(11, 12, 50, 400, 16), (12, 10, 16, 700, 16),
                                                   (13, 10, 100, 300, 16), (14, 16, 50, 300, 8),
                                                   (15, 6, 1, 300, 16), (16, 30, 0, 45, 16)])
def test_streamed_schedule_with_taller_strips(seed, n, bw, maxlen, rows):
    """Strips taller than the smallest rotating height (a call-wide setting):
    the rotation bound holds a fortiori, results are unchanged."""
    assert run_stream(seed, n, bw, maxlen, rows=rows) == 0
