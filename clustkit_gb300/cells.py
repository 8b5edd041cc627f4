"""Work accounting: the number of banded DP cells clustkit evaluates per pair.

For a pair with rows la (the shorter side), columns lb, band half-width w
(lb itself when band_width <= 0 or lb <= 50, clustkit/csrc/sw_align.c:55-58)
and band offset h, row i covers columns max(1, i+h-w) .. min(lb, i+h+w); the
reference has no early exit, so GCUPS = sum of these cells / time.
"""
from __future__ import annotations

import numpy as np


def effective_band(la, lb, band_width: int):
    lb = np.asarray(lb, np.int64)
    if band_width <= 0:
        return lb.copy()
    return np.where(lb <= 50, lb, np.int64(band_width))


def _sum_min(a, b, c, L):
    # sum_{i=a}^{b} min(L, i + c), elementwise, 0 where b < a
    t = L - c
    e1 = np.minimum(b, t)
    n1 = np.maximum(e1 - a + 1, 0)
    s = (n1 * (a + e1)) // 2 + n1 * c
    s2 = np.maximum(a, t + 1)
    n2 = np.maximum(b - s2 + 1, 0)
    return np.where(b < a, 0, s + n2 * L)


def _sum_max(a, b, c, L):
    # sum_{i=a}^{b} max(L, i + c)
    t = L - c
    e1 = np.minimum(b, t)
    n1 = np.maximum(e1 - a + 1, 0)
    s2 = np.maximum(a, t + 1)
    n2 = np.maximum(b - s2 + 1, 0)
    s = n1 * L + (n2 * (s2 + b)) // 2 + n2 * c
    return np.where(b < a, 0, s)


def band_cells(la, lb, w, h=None) -> np.ndarray:
    la = np.asarray(la, np.int64)
    lb = np.asarray(lb, np.int64)
    w = np.asarray(w, np.int64)
    h = np.zeros_like(la) if h is None else np.asarray(h, np.int64)
    c1 = h - w
    c2 = h + w
    ilo = np.maximum(1 - c2, 1)
    ihi = np.minimum(lb - c1, la)
    ok = (la > 0) & (lb > 0) & (ihi >= ilo)
    one = np.ones_like(la)
    cells = _sum_min(ilo, ihi, c2, lb) - _sum_max(ilo, ihi, c1, one) + (ihi - ilo + 1)
    return np.where(ok, cells, 0)


def band_cells_loop(la: int, lb: int, w: int, h: int = 0) -> int:
    c = 0
    for i in range(1, la + 1):
        lo, hi = max(1, i + h - w), min(lb, i + h + w)
        if hi >= lo:
            c += hi - lo + 1
    return c


def pair_cells(pairs, lengths, band_width: int, hints=None) -> np.ndarray:
    """Cells per pair for a pair list, with clustkit's swap and hint rules."""
    pairs = np.asarray(pairs).reshape(-1, 2)
    li = np.asarray(lengths, np.int64)[pairs[:, 0]]
    lj = np.asarray(lengths, np.int64)[pairs[:, 1]]
    la = np.minimum(li, lj)
    lb = np.maximum(li, lj)
    h = np.zeros_like(la)
    if hints is not None:
        hh = np.asarray(hints, np.int64)
        hh = np.where((hh > la) | (hh < -la), 0, hh)
        h = np.where(li <= lj, hh, -hh)
    return band_cells(la, lb, effective_band(la, lb, band_width), h)
