"""BLOSUM62 in clustkit's residue order, plus the derived constants the kernels use.

clustkit encodes proteins over the alphabet ``ACDEFGHIKLMNPQRSTVWY`` (codes
0..19, anything else -> 20; clustkit/io.py:9-18) and scores the Align phase
with BLOSUM62 in that order (clustkit/pairwise.py:129-151), gap open -11 and
gap extend -1 (clustkit/csrc/sw_align.c:45-46).  BLOSUM62 is the published
Henikoff & Henikoff (1992) matrix; it is written below in its customary
``ARNDCQEGHILKMFPSTWYV`` order and permuted into clustkit's order by code.
"""
from __future__ import annotations

import numpy as np

PROTEIN_ALPHABET = "ACDEFGHIKLMNPQRSTVWY"
NUCLEOTIDE_ALPHABET = "ACGT"
PROTEIN_UNKNOWN = 20
NUCLEOTIDE_UNKNOWN = 4

GAP_OPEN = -11
GAP_EXTEND = -1
UNKNOWN_SCORE = -4  # score of any pair involving a code >= 20 (sw_align.c:116-119)

_CUSTOMARY_ORDER = "ARNDCQEGHILKMFPSTWYV"
_CUSTOMARY_ROWS = """
 4 -1 -2 -2  0 -1 -1  0 -2 -1 -1 -1 -1 -2 -1  1  0 -3 -2  0
-1  5  0 -2 -3  1  0 -2  0 -3 -2  2 -1 -3 -2 -1 -1 -3 -2 -3
-2  0  6  1 -3  0  0  0  1 -3 -3  0 -2 -3 -2  1  0 -4 -2 -3
-2 -2  1  6 -3  0  2 -1 -1 -3 -4 -1 -3 -3 -1  0 -1 -4 -3 -3
 0 -3 -3 -3  9 -3 -4 -3 -3 -1 -1 -3 -1 -2 -3 -1 -1 -2 -2 -1
-1  1  0  0 -3  5  2 -2  0 -3 -2  1  0 -3 -1  0 -1 -2 -1 -2
-1  0  0  2 -4  2  5 -2  0 -3 -3  1 -2 -3 -1  0 -1 -3 -2 -2
 0 -2  0 -1 -3 -2 -2  6 -2 -4 -4 -2 -3 -3 -2  0 -2 -2 -3 -3
-2  0  1 -1 -3  0  0 -2  8 -3 -3 -1 -2 -1 -2 -1 -2 -2  2 -3
-1 -3 -3 -3 -1 -3 -3 -4 -3  4  2 -3  1  0 -3 -2 -1 -3 -1  3
-1 -2 -3 -4 -1 -2 -3 -4 -3  2  4 -2  2  0 -3 -2 -1 -2 -1  1
-1  2  0 -1 -3  1  1 -2 -1 -3 -2  5 -1 -3 -1  0 -1 -3 -2 -2
-1 -1 -2 -3 -1  0 -2 -3 -2  1  2 -1  5  0 -2 -1 -1 -1 -1  1
-2 -3 -3 -3 -2 -3 -3 -3 -1  0  0 -3  0  6 -4 -2 -2  1  3 -1
-1 -2 -2 -1 -3 -1 -1 -2 -2 -3 -3 -1 -2 -4  7 -1 -1 -4 -3 -2
 1 -1  1  0 -1  0  0  0 -1 -2 -2  0 -1 -2 -1  4  1 -3 -2 -2
 0 -1  0 -1 -1 -1 -1 -2 -2 -1 -1 -1 -1 -2 -1  1  5 -2 -2  0
-3 -3 -4 -4 -2 -2 -3 -2 -2 -3 -2 -3 -1  1 -4 -3 -2 11  2 -3
-2 -2 -2 -3 -2 -1 -2 -3  2 -1 -1 -2 -1  3 -3 -2 -2  2  7 -1
 0 -3 -3 -3 -1 -2 -2 -3 -3  3  1 -2  1 -1 -2 -2  0 -3 -1  4
"""


def _build() -> np.ndarray:
    cust = np.array([[int(v) for v in row.split()] for row in _CUSTOMARY_ROWS.strip().splitlines()],
                    dtype=np.int8)
    perm = np.array([_CUSTOMARY_ORDER.index(c) for c in PROTEIN_ALPHABET])
    out = cust[np.ix_(perm, perm)].copy()
    # clustkit's table (clustkit/pairwise.py:142, row N) scores N->D as 0 where
    # the published matrix has +1, so its table is not symmetric: S(N,D) = 0,
    # S(D,N) = 1.  Scores must match clustkit's bit for bit, so that cell is
    # kept; the kernels index the table as sub[row residue][column residue].
    out[PROTEIN_ALPHABET.index("N"), PROTEIN_ALPHABET.index("D")] = 0
    out.setflags(write=False)
    return out


BLOSUM62 = _build()


def encode_protein(seq: str) -> np.ndarray:
    """Encode a protein string as clustkit does (clustkit/io.py:134-156)."""
    table = np.full(256, PROTEIN_UNKNOWN, dtype=np.uint8)
    for i, c in enumerate(PROTEIN_ALPHABET):
        table[ord(c)] = i
        table[ord(c.lower())] = i
    raw = np.frombuffer(seq.encode("ascii", "replace"), dtype=np.uint8)
    return table[raw]
