"""CPU model of the lane-per-pair strip loop's column schedule
(csrc/sw_batched.cu: align_pair_strips, strip_group, strip_group_percol,
strip_column): for random pair geometries, band widths, hints, strip heights
and every variant, each band column of each strip is visited exactly once in
order, the prefetch queue always holds the next columns, every window slot
index stays below W, every residue read lies inside the sequence, and every
window entry a strip reads (its columns and its first row's diagonal input)
holds that column's value: for the first strip that runs, the boundary the pair
starts with; after it, a value the previous strip wrote or the boundary it
filled past its end.  The
kernel's own results are checked against the oracle on the GPU; this pins the
index arithmetic, which a GPU run can only show by faulting."""
import random

import pytest


def _strip_loop(la, lb, w, h, R, U, P, aligned, W):
    wmask = W - 1
    held = dict.fromkeys(range(W), "boundary")  # window slot -> whose entry it holds
    fresh = True
    i0 = 1
    while i0 <= la:
        lo0 = i0 + h - w
        J0, J1 = max(lo0, 1), min(i0 + R - 1 + h + w, lb)
        if J0 > lb:
            break
        if J1 < J0:
            i0 += R
            continue
        for c in range(J0 - 1 if J0 >= 2 else J0, J1 + 1):  # every entry the strip reads
            # the first strip that runs reads the pair's initial boundary (its row
            # above is row 0 or lies left of column 1); later ones what was written
            assert held[c & wmask] == ("boundary" if fresh else c), (c, J0, J1)
        fresh = False
        queue = [J0 + k for k in range(P)]
        for k in range(P):  # strip start: residues of J0 .. J0+P-1, clamped
            assert 0 <= min(J0 + k, lb) - 1 <= lb - 1
        I0, I1 = max(lo0 + R - 1, J0), min(i0 + h + w, J1)
        j, seen = J0, []
        while j <= J1:
            if aligned and j >= I0 and j % U == 0 and j + U - 1 <= I1 and j + U - 1 + P <= lb:
                cur = j & wmask
                for u in range(U):
                    assert queue.pop(0) == j + u
                    c = u + P  # column loaded: run c // U of the group, offset c % U
                    slot = ((j + (c // U) * U) & wmask) + c % U
                    assert slot == (j + c) & wmask and 0 <= slot < W
                    queue.append(j + c)
                    assert 0 <= j + P - 1 + u <= lb - 1  # residue of column j + c, unclamped
                    assert cur + u == (j + u) & wmask  # the store's slot
                    seen.append(j + u)
                j += U
            elif not aligned and j >= I0 and j + U - 1 <= I1:
                for u in range(U):
                    assert queue.pop(0) == j + u
                    queue.append(j + u + P)
                    assert 0 <= min(j + u + P, lb) - 1 <= lb - 1
                    seen.append(j + u)
                j += U
            else:
                assert queue.pop(0) == j
                queue.append(j + P)
                assert 0 <= min(j + P, lb) - 1 <= lb - 1
                seen.append(j)
                j += 1
        assert seen == list(range(J0, J1 + 1))
        for c in seen:  # the strip's last row, then the boundary past its end
            held[c & wmask] = c
        for c in range(J1 + 1, min(J1 + R, lb) + 1):
            held[c & wmask] = c
        i0 += R


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_strip_column_schedule(seed):
    rng = random.Random(seed)
    for _ in range(250):
        la = rng.randint(1, 600)
        lb = rng.randint(la, 900)
        bw = rng.choice([0, 1, 2, 3, 8, 16, 32, 50, 64, 100, 128, 300])
        w = lb if (bw <= 0 or lb <= 50) else bw
        h = rng.choice([0, 0, rng.randint(-la, la)])
        for R in (8, 16, 24, 32):
            for V in range(4):
                U, aligned = (4 if V & 2 else 2), bool(V & 1)
                P = 4 if aligned else 2
                W = 1
                while W < 2 * w + 2 * R + 2:
                    W *= 2
                _strip_loop(la, lb, w, h, R, U, P, aligned, W)
