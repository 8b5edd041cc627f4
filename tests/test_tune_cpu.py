"""Host logic of the autotuner (no GPU needed)."""
import numpy as np

from clustkit_gb300 import tune


def test_profile_key_buckets_and_band():
    L = np.array([30, 60, 120, 4000, 8000], np.int32)
    p = np.array([[0, 1], [1, 2], [3, 4], [2, 3]], np.int32)
    k1 = tune.profile_key(L, p, 64)
    k2 = tune.profile_key(L, p, 128)
    assert k1[0] == 64 and k2[0] == 128 and k1[1:] == k2[1:]
    assert len(k1[1]) == 4 and all(isinstance(x, int) for x in k1[1])


def test_candidate_sets_cover_the_tunables():
    assert set(tune.DEFAULT) == set(tune.KEYS)
    assert {r for r, _ in tune.TILINGS} == {8, 16, 24}
    assert {v for _, v in tune.TILINGS} == {0, 1, 2, 3}
    assert (tune.DEFAULT["wave_min_rows"], tune.DEFAULT["wave_adaptive"]) in tune.BIN_EDGES
