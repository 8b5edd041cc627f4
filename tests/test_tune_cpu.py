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
    assert {r for r, _, _ in tune.TILINGS} == {8, 16, 24, 32}
    assert {v for _, v, _ in tune.TILINGS} == {0, 1, 2, 3}
    assert {t for _, _, t in tune.TILINGS} == {0, 512, 640, 768}
    # the CTA's threads are a choice for 8-row strips only
    assert all(t == 0 for r, _, t in tune.TILINGS if r > 8)
    assert (tune.DEFAULT["wave_min_rows"], tune.DEFAULT["wave_adaptive"]) in tune.BIN_EDGES


def test_autotune_keeps_the_default_unless_the_winner_is_clearly_faster(monkeypatch):
    """The tuner's selection on CPU, with times from a table: a trial win
    that does not hold up on the re-time against the default, or holds up by
    less than 2 %, leaves the default in place."""
    applied = dict(tune.DEFAULT)
    monkeypatch.setattr(tune, "apply", lambda cfg: applied.update(cfg))
    monkeypatch.setattr(tune, "current", lambda: dict(applied))
    L = np.full(10, 300, np.int32)
    p = np.array([[0, 1], [2, 3]], np.int32)

    def run(trial_ms, confirm_ms):
        phase = {"confirm": False}
        real_confirm = tune.confirm

        def fake_confirm(call, cand, base, rounds=3, repeats=5):
            phase["confirm"] = True
            return real_confirm(call, cand, base, rounds, repeats)

        monkeypatch.setattr(tune, "confirm", fake_confirm)

        class Call:
            pairs = p

            def time_ms(self, repeats=5, warmup=1, engine=0):
                return (confirm_ms if phase["confirm"] else trial_ms)(applied)

        monkeypatch.setattr(tune, "_DeviceCall", lambda *a: Call())
        return tune.autotune(p, np.zeros(3000, np.uint8), np.arange(10) * 300, L, 100, use_cache=False)

    noisy = lambda cfg: 9.0 if cfg["rows_per_strip"] == 24 else 10.0
    res = run(noisy, lambda cfg: 10.0)  # the trial win does not hold up on the re-time
    assert res.config == tune.DEFAULT and res.confirm["kept"] == "default"
    res = run(noisy, lambda cfg: 9.5 if cfg["rows_per_strip"] == 24 else 10.0)  # 5 % faster: taken
    assert res.config["rows_per_strip"] == 24 and res.confirm["kept"] == "candidate"
    res = run(noisy, lambda cfg: 9.9 if cfg["rows_per_strip"] == 24 else 10.0)  # 1 %: below the bar
    assert res.config == tune.DEFAULT
