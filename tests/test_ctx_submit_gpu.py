"""The resident-database submit/poll interface of the C ABI (ck_ctx_upload_db,
ck_ctx_submit, ck_ctx_poll, ck_ctx_wait), driven through ctypes as a non-Python
host would drive it: results equal the host-buffer entry point's, two contexts
overlap, and misuse is reported by status codes."""
import numpy as np
import pytest

from clustkit_gb300 import _lib, synth
from clustkit_gb300.blosum import BLOSUM62
from clustkit_gb300.pairwise import ENGINE_BATCHED, ENGINE_PLAIN, PASS_CPU, batch_sw

pytestmark = pytest.mark.gpu
SUB = np.ascontiguousarray(BLOSUM62)


def _pinned(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()


class _Batch:
    """Page-locked host inputs and outputs of one submission."""

    def __init__(self, torch, pairs, hints=None):
        self.pairs = _pinned(torch, pairs.astype(np.int32))
        self.hints = None if hints is None else _pinned(torch, hints.astype(np.int32))
        m = len(pairs)
        self.out = {k: _pinned(torch, np.full(m, 7, dt)) for k, dt in
                    (("sims", np.float32), ("scores", np.int32), ("matches", np.int32), ("shorter", np.int32),
                     ("mask", np.uint8))}

    def submit(self, lib, ctx, bw, t, engine=ENGINE_BATCHED):
        o = self.out
        return lib.ck_ctx_submit(ctx, self.pairs.ctypes.data, len(self.pairs), bw, SUB.ctypes.data, t,
                                 None if self.hints is None else self.hints.ctypes.data, PASS_CPU, engine,
                                 o["sims"].ctypes.data, o["scores"].ctypes.data, o["matches"].ctypes.data,
                                 o["shorter"].ctypes.data, o["mask"].ctypes.data, None)


def _poll_until_done(lib, ctx):
    done = np.zeros(1, np.int32)
    for _ in range(10_000_000):
        st = lib.ck_ctx_poll(ctx, done.ctypes.data)
        if done[0]:
            return st
    raise AssertionError("submission never finished")


def test_submit_poll_matches_host_entry_point_on_two_contexts():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    data = synth.generate_families(30, 8, median=300, lo=30, hi=900, seed=81)
    p1 = synth.mixed_pairs(data, 5000, seed=1)
    p2 = synth.mixed_pairs(data, 3000, seed=2)
    rng = np.random.default_rng(3)
    sh = np.minimum(data.lengths[p2[:, 0]], data.lengths[p2[:, 1]])
    h2 = (rng.integers(-1000, 1000, len(p2)) % (2 * sh + 7) - sh - 3).astype(np.int32)
    ctxs = []
    try:
        for _ in range(2):
            h = np.zeros(1, np.int32)
            _lib.check(lib.ck_ctx_create(h.ctypes.data))
            ctxs.append(int(h[0]))
            _lib.check(lib.ck_ctx_upload_db(ctxs[-1], data.flat.ctypes.data, len(data.flat),
                                            data.offsets.ctypes.data, data.lengths.ctypes.data, data.n))
        b1, b2 = _Batch(torch, p1), _Batch(torch, p2, h2)
        for rep in range(2):  # the same contexts again: nothing of the first round leaks
            _lib.check(b1.submit(lib, ctxs[0], 100, 0.3))
            _lib.check(b2.submit(lib, ctxs[1], 50, 0.4, ENGINE_PLAIN if rep else ENGINE_BATCHED))
            # a second submission on a busy context is refused, the first one stands
            assert b1.submit(lib, ctxs[0], 100, 0.3) == _lib.CK_ERR_INVALID_ARGUMENT
            _lib.check(_poll_until_done(lib, ctxs[0]))
            _lib.check(lib.ck_ctx_wait(ctxs[1]))
            for b, pairs, bw, t, hints in ((b1, p1, 100, 0.3, None), (b2, p2, 50, 0.4, h2)):
                want = batch_sw(pairs, data.flat, data.offsets, data.lengths, bw, BLOSUM62, t, diag_hints=hints)
                for k in want:
                    assert np.array_equal(b.out[k], np.asarray(want[k]).astype(b.out[k].dtype)), (rep, k)
    finally:
        for c in ctxs:
            lib.ck_ctx_destroy(c)


def test_submit_reports_misuse_and_bad_indices():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    data = synth.generate_families(5, 4, median=120, lo=30, hi=300, seed=82)
    h = np.zeros(1, np.int32)
    _lib.check(lib.ck_ctx_create(h.ctypes.data))
    ctx = int(h[0])
    try:
        good = _Batch(torch, synth.mixed_pairs(data, 200, seed=4))
        assert good.submit(lib, ctx, 100, 0.3) == _lib.CK_ERR_INVALID_ARGUMENT  # no database yet
        done = np.zeros(1, np.int32)
        _lib.check(lib.ck_ctx_poll(ctx, done.ctypes.data))
        assert done[0] == 1  # nothing in flight
        _lib.check(lib.ck_ctx_upload_db(ctx, data.flat.ctypes.data, len(data.flat), data.offsets.ctypes.data,
                                        data.lengths.ctypes.data, data.n))
        bad_pairs = synth.mixed_pairs(data, 200, seed=5)
        bad_pairs[17, 1] = data.n + 3
        bad = _Batch(torch, bad_pairs)
        _lib.check(bad.submit(lib, ctx, 100, 0.3))
        assert _poll_until_done(lib, ctx) == _lib.CK_ERR_OUT_OF_RANGE
        # the error was read and cleared: the context serves the next batch
        _lib.check(good.submit(lib, ctx, 100, 0.3))
        _lib.check(lib.ck_ctx_wait(ctx))
        assert lib.ck_ctx_poll(99999, done.ctypes.data) == _lib.CK_ERR_INVALID_ARGUMENT
    finally:
        lib.ck_ctx_destroy(ctx)
