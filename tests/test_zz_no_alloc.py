"""The allocation-free entry point, ck_sw_batch_device_noalloc.

Some callers cannot let this library allocate GPU memory: a host system that
hands out all device memory from its own pre-sized pool, or a serving loop
that must not risk an allocation stalling or failing mid-request.  For them
the library offers one entry point whose only memory beyond the caller's
input and output buffers is a static 32 MiB workspace compiled into the
library.  These tests call it through the C ABI and require its results to be
identical to the regular device entry point's, on two calls in a row (the
static workspace keeps the previous call's contents, which must not leak
into the next call's results).

This file is collected last on purpose: run alone in a fresh process or after
every other test, it must pass either way.
"""
import numpy as np
import pytest

from clustkit_gb300 import synth
from clustkit_gb300.blosum import BLOSUM62
from clustkit_gb300.pairwise import ENGINE_BATCHED, PASS_CPU

pytestmark = pytest.mark.gpu


def _device_run(lib, torch, data, pairs, bw, threshold, noalloc, hints=None):
    dev = torch.device("cuda:0")
    s = data
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_pairs, d_flat, d_off, d_len = T(pairs), T(s.flat), T(s.offsets), T(s.lengths)
    d_hints = None if hints is None else T(hints)
    M = len(pairs)
    out = {k: torch.full((M,), 7, dtype=dt, device=dev) for k, dt in
           (("sims", torch.float32), ("scores", torch.int32), ("matches", torch.int32),
            ("shorter", torch.int32), ("mask", torch.uint8))}
    sub = np.ascontiguousarray(BLOSUM62)
    stream = torch.cuda.current_stream().cuda_stream
    common = (d_pairs.data_ptr(), M, d_flat.data_ptr(), len(s.flat), d_off.data_ptr(), d_len.data_ptr(),
              s.n, bw, sub.ctypes.data, float(threshold), None if d_hints is None else d_hints.data_ptr(),
              PASS_CPU)
    outs = (out["sims"].data_ptr(), out["scores"].data_ptr(), out["matches"].data_ptr(),
            out["shorter"].data_ptr(), out["mask"].data_ptr(), stream)
    torch.cuda.synchronize()
    if noalloc:
        st = lib.ck_sw_batch_device_noalloc(*common, *outs)
        assert st == 0, lib.ck_last_error()
    else:
        st = lib.ck_sw_batch_device(*common, ENGINE_BATCHED, *outs)
        assert st == 0, lib.ck_last_error()
        assert lib.ck_sw_status_device(stream) == 0
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def _hints(data, pairs, seed):
    """Diagonal hints across the whole range, some beyond +-shorter (clamped to 0)."""
    rng = np.random.default_rng(seed)
    sh = np.minimum(data.lengths[pairs[:, 0]], data.lengths[pairs[:, 1]])
    h = (rng.integers(-3000, 3000, len(pairs)) % (2 * sh + 41) - sh - 20).astype(np.int32)
    h[rng.random(len(pairs)) < 0.3] = 0
    return h


def test_noalloc_matches_device_entry_point_twice(ck):
    """The allocation-free entry point first (before the allocating one in each
    case), then the regular device entry point on the same inputs: equal
    outputs, on calls in a row with different shapes, with and without
    diagonal hints, up to the widest band the static workspace takes."""
    torch = pytest.importorskip("torch")
    lib = ck.load()
    cases = [
        (synth.generate_families(30, 8, median=300, lo=30, hi=900, seed=71), 100, 0.3, 6000, False),
        (synth.generate_families(25, 6, median=150, lo=20, hi=500, seed=72), 16, 0.5, 4000, False),
        (synth.generate_families(20, 6, median=250, lo=20, hi=700, seed=73), 32, 0.3, 3000, True),
        (synth.generate_families(4, 3, median=600, lo=100, hi=1500, seed=74), 8191, 0.3, 40, False),
    ]
    for data, bw, t, n_pairs, hinted in cases:
        pairs = synth.mixed_pairs(data, n_pairs, seed=bw)
        hints = _hints(data, pairs, bw) if hinted else None
        got = _device_run(lib, torch, data, pairs, bw, t, noalloc=True, hints=hints)
        want = _device_run(lib, torch, data, pairs, bw, t, noalloc=False, hints=hints)
        for k in want:
            assert np.array_equal(got[k], want[k]), (bw, k)


def test_noalloc_call_leaves_free_device_memory_unchanged(ck):
    """After one call (which may load the library's module and with it the
    static arrays), further calls take no device memory: cudaMemGetInfo's free
    bytes are the same before and after."""
    torch = pytest.importorskip("torch")
    lib = ck.load()
    data = synth.generate_families(20, 8, median=300, lo=30, hi=900, seed=75)
    pairs = synth.mixed_pairs(data, 5000, seed=3)
    dev = torch.device("cuda:0")
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_pairs, d_flat, d_off, d_len = T(pairs), T(data.flat), T(data.offsets), T(data.lengths)
    outs = [torch.empty(len(pairs), dtype=dt, device=dev)
            for dt in (torch.float32, torch.int32, torch.int32, torch.int32, torch.uint8)]
    sub = np.ascontiguousarray(BLOSUM62)
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        st = lib.ck_sw_batch_device_noalloc(d_pairs.data_ptr(), len(pairs), d_flat.data_ptr(), len(data.flat),
                                            d_off.data_ptr(), d_len.data_ptr(), data.n, 100, sub.ctypes.data,
                                            0.3, None, PASS_CPU, *[o.data_ptr() for o in outs], stream)
        assert st == 0, lib.ck_last_error()

    call()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev)[0]
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free0


def test_noalloc_rejects_sizes_beyond_its_workspace(ck):
    torch = pytest.importorskip("torch")
    lib = ck.load()
    from clustkit_gb300._lib import CK_ERR_UNSUPPORTED
    data = synth.generate_families(2, 2, median=100, lo=50, hi=200, seed=1)
    dev = torch.device("cuda:0")
    pairs = torch.zeros((1, 2), dtype=torch.int32, device=dev)
    flat = torch.from_numpy(data.flat).to(dev)
    off = torch.from_numpy(data.offsets).to(dev)
    ln = torch.from_numpy(data.lengths).to(dev)
    o = torch.empty(1, dtype=torch.float32, device=dev)
    sub = np.ascontiguousarray(BLOSUM62)
    for bw in (0, 9000):
        st = lib.ck_sw_batch_device_noalloc(pairs.data_ptr(), 1, flat.data_ptr(), len(data.flat),
                                            off.data_ptr(), ln.data_ptr(), data.n, bw, sub.ctypes.data,
                                            0.5, None, PASS_CPU, o.data_ptr(), None, None, None, None,
                                            torch.cuda.current_stream().cuda_stream)
        assert st == CK_ERR_UNSUPPORTED
