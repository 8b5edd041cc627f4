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


def _device_run(lib, torch, fn_name, data, pairs, bw, threshold, noalloc):
    dev = torch.device("cuda:0")
    s = data
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_pairs, d_flat, d_off, d_len = T(pairs), T(s.flat), T(s.offsets), T(s.lengths)
    M = len(pairs)
    out = {k: torch.full((M,), 7, dtype=dt, device=dev) for k, dt in
           (("sims", torch.float32), ("scores", torch.int32), ("matches", torch.int32),
            ("shorter", torch.int32), ("mask", torch.uint8))}
    sub = np.ascontiguousarray(BLOSUM62)
    stream = torch.cuda.current_stream().cuda_stream
    common = (d_pairs.data_ptr(), M, d_flat.data_ptr(), len(s.flat), d_off.data_ptr(), d_len.data_ptr(),
              s.n, bw, sub.ctypes.data, float(threshold), None, PASS_CPU)
    outs = (out["sims"].data_ptr(), out["scores"].data_ptr(), out["matches"].data_ptr(),
            out["shorter"].data_ptr(), out["mask"].data_ptr(), stream)
    if noalloc:
        st = lib.ck_sw_batch_device_noalloc(*common, *outs)
        assert st == 0, lib.ck_last_error()
    else:
        st = lib.ck_sw_batch_device(*common, ENGINE_BATCHED, *outs)
        assert st == 0, lib.ck_last_error()
        assert lib.ck_sw_status_device(stream) == 0
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def test_noalloc_matches_device_entry_point_twice(ck):
    torch = pytest.importorskip("torch")
    lib = ck.load()
    cases = [
        (synth.generate_families(30, 8, median=300, lo=30, hi=900, seed=71), 100, 0.3, 6000),
        (synth.generate_families(25, 6, median=150, lo=20, hi=500, seed=72), 16, 0.5, 4000),
    ]
    for data, bw, t, n_pairs in cases:  # two calls in a row, different shapes
        pairs = synth.mixed_pairs(data, n_pairs, seed=bw)
        want = _device_run(lib, torch, "ck_sw_batch_device", data, pairs, bw, t, noalloc=False)
        got = _device_run(lib, torch, "ck_sw_batch_device_noalloc", data, pairs, bw, t, noalloc=True)
        for k in want:
            assert np.array_equal(got[k], want[k]), k


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
