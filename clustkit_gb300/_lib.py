"""ctypes binding of libckgpu.so (include/clustkit_gb300.h).

The library is the only compute path: if it is missing or no GPU is visible,
calls raise; nothing falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

import numpy as np

from . import build as _build

CK_OK = 0
CK_ERR_INVALID_ARGUMENT = 1
CK_ERR_OUT_OF_RANGE = 2
CK_ERR_CUDA = 3
CK_ERR_OUT_OF_MEMORY = 4
CK_ERR_UNSUPPORTED = 5
CK_ERR_NO_DEVICE = 6
CK_ERR_CAPACITY = 7

PASS_CPU, PASS_NUMBA, PASS_CUPY, PASS_SCORE = 0, 1, 2, 3
ENGINE_BATCHED, ENGINE_PLAIN = 0, 1
CFG_ROWS_PER_STRIP = 0
CFG_STRIP_VARIANT = 1
CFG_WAVE_MIN_ROWS = 2
CFG_WAVE_ALL_BELOW = 3
CFG_WAVE_ADAPTIVE = 4
CFG_WAVE_STREAM = 5
CFG_WAVE_ROWS = 6
CFG_STRIP_KEY = 9
CFG_STRIP_THREADS = 10

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64

# name -> (restype, argtypes); the complete exported surface of the header
SIGNATURES = {
    "ck_version": (_I32, []),
    "ck_last_error": (ctypes.c_char_p, []),
    "ck_last_status": (_I32, []),
    "ck_device_count": (_I32, []),
    "batch_sw_align_c": (None, [_P, _P, _P, _P, _I32, _I32, _P, ctypes.c_float, _P, _P, _P, _P]),
    "sw_set_num_threads": (None, [_I32]),
    "ck_sw_batch": (_I32, [_P, _I64, _P, _I64, _P, _P, _I64, _I32, _P, ctypes.c_float, _P, _I32, _I32,
                           _P, _P, _P, _P, _P]),
    "ck_sw_batch_device": (_I32, [_P, _I64, _P, _I64, _P, _P, _I64, _I32, _P, ctypes.c_float, _P, _I32,
                                  _I32, _P, _P, _P, _P, _P, _P]),
    "ck_sw_batch_device_noalloc": (_I32, [_P, _I64, _P, _I64, _P, _P, _I64, _I32, _P, ctypes.c_float,
                                          _P, _I32, _P, _P, _P, _P, _P, _P]),
    "ck_sw_status_device": (_I32, [_P]),
    "ck_ctx_create": (_I32, [_P]),
    "ck_ctx_destroy": (_I32, [_I32]),
    "ck_ctx_status": (_I32, [_I32, _P]),
    "ck_sw_batch_device_ctx": (_I32, [_I32, _P, _I64, _P, _I64, _P, _P, _I64, _I32, _P, ctypes.c_float, _P,
                                      _I32, _I32, _P, _P, _P, _P, _P, _P]),
    "ck_ctx_upload_db": (_I32, [_I32, _P, _I64, _P, _P, _I64]),
    "ck_ctx_submit": (_I32, [_I32, _P, _I64, _I32, _P, ctypes.c_float, _P, _I32, _I32, _P, _P, _P, _P, _P, _P]),
    "ck_ctx_poll": (_I32, [_I32, _P]),
    "ck_ctx_wait": (_I32, [_I32]),
    "ck_kmer_index_build_device": (_I32, [_I32, _P, _I64, _P, _P, _I64, _I32, _I32, _P, _P, _I64, _P, _P,
                                          _P]),
    "ck_kmer_targets_device": (_I32, [_I32, _P, _I64, _P, _P]),
    "ck_search_pairs_device": (_I32, [_I32, _I32, _I32, _I32, _P, _P, _P, _P]),
    "ck_search_phase_a_device": (_I32, [_I32, _P, _I64, _P, _P, _I32, _I32, _I32, _I32, _P, _P, _P, _P, _I32,
                                        _I32, _I32, _I32, _P, _P, _P, _P]),
    "ck_sw_last_counters": (_I32, [_P]),
    "ck_sw_last_wave_pairs": (_I32, [_P]),
    "ck_ctx_freeze": (_I32, [_I32, _I32]),
    "ck_lsh_candidates_device": (_I32, [_I32, _P, _I64, _I32, _I32, _I32, _P, _P, _P, _I64, _P, _P]),
    "ck_search_phase_a_similar_device": (_I32, [_I32, _P, _I64, _P, _P, _I32, _I32, _P, _I32, _P, _P, _P, _P,
                                                _I32, _I32, _I32, _I32, _P, _P, _P, _I64, _P]),
    "ck_search_kmer_candidates_device": (_I32, [_I32, _P, _I64, _P, _P, _I32, _I32, _I32, _I32, _P, _P, _P, _P,
                                                _I32, _I32, _P, _I32, _I32, _I32, _I32, _I32, _P, _P, _P, _P, _I64,
                                                _P]),
    "ck_graph_csr_device": (_I32, [_I32, _P, _P, _I64, _I64, _P, _P, _P, _P, _P]),
    "ck_connected_components_device": (_I32, [_I32, _P, _I64, _I64, _P, _P, _P, _P]),
    "ck_sketch": (_I32, [_P, _I64, _P, _P, _I64, _I32, _I32, _I32, ctypes.c_uint64, _P]),
    "ck_sketch_device": (_I32, [_P, _I64, _P, _P, _I64, _I32, _I32, _I32, ctypes.c_uint64, _P, _P]),
    "ck_jaccard": (_I32, [_P, _I64, _P, _I64, _I32, ctypes.c_float, _P, _P]),
    "ck_jaccard_device": (_I32, [_P, _I64, _P, _I64, _I32, ctypes.c_float, _P, _P, _P]),
    "ck_probe_int_rate": (_I32, [_I32, _P]),
    "ck_probe_cell_rate": (_I32, [_I32, _P]),
    "ck_sw_profile": (_I32, [_I32]),
    "ck_sw_last_kernel_ms": (_I32, [_P]),
    "ck_sw_set_config": (_I32, [_I32, _I32]),
    "ck_sw_get_config": (_I32, [_I32, _P]),
}


class CkError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"libckgpu error {status}: {msg}")
        self.status = status


_lock = threading.Lock()
_lib = None


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building in-tree first if needed) and bind libckgpu.so."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if build_if_missing:
                path = _build.build()
            if not path.exists():
                raise CkError(CK_ERR_UNSUPPORTED, f"{path} not built; run __graft_entry__.build()")
            lib = ctypes.CDLL(str(path))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(status: int) -> None:
    if status != CK_OK:
        msg = load().ck_last_error()
        raise CkError(status, msg.decode() if msg else "")


def require_gpu() -> None:
    if load().ck_device_count() < 1:
        raise CkError(CK_ERR_NO_DEVICE, "no CUDA device visible; the GPU path has no CPU fallback")


def ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


def sw_counters() -> dict:
    out = np.zeros(6, np.int64)
    check(load().ck_sw_last_counters(out.ctypes.data))
    keys = ("pairs", "cells", "batched", "plain", "rerun", "launches")
    d = {k: int(v) for k, v in zip(keys, out)}
    wave = np.zeros(1, np.int64)
    check(load().ck_sw_last_wave_pairs(wave.ctypes.data))
    d["wave"] = int(wave[0])
    return d


def set_config(key: int, value: int) -> None:
    check(load().ck_sw_set_config(int(key), int(value)))


def get_config(key: int) -> int:
    v = np.zeros(1, np.int32)
    check(load().ck_sw_get_config(int(key), v.ctypes.data))
    return int(v[0])
