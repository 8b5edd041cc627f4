"""MinHash sketching, drop-in for clustkit's ``clustkit.sketch``
(clustkit/sketch.py:112-183); the hashing and bottom-s selection run in
libckgpu.so on the GPU."""
from __future__ import annotations

import numpy as np

from . import _lib

__all__ = ["compute_sketches", "sketch_sequence", "sketch_flat"]


def sketch_flat(flat_sequences, offsets, lengths, k: int, sketch_size: int,
                alphabet_size: int = 20, seed: int = 42) -> np.ndarray:
    """(N, sketch_size) uint64 sketches of sequences in clustkit's compact layout."""
    lib = _lib.load()
    _lib.require_gpu()
    flat = np.ascontiguousarray(flat_sequences, dtype=np.uint8).reshape(-1)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64).reshape(-1)
    lengths = np.ascontiguousarray(lengths, dtype=np.int32).reshape(-1)
    n = lengths.shape[0]
    out = np.empty((n, int(sketch_size)), dtype=np.uint64)
    _lib.check(lib.ck_sketch(_lib.ptr(flat), flat.shape[0], _lib.ptr(offsets), _lib.ptr(lengths), n,
                             int(k), int(sketch_size), int(alphabet_size), int(seed) & (2**64 - 1),
                             _lib.ptr(out)))
    return out


def sketch_sequence(encoded_seq, seq_length: int, k: int, sketch_size: int, alphabet_size: int,
                    seed: int = 42) -> np.ndarray:
    """clustkit/sketch.py:112-134."""
    seq = np.ascontiguousarray(encoded_seq, dtype=np.uint8)[: int(seq_length)]
    out = sketch_flat(seq, np.zeros(1, np.int64), np.array([int(seq_length)], np.int32), k,
                      sketch_size, alphabet_size, seed)
    return out[0]


def compute_sketches(encoded_sequences, lengths, k: int, sketch_size: int, mode: str,
                     seed: int = 42, device: str = "0", flat_sequences=None, offsets=None):
    """clustkit/sketch.py:137-183: (N, sketch_size) uint64 on the host."""
    alphabet_size = 20 if mode == "protein" else 4
    lengths = np.asarray(lengths)
    if flat_sequences is None or offsets is None:
        n = len(lengths)
        offsets = np.zeros(n, dtype=np.int64)
        if n > 1:
            offsets[1:] = np.cumsum(np.asarray(lengths[:-1], dtype=np.int64))
        flat_sequences = np.empty(int(np.sum(lengths)), dtype=np.uint8)
        for i in range(n):
            ln = int(lengths[i])
            flat_sequences[offsets[i]:offsets[i] + ln] = encoded_sequences[i, :ln]
    return sketch_flat(flat_sequences, offsets, lengths, k, sketch_size, alphabet_size, seed)
