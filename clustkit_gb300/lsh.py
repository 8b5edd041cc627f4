"""LSH candidate generation (the input producer of the Align phase).

``lsh_candidates_device`` runs clustkit's LSH (clustkit/lsh.py:20-178) on the
GPU (csrc/lsh.cu); ``lsh_candidates`` restates it in vectorised numpy on the
host, with numpy's own argsort, for small inputs and as the tie-order
reference.  Both:

* band indices and per-table seeds come from ``np.random.RandomState(seed)``
  in the same draw order (lsh.py:116-123);
* a bucket id is ``h = seed; h = h*0x517CC1B727220A95 + sketch[idx]`` over the
  band, then ``h = (h ^ h>>33) * 0xC4CEB9FE1A85EC53; h ^= h>>33``
  (lsh.py:20-29), all in wrapping uint64;
* per table the sequences are ordered by bucket id and every bucket
  contributes all pairs among its first 1000 members (lsh.py:51-90, 153-156)
  -- the host version with ``np.argsort`` (the same call as clustkit, so ties
  come out in the same order), the device version with a stable radix sort
  (members in ascending id; identical unless a bucket has more than 1000);
* pairs are packed ``i*N + j`` with ``i < j``, sorted and de-duplicated
  (lsh.py:163-178).
"""
from __future__ import annotations

import numpy as np

_MUL = np.uint64(0x517CC1B727220A95)
_FMIX = np.uint64(0xC4CEB9FE1A85EC53)
_S33 = np.uint64(33)
MAX_BUCKET = 1000


def band_parameters(sketch_size: int, num_tables: int, num_bands: int, seed: int = 42):
    rng = np.random.RandomState(seed)
    idx = np.empty((num_tables, num_bands), dtype=np.int32)
    seeds = np.empty(num_tables, dtype=np.int64)
    for t in range(num_tables):
        idx[t] = rng.choice(sketch_size, size=num_bands, replace=False).astype(np.int32)
        seeds[t] = int(rng.randint(0, 2**31))
    return idx, seeds


def bucket_ids(sketches: np.ndarray, band_idx: np.ndarray, seed: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        h = np.full(sketches.shape[0], np.uint64(seed), dtype=np.uint64)
        for b in band_idx:
            h = h * _MUL + sketches[:, int(b)]
        h = (h ^ (h >> _S33)) * _FMIX
        h = h ^ (h >> _S33)
    return h


_TRIU = {}


def _triu(r: int):
    t = _TRIU.get(r)
    if t is None:
        t = np.triu_indices(r, 1)
        _TRIU[r] = t
    return t


def _pairs_from_sorted(order: np.ndarray, sorted_ids: np.ndarray, n: int) -> np.ndarray:
    if sorted_ids.shape[0] < 2:
        return np.empty(0, np.int64)
    brk = np.nonzero(sorted_ids[1:] != sorted_ids[:-1])[0] + 1
    starts = np.concatenate([[0], brk])
    ends = np.concatenate([brk, [sorted_ids.shape[0]]])
    sizes = np.minimum(ends - starts, MAX_BUCKET)
    keep = sizes >= 2
    starts, sizes = starts[keep], sizes[keep]
    if starts.size == 0:
        return np.empty(0, np.int64)
    out = []
    order64 = order.astype(np.int64)
    for r in np.unique(sizes):
        st = starts[sizes == r]
        a, b = _triu(int(r))
        x = order64[st[:, None] + a[None, :]].ravel()
        y = order64[st[:, None] + b[None, :]].ravel()
        lo = np.minimum(x, y)
        hi = np.maximum(x, y)
        out.append(lo * np.int64(n) + hi)
    return np.concatenate(out)


def lsh_candidates(sketches: np.ndarray, num_tables: int, num_bands: int, seed: int = 42) -> np.ndarray:
    """(M, 2) int32 de-duplicated candidate pairs with i < j (clustkit/lsh.py:93-178)."""
    sketches = np.ascontiguousarray(sketches, dtype=np.uint64)
    n, s = sketches.shape
    if n < 2:
        return np.empty((0, 2), dtype=np.int32)
    idx, seeds = band_parameters(s, num_tables, num_bands, seed)
    packed = []
    for t in range(num_tables):
        ids = bucket_ids(sketches, idx[t], int(np.uint64(seeds[t])))
        order = np.argsort(ids)
        p = _pairs_from_sorted(order, ids[order], n)
        if p.size:
            packed.append(p)
    if not packed:
        return np.empty((0, 2), dtype=np.int32)
    allp = np.unique(np.concatenate(packed))
    pairs = np.empty((allp.shape[0], 2), dtype=np.int32)
    pairs[:, 0] = (allp // n).astype(np.int32)
    pairs[:, 1] = (allp % n).astype(np.int32)
    return pairs


def lsh_candidates_device(sketches, num_tables: int, num_bands: int, seed: int = 42, ctx: int = 0):
    """(M, 2) int32 torch tensor on the sketches' device: the de-duplicated
    candidate pairs (i < j, sorted), computed on the GPU.  ``sketches`` is a
    uint64 numpy array or an int64/uint64-bit torch CUDA tensor [N, s]."""
    import torch

    from . import _lib
    lib = _lib.load()
    _lib.require_gpu()
    if isinstance(sketches, np.ndarray):
        sk = torch.from_numpy(np.ascontiguousarray(sketches, np.uint64).view(np.int64)).cuda()
    else:
        sk = sketches.contiguous()
    n, s = int(sk.shape[0]), int(sk.shape[1])
    idx, seeds = band_parameters(s, num_tables, num_bands, seed)
    idx = np.ascontiguousarray(idx, np.int32)
    seeds_u = np.ascontiguousarray(seeds.astype(np.uint64))
    stream = torch.cuda.current_stream(sk.device).cuda_stream
    # room for tables x N pairs (each sequence in one multi-member bucket per
    # table), within a quarter of the free device memory: a call that finds
    # more reports the count, and is repeated once with room for all of them
    free_bytes, _ = torch.cuda.mem_get_info(sk.device)
    cap = max(min(num_tables * n, free_bytes // 32), 1 << 20)
    count = np.zeros(1, np.int64)
    for _ in range(2):
        out = torch.empty((cap, 2), dtype=torch.int32, device=sk.device)
        st = lib.ck_lsh_candidates_device(ctx, sk.data_ptr(), n, s, num_tables, num_bands, idx.ctypes.data,
                                          seeds_u.ctypes.data, out.data_ptr(), cap, count.ctypes.data, stream)
        if st == _lib.CK_ERR_OUT_OF_MEMORY and int(count[0]) > cap:
            cap = int(count[0])
            continue
        _lib.check(st)
        return out[: int(count[0])]
    raise _lib.CkError(_lib.CK_ERR_OUT_OF_MEMORY, "LSH output did not fit after resizing")


def auto_lsh_params(threshold: float, sensitivity: str, k: int = 5) -> dict:
    """clustkit/utils.py:99-141."""
    import math
    target_miss = {"low": 0.05, "medium": 0.01, "high": 0.001}.get(sensitivity, 0.01)
    J = max(threshold ** k, 1e-9)
    b = 1 if J < 0.15 else (2 if J < 0.5 else 3)
    cp = min(J ** b, 1.0 - 1e-12)
    L = math.ceil(math.log(target_miss) / math.log(1.0 - cp))
    return {"num_tables": max(8, min(L, 512)), "num_bands": b}
