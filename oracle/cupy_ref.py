"""The reference's CuPy GPU path, run without CuPy.

BASELINE AND TEST INFRASTRUCTURE ONLY: bench.py times it as the reference's GPU
baseline beside the CPU baseline; nothing in the product calls it.

The kernel is clustkit's own CuPy source (clustkit/pairwise.py:1215-1402),
compiled from the reference checkout into oracle/_ref/sw_cupy_ref.cubin by
oracle/build.py.  This module loads that cubin through the CUDA driver API
(ctypes on libcuda) and restates the host side of
``_compute_pairwise_alignment_gpu`` (clustkit/pairwise.py:1480-1547): pairs
sorted by their longer length (mergesort), per-pair band width (the longer
length when it is <= 50), batches of 500,000 pairs, threads per block sized to
fill ``sharedMemPerBlock`` with 8 x (2 * batch max band + 3) int32 per thread
(rounded down to a multiple of 32 when that leaves any), one launch per batch.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

CUBIN = Path(__file__).resolve().parent / "_ref" / "sw_cupy_ref.cubin"
CU_DEVICE_ATTRIBUTE_MAX_SHARED_MEMORY_PER_BLOCK = 8
BATCH = 500_000


def available() -> bool:
    return CUBIN.exists()


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with CUDA driver error {rc}")


class CupyPathKernel:
    """clustkit's CuPy SW kernel with its host batching, on the current torch device."""

    def __init__(self):
        import torch
        self.torch = torch
        torch.zeros(1, device="cuda")  # the runtime's primary context, current on this thread
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._image = CUBIN.read_bytes()
        self.mod = ctypes.c_void_p()
        _check(self.cu.cuModuleLoadData(ctypes.byref(self.mod), ctypes.c_char_p(self._image)), "cuModuleLoadData")
        self.fn = ctypes.c_void_p()
        _check(self.cu.cuModuleGetFunction(ctypes.byref(self.fn), self.mod, b"sw_align_kernel"),
               "cuModuleGetFunction")
        dev = ctypes.c_int()
        _check(self.cu.cuCtxGetDevice(ctypes.byref(dev)), "cuCtxGetDevice")
        smem = ctypes.c_int()
        _check(self.cu.cuDeviceGetAttribute(ctypes.byref(smem), CU_DEVICE_ATTRIBUTE_MAX_SHARED_MEMORY_PER_BLOCK,
                                            dev), "cuDeviceGetAttribute")
        self.smem_per_block = int(smem.value)

    def prepare(self, pairs, lengths, band_width, sub_matrix):
        """Host-side sort and batch plan; uploads the sorted pairs.  Returns a plan.

        Band widths below 50 are refused: there clustkit's batching sizes a
        batch's per-thread workspace from its last pair's band while earlier
        short pairs use their full length as band, overrunning the workspace
        (its shared-memory overflow); this baseline runs only where it is sound."""
        if band_width < 50:
            raise ValueError("the reference CuPy path is only sound for band widths >= 50")
        torch = self.torch
        pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        lengths = np.asarray(lengths)
        m = len(pairs)
        max_lens = np.maximum(lengths[pairs[:, 0]], lengths[pairs[:, 1]])
        order = np.argsort(max_lens, kind="mergesort")
        sorted_max = max_lens[order]
        eff_bw = np.full(m, band_width, dtype=np.int32)
        short = sorted_max <= 50
        eff_bw[short] = sorted_max[short].astype(np.int32)
        batches = []
        start = 0
        while start < m:
            end = min(start + BATCH, m)
            max_band_cols = 2 * int(eff_bw[end - 1]) + 3
            ws_per_pair = 8 * max_band_cols * 4
            threads = max(1, self.smem_per_block // ws_per_pair)
            threads = max(1, (threads // 32) * 32 or threads)
            batches.append((start, end, max_band_cols, threads))
            start = end
        dev = torch.device("cuda", torch.cuda.current_device())
        d_pairs = torch.from_numpy(pairs[order].copy()).to(dev)
        d_sub = torch.from_numpy(np.ascontiguousarray(sub_matrix, np.int8).reshape(-1).copy()).to(dev)
        d_sims = torch.empty(m, dtype=torch.float32, device=dev)
        d_mask = torch.empty(m, dtype=torch.int32, device=dev)
        return dict(m=m, order=order, batches=batches, d_pairs=d_pairs, d_sub=d_sub, d_sims=d_sims, d_mask=d_mask,
                    band_width=int(band_width))

    def launch(self, plan, d_flat, d_offsets, d_lengths, threshold, stream):
        """One launch per batch, as clustkit issues them, on ``stream`` (a cudaStream_t)."""
        for (b0, b1, max_band_cols, threads) in plan["batches"]:
            bm = b1 - b0
            blocks = (bm + threads - 1) // threads
            smem = threads * 8 * max_band_cols * 4
            args = [ctypes.c_void_p(plan["d_pairs"].data_ptr() + b0 * 8), ctypes.c_void_p(d_flat.data_ptr()),
                    ctypes.c_void_p(d_offsets.data_ptr()), ctypes.c_void_p(d_lengths.data_ptr()),
                    ctypes.c_void_p(plan["d_sub"].data_ptr()), ctypes.c_void_p(plan["d_sims"].data_ptr() + b0 * 4),
                    ctypes.c_void_p(plan["d_mask"].data_ptr() + b0 * 4), ctypes.c_int(bm),
                    ctypes.c_int(max_band_cols), ctypes.c_int(plan["band_width"]), ctypes.c_float(threshold)]
            params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
            _check(self.cu.cuLaunchKernel(self.fn, blocks, 1, 1, threads, 1, 1, smem, ctypes.c_void_p(stream),
                                          params, None), "cuLaunchKernel")

    def results(self, plan):
        """(sims float32, mask bool) in the caller's pair order."""
        sims = np.empty(plan["m"], np.float32)
        mask = np.empty(plan["m"], bool)
        sims[plan["order"]] = plan["d_sims"].cpu().numpy()
        mask[plan["order"]] = plan["d_mask"].cpu().numpy().astype(bool)
        return sims, mask
