"""Similarity graph and connected components on the GPU (the step after Align).

Drop-ins for clustkit's ``build_similarity_graph`` (clustkit/graph.py:7-39)
and ``cluster_connected_components`` (clustkit/cluster.py:43-55): the same
arguments and the same results -- a scipy CSR matrix with scipy's canonical
layout (columns ascending per row, repeated entries summed), and int32
component labels numbered in order of each component's smallest node, as
scipy's ``connected_components`` numbers them.  The work runs in libckgpu.so
(csrc/graph.cu); Leiden and greedy clustering stay with clustkit.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def _torch():
    import torch
    return torch


def graph_csr_device(pairs, sims, num_sequences: int, ctx: int = 0):
    """(indptr int64 [N+1], indices int32, data float32) torch tensors on the GPU."""
    torch = _torch()
    lib = _lib.load()
    _lib.require_gpu()
    dev = torch.device("cuda", torch.cuda.current_device())
    p = pairs if torch.is_tensor(pairs) else torch.from_numpy(np.ascontiguousarray(pairs, np.int32).reshape(-1, 2))
    p = p.to(dev).contiguous()
    K = int(p.shape[0])
    s = None
    if sims is not None:
        s = sims if torch.is_tensor(sims) else torch.from_numpy(np.ascontiguousarray(sims, np.float32))
        s = s.to(dev).contiguous()
    N = int(num_sequences)
    indptr = torch.empty(N + 1, dtype=torch.int64, device=dev)
    indices = torch.empty(max(2 * K, 1), dtype=torch.int32, device=dev)
    data = torch.empty(max(2 * K, 1), dtype=torch.float32, device=dev)
    nnz = np.zeros(1, np.int64)
    st = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(lib.ck_graph_csr_device(ctx, p.data_ptr(), s.data_ptr() if s is not None else None, K, N,
                                       indptr.data_ptr(), indices.data_ptr(), data.data_ptr(), nnz.ctypes.data, st))
    m = int(nnz[0])
    return indptr, indices[:m], data[:m]


def build_similarity_graph(num_sequences: int, filtered_pairs: np.ndarray, similarities: np.ndarray):
    """clustkit/graph.py:7-39 -- (N, N) scipy CSR, symmetric, float32 weights."""
    from scipy import sparse
    n = int(num_sequences)
    if len(filtered_pairs) == 0:
        return sparse.csr_matrix((n, n), dtype=np.float32)
    indptr, indices, data = graph_csr_device(filtered_pairs, similarities, n)
    return sparse.csr_matrix((data.cpu().numpy(), indices.cpu().numpy(), indptr.cpu().numpy()),
                             shape=(n, n))


def connected_components_device(pairs, num_sequences: int, ctx: int = 0):
    """(n_components, labels int32 torch tensor on the GPU, union-find rounds)."""
    torch = _torch()
    lib = _lib.load()
    _lib.require_gpu()
    dev = torch.device("cuda", torch.cuda.current_device())
    p = pairs if torch.is_tensor(pairs) else torch.from_numpy(np.ascontiguousarray(pairs, np.int32).reshape(-1, 2))
    p = p.to(dev).contiguous()
    N = int(num_sequences)
    labels = torch.empty(max(N, 1), dtype=torch.int32, device=dev)
    n_comp = np.zeros(1, np.int64)
    rounds = np.zeros(1, np.int32)
    st = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(lib.ck_connected_components_device(ctx, p.data_ptr(), int(p.shape[0]), N, labels.data_ptr(),
                                                  n_comp.ctypes.data, rounds.ctypes.data, st))
    return int(n_comp[0]), labels[:N], int(rounds[0])


def cluster_connected_components(graph) -> np.ndarray:
    """clustkit/cluster.py:43-55 -- (N,) int32 labels of the graph's components."""
    coo = graph.tocoo()
    pairs = np.stack([coo.row, coo.col], 1).astype(np.int32)
    _, labels, _ = connected_components_device(pairs, graph.shape[0])
    return labels.cpu().numpy()
