"""CPU restatement of clustkit's graph construction and connected components.

TEST INFRASTRUCTURE ONLY -- the checker for clustkit_gb300.graph.  Reference
paths are relative to the clustkit project root.

* ``build_similarity_graph``       -- clustkit/graph.py:7-39 (scipy COO -> CSR)
* ``cluster_connected_components`` -- clustkit/cluster.py:43-55 (scipy)
"""
from __future__ import annotations

import numpy as np
from scipy import sparse


def build_similarity_graph(num_sequences, filtered_pairs, similarities):
    if len(filtered_pairs) == 0:
        return sparse.csr_matrix((num_sequences, num_sequences), dtype=np.float32)
    rows, cols = filtered_pairs[:, 0], filtered_pairs[:, 1]
    all_rows = np.concatenate([rows, cols])
    all_cols = np.concatenate([cols, rows])
    all_data = np.concatenate([similarities, similarities])
    g = sparse.coo_matrix((all_data, (all_rows, all_cols)), shape=(num_sequences, num_sequences),
                          dtype=np.float32)
    return g.tocsr()


def cluster_connected_components(graph):
    _, labels = sparse.csgraph.connected_components(graph, directed=False, return_labels=True)
    return labels.astype(np.int32)
