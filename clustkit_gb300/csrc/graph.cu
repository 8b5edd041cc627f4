// graph.cu -- similarity graph (CSR) and connected components on the device.
//
// Graph (clustkit/graph.py:7-39): the edges (i, j) and (j, i) of every
// passing pair with its identity as weight, in CSR form with the columns of
// each row ascending and repeated (row, column) entries summed -- scipy's
// canonical form after coo_matrix(...).tocsr().  Built by one radix sort of
// (row << 32 | column) keys with their weights, a reduce-by-key for the
// duplicates and a histogram + scan of the rows for the row pointers.
//
// Connected components (clustkit/cluster.py:43-55, scipy's
// connected_components on the undirected graph): union-find over the edge
// list.  Rounds of "hook" (an edge whose endpoints have different roots links
// the larger root under the smaller with atomicMin, so a root's parent only
// ever decreases) and "compress" (pointer jumping) run until no edge joins two
// roots; every component's root is then its smallest node.  scipy numbers
// components in order of their smallest node, so a node's label is the number
// of roots below its root.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>

#include "ck_common.cuh"

namespace ck {

struct FAdd {
    __device__ __forceinline__ float operator()(float x, float y) const { return x + y; }
};

static int grid_n(int64_t work, int threads) {
    int64_t b = (work + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count() * 32;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

__global__ void graph_edges_kernel(const int32_t *__restrict__ pairs, const float *__restrict__ sims, int64_t K,
                                   int64_t N, uint64_t *__restrict__ keys, float *__restrict__ w,
                                   int32_t *err) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < K; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = pairs[2 * e], j = pairs[2 * e + 1];
        if (i < 0 || j < 0 || i >= N || j >= N) {
            atomicOr(err, ERRBIT_PAIR_INDEX);
            i = j = 0;  // harmless placeholder; the call reports the error
        }
        keys[e] = ((uint64_t)i << 32) | (uint64_t)j;
        keys[K + e] = ((uint64_t)j << 32) | (uint64_t)i;
        const float s = sims ? sims[e] : 1.0f;
        w[e] = s;
        w[K + e] = s;
    }
}

__global__ void graph_rows_kernel(const uint64_t *__restrict__ ukeys, const int64_t *__restrict__ nnz_p,
                                  int32_t *__restrict__ indices, int64_t *__restrict__ row_count) {
    const int64_t nnz = *nnz_p;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = ukeys[e];
        indices[e] = (int32_t)(k & 0xffffffffu);
        atomicAdd((unsigned long long *)&row_count[k >> 32], 1ull);
    }
}

struct GraphArgs {
    const int32_t *pairs; const float *sims; int64_t K, N;
    int64_t *indptr; int32_t *indices; float *data; int64_t *out_nnz; cudaStream_t st;
};

static int32_t graph_impl(void *pv) {
    GraphArgs &a = *(GraphArgs *)pv;
    int32_t status = CK_OK;
    cudaStream_t st = a.st;
    int32_t *err = device_error_word(&status);
    if (!err) return status;
    const int64_t E = 2 * a.K;
    CK_CUDA(cudaMemsetAsync(a.indptr, 0, (size_t)(a.N + 1) * 8, st));
    *a.out_nnz = 0;
    if (E == 0) return CK_OK;
    uint64_t *keys = (uint64_t *)scratch(SLOT_SEARCH_TMP1, (size_t)E * 8 * 2, &status);
    float *w = (float *)scratch(SLOT_SEARCH_TMP2, (size_t)E * 4 * 2, &status);
    int64_t *nnz_d = (int64_t *)scratch(SLOT_MAXLEN, 64, &status);
    if (!keys || !w || !nnz_d) return status;
    graph_edges_kernel<<<grid_n(a.K, 256), 256, 0, st>>>(a.pairs, a.sims, a.K, a.N, keys, w, err);
    CK_CUDA(cudaGetLastError());
    int bits = 33;
    while (bits < 64 && ((uint64_t)1 << (bits - 32)) <= (uint64_t)a.N) ++bits;
    cub::DoubleBuffer<uint64_t> dk(keys, keys + E);
    cub::DoubleBuffer<float> dv(w, w + E);
    size_t t1 = 0, t2 = 0;
    CK_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, t1, dk, dv, E, 0, bits, st));
    CK_CUDA(cub::DeviceReduce::ReduceByKey(nullptr, t2, dk.Current(), dk.Alternate(), dv.Current(), a.data,
                                           nnz_d, FAdd(), E, st));
    void *tmp = scratch(SLOT_SORT_TEMP, std::max(t1, t2), &status);
    if (!tmp) return status;
    CK_CUDA(cub::DeviceRadixSort::SortPairs(tmp, t1, dk, dv, E, 0, bits, st));
    // unique keys into the alternate key buffer, summed weights straight into data
    size_t tt = std::max(t1, t2);
    CK_CUDA(cub::DeviceReduce::ReduceByKey(tmp, tt, dk.Current(), dk.Alternate(), dv.Current(), a.data, nnz_d,
                                           FAdd(), E, st));
    graph_rows_kernel<<<grid_n(E, 256), 256, 0, st>>>(dk.Alternate(), nnz_d, a.indices, a.indptr + 1);
    CK_CUDA(cudaGetLastError());
    size_t ts = 0;
    CK_CUDA(cub::DeviceScan::InclusiveSum(nullptr, ts, a.indptr + 1, a.indptr + 1, a.N, st));
    void *tmp2 = scratch(SLOT_SORT_TEMP, std::max(std::max(t1, t2), ts), &status);
    if (!tmp2) return status;
    CK_CUDA(cub::DeviceScan::InclusiveSum(tmp2, ts, a.indptr + 1, a.indptr + 1, a.N, st));
    int32_t h = 0;
    CK_CUDA(cudaMemcpyAsync(a.out_nnz, nnz_d, 8, cudaMemcpyDeviceToHost, st));
    CK_CUDA(cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, st));
    CK_CUDA(cudaMemsetAsync(err, 0, 4, st));
    CK_CUDA(cudaStreamSynchronize(st));
    if (h) {
        set_error(CK_ERR_OUT_OF_RANGE, "graph: pair index outside [0, N)");
        return CK_ERR_OUT_OF_RANGE;
    }
    return CK_OK;
}

// ------------------------------------------------------------ components
__device__ __forceinline__ int32_t uf_find(const int32_t *parent, int32_t x) {
    int32_t p = parent[x];
    while (p != x) {
        x = p;
        p = parent[x];
    }
    return x;
}

__global__ void cc_init_kernel(int32_t *parent, int64_t N) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
        parent[i] = (int32_t)i;
}

__global__ void cc_hook_kernel(const int32_t *__restrict__ pairs, int64_t K, int64_t N, int32_t *parent,
                               int32_t *changed, int32_t *err) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < K; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = pairs[2 * e], v = pairs[2 * e + 1];
        if (u < 0 || v < 0 || u >= N || v >= N) {
            atomicOr(err, ERRBIT_PAIR_INDEX);
            continue;
        }
        const int32_t ru = uf_find(parent, u), rv = uf_find(parent, v);
        if (ru == rv) continue;
        const int32_t hi = ru > rv ? ru : rv, lo = ru ^ rv ^ hi;
        atomicMin(&parent[hi], lo);
        *changed = 1;
    }
}

__global__ void cc_compress_kernel(int32_t *parent, int64_t N) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
        parent[i] = uf_find(parent, (int32_t)i);
}

__global__ void cc_root_flags_kernel(const int32_t *parent, int64_t N, int32_t *flag) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = parent[i] == (int32_t)i ? 1 : 0;
}

__global__ void cc_label_kernel(const int32_t *parent, const int32_t *rank, int64_t N, int32_t *labels) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
        labels[i] = rank[parent[i]];
}

struct CcArgs {
    const int32_t *pairs; int64_t K, N; int32_t *labels; int64_t *out_n; int32_t *out_rounds; cudaStream_t st;
};

static int32_t cc_impl(void *pv) {
    CcArgs &a = *(CcArgs *)pv;
    int32_t status = CK_OK;
    cudaStream_t st = a.st;
    *a.out_n = 0;
    if (a.out_rounds) *a.out_rounds = 0;
    if (a.N == 0) return CK_OK;
    int32_t *err = device_error_word(&status);
    int32_t *parent = (int32_t *)scratch(SLOT_SEARCH_TMP3, (size_t)a.N * 4 * 2 + 8, &status);
    int32_t *flags = (int32_t *)scratch(SLOT_MAXLEN, 64, &status);
    if (!err || !parent || !flags) return status;
    int32_t *rank = parent + a.N;
    int32_t *changed = flags;
    cc_init_kernel<<<grid_n(a.N, 256), 256, 0, st>>>(parent, a.N);
    CK_CUDA(cudaGetLastError());
    // a round in which some edge still joins two roots lowers at least one
    // root's parent, so at most N rounds can report a change (in practice a
    // handful: hooking merges most trees of a component per round)
    int32_t rounds = 0, h = 1;
    while (h && a.K > 0) {
        if ((int64_t)rounds > a.N + 1) {
            set_error(CK_ERR_CUDA, "connected components did not converge");
            return CK_ERR_CUDA;
        }
        CK_CUDA(cudaMemsetAsync(changed, 0, 4, st));
        cc_hook_kernel<<<grid_n(a.K, 256), 256, 0, st>>>(a.pairs, a.K, a.N, parent, changed, err);
        CK_CUDA(cudaGetLastError());
        cc_compress_kernel<<<grid_n(a.N, 256), 256, 0, st>>>(parent, a.N);
        CK_CUDA(cudaGetLastError());
        CK_CUDA(cudaMemcpyAsync(&h, changed, 4, cudaMemcpyDeviceToHost, st));
        CK_CUDA(cudaStreamSynchronize(st));
        ++rounds;
    }
    int32_t e_h = 0;
    CK_CUDA(cudaMemcpyAsync(&e_h, err, 4, cudaMemcpyDeviceToHost, st));
    CK_CUDA(cudaMemsetAsync(err, 0, 4, st));
    CK_CUDA(cudaStreamSynchronize(st));
    if (e_h) {
        set_error(CK_ERR_OUT_OF_RANGE, "components: pair index outside [0, N)");
        return CK_ERR_OUT_OF_RANGE;
    }
    cc_root_flags_kernel<<<grid_n(a.N, 256), 256, 0, st>>>(parent, a.N, a.labels);
    CK_CUDA(cudaGetLastError());
    size_t ts = 0;
    CK_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, ts, a.labels, rank, a.N, st));
    void *tmp = scratch(SLOT_SORT_TEMP, ts, &status);
    if (!tmp) return status;
    CK_CUDA(cub::DeviceScan::ExclusiveSum(tmp, ts, a.labels, rank, a.N, st));
    int32_t last_flag = 0, last_rank = 0;
    CK_CUDA(cudaMemcpyAsync(&last_flag, a.labels + a.N - 1, 4, cudaMemcpyDeviceToHost, st));
    CK_CUDA(cudaMemcpyAsync(&last_rank, rank + a.N - 1, 4, cudaMemcpyDeviceToHost, st));
    cc_label_kernel<<<grid_n(a.N, 256), 256, 0, st>>>(parent, rank, a.N, a.labels);
    CK_CUDA(cudaGetLastError());
    CK_CUDA(cudaStreamSynchronize(st));
    *a.out_n = (int64_t)last_rank + last_flag;
    if (a.out_rounds) *a.out_rounds = rounds;
    return CK_OK;
}

}  // namespace ck

using namespace ck;

extern "C" int32_t ck_graph_csr_device(int32_t ctx, const int32_t *d_pairs, const float *d_sims, int64_t K,
                                       int64_t N, int64_t *d_indptr, int32_t *d_indices, float *d_data,
                                       int64_t *out_nnz, void *stream) {
    std::lock_guard<std::mutex> lock(library_mutex());
    reset_thread_status();
    if (K < 0 || N < 0 || N >= ((int64_t)1 << 31) || !out_nnz || !d_indptr ||
        (K > 0 && (!d_pairs || !d_indices || !d_data))) {
        set_error(CK_ERR_INVALID_ARGUMENT, "graph: bad arguments");
        return CK_ERR_INVALID_ARGUMENT;
    }
    GraphArgs a{d_pairs, d_sims, K, N, d_indptr, d_indices, d_data, out_nnz, (cudaStream_t)stream};
    return run_in_context(ctx, graph_impl, &a);
}

extern "C" int32_t ck_connected_components_device(int32_t ctx, const int32_t *d_pairs, int64_t K, int64_t N,
                                                  int32_t *d_labels, int64_t *out_n_components,
                                                  int32_t *out_rounds, void *stream) {
    std::lock_guard<std::mutex> lock(library_mutex());
    reset_thread_status();
    if (K < 0 || N < 0 || N >= ((int64_t)1 << 31) || !out_n_components || (N > 0 && !d_labels) ||
        (K > 0 && !d_pairs)) {
        set_error(CK_ERR_INVALID_ARGUMENT, "components: bad arguments");
        return CK_ERR_INVALID_ARGUMENT;
    }
    CcArgs a{d_pairs, K, N, d_labels, out_n_components, out_rounds, (cudaStream_t)stream};
    return run_in_context(ctx, cc_impl, &a);
}
