// lsh.cu -- LSH candidate pairs from MinHash sketches on the device.
//
// Same pairs as clustkit/lsh.py:20-178: for every table t a bucket id per
// sequence, h = seed_t; h = h * 0x517CC1B727220A95 + sketch[band index] over
// the table's band, then h = (h ^ h >> 33) * 0xC4CEB9FE1A85EC53, h ^= h >> 33
// (wrapping uint64); sequences are ordered by bucket id, every bucket
// contributes all pairs among its first 1000 members, and the pairs of all
// tables, packed as lo * N + hi (lo < hi), are sorted and de-duplicated.
//
// Tie order inside a bucket: clustkit orders a table with numpy's argsort
// (an unstable introsort); here the radix sort is stable, so a bucket's
// members come in ascending sequence id.  The two agree on every bucket of at
// most 1000 members (all pairs of such a bucket are taken in either order);
// in a larger bucket clustkit keeps whichever 1000 members its sort happens to
// put first, and this keeps the 1000 lowest ids.
//
// Layout: sketches are transposed once to [s][N] so a table's band columns are
// read coalesced.  Two passes over the tables -- count, then emit -- size the
// raw pair buffer exactly; one radix sort + unique de-duplicates all tables.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include <cmath>
#include <vector>

#include "ck_common.cuh"

namespace ck {

constexpr uint64_t LSH_MUL = 0x517CC1B727220A95ull;
constexpr uint64_t LSH_FMIX = 0xC4CEB9FE1A85EC53ull;
constexpr int32_t LSH_MAX_BUCKET = 1000;

__global__ void transpose_sketch_kernel(const uint64_t *__restrict__ sk, int64_t n, int32_t s,
                                        uint64_t *__restrict__ skT) {
    // 32 x 32 tiles through shared memory: reads along s, writes along n
    __shared__ uint64_t tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32;
    const int32_t c0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = i0 + r;
        const int32_t c = c0 + threadIdx.x;
        if (i < n && c < s) tile[r][threadIdx.x] = sk[i * s + c];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int32_t c = c0 + r;
        const int64_t i = i0 + threadIdx.x;
        if (i < n && c < s) skT[(int64_t)c * n + i] = tile[threadIdx.x][r];
    }
}

__global__ void lsh_hash_kernel(const uint64_t *__restrict__ skT, int64_t n, const int32_t *__restrict__ band,
                                int32_t nb, uint64_t seed, uint64_t *__restrict__ keys,
                                int32_t *__restrict__ vals) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t h = seed;
        for (int32_t b = 0; b < nb; ++b) h = h * LSH_MUL + skT[(int64_t)band[b] * n + i];
        h = (h ^ (h >> 33)) * LSH_FMIX;
        h ^= h >> 33;
        keys[i] = h;
        vals[i] = (int32_t)i;
    }
}

// pairs a bucket of `count` members contributes (first 1000 only)
__global__ void lsh_bucket_pairs_kernel(const int32_t *__restrict__ counts, const int32_t *__restrict__ n_runs,
                                        int64_t n, int64_t *__restrict__ npairs) {
    const int32_t R = *n_runs;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= n; r += (int64_t)gridDim.x * blockDim.x) {
        if (r >= R) { npairs[r] = 0; continue; }
        const int64_t c = counts[r] < LSH_MAX_BUCKET ? counts[r] : LSH_MAX_BUCKET;
        npairs[r] = c >= 2 ? c * (c - 1) / 2 : 0;
    }
}

// one thread per output pair: find its bucket (binary search over the pair
// offsets), decode its (x < y) member positions from the triangular index
__global__ void lsh_emit_kernel(const int32_t *__restrict__ order, const int32_t *__restrict__ run_start,
                                const int64_t *__restrict__ pair_off, const int32_t *__restrict__ n_runs,
                                int64_t total, int64_t n, uint64_t *__restrict__ out) {
    const int32_t R = *n_runs;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (int64_t)gridDim.x * blockDim.x) {
        int32_t lo = 0, hi = R - 1;  // last run with pair_off <= k
        while (lo < hi) {
            const int32_t mid = (lo + hi + 1) >> 1;
            if (pair_off[mid] <= k) lo = mid; else hi = mid - 1;
        }
        const int64_t u = k - pair_off[lo];
        int64_t y = (int64_t)((1.0 + sqrt(1.0 + 8.0 * (double)u)) * 0.5);
        while (y * (y - 1) / 2 > u) --y;
        while ((y + 1) * y / 2 <= u) ++y;
        const int64_t x = u - y * (y - 1) / 2;
        const int64_t a = order[run_start[lo] + x], b = order[run_start[lo] + y];
        out[k] = a < b ? (uint64_t)(a * n + b) : (uint64_t)(b * n + a);
    }
}

__global__ void lsh_unpack_kernel(const uint64_t *__restrict__ keys, int64_t m, int64_t n,
                                  int32_t *__restrict__ pairs) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
        pairs[2 * k] = (int32_t)(keys[k] / (uint64_t)n);
        pairs[2 * k + 1] = (int32_t)(keys[k] % (uint64_t)n);
    }
}

static int grid_of(int64_t work, int threads) {
    int64_t b = (work + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count() * 32;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

struct LshArgs {
    const uint64_t *sk; int64_t n; int32_t s; int32_t tables, bands;
    const int32_t *band_idx_host; const uint64_t *seeds_host;
    int32_t *out_pairs; int64_t capacity; int64_t *out_count; cudaStream_t st;
};

static int32_t lsh_impl(void *pv) {
    LshArgs &a = *(LshArgs *)pv;
    int32_t status = CK_OK;
    const int64_t n = a.n;
    cudaStream_t st = a.st;
    *a.out_count = 0;
    if (n < 2 || a.tables == 0) return CK_OK;
    // band indices on the device
    int32_t *d_band = (int32_t *)scratch(SLOT_SEARCH_TMP0, (size_t)a.tables * a.bands * 4, &status);
    uint64_t *skT = (uint64_t *)scratch(SLOT_SEARCH_TMP1, (size_t)n * a.s * 8, &status);
    uint64_t *k0 = (uint64_t *)scratch(SLOT_SEARCH_TMP2, (size_t)n * 8 * 2, &status);
    int32_t *v0 = (int32_t *)scratch(SLOT_SEARCH_TMP3, (size_t)n * 4 * 2, &status);
    // run-length outputs: unique keys (discarded), counts, run count, starts, pair offsets
    char *rle = (char *)scratch(SLOT_SEARCH_TMP4, (size_t)n * (8 + 4 + 4 + 8) + 64, &status);
    if (!d_band || !skT || !k0 || !v0 || !rle) return status;
    uint64_t *k1 = k0 + n;
    int32_t *v1 = v0 + n;
    uint64_t *uniq = (uint64_t *)rle;
    int32_t *counts = (int32_t *)(uniq + n);
    int32_t *starts = counts + n;
    int64_t *pair_off = (int64_t *)(starts + n);  // n + 1 entries: 8-byte aligned (n*16 bytes before)
    int32_t *n_runs = (int32_t *)scratch(SLOT_MAXLEN, 64, &status);
    if (!n_runs) return status;
    CK_CUDA(cudaMemcpyAsync(d_band, a.band_idx_host, (size_t)a.tables * a.bands * 4, cudaMemcpyHostToDevice, st));
    {
        dim3 grid((unsigned)((n + 31) / 32), (unsigned)((a.s + 31) / 32));
        transpose_sketch_kernel<<<grid, dim3(32, 8), 0, st>>>(a.sk, n, a.s, skT);
        CK_CUDA(cudaGetLastError());
    }
    // temp storage sizes (the largest of the calls below)
    size_t t_sort = 0, t_rle = 0, t_scan = 0, t_scan2 = 0;
    {
        cub::DoubleBuffer<uint64_t> dk(k0, k1);
        cub::DoubleBuffer<int32_t> dv(v0, v1);
        CK_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, t_sort, dk, dv, (int)n, 0, 64, st));
        CK_CUDA(cub::DeviceRunLengthEncode::Encode(nullptr, t_rle, k0, uniq, counts, n_runs, (int)n, st));
        CK_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t_scan, counts, starts, (int)n, st));
        CK_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t_scan2, pair_off, pair_off, (int)n + 1, st));
    }
    const size_t t_max = std::max(std::max(t_sort, t_rle), std::max(t_scan, t_scan2));
    void *tmp = scratch(SLOT_SORT_TEMP, t_max, &status);
    if (!tmp) return status;

    // one table: bucket ids, stable sort, runs, pair offsets; returns the pair total
    auto table = [&](int32_t t, cub::DoubleBuffer<uint64_t> &dk, cub::DoubleBuffer<int32_t> &dv,
                     int64_t *total) -> int32_t {
        lsh_hash_kernel<<<grid_of(n, 256), 256, 0, st>>>(skT, n, d_band + (size_t)t * a.bands, a.bands,
                                                         a.seeds_host[t], dk.Current(), dv.Current());
        CK_CUDA(cudaGetLastError());
        size_t tb = t_max;
        CK_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, dk, dv, (int)n, 0, 64, st));
        tb = t_max;
        CK_CUDA(cub::DeviceRunLengthEncode::Encode(tmp, tb, dk.Current(), uniq, counts, n_runs, (int)n, st));
        tb = t_max;
        CK_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, counts, starts, (int)n, st));
        lsh_bucket_pairs_kernel<<<grid_of(n + 1, 256), 256, 0, st>>>(counts, n_runs, n, pair_off);
        CK_CUDA(cudaGetLastError());
        tb = t_max;
        CK_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, pair_off, pair_off, (int)n + 1, st));
        // pair_off[R] (R = runs) is the table's total; runs <= n, entries past R are 0
        int32_t R = 0;
        CK_CUDA(cudaMemcpyAsync(&R, n_runs, 4, cudaMemcpyDeviceToHost, st));
        CK_CUDA(cudaStreamSynchronize(st));
        CK_CUDA(cudaMemcpyAsync(total, pair_off + R, 8, cudaMemcpyDeviceToHost, st));
        CK_CUDA(cudaStreamSynchronize(st));
        return CK_OK;
    };

    // pass 1: count every table's pairs
    std::vector<int64_t> per_table((size_t)a.tables, 0);
    int64_t raw = 0;
    for (int32_t t = 0; t < a.tables; ++t) {
        cub::DoubleBuffer<uint64_t> dk(k0, k1);
        cub::DoubleBuffer<int32_t> dv(v0, v1);
        CK_TRY(table(t, dk, dv, &per_table[t]));
        raw += per_table[t];
    }
    if (raw == 0) return CK_OK;
    // pass 2: emit into one raw buffer (double, for the de-duplicating sort)
    uint64_t *rk = (uint64_t *)scratch(SLOT_FALLBACK, (size_t)raw * 8 * 2, &status);
    if (!rk) return status;
    int64_t at = 0;
    for (int32_t t = 0; t < a.tables; ++t) {
        if (per_table[t] == 0) continue;
        cub::DoubleBuffer<uint64_t> dk(k0, k1);
        cub::DoubleBuffer<int32_t> dv(v0, v1);
        int64_t tot = 0;
        CK_TRY(table(t, dk, dv, &tot));
        lsh_emit_kernel<<<grid_of(tot, 256), 256, 0, st>>>(dv.Current(), starts, pair_off, n_runs, tot, n,
                                                           rk + at);
        CK_CUDA(cudaGetLastError());
        at += tot;
    }
    // de-duplicate: sort packed keys (enough bits for n * n), unique
    int bits = 1;
    while (bits < 64 && ((uint64_t)1 << bits) <= (uint64_t)n * (uint64_t)n) ++bits;
    cub::DoubleBuffer<uint64_t> rb(rk, rk + raw);
    size_t ts = 0, tu = 0;
    CK_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, ts, rb, raw, 0, bits, st));
    uint64_t *uq = rb.Alternate();
    int64_t *n_uniq = (int64_t *)(n_runs + 2);
    CK_CUDA(cub::DeviceSelect::Unique(nullptr, tu, rk, uq, n_uniq, raw, st));
    void *tmp2 = scratch(SLOT_SORT_TEMP, std::max(ts, tu), &status);
    if (!tmp2) return status;
    CK_CUDA(cub::DeviceRadixSort::SortKeys(tmp2, ts, rb, raw, 0, bits, st));
    size_t tu2 = std::max(ts, tu);
    CK_CUDA(cub::DeviceSelect::Unique(tmp2, tu2, rb.Current(), rb.Alternate(), n_uniq, raw, st));
    int64_t m = 0;
    CK_CUDA(cudaMemcpyAsync(&m, n_uniq, 8, cudaMemcpyDeviceToHost, st));
    CK_CUDA(cudaStreamSynchronize(st));
    *a.out_count = m;
    if (m > a.capacity) {
        set_error(CK_ERR_OUT_OF_MEMORY, "LSH: more candidate pairs than the output capacity (count returned)");
        return CK_ERR_OUT_OF_MEMORY;
    }
    lsh_unpack_kernel<<<grid_of(m, 256), 256, 0, st>>>(rb.Alternate(), m, n, a.out_pairs);
    CK_CUDA(cudaGetLastError());
    CK_CUDA(cudaStreamSynchronize(st));
    return CK_OK;
}

}  // namespace ck

using namespace ck;

extern "C" int32_t ck_lsh_candidates_device(int32_t ctx, const uint64_t *d_sketches, int64_t n, int32_t s,
                                            int32_t num_tables, int32_t num_bands,
                                            const int32_t *band_idx_host, const uint64_t *seeds_host,
                                            int32_t *d_out_pairs, int64_t capacity, int64_t *out_count,
                                            void *stream) {
    std::lock_guard<std::mutex> lock(library_mutex());
    reset_thread_status();
    if (!out_count || n < 0 || n >= ((int64_t)1 << 31) || s < 1 || num_tables < 0 || num_bands < 1 ||
        num_bands > s || capacity < 0 || (n > 0 && !d_sketches) || (num_tables > 0 && (!band_idx_host || !seeds_host)) ||
        (capacity > 0 && !d_out_pairs)) {
        set_error(CK_ERR_INVALID_ARGUMENT, "LSH: bad arguments");
        return CK_ERR_INVALID_ARGUMENT;
    }
    for (int64_t i = 0; i < (int64_t)num_tables * num_bands; ++i)
        if (band_idx_host[i] < 0 || band_idx_host[i] >= s) {
            set_error(CK_ERR_OUT_OF_RANGE, "LSH: band index outside the sketch");
            return CK_ERR_OUT_OF_RANGE;
        }
    LshArgs a{d_sketches, n, s, num_tables, num_bands, band_idx_host, seeds_host, d_out_pairs, capacity,
              out_count, (cudaStream_t)stream};
    return run_in_context(ctx, lsh_impl, &a);
}
