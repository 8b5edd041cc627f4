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
// read coalesced.  Tables are processed in batches (as many as fit a few GB of
// scratch; every table at once for moderate N): a batch's bucket ids are keyed
// (table, id) and sorted together, stably, so each bucket is one run in table
// order with its members in ascending sequence id, and the run-length, scan,
// pair-count and emit steps cover the whole batch in one launch each.  Two
// passes over the batches -- count, then emit -- size the raw pair buffer
// exactly; one radix sort + unique de-duplicates all tables.
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

// A batch's sort key: the table (within the batch) above the bucket id.
struct LshKey {
    uint64_t h;  // bucket id in its table
    uint32_t t;  // table, counted from the batch's first
    uint32_t pad;
};
__host__ __device__ inline bool operator==(const LshKey &a, const LshKey &b) { return a.h == b.h && a.t == b.t; }
// radix-sort view of a key: (table, bucket id), most significant first
struct LshKeyParts {
    __host__ __device__ ::cuda::std::tuple<uint32_t &, uint64_t &> operator()(LshKey &k) const { return {k.t, k.h}; }
};

// bucket ids of tables t0 .. t0 + tb - 1 for every sequence, table-major
__global__ void lsh_hash_kernel(const uint64_t *__restrict__ skT, int64_t n, const int32_t *__restrict__ band,
                                int32_t nb, const uint64_t *__restrict__ seeds, int32_t t0, int32_t tb,
                                LshKey *__restrict__ keys, int32_t *__restrict__ vals) {
    const int64_t total = (int64_t)tb * n;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t tl = (int32_t)(k / n);
        const int64_t i = k - (int64_t)tl * n;
        const int32_t t = t0 + tl;
        const int32_t *bt = band + (int64_t)t * nb;
        uint64_t h = seeds[t];
        for (int32_t b = 0; b < nb; ++b) h = h * LSH_MUL + skT[(int64_t)bt[b] * n + i];
        h = (h ^ (h >> 33)) * LSH_FMIX;
        h ^= h >> 33;
        keys[k] = LshKey{h, (uint32_t)tl, 0u};
        vals[k] = (int32_t)i;
    }
}

// the batch's pair total, pair_off[runs], for the host
__global__ void lsh_total_kernel(const int32_t *__restrict__ n_runs, const int64_t *__restrict__ pair_off,
                                 int64_t *__restrict__ total) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *total = pair_off[*n_runs];
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

// Emission by bucket: a thread writes the pairs of a bucket of at most 32
// members (pair (x, y), x < y, at offset y(y - 1) / 2 + x of the bucket's
// range), and lists larger buckets for lsh_emit_big_kernel.  The raw pairs
// are sorted and de-duplicated afterwards, so only the set matters.
constexpr int32_t LSH_SMALL_BUCKET = 32;
__global__ void lsh_emit_runs_kernel(const int32_t *__restrict__ order, const int32_t *__restrict__ run_start,
                                     const int32_t *__restrict__ counts, const int64_t *__restrict__ pair_off,
                                     const int32_t *__restrict__ n_runs, int64_t n, uint64_t *__restrict__ out,
                                     int32_t *__restrict__ big, int32_t *__restrict__ n_big) {
    const int32_t R = *n_runs;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < R; r += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = counts[r] < LSH_MAX_BUCKET ? counts[r] : LSH_MAX_BUCKET;
        if (c < 2) continue;
        if (c > LSH_SMALL_BUCKET) {
            big[atomicAdd(n_big, 1)] = (int32_t)r;
            continue;
        }
        const int32_t s0 = run_start[r];
        uint64_t *o = out + pair_off[r];
        for (int32_t y = 1; y < c; ++y) {
            const int64_t b = order[s0 + y];
            for (int32_t x = 0; x < y; ++x) {
                const int64_t v = order[s0 + x];
                *o++ = v < b ? (uint64_t)(v * n + b) : (uint64_t)(b * n + v);
            }
        }
    }
}

// one warp per listed bucket (more than 32 members, at most 1000 taken): its
// lanes split each member's pairs with the members before it
__global__ void lsh_emit_big_kernel(const int32_t *__restrict__ order, const int32_t *__restrict__ run_start,
                                    const int32_t *__restrict__ counts, const int64_t *__restrict__ pair_off,
                                    const int32_t *__restrict__ big, const int32_t *__restrict__ n_big, int64_t n,
                                    uint64_t *__restrict__ out) {
    const int32_t lane = threadIdx.x & 31;
    const int32_t nb = *n_big;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nb; w += warps) {
        const int32_t r = big[w];
        const int32_t c = counts[r] < LSH_MAX_BUCKET ? counts[r] : LSH_MAX_BUCKET;
        const int32_t s0 = run_start[r];
        uint64_t *o = out + pair_off[r];
        for (int32_t y = 1; y < c; ++y) {
            const int64_t b = order[s0 + y];
            uint64_t *row = o + (int64_t)y * (y - 1) / 2;
            for (int32_t x = lane; x < y; x += 32) {
                const int64_t v = order[s0 + x];
                row[x] = v < b ? (uint64_t)(v * n + b) : (uint64_t)(b * n + v);
            }
        }
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
    // tables per batch: about 4 GB of keys, values and run data (80 B an item),
    // and fewer than 2^31 items (the run-length encoder counts in int)
    int64_t tb64 = ((int64_t)4 << 30) / (80 * n);
    if (tb64 * n > ((int64_t)1 << 30)) tb64 = ((int64_t)1 << 30) / n;
    if (tb64 < 1) tb64 = 1;
    if (tb64 > a.tables) tb64 = a.tables;
    const int32_t TB = (int32_t)tb64;
    const int64_t items = (int64_t)TB * n;
    int tbits = 1;  // bits of a table index within a batch
    while (tbits < 31 && ((int64_t)1 << tbits) < TB) ++tbits;
    // band indices and seeds on the device
    int32_t *d_band = (int32_t *)scratch(SLOT_SEARCH_TMP0, (size_t)a.tables * a.bands * 4 + (size_t)a.tables * 8 + 16,
                                         &status);
    uint64_t *skT = (uint64_t *)scratch(SLOT_SEARCH_TMP1, (size_t)n * a.s * 8, &status);
    LshKey *k0 = (LshKey *)scratch(SLOT_SEARCH_TMP2, (size_t)items * sizeof(LshKey) * 2, &status);
    int32_t *v0 = (int32_t *)scratch(SLOT_SEARCH_TMP3, (size_t)items * 4 * 2, &status);
    // run data: unique keys (unused), counts, starts (int32), pair offsets
    // (int64, items + 1), then the list of buckets of more than 32 members (at
    // most items / 33 of them)
    const int64_t n_big_max = items / (LSH_SMALL_BUCKET + 1) + 1;
    char *rle = (char *)scratch(SLOT_SEARCH_TMP4, (size_t)items * (sizeof(LshKey) + 4 + 4 + 8) + 64 + (size_t)n_big_max * 4,
                                &status);
    int32_t *n_runs = (int32_t *)scratch(SLOT_MAXLEN, 64, &status);
    if (!d_band || !skT || !k0 || !v0 || !rle || !n_runs) return status;
    int32_t *n_big = n_runs + 8;
    uint64_t *d_seeds = (uint64_t *)(((uintptr_t)(d_band + (size_t)a.tables * a.bands) + 15) & ~(uintptr_t)15);
    LshKey *k1 = k0 + items;
    int32_t *v1 = v0 + items;
    LshKey *uniq = (LshKey *)rle;
    int32_t *counts = (int32_t *)(uniq + items);
    int32_t *starts = counts + items;
    int64_t *pair_off = (int64_t *)(starts + items);  // 8-byte aligned: items * 24 bytes before
    int32_t *big = (int32_t *)(pair_off + items + 1);
    int64_t *d_total = (int64_t *)(n_runs + 4);
    CK_CUDA(cudaMemcpyAsync(d_band, a.band_idx_host, (size_t)a.tables * a.bands * 4, cudaMemcpyHostToDevice, st));
    CK_CUDA(cudaMemcpyAsync(d_seeds, a.seeds_host, (size_t)a.tables * 8, cudaMemcpyHostToDevice, st));
    {
        dim3 grid((unsigned)((n + 31) / 32), (unsigned)((a.s + 31) / 32));
        transpose_sketch_kernel<<<grid, dim3(32, 8), 0, st>>>(a.sk, n, a.s, skT);
        CK_CUDA(cudaGetLastError());
    }
    // temp storage sizes (the largest of the calls below, at a full batch)
    size_t t_sort = 0, t_rle = 0, t_scan = 0, t_scan2 = 0;
    {
        cub::DoubleBuffer<LshKey> dk(k0, k1);
        cub::DoubleBuffer<int32_t> dv(v0, v1);
        CK_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, t_sort, dk, dv, items, LshKeyParts{}, 0, 64 + tbits, st));
        CK_CUDA(cub::DeviceRunLengthEncode::Encode(nullptr, t_rle, k0, uniq, counts,
                                                   n_runs, (int)items, st));
        CK_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t_scan, counts, starts, (int)items, st));
        CK_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t_scan2, pair_off, pair_off, (int)items + 1, st));
    }
    const size_t t_max = std::max(std::max(t_sort, t_rle), std::max(t_scan, t_scan2));
    void *tmp = scratch(SLOT_SORT_TEMP, t_max, &status);
    if (!tmp) return status;

    // one batch: bucket ids, stable sort, runs, pair offsets; *total its pair count
    auto batch = [&](int32_t t0, int32_t tb, cub::DoubleBuffer<LshKey> &dk, cub::DoubleBuffer<int32_t> &dv,
                     int64_t *total) -> int32_t {
        const int64_t m = (int64_t)tb * n;
        lsh_hash_kernel<<<grid_of(m, 256), 256, 0, st>>>(skT, n, d_band, a.bands, d_seeds, t0, tb, dk.Current(),
                                                         dv.Current());
        CK_CUDA(cudaGetLastError());
        size_t tbytes = t_max;
        CK_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tbytes, dk, dv, m, LshKeyParts{}, 0, 64 + tbits, st));
        tbytes = t_max;
        CK_CUDA(cub::DeviceRunLengthEncode::Encode(tmp, tbytes, dk.Current(), uniq, counts,
                                                   n_runs, (int)m, st));
        tbytes = t_max;
        CK_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tbytes, counts, starts, (int)m, st));
        lsh_bucket_pairs_kernel<<<grid_of(m + 1, 256), 256, 0, st>>>(counts, n_runs, m, pair_off);
        CK_CUDA(cudaGetLastError());
        tbytes = t_max;
        CK_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tbytes, pair_off, pair_off, (int)m + 1, st));
        // pair_off[R] (R = runs) is the batch's total; runs <= m, entries past R are 0
        lsh_total_kernel<<<1, 32, 0, st>>>(n_runs, pair_off, d_total);
        CK_CUDA(cudaGetLastError());
        CK_CUDA(cudaMemcpyAsync(total, d_total, 8, cudaMemcpyDeviceToHost, st));
        CK_CUDA(cudaStreamSynchronize(st));
        return CK_OK;
    };

    // pass 1: count every batch's pairs
    const int32_t n_batches = (a.tables + TB - 1) / TB;
    std::vector<int64_t> per_batch((size_t)n_batches, 0);
    int64_t raw = 0;
    for (int32_t b = 0; b < n_batches; ++b) {
        const int32_t t0 = b * TB, tb = a.tables - t0 < TB ? a.tables - t0 : TB;
        cub::DoubleBuffer<LshKey> dk(k0, k1);
        cub::DoubleBuffer<int32_t> dv(v0, v1);
        CK_TRY(batch(t0, tb, dk, dv, &per_batch[b]));
        raw += per_batch[b];
    }
    if (raw == 0) return CK_OK;
    // pass 2: emit into one raw buffer (double, for the de-duplicating sort)
    uint64_t *rk = (uint64_t *)scratch(SLOT_FALLBACK, (size_t)raw * 8 * 2, &status);
    if (!rk) return status;
    int64_t at = 0;
    for (int32_t b = 0; b < n_batches; ++b) {
        if (per_batch[b] == 0) continue;
        const int32_t t0 = b * TB, tb = a.tables - t0 < TB ? a.tables - t0 : TB;
        cub::DoubleBuffer<LshKey> dk(k0, k1);
        cub::DoubleBuffer<int32_t> dv(v0, v1);
        int64_t tot = 0;
        CK_TRY(batch(t0, tb, dk, dv, &tot));
        const int64_t m = (int64_t)tb * n;
        CK_CUDA(cudaMemsetAsync(n_big, 0, 4, st));
        lsh_emit_runs_kernel<<<grid_of(m, 256), 256, 0, st>>>(dv.Current(), starts, counts, pair_off, n_runs, n,
                                                              rk + at, big, n_big);
        CK_CUDA(cudaGetLastError());
        lsh_emit_big_kernel<<<(int)sm_count() * 8, 256, 0, st>>>(dv.Current(), starts, counts, pair_off, big, n_big,
                                                                n, rk + at);
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
