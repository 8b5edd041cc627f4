// search.cu -- k-mer inverted index and Phase-A k-mer scoring for search.
//
// Index (clustkit/kmer_index.py:77-166): CSR over all alpha^k k-mer values;
// kmer_freqs[v] = occurrences of v, kmer_offsets = exclusive prefix sum,
// kmer_entries = (sequence << 32 | position) grouped by k-mer and, inside a
// k-mer, in (sequence, position) order.  k-mers holding a code >= alpha are
// not indexed.  Built on the GPU: every position emits (k-mer, entry), a
// stable radix sort by k-mer keeps the (sequence, position) order.
//
// Phase A (clustkit/kmer_index.py:470-534, :858-902): for each query k-mer
// (valid, frequency <= freq_thresh) every posting adds one hit to its target;
// counts saturate at 32767 as clustkit's int16 counters do; targets with
// count >= min_total_hits survive; at most top_k survive per query, chosen by
// count (ties: lower target id first), returned in target-id order.
#include <cub/block/block_scan.cuh>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_segmented_sort.cuh>
#include <cooperative_groups.h>

#include <algorithm>
#include <vector>

#include "ck_common.cuh"

namespace ck {

// ----------------------------------------------------------------- index build
__global__ void kmer_pos_count_kernel(const int32_t *lengths, int64_t n, int32_t k, int64_t *cnt) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t L = lengths[i];
        cnt[i] = L >= k ? (int64_t)(L - k + 1) : 0;
    }
}

__global__ void kmer_emit_kernel(const uint8_t *__restrict__ flat, int64_t flat_len,
                                 const int64_t *__restrict__ offsets,
                                 const int32_t *__restrict__ lengths, int64_t n, int32_t k,
                                 int32_t alpha, const int64_t *__restrict__ pos_base,
                                 uint32_t *__restrict__ keys, int64_t *__restrict__ vals,
                                 int32_t *__restrict__ freqs, uint32_t sentinel, int32_t *err) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < n; q += warps) {
        const int32_t L = lengths[q];
        const int64_t o = offsets[q];
        if (L < k) continue;
        if (o < 0 || o + L > flat_len) {
            if (lane == 0) atomicOr(err, ERRBIT_SEQ_EXTENT);
            continue;
        }
        const int64_t base = pos_base[q];
        for (int32_t p = lane; p <= L - k; p += 32) {
            uint32_t v = 0;
            bool ok = true;
            for (int32_t m = 0; m < k; ++m) {
                const uint32_t c = flat[o + p + m];
                ok &= c < (uint32_t)alpha;
                v = v * (uint32_t)alpha + c;
            }
            keys[base + p] = ok ? v : sentinel;
            vals[base + p] = ((int64_t)q << 32) | (int64_t)p;
            if (ok) atomicAdd(&freqs[v], 1);
        }
    }
}

__global__ void widen_kernel(const int32_t *in, int64_t n, int64_t *out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = i < n ? (int64_t)in[i] : 0;
}

static int grid_for(int64_t n, int threads, int cap_per_sm = 16) {
    int64_t b = (n + threads - 1) / threads;
    int64_t cap = (int64_t)sm_count() * cap_per_sm;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

struct IndexBuildArgs {
    const uint8_t *flat; int64_t flat_len; const int64_t *offsets; const int32_t *lengths; int64_t n;
    int32_t k, alpha; int64_t *kmer_offsets; int64_t *kmer_entries; int64_t capacity;
    int32_t *kmer_freqs; int64_t *out_total; cudaStream_t st;
};

static int32_t index_build_impl(void *pv) {
    IndexBuildArgs &a = *(IndexBuildArgs *)pv;
    int32_t status = CK_OK;
    int64_t nk = 1;
    for (int32_t i = 0; i < a.k; ++i) nk *= a.alpha;
    int32_t *err = device_error_word(&status);
    if (!err) return status;
    const size_t n1 = (size_t)(a.n > 0 ? a.n : 1);
    int64_t *cnt = (int64_t *)scratch(SLOT_SEARCH_TMP0, (n1 + 1) * 8, &status);
    if (!cnt) return status;
    kmer_pos_count_kernel<<<grid_for(a.n, 256), 256, 0, a.st>>>(a.lengths, a.n, a.k, cnt);
    CK_CUDA(cudaGetLastError());
    CK_CUDA(cudaMemsetAsync(cnt + a.n, 0, 8, a.st));
    size_t tb = 0;
    CK_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt, cnt, a.n + 1, a.st));
    void *tmp = scratch(SLOT_SEARCH_TMP4, tb, &status);
    if (!tmp) return status;
    CK_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, cnt, cnt, a.n + 1, a.st));
    int64_t P = 0;
    CK_CUDA(cudaMemcpyAsync(&P, cnt + a.n, 8, cudaMemcpyDeviceToHost, a.st));
    CK_CUDA(cudaStreamSynchronize(a.st));
    if (P >= ((int64_t)1 << 31)) {
        set_error(CK_ERR_INVALID_ARGUMENT, "kmer index: more than 2^31-1 k-mer positions in one build");
        return CK_ERR_INVALID_ARGUMENT;
    }
    if (P > a.capacity) {
        set_error(CK_ERR_INVALID_ARGUMENT, "kmer index: entries capacity below the number of k-mer positions");
        return CK_ERR_INVALID_ARGUMENT;
    }
    CK_CUDA(cudaMemsetAsync(a.kmer_freqs, 0, (size_t)nk * 4, a.st));
    const size_t P1 = (size_t)(P > 0 ? P : 1);
    uint32_t *k0 = (uint32_t *)scratch(SLOT_SEARCH_TMP1, P1 * 4, &status);
    uint32_t *k1 = (uint32_t *)scratch(SLOT_SEARCH_TMP2, P1 * 4, &status);
    int64_t *v0 = (int64_t *)scratch(SLOT_SEARCH_TMP3, P1 * 8, &status);
    if (!k0 || !k1 || !v0) return status;
    const uint32_t sentinel = (uint32_t)nk;
    if (a.n > 0)
        kmer_emit_kernel<<<grid_for(a.n * 32, 256), 256, 0, a.st>>>(
            a.flat, a.flat_len, a.offsets, a.lengths, a.n, a.k, a.alpha, cnt, k0, v0, a.kmer_freqs,
            sentinel, err);
    CK_CUDA(cudaGetLastError());
    int bits = 1;
    while (((int64_t)1 << bits) <= (int64_t)sentinel) ++bits;
    if (P > 0) {
        // the caller's entries buffer is the sort's second value buffer
        cub::DoubleBuffer<uint32_t> dk(k0, k1);
        cub::DoubleBuffer<int64_t> dv(v0, a.kmer_entries);
        size_t sb = 0;
        CK_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, sb, dk, dv, (int)P, 0, bits, a.st));
        void *stmp = scratch(SLOT_SEARCH_TMP4, sb, &status);
        if (!stmp) return status;
        CK_CUDA(cub::DeviceRadixSort::SortPairs(stmp, sb, dk, dv, (int)P, 0, bits, a.st));
        if (dv.Current() != a.kmer_entries)
            CK_CUDA(cudaMemcpyAsync(a.kmer_entries, dv.Current(), (size_t)P * 8, cudaMemcpyDeviceToDevice, a.st));
    }
    widen_kernel<<<grid_for(nk + 1, 256), 256, 0, a.st>>>(a.kmer_freqs, nk, a.kmer_offsets);
    CK_CUDA(cudaGetLastError());
    size_t tb2 = 0;
    CK_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb2, a.kmer_offsets, a.kmer_offsets, nk + 1, a.st));
    void *tmp2 = scratch(SLOT_SEARCH_TMP4, tb2, &status);
    if (!tmp2) return status;
    CK_CUDA(cub::DeviceScan::ExclusiveSum(tmp2, tb2, a.kmer_offsets, a.kmer_offsets, nk + 1, a.st));
    int64_t total = 0;
    CK_CUDA(cudaMemcpyAsync(&total, a.kmer_offsets + nk, 8, cudaMemcpyDeviceToHost, a.st));
    int32_t h = 0;
    CK_CUDA(cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, a.st));
    CK_CUDA(cudaMemsetAsync(err, 0, 4, a.st));
    CK_CUDA(cudaStreamSynchronize(a.st));
    if (h) {
        set_error(CK_ERR_OUT_OF_RANGE, "kmer index: sequence extent outside the flat buffer");
        return CK_ERR_OUT_OF_RANGE;
    }
    *a.out_total = total;
    return CK_OK;
}

// ----------------------------------------------------------------- phase A
// Targets that reach min_hits are listed as they cross it; up to CAND_CAP per
// query the select works on that list, beyond it on the full count row.
constexpr int32_t CAND_CAP = 4096;

// Grid (blocks, nq): the warps of a query's blocks take its k-mer positions
// in turn; a warp walks one posting list, lanes adding hits in parallel.
// Target of posting entry h: from the compact int32 copy when there is one
// (clustkit's kmer_entries_compact, clustkit/database.py:128-135: half the
// bytes per posting for the Phase-A walks), else the full entry's high half.
__device__ __forceinline__ int32_t entry_target(const int64_t *__restrict__ entries,
                                                const int32_t *__restrict__ targets, int64_t h) {
    return targets ? __ldg(targets + h) : (int32_t)(entries[h] >> 32);
}

// Dense pair list of a search batch for the SW engine: pair q * K + c is
// (seq0 + q, targets[q * K + c]) for the query's first n[q] candidates and
// (empty, empty) after them (an empty sequence aligns to nothing).
__global__ void search_pairs_kernel(int32_t nq, int32_t K, int32_t seq0, int32_t empty_idx,
                                    const int32_t *__restrict__ n, const int32_t *__restrict__ targets,
                                    int2 *__restrict__ pairs) {
    const int64_t M = (int64_t)nq * K;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t q = (int32_t)(i / K), c = (int32_t)(i - (int64_t)q * K);
        pairs[i] = c < __ldg(n + q) ? make_int2(seq0 + q, __ldg(targets + i)) : make_int2(empty_idx, empty_idx);
    }
}

__global__ void compact_targets_kernel(const int64_t *__restrict__ entries, int64_t n,
                                       int32_t *__restrict__ targets) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        targets[i] = (int32_t)(entries[i] >> 32);
}

__global__ void phase_a_count_kernel(const uint8_t *__restrict__ qflat, int64_t qflat_len,
                                     const int64_t *__restrict__ qoff,
                                     const int32_t *__restrict__ qlen, int32_t k, int32_t alpha,
                                     const int64_t *__restrict__ kmer_offsets,
                                     const int64_t *__restrict__ kmer_entries,
                                     const int32_t *__restrict__ kmer_targets,
                                     const int32_t *__restrict__ kmer_freqs, int32_t freq_thresh,
                                     int32_t num_db, int32_t *__restrict__ counts, int32_t min_hits,
                                     int32_t *__restrict__ cand, int32_t *__restrict__ n_cand,
                                     int32_t *err) {
    const int32_t q = blockIdx.y;
    const int lane = threadIdx.x & 31;
    const int32_t L = qlen[q];
    const int64_t o = qoff[q];
    if (L < 0 || o < 0 || o + L > qflat_len) {
        if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(err, ERRBIT_SEQ_EXTENT);
        return;
    }
    const uint8_t *s = qflat + o;
    int32_t *c = counts + (int64_t)q * num_db;
    const int32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (int32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p <= L - k; p += warps) {
        uint32_t v = 0;
        bool ok = true;
        for (int32_t m = 0; m < k; ++m) {
            const uint32_t r = s[p + m];
            ok &= r < (uint32_t)alpha;
            v = v * (uint32_t)alpha + r;
        }
        if (!ok || kmer_freqs[v] > freq_thresh) continue;
        const int64_t b = kmer_offsets[v], e = kmer_offsets[v + 1];
        for (int64_t h = b + lane; h < e; h += 32) {
            const int32_t t = entry_target(kmer_entries, kmer_targets, h);
            if (t >= 0 && t < num_db) {
                // the hit that lifts a target to min_hits lists it (once: counts only grow)
                if (atomicAdd(&c[t], 1) == min_hits - 1) {
                    const int32_t pos = atomicAdd(&n_cand[q], 1);
                    if (pos < CAND_CAP) cand[(int64_t)q * CAND_CAP + pos] = t;
                }
            } else {
                atomicOr(err, ERRBIT_PAIR_INDEX);
            }
        }
    }
}

constexpr int SELECT_THREADS = 1024;
constexpr int SELECT_UNROLL = 8;  // row values a thread loads at once

// Block-wide radix selection, 8 bits per level from bit `top_shift` down, over
// the values get(i), i < n, that are >= min_hits: sh[2] = their number; when it
// exceeds top_k, sh[0] = thr, the top_k-th largest value, and sh[1] = the
// number of values above thr (so top_k - sh[1] of those equal to thr are
// taken); else sh[0] = -1.
template <class Get>
__device__ void radix_threshold(Get get, int32_t n, int32_t min_hits, int32_t top_k, int top_shift, int32_t *hist,
                                int32_t *sh) {
    const int tid = threadIdx.x;
    if (tid == 0) { sh[0] = 0; sh[1] = 0; sh[2] = 0; }
    uint32_t mask = 0;
    for (int shift = top_shift; shift >= 0; shift -= 8) {
        for (int i = tid; i < 256; i += SELECT_THREADS) hist[i] = 0;
        __syncthreads();
        const uint32_t prefix = (uint32_t)sh[0];
        // SELECT_UNROLL independent loads per thread before any is used:
        // one block reads a whole count row per pass, so the pass is bound
        // by the loads it keeps in flight
        for (int32_t base = 0; base < n; base += SELECT_UNROLL * SELECT_THREADS) {
            int32_t v[SELECT_UNROLL];
#pragma unroll
            for (int u = 0; u < SELECT_UNROLL; ++u) {
                const int32_t i = base + u * SELECT_THREADS + tid;
                v[u] = i < n ? get(i) : 0;
            }
#pragma unroll
            for (int u = 0; u < SELECT_UNROLL; ++u) {
                const int32_t i = base + u * SELECT_THREADS + tid;
                if (i < n && v[u] >= min_hits && ((uint32_t)v[u] & mask) == prefix)
                    atomicAdd(&hist[((uint32_t)v[u] >> shift) & 255u], 1);
            }
        }
        __syncthreads();
        if (tid == 0) {
            if (shift == top_shift) {
                int32_t total = 0;
                for (int b = 0; b < 256; ++b) total += hist[b];
                sh[2] = total;
            }
            if (sh[2] > top_k) {
                int32_t above = sh[1], b = 255;
                for (; b > 0; --b) {
                    if (above + hist[b] >= top_k) break;
                    above += hist[b];
                }
                sh[0] = (int32_t)(prefix | ((uint32_t)b << shift));
                sh[1] = above;
            }
        }
        __syncthreads();
        if (sh[2] <= top_k) break;
        mask |= 255u << shift;
    }
    __syncthreads();
    if (tid == 0 && sh[2] <= top_k) { sh[0] = -1; sh[1] = 0; }
    __syncthreads();
}

// Bitonic sort of n (<= 2 * CAND_CAP 32-bit, or CAND_CAP 64-bit) keys in shared memory, ascending.
template <class K>
__device__ void block_bitonic(K *a, int32_t n, K pad) {
    const int tid = threadIdx.x;
    int32_t P = 1;
    while (P < n) P <<= 1;
    for (int32_t i = n + tid; i < P; i += SELECT_THREADS) a[i] = pad;
    __syncthreads();
    for (int32_t k = 2; k <= P; k <<= 1) {
        for (int32_t j = k >> 1; j > 0; j >>= 1) {
            for (int32_t i = tid; i < P; i += SELECT_THREADS) {
                const int32_t l = i ^ j;
                if (l > i) {
                    const K x = a[i], y = a[l];
                    if (((i & k) == 0) == (x > y)) { a[i] = y; a[l] = x; }
                }
            }
            __syncthreads();
        }
    }
}

// One block per query.  The surviving targets (value >= min_hits; values are
// the counts clamped to `clamp`): all of them in target-id order when at most
// top_k, else the top_k by value -- ties to the lower target id -- in
// descending value order, as clustkit's argsort(-scores) gives them
// (kmer_index.py:893-899, :1320-1325).  This kernel takes the queries whose
// candidate list is complete (min_hits >= 1, at most CAND_CAP listed: sorted
// by id in shared memory); the others are selected from their whole count row
// by the row_* kernels.
__global__ void __launch_bounds__(SELECT_THREADS)
phase_a_select_kernel(const int32_t *__restrict__ counts, int32_t num_db, int32_t min_hits, int32_t top_k,
                      int32_t clamp, int32_t top_shift, const int32_t *__restrict__ cand,
                      const int32_t *__restrict__ n_cand, int32_t *__restrict__ out_targets,
                      int32_t *__restrict__ out_scores, int32_t *__restrict__ out_n,
                      int32_t *__restrict__ capped_n) {
    using BlockScan = cub::BlockScan<int32_t, SELECT_THREADS>;
    __shared__ typename BlockScan::TempStorage scan_tmp;
    __shared__ uint64_t s_buf[CAND_CAP];  // sorted candidate ids, later the capped output's sort keys
    __shared__ int32_t hist[256];
    __shared__ int32_t sh[4], sh_run_eq, sh_run_sel;
    const int32_t q = blockIdx.x;
    const int tid = threadIdx.x;
    const int32_t *c = counts + (int64_t)q * num_db;
    int32_t *o_t = out_targets + (int64_t)q * top_k;
    int32_t *o_s = out_scores ? out_scores + (int64_t)q * top_k : nullptr;
    auto val = [&](int32_t t) { const int32_t v = c[t]; return v > clamp ? clamp : v; };
    if (!(min_hits >= 1 && n_cand[q] <= CAND_CAP)) return;  // a row query: the row_* kernels
    int32_t *s_id = (int32_t *)s_buf;
    {
        const int32_t n = n_cand[q];
        const int32_t *list = cand + (int64_t)q * CAND_CAP;
        for (int32_t i = tid; i < n; i += SELECT_THREADS) s_id[i] = list[i];
        block_bitonic<int32_t>(s_id, n, INT32_MAX);
        radix_threshold([&](int32_t i) { return val(s_id[i]); }, n, min_hits, top_k, top_shift, hist, sh);
        const int32_t thr = sh[0], take_eq = top_k - sh[1];
        if (tid == 0) { sh_run_eq = 0; sh_run_sel = 0; }
        __syncthreads();
        for (int32_t base = 0; base < n; base += SELECT_THREADS) {
            const int32_t i = base + tid;
            const int32_t t = i < n ? s_id[i] : 0;
            const int32_t v = i < n ? val(t) : -1;
            const int32_t is_eq = (i < n && thr >= 0 && v == thr) ? 1 : 0;
            int32_t eq_rank, eq_tot;
            BlockScan(scan_tmp).ExclusiveSum(is_eq, eq_rank, eq_tot);
            __syncthreads();
            const bool sel = i < n && (thr < 0 || v > thr || (is_eq && sh_run_eq + eq_rank < take_eq));
            int32_t pos, sel_tot;
            BlockScan(scan_tmp).ExclusiveSum(sel ? 1 : 0, pos, sel_tot);
            if (sel) {
                o_t[sh_run_sel + pos] = t;
                if (o_s) o_s[sh_run_sel + pos] = v;
            }
            __syncthreads();
            if (tid == 0) { sh_run_eq += eq_tot; sh_run_sel += sel_tot; }
            __syncthreads();
        }
    }
    const int32_t total = sh[2];
    const int32_t n_out = total < top_k ? total : top_k;
    __syncthreads();
    // capped: the kept targets in descending value order, ties by id
    if (total > top_k && top_k <= CAND_CAP) {
        for (int32_t i = tid; i < n_out; i += SELECT_THREADS) {
            const int32_t t = o_t[i];
            s_buf[i] = ((uint64_t)(uint32_t)(0x7fffffff - val(t)) << 32) | (uint32_t)t;
        }
        block_bitonic<uint64_t>(s_buf, n_out, ~0ull);
        for (int32_t i = tid; i < n_out; i += SELECT_THREADS) {
            const int32_t t = (int32_t)(s_buf[i] & 0xffffffffu);
            o_t[i] = t;
            if (o_s) o_s[i] = 0x7fffffff - (int32_t)(s_buf[i] >> 32);
        }
    }
    if (tid == 0) {
        out_n[q] = n_out;
        if (capped_n) capped_n[q] = (total > top_k && top_k > CAND_CAP) ? n_out : 0;
    }
}

// ----------------------------------------------------------------- row select
// The same selection for the queries whose survivors are not all in their
// candidate list, over the whole count row, by ROW_BLOCKS blocks per query
// (one block scanning a 500,000-counter row took 0.37 ms for one query).
// The row is cut into ROW_SLOTS warp slices in target order.  The radix
// threshold runs digit by digit: row_hist_kernel adds each block's histogram
// of the surviving values that match the digits so far into the query's
// global one and its last block picks the digit (the state stays on the
// device: no host synchronisation).  Then row_count_kernel counts each
// slice's values above and at the threshold, row_offsets_kernel turns those
// into each slice's output position and its share of the ties (lowest ids
// first), row_write_kernel writes the kept targets in id order and
// row_sort_kernel puts a capped row in (value desc, id asc) order.
// Per-query state: threshold (or -1: keep every survivor), count above its
// last digit, survivors, mode (0 in progress, 1 threshold known, 2 a list
// query: left to phase_a_select_kernel).  The digit pick runs in the last
// histogram block of each query (no launch of its own).
constexpr int ROW_BLOCKS = 128;
constexpr int ROW_THREADS = 256;
constexpr int ROW_SLOTS = ROW_BLOCKS * (ROW_THREADS / 32);  // 1,024 warp slices per row

__device__ __forceinline__ int32_t row_value(const int32_t *c, int64_t t, int32_t clamp) {
    const int32_t v = c[t];
    return v > clamp ? clamp : v;
}

// One radix digit of every row query's threshold.  Each block adds its
// slice's histogram into the query's global one; the last block of the query
// to finish (a counter, after a fence) picks the digit as radix_threshold
// does, records the state and clears the histogram and the counter for the
// next pass.  The first pass also sets every query's mode (a list query is
// marked and skipped).
__global__ void __launch_bounds__(ROW_THREADS)
row_hist_kernel(const int32_t *__restrict__ counts, int32_t num_db, int32_t min_hits, int32_t clamp, int32_t shift,
                uint32_t mask, int32_t first, int32_t last, const int32_t *__restrict__ n_cand, int32_t top_k,
                int32_t *__restrict__ state, int32_t *__restrict__ ghist, int32_t *__restrict__ done, int32_t W) {
    __shared__ int32_t h[256];
    __shared__ int32_t is_last;
    const int32_t q = blockIdx.y;
    int32_t *s = state + 4 * q;
    uint32_t prefix = 0;
    if (first) {
        if (min_hits >= 1 && n_cand[q] <= CAND_CAP) {  // a list query, the same for the whole block
            if (blockIdx.x == 0 && threadIdx.x == 0) { s[0] = 0; s[1] = 0; s[2] = 0; s[3] = 2; }
            return;
        }
    } else {
        if (s[3] != 0) return;  // the same for the whole block
        prefix = (uint32_t)s[0];
    }
    for (int i = threadIdx.x; i < 256; i += ROW_THREADS) h[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t slot = (int64_t)blockIdx.x * (ROW_THREADS / 32) + (threadIdx.x >> 5);
    const int64_t a0 = slot * W, a1 = a0 + W < num_db ? a0 + W : num_db;
    const int32_t *c = counts + (int64_t)q * num_db;
    for (int64_t base = a0; base < a1; base += 32 * SELECT_UNROLL) {
        int32_t v[SELECT_UNROLL];
#pragma unroll
        for (int u = 0; u < SELECT_UNROLL; ++u) {
            const int64_t t = base + u * 32 + lane;
            v[u] = t < a1 ? row_value(c, t, clamp) : 0;
        }
#pragma unroll
        for (int u = 0; u < SELECT_UNROLL; ++u) {
            const int64_t t = base + u * 32 + lane;
            if (t < a1 && v[u] >= min_hits && ((uint32_t)v[u] & mask) == prefix)
                atomicAdd(&h[((uint32_t)v[u] >> shift) & 255u], 1);
        }
    }
    __syncthreads();
    int32_t *g = ghist + (int64_t)q * 256;
    for (int i = threadIdx.x; i < 256; i += ROW_THREADS)
        if (h[i]) atomicAdd(&g[i], h[i]);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = atomicAdd(&done[q], 1) == (int32_t)gridDim.x - 1;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    for (int i = threadIdx.x; i < 256; i += ROW_THREADS) h[i] = __ldcg(&g[i]);
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t above = first ? 0 : s[1], total = first ? 0 : s[2];
        bool decided = false;
        if (first) {
            for (int b = 0; b < 256; ++b) total += h[b];
            if (total <= top_k) { s[0] = -1; s[1] = 0; s[2] = total; s[3] = 1; decided = true; }
        }
        if (!decided) {
            int32_t b = 255;
            for (; b > 0; --b) {
                if (above + h[b] >= top_k) break;
                above += h[b];
            }
            s[0] = (int32_t)(prefix | ((uint32_t)b << shift));
            s[1] = above;
            s[2] = total;
            s[3] = last ? 1 : 0;
        }
        done[q] = 0;
    }
    for (int i = threadIdx.x; i < 256; i += ROW_THREADS) g[i] = 0;
}

__global__ void __launch_bounds__(ROW_THREADS)
row_count_kernel(const int32_t *__restrict__ counts, int32_t num_db, int32_t min_hits, int32_t clamp,
                 const int32_t *__restrict__ state, int32_t W, int32_t *__restrict__ wcnt) {
    const int32_t q = blockIdx.y;
    if (state[4 * q + 3] != 1) return;
    const int32_t thr = state[4 * q];
    const int lane = threadIdx.x & 31;
    const int64_t slot = (int64_t)blockIdx.x * (ROW_THREADS / 32) + (threadIdx.x >> 5);
    const int64_t a0 = slot * W, a1 = a0 + W < num_db ? a0 + W : num_db;
    const int32_t *c = counts + (int64_t)q * num_db;
    int32_t n_strict = 0, n_eq = 0;
    for (int64_t base = a0; base < a1; base += 32 * SELECT_UNROLL) {
        int32_t v[SELECT_UNROLL];
#pragma unroll
        for (int u = 0; u < SELECT_UNROLL; ++u) {
            const int64_t t = base + u * 32 + lane;
            v[u] = t < a1 ? row_value(c, t, clamp) : 0;
        }
#pragma unroll
        for (int u = 0; u < SELECT_UNROLL; ++u) {
            const int64_t t = base + u * 32 + lane;
            const bool surv = t < a1 && v[u] >= min_hits;
            n_strict += __popc(__ballot_sync(0xffffffffu, surv && (thr < 0 || v[u] > thr)));
            n_eq += __popc(__ballot_sync(0xffffffffu, surv && thr >= 0 && v[u] == thr));
        }
    }
    if (lane == 0) {
        wcnt[((int64_t)q * ROW_SLOTS + slot) * 2] = n_strict;
        wcnt[((int64_t)q * ROW_SLOTS + slot) * 2 + 1] = n_eq;
    }
}

// One thread per slice: ties are taken from the lowest slices (lowest ids)
// until take_eq; each slice's output starts after the kept targets of the
// slices before it.
__global__ void __launch_bounds__(ROW_SLOTS)
row_offsets_kernel(const int32_t *__restrict__ state, const int32_t *__restrict__ wcnt, int32_t top_k,
                   int32_t *__restrict__ woff, int32_t *__restrict__ out_n, int32_t *__restrict__ capped_n) {
    using Scan = cub::BlockScan<int32_t, ROW_SLOTS>;
    __shared__ typename Scan::TempStorage tmp;
    const int32_t q = blockIdx.x;
    if (state[4 * q + 3] != 1) return;
    const int32_t thr = state[4 * q], take_eq = top_k - state[4 * q + 1], total = state[4 * q + 2];
    const int32_t i = threadIdx.x;
    const int32_t strict = wcnt[((int64_t)q * ROW_SLOTS + i) * 2], eq = wcnt[((int64_t)q * ROW_SLOTS + i) * 2 + 1];
    int32_t eq_base;
    Scan(tmp).ExclusiveSum(eq, eq_base);
    __syncthreads();
    int32_t take = take_eq - eq_base;
    take = thr < 0 ? 0 : (take < 0 ? 0 : (take > eq ? eq : take));
    int32_t out_base;
    Scan(tmp).ExclusiveSum(strict + take, out_base);
    woff[((int64_t)q * ROW_SLOTS + i) * 2] = eq_base;
    woff[((int64_t)q * ROW_SLOTS + i) * 2 + 1] = out_base;
    if (i == 0) {
        const int32_t n_out = total < top_k ? total : top_k;
        out_n[q] = n_out;
        if (capped_n) capped_n[q] = (total > top_k && top_k > CAND_CAP) ? n_out : 0;
    }
}

__global__ void __launch_bounds__(ROW_THREADS)
row_write_kernel(const int32_t *__restrict__ counts, int32_t num_db, int32_t min_hits, int32_t clamp,
                 const int32_t *__restrict__ state, int32_t W, const int32_t *__restrict__ woff, int32_t top_k,
                 int32_t *__restrict__ out_targets, int32_t *__restrict__ out_scores) {
    const int32_t q = blockIdx.y;
    if (state[4 * q + 3] != 1) return;
    const int32_t thr = state[4 * q], take_eq = top_k - state[4 * q + 1];
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    const int64_t slot = (int64_t)blockIdx.x * (ROW_THREADS / 32) + (threadIdx.x >> 5);
    const int64_t a0 = slot * W, a1 = a0 + W < num_db ? a0 + W : num_db;
    const int32_t *c = counts + (int64_t)q * num_db;
    int32_t *o_t = out_targets + (int64_t)q * top_k;
    int32_t *o_s = out_scores ? out_scores + (int64_t)q * top_k : nullptr;
    int32_t eq_seen = woff[((int64_t)q * ROW_SLOTS + slot) * 2], written = woff[((int64_t)q * ROW_SLOTS + slot) * 2 + 1];
    for (int64_t base = a0; base < a1; base += 32 * SELECT_UNROLL) {
        int32_t v[SELECT_UNROLL];
#pragma unroll
        for (int u = 0; u < SELECT_UNROLL; ++u) {
            const int64_t t = base + u * 32 + lane;
            v[u] = t < a1 ? row_value(c, t, clamp) : 0;
        }
#pragma unroll
        for (int u = 0; u < SELECT_UNROLL; ++u) {
            const int64_t t = base + u * 32 + lane;
            const bool surv = t < a1 && v[u] >= min_hits;
            const bool strict = surv && (thr < 0 || v[u] > thr);
            const bool is_eq = surv && thr >= 0 && v[u] == thr;
            const uint32_t eq_b = __ballot_sync(0xffffffffu, is_eq);
            const bool sel = strict || (is_eq && eq_seen + __popc(eq_b & lt) < take_eq);
            const uint32_t sel_b = __ballot_sync(0xffffffffu, sel);
            if (sel) {
                const int32_t at = written + __popc(sel_b & lt);
                o_t[at] = (int32_t)t;
                if (o_s) o_s[at] = v[u];
            }
            eq_seen += __popc(eq_b);
            written += __popc(sel_b);
        }
    }
}

// A capped row of at most CAND_CAP kept targets in (value desc, id asc)
// order, in shared memory (longer capped rows take the segmented sort).
__global__ void __launch_bounds__(SELECT_THREADS)
row_sort_kernel(const int32_t *__restrict__ counts, int32_t num_db, int32_t clamp, const int32_t *__restrict__ state,
                int32_t top_k, int32_t *__restrict__ out_targets, int32_t *__restrict__ out_scores) {
    __shared__ uint64_t s_buf[CAND_CAP];
    const int32_t q = blockIdx.x;
    if (state[4 * q + 3] != 1 || state[4 * q + 2] <= top_k || top_k > CAND_CAP) return;
    const int32_t *c = counts + (int64_t)q * num_db;
    int32_t *o_t = out_targets + (int64_t)q * top_k;
    int32_t *o_s = out_scores ? out_scores + (int64_t)q * top_k : nullptr;
    for (int32_t i = threadIdx.x; i < top_k; i += SELECT_THREADS) {
        const int32_t t = o_t[i];
        s_buf[i] = ((uint64_t)(uint32_t)(0x7fffffff - row_value(c, t, clamp)) << 32) | (uint32_t)t;
    }
    block_bitonic<uint64_t>(s_buf, top_k, ~0ull);
    for (int32_t i = threadIdx.x; i < top_k; i += SELECT_THREADS) {
        o_t[i] = (int32_t)(s_buf[i] & 0xffffffffu);
        if (o_s) o_s[i] = 0x7fffffff - (int32_t)(s_buf[i] >> 32);
    }
}

// Rows capped at more than CAND_CAP targets leave the select in id order; a
// segmented sort of (score desc, id asc) keys puts them in the order the
// shorter capped rows get in shared memory.  Rows that were not capped are
// empty segments.
__global__ void cap_keys_kernel(const int32_t *__restrict__ t, const int32_t *__restrict__ sc,
                                const int32_t *__restrict__ capped_n, int32_t top_k, uint64_t *__restrict__ keys,
                                int32_t *__restrict__ beg, int32_t *__restrict__ end) {
    const int32_t q = blockIdx.y;
    const int32_t n = capped_n[q];
    const int64_t row = (int64_t)q * top_k;
    if (blockIdx.x == 0 && threadIdx.x == 0) { beg[q] = (int32_t)row; end[q] = (int32_t)(row + n); }
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        keys[row + j] = ((uint64_t)(uint32_t)(0x7fffffff - sc[row + j]) << 32) | (uint32_t)t[row + j];
}

__global__ void cap_unpack_kernel(const uint64_t *__restrict__ keys, const int32_t *__restrict__ capped_n,
                                  int32_t top_k, int32_t *__restrict__ t, int32_t *__restrict__ sc) {
    const int32_t q = blockIdx.y;
    const int32_t n = capped_n[q];
    const int64_t row = (int64_t)q * top_k;
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint64_t k = keys[row + j];
        t[row + j] = (int32_t)(k & 0xffffffffu);
        sc[row + j] = 0x7fffffff - (int32_t)(k >> 32);
    }
}

// ----------------------------------------------------------------- similar k-mers
// clustkit/kmer_index.py:1187-1291: with k = 5 every 5-mer whose BLOSUM62
// column sum against a query 5-mer reaches the threshold T adds that sum to
// each target of its posting list (frequency in (0, freq_thresh]).  Stage 1
// (nbr_list_kernel) lists the (query, 5-mer, score) triples in one pass;
// stage 2 (nbr_walk_kernel) walks their posting lists.
//
// Stage 1 work items are (query position p, first two residues a0 a1), 400
// per position.  A warp tests 32 items against clustkit's pruning bound (the
// score so far plus the best remaining row scores must reach T); then, one
// surviving item at a time, its lanes split the 400 (a2, a3) continuations
// and each lane tries the 20 last residues, so no thread walks a heavy prefix
// alone.  Hits go to the warp's shared-memory stage as 4-byte entries (value
// | score << 22; 20^5 < 2^22, a score is at most 5 x 127); a full stage is
// flushed to the list with one global reservation, as 8-byte entries
// (query << 48 | score << 32 | value).  Which warp lists a triple first
// varies from run to run; the walk's integer sums do not depend on the order.
constexpr int32_t NB_PREFIX = 400;
constexpr int NB_WARPS = 8;              // warps per block
constexpr int32_t NB_STAGE = 1024;       // staged entries per warp (a round adds at most 32 x 20)
constexpr uint32_t NB_SCORE_SHIFT = 22;
constexpr int64_t NB_BLOCKS_PER_QUERY = 512;

__device__ __forceinline__ void nbr_flush(const uint32_t *stage, int32_t fill, int32_t q, uint64_t *list,
                                          int64_t cap, unsigned long long *cursor, int lane) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(cursor, (unsigned long long)fill);
    base = __shfl_sync(0xffffffffu, base, 0);
    for (int32_t i = lane; i < fill; i += 32) {
        const unsigned long long at = base + (unsigned long long)i;
        if (at < (unsigned long long)cap) {
            const uint32_t x = stage[i];
            list[at] = ((uint64_t)(uint32_t)q << 48) | ((uint64_t)(x >> NB_SCORE_SHIFT) << 32) |
                       (uint64_t)(x & ((1u << NB_SCORE_SHIFT) - 1u));
        }
    }
}

// Lists every (query, 5-mer, score) triple; *cursor (zeroed by the caller)
// ends as the number of triples, of which the first `cap` are written.
__global__ void __launch_bounds__(NB_WARPS * 32)
nbr_list_kernel(const uint8_t *__restrict__ qflat, int64_t qflat_len, const int64_t *__restrict__ qoff,
                const int32_t *__restrict__ qlen, const int8_t *__restrict__ sub, int32_t T,
                const int32_t *__restrict__ kmer_freqs, int32_t freq_thresh, uint64_t *__restrict__ list, int64_t cap,
                unsigned long long *__restrict__ cursor, int32_t *err) {
    constexpr uint32_t FULL = 0xffffffffu;
    __shared__ int32_t S[400];
    __shared__ int32_t mx[20];
    __shared__ uint32_t stage_all[NB_WARPS][NB_STAGE];
    const int32_t q = blockIdx.y;
    const int32_t L = qlen[q];
    const int64_t o = qoff[q];
    // both exits are the same for the whole block (before its first barrier)
    if (L < 0 || o < 0 || o + L > qflat_len) {
        if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(err, ERRBIT_SEQ_EXTENT);
        return;
    }
    const int64_t work = (int64_t)(L >= 5 ? L - 4 : 0) * NB_PREFIX;
    if ((int64_t)blockIdx.x * NB_WARPS * 32 >= work) return;  // a shorter query than the batch's longest
    for (int i = threadIdx.x; i < 400; i += blockDim.x) S[i] = sub[i];
    __syncthreads();
    if (threadIdx.x < 20) {
        int32_t m = -1000;
        for (int j = 0; j < 20; ++j) m = max(m, S[threadIdx.x * 20 + j]);
        mx[threadIdx.x] = m;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t *stage = stage_all[warp];
    const uint8_t *sq = qflat + o;
    const int64_t step = (int64_t)gridDim.x * NB_WARPS * 32;
    int32_t fill = 0;  // warp-uniform
    for (int64_t t0 = ((int64_t)blockIdx.x * NB_WARPS + warp) * 32; t0 < work; t0 += step) {
        const int64_t t = t0 + lane;
        bool live = false;
        int32_t p = 0, s1 = 0, v1 = 0;
        if (t < work) {
            p = (int32_t)(t / NB_PREFIX);
            const int32_t pre = (int32_t)(t - (int64_t)p * NB_PREFIX);
            const int32_t a0 = pre / 20, a1 = pre - a0 * 20;
            const int32_t q0 = sq[p], q1 = sq[p + 1], q2 = sq[p + 2], q3 = sq[p + 3], q4 = sq[p + 4];
            if (q0 < 20 && q1 < 20 && q2 < 20 && q3 < 20 && q4 < 20) {
                const int32_t m234 = mx[q2] + mx[q3] + mx[q4];
                const int32_t s0 = S[q0 * 20 + a0];
                s1 = s0 + S[q1 * 20 + a1];
                live = s0 + mx[q1] + m234 >= T && s1 + m234 >= T;
                v1 = a0 * 160000 + a1 * 8000;
            }
        }
        uint32_t lm = __ballot_sync(FULL, live);
        while (lm) {
            const int src = __ffs(lm) - 1;
            lm &= lm - 1;
            const int32_t P = __shfl_sync(FULL, p, src);
            const int32_t S1 = __shfl_sync(FULL, s1, src);
            const int32_t V1 = __shfl_sync(FULL, v1, src);
            const int32_t q2 = sq[P + 2], q3 = sq[P + 3], q4 = sq[P + 4];
            const int32_t m4 = mx[q4], m34 = mx[q3] + m4;
            const int32_t *S4 = S + q4 * 20;
            for (int32_t c0 = 0; c0 < 400; c0 += 32) {
                const int32_t c = c0 + lane;
                uint32_t bits = 0;
                int32_t s3 = 0, v3 = 0;
                if (c < 400) {
                    const int32_t a2 = c / 20, a3 = c - a2 * 20;
                    const int32_t s2 = S1 + S[q2 * 20 + a2];
                    s3 = s2 + S[q3 * 20 + a3];
                    if (s2 + m34 >= T && s3 + m4 >= T) {
                        v3 = V1 + a2 * 400 + a3 * 20;
#pragma unroll
                        for (int a4 = 0; a4 < 20; ++a4) {
                            if (s3 + S4[a4] >= T) {
                                const int32_t f = __ldg(kmer_freqs + v3 + a4);
                                if (f != 0 && f <= freq_thresh) bits |= 1u << a4;
                            }
                        }
                    }
                }
                if (!__any_sync(FULL, bits != 0)) continue;
                const int32_t n = __popc(bits);
                int32_t incl = n;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int32_t x = __shfl_up_sync(FULL, incl, d);
                    if (lane >= d) incl += x;
                }
                const int32_t tot = __shfl_sync(FULL, incl, 31);
                if (fill + tot > NB_STAGE) {
                    __syncwarp();
                    nbr_flush(stage, fill, q, list, cap, cursor, lane);
                    __syncwarp();
                    fill = 0;
                }
                int32_t at = fill + incl - n;
                while (bits) {
                    const int b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    stage[at++] = (uint32_t)(v3 + b) | ((uint32_t)(s3 + S4[b]) << NB_SCORE_SHIFT);
                }
                fill += tot;
            }
        }
    }
    if (fill > 0) {
        __syncwarp();
        nbr_flush(stage, fill, q, list, cap, cursor, lane);
    }
}

__global__ void fill_kernel(int32_t *a, int32_t n, int32_t v) {
    for (int32_t i = threadIdx.x; i < n; i += blockDim.x) a[i] = v;
}

// Stage 2.  A persistent grid; each block takes chunks of the list in order
// (a ticket counter) and walks them.  The listing pass fills the list about
// one query at a time, so the blocks in flight add into one or two queries'
// count rows, which stay in L2 (a grid-stride walk, whose warps drift apart
// over the whole list, kept every row of a 64-query batch live: 25.7 GB of
// DRAM writes instead of 0.24, and 1.5x the time).  The chunk comes from the
// count on the device (a multiple of 256, at most 2,048 triples): at least
// two per block, and the blocks in flight within about two queries' triples;
// so the launch needs no count from the host.
// A warp takes 32 triples at once: each lane loads one and its posting-list
// bounds -- 32 independent loads instead of 32 chains -- then the warp walks
// the concatenated lists, lane k of each round taking entry k of the stream
// (its list found by a binary search over the lanes' exclusive prefix sums
// of list lengths) and adding the triple's score to the entry's target in
// the triple's query row.  A list longer than `cap` (the listing pass
// counted more triples than it could write) is reported.
// Warps of the block take 32 triples of [c0, c1) at a time.
__device__ __forceinline__ void walk_chunk(const uint64_t *__restrict__ list, int64_t c0, int64_t c1, int32_t nq,
                                           const int64_t *__restrict__ kmer_offsets,
                                           const int64_t *__restrict__ kmer_entries,
                                           const int32_t *__restrict__ kmer_targets, int32_t num_db,
                                           int32_t *__restrict__ counts, int32_t *err, int lane) {
    constexpr uint32_t FULL = 0xffffffffu;
    for (int64_t base = c0 + (threadIdx.x >> 5) * 32; base < c1; base += blockDim.x) {
        const int64_t e = base + lane;
        int64_t b = 0;
        int32_t len = 0, w = 0, qq = 0;
        if (e < c1) {
            const uint64_t x = list[e];
            const int32_t v = (int32_t)(x & 0xffffffffu);
            w = (int32_t)((x >> 32) & 0xffffu);
            qq = (int32_t)(x >> 48);
            if (qq < nq) {
                b = kmer_offsets[v];
                len = (int32_t)(kmer_offsets[v + 1] - b);
            } else {
                atomicOr(err, ERRBIT_PAIR_INDEX);
            }
        }
        int32_t incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += t;
        }
        const int32_t excl = incl - len;
        const int32_t total = __shfl_sync(FULL, incl, 31);
        // rounds are warp-uniform so that every shuffle reads a live lane
        for (int32_t k0 = 0; k0 < total; k0 += 32) {
            const int32_t k = k0 + lane;
            // the stream's entry k belongs to the last lane whose list starts
            // at or before k (lanes with empty lists share their successor's
            // start and lose to it)
            int32_t o = 0;
#pragma unroll
            for (int step = 16; step; step >>= 1) {
                const int32_t cand = o + step;
                if (__shfl_sync(FULL, excl, cand) <= k) o = cand;
            }
            const int64_t h = __shfl_sync(FULL, b, o) + (k - __shfl_sync(FULL, excl, o));
            const int32_t wo = __shfl_sync(FULL, w, o);
            const int32_t qo = __shfl_sync(FULL, qq, o);
            if (k < total) {
                const int32_t t = entry_target(kmer_entries, kmer_targets, h);
                if (t < 0 || t >= num_db) {
                    atomicOr(err, ERRBIT_PAIR_INDEX);
                } else {
                    // no candidate list here (most of the database crosses
                    // min_hits in this mode; the select scans the row): the
                    // add's result is unused
                    atomicAdd(&counts[(int64_t)qo * num_db + t], wo);
                }
            }
        }
    }
}

__global__ void nbr_walk_kernel(const uint64_t *__restrict__ list, const unsigned long long *__restrict__ cursor,
                                int64_t cap, int32_t nq, const int64_t *__restrict__ kmer_offsets,
                                const int64_t *__restrict__ kmer_entries, const int32_t *__restrict__ kmer_targets,
                                int32_t num_db, int32_t *__restrict__ counts, unsigned long long *__restrict__ ticket,
                                int32_t *err) {
    __shared__ int64_t s_c0;
    const int lane = threadIdx.x & 31;
    const unsigned long long listed = *cursor;
    if (listed > (unsigned long long)cap && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, ERRBIT_LIST);
    const int64_t n = (int64_t)(listed < (unsigned long long)cap ? listed : (unsigned long long)cap);
    const int64_t G = gridDim.x;
    int64_t chunk = 2 * n / ((int64_t)(nq > 0 ? nq : 1) * G);
    if (n / (2 * G) < chunk) chunk = n / (2 * G);
    chunk = chunk / 256 * 256;
    chunk = chunk < 256 ? 256 : (chunk > 2048 ? 2048 : chunk);
    for (;;) {
        if (threadIdx.x == 0) s_c0 = (int64_t)atomicAdd(ticket, 1ull) * chunk;
        __syncthreads();
        const int64_t c0 = s_c0;
        __syncthreads();  // every thread has read s_c0 before it is written again
        if (c0 >= n) break;  // the same for the whole block
        const int64_t c1 = c0 + chunk < n ? c0 + chunk : n;
        walk_chunk(list, c0, c1, nq, kmer_offsets, kmer_entries, kmer_targets, num_db, counts, err, lane);
    }
}

// ----------------------------------------------------------------- Phase B
// clustkit's C scorer (csrc/kmer_score.c:195-415): after Phase A the top
// phase_a_topk targets by (count desc, id asc) are rescored by their hits'
// diagonals -- per target the longest run of hits in one diagonal bin
// (tpos - qpos + qlen) / diag_bin_width, the first such bin on ties -- and
// kept when that run reaches min_diag_hits, with the diagonal hint
// bin * width - qlen + width / 2.  Here every selected target owns a dense
// row of bin counters (its bins: (qlen + tlen) / width + 1), found through a
// per-query target -> selection-index row.
__global__ void pb_mark_kernel(const int32_t *__restrict__ sel, const int32_t *__restrict__ sel_n, int32_t topk,
                               const int32_t *__restrict__ db_len, const int32_t *__restrict__ qlen, int32_t width,
                               int32_t num_db, int32_t *__restrict__ idx_row, int64_t *__restrict__ nbins) {
    const int32_t q = blockIdx.y;
    const int32_t n = sel_n[q];
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < topk; i += gridDim.x * blockDim.x) {
        int64_t nb = 0;
        if (i < n) {
            const int32_t t = sel[(int64_t)q * topk + i];
            idx_row[(int64_t)q * num_db + t] = i;
            nb = (int64_t)(qlen[q] + db_len[t]) / width + 1;
        }
        nbins[(int64_t)q * topk + i] = nb;
    }
}

__global__ void pb_bin_count_kernel(const uint8_t *__restrict__ qflat, int64_t qflat_len,
                                    const int64_t *__restrict__ qoff, const int32_t *__restrict__ qlen, int32_t k,
                                    int32_t alpha, const int64_t *__restrict__ kmer_offsets,
                                    const int64_t *__restrict__ kmer_entries, const int32_t *__restrict__ kmer_freqs,
                                    int32_t freq_thresh, int32_t num_db, const int32_t *__restrict__ idx_row,
                                    int32_t topk, const int64_t *__restrict__ base, int32_t width,
                                    int32_t *__restrict__ bins, int64_t bins_cap, int32_t *err) {
    const int32_t q = blockIdx.y;
    const int lane = threadIdx.x & 31;
    const int32_t L = qlen[q];
    const int64_t o = qoff[q];
    if (L < 0 || o < 0 || o + L > qflat_len) {
        if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(err, ERRBIT_SEQ_EXTENT);
        return;
    }
    const uint8_t *s = qflat + o;
    const int32_t *ix = idx_row + (int64_t)q * num_db;
    const int64_t *bq = base + (int64_t)q * topk;
    const int32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (int32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p <= L - k; p += warps) {
        uint32_t v = 0;
        bool ok = true;
        for (int32_t m = 0; m < k; ++m) {
            const uint32_t r = s[p + m];
            ok &= r < (uint32_t)alpha;
            v = v * (uint32_t)alpha + r;
        }
        if (!ok || kmer_freqs[v] > freq_thresh) continue;
        const int64_t b = kmer_offsets[v], e = kmer_offsets[v + 1];
        for (int64_t h = b + lane; h < e; h += 32) {
            const int64_t entry = kmer_entries[h];
            const int32_t t = (int32_t)(entry >> 32);
            if (t < 0 || t >= num_db) { atomicOr(err, ERRBIT_PAIR_INDEX); continue; }
            const int32_t i = ix[t];
            if (i < 0) continue;
            const int64_t dbin = ((int64_t)(int32_t)(entry & 0xffffffff) - p + L) / width;
            const int64_t at = bq[i] + dbin;
            if (dbin < 0 || at >= bq[i + 1]) { atomicOr(err, ERRBIT_SEQ_EXTENT); continue; }
            if (at >= bins_cap) { atomicOr(err, ERRBIT_CAPACITY); continue; }
            atomicAdd(&bins[at], 1);
        }
    }
}

// A warp per selected target: its longest run (first bin on ties); kept ones
// are written into the (cleared) count row and listed for the final selection.
// The bins it reads are reset to zero, so a kept-zero bin buffer needs no
// clearing before the next call.
__global__ void pb_best_kernel(const int32_t *__restrict__ sel, const int32_t *__restrict__ sel_n, int32_t topk,
                               const int64_t *__restrict__ base, int32_t *__restrict__ bins, int64_t bins_cap,
                               const int32_t *__restrict__ qlen, int32_t width, int32_t min_diag_hits,
                               int32_t num_db, int32_t *__restrict__ counts, int32_t *__restrict__ hint_sel,
                               int32_t *__restrict__ cand, int32_t *__restrict__ n_cand) {
    const int32_t q = blockIdx.y;
    const int lane = threadIdx.x & 31;
    const int32_t n = sel_n[q];
    const int32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (int32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const int64_t b0 = base[(int64_t)q * topk + i];
        const int64_t b1 = min(base[(int64_t)q * topk + i + 1], bins_cap);
        int32_t best = 0, first = INT32_MAX;
        for (int64_t x = b0 + lane; x < b1; x += 32) {
            const int32_t c = bins[x];
            if (c) bins[x] = 0;
            if (c > best) { best = c; first = (int32_t)(x - b0); }
        }
        const int32_t m = __reduce_max_sync(0xffffffffu, best);
        const int32_t fb = __reduce_min_sync(0xffffffffu, (best == m && m > 0) ? first : INT32_MAX);
        if (lane == 0 && m >= min_diag_hits && m > 0) {
            const int32_t t = sel[(int64_t)q * topk + i];
            counts[(int64_t)q * num_db + t] = m;
            hint_sel[(int64_t)q * topk + i] = fb * width - qlen[q] + width / 2;
            const int32_t at = atomicAdd(&n_cand[q], 1);
            if (at < CAND_CAP) cand[(int64_t)q * CAND_CAP + at] = t;
        }
    }
}

__global__ void pb_hints_kernel(const int32_t *__restrict__ out_t, const int32_t *__restrict__ out_n, int32_t mc,
                                const int32_t *__restrict__ idx_row, int32_t num_db,
                                const int32_t *__restrict__ hint_sel, int32_t topk, int32_t *__restrict__ out_d) {
    const int32_t q = blockIdx.y;
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < out_n[q]; j += gridDim.x * blockDim.x) {
        const int32_t t = out_t[(int64_t)q * mc + j];
        const int32_t i = idx_row[(int64_t)q * num_db + t];
        out_d[(int64_t)q * mc + j] = i >= 0 ? hint_sel[(int64_t)q * topk + i] : 0;
    }
}

struct PhaseAArgs {
    const int8_t *sub_host; int32_t score_thresh;  // similar k-mers when sub_host != nullptr
    const uint8_t *qflat; int64_t qflat_len; const int64_t *qoff; const int32_t *qlen; int32_t nq; int32_t max_qlen;
    int32_t k, alpha; const int64_t *kmer_offsets; const int64_t *kmer_entries; const int32_t *kmer_targets;
    const int32_t *kmer_freqs; int32_t freq_thresh; int32_t num_db; int32_t min_hits; int32_t top_k;
    int32_t *out_targets; int32_t *out_scores; int32_t *out_n; cudaStream_t st;
    bool ordered = true;  // capped rows in (score desc, id asc) order, not only the set
    int64_t list_capacity = -1;  // similar k-mers: caller's bound on listed triples, < 0 sized here
};

// The select, then the order of rows capped above CAND_CAP.  `ordered`:
// the rows are a call's output (without it only the set matters, as for the
// Phase-B selection); their scores go to a scratch row when the caller
// takes none.
static int32_t select_rows(const int32_t *counts, int32_t nq, int32_t num_db, int32_t min_hits, int32_t top_k,
                           int32_t clamp, int32_t top_shift, const int32_t *cand, const int32_t *n_cand,
                           int32_t *out_t, int32_t *out_s, int32_t *out_n, bool ordered, cudaStream_t st) {
    int32_t status = CK_OK;
    if (nq <= 0) return CK_OK;
    const bool sort = top_k > CAND_CAP && ordered;
    int32_t *aux = nullptr;
    if (sort) {
        if ((int64_t)nq * top_k >= INT32_MAX) {
            set_error(CK_ERR_UNSUPPORTED, "search select: nq * top_k must stay below 2^31");
            return CK_ERR_UNSUPPORTED;
        }
        aux = (int32_t *)scratch(SLOT_SEARCH_TMP3, (size_t)nq * 12, &status);
        if (!aux) return status;
        if (!out_s) {
            out_s = (int32_t *)scratch(SLOT_SEARCH_SCORES, (size_t)nq * top_k * 4, &status);
            if (!out_s) return status;
        }
    }
    // queries selected from their whole row: the row_* kernels
    const size_t rs_ints = (size_t)nq * (4 + 256 + 1 + 4 * ROW_SLOTS);
    int32_t *rs = (int32_t *)scratch(SLOT_SEARCH_ROWSEL, rs_ints * 4, &status);
    if (!rs) return status;
    int32_t *state = rs, *ghist = rs + 4 * (size_t)nq, *done = ghist + 256 * (size_t)nq;
    int32_t *wcnt = done + (size_t)nq, *woff = wcnt + 2 * (size_t)ROW_SLOTS * nq;
    CK_CUDA(cudaMemsetAsync(ghist, 0, (size_t)nq * 257 * 4, st));  // histograms and block counters
    const int64_t slice = ((int64_t)num_db + ROW_SLOTS - 1) / ROW_SLOTS;
    const int32_t W = (int32_t)std::max<int64_t>(32, (slice + 31) / 32 * 32);
    const dim3 rg((unsigned)ROW_BLOCKS, (unsigned)nq);
    for (int shift = top_shift; shift >= 0; shift -= 8) {
        // the digits already fixed: bits shift + 8 .. top_shift + 7
        const uint32_t mask = (uint32_t)((((uint64_t)1 << (top_shift + 8)) - 1) & ~(((uint64_t)1 << (shift + 8)) - 1));
        row_hist_kernel<<<rg, ROW_THREADS, 0, st>>>(counts, num_db, min_hits, clamp, shift, mask,
                                                    shift == top_shift, shift == 0, n_cand, top_k, state, ghist,
                                                    done, W);
        CK_CUDA(cudaGetLastError());
    }
    row_count_kernel<<<rg, ROW_THREADS, 0, st>>>(counts, num_db, min_hits, clamp, state, W, wcnt);
    CK_CUDA(cudaGetLastError());
    row_offsets_kernel<<<nq, ROW_SLOTS, 0, st>>>(state, wcnt, top_k, woff, out_n, aux);
    CK_CUDA(cudaGetLastError());
    row_write_kernel<<<rg, ROW_THREADS, 0, st>>>(counts, num_db, min_hits, clamp, state, W, woff, top_k, out_t, out_s);
    CK_CUDA(cudaGetLastError());
    row_sort_kernel<<<nq, SELECT_THREADS, 0, st>>>(counts, num_db, clamp, state, top_k, out_t, out_s);
    CK_CUDA(cudaGetLastError());
    // queries whose candidate lists hold all their survivors
    phase_a_select_kernel<<<nq, SELECT_THREADS, 0, st>>>(counts, num_db, min_hits, top_k, clamp, top_shift, cand,
                                                         n_cand, out_t, out_s, out_n, aux);
    CK_CUDA(cudaGetLastError());
    if (!sort) return CK_OK;
    const size_t items = (size_t)nq * top_k;
    uint64_t *k0 = (uint64_t *)scratch(SLOT_SORT_KEYS, items * 8, &status);
    uint64_t *k1 = (uint64_t *)scratch(SLOT_SORT_KEYS_ALT, items * 8, &status);
    if (!k0 || !k1) return status;
    int32_t *beg = aux + nq, *end = aux + 2 * (size_t)nq;
    const dim3 g((unsigned)std::min(64, (top_k + 255) / 256), (unsigned)nq);
    cap_keys_kernel<<<g, 256, 0, st>>>(out_t, out_s, aux, top_k, k0, beg, end);
    CK_CUDA(cudaGetLastError());
    size_t tb = 0;
    CK_CUDA(cub::DeviceSegmentedSort::SortKeys(nullptr, tb, k0, k1, (int)items, nq, beg, end, st));
    void *tmp = scratch(SLOT_SORT_TEMP, tb, &status);
    if (!tmp) return status;
    CK_CUDA(cub::DeviceSegmentedSort::SortKeys(tmp, tb, k0, k1, (int)items, nq, beg, end, st));
    cap_unpack_kernel<<<g, 256, 0, st>>>(k1, aux, top_k, out_t, out_s);
    CK_CUDA(cudaGetLastError());
    return CK_OK;
}

static int32_t phase_a_impl(void *pv) {
    PhaseAArgs &a = *(PhaseAArgs *)pv;
    int32_t status = CK_OK;
    int32_t *err = device_error_word(&status);
    if (!err) return status;
    if (a.nq == 0) return CK_OK;
    const size_t nc = (size_t)a.nq * (size_t)a.num_db;
    int32_t *counts = (int32_t *)scratch(SLOT_SEARCH_COUNTS, nc * 4 + 4, &status);
    if (!counts) return status;
    int32_t *cand = (int32_t *)scratch(SLOT_SEARCH_CAND, (size_t)a.nq * (CAND_CAP + 1) * 4, &status);
    if (!cand) return status;
    int32_t *n_cand = cand + (size_t)a.nq * CAND_CAP;
    CK_CUDA(cudaMemsetAsync(counts, 0, nc * 4, a.st));
    CK_CUDA(cudaMemsetAsync(n_cand, 0, (size_t)a.nq * 4, a.st));
    const int32_t npos = a.max_qlen - a.k + 1;
    int32_t clamp = 32767, top_shift = 8;  // clustkit's int16 hit counters
    if (!a.sub_host) {
        if (npos > 0) {
            int bx = (npos + 7) / 8;  // 8 warps per block
            if (bx > 16) bx = 16;
            dim3 grid((unsigned)bx, (unsigned)a.nq);
            phase_a_count_kernel<<<grid, 256, 0, a.st>>>(a.qflat, a.qflat_len, a.qoff, a.qlen, a.k, a.alpha,
                                                          a.kmer_offsets, a.kmer_entries, a.kmer_targets,
                                                          a.kmer_freqs,
                                                          a.freq_thresh, a.num_db, counts, a.min_hits, cand,
                                                          n_cand, err);
            CK_CUDA(cudaGetLastError());
        }
    } else {
        clamp = INT32_MAX;  // score-weighted int32 sums
        top_shift = 24;
        const int8_t *d_sub = device_sub_matrix(a.sub_host, &status);
        if (!d_sub) return status;
        if (npos > 0) {
            // the listing's cursor and the walk's chunk ticket
            unsigned long long *cursor = (unsigned long long *)scratch(SLOT_SEARCH_TMP0, 16, &status);
            if (!cursor) return status;
            unsigned long long *ticket = cursor + 1;
            const bool bounded = a.list_capacity >= 0;
            // unbounded: the list scratch as it stands (at least 1 Mi triples); a
            // call that lists more reads the count, grows the list past it and
            // lists again.  bounded: the caller's capacity, no host read
            int64_t cap = bounded ? a.list_capacity
                                  : std::max<int64_t>((int64_t)(scratch_capacity(SLOT_SEARCH_TMP1) / 8), 1 << 20);
            uint64_t *list = (uint64_t *)scratch(SLOT_SEARCH_TMP1, (size_t)std::max<int64_t>(cap, 1) * 8, &status);
            if (!list) return status;
            if (!bounded) cap = (int64_t)(scratch_capacity(SLOT_SEARCH_TMP1) / 8);
            // one block per 256 items of the longest query, at most
            // NB_BLOCKS_PER_QUERY (longer queries loop; a graph captured for
            // an arena-long query would otherwise launch ~10^5 empty blocks per
            // query): blocks start in query order, so the list fills (and the
            // walk later runs) about one query at a time -- the walk's
            // count-row atomics then hit L2
            const int64_t groups = ((int64_t)npos * NB_PREFIX + NB_WARPS * 32 - 1) / (NB_WARPS * 32);
            const dim3 grid((unsigned)std::min<int64_t>(groups, NB_BLOCKS_PER_QUERY), (unsigned)a.nq);
            int64_t listed = -1;
            for (int pass = 0; pass < 2; ++pass) {
                CK_CUDA(cudaMemsetAsync(cursor, 0, 8, a.st));
                nbr_list_kernel<<<grid, NB_WARPS * 32, 0, a.st>>>(a.qflat, a.qflat_len, a.qoff, a.qlen, d_sub,
                                                                   a.score_thresh, a.kmer_freqs, a.freq_thresh, list,
                                                                   cap, cursor, err);
                CK_CUDA(cudaGetLastError());
                if (bounded) break;
                unsigned long long h = 0;
                CK_CUDA(cudaMemcpyAsync(&h, cursor, 8, cudaMemcpyDeviceToHost, a.st));
                CK_CUDA(cudaStreamSynchronize(a.st));
                listed = (int64_t)h;
                if (listed <= cap) break;
                // a quarter over the count, so that the next, slightly larger
                // batch does not list twice as well
                list = (uint64_t *)scratch(SLOT_SEARCH_TMP1, (size_t)(listed + listed / 4) * 8, &status);
                if (!list) return status;
                cap = (int64_t)(scratch_capacity(SLOT_SEARCH_TMP1) / 8);
            }
            // the walk: one resident block per slot (8 of 256 threads per
            // SM), fewer when the count is known to be small
            const int64_t n_walk = listed >= 0 ? listed : cap;
            const int64_t bw = std::max<int64_t>(1, std::min<int64_t>((int64_t)8 * sm_count(), (n_walk + 255) / 256));
            CK_CUDA(cudaMemsetAsync(ticket, 0, 8, a.st));
            nbr_walk_kernel<<<(unsigned)bw, 256, 0, a.st>>>(list, cursor, cap, a.nq, a.kmer_offsets, a.kmer_entries,
                                                            a.kmer_targets, a.num_db, counts, ticket, err);
            CK_CUDA(cudaGetLastError());
            // the select scans the whole count row (no candidate list in this mode)
            fill_kernel<<<1, 256, 0, a.st>>>(n_cand, a.nq, CAND_CAP + 1);
            CK_CUDA(cudaGetLastError());
        }
    }
    return select_rows(counts, a.nq, a.num_db, a.min_hits, a.top_k, clamp, top_shift, cand, n_cand,
                       a.out_targets, a.out_scores, a.out_n, a.ordered, a.st);
}

}  // namespace ck

using namespace ck;

extern "C" int32_t ck_kmer_index_build_device(int32_t ctx, const uint8_t *d_flat, int64_t flat_len,
                                              const int64_t *d_offsets, const int32_t *d_lengths,
                                              int64_t n_seqs, int32_t k, int32_t alpha,
                                              int64_t *d_kmer_offsets, int64_t *d_kmer_entries,
                                              int64_t entries_capacity, int32_t *d_kmer_freqs,
                                              int64_t *out_total, void *stream) {
    std::lock_guard<std::mutex> lock(library_mutex());
    reset_thread_status();
    int64_t nk = 1;
    for (int32_t i = 0; i < k && nk < ((int64_t)1 << 31); ++i) nk *= (alpha > 0 ? alpha : 1);
    if (k < 1 || alpha < 1 || nk >= ((int64_t)1 << 31) || n_seqs < 0 || flat_len < 0 || !out_total ||
        !d_kmer_offsets || !d_kmer_freqs || (n_seqs > 0 && (!d_offsets || !d_lengths))) {
        set_error(CK_ERR_INVALID_ARGUMENT, "kmer index: bad arguments (need alpha^k < 2^31)");
        return CK_ERR_INVALID_ARGUMENT;
    }
    IndexBuildArgs a{d_flat, flat_len, d_offsets, d_lengths, n_seqs, k, alpha, d_kmer_offsets,
                     d_kmer_entries, entries_capacity, d_kmer_freqs, out_total, (cudaStream_t)stream};
    return run_in_context(ctx, index_build_impl, &a);
}

extern "C" int32_t ck_kmer_targets_device(int32_t ctx, const int64_t *d_kmer_entries, int64_t n_entries,
                                          int32_t *d_kmer_targets, void *stream) {
    std::lock_guard<std::mutex> lock(library_mutex());
    reset_thread_status();
    if (n_entries < 0 || (n_entries > 0 && (!d_kmer_entries || !d_kmer_targets))) {
        set_error(CK_ERR_INVALID_ARGUMENT, "kmer targets: bad arguments");
        return CK_ERR_INVALID_ARGUMENT;
    }
    struct Args { const int64_t *e; int64_t n; int32_t *t; cudaStream_t st; } a{d_kmer_entries, n_entries,
                                                                                 d_kmer_targets, (cudaStream_t)stream};
    return run_in_context(ctx, [](void *pv) -> int32_t {
        const Args &a = *(const Args *)pv;
        if (a.n == 0) return CK_OK;
        compact_targets_kernel<<<grid_for(a.n, 256), 256, 0, a.st>>>(a.e, a.n, a.t);
        CK_CUDA(cudaGetLastError());
        return CK_OK;
    }, &a);
}

extern "C" int32_t ck_search_pairs_device(int32_t nq, int32_t max_cands, int32_t seq0, int32_t empty_idx,
                                          const int32_t *d_n, const int32_t *d_targets, int32_t *d_pairs,
                                          void *stream) {
    std::lock_guard<std::mutex> lock(library_mutex());
    reset_thread_status();
    if (nq < 0 || max_cands < 0 || (nq > 0 && max_cands > 0 && (!d_n || !d_targets || !d_pairs))) {
        set_error(CK_ERR_INVALID_ARGUMENT, "search pairs: bad arguments");
        return CK_ERR_INVALID_ARGUMENT;
    }
    const int64_t M = (int64_t)nq * max_cands;
    if (M == 0) return CK_OK;
    search_pairs_kernel<<<grid_for(M, 256), 256, 0, (cudaStream_t)stream>>>(nq, max_cands, seq0, empty_idx, d_n,
                                                                             d_targets, (int2 *)d_pairs);
    CK_CUDA(cudaGetLastError());
    return CK_OK;
}

extern "C" int32_t ck_search_phase_a_device(int32_t ctx, const uint8_t *d_qflat, int64_t qflat_len,
                                            const int64_t *d_qoffsets,
                                            const int32_t *d_qlengths, int32_t nq, int32_t max_qlen,
                                            int32_t k, int32_t alpha, const int64_t *d_kmer_offsets,
                                            const int64_t *d_kmer_entries, const int32_t *d_kmer_targets,
                                            const int32_t *d_kmer_freqs, int32_t freq_thresh, int32_t num_db,
                                            int32_t min_total_hits, int32_t top_k, int32_t *d_out_targets,
                                            int32_t *d_out_scores, int32_t *d_out_n, void *stream) {
    std::lock_guard<std::mutex> lock(library_mutex());
    reset_thread_status();
    if (nq < 0 || nq > 65535 || qflat_len < 0 || top_k < 1 || k < 1 || alpha < 1 || num_db < 0 || !d_out_targets || !d_out_n ||
        (nq > 0 && (!d_qflat || !d_qoffsets || !d_qlengths)) || !d_kmer_offsets || !d_kmer_freqs ||
        (!d_kmer_entries && !d_kmer_targets)) {
        set_error(CK_ERR_INVALID_ARGUMENT, "phase A: bad arguments");
        return CK_ERR_INVALID_ARGUMENT;
    }
    PhaseAArgs a{nullptr, 0, d_qflat, qflat_len, d_qoffsets, d_qlengths, nq, max_qlen, k, alpha, d_kmer_offsets, d_kmer_entries,
                 d_kmer_targets, d_kmer_freqs, freq_thresh, num_db, min_total_hits, top_k, d_out_targets, d_out_scores,
                 d_out_n, (cudaStream_t)stream};
    return run_in_context(ctx, phase_a_impl, &a);
}

extern "C" int32_t ck_search_phase_a_similar_device(int32_t ctx, const uint8_t *d_qflat, int64_t qflat_len,
                                                    const int64_t *d_qoffsets, const int32_t *d_qlengths,
                                                    int32_t nq, int32_t max_qlen, const int8_t *sub_matrix_host,
                                                    int32_t kmer_score_thresh, const int64_t *d_kmer_offsets,
                                                    const int64_t *d_kmer_entries, const int32_t *d_kmer_targets,
                                                    const int32_t *d_kmer_freqs, int32_t freq_thresh, int32_t num_db,
                                                    int32_t min_total_hits, int32_t top_k, int32_t *d_out_targets,
                                                    int32_t *d_out_scores, int32_t *d_out_n, int64_t list_capacity,
                                                    void *stream) {
    std::lock_guard<std::mutex> lock(library_mutex());
    reset_thread_status();
    if (nq < 0 || nq > 65535 || qflat_len < 0 || top_k < 1 || num_db < 0 || !sub_matrix_host ||
        kmer_score_thresh < 1 || !d_out_targets || !d_out_n || (nq > 0 && (!d_qflat || !d_qoffsets || !d_qlengths)) ||
        !d_kmer_offsets || !d_kmer_freqs || (!d_kmer_entries && !d_kmer_targets)) {
        set_error(CK_ERR_INVALID_ARGUMENT, "similar k-mer phase A: bad arguments");
        return CK_ERR_INVALID_ARGUMENT;
    }
    PhaseAArgs a{sub_matrix_host, kmer_score_thresh, d_qflat, qflat_len, d_qoffsets, d_qlengths, nq, max_qlen, 5,
                 20, d_kmer_offsets, d_kmer_entries, d_kmer_targets, d_kmer_freqs, freq_thresh, num_db,
                 min_total_hits, top_k, d_out_targets, d_out_scores, d_out_n, (cudaStream_t)stream};
    a.list_capacity = list_capacity;
    return run_in_context(ctx, phase_a_impl, &a);
}

namespace ck {

struct CandArgs {
    PhaseAArgs a;  // Phase A part (sub_host null); top_k there = max_cands
    const int32_t *db_len; int32_t min_diag_hits, width, phase_a_topk; int32_t *out_diags;
    int64_t bins_capacity;  // >= 0: the caller's bound on the bins (no host sync); < 0: sized from the scan
};

static int32_t candidates_impl(void *pv) {
    CandArgs &c = *(CandArgs *)pv;
    PhaseAArgs &a = c.a;
    int32_t status = CK_OK;
    const size_t nq = (size_t)a.nq;
    if (c.min_diag_hits <= 1) {  // Phase A and the cap, hints zero
        CK_TRY(phase_a_impl(&a));
        if (c.out_diags && a.nq > 0) CK_CUDA(cudaMemsetAsync(c.out_diags, 0, nq * a.top_k * 4, a.st));
        return CK_OK;
    }
    int32_t *err = device_error_word(&status);
    if (!err) return status;
    if (a.nq == 0) return CK_OK;
    const int32_t topk = c.phase_a_topk;
    // Phase A with the Phase-B top-K as its cap, into the selection buffers
    int32_t *sel = (int32_t *)scratch(SLOT_SEARCH_TMP2, nq * topk * 4 + nq * 4, &status);
    int64_t *base = (int64_t *)scratch(SLOT_SEARCH_TMP4, (nq * topk + 1) * 8, &status);
    int32_t *hint_sel = (int32_t *)scratch(SLOT_SEARCH_TMP0, nq * topk * 4, &status);
    int32_t *idx_row = (int32_t *)scratch(SLOT_SEARCH_IDX, nq * (size_t)a.num_db * 4 + 4, &status);
    if (!sel || !base || !hint_sel || !idx_row) return status;
    int32_t *sel_n = sel + nq * topk;
    PhaseAArgs a1 = a;
    a1.top_k = topk;
    a1.out_targets = sel;
    a1.out_scores = nullptr;
    a1.out_n = sel_n;
    a1.ordered = false;  // only the selected set matters
    CK_TRY(phase_a_impl(&a1));
    int32_t *counts = (int32_t *)scratch(SLOT_SEARCH_COUNTS, nq * (size_t)a.num_db * 4 + 4, &status);
    if (!counts) return status;
    CK_CUDA(cudaMemsetAsync(idx_row, 0xff, nq * (size_t)a.num_db * 4, a.st));
    const dim3 g1((unsigned)std::min(64, (topk + 255) / 256), (unsigned)a.nq);
    pb_mark_kernel<<<g1, 256, 0, a.st>>>(sel, sel_n, topk, c.db_len, a.qlen, c.width, a.num_db, idx_row, base);
    CK_CUDA(cudaGetLastError());
    // bin offsets: one exclusive scan over every (query, selected target); the
    // trailing entry is the total
    CK_CUDA(cudaMemsetAsync(base + nq * topk, 0, 8, a.st));
    size_t tb = 0;
    CK_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, base, base, (int64_t)(nq * topk + 1), a.st));
    void *tmp = scratch(SLOT_SORT_TEMP, tb, &status);
    if (!tmp) return status;
    CK_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, base, base, (int64_t)(nq * topk + 1), a.st));
    // the bins: a kept-zero buffer of the caller's bounded size (pb_best_kernel
    // resets what it reads; bins past the bound are skipped and flagged), or
    // sized from the scan's total read back here
    int64_t cap = c.bins_capacity;
    int32_t *bins = nullptr;
    if (cap >= 0) {
        bins = (int32_t *)scratch_zeroed(SLOT_SEARCH_BINS, (size_t)(cap > 0 ? cap : 1) * 4, a.st, &status);
    } else {
        CK_CUDA(cudaMemcpyAsync(&cap, base + nq * topk, 8, cudaMemcpyDeviceToHost, a.st));
        CK_CUDA(cudaStreamSynchronize(a.st));
        bins = (int32_t *)scratch(SLOT_SEARCH_TMP1, (size_t)(cap > 0 ? cap : 1) * 4, &status);
        if (bins && cap > 0) CK_CUDA(cudaMemsetAsync(bins, 0, (size_t)cap * 4, a.st));
    }
    if (!bins) return status;
    // from here to pb_best_kernel a failure leaves counts in the kept-zero buffer
    if (c.bins_capacity >= 0) scratch_mark_dirty(SLOT_SEARCH_BINS);
    const int32_t npos = a.max_qlen - a.k + 1;
    if (npos > 0) {
        int bx = (npos + 7) / 8;
        if (bx > 16) bx = 16;
        pb_bin_count_kernel<<<dim3((unsigned)bx, (unsigned)a.nq), 256, 0, a.st>>>(
            a.qflat, a.qflat_len, a.qoff, a.qlen, a.k, a.alpha, a.kmer_offsets, a.kmer_entries, a.kmer_freqs,
            a.freq_thresh, a.num_db, idx_row, topk, base, c.width, bins, cap, err);
        CK_CUDA(cudaGetLastError());
    }
    // final cap over the kept targets: from their list, or a scan of the row
    // when more than CAND_CAP were kept; runs are not clamped (int32 select)
    int32_t *cand = (int32_t *)scratch(SLOT_SEARCH_CAND, nq * (CAND_CAP + 1) * 4, &status);
    if (!cand) return status;
    int32_t *n_cand = cand + nq * CAND_CAP;
    CK_CUDA(cudaMemsetAsync(n_cand, 0, nq * 4, a.st));
    CK_CUDA(cudaMemsetAsync(counts, 0, nq * (size_t)a.num_db * 4, a.st));
    const dim3 g2((unsigned)std::min(64, (topk + 7) / 8), (unsigned)a.nq);
    pb_best_kernel<<<g2, 256, 0, a.st>>>(sel, sel_n, topk, base, bins, cap, a.qlen, c.width, c.min_diag_hits,
                                         a.num_db, counts, hint_sel, cand, n_cand);
    CK_CUDA(cudaGetLastError());
    if (c.bins_capacity >= 0) scratch_clear_dirty(SLOT_SEARCH_BINS);
    CK_TRY(select_rows(counts, a.nq, a.num_db, c.min_diag_hits, a.top_k, INT32_MAX, 24, cand, n_cand,
                       a.out_targets, a.out_scores, a.out_n, true, a.st));
    if (c.out_diags) {
        const dim3 g3((unsigned)std::min(64, (a.top_k + 255) / 256), (unsigned)a.nq);
        pb_hints_kernel<<<g3, 256, 0, a.st>>>(a.out_targets, a.out_n, a.top_k, idx_row, a.num_db, hint_sel, topk,
                                              c.out_diags);
        CK_CUDA(cudaGetLastError());
    }
    return CK_OK;
}

}  // namespace ck

extern "C" int32_t ck_search_kmer_candidates_device(
    int32_t ctx, const uint8_t *d_qflat, int64_t qflat_len, const int64_t *d_qoffsets, const int32_t *d_qlengths,
    int32_t nq, int32_t max_qlen, int32_t k, int32_t alpha, const int64_t *d_kmer_offsets,
    const int64_t *d_kmer_entries, const int32_t *d_kmer_targets, const int32_t *d_kmer_freqs, int32_t freq_thresh,
    int32_t num_db, const int32_t *d_db_lengths, int32_t min_total_hits, int32_t min_diag_hits,
    int32_t diag_bin_width, int32_t max_cands, int32_t phase_a_topk, int32_t *d_out_targets, int32_t *d_out_scores,
    int32_t *d_out_diags, int32_t *d_out_n, int64_t bins_capacity, void *stream) {
    std::lock_guard<std::mutex> lock(library_mutex());
    reset_thread_status();
    if (nq < 0 || nq > 65535 || qflat_len < 0 || max_cands < 1 || k < 1 || alpha < 1 || num_db < 0 ||
        !d_out_targets || !d_out_n || (nq > 0 && (!d_qflat || !d_qoffsets || !d_qlengths)) || !d_kmer_offsets ||
        !d_kmer_freqs || (!d_kmer_entries && !d_kmer_targets) ||
        (min_diag_hits >= 2 && (!d_kmer_entries || !d_db_lengths || diag_bin_width < 1 || phase_a_topk < 1))) {
        set_error(CK_ERR_INVALID_ARGUMENT, "k-mer candidates: bad arguments");
        return CK_ERR_INVALID_ARGUMENT;
    }
    CandArgs c{PhaseAArgs{nullptr, 0, d_qflat, qflat_len, d_qoffsets, d_qlengths, nq, max_qlen, k, alpha,
                          d_kmer_offsets, d_kmer_entries, d_kmer_targets, d_kmer_freqs, freq_thresh, num_db,
                          min_total_hits, max_cands, d_out_targets, d_out_scores, d_out_n, (cudaStream_t)stream},
               d_db_lengths, min_diag_hits, diag_bin_width, phase_a_topk, d_out_diags, bins_capacity};
    return run_in_context(ctx, candidates_impl, &c);
}
