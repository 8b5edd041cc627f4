// ck_common.cuh -- shared definitions of the libckgpu kernels and entry points.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "clustkit_gb300.h"

namespace ck {

// ---------------------------------------------------------------- errors
void set_error(int32_t status, const std::string &msg);
int32_t cuda_status(cudaError_t e, const char *what);

#define CK_CUDA(call)                                          \
    do {                                                       \
        cudaError_t ck_e_ = (call);                            \
        if (ck_e_ != cudaSuccess) return ::ck::cuda_status(ck_e_, #call); \
    } while (0)

#define CK_TRY(expr)                                           \
    do {                                                       \
        int32_t ck_s_ = (expr);                                \
        if (ck_s_ != CK_OK) return ck_s_;                      \
    } while (0)

// Bits of the per-device error word written by kernels.
enum : int32_t {
    ERRBIT_PAIR_INDEX = 1,     // pair index outside [0, n_seqs)
    ERRBIT_SEQ_EXTENT = 2,     // offsets[i] + lengths[i] outside [0, flat_len]
    ERRBIT_SCHEDULE = 4,       // a streamed warp-per-pair strip missed its start step (internal)
    ERRBIT_CAPACITY = 8,       // a device-side count passed the caller's bound (Phase-B bins)
    ERRBIT_LIST = 16,          // the similar-k-mer neighbour list passed the caller's bound
};

// ---------------------------------------------------------------- SW constants
// clustkit/csrc/sw_align.c:45-47
constexpr int32_t GAP_OPEN = -11;
constexpr int32_t GAP_EXTEND = -1;
constexpr int32_t NEG_INF = -1000000;
constexpr int32_t N_CODES = 21;       // residue codes the batched kernel tables cover (0..20)

struct SwOut {
    float *sims;
    int32_t *scores;
    int32_t *matches;
    int32_t *shorter;
    uint8_t *mask;
};

struct SwIn {
    const int32_t *pairs;
    const uint8_t *flat;
    const int64_t *offsets;
    const int32_t *lengths;
    const int32_t *hints;   // nullable
    int64_t n_seqs;
    int64_t flat_len;
    int32_t band_width;
    float threshold;
    int32_t pass_rule;
};

// Per-pair geometry shared by every SW kernel: which sequence is the row
// side, the effective band half-width and the clamped band offset
// (clustkit/csrc/sw_align.c:227-256 and :55-58).
struct PairGeom {
    int32_t a_idx, b_idx;   // a = rows (shorter; i when len_i <= len_j), b = columns
    int32_t la, lb;
    int32_t w;              // band half-width
    int32_t h;              // band centre offset (diagonal hint)
    int32_t valid;          // 0 when an index or extent check failed
};

__device__ __forceinline__ PairGeom pair_geometry(const SwIn &in, int64_t p, int32_t *err) {
    PairGeom g;
    int32_t i = __ldg(in.pairs + 2 * p), j = __ldg(in.pairs + 2 * p + 1);
    g.valid = 1;
    if (i < 0 || j < 0 || (int64_t)i >= in.n_seqs || (int64_t)j >= in.n_seqs) {
        atomicOr(err, ERRBIT_PAIR_INDEX);
        g.valid = 0;
        g.a_idx = g.b_idx = 0; g.la = g.lb = 0; g.w = 0; g.h = 0;
        return g;
    }
    int32_t li = __ldg(in.lengths + i), lj = __ldg(in.lengths + j);
    int64_t oi = __ldg(in.offsets + i), oj = __ldg(in.offsets + j);
    if (li < 0 || lj < 0 || oi < 0 || oj < 0 || oi + li > in.flat_len || oj + lj > in.flat_len) {
        atomicOr(err, ERRBIT_SEQ_EXTENT);
        g.valid = 0;
        g.a_idx = g.b_idx = 0; g.la = g.lb = 0; g.w = 0; g.h = 0;
        return g;
    }
    int32_t hint = in.hints ? __ldg(in.hints + p) : 0;
    int32_t shorter = li < lj ? li : lj;
    if (hint > shorter || hint < -shorter) hint = 0;
    if (li <= lj) { g.a_idx = i; g.b_idx = j; g.la = li; g.lb = lj; g.h = hint; }
    else          { g.a_idx = j; g.b_idx = i; g.la = lj; g.lb = li; g.h = -hint; }
    int32_t longer = g.lb;
    g.w = (in.band_width <= 0 || longer <= 50) ? longer : in.band_width;
    return g;
}

// Number of DP cells clustkit evaluates for a pair (its work unit).
__host__ __device__ __forceinline__ int64_t band_cells(int32_t la, int32_t lb, int32_t w, int32_t h) {
    int64_t c = 0;
    if (la <= 0 || lb <= 0) return 0;
    // rows i with a non-empty band: lo = max(1, i+h-w) <= hi = min(lb, i+h+w)
    for (int32_t i = 1; i <= la; i++) {
        int64_t lo = (int64_t)i + h - w, hi = (int64_t)i + h + w;
        if (lo < 1) lo = 1;
        if (hi > lb) hi = lb;
        if (hi >= lo) c += hi - lo + 1;
    }
    return c;
}

// Final per-pair write-out under the chosen pass rule.
__device__ __forceinline__ void write_result(const SwOut &o, const SwIn &in, int64_t p,
                                             int32_t score, int32_t matches, int32_t shorter,
                                             int32_t la, int32_t lb) {
    float ident = 0.0f;
    if (score <= 0) { score = 0; matches = 0; }
    else ident = __fdiv_rn((float)matches, (float)shorter);
    uint8_t pass;
    switch (in.pass_rule) {
        case CK_PASS_CPU: pass = ident >= in.threshold; break;
        case CK_PASS_NUMBA: pass = (score > 0) && (ident >= in.threshold); break;
        case CK_PASS_CUPY: {
            int32_t longer = la > lb ? la : lb, sh = la < lb ? la : lb;
            bool ratio_fail = longer > 0 && __fdiv_rn((float)sh, (float)longer) < in.threshold;
            pass = !ratio_fail && (score > 0) && (ident >= in.threshold);
            break;
        }
        default: pass = score > 0; break;
    }
    if (o.sims) o.sims[p] = ident;
    if (o.scores) o.scores[p] = score;
    if (o.matches) o.matches[p] = matches;
    if (o.shorter) o.shorter[p] = shorter;
    if (o.mask) o.mask[p] = pass;
}

// CK_PASS_CUPY skips the alignment of pairs that fail the length ratio, as
// clustkit's CUDA kernel does (clustkit/pairwise.py:1246-1252).
__device__ __forceinline__ bool cupy_ratio_skip(const SwIn &in, int32_t la, int32_t lb) {
    if (in.pass_rule != CK_PASS_CUPY) return false;
    int32_t longer = la > lb ? la : lb, sh = la < lb ? la : lb;
    return longer > 0 && __fdiv_rn((float)sh, (float)longer) < in.threshold;
}

// ---------------------------------------------------------------- launchers
struct SwCounters {
    int64_t pairs, cells, batched, plain, rerun, launches, wave;
};

int32_t sw_plain_launch(const SwIn &in, const SwOut &out, int64_t M, const int32_t *d_index,
                        const int32_t *d_count, int32_t *d_err, cudaStream_t st,
                        SwCounters *ctr);
int32_t widest_band(const SwIn &in, cudaStream_t st, int32_t *w_out);
int32_t sw_batched_launch(const SwIn &in, const SwOut &out, int64_t M, const int8_t *d_sub,
                          int32_t *d_err, cudaStream_t st, SwCounters *ctr, bool read_counters);
int32_t sw_set_rows_per_strip(int32_t r);
int32_t sw_rows_per_strip();
int32_t sw_set_strip_threads(int32_t v);
int32_t sw_strip_threads();
int32_t sw_set_wide_key(int32_t v);
int32_t sw_wide_key();
int32_t sw_set_variant(int32_t v);
int32_t sw_variant();
int32_t sw_set_wave(int32_t key, int32_t v);  // key 0: min rows, 1: all-pairs batch limit, 2: adaptive, 3: stream, 4: streamed strip rows
int32_t sw_wave(int32_t key);
int32_t sw_run_device(const SwIn &in, const SwOut &out, int64_t M, int32_t engine,
                      const int8_t *sub_host, cudaStream_t st, SwCounters *ctr,
                      bool read_counters);

int32_t sketch_launch(const uint8_t *flat, int64_t flat_len, const int64_t *offsets,
                      const int32_t *lengths, int64_t N, int32_t k, int32_t s, int32_t alphabet,
                      uint64_t seed, uint64_t *out, int32_t *d_err, cudaStream_t st);
int32_t jaccard_launch(const int32_t *pairs, int64_t M, const uint64_t *sk, int64_t N, int32_t s,
                       float floor, float *sims, uint8_t *mask, int32_t *d_err, cudaStream_t st);

// Kernel timing hook: when enabled (ck_sw_profile), returns the event pair
// to record around the dominant kernel's launch on its own stream.
bool profile_events(cudaEvent_t *start, cudaEvent_t *stop);

// Lock and context plumbing for entry points defined outside capi.cu.
std::mutex &library_mutex();
int32_t run_in_context(int32_t handle, int32_t (*fn)(void *), void *arg);
void reset_thread_status();

// Per-device scratch: grow-only buffers owned by the library.
void *scratch(int slot, size_t bytes, int32_t *status);
void *scratch_zeroed(int slot, size_t bytes, cudaStream_t st, int32_t *status);
size_t scratch_capacity(int slot);  // bytes the slot holds now (0 when unallocated)
void scratch_mark_dirty(int slot);
void scratch_clear_dirty(int slot);
int32_t *device_error_word(int32_t *status);
const int8_t *device_sub_matrix(const int8_t *host20x20, int32_t *status);
int current_device();
int sm_count();

enum ScratchSlot {
    SLOT_PLAIN_WS = 0,
    SLOT_SORT_KEYS,
    SLOT_SORT_VALS,
    SLOT_SORT_KEYS_ALT,
    SLOT_SORT_VALS_ALT,
    SLOT_SORT_TEMP,
    SLOT_FALLBACK,
    SLOT_COUNTERS,
    SLOT_WINDOW,
    SLOT_INC,
    SLOT_SEQ_OK,
    SLOT_MAXLEN,
    SLOT_SEARCH_COUNTS,
    SLOT_SEARCH_CAND,
    SLOT_SEARCH_IDX,
    SLOT_SEARCH_SCORES,
    SLOT_SEARCH_BINS,
    SLOT_SEARCH_TMP0,
    SLOT_SEARCH_TMP1,
    SLOT_SEARCH_TMP2,
    SLOT_SEARCH_TMP3,
    SLOT_SEARCH_TMP4,
    SLOT_SEARCH_ROWSEL,
    SLOT_HOST_IO0,
    SLOT_HOST_IO1,
    SLOT_HOST_IO2,
    SLOT_HOST_IO3,
    SLOT_HOST_IO4,
    SLOT_HOST_IO5,
    SLOT_HOST_IO6,
    SLOT_HOST_IO7,
    SLOT_HOST_IO8,
    SLOT_COUNT
};

}  // namespace ck
