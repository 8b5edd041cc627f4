// capi.cu -- runtime and C entry points of libckgpu.so (declared in
// include/clustkit_gb300.h).
//
// Runtime: per device, a set of grow-only scratch buffers, a device copy of
// the substitution matrix, an error word that kernels OR bits into, and one
// non-blocking stream for the host-buffer entry points.  Every entry point
// holds one library mutex (clustkit's own C entry point is not re-entrant
// either) and reports failures as a status code plus a per-thread message.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "ck_common.cuh"

namespace ck {

namespace {

constexpr int MAX_DEVICES = 16;

// One set of grow-only scratch buffers plus an error word.  Each device has
// a default set; contexts (ck_ctx_create) own further sets so that work
// enqueued on different streams never shares scratch.
struct ScratchSet {
    int device = -1;
    void *buf[SLOT_COUNT] = {};
    size_t cap[SLOT_COUNT] = {};
    int32_t *err = nullptr;
    bool frozen = false;  // buffers may be baked into a captured CUDA graph: never reallocate
    bool dirty[SLOT_COUNT] = {};  // a kept-zero buffer whose last user may not have cleaned it
    // resident sequence database of the submit/poll interface (ck_ctx_upload_db)
    uint8_t *db_flat = nullptr;
    int64_t *db_offsets = nullptr;
    int32_t *db_lengths = nullptr;
    int64_t db_flat_len = 0, db_n = 0;
    bool db_ready = false;
    // the one submission in flight (ck_ctx_submit .. ck_ctx_poll / ck_ctx_wait)
    cudaEvent_t done = nullptr;
    cudaStream_t pending_stream = nullptr;
    bool pending = false;
};

void free_db(ScratchSet *set) {
    if (set->db_flat) cudaFree(set->db_flat);
    if (set->db_offsets) cudaFree(set->db_offsets);
    if (set->db_lengths) cudaFree(set->db_lengths);
    set->db_flat = nullptr;
    set->db_offsets = nullptr;
    set->db_lengths = nullptr;
    set->db_flat_len = set->db_n = 0;
    set->db_ready = false;
}

struct DeviceState {
    bool init = false;
    int sms = 0;
    cudaStream_t stream = nullptr;
    ScratchSet def;
    int8_t *sub = nullptr;
    int8_t sub_host[400] = {};
    bool sub_valid = false;
};

std::mutex g_mutex;
DeviceState g_dev[MAX_DEVICES];
std::vector<ScratchSet *> g_ctx;  // handle h -> g_ctx[h - 1]
thread_local std::string t_error;
thread_local int32_t t_status = CK_OK;
thread_local SwCounters t_counters = {};
thread_local ScratchSet *t_set = nullptr;  // context of the entry point running on this thread

DeviceState *state(int32_t *status) {
    int d = 0;
    cudaError_t e = cudaGetDevice(&d);
    if (e != cudaSuccess) {
        *status = cuda_status(e, "cudaGetDevice");
        return nullptr;
    }
    if (d < 0 || d >= MAX_DEVICES) {
        set_error(CK_ERR_NO_DEVICE, "device ordinal out of range");
        *status = CK_ERR_NO_DEVICE;
        return nullptr;
    }
    DeviceState &s = g_dev[d];
    if (!s.init) {
        cudaDeviceProp prop;
        e = cudaGetDeviceProperties(&prop, d);
        if (e != cudaSuccess) { *status = cuda_status(e, "cudaGetDeviceProperties"); return nullptr; }
        s.sms = prop.multiProcessorCount;
        e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { *status = cuda_status(e, "cudaStreamCreate"); return nullptr; }
        s.def.device = d;
        e = cudaMalloc(&s.def.err, 64);
        if (e != cudaSuccess) { *status = cuda_status(e, "cudaMalloc(error word)"); return nullptr; }
        e = cudaMemset(s.def.err, 0, 64);
        if (e != cudaSuccess) { *status = cuda_status(e, "cudaMemset(error word)"); return nullptr; }
        e = cudaMalloc(&s.sub, 512);
        if (e != cudaSuccess) { *status = cuda_status(e, "cudaMalloc(sub)"); return nullptr; }
        s.init = true;
    }
    return &s;
}

}  // namespace

void set_error(int32_t status, const std::string &msg) {
    t_status = status;
    t_error = msg;
}

int32_t cuda_status(cudaError_t e, const char *what) {
    int32_t st = (e == cudaErrorMemoryAllocation) ? CK_ERR_OUT_OF_MEMORY
               : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? CK_ERR_NO_DEVICE
               : CK_ERR_CUDA;
    set_error(st, std::string(what) + ": " + cudaGetErrorString(e));
    return st;
}

int current_device() {
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

int sm_count() {
    int32_t st = CK_OK;
    DeviceState *s = state(&st);
    return s ? s->sms : 1;
}

static ScratchSet *current_set(int32_t *status) {
    DeviceState *d = state(status);
    if (!d) return nullptr;
    if (t_set && t_set->device == current_device()) return t_set;
    return &d->def;
}

void *scratch(int slot, size_t bytes, int32_t *status) {
    ScratchSet *s = current_set(status);
    if (!s) return nullptr;
    if (bytes == 0) bytes = 1;
    if (s->cap[slot] < bytes) {
        if (s->frozen) {
            set_error(CK_ERR_UNSUPPORTED, "context scratch is frozen (its buffers may be captured in a "
                                          "CUDA graph) and too small for this call");
            *status = CK_ERR_UNSUPPORTED;
            return nullptr;
        }
        // grow by at least half again, so that a growing workload reallocates
        // (and, through cudaFree, synchronises the device) only a few times
        const size_t old = s->cap[slot];
        if (s->buf[slot]) {
            cudaError_t e = cudaFree(s->buf[slot]);  // synchronises with work still using it
            s->buf[slot] = nullptr;
            s->cap[slot] = 0;
            if (e != cudaSuccess) { *status = cuda_status(e, "cudaFree(scratch)"); return nullptr; }
        }
        size_t want = std::max(bytes, old + old / 2);
        want = (want + 255) & ~(size_t)255;
        cudaError_t e = cudaMalloc(&s->buf[slot], want);
        if (e != cudaSuccess) {
            s->buf[slot] = nullptr;
            *status = cuda_status(e, "cudaMalloc(scratch)");
            return nullptr;
        }
        s->cap[slot] = want;
    }
    return s->buf[slot];
}

// A buffer that is all zero when the call's work starts, for users that
// restore the zeros they write (so no per-call clear is needed): cleared on
// the stream when it is (re)allocated or after scratch_mark_dirty.
void *scratch_zeroed(int slot, size_t bytes, cudaStream_t st, int32_t *status) {
    ScratchSet *s = current_set(status);
    if (!s) return nullptr;
    const void *before = s->buf[slot];
    void *p = scratch(slot, bytes, status);
    if (!p) return nullptr;
    if (p != before || s->dirty[slot]) {
        const cudaError_t e = cudaMemsetAsync(p, 0, s->cap[slot], st);
        if (e != cudaSuccess) { *status = cuda_status(e, "cudaMemsetAsync(zeroed scratch)"); return nullptr; }
        s->dirty[slot] = false;
    }
    return p;
}

size_t scratch_capacity(int slot) {
    int32_t status = CK_OK;
    ScratchSet *s = current_set(&status);
    return s ? s->cap[slot] : 0;
}

void scratch_mark_dirty(int slot) {
    int32_t status = CK_OK;
    ScratchSet *s = current_set(&status);
    if (s) s->dirty[slot] = true;
}

void scratch_clear_dirty(int slot) {
    int32_t status = CK_OK;
    ScratchSet *s = current_set(&status);
    if (s) s->dirty[slot] = false;
}

int32_t *device_error_word(int32_t *status) {
    ScratchSet *s = current_set(status);
    return s ? s->err : nullptr;
}

// Runs `fn` with the scratch set of context `handle` (0 = the device default).
template <class F>
static int32_t with_context(int32_t handle, F fn) {
    if (handle < 0 || handle > (int32_t)g_ctx.size() || (handle > 0 && !g_ctx[handle - 1])) {
        set_error(CK_ERR_INVALID_ARGUMENT, "unknown context handle");
        return CK_ERR_INVALID_ARGUMENT;
    }
    ScratchSet *set = handle > 0 ? g_ctx[handle - 1] : nullptr;
    if (set && set->device != current_device()) {
        set_error(CK_ERR_INVALID_ARGUMENT, "context belongs to another device");
        return CK_ERR_INVALID_ARGUMENT;
    }
    t_set = set;
    const int32_t st = fn();
    t_set = nullptr;
    return st;
}

const int8_t *device_sub_matrix(const int8_t *host, int32_t *status) {
    DeviceState *s = state(status);
    if (!s) return nullptr;
    if (host && (!s->sub_valid || memcmp(host, s->sub_host, 400) != 0)) {
        cudaError_t e = cudaMemcpy(s->sub, host, 400, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { *status = cuda_status(e, "upload sub_matrix"); return nullptr; }
        memcpy(s->sub_host, host, 400);
        s->sub_valid = true;
    }
    if (!s->sub_valid) {
        set_error(CK_ERR_INVALID_ARGUMENT, "substitution matrix not set");
        *status = CK_ERR_INVALID_ARGUMENT;
        return nullptr;
    }
    return s->sub;
}

std::mutex &library_mutex() { return g_mutex; }
void reset_thread_status() { t_status = CK_OK; }
int32_t run_in_context(int32_t handle, int32_t (*fn)(void *), void *arg) {
    return with_context(handle, [&] { return fn(arg); });
}

static cudaStream_t lib_stream(int32_t *status) {
    DeviceState *s = state(status);
    return s ? s->stream : nullptr;
}

int32_t sw_run_device(const SwIn &in, const SwOut &out, int64_t M, int32_t engine,
                      const int8_t *sub_host, cudaStream_t st, SwCounters *ctr,
                      bool read_counters) {
    int32_t status = CK_OK;
    const int8_t *d_sub = device_sub_matrix(sub_host, &status);
    if (!d_sub) return status;
    int32_t *err = device_error_word(&status);
    if (!err) return status;
    if (ctr) ctr->pairs += M;
    if (engine == CK_SW_PLAIN) {
        if (M == 0) return CK_OK;
        cudaEvent_t ev0 = nullptr, ev1 = nullptr;
        if (profile_events(&ev0, &ev1)) CK_CUDA(cudaEventRecord(ev0, st));
        CK_TRY(sw_plain_launch(in, out, M, nullptr, nullptr, err, st, ctr));
        if (ev1) CK_CUDA(cudaEventRecord(ev1, st));
        if (ctr) ctr->plain += M;
        return CK_OK;
    }
    return sw_batched_launch(in, out, M, d_sub, err, st, ctr, read_counters);
}

namespace {
bool g_profile = false;
cudaEvent_t g_ev[2] = {nullptr, nullptr};
bool g_ev_recorded = false;
}  // namespace

bool profile_events(cudaEvent_t *start, cudaEvent_t *stop) {
    if (!g_profile) return false;
    if (!g_ev[0]) {
        if (cudaEventCreate(&g_ev[0]) != cudaSuccess || cudaEventCreate(&g_ev[1]) != cudaSuccess) {
            g_profile = false;
            return false;
        }
    }
    *start = g_ev[0];
    *stop = g_ev[1];
    g_ev_recorded = true;
    return true;
}

// Copies `bytes` of host data into a scratch slot on `st`.
static void *upload(int slot, const void *host, size_t bytes, cudaStream_t st, int32_t *status) {
    void *d = scratch(slot, bytes, status);
    if (!d) return nullptr;
    if (bytes) {
        cudaError_t e = cudaMemcpyAsync(d, host, bytes, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) { *status = cuda_status(e, "cudaMemcpyAsync H2D"); return nullptr; }
    }
    return d;
}

static int32_t read_and_clear_error(cudaStream_t st) {
    int32_t status = CK_OK;
    int32_t *err = device_error_word(&status);
    if (!err) return status;
    int32_t h = 0;
    CK_CUDA(cudaMemcpyAsync(&h, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK_CUDA(cudaMemsetAsync(err, 0, sizeof(int32_t), st));
    CK_CUDA(cudaStreamSynchronize(st));
    if (h & ERRBIT_PAIR_INDEX) {
        set_error(CK_ERR_OUT_OF_RANGE, "pair index outside [0, n_seqs)");
        return CK_ERR_OUT_OF_RANGE;
    }
    if (h & ERRBIT_SEQ_EXTENT) {
        set_error(CK_ERR_OUT_OF_RANGE, "sequence extent outside the flat buffer");
        return CK_ERR_OUT_OF_RANGE;
    }
    if (h & ERRBIT_CAPACITY) {
        set_error(CK_ERR_CAPACITY, "Phase-B diagonal bins beyond the caller's bins_capacity (skipped)");
        return CK_ERR_CAPACITY;
    }
    if (h & ERRBIT_LIST) {
        set_error(CK_ERR_CAPACITY, "similar k-mer neighbour list beyond the caller's list_capacity (truncated)");
        return CK_ERR_CAPACITY;
    }
    if (h & ERRBIT_SCHEDULE) {
        set_error(CK_ERR_CUDA, "internal: a streamed warp-per-pair strip missed its start step");
        return CK_ERR_CUDA;
    }
    return CK_OK;
}

}  // namespace ck

using namespace ck;

extern "C" {

int32_t ck_version(void) { return 100; }

const char *ck_last_error(void) { return t_error.c_str(); }

int32_t ck_last_status(void) { return t_status; }

int32_t ck_device_count(void) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return 0;
    return n;
}

int32_t ck_sw_last_counters(int64_t *out6) {
    if (!out6) return CK_ERR_INVALID_ARGUMENT;
    out6[0] = t_counters.pairs;
    out6[1] = t_counters.cells;
    out6[2] = t_counters.batched;
    out6[3] = t_counters.plain;
    out6[4] = t_counters.rerun;
    out6[5] = t_counters.launches;
    return CK_OK;
}

int32_t ck_sw_last_wave_pairs(int64_t *out) {
    if (!out) return CK_ERR_INVALID_ARGUMENT;
    *out = t_counters.wave;
    return CK_OK;
}

static int32_t check_sw_args(const void *pairs, int64_t M, const void *flat, int64_t flat_len,
                             const void *offsets, const void *lengths, int64_t n_seqs,
                             const int8_t *sub, int32_t pass_rule, int32_t engine) {
    if (M < 0 || flat_len < 0 || n_seqs < 0) {
        set_error(CK_ERR_INVALID_ARGUMENT, "negative size");
        return CK_ERR_INVALID_ARGUMENT;
    }
    if ((M > 0 && !pairs) || (n_seqs > 0 && (!offsets || !lengths)) || (flat_len > 0 && !flat) || !sub) {
        set_error(CK_ERR_INVALID_ARGUMENT, "NULL input pointer");
        return CK_ERR_INVALID_ARGUMENT;
    }
    if (pass_rule < CK_PASS_CPU || pass_rule > CK_PASS_SCORE) {
        set_error(CK_ERR_INVALID_ARGUMENT, "unknown pass_rule");
        return CK_ERR_INVALID_ARGUMENT;
    }
    if (engine != CK_SW_BATCHED && engine != CK_SW_PLAIN) {
        set_error(CK_ERR_INVALID_ARGUMENT, "unknown engine");
        return CK_ERR_INVALID_ARGUMENT;
    }
    return CK_OK;
}

int32_t ck_sw_batch(const int32_t *pairs, int64_t M, const uint8_t *flat, int64_t flat_len,
                    const int64_t *offsets, const int32_t *lengths, int64_t n_seqs,
                    int32_t band_width, const int8_t *sub_matrix, float threshold,
                    const int32_t *diag_hints, int32_t pass_rule, int32_t engine,
                    float *out_sims, int32_t *out_scores, int32_t *out_matches,
                    int32_t *out_shorter, uint8_t *out_mask) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    t_counters = SwCounters{};
    CK_TRY(check_sw_args(pairs, M, flat, flat_len, offsets, lengths, n_seqs, sub_matrix, pass_rule, engine));
    int32_t status = CK_OK;
    cudaStream_t st = lib_stream(&status);
    if (status != CK_OK) return status;
    if (M == 0) return CK_OK;

    SwIn in{};
    in.pairs = (const int32_t *)upload(SLOT_HOST_IO0, pairs, (size_t)M * 8, st, &status);
    in.flat = (const uint8_t *)upload(SLOT_HOST_IO1, flat, (size_t)flat_len, st, &status);
    in.offsets = (const int64_t *)upload(SLOT_HOST_IO2, offsets, (size_t)n_seqs * 8, st, &status);
    in.lengths = (const int32_t *)upload(SLOT_HOST_IO3, lengths, (size_t)n_seqs * 4, st, &status);
    in.hints = diag_hints ? (const int32_t *)upload(SLOT_HOST_IO4, diag_hints, (size_t)M * 4, st, &status)
                          : nullptr;
    if (status != CK_OK) return status;
    in.n_seqs = n_seqs;
    in.flat_len = flat_len;
    in.band_width = band_width;
    in.threshold = threshold;
    in.pass_rule = pass_rule;

    // one output region: sims | scores | matches | shorter | mask
    const size_t m = (size_t)M;
    char *o = (char *)scratch(SLOT_HOST_IO5, m * 17 + 256, &status);
    if (!o) return status;
    SwOut out{};
    out.sims = out_sims ? (float *)o : nullptr;
    out.scores = out_scores ? (int32_t *)(o + m * 4) : nullptr;
    out.matches = out_matches ? (int32_t *)(o + m * 8) : nullptr;
    out.shorter = out_shorter ? (int32_t *)(o + m * 12) : nullptr;
    out.mask = out_mask ? (uint8_t *)(o + m * 16) : nullptr;

    CK_TRY(sw_run_device(in, out, M, engine, sub_matrix, st, &t_counters, true));
    if (out_sims) CK_CUDA(cudaMemcpyAsync(out_sims, out.sims, m * 4, cudaMemcpyDeviceToHost, st));
    if (out_scores) CK_CUDA(cudaMemcpyAsync(out_scores, out.scores, m * 4, cudaMemcpyDeviceToHost, st));
    if (out_matches) CK_CUDA(cudaMemcpyAsync(out_matches, out.matches, m * 4, cudaMemcpyDeviceToHost, st));
    if (out_shorter) CK_CUDA(cudaMemcpyAsync(out_shorter, out.shorter, m * 4, cudaMemcpyDeviceToHost, st));
    if (out_mask) CK_CUDA(cudaMemcpyAsync(out_mask, out.mask, m, cudaMemcpyDeviceToHost, st));
    return read_and_clear_error(st);
}

int32_t ck_sw_batch_device(const int32_t *d_pairs, int64_t M, const uint8_t *d_flat,
                           int64_t flat_len, const int64_t *d_offsets, const int32_t *d_lengths,
                           int64_t n_seqs, int32_t band_width, const int8_t *sub_matrix_host,
                           float threshold, const int32_t *d_diag_hints, int32_t pass_rule,
                           int32_t engine, float *d_sims, int32_t *d_scores, int32_t *d_matches,
                           int32_t *d_shorter, uint8_t *d_mask, void *stream) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    t_counters = SwCounters{};
    CK_TRY(check_sw_args(d_pairs, M, d_flat, flat_len, d_offsets, d_lengths, n_seqs, sub_matrix_host,
                         pass_rule, engine));
    if (M == 0) return CK_OK;
    SwIn in{d_pairs, d_flat, d_offsets, d_lengths, d_diag_hints, n_seqs, flat_len, band_width,
            threshold, pass_rule};
    SwOut out{d_sims, d_scores, d_matches, d_shorter, d_mask};
    return sw_run_device(in, out, M, engine, sub_matrix_host, (cudaStream_t)stream, &t_counters,
                         false);
}

int32_t ck_ctx_create(int32_t *out_handle) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    if (!out_handle) return CK_ERR_INVALID_ARGUMENT;
    int32_t status = CK_OK;
    if (!state(&status)) return status;
    ScratchSet *set = new ScratchSet();
    set->device = current_device();
    cudaError_t e = cudaMalloc(&set->err, 64);
    if (e != cudaSuccess) { delete set; return cuda_status(e, "cudaMalloc(context error word)"); }
    e = cudaMemset(set->err, 0, 64);
    if (e != cudaSuccess) { cudaFree(set->err); delete set; return cuda_status(e, "cudaMemset"); }
    for (size_t i = 0; i < g_ctx.size(); ++i)
        if (!g_ctx[i]) { g_ctx[i] = set; *out_handle = (int32_t)i + 1; return CK_OK; }
    g_ctx.push_back(set);
    *out_handle = (int32_t)g_ctx.size();
    return CK_OK;
}

int32_t ck_ctx_freeze(int32_t handle, int32_t frozen) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    if (handle < 1 || handle > (int32_t)g_ctx.size() || !g_ctx[handle - 1]) {
        set_error(CK_ERR_INVALID_ARGUMENT, "unknown context handle");
        return CK_ERR_INVALID_ARGUMENT;
    }
    g_ctx[handle - 1]->frozen = frozen != 0;
    return CK_OK;
}

int32_t ck_ctx_destroy(int32_t handle) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    if (handle < 1 || handle > (int32_t)g_ctx.size() || !g_ctx[handle - 1]) {
        set_error(CK_ERR_INVALID_ARGUMENT, "unknown context handle");
        return CK_ERR_INVALID_ARGUMENT;
    }
    ScratchSet *set = g_ctx[handle - 1];
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(set->device);
    cudaDeviceSynchronize();
    for (int i = 0; i < SLOT_COUNT; ++i)
        if (set->buf[i]) cudaFree(set->buf[i]);
    if (set->err) cudaFree(set->err);
    free_db(set);
    if (set->done) cudaEventDestroy(set->done);
    cudaSetDevice(prev);
    delete set;
    g_ctx[handle - 1] = nullptr;
    return CK_OK;
}

int32_t ck_ctx_status(int32_t handle, void *stream) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    return with_context(handle, [&] { return read_and_clear_error((cudaStream_t)stream); });
}

int32_t ck_sw_batch_device_ctx(int32_t ctx, const int32_t *d_pairs, int64_t M, const uint8_t *d_flat,
                               int64_t flat_len, const int64_t *d_offsets, const int32_t *d_lengths,
                               int64_t n_seqs, int32_t band_width, const int8_t *sub_matrix_host,
                               float threshold, const int32_t *d_diag_hints, int32_t pass_rule,
                               int32_t engine, float *d_sims, int32_t *d_scores, int32_t *d_matches,
                               int32_t *d_shorter, uint8_t *d_mask, void *stream) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    t_counters = SwCounters{};
    CK_TRY(check_sw_args(d_pairs, M, d_flat, flat_len, d_offsets, d_lengths, n_seqs, sub_matrix_host,
                         pass_rule, engine));
    if (M == 0) return CK_OK;
    SwIn in{d_pairs, d_flat, d_offsets, d_lengths, d_diag_hints, n_seqs, flat_len, band_width,
            threshold, pass_rule};
    SwOut out{d_sims, d_scores, d_matches, d_shorter, d_mask};
    return with_context(ctx, [&] {
        return sw_run_device(in, out, M, engine, sub_matrix_host, (cudaStream_t)stream, &t_counters,
                             false);
    });
}

// ------------------------------------------------ resident database, submit/poll
static ScratchSet *ctx_set(int32_t handle) {
    if (handle < 1 || handle > (int32_t)g_ctx.size() || !g_ctx[handle - 1]) {
        set_error(CK_ERR_INVALID_ARGUMENT, "unknown context handle");
        return nullptr;
    }
    ScratchSet *set = g_ctx[handle - 1];
    if (set->device != current_device()) {
        set_error(CK_ERR_INVALID_ARGUMENT, "context belongs to another device");
        return nullptr;
    }
    return set;
}

int32_t ck_ctx_upload_db(int32_t ctx, const uint8_t *flat, int64_t flat_len, const int64_t *offsets,
                         const int32_t *lengths, int64_t n_seqs) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    ScratchSet *set = ctx_set(ctx);
    if (!set) return CK_ERR_INVALID_ARGUMENT;
    if (flat_len < 0 || n_seqs < 0 || (flat_len > 0 && !flat) || (n_seqs > 0 && (!offsets || !lengths))) {
        set_error(CK_ERR_INVALID_ARGUMENT, "upload_db: NULL pointer or negative size");
        return CK_ERR_INVALID_ARGUMENT;
    }
    if (set->pending) {
        set_error(CK_ERR_INVALID_ARGUMENT, "upload_db: a submission on this context is still in flight");
        return CK_ERR_INVALID_ARGUMENT;
    }
    free_db(set);
    CK_CUDA(cudaMalloc(&set->db_flat, (size_t)(flat_len > 0 ? flat_len : 1)));
    CK_CUDA(cudaMalloc(&set->db_offsets, (size_t)(n_seqs > 0 ? n_seqs : 1) * 8));
    CK_CUDA(cudaMalloc(&set->db_lengths, (size_t)(n_seqs > 0 ? n_seqs : 1) * 4));
    if (flat_len) CK_CUDA(cudaMemcpy(set->db_flat, flat, (size_t)flat_len, cudaMemcpyHostToDevice));
    if (n_seqs) {
        CK_CUDA(cudaMemcpy(set->db_offsets, offsets, (size_t)n_seqs * 8, cudaMemcpyHostToDevice));
        CK_CUDA(cudaMemcpy(set->db_lengths, lengths, (size_t)n_seqs * 4, cudaMemcpyHostToDevice));
    }
    set->db_flat_len = flat_len;
    set->db_n = n_seqs;
    set->db_ready = true;
    return CK_OK;
}

int32_t ck_ctx_submit(int32_t ctx, const int32_t *pairs, int64_t M, int32_t band_width,
                      const int8_t *sub_matrix, float threshold, const int32_t *diag_hints,
                      int32_t pass_rule, int32_t engine, float *out_sims, int32_t *out_scores,
                      int32_t *out_matches, int32_t *out_shorter, uint8_t *out_mask, void *stream) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    t_counters = SwCounters{};
    ScratchSet *set = ctx_set(ctx);
    if (!set) return CK_ERR_INVALID_ARGUMENT;
    if (!set->db_ready) {
        set_error(CK_ERR_INVALID_ARGUMENT, "submit: no database uploaded to this context (ck_ctx_upload_db)");
        return CK_ERR_INVALID_ARGUMENT;
    }
    if (set->pending) {
        set_error(CK_ERR_INVALID_ARGUMENT, "submit: the previous submission on this context is still in "
                                           "flight (ck_ctx_poll / ck_ctx_wait it first)");
        return CK_ERR_INVALID_ARGUMENT;
    }
    CK_TRY(check_sw_args(pairs, M, set->db_flat, set->db_flat_len, set->db_offsets, set->db_lengths, set->db_n,
                         sub_matrix, pass_rule, engine));
    if (!set->done) CK_CUDA(cudaEventCreateWithFlags(&set->done, cudaEventDisableTiming));
    cudaStream_t st = (cudaStream_t)stream;
    return with_context(ctx, [&]() -> int32_t {
        int32_t status = CK_OK;
        const size_t m = (size_t)M;
        SwIn in{};
        in.pairs = m ? (const int32_t *)upload(SLOT_HOST_IO0, pairs, m * 8, st, &status) : nullptr;
        in.hints = (diag_hints && m) ? (const int32_t *)upload(SLOT_HOST_IO4, diag_hints, m * 4, st, &status)
                                     : nullptr;
        if (status != CK_OK) return status;
        in.flat = set->db_flat;
        in.offsets = set->db_offsets;
        in.lengths = set->db_lengths;
        in.n_seqs = set->db_n;
        in.flat_len = set->db_flat_len;
        in.band_width = band_width;
        in.threshold = threshold;
        in.pass_rule = pass_rule;
        if (m) {
            char *o = (char *)scratch(SLOT_HOST_IO5, m * 17 + 256, &status);
            if (!o) return status;
            SwOut out{};
            out.sims = out_sims ? (float *)o : nullptr;
            out.scores = out_scores ? (int32_t *)(o + m * 4) : nullptr;
            out.matches = out_matches ? (int32_t *)(o + m * 8) : nullptr;
            out.shorter = out_shorter ? (int32_t *)(o + m * 12) : nullptr;
            out.mask = out_mask ? (uint8_t *)(o + m * 16) : nullptr;
            CK_TRY(sw_run_device(in, out, M, engine, sub_matrix, st, &t_counters, false));
            if (out_sims) CK_CUDA(cudaMemcpyAsync(out_sims, out.sims, m * 4, cudaMemcpyDeviceToHost, st));
            if (out_scores) CK_CUDA(cudaMemcpyAsync(out_scores, out.scores, m * 4, cudaMemcpyDeviceToHost, st));
            if (out_matches)
                CK_CUDA(cudaMemcpyAsync(out_matches, out.matches, m * 4, cudaMemcpyDeviceToHost, st));
            if (out_shorter)
                CK_CUDA(cudaMemcpyAsync(out_shorter, out.shorter, m * 4, cudaMemcpyDeviceToHost, st));
            if (out_mask) CK_CUDA(cudaMemcpyAsync(out_mask, out.mask, m, cudaMemcpyDeviceToHost, st));
        }
        CK_CUDA(cudaEventRecord(set->done, st));
        set->pending_stream = st;
        set->pending = true;
        return CK_OK;
    });
}

// The submission's outcome once its event has completed: the context's GPU
// input checks since the last read.
static int32_t ctx_finish(int32_t ctx, ScratchSet *set) {
    set->pending = false;
    return with_context(ctx, [&] { return read_and_clear_error(set->pending_stream); });
}

int32_t ck_ctx_poll(int32_t ctx, int32_t *out_done) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    if (!out_done) return CK_ERR_INVALID_ARGUMENT;
    ScratchSet *set = ctx_set(ctx);
    if (!set) return CK_ERR_INVALID_ARGUMENT;
    *out_done = 1;
    if (!set->pending) return CK_OK;
    const cudaError_t e = cudaEventQuery(set->done);
    if (e == cudaErrorNotReady) {
        *out_done = 0;
        return CK_OK;
    }
    if (e != cudaSuccess) {
        set->pending = false;
        return cuda_status(e, "ck_ctx_poll");
    }
    return ctx_finish(ctx, set);
}

int32_t ck_ctx_wait(int32_t ctx) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    ScratchSet *set = ctx_set(ctx);
    if (!set) return CK_ERR_INVALID_ARGUMENT;
    if (!set->pending) return CK_OK;
    const cudaError_t e = cudaEventSynchronize(set->done);
    if (e != cudaSuccess) {
        set->pending = false;
        return cuda_status(e, "ck_ctx_wait");
    }
    return ctx_finish(ctx, set);
}

int32_t ck_sw_profile(int32_t enable) {
    std::lock_guard<std::mutex> lock(g_mutex);
    g_profile = enable != 0;
    g_ev_recorded = false;
    return CK_OK;
}

int32_t ck_sw_last_kernel_ms(float *out_ms) {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!out_ms) return CK_ERR_INVALID_ARGUMENT;
    *out_ms = -1.0f;
    if (!g_ev_recorded || !g_ev[1]) return CK_OK;
    CK_CUDA(cudaEventSynchronize(g_ev[1]));
    CK_CUDA(cudaEventElapsedTime(out_ms, g_ev[0], g_ev[1]));
    return CK_OK;
}

int32_t ck_sw_set_config(int32_t key, int32_t value) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    if (key == CK_CFG_ROWS_PER_STRIP) return sw_set_rows_per_strip(value);
    if (key == CK_CFG_STRIP_VARIANT) return sw_set_variant(value);
    if (key == CK_CFG_WAVE_MIN_ROWS) return sw_set_wave(0, value);
    if (key == CK_CFG_WAVE_ALL_BELOW) return sw_set_wave(1, value);
    if (key == CK_CFG_WAVE_ADAPTIVE) return sw_set_wave(2, value);
    if (key == CK_CFG_WAVE_STREAM) return sw_set_wave(3, value);
    if (key == CK_CFG_WAVE_ROWS) return sw_set_wave(4, value);
    if (key == CK_CFG_STRIP_THREADS) return sw_set_strip_threads(value);
    if (key == CK_CFG_STRIP_KEY) return sw_set_wide_key(value);
    set_error(CK_ERR_INVALID_ARGUMENT, "unknown config key");
    return CK_ERR_INVALID_ARGUMENT;
}

int32_t ck_sw_get_config(int32_t key, int32_t *value) {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!value) return CK_ERR_INVALID_ARGUMENT;
    if (key == CK_CFG_ROWS_PER_STRIP) { *value = sw_rows_per_strip(); return CK_OK; }
    if (key == CK_CFG_STRIP_VARIANT) { *value = sw_variant(); return CK_OK; }
    if (key == CK_CFG_WAVE_MIN_ROWS) { *value = sw_wave(0); return CK_OK; }
    if (key == CK_CFG_WAVE_ALL_BELOW) { *value = sw_wave(1); return CK_OK; }
    if (key == CK_CFG_WAVE_ADAPTIVE) { *value = sw_wave(2); return CK_OK; }
    if (key == CK_CFG_WAVE_STREAM) { *value = sw_wave(3); return CK_OK; }
    if (key == CK_CFG_WAVE_ROWS) { *value = sw_wave(4); return CK_OK; }
    if (key == CK_CFG_STRIP_THREADS) { *value = sw_strip_threads(); return CK_OK; }
    if (key == CK_CFG_STRIP_KEY) { *value = sw_wide_key(); return CK_OK; }
    set_error(CK_ERR_INVALID_ARGUMENT, "unknown config key");
    return CK_ERR_INVALID_ARGUMENT;
}

int32_t ck_sw_status_device(void *stream) {
    std::lock_guard<std::mutex> lock(g_mutex);
    return read_and_clear_error((cudaStream_t)stream);
}

void sw_set_num_threads(int32_t n) { (void)n; }

void batch_sw_align_c(const int32_t *pairs, const uint8_t *flat_sequences, const int64_t *offsets,
                      const int32_t *lengths, int32_t M, int32_t band_width,
                      const int8_t *sub_matrix, float threshold, const int32_t *diag_hints,
                      float *out_sims, int32_t *out_scores, uint8_t *out_mask) {
    // clustkit's entry point receives no array sizes: the number of
    // sequences is one past the largest pair index and the flat length the
    // furthest sequence end among them.
    int32_t status = CK_OK;
    int64_t n = 0, flat_len = 0;
    for (int64_t p = 0; p < 2 * (int64_t)M; ++p) {
        if (pairs[p] < 0) { status = CK_ERR_OUT_OF_RANGE; break; }
        n = std::max<int64_t>(n, (int64_t)pairs[p] + 1);
    }
    if (status == CK_OK)
        for (int64_t i = 0; i < n; ++i) flat_len = std::max<int64_t>(flat_len, offsets[i] + lengths[i]);
    if (status == CK_OK)
        status = ck_sw_batch(pairs, M, flat_sequences, flat_len, offsets, lengths, n, band_width,
                             sub_matrix, threshold, diag_hints, CK_PASS_SCORE, CK_SW_BATCHED,
                             out_sims, out_scores, nullptr, nullptr, out_mask);
    else
        set_error(status, "negative pair index");
    if (status != CK_OK) {
        for (int32_t p = 0; p < M; ++p) { out_sims[p] = 0.0f; out_scores[p] = 0; out_mask[p] = 0; }
        fprintf(stderr, "libckgpu batch_sw_align_c failed (%d): %s\n", status, t_error.c_str());
        t_status = status;
    }
}

int32_t ck_sketch(const uint8_t *flat, int64_t flat_len, const int64_t *offsets,
                  const int32_t *lengths, int64_t N, int32_t k, int32_t s, int32_t alphabet,
                  uint64_t seed, uint64_t *out) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    if (N < 0 || flat_len < 0 || (N > 0 && (!offsets || !lengths || !out)) || (flat_len > 0 && !flat)) {
        set_error(CK_ERR_INVALID_ARGUMENT, "sketch: bad pointer or size");
        return CK_ERR_INVALID_ARGUMENT;
    }
    int32_t status = CK_OK;
    cudaStream_t st = lib_stream(&status);
    if (status != CK_OK) return status;
    if (N == 0) return CK_OK;
    const uint8_t *d_flat = (const uint8_t *)upload(SLOT_HOST_IO1, flat, (size_t)flat_len, st, &status);
    const int64_t *d_off = (const int64_t *)upload(SLOT_HOST_IO2, offsets, (size_t)N * 8, st, &status);
    const int32_t *d_len = (const int32_t *)upload(SLOT_HOST_IO3, lengths, (size_t)N * 4, st, &status);
    uint64_t *d_out = (uint64_t *)scratch(SLOT_HOST_IO6, (size_t)N * s * 8, &status);
    int32_t *err = device_error_word(&status);
    if (status != CK_OK || !d_out || !err) return status != CK_OK ? status : CK_ERR_CUDA;
    CK_TRY(sketch_launch(d_flat, flat_len, d_off, d_len, N, k, s, alphabet, seed, d_out, err, st));
    CK_CUDA(cudaMemcpyAsync(out, d_out, (size_t)N * s * 8, cudaMemcpyDeviceToHost, st));
    return read_and_clear_error(st);
}

int32_t ck_sketch_device(const uint8_t *d_flat, int64_t flat_len, const int64_t *d_offsets,
                         const int32_t *d_lengths, int64_t N, int32_t k, int32_t s, int32_t alphabet,
                         uint64_t seed, uint64_t *d_out, void *stream) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    if (N < 0 || flat_len < 0) {
        set_error(CK_ERR_INVALID_ARGUMENT, "sketch: negative size");
        return CK_ERR_INVALID_ARGUMENT;
    }
    int32_t status = CK_OK;
    int32_t *err = device_error_word(&status);
    if (!err) return status;
    return sketch_launch(d_flat, flat_len, d_offsets, d_lengths, N, k, s, alphabet, seed, d_out, err,
                         (cudaStream_t)stream);
}

int32_t ck_jaccard(const int32_t *pairs, int64_t M, const uint64_t *sketches, int64_t N, int32_t s,
                   float floor, float *out_sims, uint8_t *out_mask) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    if (M < 0 || N < 0 || (M > 0 && (!pairs || !out_sims)) || (N > 0 && !sketches)) {
        set_error(CK_ERR_INVALID_ARGUMENT, "jaccard: bad pointer or size");
        return CK_ERR_INVALID_ARGUMENT;
    }
    int32_t status = CK_OK;
    cudaStream_t st = lib_stream(&status);
    if (status != CK_OK) return status;
    if (M == 0) return CK_OK;
    const int32_t *d_pairs = (const int32_t *)upload(SLOT_HOST_IO0, pairs, (size_t)M * 8, st, &status);
    const uint64_t *d_sk = (const uint64_t *)upload(SLOT_HOST_IO6, sketches, (size_t)N * s * 8, st, &status);
    char *o = (char *)scratch(SLOT_HOST_IO5, (size_t)M * 5 + 256, &status);
    int32_t *err = device_error_word(&status);
    if (status != CK_OK || !o || !err) return status != CK_OK ? status : CK_ERR_CUDA;
    float *d_sims = (float *)o;
    uint8_t *d_mask = out_mask ? (uint8_t *)(o + (size_t)M * 4) : nullptr;
    CK_TRY(jaccard_launch(d_pairs, M, d_sk, N, s, floor, d_sims, d_mask, err, st));
    CK_CUDA(cudaMemcpyAsync(out_sims, d_sims, (size_t)M * 4, cudaMemcpyDeviceToHost, st));
    if (out_mask) CK_CUDA(cudaMemcpyAsync(out_mask, d_mask, (size_t)M, cudaMemcpyDeviceToHost, st));
    return read_and_clear_error(st);
}

int32_t ck_jaccard_device(const int32_t *d_pairs, int64_t M, const uint64_t *d_sketches, int64_t N,
                          int32_t s, float floor, float *d_sims, uint8_t *d_mask, void *stream) {
    std::lock_guard<std::mutex> lock(g_mutex);
    t_status = CK_OK;
    if (M < 0 || N < 0) {
        set_error(CK_ERR_INVALID_ARGUMENT, "jaccard: negative size");
        return CK_ERR_INVALID_ARGUMENT;
    }
    int32_t status = CK_OK;
    int32_t *err = device_error_word(&status);
    if (!err) return status;
    return jaccard_launch(d_pairs, M, d_sketches, N, s, floor, d_sims, d_mask, err, (cudaStream_t)stream);
}

}  // extern "C"
