// sw_noalloc.cu -- the allocation-free Smith-Waterman entry point.
//
// Some callers cannot let a library allocate GPU memory: an aligner embedded
// in a host system that owns every byte of device memory (a pre-sized pool
// handed out by a database engine or pipeline framework, where an outside
// cudaMalloc would break its accounting or fail), or a latency-bound serving
// loop in which an allocation could stall or fail in the middle of a request.
// ck_sw_batch_device_noalloc serves them: the caller passes device buffers
// for inputs and outputs, and the only other memory it touches is declared
// in this file as static __device__ arrays, which exist from the moment the
// library is loaded on a GPU until the process exits.
//
// It runs the plain Smith-Waterman kernel (one thread per pair, same
// results as every other entry point) with that kernel's per-thread
// workspace carved out of g_noalloc_ws instead of library scratch.
#include <mutex>

#include "ck_common.cuh"

namespace ck {

// Declared here, defined in sw_plain.cu.
__global__ void __launch_bounds__(128)
sw_plain_kernel(SwIn in, SwOut out, int64_t M, const int32_t *__restrict__ index,
                                const int32_t *__restrict__ count_dev,
                                const int8_t *__restrict__ sub, int4 *__restrict__ ws,
                                int32_t ws_stride, int32_t *err);

// 32 MiB of workspace: (2 * band + 2) int4 per thread, so band width 100
// leaves room for 10,368 threads and the widest band accepted is 8191.
constexpr size_t NOALLOC_WS_BYTES = (size_t)32 << 20;
constexpr int NOALLOC_THREADS = 128;

static __device__ __align__(256) int4 g_noalloc_ws[NOALLOC_WS_BYTES / sizeof(int4)];
static __device__ __align__(256) int8_t g_noalloc_sub[512];
static __device__ __align__(256) int32_t g_noalloc_err[64];

namespace {
constexpr int MAX_DEV = 16;
struct NoallocDev {
    std::mutex lock;  // one call at a time per device: they share that device's arrays
    bool ready = false;
    int4 *ws = nullptr;
    int8_t *sub = nullptr;
    int32_t *err = nullptr;
    int sms = 0;
};
NoallocDev g_na[MAX_DEV];
}  // namespace

// The current device's entry, or an error for an ordinal beyond the table.
static int32_t noalloc_device(NoallocDev **out, int *ordinal) {
    int d = 0;
    CK_CUDA(cudaGetDevice(&d));
    if (d < 0 || d >= MAX_DEV) {
        set_error(CK_ERR_NO_DEVICE, "device ordinal out of range");
        return CK_ERR_NO_DEVICE;
    }
    *out = &g_na[d];
    *ordinal = d;
    return CK_OK;
}

// Device addresses of the static arrays, looked up once per device with that
// device current (the caller holds the device's lock).  The host-side names
// of __device__ arrays are stand-ins, not device addresses, so they are never
// handed to a kernel directly.  The addresses belong to the device's primary
// context: after cudaDeviceReset in this process they are stale, and this
// entry point is not to be used again on that device.
static int32_t noalloc_setup(NoallocDev &s, int d) {
    if (!s.ready) {
        CK_CUDA(cudaGetSymbolAddress((void **)&s.ws, g_noalloc_ws));
        CK_CUDA(cudaGetSymbolAddress((void **)&s.sub, g_noalloc_sub));
        CK_CUDA(cudaGetSymbolAddress((void **)&s.err, g_noalloc_err));
        CK_CUDA(cudaDeviceGetAttribute(&s.sms, cudaDevAttrMultiProcessorCount, d));
        s.ready = true;
    }
    return CK_OK;
}

}  // namespace ck

using namespace ck;

extern "C" int32_t ck_sw_batch_device_noalloc(
    const int32_t *d_pairs, int64_t M, const uint8_t *d_flat, int64_t flat_len,
    const int64_t *d_offsets, const int32_t *d_lengths, int64_t n_seqs, int32_t band_width,
    const int8_t *sub_matrix_host, float threshold, const int32_t *d_diag_hints, int32_t pass_rule,
    float *d_sims, int32_t *d_scores, int32_t *d_matches, int32_t *d_shorter, uint8_t *d_mask,
    void *stream) {
    if (M < 0 || flat_len < 0 || n_seqs < 0 || !sub_matrix_host ||
        (M > 0 && !d_pairs) || (n_seqs > 0 && (!d_offsets || !d_lengths)) || (flat_len > 0 && !d_flat)) {
        set_error(CK_ERR_INVALID_ARGUMENT, "noalloc: NULL pointer or negative size");
        return CK_ERR_INVALID_ARGUMENT;
    }
    if (pass_rule < CK_PASS_CPU || pass_rule > CK_PASS_SCORE) {
        set_error(CK_ERR_INVALID_ARGUMENT, "noalloc: unknown pass_rule");
        return CK_ERR_INVALID_ARGUMENT;
    }
    // Every pair's band half-width is band_width, or its longer length when
    // that is <= 50; band_width <= 0 (full matrix) needs up to the longest
    // sequence and is not taken here.
    if (band_width <= 0) {
        set_error(CK_ERR_UNSUPPORTED, "noalloc: band_width must be >= 1 (full-matrix mode needs "
                                      "ck_sw_batch_device)");
        return CK_ERR_UNSUPPORTED;
    }
    const int64_t wmax = band_width > 50 ? band_width : 50;
    const int64_t stride = 2 * wmax + 2;  // int4 per thread
    int64_t threads = (int64_t)(NOALLOC_WS_BYTES / sizeof(int4)) / stride;
    threads = threads / NOALLOC_THREADS * NOALLOC_THREADS;
    if (threads < NOALLOC_THREADS) {
        set_error(CK_ERR_UNSUPPORTED, "noalloc: band_width above 8191 does not fit the 32 MiB "
                                      "static workspace");
        return CK_ERR_UNSUPPORTED;
    }
    NoallocDev *dev = nullptr;
    int ordinal = 0;
    CK_TRY(noalloc_device(&dev, &ordinal));
    // Calls on one device are serialised here and each returns only after its
    // kernel has finished, so within this process two calls never use the
    // device's arrays at the same time; calls on different devices run in
    // parallel (each device has its own copy of the arrays).
    std::lock_guard<std::mutex> lock(dev->lock);
    CK_TRY(noalloc_setup(*dev, ordinal));
    if (M == 0) return CK_OK;
    const int64_t cap = (int64_t)dev->sms * 8 * NOALLOC_THREADS;
    if (threads > cap) threads = cap;
    const int64_t want = (M + NOALLOC_THREADS - 1) / NOALLOC_THREADS * NOALLOC_THREADS;
    if (threads > want) threads = want;

    cudaStream_t st = (cudaStream_t)stream;
    CK_CUDA(cudaMemcpyAsync(dev->sub, sub_matrix_host, 400, cudaMemcpyHostToDevice, st));
    CK_CUDA(cudaMemsetAsync(dev->err, 0, sizeof(int32_t), st));
    SwIn in{d_pairs, d_flat, d_offsets, d_lengths, d_diag_hints, n_seqs, flat_len, band_width,
            threshold, pass_rule};
    SwOut out{d_sims, d_scores, d_matches, d_shorter, d_mask};
    sw_plain_kernel<<<(int)(threads / NOALLOC_THREADS), NOALLOC_THREADS, 0, st>>>(
        in, out, M, nullptr, nullptr, dev->sub, dev->ws, (int32_t)stride, dev->err);
    CK_CUDA(cudaGetLastError());
    int32_t h = 0;
    CK_CUDA(cudaMemcpyAsync(&h, dev->err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK_CUDA(cudaStreamSynchronize(st));
    if (h & (ERRBIT_PAIR_INDEX | ERRBIT_SEQ_EXTENT)) {
        set_error(CK_ERR_OUT_OF_RANGE, "noalloc: pair index or sequence extent out of range");
        return CK_ERR_OUT_OF_RANGE;
    }
    return CK_OK;
}
