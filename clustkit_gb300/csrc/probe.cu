// probe.cu -- sustained lane-operation rate of the integer instructions the
// SW kernels are built from, measured on the running GPU.  This is the
// roofline denominator for the SW kernels, which are bound by integer issue,
// not by HBM or tensor throughput.
//
// Each thread keeps 8 registers and updates each from two others per step
// (x[q] = op(x[q], x[q+1], x[q+3])), so no chain can be folded at compile
// time and every warp has 8-way independent work; the grid is 2 CTAs x 1024
// threads per SM.
#include "ck_common.cuh"

namespace ck {

template <int WHICH>
__global__ void __launch_bounds__(1024) probe_kernel(int32_t iters, int32_t seed, int32_t *sink) {
    int32_t x[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = (int32_t)(threadIdx.x * 8 + q) ^ (seed * (q + 1));
    for (int32_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int32_t b = x[(q + 1) & 7], c = x[(q + 3) & 7];
                if (WHICH == 0) x[q] = __viaddmax_s32(x[q], b, c);
                else if (WHICH == 1) x[q] = __vimax3_s32(x[q], b, c);
                else if (WHICH == 2) x[q] = x[q] + b + c;
                else if (WHICH == 3) x[q] = (int32_t)__viaddmax_s16x2((uint32_t)x[q], (uint32_t)b, (uint32_t)c);
                else if (WHICH == 4) x[q] = (x[q] & b) ^ c;
                else x[q] = x[q] * b + c;
            }
        }
    }
    int32_t acc = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) acc ^= x[q];
    if (acc == 0x7fffabcd) sink[0] = acc;  // keeps the chains live
}

}  // namespace ck

using namespace ck;

extern "C" int32_t ck_probe_int_rate(int32_t which, double *out_ops_per_s) {
    if (!out_ops_per_s || which < 0 || which > 5) {
        set_error(CK_ERR_INVALID_ARGUMENT, "probe: bad argument");
        return CK_ERR_INVALID_ARGUMENT;
    }
    int32_t status = CK_OK;
    int32_t *sink = (int32_t *)scratch(SLOT_MAXLEN, 64, &status);
    if (!sink) return status;
    const int blocks = sm_count() * 2, threads = 1024;
    const int32_t iters = 1024;
    cudaEvent_t e0, e1;
    CK_CUDA(cudaEventCreate(&e0));
    CK_CUDA(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        CK_CUDA(cudaEventRecord(e0, 0));
        switch (which) {
            case 0: probe_kernel<0><<<blocks, threads>>>(iters, rep + 7, sink); break;
            case 1: probe_kernel<1><<<blocks, threads>>>(iters, rep + 7, sink); break;
            case 2: probe_kernel<2><<<blocks, threads>>>(iters, rep + 7, sink); break;
            case 3: probe_kernel<3><<<blocks, threads>>>(iters, rep + 7, sink); break;
            case 4: probe_kernel<4><<<blocks, threads>>>(iters, rep + 7, sink); break;
            default: probe_kernel<5><<<blocks, threads>>>(iters, rep + 7, sink); break;
        }
        CK_CUDA(cudaGetLastError());
        CK_CUDA(cudaEventRecord(e1, 0));
        CK_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        CK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best_ms) best_ms = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double instr = (double)blocks * threads * iters * 16.0 * 8.0;
    const double lanes = which == 3 ? 2.0 : 1.0;
    *out_ops_per_s = instr * lanes / (best_ms * 1e-3);
    return CK_OK;
}
