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

// ---------------------------------------------------------------- cell forms
// Cell-rate probes of three forms of the Smith-Waterman cell, each run as the
// strip kernel runs it (a lane holds the H and F values of 16 rows and sweeps
// columns), on registers and a shared-memory increment table only -- no
// window, residue stream or first-max tracking -- so they compare the
// arithmetic of the forms, not the kernels around them:
//   0  the int32 packed key this library uses (score, priority, tie, match
//      count in one int32; exact): 4 DPX + 3 logic ops + 3 adds + 1 LDS;
//   1  int16x2, score only (two pairs per lane, one per 16-bit half): no
//      priority, tie or match count, so it cannot give clustkit's identity;
//      E and F are kept offset by their row / column index so that each
//      update is one DPX op: 5 DPX + 1 PRMT + 2 LDS per cell pair;
//   2  int16x2 with the match count carried in a second int16x2 register:
//      each max picks its winner's count through a compare mask and a
//      select, as exact tracking at two pairs per lane would need;
//   3  form 0 with the strip's lower 8 rows one column behind the upper 8:
//      the lower half's top row takes the upper half's bottom row as it stood
//      a column earlier, so a column holds two independent 8-row chains;
//   4  a compact key: 11-bit match count and a 3-bit extension counter (each
//      gap extension adds 1, so it wins ties against an opening) in place of
//      the tie bit, cleared every 4 rows (E) and every 2 columns (F) instead
//      of a tie bit set after every max.
// Each reports DP cells per second (forms 1 and 2: two cells per lane op).
// Every table index is (arow + bcol) >> 2 with arow <= 31 * 128 and bcol <=
// 31 * 4, so below 1024, and t ^ 16 stays below 1024 too.
template <int FORM>
__global__ void __launch_bounds__(256, 2) cell_probe_kernel(int32_t cols, int32_t seed, int32_t *sink) {
    __shared__ int32_t tab[32 * 32];
    for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x)
        tab[t] = ((t * 7 + seed) % 23 - 11) << ((FORM == 0 || FORM >= 3) ? 16 : 0);
    __syncthreads();
    constexpr int R = 16;
    const int lane = threadIdx.x & 31;
    int32_t hc[R], fT[R], mh[R], mf[R];
    uint32_t arow[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        hc[r] = 0;
        fT[r] = (FORM == 0 || FORM >= 3) ? -(16 << 16) : (int32_t)0x80408040u;
        mh[r] = 0;
        mf[r] = 0;
        arow[r] = (uint32_t)(((r * 5 + seed + threadIdx.x) & 31) * 32 * 4);
    }
    int32_t hd0 = 0, e_in = (FORM == 0 || FORM >= 3) ? -(16 << 16) : (int32_t)0x80408040u, acc = 0;
    int32_t h_mid = 0, e_mid = -(16 << 16), h_mid_prev = 0;  // form 3: the upper half's bottom row, delayed
    for (int32_t j = 0; j < cols; ++j) {
        const uint32_t bcol = (uint32_t)(((j * 13 + lane) & 31) * 4);
        const uint32_t offj = (uint32_t)(((j - 10) & 0xffff) * 0x10001u);
        const uint32_t negj = (uint32_t)(((-j) & 0xffff) * 0x10001u);
        int32_t hu = (j * 3) & 0xff, eu = e_in, hdiag = hd0, mu = 0, me = 0;
        hd0 = hu;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (FORM == 3 && r == R / 2) {
                // lower half one column behind: its top row reads the upper half's
                // bottom row as it stood after the previous column, not this one
                const int32_t h_now = hu, e_now = eu;
                hu = h_mid;
                eu = e_mid;
                hdiag = h_mid_prev;
                h_mid_prev = h_mid;
                h_mid = h_now;
                e_mid = e_now;
            }
            const uint32_t t = (arow[r] + bcol) >> 2;
            if (FORM == 4) {
                // compact key: 11-bit match count, a 3-bit extension counter in
                // bits 11..13 instead of a tie bit; E's counter cleared every 4
                // rows, F's every 2 columns, H cleaned as before
                constexpr int32_t CM = 7 << 11;
                const int32_t inc = tab[t];
                const int32_t diagc = __viaddmax_s32(hdiag, inc, 3 << 14);
                const int32_t eR = __viaddmax_s32(hu, (-11 << 16) + (1 << 14), eu + (-1 << 16) + (1 << 11));
                const int32_t fTn = __viaddmax_s32(fT[r], (-1 << 16) + (1 << 11), hc[r] + (-11 << 16));
                const int32_t hn = __vimax3_s32(diagc, eR, fTn) & ~(CM | (3 << 14));
                hdiag = hc[r];
                hc[r] = hn;
                fT[r] = fTn;
                hu = hn;
                eu = (r & 3) == 3 ? (eR & ~CM) : eR;
            } else if (FORM == 0 || FORM == 3) {
                const int32_t inc = tab[t];
                const int32_t diagc = __viaddmax_s32(hdiag, inc, 3 << 14);
                const int32_t eR = __viaddmax_s32(hu, (-11 << 16) + (1 << 14), eu + (-1 << 16));
                const int32_t fTn = __viaddmax_s32(fT[r], -1 << 16, hc[r] + (-11 << 16)) | (1 << 13);
                const int32_t hn = __vimax3_s32(diagc, eR, fTn) & ~((1 << 13) | (3 << 14));
                hdiag = hc[r];
                hc[r] = hn;
                fT[r] = fTn;
                hu = hn;
                eu = eR | (1 << 13);
            } else {
                // two pairs' increments: two table reads, packed into halves
                const uint32_t inc = __byte_perm((uint32_t)tab[t], (uint32_t)tab[t ^ 16u], 0x5410);
                const uint32_t offr = (uint32_t)(((r - 10) & 0xffff) * 0x10001u);
                const uint32_t negr = (uint32_t)(((-r) & 0xffff) * 0x10001u);
                const uint32_t diag = __viaddmax_s16x2((uint32_t)hdiag, inc, 0u);
                const uint32_t e_term = __viaddmax_s16x2((uint32_t)eu, negr, diag);
                const uint32_t hn = __viaddmax_s16x2((uint32_t)fT[r], negj, e_term);
                if (FORM == 2) {
                    // the winner's match count: diagonal (+1 on a match), else E's or F's count
                    const uint32_t from_diag = __vcmpeq2(hn, diag);
                    const uint32_t from_e = __vcmpeq2(hn, __viaddmax_s16x2((uint32_t)eu, negr, 0x80008000u));
                    const uint32_t md = (uint32_t)mh[r] + (inc & 0x00010001u);
                    const uint32_t m_ef = (from_e & (uint32_t)me) | (~from_e & (uint32_t)mf[r]);
                    const uint32_t mn = (from_diag & md) | (~from_diag & m_ef);
                    mu = (int32_t)mn;
                    // E's and F's counts follow their own extend / open choice
                    const uint32_t e_next = __viaddmax_s16x2(hn, offr, (uint32_t)eu);
                    const uint32_t e_open = __vcmpeq2(e_next, __viaddmax_s16x2(hn, offr, 0x80008000u));
                    me = (int32_t)((e_open & mn) | (~e_open & (uint32_t)me));
                    const uint32_t f_next = __viaddmax_s16x2(hn, offj, (uint32_t)fT[r]);
                    const uint32_t f_open = __vcmpeq2(f_next, __viaddmax_s16x2(hn, offj, 0x80008000u));
                    mf[r] = (int32_t)((f_open & mn) | (~f_open & (uint32_t)mf[r]));
                    mh[r] = (int32_t)mn;
                    eu = (int32_t)e_next;
                    fT[r] = (int32_t)f_next;
                } else {
                    eu = (int32_t)__viaddmax_s16x2(hn, offr, (uint32_t)eu);
                    fT[r] = (int32_t)__viaddmax_s16x2(hn, offj, (uint32_t)fT[r]);
                }
                hdiag = hc[r];
                hc[r] = (int32_t)hn;
                hu = (int32_t)hn;
            }
        }
        e_in = eu;
        acc ^= hu ^ mu;
        if (FORM == 4 && (j & 1)) {
#pragma unroll
            for (int r = 0; r < R; ++r) fT[r] &= ~(7 << 11);
        }
    }
    if (acc == 0x7fffabcd) sink[0] = acc;  // keeps the chains live
}

}  // namespace ck

using namespace ck;

extern "C" int32_t ck_probe_cell_rate(int32_t form, double *out_cells_per_s) {
    if (!out_cells_per_s || form < 0 || form > 4) {
        set_error(CK_ERR_INVALID_ARGUMENT, "cell probe: bad argument");
        return CK_ERR_INVALID_ARGUMENT;
    }
    int32_t status = CK_OK;
    int32_t *sink = (int32_t *)scratch(SLOT_MAXLEN, 64, &status);
    if (!sink) return status;
    const int blocks = sm_count() * 2, threads = 256;
    const int32_t cols = 4096;
    cudaEvent_t e0, e1;
    CK_CUDA(cudaEventCreate(&e0));
    CK_CUDA(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        CK_CUDA(cudaEventRecord(e0, 0));
        switch (form) {
            case 0: cell_probe_kernel<0><<<blocks, threads>>>(cols, rep + 3, sink); break;
            case 1: cell_probe_kernel<1><<<blocks, threads>>>(cols, rep + 3, sink); break;
            case 2: cell_probe_kernel<2><<<blocks, threads>>>(cols, rep + 3, sink); break;
            case 3: cell_probe_kernel<3><<<blocks, threads>>>(cols, rep + 3, sink); break;
            default: cell_probe_kernel<4><<<blocks, threads>>>(cols, rep + 3, sink); break;
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
    const double cells = (double)blocks * threads * cols * 16.0 * ((form == 1 || form == 2) ? 2.0 : 1.0);
    *out_cells_per_s = cells / (best_ms * 1e-3);
    return CK_OK;
}

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
