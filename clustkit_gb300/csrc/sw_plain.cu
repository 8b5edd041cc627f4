// sw_plain.cu -- the plain GPU form of clustkit's banded Smith-Waterman.
//
// One thread per pair, unbinned, one launch per chunk of pairs.  The
// recurrence is clustkit's (clustkit/csrc/sw_align.c:25-177): BLOSUM62 lookup
// with -4 for codes >= 20, affine gaps -11/-1 with extension preferred on
// ties, H = max(0, diag, E, F) with priority 0 > diag > E > F, match counts
// carried with the winning term, and the first row-major cell reaching the
// best score supplies the identity numerator.
//
// Plain int32 throughout (no packing), so it takes every pair: any length,
// any residue code.  The batched engine sends it the pairs its packed lanes
// cannot hold.
//
// Workspace: one row of (H, E, Hm, Em) per thread indexed band-relative,
// k = j - (i + h) + w, updated in place.  Row i-1's column j lives at k + 1
// when row i visits column j, so a left-to-right sweep reads k + 1 before
// overwriting k.  Index 2w + 1 is never written and keeps the out-of-band
// boundary (H = 0, E = -inf); indices left of a row's first column keep
// their initial zeros, which is column 0.
#include "ck_common.cuh"

namespace ck {

__global__ void __launch_bounds__(128)
sw_plain_kernel(SwIn in, SwOut out, int64_t M, const int32_t *__restrict__ index,
                const int32_t *__restrict__ count_dev, const int8_t *__restrict__ sub,
                int4 *__restrict__ ws, int32_t ws_stride, int32_t *err) {
    __shared__ int8_t s_sub[400];
    for (int t = threadIdx.x; t < 400; t += blockDim.x) s_sub[t] = sub[t];
    __syncthreads();

    const int64_t n = count_dev ? (int64_t)*count_dev : M;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int4 *W = ws + tid * (int64_t)ws_stride;

    for (int64_t t = tid; t < n; t += stride) {
        const int64_t p = index ? (int64_t)index[t] : t;
        PairGeom g = pair_geometry(in, p, err);
        if (!g.valid) {
            write_result(out, in, p, 0, 0, 0, 0, 0);
            continue;
        }
        const int32_t la = g.la, lb = g.lb, w = g.w, h = g.h;
        if (la == 0 || cupy_ratio_skip(in, la, lb)) {
            write_result(out, in, p, 0, 0, la, la, lb);
            continue;
        }
        const uint8_t *A = in.flat + in.offsets[g.a_idx];
        const uint8_t *B = in.flat + in.offsets[g.b_idx];
        const int32_t span = 2 * w + 2;
        for (int32_t k = 0; k < span; ++k) W[k] = make_int4(0, NEG_INF, 0, 0);

        int32_t best = 0, bestm = 0;
        for (int32_t i = 1; i <= la; ++i) {
            const int64_t lo = (int64_t)i + h - w, hi = (int64_t)i + h + w;
            if (hi < 1) continue;   // band left of column 1 (diagonal hints only)
            if (lo > lb) break;     // band right of the last column
            const int32_t js = lo < 1 ? 1 : (int32_t)lo;
            const int32_t je = hi > lb ? lb : (int32_t)hi;
            const int32_t base = w - i - h;  // k = j + base
            const uint8_t ai = A[i - 1];
            const int8_t *srow = s_sub + (ai < 20 ? ai * 20 : 0);

            int4 d = W[js + base];
            int32_t hd = d.x, hmd = d.z;
            int32_t hl = 0, hml = 0, f = NEG_INF, fm = 0;
            for (int32_t j = js; j <= je; ++j) {
                const int32_t k = j + base;
                const int4 u = W[k + 1];
                const uint8_t bj = B[j - 1];
                const int32_t s = (ai < 20 && bj < 20) ? (int32_t)srow[bj] : -4;
                const int32_t diag = hd + s;
                const int32_t diag_m = hmd + (ai == bj ? 1 : 0);

                int32_t e, em;
                if (u.y + GAP_EXTEND >= u.x + GAP_OPEN) { e = u.y + GAP_EXTEND; em = u.w; }
                else { e = u.x + GAP_OPEN; em = u.z; }

                const int32_t fx = (j > js) ? f + GAP_EXTEND : NEG_INF;
                if (fx >= hl + GAP_OPEN) { f = fx; }
                else { f = hl + GAP_OPEN; fm = hml; }

                int32_t hh = 0, hm = 0;
                if (diag > hh) { hh = diag; hm = diag_m; }
                if (e > hh) { hh = e; hm = em; }
                if (f > hh) { hh = f; hm = fm; }
                if (hh > best) { best = hh; bestm = hm; }

                W[k] = make_int4(hh, e, hm, em);
                hd = u.x; hmd = u.z;
                hl = hh; hml = hm;
            }
        }
        write_result(out, in, p, best, bestm, la, la, lb);
    }
}

__global__ void max_len_kernel(const int32_t *lengths, int64_t n, int32_t *out) {
    int32_t m = 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x)
        m = max(m, lengths[t]);
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Widest band half-width any pair of this call can use.
int32_t widest_band(const SwIn &in, cudaStream_t st, int32_t *w_out) {
    if (in.band_width > 0) {
        *w_out = in.band_width > 50 ? in.band_width : 50;
        return CK_OK;
    }
    int32_t status = CK_OK;
    int32_t *d = (int32_t *)scratch(SLOT_MAXLEN, 64, &status);
    if (!d) return status;
    CK_CUDA(cudaMemsetAsync(d, 0, sizeof(int32_t), st));
    int64_t n = in.n_seqs;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    max_len_kernel<<<blocks, 256, 0, st>>>(in.lengths, n, d);
    CK_CUDA(cudaGetLastError());
    int32_t m = 0;
    CK_CUDA(cudaMemcpyAsync(&m, d, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK_CUDA(cudaStreamSynchronize(st));
    *w_out = m > 50 ? m : 50;
    return CK_OK;
}

// Launch the plain kernel over pairs [0, M) (index == NULL) or over the
// device-resident list index[0 .. *d_count).
int32_t sw_plain_launch(const SwIn &in, const SwOut &out, int64_t M, const int32_t *d_index,
                        const int32_t *d_count, int32_t *d_err, cudaStream_t st,
                        SwCounters *ctr) {
    int32_t status = CK_OK;
    const int8_t *sub = device_sub_matrix(nullptr, &status);
    if (!sub) return status;
    int32_t wmax = 0;
    CK_TRY(widest_band(in, st, &wmax));
    const int64_t stride = 2 * (int64_t)wmax + 2;
    // Workspace budget: at most 4 GiB, at most one slot per work item.
    const int64_t budget = (int64_t)4 << 30;
    int64_t slots = budget / (stride * (int64_t)sizeof(int4));
    const int64_t want = d_count ? (int64_t)sm_count() * 8 * 128 : M;
    if (slots > want) slots = want;
    slots = (slots + 127) / 128 * 128;
    if (slots < 128) slots = 128;
    int4 *ws = (int4 *)scratch(SLOT_PLAIN_WS, (size_t)(slots * stride * sizeof(int4)), &status);
    if (!ws) return status;
    if (!d_count && M == 0) return CK_OK;
    const int blocks = (int)(slots / 128);
    sw_plain_kernel<<<blocks, 128, 0, st>>>(in, out, M, d_index, d_count, sub, ws,
                                             (int32_t)stride, d_err);
    CK_CUDA(cudaGetLastError());
    if (ctr) ctr->launches += 1;
    return CK_OK;
}

}  // namespace ck
