// jaccard.cu -- merge-walk Jaccard of sorted MinHash sketches
// (clustkit/pairwise.py:1564-1612) and the pre-filter mask
// (clustkit/pairwise.py:949-1001).
//
// clustkit walks the two sorted sketches A and B with two heads: equal heads
// are one shared step that advances both, otherwise the smaller head
// advances; it stops after s steps or when both heads are UINT64_MAX, and
// J = shared / steps.  Here one warp evaluates a pair without walking: with
// A and B in shared memory, every element A[i] of value v knows
//   lowB = #B < v, cntB = #B == v, firstA = index of the first v in A,
// it is paired (consumed in the same step as a B element) iff
// v != MAX and i - firstA < cntB, and it is consumed at step
//   i + lowB - P(firstA),  P(x) = number of paired elements among A[0..x),
// because every step before it consumed either an A element before i, a B
// element below v, or both at once (a paired step).  The walk takes
// T = #nonMAX(A) + #nonMAX(B) - #pairs steps in all, so
//   steps  = min(s, T),  shared = #paired A elements consumed at step < s.
// J = shared / steps is the float32 rounding of the quotient, as clustkit's
// float32(shared / union) gives for these small integers.
#include "ck_common.cuh"

namespace ck {

__device__ __forceinline__ int lower_bound_u64(const uint64_t *a, int n, uint64_t v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ int upper_bound_u64(const uint64_t *a, int n, uint64_t v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void jaccard_kernel(const int32_t *__restrict__ pairs, int64_t M,
                               const uint64_t *__restrict__ sk, int64_t N, int32_t s, float floor,
                               float *__restrict__ sims, uint8_t *__restrict__ mask, int32_t *err) {
    extern __shared__ uint64_t s_mem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    uint64_t *A = s_mem + (size_t)wib * (2 * s + s / 2 + 2);
    uint64_t *B = A + s;
    int32_t *P = (int32_t *)(B + s);  // s + 1 prefix counts
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t MAXV = ~0ULL;

    for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < M; p += warps) {
        const int32_t ia = pairs[2 * p], ib = pairs[2 * p + 1];
        if (ia < 0 || ib < 0 || ia >= N || ib >= N) {
            if (lane == 0) {
                atomicOr(err, ERRBIT_PAIR_INDEX);
                sims[p] = 0.0f;
                if (mask) mask[p] = 0;
            }
            continue;
        }
        const uint64_t *ga = sk + (int64_t)ia * s, *gb = sk + (int64_t)ib * s;
        for (int t = lane; t < s; t += 32) { A[t] = ga[t]; B[t] = gb[t]; }
        __syncwarp();
        // pass 1: paired flags -> exclusive prefix P over A
        int32_t run = 0;
        for (int base = 0; base < s; base += 32) {
            const int i = base + lane;
            int paired = 0;
            if (i < s) {
                const uint64_t v = A[i];
                if (v != MAXV) {
                    const int fa = lower_bound_u64(A, s, v);
                    const int lb = lower_bound_u64(B, s, v);
                    const int ub = upper_bound_u64(B, s, v);
                    paired = (i - fa) < (ub - lb);
                }
            }
            const unsigned bal = __ballot_sync(0xffffffffu, paired);
            if (i < s) P[i] = run + __popc(bal & ((1u << lane) - 1u));
            run += __popc(bal);
        }
        if (lane == 0) P[s] = run;
        __syncwarp();
        // pass 2: shared steps among the first s
        int32_t shared = 0;
        for (int i = lane; i < s; i += 32) {
            const uint64_t v = A[i];
            if (v == MAXV) continue;
            const int fa = lower_bound_u64(A, s, v);
            const int lb = lower_bound_u64(B, s, v);
            const int ub = upper_bound_u64(B, s, v);
            if ((i - fa) < (ub - lb)) {
                const int step = i + lb - P[fa];
                shared += step < s;
            }
        }
        for (int o = 16; o; o >>= 1) shared += __shfl_xor_sync(0xffffffffu, shared, o);
        if (lane == 0) {
            const int nA = lower_bound_u64(A, s, MAXV);
            const int nB = lower_bound_u64(B, s, MAXV);
            const int T = nA + nB - P[s];
            const int steps = T < s ? T : s;
            const float j = steps == 0 ? 0.0f : __fdiv_rn((float)shared, (float)steps);
            sims[p] = j;
            if (mask) mask[p] = j >= floor;
        }
        __syncwarp();
    }
}

int32_t jaccard_launch(const int32_t *pairs, int64_t M, const uint64_t *sk, int64_t N, int32_t s,
                       float floor, float *sims, uint8_t *mask, int32_t *d_err, cudaStream_t st) {
    if (s < 1 || s > 4096) {
        set_error(CK_ERR_UNSUPPORTED, "jaccard: need 1 <= s <= 4096");
        return CK_ERR_UNSUPPORTED;
    }
    if (M == 0) return CK_OK;
    const size_t per_warp = ((size_t)2 * s + s / 2 + 2) * sizeof(uint64_t);
    int wpb = (int)((48 * 1024) / per_warp);
    if (wpb > 8) wpb = 8;
    if (wpb < 1) {
        wpb = 1;
        CK_CUDA(cudaFuncSetAttribute(jaccard_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)per_warp));
    }
    int64_t want = (M + wpb - 1) / wpb;
    int64_t cap = (int64_t)sm_count() * 32;
    const int blocks = (int)(want < cap ? want : cap);
    jaccard_kernel<<<blocks, wpb * 32, per_warp * wpb, st>>>(pairs, M, sk, N, s, floor, sims, mask, d_err);
    CK_CUDA(cudaGetLastError());
    return CK_OK;
}

}  // namespace ck
