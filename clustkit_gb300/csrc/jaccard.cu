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

// The same closed form with each lane owning E = s / 32 consecutive elements
// of A (s a multiple of 32, at most 256): one binary search gives the lower
// bound in B of the lane's first element, later ones advance it (A is
// sorted, so lower bounds only grow); the count of equal B elements and the
// first index of a value in A come from short scans (sketch values rarely
// repeat); per-element results stay in registers for the second pass.
template <int E>
__global__ void jaccard_kernel_chunked(const int32_t *__restrict__ pairs, int64_t M,
                                       const uint64_t *__restrict__ sk, int64_t N, float floor,
                                       float *__restrict__ sims, uint8_t *__restrict__ mask, int32_t *err) {
    constexpr int S = 32 * E;
    extern __shared__ uint64_t s_mem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    uint64_t *A = s_mem + (size_t)wib * (2 * S + S / 2 + 2);
    uint64_t *B = A + S;
    int32_t *P = (int32_t *)(B + S);  // S + 1 prefix counts of paired A elements
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t MAXV = ~0ULL;
    const int e0 = lane * E;

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
        const uint64_t *ga = sk + (int64_t)ia * S, *gb = sk + (int64_t)ib * S;
#pragma unroll
        for (int k = 0; k < E; ++k) { A[k * 32 + lane] = ga[k * 32 + lane]; B[k * 32 + lane] = gb[k * 32 + lane]; }
        __syncwarp();
        int lbv[E], fav[E];
        uint32_t pbits = 0;
        int n_a = 0, n_b = 0;
        {
            int lb = lower_bound_u64(B, S, A[e0]);
            int fa = e0;  // a run of equal values may start in an earlier lane's chunk
            if (e0 > 0 && A[e0] != MAXV && A[e0 - 1] == A[e0]) fa = lower_bound_u64(A, S, A[e0]);
#pragma unroll
            for (int k = 0; k < E; ++k) {
                const int i = e0 + k;
                const uint64_t v = A[i];
                lbv[k] = 0;
                fav[k] = i;
                if (v == MAXV) continue;
                ++n_a;
                while (lb < S && B[lb] < v) ++lb;
                int c = 0;
                while (lb + c < S && B[lb + c] == v) ++c;
                if (k > 0 && A[i - 1] == v) fav[k] = fa; else if (k > 0) fa = i;
                if (k == 0) fav[k] = fa;
                lbv[k] = lb;
                if (i - fav[k] < c) pbits |= 1u << k;
            }
#pragma unroll
            for (int k = 0; k < E; ++k) n_b += B[e0 + k] != MAXV;
        }
        // exclusive prefix of paired elements: lanes (warp scan), then within the lane
        const int cnt = __popc(pbits);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        {
            int run = incl - cnt;
#pragma unroll
            for (int k = 0; k < E; ++k) { P[e0 + k] = run; run += (pbits >> k) & 1u; }
        }
        if (lane == 31) P[S] = total;
        __syncwarp();
        int shared = 0;
#pragma unroll
        for (int k = 0; k < E; ++k)
            if ((pbits >> k) & 1u) shared += (e0 + k + lbv[k] - P[fav[k]]) < S;
        for (int o = 16; o; o >>= 1) {
            shared += __shfl_xor_sync(0xffffffffu, shared, o);
            n_a += __shfl_xor_sync(0xffffffffu, n_a, o);
            n_b += __shfl_xor_sync(0xffffffffu, n_b, o);
        }
        if (lane == 0) {
            const int T = n_a + n_b - total;
            const int steps = T < S ? T : S;
            const float j = steps == 0 ? 0.0f : __fdiv_rn((float)shared, (float)steps);
            sims[p] = j;
            if (mask) mask[p] = j >= floor;
        }
        __syncwarp();
    }
}

template <int E>
static int32_t launch_chunked(const int32_t *pairs, int64_t M, const uint64_t *sk, int64_t N, float floor,
                              float *sims, uint8_t *mask, int32_t *d_err, cudaStream_t st) {
    constexpr int S = 32 * E;
    const size_t per_warp = ((size_t)2 * S + S / 2 + 2) * sizeof(uint64_t);
    const int wpb = 8;
    int64_t want = (M + wpb - 1) / wpb;
    int64_t cap = (int64_t)sm_count() * 32;
    const int blocks = (int)(want < cap ? want : cap);
    jaccard_kernel_chunked<E><<<blocks, wpb * 32, per_warp * wpb, st>>>(pairs, M, sk, N, floor, sims, mask, d_err);
    CK_CUDA(cudaGetLastError());
    return CK_OK;
}

int32_t jaccard_launch(const int32_t *pairs, int64_t M, const uint64_t *sk, int64_t N, int32_t s,
                       float floor, float *sims, uint8_t *mask, int32_t *d_err, cudaStream_t st) {
    if (s < 1 || s > 4096) {
        set_error(CK_ERR_UNSUPPORTED, "jaccard: need 1 <= s <= 4096");
        return CK_ERR_UNSUPPORTED;
    }
    if (M == 0) return CK_OK;
    switch (s) {
        case 32: return launch_chunked<1>(pairs, M, sk, N, floor, sims, mask, d_err, st);
        case 64: return launch_chunked<2>(pairs, M, sk, N, floor, sims, mask, d_err, st);
        case 128: return launch_chunked<4>(pairs, M, sk, N, floor, sims, mask, d_err, st);
        case 256: return launch_chunked<8>(pairs, M, sk, N, floor, sims, mask, d_err, st);
        default: break;
    }
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
