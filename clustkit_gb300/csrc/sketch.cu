// sketch.cu -- bottom-s MinHash sketches (clustkit/sketch.py:17-183).
//
// Output for a sequence of length L: s zeros if L < k; otherwise the sorted
// multiset of the s smallest values fmix64(v_i ^ seed) over the L-k+1 k-mers,
// where v_i = sum_m code[i+m] * alphabet^(k-1-m) in wrapping uint64 (the
// value clustkit's rolling update produces), padded with UINT64_MAX.
//
// One warp per sequence.  Lanes hash 32 consecutive k-mers at a time; a
// k-mer is kept only while fewer than s values are held or when it is below
// the current s-th smallest value, and kept values are appended to a
// pending area in shared memory.  When the pending area fills, the warp
// bitonic-sorts best+pending (2*BUF entries, BUF = pow2 >= s) and keeps the
// smallest s.  Strict '<' against the s-th smallest keeps the multiset
// semantics of clustkit's replace-the-maximum loop (a value equal to the
// current maximum never enters).
#include "ck_common.cuh"

namespace ck {

__device__ __forceinline__ uint64_t fmix64(uint64_t key, uint64_t seed) {
    uint64_t h = key ^ seed;
    h ^= h >> 33;
    h *= 0xFF51AFD7ED558CCDULL;
    h ^= h >> 33;
    h *= 0xC4CEB9FE1A85EC53ULL;
    h ^= h >> 33;
    return h;
}

__device__ __forceinline__ void warp_bitonic_sort(uint64_t *buf, int cap, int lane) {
    for (int k = 2; k <= cap; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int t = lane; t < (cap >> 1); t += 32) {
                const int i = 2 * j * (t / j) + (t % j);
                const int ixj = i + j;
                const bool up = (i & k) == 0;
                const uint64_t a = buf[i], b = buf[ixj];
                if ((a > b) == up) { buf[i] = b; buf[ixj] = a; }
            }
            __syncwarp();
        }
    }
}

__global__ void sketch_kernel(const uint8_t *__restrict__ flat, int64_t flat_len,
                              const int64_t *__restrict__ offsets, const int32_t *__restrict__ lengths,
                              int64_t N, int32_t k, int32_t s, int32_t BUF, uint64_t alphabet,
                              uint64_t seed, uint64_t *__restrict__ out, int32_t *err) {
    extern __shared__ uint64_t s_buf[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int cap = 2 * BUF;
    uint64_t *buf = s_buf + (size_t)wib * cap;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t MAXV = ~0ULL;

    for (int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < N; q += warps) {
        uint64_t *o = out + q * (int64_t)s;
        const int32_t L = lengths[q];
        const int64_t off = offsets[q];
        if (L < 0 || off < 0 || off + L > flat_len) {
            if (lane == 0) atomicOr(err, ERRBIT_SEQ_EXTENT);
            for (int t = lane; t < s; t += 32) o[t] = 0ULL;
            continue;
        }
        if (L < k) {
            for (int t = lane; t < s; t += 32) o[t] = 0ULL;
            continue;
        }
        const uint8_t *seq = flat + off;
        const int32_t nk = L - k + 1;
        for (int t = lane; t < cap; t += 32) buf[t] = MAXV;
        __syncwarp();
        int32_t cnt = 0, npend = 0;
        uint64_t tau = MAXV;
        for (int32_t base = 0; base < nk; base += 32) {
            const int32_t i = base + lane;
            bool take = false;
            uint64_t hv = 0;
            if (i < nk) {
                uint64_t v = 0;
                for (int32_t m = 0; m < k; ++m) v = v * alphabet + (uint64_t)seq[i + m];
                hv = fmix64(v, seed);
                take = (cnt < s) || (hv < tau);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, take);
            if (take) buf[BUF + npend + __popc(bal & ((1u << lane) - 1u))] = hv;
            npend += __popc(bal);
            const bool last = base + 32 >= nk;
            if (npend > 0 && (npend + 32 > BUF || last)) {
                __syncwarp();
                warp_bitonic_sort(buf, cap, lane);
                const int32_t total = cnt + npend;
                cnt = total < s ? total : s;
                for (int t = s + lane; t < cap; t += 32) buf[t] = MAXV;
                __syncwarp();
                tau = (cnt == s) ? buf[s - 1] : MAXV;
                npend = 0;
            }
        }
        __syncwarp();
        for (int t = lane; t < s; t += 32) o[t] = t < cnt ? buf[t] : MAXV;
        __syncwarp();
    }
}

int32_t sketch_launch(const uint8_t *flat, int64_t flat_len, const int64_t *offsets,
                      const int32_t *lengths, int64_t N, int32_t k, int32_t s, int32_t alphabet,
                      uint64_t seed, uint64_t *out, int32_t *d_err, cudaStream_t st) {
    if (k < 1 || k > 32 || s < 1 || s > 4096 || alphabet < 1 || N < 0) {
        set_error(CK_ERR_UNSUPPORTED, "sketch: need 1 <= k <= 32, 1 <= s <= 4096, alphabet >= 1");
        return CK_ERR_UNSUPPORTED;
    }
    if (N == 0) return CK_OK;
    int32_t BUF = 32;
    while (BUF < s) BUF <<= 1;
    const size_t per_warp = (size_t)2 * BUF * sizeof(uint64_t);
    int warps_per_block = (int)((48 * 1024) / per_warp);
    if (warps_per_block > 8) warps_per_block = 8;
    size_t smem = per_warp * (warps_per_block > 0 ? warps_per_block : 1);
    if (warps_per_block < 1) {
        warps_per_block = 1;
        CK_CUDA(cudaFuncSetAttribute(sketch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    }
    int64_t want = (N + warps_per_block - 1) / warps_per_block;
    int64_t cap = (int64_t)sm_count() * 16;
    const int blocks = (int)(want < cap ? want : cap);
    sketch_kernel<<<blocks, warps_per_block * 32, smem, st>>>(flat, flat_len, offsets, lengths, N, k, s,
                                                              BUF, (uint64_t)alphabet, seed, out, d_err);
    CK_CUDA(cudaGetLastError());
    return CK_OK;
}

}  // namespace ck
