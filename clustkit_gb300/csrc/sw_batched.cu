// sw_batched.cu -- length-binned, persistent, register-strip Smith-Waterman.
//
// Same results as clustkit/csrc/sw_align.c:25-266, organised for the GPU:
//
//  1. prep: per pair, the geometry (shorter side = rows), the band cell count
//     and a sort key (rows, columns); pairs the packed lanes cannot hold
//     (rows > 8191, residue codes > 20) go to a fallback list.
//  2. sort: pairs are ordered by descending (rows, columns), so a warp's 32
//     pairs have near-identical shapes and the longest work is issued first.
//  3. strip kernel: one persistent CTA per SM (512 threads for 16-row strips,
//     640 for 8-row ones); each warp takes the next 32 sorted pairs from a
//     global ticket counter and every lane aligns one pair.  A lane sweeps
//     its pair in strips of R rows: the strip's R rows live in registers and
//     advance one column at a time, so per column only the row above the
//     strip is read from (and the strip's last row written to) a per-lane
//     circular window in global scratch.
//  4. the plain kernel runs the fallback list, plus any pair whose score
//     reached the packed lane's limit (re-run exactly in plain int32).
//
// Packed key.  Each DP value is one int32
//     key = score * 2^16 + prio * 2^14 + tie * 2^13 + matches
// with matches in 13 bits (<= 8191 rows), a 2-bit priority (zero 3, diag 2,
// E 1, F 0) and a tie bit (gap extension 1, gap opening 0).  Signed integer
// max over keys then orders candidates exactly as clustkit's comparisons do
// (score first, then H's 0 > diag > E > F priority, then E/F's preference for
// extension on ties) and carries the match count of the winner for free.
// Pairs of at most 2047 rows use a compact form of the key (KeyCompact below:
// an 11-bit match count and a gap-extension counter in place of the tie bit),
// which needs fewer logic ops a cell.  The BLOSUM62 increment of a cell is a
// table of keys: s(a,b) * 2^16 + 2 * 2^14 + (a == b), looked up in shared
// memory, replicated per lane so that the 32 lanes of a warp always hit 32
// different banks.  Per cell:
//     diag = max(Hdiag + inc, ZERO)          (__viaddmax_s32)
//     E    = max(E_up - 2^16, H_up + OPEN_E) (__viaddmax_s32)
//     F    = max(F_left - 2^16, H_left + OPEN_F)
//     H    = max(diag, E, F)                 (__vimax3_s32)
// and H's priority/tie bits (or counter) are cleared before it feeds other
// cells.
// The first row-major cell holding the best score is tracked per row (strict
// '>' along the row) and the rows are merged in row order after each strip;
// a warp vote once per group of interior columns decides whether any lane's
// cells reached its threshold, so most columns never touch the trackers.
// Rows of a pair's last strip below its last row read a pad code (their
// diagonal always loses to zero), so every strip runs the same column code.
// Scores use the key's top 16 bits; a pair whose best score comes within 24
// of 32767 is re-run on the plain kernel, so no overflow reaches the output.
#include <cub/device/device_radix_sort.cuh>

#include <cstring>

#include "ck_common.cuh"

namespace ck {

namespace key {
constexpr int32_t TBIT = 1 << 13;
constexpr int32_t PU = 1 << 14;
constexpr int32_t KU = 1 << 16;
constexpr int32_t CLEAN = ~(TBIT | 3 * PU);
constexpr int32_t ZKEY = 3 * PU;
constexpr int32_t OPEN_E = GAP_OPEN * KU + 1 * PU;
constexpr int32_t OPEN_F = GAP_OPEN * KU;
constexpr int32_t EXT = GAP_EXTEND * KU;
constexpr int32_t NEG_E = -16 * KU + 1 * PU + TBIT;
constexpr int32_t NEG_F = -16 * KU + TBIT;
constexpr int32_t ROWS_MAX = (1 << 13) - 1;
constexpr int32_t SCORE_LIMIT = 32767 - 24;
constexpr int32_t MATCH_MASK = (1 << 13) - 1;
}  // namespace key

// The two key forms of the strip kernel.  Wide (above): 13 bits of match
// count, and a tie bit set on every stored E and F so that a gap extension
// beats a gap opening of the same score.  Compact, for pairs of at most 2047
// rows: 11 bits of match count and, in bits 11..13, a counter that every gap
// extension increments.  An opening starts from a clean H (counter 0) and an
// extension from E or F plus one (counter >= 1), so extension still wins
// every tie.  E's counter is cleared at strip rows 5, 11, 17, ... and the
// strip's last row (at most 6 extensions between clears, the window carrying
// the count from one strip's last row into the next strip's first), F's after
// every group of at most 4 columns, before either could carry into the
// priority bits: a few logic ops per group instead of two per cell.
struct KeyWide {
    static constexpr bool COMPACT = false;
    static constexpr int32_t CTR = 0;
    static constexpr int32_t CLEAN = key::CLEAN;
    static constexpr int32_t EXT = key::EXT;
    static constexpr int32_t NEG_E = key::NEG_E;
    static constexpr int32_t NEG_F = key::NEG_F;
    static constexpr int32_t MATCH_MASK = key::MATCH_MASK;
};
struct KeyCompact {
    static constexpr bool COMPACT = true;
    static constexpr int32_t CTR = 7 << 11;
    static constexpr int32_t CLEAN = ~(CTR | 3 * key::PU);
    static constexpr int32_t EXT = key::EXT + (1 << 11);
    static constexpr int32_t NEG_E = -16 * key::KU + 1 * key::PU;
    static constexpr int32_t NEG_F = -16 * key::KU;
    static constexpr int32_t MATCH_MASK = (1 << 11) - 1;
    static constexpr int32_t ROWS_MAX = (1 << 11) - 1;
};

// Threads of the strip kernel's one persistent CTA per SM: 512 (16 warps at
// up to 128 registers) for strips of 8 or 16 rows, 640 or 768 (20 or 24
// warps at 96 or 80 registers) for 8-row strips, 256 (8 warps, up to 255
// registers) for 24 or 32 rows.  One CTA per SM holds one increment table,
// so the warps a CTA adds cost no table copy.  Each warp keeps its strip
// rows' first-maximum trackers in a block of its own (row r of lane l at
// r * 32 + l), so the layout does not depend on the CTA's size.
// per warp, the streamed warp-per-pair phase's pair slots in shared memory
constexpr size_t WAVE_SLOT_BYTES = 72;  // sizeof(WaveSlot), checked where it is defined
constexpr int WAVE_SLOTS_PER_WARP = 16;

// a * one + b with `one` a runtime 1: issued as an integer multiply-add on
// the FMA pipe, which the recurrence leaves mostly idle, instead of an add on
// the ALU pipe, which the DPX max operations and logic ops already saturate.
__device__ __forceinline__ int32_t fadd(int32_t a, int32_t b, int32_t one) {
    int32_t d;
    asm("mad.lo.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(one), "r"(b));
    return d;
}
// Row code of the rows of a pair's last strip below its last row.  Their
// increments are so negative that the diagonal candidate always loses to
// zero, so such a row only carries gap values down and along from the real
// rows (each strictly below the score it came from): it can never hold the
// pair's first maximum, and the last strip runs the unmasked column code.
constexpr uint32_t PAD_CODE = N_CODES;
constexpr int32_t PAD_INC = INT32_MIN + 1;  // H keys are >= 0, so H + PAD_INC never wraps
constexpr int INC_ENTRIES = (N_CODES + 1) * N_CODES;     // 462: row code (0..21) x column code (0..20)
constexpr size_t INC_SMEM = (size_t)INC_ENTRIES * 32 * 4;  // replicated per lane

// ----------------------------------------------------------------- tables
__global__ void build_inc_kernel(const int8_t *sub, int32_t *inc) {
    int t = threadIdx.x + blockIdx.x * blockDim.x;
    if (t >= INC_ENTRIES) return;
    int a = t / N_CODES, b = t % N_CODES;
    int s = (a < 20 && b < 20) ? (int)sub[a * 20 + b] : -4;
    inc[t] = a == (int)PAD_CODE ? PAD_INC : s * key::KU + 2 * key::PU + (a == b ? 1 : 0);
}

// Whether every residue code of sequence i is <= 20, memoised per call in
// ok[i] (0 unknown, 1 yes, 2 no): only sequences that some pair references
// are read, once or a few times (concurrent first readers agree).
__device__ __forceinline__ bool seq_codes_ok(const SwIn &in, int32_t i, uint8_t *ok) {
    const uint8_t m = ok[i];
    if (m) return m == 1;
    const uint8_t *s = in.flat + in.offsets[i];
    const int32_t L = in.lengths[i];
    // bytes up to a 16-byte boundary, then 16 per load (four compared per
    // instruction), then the tail
    int32_t head = (int32_t)((16u - ((uint32_t)(uintptr_t)s & 15u)) & 15u);
    if (head > L) head = L;
    uint32_t bad = 0;
    for (int32_t t = 0; t < head; ++t) bad |= __ldg(s + t) > 20 ? 1u : 0u;
    const uint4 *v = (const uint4 *)(s + head);
    const int32_t nv = (L - head) >> 4;
#pragma unroll 4
    for (int32_t k = 0; k < nv; ++k) {
        const uint4 x = __ldg(v + k);
        bad |= __vcmpgtu4(x.x, 0x14141414u) | __vcmpgtu4(x.y, 0x14141414u) |
               __vcmpgtu4(x.z, 0x14141414u) | __vcmpgtu4(x.w, 0x14141414u);
    }
    for (int32_t t = head + nv * 16; t < L; ++t) bad |= __ldg(s + t) > 20 ? 1u : 0u;
    const bool good = bad == 0;
    ok[i] = good ? 1 : 2;
    return good;
}

// Closed-form count of the band cells of a pair (the cells clustkit's loop
// visits): rows i in [1, la] with columns max(1, i+h-w) .. min(lb, i+h+w).
__host__ __device__ inline int64_t sum_min(int64_t a, int64_t b, int64_t c, int64_t L) {
    // sum_{i=a}^{b} min(L, i + c)
    if (b < a) return 0;
    int64_t t = L - c;  // i <= t  <=>  i + c <= L
    int64_t s = 0;
    int64_t e1 = b < t ? b : t;
    if (e1 >= a) s += (e1 - a + 1) * (a + e1) / 2 + (e1 - a + 1) * c;
    int64_t s2 = a > t + 1 ? a : t + 1;
    if (b >= s2) s += (b - s2 + 1) * L;
    return s;
}
__host__ __device__ inline int64_t sum_max(int64_t a, int64_t b, int64_t c, int64_t L) {
    // sum_{i=a}^{b} max(L, i + c)
    if (b < a) return 0;
    int64_t t = L - c;  // i <= t  <=>  i + c <= L  -> value L
    int64_t s = 0;
    int64_t e1 = b < t ? b : t;
    if (e1 >= a) s += (e1 - a + 1) * L;
    int64_t s2 = a > t + 1 ? a : t + 1;
    if (b >= s2) s += (b - s2 + 1) * (s2 + b) / 2 + (b - s2 + 1) * c;
    return s;
}
__host__ __device__ inline int64_t band_cells_closed(int32_t la, int32_t lb, int32_t w, int32_t h) {
    if (la <= 0 || lb <= 0) return 0;
    int64_t c1 = (int64_t)h - w, c2 = (int64_t)h + w;
    int64_t ilo = 1 - c2 > 1 ? 1 - c2 : 1;           // i + c2 >= 1
    int64_t ihi = (int64_t)lb - c1 < la ? (int64_t)lb - c1 : la;  // i + c1 <= lb
    if (ihi < ilo) return 0;
    return sum_min(ilo, ihi, c2, lb) - sum_max(ilo, ihi, c1, 1) + (ihi - ilo + 1);
}

// Rows per lane strip for the warp-per-pair kernel, 0 when it cannot take
// the pair.  Lane l runs strips l, l + 32, ... one column behind lane l - 1;
// a lane may only start its next strip once its previous one (R + 2w - 1
// steps) is done and its upstream lane has moved past the band, which holds
// when 2w < 31 R + 32, or trivially when the pair has at most 32 strips.
// The smallest such R keeps the most lanes busy.
__host__ __device__ inline int32_t wave_rows_per_strip(int32_t la, int32_t w) {
    if (la <= 128 || 2 * w < 31 * 4 + 32) return 4;
    if (la <= 256 || 2 * w < 31 * 8 + 32) return 8;
    if (la <= 512 || 2 * w < 31 * 16 + 32) return 16;
    return 0;
}

// ----------------------------------------------------------------- prep
__global__ void sw_prep_kernel(SwIn in, SwOut out, int64_t M, uint8_t *__restrict__ seq_ok,
                               uint32_t *__restrict__ keys, uint32_t *__restrict__ vals,
                               int32_t *__restrict__ fallback, int32_t *__restrict__ counters,
                               unsigned long long *__restrict__ cells, int32_t *err) {
    // counters[0] = eligible, counters[1] = fallback count
    int64_t local_cells = 0;
    int32_t elig = 0;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < M;
         p += (int64_t)gridDim.x * blockDim.x) {
        PairGeom g = pair_geometry(in, p, err);
        uint32_t k = 0;
        if (!g.valid) {
            write_result(out, in, p, 0, 0, 0, 0, 0);
        } else if (g.la == 0 || cupy_ratio_skip(in, g.la, g.lb)) {
            write_result(out, in, p, 0, 0, g.la, g.la, g.lb);
        } else {
            local_cells += band_cells_closed(g.la, g.lb, g.w, g.h);
            if (g.la <= key::ROWS_MAX && seq_codes_ok(in, g.a_idx, seq_ok) &&
                seq_codes_ok(in, g.b_idx, seq_ok)) {
                int32_t cb = g.lb < key::ROWS_MAX ? g.lb : key::ROWS_MAX;
                k = ((uint32_t)g.la << 13) | (uint32_t)cb;
                elig++;
            } else {
                int32_t pos = atomicAdd(&counters[1], 1);
                fallback[pos] = (int32_t)p;
            }
        }
        keys[p] = k;
        vals[p] = (uint32_t)p;
    }
    for (int o = 16; o; o >>= 1) {
        local_cells += __shfl_xor_sync(0xffffffffu, local_cells, o);
        elig += __shfl_xor_sync(0xffffffffu, elig, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (local_cells) atomicAdd(cells, (unsigned long long)local_cells);
        if (elig) atomicAdd(&counters[0], elig);
    }
}

// Which sorted pairs (a prefix: rows descending) run one warp per pair,
// decided on the device from the call's own counts.  Only when every
// eligible pair can (wave_rows_per_strip > 0: band half-width <= 263, or at
// most 512 rows).  A call with at most `all_below` eligible pairs: all of
// them (too few to fill the GPU one per lane).  Otherwise, with a band width
// > 0, the long pairs whose one-lane time would exceed the call's expected
// run time: a pair of `rows` rows costs one lane about rows * (2w + 1) cell
// steps, the whole call about cells / lanes steps per lane (the longest
// pairs start first, so a pair below that bound does not set the tail).
// Pairs at or above max(min_rows, that bound) are counted by a binary search
// over the sorted keys.
__global__ void wave_split_kernel(const uint32_t *__restrict__ sorted_keys, int32_t *counters,
                                  int32_t band_width, int32_t all_below, int32_t min_rows,
                                  int32_t adaptive, int64_t lanes) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int32_t n_elig = counters[0];
    counters[6] = 0;
    if (n_elig <= 0) return;
    const int32_t max_rows = (int32_t)(sorted_keys[0] >> 13);
    counters[8] = max_rows;  // the warp-per-pair phase's key form depends on it
    const bool all_capable = (band_width >= 1 && 2 * band_width < 31 * 16 + 32) || max_rows <= 512;
    if (!all_capable) return;
    if (n_elig <= all_below) { counters[6] = n_elig; return; }
    if (band_width <= 0 || min_rows >= (1 << 13)) return;
    unsigned long long cells = 0;
    memcpy(&cells, counters + 4, sizeof(cells));
    int64_t rows_thr = min_rows;
    if (adaptive) {
        const int64_t per_lane = (int64_t)(cells / (unsigned long long)(lanes > 0 ? lanes : 1));
        const int64_t r = per_lane / (2 * (int64_t)band_width + 1) + 1;
        if (r > rows_thr) rows_thr = r;
    }
    // keys are (rows << 13 | cols), descending: count the prefix with rows >= rows_thr
    int32_t lo = 0, hi = n_elig;
    while (lo < hi) {
        const int32_t mid = (lo + hi) >> 1;
        if ((int64_t)(sorted_keys[mid] >> 13) >= rows_thr) lo = mid + 1; else hi = mid;
    }
    counters[6] = lo;
}

// ----------------------------------------------------------------- strip kernel
// Registers of one lane for the strip in flight.
template <int R>
struct StripRegs {
    int32_t hc[R];     // H (clean key) of row r at the last column done
    int32_t fT[R];     // F key (tie bit set) of row r at the last column done
    uint32_t arow[R];  // byte offset of row r's residue block in the increment table
    int32_t hd0;       // H(i0 - 1, j - 1): diagonal input of the strip's first row
    int2 bq[4];        // window entries (row i0 - 1) of the next P columns, prefetched
    uint32_t cq[4];    // residue offsets of the same columns' b
};

// Structural variants of the strip kernel (picked by the autotuner): bit 1
// runs interior columns in groups of 4 instead of 2 (one first-max vote per
// group); bit 0 starts the groups at columns aligned to their size,
// addresses each run of a group's window slots from one base pointer and
// prefetches window entries and residues four columns ahead, instead of
// computing each column's addresses on its own and prefetching two ahead.
template <int V> struct StripVariant {
    static constexpr int UNROLL = (V & 2) ? 4 : 2;
    static constexpr bool ALIGNED = (V & 1) != 0;
    static constexpr int PREFETCH = ALIGNED ? 4 : 2;  // columns ahead
};

// Rows of a strip inside their band at a column, as a bit mask: row r
// (0 <= r < alive) of the strip whose first row's band starts at column lo0
// covers column j when 0 <= j - r - lo0 <= w2, i.e. r in
// [d - w2, d] with d = j - lo0.
__device__ __forceinline__ uint32_t band_rows(int32_t d, uint32_t w2, int32_t alive) {
    const int32_t lo = d - (int32_t)w2 > 0 ? d - (int32_t)w2 : 0;
    const int32_t hi = d < alive - 1 ? d : alive - 1;
    return hi < lo ? 0u : (2u << hi) - (1u << lo);  // 0 <= lo <= hi < alive <= 16 (wave kernel)
}

// Cells of rows [RB, RE) at one column, top to bottom.  (hu, eu) enter as
// H and E of row RB - 1 at column j, hdiag as H of row RB - 1 at column
// j - 1; they leave as the values of row RE - 1.  Stored keys: H clean
// (score * 2^16 + matches), E and F with the tie bit set (wide key) or their
// extension counters (compact key: E's cleared here at the strip rows the
// lane-per-pair kernel clears them, F's by the caller every 4 columns).
//     diag = max(Hdiag + inc, ZERO)
//     E    = max(E_up - 2^16, H_up + OPEN_E) | tie
//     F    = max(F_left - 2^16, H_left + OPEN_F) | tie
//     H    = max(diag, E, F) & CLEAN
template <int R, int RB, int RE, bool MASKED, class K>
__device__ __forceinline__ void strip_cells(uint32_t bcol, int32_t &hu, int32_t &eu, int32_t hdiag,
                                            StripRegs<R> &S, const char *s_inc, uint32_t rmask, int32_t one) {
    using namespace key;
#pragma unroll
    for (int r = RB; r < RE; ++r) {
        const int32_t inc = *(const int32_t *)(s_inc + fadd((int32_t)S.arow[r], (int32_t)bcol, one));
        const int32_t diagc = __viaddmax_s32(hdiag, inc, ZKEY);
        // E's extension term comes from E of the row above, known before that
        // row's H: only H_up + OPEN_E and the max-of-three sit on the
        // row-to-row dependency chain.  E's tie mark plays no part in H (E, F,
        // diag and zero differ in priority), so it is set off the chain.
        const int32_t eR = __viaddmax_s32(hu, OPEN_E, fadd(eu, K::EXT, one));
        int32_t fTn = __viaddmax_s32(S.fT[r], K::EXT, fadd(S.hc[r], OPEN_F, one));
        if constexpr (!K::COMPACT) fTn |= TBIT;
        const int32_t hn = __vimax3_s32(diagc, eR, fTn) & K::CLEAN;
        int32_t en;
        if constexpr (K::COMPACT) en = (r % 6 == 5 || r == R - 1) ? (eR & ~K::CTR) : eR;
        else en = eR | TBIT;
        hdiag = S.hc[r];
        if constexpr (MASKED) {
            // A row outside its band at this column (bit r of rmask clear) is
            // computed like the others and its results dropped by selects (no
            // branch: the lanes of a warp are at different columns of their
            // strips): a row that has not reached its band keeps H = 0 and its
            // F; a row that has left it hands the out-of-band boundary (H = 0,
            // E = -inf) to the row below and its last H as that row's diagonal
            // input (hdiag above, as for a row inside its band).
            const bool inb = (rmask >> r) & 1u;
            const int32_t hs = inb ? hn : 0;
            S.hc[r] = hs;
            S.fT[r] = inb ? fTn : S.fT[r];
            hu = hs;
            eu = inb ? en : K::NEG_E;
        } else {
            S.hc[r] = hn;
            S.fT[r] = fTn;
            hu = hn;
            eu = en;
        }
    }
}

// One DP cell of strip row r (all inputs inside the band).  (hu, eu) enter as
// H and E of the row above at this column and leave as this row's; hdiag
// enters as H of the row above at the previous column and leaves as this
// row's H at the previous column (the next row's diagonal input).
template <int R, int r, class K>
__device__ __forceinline__ void strip_cell(uint32_t bcol, int32_t &hu, int32_t &eu, int32_t &hdiag,
                                           StripRegs<R> &S, const char *s_inc, int32_t one) {
    using namespace key;
    const int32_t inc = *(const int32_t *)(s_inc + fadd((int32_t)S.arow[r], (int32_t)bcol, one));
    const int32_t diagc = __viaddmax_s32(hdiag, inc, ZKEY);
    // E's extension term comes from E of the row above, known before that
    // row's H: only H_up + OPEN_E and the max-of-three sit on the row-to-row
    // dependency chain.  E's tie mark plays no part in H (E, F, diag and zero
    // differ in priority), so it is set off the chain.
    const int32_t eR = __viaddmax_s32(hu, OPEN_E, fadd(eu, K::EXT, one));
    int32_t fTn = __viaddmax_s32(S.fT[r], K::EXT, fadd(S.hc[r], OPEN_F, one));
    if constexpr (!K::COMPACT) fTn |= TBIT;
    const int32_t hn = __vimax3_s32(diagc, eR, fTn) & K::CLEAN;
    hdiag = S.hc[r];
    S.hc[r] = hn;
    S.fT[r] = fTn;
    hu = hn;
    if constexpr (K::COMPACT) eu = (r % 6 == 5 || r == R - 1) ? (eR & ~K::CTR) : eR;
    else eu = eR | TBIT;
}

// Rows r .. R-1 of a column, all inside their band.
template <int R, class K, int r = 0>
__device__ __forceinline__ void strip_cells_from(uint32_t bcol, int32_t &hu, int32_t &eu, int32_t &hdiag,
                                                 StripRegs<R> &S, const char *s_inc, int32_t one) {
    if constexpr (r < R) {
        strip_cell<R, r, K>(bcol, hu, eu, hdiag, S, s_inc, one);
        strip_cells_from<R, K, r + 1>(bcol, hu, eu, hdiag, S, s_inc, one);
    }
}

// Compact key: clear the F counters of the strip's rows after a group of
// columns (at most 4 extensions since the last clear).
template <int R, class K>
__device__ __forceinline__ void strip_clear_f(StripRegs<R> &S) {
    if constexpr (K::COMPACT) {
#pragma unroll
        for (int r = 0; r < R; ++r) S.fT[r] &= ~K::CTR;
    }
}

// A ramp or clipped column: only rows klo..khi lie inside their band.  A row
// above klo has left it (it hands H = 0, E = -inf down and its last H as the
// next row's diagonal input); a row below khi has not reached it (left
// untouched, and the strip's bottom output is the out-of-band boundary).
// The left ramp (klo = 0) is a prefix of the rows and the right ramp
// (khi = R - 1) a suffix, so each needs one compare a row; a column that is
// both (a band narrower than the strip) takes the two-sided test.  Every
// row's cell appears once in the code.
template <int R, class K, int r = 0>
__device__ __forceinline__ void strip_rows_prefix(uint32_t bcol, int32_t &hu, int32_t &eu, int32_t &hdiag,
                                                  StripRegs<R> &S, const char *s_inc, int32_t khi, int32_t one) {
    if constexpr (r < R) {
        if (r <= khi) strip_cell<R, r, K>(bcol, hu, eu, hdiag, S, s_inc, one);
        strip_rows_prefix<R, K, r + 1>(bcol, hu, eu, hdiag, S, s_inc, khi, one);
    }
}

template <int R, class K, int r = 0>
__device__ __forceinline__ void strip_rows_suffix(uint32_t bcol, int32_t &hu, int32_t &eu, int32_t &hdiag,
                                                  StripRegs<R> &S, const char *s_inc, int32_t klo, int32_t one) {
    if constexpr (r < R) {
        if (r >= klo) strip_cell<R, r, K>(bcol, hu, eu, hdiag, S, s_inc, one);
        else hdiag = S.hc[r];
        strip_rows_suffix<R, K, r + 1>(bcol, hu, eu, hdiag, S, s_inc, klo, one);
    }
}

template <int R, class K, int r = 0>
__device__ __forceinline__ void strip_rows_between(uint32_t bcol, int32_t &hu, int32_t &eu, int32_t &hdiag,
                                                   StripRegs<R> &S, const char *s_inc, int32_t klo, int32_t khi,
                                                   int32_t one) {
    if constexpr (r < R) {
        if (r < klo) hdiag = S.hc[r];
        else if (r <= khi) strip_cell<R, r, K>(bcol, hu, eu, hdiag, S, s_inc, one);
        strip_rows_between<R, K, r + 1>(bcol, hu, eu, hdiag, S, s_inc, klo, khi, one);
    }
}

template <int R, class K>
__device__ __forceinline__ void strip_rows_masked(uint32_t bcol, int32_t &hu, int32_t &eu, int32_t &hdiag,
                                                  StripRegs<R> &S, const char *s_inc, int32_t klo, int32_t khi,
                                                  int32_t one) {
    if (klo == 0) {
        strip_rows_prefix<R, K>(bcol, hu, eu, hdiag, S, s_inc, khi, one);
    } else {
        hu = 0;  // the first row inside the band has the boundary above it
        eu = K::NEG_E;
        if (khi == R - 1) strip_rows_suffix<R, K>(bcol, hu, eu, hdiag, S, s_inc, klo, one);
        else strip_rows_between<R, K>(bcol, hu, eu, hdiag, S, s_inc, klo, khi, one);
    }
    if (khi < R - 1) { hu = 0; eu = K::NEG_E; }  // the bottom row has not started
}

// First-max trackers (one per row, in shared memory) are touched only when
// some lane holds a cell at or above its trigger threshold `tthr`: above the
// pair's best when the strip began, and once this strip has set a best M, at
// least M (an equal score in an earlier row still comes first in row-major
// order; a lower one never can).  Only cells above the threshold read their
// row's tracker; the strict '>' there keeps each row's first column.  The
// check covers the U columns of `hs` (oldest first) at once, so that the
// warp's vote and branch come once per U columns and the columns' row chains
// can overlap in between.
template <int R, int U>
__device__ __forceinline__ void strip_track(const int32_t (&hs)[U][R], int32_t &tthr, int32_t *s_best) {
    using namespace key;
    int32_t cm = hs[0][0];
#pragma unroll
    for (int k = 1; k + 1 < U * R; k += 2) cm = __vimax3_s32(cm, hs[k / R][k % R], hs[(k + 1) / R][(k + 1) % R]);
    if (((U * R) & 1) == 0) cm = max(cm, hs[U - 1][R - 1]);
    if (__any_sync(__activemask(), cm > tthr)) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int32_t v = hs[u][r];
                if (v > tthr) {
                    const int32_t b = s_best[r * 32];
                    if (v > (b | (KU - 1))) s_best[r * 32] = v;
                }
            }
        }
        if (cm > tthr) tthr = (cm & ~(KU - 1)) - 1;
    }
}

// The next column's inputs: the window entry (H, E of the row above the
// strip) and the residue offset of column j, from the P-deep prefetch queue;
// column j + P is loaded behind them (its residue clamped to the sequence).
template <int R, int P>
__device__ __forceinline__ void column_inputs(int32_t j, int32_t lb, StripRegs<R> &S, const int2 *win,
                                              int32_t wmask, const uint8_t *B, int2 &bnd, uint32_t &bcol) {
    bnd = S.bq[0];
    bcol = S.cq[0];
#pragma unroll
    for (int k = 0; k + 1 < P; ++k) {
        S.bq[k] = S.bq[k + 1];
        S.cq[k] = S.cq[k + 1];
    }
    const int32_t jn = j + P < lb ? j + P : lb;  // column whose residue is prefetched
    S.bq[P - 1] = win[(size_t)((j + P) & wmask) * 32];
    S.cq[P - 1] = (uint32_t)__ldg(B + jn - 1) * 128u;
}

// U interior columns j .. j + U - 1 (every row inside its band), each
// addressing its own window slots and residues, then one first-max check
// over all of them.
template <int R, int U, int P, class K>
__device__ __forceinline__ void strip_group_percol(int32_t j, int32_t lb, StripRegs<R> &S, const char *s_inc,
                                                   int2 *win, int32_t wmask, const uint8_t *B, int32_t &tthr,
                                                   int32_t *s_best, int32_t one) {
    int32_t hs[U][R];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        int2 bnd;
        uint32_t bcol;
        column_inputs<R, P>(j + u, lb, S, win, wmask, B, bnd, bcol);
        int32_t hu = bnd.x, eu = bnd.y, hdiag = S.hd0;
        S.hd0 = hu;
        strip_cells_from<R, K>(bcol, hu, eu, hdiag, S, s_inc, one);
        win[(size_t)((j + u) & wmask) * 32] = make_int2(hu, eu);
#pragma unroll
        for (int r = 0; r < R; ++r) hs[u][r] = S.hc[r];
    }
    strip_clear_f<R, K>(S);
    strip_track<R, U>(hs, tthr, s_best);
}

// U interior columns j .. j + U - 1 with j a multiple of U, inputs prefetched
// P columns ahead.  W is a power of two >= 32 and U divides it, so every run
// of U columns that starts at a multiple of U has consecutive slots: one base
// address per run, immediate offsets after it.  The caller runs a group only
// where j + U - 1 + P <= lb, so the prefetched residues lie inside the
// sequence.
template <int R, int U, int P, class K>
__device__ __forceinline__ void strip_group(int32_t j, StripRegs<R> &S, const char *s_inc, int2 *win,
                                            int32_t wmask, const uint8_t *B, int32_t &tthr, int32_t *s_best,
                                            int32_t one) {
    int2 *cur = win + (size_t)(j & wmask) * 32;
    const uint8_t *pb = B + j + P - 1;  // residue of column j + P (columns are 1-based)
    int32_t hs[U][R];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int2 bnd = S.bq[0];
        const uint32_t bcol = S.cq[0];
#pragma unroll
        for (int k = 0; k + 1 < P; ++k) {
            S.bq[k] = S.bq[k + 1];
            S.cq[k] = S.cq[k + 1];
        }
        const int c = u + P;  // column j + c is loaded: run c / U of the group's window, offset c % U
        const int2 *run = win + (size_t)((j + (c / U) * U) & wmask) * 32;
        S.bq[P - 1] = run[(c % U) * 32];
        S.cq[P - 1] = (uint32_t)__ldg(pb + u) * 128u;
        int32_t hu = bnd.x, eu = bnd.y, hdiag = S.hd0;
        S.hd0 = hu;
        strip_cells_from<R, K>(bcol, hu, eu, hdiag, S, s_inc, one);
        cur[u * 32] = make_int2(hu, eu);
#pragma unroll
        for (int r = 0; r < R; ++r) hs[u][r] = S.hc[r];
    }
    strip_clear_f<R, K>(S);
    strip_track<R, U>(hs, tthr, s_best);
}

// One column outside the aligned interior groups: a ramp or clipped column
// (rows klo..khi inside their band) or an interior column at a group's edge.
template <int R, int P, class K>
__device__ __forceinline__ void strip_column(int32_t j, int32_t lb, StripRegs<R> &S, const char *s_inc,
                                             int2 *win, int32_t wmask, const uint8_t *B, int32_t lo0,
                                             int32_t w2, int32_t &tthr, int32_t *s_best, int32_t one) {
    int2 bnd;
    uint32_t bcol;
    column_inputs<R, P>(j, lb, S, win, wmask, B, bnd, bcol);
    int32_t hu = bnd.x, eu = bnd.y, hdiag = S.hd0;
    S.hd0 = hu;
    // rows r with lo0 + r <= j <= lo0 + r + 2w are inside their band
    const int32_t d = j - lo0;
    const int32_t klo = d - w2 > 0 ? d - w2 : 0;
    const int32_t khi = d < R - 1 ? d : R - 1;
    strip_rows_masked<R, K>(bcol, hu, eu, hdiag, S, s_inc, klo, khi, one);
    win[(size_t)(j & wmask) * 32] = make_int2(hu, eu);
    strip_clear_f<R, K>(S);
    int32_t hs[1][R];
#pragma unroll
    for (int r = 0; r < R; ++r) hs[0][r] = S.hc[r];
    strip_track<R, 1>(hs, tthr, s_best);
}

template <int R, int V, class K>
__device__ __forceinline__ void align_pair_strips_k(const SwIn &in, const SwOut &out, int64_t p,
                                                    const PairGeom &g, const char *s_inc, int32_t *s_best,
                                                    int2 *win, int32_t W, int32_t lane, int32_t *fallback,
                                                    int32_t *fallback_count, int32_t one) {
    using namespace key;
    const int32_t la = g.la, lb = g.lb, w = g.w, h = g.h;
    const uint8_t *A = in.flat + in.offsets[g.a_idx];
    const uint8_t *B = in.flat + in.offsets[g.b_idx];
    const int32_t wmask = W - 1;
    const int32_t w2 = 2 * w;

    // every slot reads as the boundary (H = 0, E = -inf) before the first strip;
    // writing the whole window, not only the first strip's columns, measured
    // faster (its lines are then in place for the strips that follow)
    for (int32_t s = 0; s < W; ++s) win[(size_t)s * 32] = make_int2(0, K::NEG_E);

    int32_t gbest = 0;
    StripRegs<R> S;
    for (int32_t i0 = 1; i0 <= la; i0 += R) {
        const int32_t lo0 = i0 + h - w;  // unclipped first column of row i0
        const int32_t J0 = lo0 < 1 ? 1 : lo0;
        const int32_t hi_last = i0 + R - 1 + h + w;
        const int32_t J1 = hi_last < lb ? hi_last : lb;
        if (J0 > lb) break;
        if (J1 < J0) continue;

        int32_t tthr = gbest | (KU - 1);
        const int32_t alive = la - i0 + 1 < R ? la - i0 + 1 : R;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            S.hc[r] = 0;
            S.fT[r] = K::NEG_F;
            s_best[r * 32] = gbest;
            // rows below the pair's last row (last strip only) read the pad code
            const uint32_t code = (r < alive) ? (uint32_t)A[i0 + r - 1] : PAD_CODE;
            S.arow[r] = (code * (uint32_t)N_CODES * 32u + (uint32_t)lane) * 4u;
        }
        S.hd0 = (J0 >= 2) ? win[(size_t)((J0 - 1) & wmask) * 32].x : 0;
        constexpr int P = StripVariant<V>::PREFETCH;
#pragma unroll
        for (int k = 0; k < P; ++k) {
            S.bq[k] = win[(size_t)((J0 + k) & wmask) * 32];
            S.cq[k] = (uint32_t)__ldg(B + (J0 + k < lb ? J0 + k : lb) - 1) * 128u;
        }

        // Interior columns (every row inside its band) run unmasked in aligned
        // groups of U; ramp and clipped columns, and interior columns at a
        // group's edge, run one at a time.  One loop keeps a single copy of
        // each body in the instruction cache.
        int32_t I0 = lo0 + R - 1;
        if (I0 < J0) I0 = J0;
        int32_t I1 = i0 + h + w;
        if (I1 > J1) I1 = J1;
        constexpr int U = StripVariant<V>::UNROLL;
        constexpr bool ALIGNED = StripVariant<V>::ALIGNED;
        for (int32_t j = J0; j <= J1;) {
            if (ALIGNED && j >= I0 && (j & (U - 1)) == 0 && j + U - 1 <= I1 && j + U - 1 + P <= lb) {
                strip_group<R, U, P, K>(j, S, s_inc, win, wmask, B, tthr, s_best, one);
                j += U;
            } else if (!ALIGNED && j >= I0 && j + U - 1 <= I1) {
                strip_group_percol<R, U, P, K>(j, lb, S, s_inc, win, wmask, B, tthr, s_best, one);
                j += U;
            } else {
                strip_column<R, P, K>(j, lb, S, s_inc, win, wmask, B, lo0, w2, tthr, s_best, one);
                j += 1;
            }
        }
        // rows merge in row order: strict '>' keeps the earliest row on ties
        // (pad rows never hold a new best: their values stay below a real cell's)
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int32_t b = s_best[r * 32];
            if (b > (gbest | (KU - 1))) gbest = b;
        }
        // the columns right of this strip's band read as out-of-band for the next strip
        const int32_t fill_end = J1 + R < lb ? J1 + R : lb;
        for (int32_t j = J1 + 1; j <= fill_end; ++j)
            win[(size_t)(j & wmask) * 32] = make_int2(0, K::NEG_E);
    }
    const int32_t score = gbest >> 16;
    if (score >= SCORE_LIMIT) {
        int32_t pos = atomicAdd(fallback_count, 1);
        fallback[pos] = (int32_t)p;
        atomicAdd(fallback_count + 2, 1);  // re-run counter
        return;
    }
    write_result(out, in, p, score, gbest & K::MATCH_MASK, la, la, lb);
}

// One pair, one lane: the compact key when its rows fit (and wide_key is 0),
// else the wide one.  Only a group of 32 sorted pairs that straddles 2047
// rows runs both forms.
template <int R, int V>
__device__ void align_pair_strips(const SwIn &in, const SwOut &out, int64_t p, const char *s_inc,
                                  int32_t *s_best, int2 *win, int32_t W, int32_t lane,
                                  int32_t *fallback, int32_t *fallback_count, int32_t *err,
                                  int32_t one, int32_t wide_key) {
    const PairGeom g = pair_geometry(in, p, err);
    if (!wide_key && g.la <= KeyCompact::ROWS_MAX)
        align_pair_strips_k<R, V, KeyCompact>(in, out, p, g, s_inc, s_best, win, W, lane, fallback,
                                              fallback_count, one);
    else
        align_pair_strips_k<R, V, KeyWide>(in, out, p, g, s_inc, s_best, win, W, lane, fallback,
                                           fallback_count, one);
}

// increment table + per-row first-max trackers (16 rows for the warp-per-pair
// phase) + the warp-per-pair slots, for a CTA of NT threads
template <int R>
constexpr int track_rows() { return R > 16 ? R : 16; }
template <int R, int NT>
__host__ __device__ constexpr size_t strip_smem() {
    return INC_SMEM + (size_t)track_rows<R>() * NT * sizeof(int32_t) +
           (size_t)(NT / 32) * WAVE_SLOTS_PER_WARP * WAVE_SLOT_BYTES;
}

__device__ __noinline__ void align_pair_wave_any(const SwIn &in, const SwOut &out, int64_t p,
                                                 const char *s_inc, int32_t *s_best, int32_t lane,
                                                 int32_t *fallback, int32_t *fallback_count,
                                                 int32_t *err, int32_t one, int32_t wide_key);
struct WaveSlot;
__device__ __noinline__ void wave_stream_any(int32_t rows, const SwIn &in, const SwOut &out, const uint32_t *order,
                                             int32_t n_wave, int32_t *ticket, const char *s_inc, int32_t *s_best,
                                             WaveSlot *slots, int32_t lane, int32_t *fallback,
                                             int32_t *fallback_count, int32_t *err, int32_t one, int32_t compact);

// Persistent alignment kernel.  Its warps first take the leading
// counters[6] sorted pairs one warp per pair (long pairs, or every pair of a
// small call), then the rest 32 pairs per warp, one lane per pair, in
// register strips of R rows.  Long pairs thus start first and the lane-per-
// pair groups fill in around them.
template <int R, int V, int NT>
__global__ void __launch_bounds__(NT, 1)
sw_strip_kernel(SwIn in, SwOut out, const uint32_t *__restrict__ order,
                const int32_t *__restrict__ counters, const int32_t *__restrict__ inc_global,
                int2 *__restrict__ window, int32_t W, int32_t *__restrict__ ticket,
                int32_t *__restrict__ wave_ticket, int32_t *__restrict__ fallback,
                int32_t *__restrict__ fallback_count, int32_t *err, int32_t one, int32_t wave_rows,
                int32_t wave_rows_force, int32_t wide_key) {
    extern __shared__ int32_t s_inc[];
    if (counters[0] <= 0) return;
    for (int t = threadIdx.x; t < INC_ENTRIES * 32; t += blockDim.x) s_inc[t] = inc_global[t >> 5];
    __syncthreads();
    int32_t *s_best = s_inc + INC_ENTRIES * 32 + (threadIdx.x >> 5) * (track_rows<R>() * 32) + (threadIdx.x & 31);
    const int32_t lane = threadIdx.x & 31;
    const int32_t n_wave = counters[6];
    // stream the pairs' strips through each warp when there are more pairs than
    // warps (each warp then sees several); with fewer, one pair per warp at the
    // rows per strip each pair allows has the shorter wavefronts
    const int32_t n_warps = (int32_t)((gridDim.x * blockDim.x) >> 5);
    if (wave_rows > 0 && (wave_rows_force || n_wave > n_warps)) {
        // slots behind the increment table and the per-row trackers
        char *slot_base = (char *)(s_inc + INC_ENTRIES * 32 + track_rows<R>() * NT);
        WaveSlot *slots = (WaveSlot *)(slot_base + (size_t)(threadIdx.x >> 5) * WAVE_SLOTS_PER_WARP *
                                                       WAVE_SLOT_BYTES);
        // the compact key when every pair of the call (so every warp-per-pair
        // pair) has at most 2047 rows
        if (n_wave > 0)
            wave_stream_any(wave_rows, in, out, order, n_wave, wave_ticket, (const char *)s_inc, s_best, slots,
                            lane, fallback, fallback_count, err, one,
                            !wide_key && counters[8] <= KeyCompact::ROWS_MAX);
    } else {
        for (;;) {
            __syncwarp();
            int32_t q = 0;
            if (lane == 0) q = atomicAdd(wave_ticket, 1);
            q = __shfl_sync(0xffffffffu, q, 0);
            if (q >= n_wave) break;
            align_pair_wave_any(in, out, (int64_t)order[q], (const char *)s_inc, s_best, lane, fallback,
                                fallback_count, err, one, wide_key);
        }
    }
    const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int2 *win = window + (size_t)gwarp * (size_t)W * 32 + lane;
    const int32_t n_elig = counters[0] - n_wave;
    const int32_t n_groups = (n_elig + 31) >> 5;
    order += n_wave;
    for (;;) {
        __syncwarp();
        int32_t grp = 0;
        if (lane == 0) grp = atomicAdd(ticket, 1);
        grp = __shfl_sync(0xffffffffu, grp, 0);
        if (grp >= n_groups) break;
        const int32_t q = grp * 32 + lane;
        if (q < n_elig)
            align_pair_strips<R, V>(in, out, (int64_t)order[q], (const char *)s_inc, s_best, win, W, lane,
                                 fallback, fallback_count, err, one, wide_key);
    }
}

// ----------------------------------------------------------------- wave kernel
// One warp per pair, for pairs too few to fill the GPU one per lane and for
// long pairs whose serial time would set the strip kernel's tail.  Rows are
// cut into strips of R; lane l computes strips l, l + 32, l + 64, ..., and
// at step T strip s works on column j = T - s + 1 + h - w, one column behind
// strip s - 1.  Each step a lane receives by shuffle the (H, E) of the row
// above its strip at column j, which the upstream lane produced the step
// before, and the H it received the step before is its diagonal input.  A
// lane outside its strip's columns sends the out-of-band boundary
// (H = 0, E = -inf), and a lane whose upstream row has left its band
// replaces what it receives by that boundary, so a lane that has moved on to
// its next strip is never read.  Cells use the strip kernel's masked step.
//
// First maximum: a warp-wide running best score gs; when some lane's column
// holds a score >= gs, every lane updates its per-row trackers (strict '>'
// along a row) and gs rises.  A cell below gs cannot be the pair's maximum;
// one equal to it may be, in an earlier row, so '>=' triggers.  At the end
// of a strip its rows merge into the lane's best in row order (strict '>');
// at the end of the pair the lanes agree on the best score, then on the
// lowest row holding it -- clustkit's first cell in row-major order.
template <int R, class K>
__device__ void align_pair_wave(const SwIn &in, const SwOut &out, int64_t p, const PairGeom &g,
                                const char *s_inc, int32_t *s_best, int32_t lane, int32_t *fallback,
                                int32_t *fallback_count, int32_t one) {
    using namespace key;
    constexpr int32_t D = R + 1;
    const int32_t la = g.la, lb = g.lb, w = g.w, h = g.h;
    const uint8_t *A = in.flat + in.offsets[g.a_idx];
    const uint8_t *B = in.flat + in.offsets[g.b_idx];
    const uint32_t w2 = 2u * (uint32_t)w;
    const int32_t c0 = 1 + h - w;  // j = T - s + c0

    // strips that reach column <= lb (later ones lie right of the matrix)
    int32_t n_strips = (la + R - 1) / R;
    {
        const int64_t lim = (int64_t)lb - 1 - h + w;  // s * R <= lim
        const int64_t s_lim = lim < 0 ? 0 : lim / R + 1;
        if (s_lim < n_strips) n_strips = (int32_t)s_lim;
    }
    int32_t lbest = 0, lrow = INT32_MAX;
    if (n_strips > 0) {
        const int32_t J0_0 = c0 > 1 ? c0 : 1;
        const int32_t T_first = J0_0 - c0;
        const int32_t sl = n_strips - 1;
        const int32_t J1_l = sl * R + R + h + w < lb ? sl * R + R + h + w : lb;
        const int32_t T_last = J1_l + sl - c0;

        // this lane's strip at T_first; with at most 32 strips each lane has
        // one and keeps it (its band may then be wider than the rotation allows)
        const bool rotate = n_strips > 32;
        int32_t s = lane;
        if (rotate && T_first >= lane * D) s = lane + 32 * ((T_first - lane * D) / (32 * D));
        int32_t next_switch = rotate ? (s + 32) * D : INT32_MAX;
        int32_t i0 = 0, lo0 = 0, J0 = 0, J1 = -1, alive = 0;
        uint32_t bcol_n = 0;  // residue offset of the strip's next column, loaded a step ahead
        StripRegs<R> S;
        auto setup = [&]() {
            i0 = s * R + 1;
            lo0 = i0 + h - w;
            J0 = lo0 > 1 ? lo0 : 1;
            J1 = i0 + R - 1 + h + w < lb ? i0 + R - 1 + h + w : lb;
            if (s >= n_strips) { J0 = 1; J1 = 0; }
            bcol_n = J0 <= J1 ? (uint32_t)__ldg(B + J0 - 1) * 128u : 0u;
            alive = la - i0 + 1 < R ? la - i0 + 1 : R;
            if (alive < 0) alive = 0;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                S.hc[r] = 0;
                S.fT[r] = K::NEG_F;
                s_best[r * 32] = 0;
                const uint32_t code = (r < alive && s < n_strips) ? (uint32_t)A[i0 + r - 1] : 0u;
                S.arow[r] = (code * (uint32_t)N_CODES * 32u + (uint32_t)lane) * 4u;
            }
        };
        auto merge = [&]() {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int32_t b = s_best[r * 32];
                if (r < alive && b > (lbest | (KU - 1))) { lbest = b; lrow = i0 + r; }
            }
        };
        setup();
        int32_t hout = 0, eout = K::NEG_E, hprev = 0, gs = 1;
        for (int32_t T = T_first; T <= T_last; ++T) {
            if (T == next_switch) {
                merge();
                s += 32;
                next_switch += 32 * D;
                setup();
            }
            const int32_t j = T - s + c0;
            int32_t hin = __shfl_sync(0xffffffffu, hout, (lane + 31) & 31);
            int32_t ein = __shfl_sync(0xffffffffu, eout, (lane + 31) & 31);
            // H(row above, j - 1) arrived the step before; both it and this
            // step's values are judged against the strip held now
            const int32_t top = s * R + h + w;  // last in-band column of the row above
            const int32_t hdiag = (s == 0 || j - 1 > top) ? 0 : hprev;
            hprev = hin;
            if (s == 0 || j > top) { hin = 0; ein = K::NEG_E; }
            int32_t cm = 0;
            if (j >= J0 && j <= J1) {
                const uint32_t bcol = bcol_n;
                if (j < J1) bcol_n = (uint32_t)__ldg(B + j) * 128u;  // column j + 1
                int32_t hu = hin, eu = ein;
                strip_cells<R, 0, R, true, K>(bcol, hu, eu, hdiag, S, s_inc, band_rows(j - lo0, w2, alive), one);
                hout = hu;
                eout = eu;
                cm = S.hc[0];
#pragma unroll
                for (int r = 1; r + 1 < R; r += 2) cm = __vimax3_s32(cm, S.hc[r], S.hc[r + 1]);
                if ((R & 1) == 0) cm = max(cm, S.hc[R - 1]);
            } else {
                hout = 0;
                eout = K::NEG_E;
            }
            if constexpr (K::COMPACT) {
                if ((T & 3) == 3) {  // at most 4 F extensions between clears (T is warp-uniform)
#pragma unroll
                    for (int r = 0; r < R; ++r) S.fT[r] &= ~K::CTR;
                }
            }
            if (__any_sync(0xffffffffu, (cm >> 16) >= gs)) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int32_t b = s_best[r * 32];
                    if (S.hc[r] > (b | (KU - 1))) s_best[r * 32] = S.hc[r];
                }
                const int32_t m = __reduce_max_sync(0xffffffffu, cm >> 16);
                if (m > gs) gs = m;
            }
        }
        merge();
    }
    // lanes agree on the best score, then on the lowest row holding it
    const int32_t best = __reduce_max_sync(0xffffffffu, lbest >> 16);
    const int32_t row = __reduce_min_sync(0xffffffffu, (best > 0 && (lbest >> 16) == best) ? lrow : INT32_MAX);
    const bool writer = best > 0 ? ((lbest >> 16) == best && lrow == row) : lane == 0;
    const uint32_t wmask = __ballot_sync(0xffffffffu, writer);
    if (lane != __ffs(wmask) - 1) return;
    if (best >= SCORE_LIMIT) {
        const int32_t pos = atomicAdd(fallback_count, 1);
        fallback[pos] = (int32_t)p;
        atomicAdd(fallback_count + 2, 1);  // re-run counter
        return;
    }
    write_result(out, in, p, best, best > 0 ? (lbest & K::MATCH_MASK) : 0, la, la, lb);
}

// One sorted wave pair, at the rows per strip its shape allows.
template <class K>
__device__ __forceinline__ void align_pair_wave_k(const SwIn &in, const SwOut &out, int64_t p, const PairGeom &g,
                                                  const char *s_inc, int32_t *s_best, int32_t lane,
                                                  int32_t *fallback, int32_t *fallback_count, int32_t one) {
    switch (wave_rows_per_strip(g.la, g.w)) {
        case 4: align_pair_wave<4, K>(in, out, p, g, s_inc, s_best, lane, fallback, fallback_count, one); break;
        case 8: align_pair_wave<8, K>(in, out, p, g, s_inc, s_best, lane, fallback, fallback_count, one); break;
        default: align_pair_wave<16, K>(in, out, p, g, s_inc, s_best, lane, fallback, fallback_count, one); break;
    }
}

// the compact key for a pair of at most 2047 rows (unless wide_key)
__device__ __noinline__ void align_pair_wave_any(const SwIn &in, const SwOut &out, int64_t p,
                                                 const char *s_inc, int32_t *s_best, int32_t lane,
                                                 int32_t *fallback, int32_t *fallback_count,
                                                 int32_t *err, int32_t one, int32_t wide_key) {
    const PairGeom g = pair_geometry(in, p, err);
    if (!wide_key && g.la <= KeyCompact::ROWS_MAX)
        align_pair_wave_k<KeyCompact>(in, out, p, g, s_inc, s_best, lane, fallback, fallback_count, one);
    else
        align_pair_wave_k<KeyWide>(in, out, p, g, s_inc, s_best, lane, fallback, fallback_count, one);
}

// ----------------------------------------------------------------- streamed warp-per-pair
// The warp-per-pair phase with the strips of consecutive pairs streamed
// through one warp, so that lanes freed by one pair's strips take the next
// pair's instead of idling while the pair's wavefront fills and drains.  All
// pairs of the call share R (chosen from the band width so every pair can
// rotate).  Strips carry one global sequence number g; lane g mod 32 runs
// strip g.  Strip s of a pair starting at T0 runs column j at step
// T0 + s + j - J0(strip 0), i.e. exactly one step behind its upstream strip
// s - 1 at every column, so the (H, E) hand-over by shuffle works as in the
// single-pair schedule.  A pair is issued (one per step, once every strip
// of the previous one has started) with the smallest T0 at which each of its
// first 32 strips finds its lane free; its later strips rotate through the
// same lanes as before.  A lane's strip whose upstream lane belongs to
// another pair or strip reads the out-of-band boundary instead (overrides
// below), so a lane never reads a neighbour's unrelated values.
//
// Per pair, a slot in shared memory holds its geometry, the running best
// score (first-maximum trigger; each lane compares with its own copy, taken
// when its strip starts and refreshed when it triggers, which is never above
// the slot's, so a copy that lags only adds trigger steps) and the best cell
// as one packed 64-bit value
// (score, then lower row, then match count), merged by atomicMax at each
// strip's end; the pair's last strip ends last and writes the result.
constexpr int WS_SLOTS = 16;

struct WaveSlot {
    unsigned long long acc;   // score << 27 | (16383 - row) << 13 | matches
    int64_t a_off, b_off;     // residues of the row and column sequences
    int64_t p;                // pair index
    int32_t la, lb, w, h, c0, S, J00, T0;
    int32_t gs;               // running best score of the pair (first-maximum trigger)
    int32_t live;
};

static_assert(sizeof(WaveSlot) == WAVE_SLOT_BYTES, "slot layout");
static_assert(WS_SLOTS == WAVE_SLOTS_PER_WARP, "slot count");

template <int R>
__device__ __forceinline__ void strip_bounds(const WaveSlot &sl, int32_t s, int32_t &i0, int32_t &lo,
                                             int32_t &J0, int32_t &J1, int32_t &alive) {
    i0 = s * R + 1;
    lo = s * R + sl.c0;
    J0 = lo > 1 ? lo : 1;
    const int32_t hi = lo + R - 1 + 2 * sl.w;
    J1 = hi < sl.lb ? hi : sl.lb;
    alive = sl.la - i0 + 1 < R ? sl.la - i0 + 1 : R;
    if (alive < 0) alive = 0;
}
template <int R>
__device__ __forceinline__ int32_t strip_t0(const WaveSlot &sl, int32_t s) {
    const int32_t lo = s * R + sl.c0;
    return sl.T0 + s + (lo > 1 ? lo : 1) - sl.J00;
}
template <int R>
__device__ __forceinline__ int32_t strip_te(const WaveSlot &sl, int32_t s) {
    const int32_t lo = s * R + sl.c0;
    const int32_t hi = lo + R - 1 + 2 * sl.w;
    const int32_t J1 = hi < sl.lb ? hi : sl.lb;
    const int32_t te = sl.T0 + s + J1 - sl.J00;
    const int32_t t0 = strip_t0<R>(sl, s);
    return te > t0 ? te : t0;  // a strip whose band lies left of column 1 ends where it starts
}

template <int R, class K>
__device__ void wave_stream(const SwIn &in, const SwOut &out, const uint32_t *order, int32_t n_wave,
                            int32_t *ticket, const char *s_inc, int32_t *s_best, WaveSlot *slots, int32_t lane,
                            int32_t *fallback, int32_t *fallback_count, int32_t *err, int32_t one) {
    using namespace key;
    constexpr uint32_t FULL = 0xffffffffu;
    // warp-uniform schedule state
    int32_t T = 0, T_issue = -1, g_next = 0, seq = 0;
    bool exhausted = false;
    for (int i = lane; i < WS_SLOTS; i += 32) slots[i].live = 0;
    __syncwarp();
    // per-lane strip state
    int32_t cur_slot = -1, cur_s = 0, i0 = 0, lo0 = 0, J0 = 1, J1 = 0, alive = 0, te = 0, top = 0;
    int32_t jb = 0;    // j = T + jb for the strip held
    uint32_t w2s = 0;  // 2w of its pair
    uint32_t bcol_n = 0;  // residue offset of its next column, loaded a step ahead
    int32_t pend_slot = -1, pend_s = 0, pend_t0 = 0;
    int32_t F = -1;
    int32_t hout = 0, eout = K::NEG_E, hprev = 0;
    // the held strip's pair's running best score as last seen by this lane: at
    // most the slot's, so its trigger fires at least whenever the slot's would
    int32_t gs_l = 1;
    const uint8_t *B = nullptr;
    StripRegs<R> S;
    for (;;) {
        // ---- issue one pair (warp-uniform)
        if (!exhausted && T > T_issue && !slots[seq % WS_SLOTS].live) {
            int32_t q = 0;
            if (lane == 0) q = atomicAdd(ticket, 1);
            q = __shfl_sync(FULL, q, 0);
            if (q >= n_wave) {
                exhausted = true;
            } else {
                const int64_t p = (int64_t)order[q];
                const PairGeom g = pair_geometry(in, p, err);
                int32_t n_strips = (g.la + R - 1) / R;
                {
                    const int64_t lim = (int64_t)g.lb - 1 - g.h + g.w;
                    const int64_t s_lim = lim < 0 ? 0 : lim / R + 1;
                    if (s_lim < n_strips) n_strips = (int32_t)s_lim;
                }
                if (n_strips <= 0) {
                    if (lane == 0) write_result(out, in, p, 0, 0, g.la, g.la, g.lb);
                } else {
                    WaveSlot &sl = slots[seq % WS_SLOTS];
                    const int32_t c0 = 1 + g.h - g.w;
                    const int32_t J00 = c0 > 1 ? c0 : 1;
                    const int32_t m = (lane - g_next) & 31;
                    const int32_t first = n_strips < 32 ? n_strips : 32;
                    int32_t req = T;
                    if (m < first) {
                        const int32_t lom = m * R + c0;
                        const int32_t r = F + 1 - m - ((lom > 1 ? lom : 1) - J00);
                        req = r > T ? r : T;
                    }
                    const int32_t T0p = __reduce_max_sync(FULL, req);
                    if (lane == 0) {
                        sl.acc = 0;
                        sl.a_off = in.offsets[g.a_idx];
                        sl.b_off = in.offsets[g.b_idx];
                        sl.p = p;
                        sl.la = g.la; sl.lb = g.lb; sl.w = g.w; sl.h = g.h; sl.c0 = c0;
                        sl.S = n_strips; sl.J00 = J00; sl.T0 = T0p; sl.gs = 1; sl.live = 1;
                    }
                    __syncwarp();
                    if (m < first) {
                        pend_slot = seq % WS_SLOTS;
                        pend_s = m;
                        pend_t0 = strip_t0<R>(sl, m);
                        const int32_t last = m + 32 * ((n_strips - 1 - m) / 32);
                        F = strip_te<R>(sl, last);
                    }
                    T_issue = strip_t0<R>(sl, n_strips - 1);
                    g_next += n_strips;
                    ++seq;
                }
            }
        }
        // ---- start this lane's next strip.  Its start step is never in the past
        // (the rotation bound on R); were it, the strip starts now and the call
        // reports an internal error rather than the warp waiting forever.
        if (pend_slot >= 0 && T >= pend_t0) {
            if (T > pend_t0) atomicOr(err, ERRBIT_SCHEDULE);
            const WaveSlot &sl = slots[pend_slot];
            cur_slot = pend_slot;
            cur_s = pend_s;
            pend_slot = -1;
            gs_l = sl.gs;
            strip_bounds<R>(sl, cur_s, i0, lo0, J0, J1, alive);
            te = strip_te<R>(sl, cur_s);
            if (te < T) te = T;  // only after a late start: the strip still ends
            top = cur_s * R + sl.h + sl.w;
            jb = sl.J00 - sl.T0 - cur_s;
            w2s = 2u * (uint32_t)sl.w;
            B = in.flat + sl.b_off;
            bcol_n = J0 <= J1 ? (uint32_t)__ldg(B + J0 - 1) * 128u : 0u;
            const uint8_t *A = in.flat + sl.a_off;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                S.hc[r] = 0;
                S.fT[r] = K::NEG_F;
                s_best[r * 32] = 0;
                const uint32_t code = r < alive ? (uint32_t)A[i0 + r - 1] : 0u;
                S.arow[r] = (code * (uint32_t)N_CODES * 32u + (uint32_t)lane) * 4u;
            }
        }
        // ---- one column of this lane's strip
        int32_t hin = __shfl_sync(FULL, hout, (lane + 31) & 31);
        int32_t ein = __shfl_sync(FULL, eout, (lane + 31) & 31);
        int32_t cm = 0;
        const bool has = cur_slot >= 0;
        int32_t j = 0;
        if (has) {
            j = T + jb;
            const int32_t hdiag = (cur_s == 0 || j - 1 > top || j - 1 < 1) ? 0 : hprev;
            hprev = hin;
            if (cur_s == 0 || j > top) { hin = 0; ein = K::NEG_E; }
            if (j >= J0 && j <= J1) {
                const uint32_t bcol = bcol_n;
                if (j < J1) bcol_n = (uint32_t)__ldg(B + j) * 128u;  // column j + 1
                int32_t hu = hin, eu = ein;
                strip_cells<R, 0, R, true, K>(bcol, hu, eu, hdiag, S, s_inc, band_rows(j - lo0, w2s, alive), one);
                hout = hu;
                eout = eu;
                cm = S.hc[0];
#pragma unroll
                for (int r = 1; r + 1 < R; r += 2) cm = __vimax3_s32(cm, S.hc[r], S.hc[r + 1]);
                if ((R & 1) == 0) cm = max(cm, S.hc[R - 1]);
            } else {
                hout = 0;
                eout = K::NEG_E;
            }
        } else {
            hprev = hin;
            hout = 0;
            eout = K::NEG_E;
        }
        if constexpr (K::COMPACT) {
            if ((T & 3) == 3) {  // at most 4 F extensions between clears (T is warp-uniform)
#pragma unroll
                for (int r = 0; r < R; ++r) S.fT[r] &= ~K::CTR;
            }
        }
        // ---- first-maximum trackers: per-pair running best score
        const bool trig = has && (cm >> 16) >= gs_l;
        if (__any_sync(FULL, trig)) {
            if (has) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int32_t b = s_best[r * 32];
                    if (S.hc[r] > (b | (KU - 1))) s_best[r * 32] = S.hc[r];
                }
                if (cm > 0) gs_l = max(atomicMax(&slots[cur_slot].gs, cm >> 16), cm >> 16);
            }
        }
        // ---- strip end: merge its rows into the pair's best; the last strip writes
        if (has && T == te) {
            int32_t bk = 0, br = 0;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int32_t b = s_best[r * 32];
                if (r < alive && b > (bk | (KU - 1))) { bk = b; br = i0 + r; }
            }
            WaveSlot &sl = slots[cur_slot];
            if (bk > 0)
                atomicMax(&sl.acc, ((unsigned long long)(uint32_t)(bk >> 16) << 27) |
                                       ((unsigned long long)(uint32_t)(16383 - br) << 13) |
                                       (unsigned long long)(uint32_t)(bk & K::MATCH_MASK));
            if (cur_s == sl.S - 1) {
                __threadfence_block();
                const unsigned long long acc = atomicAdd(&sl.acc, 0ull);
                const int32_t score = (int32_t)(acc >> 27);
                if (score >= SCORE_LIMIT) {
                    const int32_t pos = atomicAdd(fallback_count, 1);
                    fallback[pos] = (int32_t)sl.p;
                    atomicAdd(fallback_count + 2, 1);  // re-run counter
                } else {
                    write_result(out, in, sl.p, score, score > 0 ? (int32_t)(acc & MATCH_MASK) : 0, sl.la, sl.la,
                                 sl.lb);
                }
                sl.live = 0;
            } else if (cur_s + 32 < sl.S) {
                pend_slot = cur_slot;
                pend_s = cur_s + 32;
                pend_t0 = strip_t0<R>(sl, pend_s);
            }
            cur_slot = -1;
        }
        __syncwarp();
        ++T;
        if (__all_sync(FULL, exhausted && cur_slot < 0 && pend_slot < 0)) break;
    }
}

template <class K>
__device__ __forceinline__ void wave_stream_k(int32_t rows, const SwIn &in, const SwOut &out, const uint32_t *order,
                                              int32_t n_wave, int32_t *ticket, const char *s_inc, int32_t *s_best,
                                              WaveSlot *slots, int32_t lane, int32_t *fallback,
                                              int32_t *fallback_count, int32_t *err, int32_t one) {
    switch (rows) {
        case 4: wave_stream<4, K>(in, out, order, n_wave, ticket, s_inc, s_best, slots, lane, fallback, fallback_count, err, one); break;
        case 8: wave_stream<8, K>(in, out, order, n_wave, ticket, s_inc, s_best, slots, lane, fallback, fallback_count, err, one); break;
        default: wave_stream<16, K>(in, out, order, n_wave, ticket, s_inc, s_best, slots, lane, fallback, fallback_count, err, one); break;
    }
}

__device__ __noinline__ void wave_stream_any(int32_t rows, const SwIn &in, const SwOut &out, const uint32_t *order,
                                             int32_t n_wave, int32_t *ticket, const char *s_inc, int32_t *s_best,
                                             WaveSlot *slots, int32_t lane, int32_t *fallback,
                                             int32_t *fallback_count, int32_t *err, int32_t one, int32_t compact) {
    if (compact)
        wave_stream_k<KeyCompact>(rows, in, out, order, n_wave, ticket, s_inc, s_best, slots, lane, fallback,
                                  fallback_count, err, one);
    else
        wave_stream_k<KeyWide>(rows, in, out, order, n_wave, ticket, s_inc, s_best, slots, lane, fallback,
                               fallback_count, err, one);
}

// ----------------------------------------------------------------- driver
static int32_t pow2_at_least(int64_t x) {
    int32_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

// Tunables (set by ck_sw_set_config, chosen by the autotuner).
static int32_t g_rows_per_strip = 0;  // 0: by band width (8 up to w = 64, else 16)
// -1 (default): by strip height -- groups of 4 columns at 8 rows (3), of 2
// above (1); 0..3 as set (see StripVariant)
static int32_t g_variant = -1;
// threads of the strip kernel's CTA for 8-row strips: 512, 640 or 768; 0 =
// 640.  16-row strips run 512, taller ones 256.
static int32_t g_strip_threads = 0;
// 1: the wide key for every pair of the strip kernel (measurement); 0
// (default): the compact key for pairs of at most 2047 rows
static int32_t g_wide_key = 0;
// every pair runs one warp per pair when a call has at most this many pairs;
// in larger calls, long pairs do: rows >= max(min rows, the adaptive bound)
static int32_t g_wave_all_below = 40960;
static int32_t g_wave_min_rows = 512;
static int32_t g_wave_adaptive = 1;
// stream the strips of consecutive pairs through a warp: 1 when the call has
// more warp-per-pair pairs than warps, 2 always, 0 never
static int32_t g_wave_stream = 1;
// rows per strip of the streamed schedule: 0 = the smallest that rotates,
// else 4, 8 or 16 when at least that (taller strips rotate a fortiori)
static int32_t g_wave_rows = 0;

// Rows per strip shared by every warp-per-pair pair of a call: the smallest
// that lets a strip of any of them rotate through 32 lanes (half-widths up to
// max(band width, 50); with a wider band every pair has at most 512 rows, as
// the routing guarantees, so 16 rows give at most 32 strips).  0: one pair
// per warp at a time.
static int32_t wave_rows_for(int32_t wmax) {
    if (!g_wave_stream) return 0;
    const int32_t r = 2 * wmax < 31 * 4 + 32 ? 4 : 2 * wmax < 31 * 8 + 32 ? 8 : 16;
    return g_wave_rows > r ? g_wave_rows : r;
}

int32_t sw_set_wave(int32_t key, int32_t v) {
    if (v < 0) {
        set_error(CK_ERR_INVALID_ARGUMENT, "warp-per-pair settings must be >= 0");
        return CK_ERR_INVALID_ARGUMENT;
    }
    if (key == 4 && v != 0 && v != 4 && v != 8 && v != 16) {
        set_error(CK_ERR_UNSUPPORTED, "streamed strip rows must be 0 (smallest rotating), 4, 8 or 16");
        return CK_ERR_UNSUPPORTED;
    }
    if (key == 0) g_wave_min_rows = v;
    else if (key == 1) g_wave_all_below = v;
    else if (key == 2) g_wave_adaptive = v ? 1 : 0;
    else if (key == 3) g_wave_stream = v > 2 ? 2 : v;
    else g_wave_rows = v;
    return CK_OK;
}
int32_t sw_wave(int32_t key) {
    return key == 0 ? g_wave_min_rows : key == 1 ? g_wave_all_below : key == 2 ? g_wave_adaptive
         : key == 3 ? g_wave_stream : g_wave_rows;
}

int32_t sw_set_variant(int32_t v) {
    if (v < -1 || v > 3) {
        set_error(CK_ERR_UNSUPPORTED, "strip kernel variant must be -1 (by strip height) or 0..3");
        return CK_ERR_UNSUPPORTED;
    }
    g_variant = v;
    return CK_OK;
}
int32_t sw_variant() { return g_variant; }


int32_t sw_set_rows_per_strip(int32_t r) {
    if (r != 0 && r != 8 && r != 16 && r != 24 && r != 32) {
        set_error(CK_ERR_UNSUPPORTED, "rows per strip must be 0 (by band width), 8, 16, 24 or 32");
        return CK_ERR_UNSUPPORTED;
    }
    g_rows_per_strip = r;
    return CK_OK;
}
int32_t sw_rows_per_strip() { return g_rows_per_strip; }

int32_t sw_set_strip_threads(int32_t v) {
    if (v != 0 && v != 512 && v != 640 && v != 768) {
        set_error(CK_ERR_UNSUPPORTED, "strip kernel threads per CTA must be 0 (default), 512, 640 or 768");
        return CK_ERR_UNSUPPORTED;
    }
    g_strip_threads = v;
    return CK_OK;
}
int32_t sw_strip_threads() { return g_strip_threads; }

int32_t sw_set_wide_key(int32_t v) {
    if (v != 0 && v != 1) {
        set_error(CK_ERR_UNSUPPORTED, "strip key form must be 0 (compact where rows fit) or 1 (wide)");
        return CK_ERR_UNSUPPORTED;
    }
    g_wide_key = v;
    return CK_OK;
}
int32_t sw_wide_key() { return g_wide_key; }

// threads of the strip kernel's CTA (one per SM) for strips of `rows` rows
static int32_t strip_threads(int32_t rows) {
    if (rows >= 24) return 256;
    if (rows == 16) return 512;
    return g_strip_threads ? g_strip_threads : 640;
}

template <int R, int V, int NT>
static int32_t launch_strips(const SwIn &in, const SwOut &out, const uint32_t *order,
                             const int32_t *counters, const int32_t *inc, int32_t wmax,
                             int32_t *ticket, int32_t *fallback, int32_t *fb_count,
                             int32_t *err, cudaStream_t st, SwCounters *ctr) {
    int32_t status = CK_OK;
    auto kern = sw_strip_kernel<R, V, NT>;
    const size_t smem = strip_smem<R, NT>();
    CK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    CK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem));
    if (per_sm < 1) {
        set_error(CK_ERR_UNSUPPORTED, "strip kernel CTA does not fit an SM");
        return CK_ERR_UNSUPPORTED;
    }
    const int32_t W = pow2_at_least(2 * (int64_t)wmax + 2 * R + 2);
    // one window of W columns per lane; keep the total under 8 GiB
    const size_t per_block = (size_t)NT * (size_t)W * sizeof(int2);
    int blocks = sm_count();  // one persistent CTA per SM
    const size_t cap = (size_t)8 << 30;
    if ((size_t)blocks * per_block > cap) blocks = (int)(cap / per_block);
    if (blocks < 1) blocks = 1;
    int2 *window = (int2 *)scratch(SLOT_WINDOW, (size_t)blocks * per_block, &status);
    if (!window) return status;
    kern<<<blocks, NT, smem, st>>>(in, out, order, counters, inc, window, W, ticket,
                                              ticket + 5, fallback, fb_count, err, 1, wave_rows_for(wmax),
                                              g_wave_stream == 2 ? 1 : 0, g_wide_key);
    CK_CUDA(cudaGetLastError());
    if (ctr) ctr->launches += 1;
    return CK_OK;
}

template <int R, int NT>
static int32_t launch_strips_m(const SwIn &in, const SwOut &out, const uint32_t *order,
                               const int32_t *counters, const int32_t *inc, int32_t wmax,
                               int32_t *ticket, int32_t *fallback, int32_t *fb_count,
                               int32_t *err, cudaStream_t st, SwCounters *ctr) {
    switch (g_variant >= 0 ? g_variant : (R <= 8 ? 3 : 1)) {
        case 0: return launch_strips<R, 0, NT>(in, out, order, counters, inc, wmax, ticket, fallback, fb_count, err, st, ctr);
        case 2: return launch_strips<R, 2, NT>(in, out, order, counters, inc, wmax, ticket, fallback, fb_count, err, st, ctr);
        case 3: return launch_strips<R, 3, NT>(in, out, order, counters, inc, wmax, ticket, fallback, fb_count, err, st, ctr);
        default: return launch_strips<R, 1, NT>(in, out, order, counters, inc, wmax, ticket, fallback, fb_count, err, st, ctr);
    }
}

// strips of R rows in CTAs of nt threads (strip_threads: 512/640/768 for 8 rows,
// 512 for 16, 256 for 24 and 32)
template <int R>
static int32_t launch_strips_v(const SwIn &in, const SwOut &out, const uint32_t *order,
                               const int32_t *counters, const int32_t *inc, int32_t wmax,
                               int32_t *ticket, int32_t *fallback, int32_t *fb_count,
                               int32_t *err, cudaStream_t st, SwCounters *ctr, int32_t nt) {
    if constexpr (R >= 24) {
        return launch_strips_m<R, 256>(in, out, order, counters, inc, wmax, ticket, fallback, fb_count, err, st, ctr);
    } else if constexpr (R == 8) {
        if (nt == 768)
            return launch_strips_m<R, 768>(in, out, order, counters, inc, wmax, ticket, fallback, fb_count, err, st, ctr);
        if (nt == 640)
            return launch_strips_m<R, 640>(in, out, order, counters, inc, wmax, ticket, fallback, fb_count, err, st, ctr);
        return launch_strips_m<R, 512>(in, out, order, counters, inc, wmax, ticket, fallback, fb_count, err, st, ctr);
    } else {
        return launch_strips_m<R, 512>(in, out, order, counters, inc, wmax, ticket, fallback, fb_count, err, st, ctr);
    }
}

int32_t sw_batched_launch(const SwIn &in, const SwOut &out, int64_t M, const int8_t *d_sub,
                          int32_t *d_err, cudaStream_t st, SwCounters *ctr, bool read_counters) {
    int32_t status = CK_OK;
    if (M >= (int64_t)INT32_MAX) {
        set_error(CK_ERR_UNSUPPORTED, "more than 2^31-1 pairs in one call");
        return CK_ERR_UNSUPPORTED;
    }
    // counters: [0] eligible, [1] fallback list length, [2] ticket, [3] overflow re-runs,
    // [4..5] cells (u64)
    int32_t *cnt = (int32_t *)scratch(SLOT_COUNTERS, 256, &status);
    if (!cnt) return status;
    CK_CUDA(cudaMemsetAsync(cnt, 0, 64, st));
    unsigned long long *cells = (unsigned long long *)(cnt + 4);

    uint8_t *ok = (uint8_t *)scratch(SLOT_SEQ_OK, (size_t)(in.n_seqs > 0 ? in.n_seqs : 1), &status);
    if (!ok) return status;
    CK_CUDA(cudaMemsetAsync(ok, 0, (size_t)(in.n_seqs > 0 ? in.n_seqs : 1), st));
    int32_t *inc = (int32_t *)scratch(SLOT_INC, INC_ENTRIES * sizeof(int32_t), &status);
    if (!inc) return status;
    build_inc_kernel<<<(INC_ENTRIES + 127) / 128, 128, 0, st>>>(d_sub, inc);
    CK_CUDA(cudaGetLastError());

    const size_t n = (size_t)(M > 0 ? M : 1);
    uint32_t *k0 = (uint32_t *)scratch(SLOT_SORT_KEYS, n * 4, &status);
    uint32_t *v0 = (uint32_t *)scratch(SLOT_SORT_VALS, n * 4, &status);
    uint32_t *k1 = (uint32_t *)scratch(SLOT_SORT_KEYS_ALT, n * 4, &status);
    uint32_t *v1 = (uint32_t *)scratch(SLOT_SORT_VALS_ALT, n * 4, &status);
    int32_t *fb = (int32_t *)scratch(SLOT_FALLBACK, n * 4, &status);
    if (!k0 || !v0 || !k1 || !v1 || !fb) return status;
    if (ctr) ctr->launches += 2;
    if (M > 0) {
        int64_t want = (M + 255) / 256;
        int blocks = (int)(want < 16 * (int64_t)sm_count() ? want : 16 * (int64_t)sm_count());
        sw_prep_kernel<<<blocks, 256, 0, st>>>(in, out, M, ok, k0, v0, fb, cnt, cells, d_err);
        CK_CUDA(cudaGetLastError());
        cub::DoubleBuffer<uint32_t> dk(k0, k1), dv(v0, v1);
        size_t temp = 0;
        CK_CUDA(cub::DeviceRadixSort::SortPairsDescending(nullptr, temp, dk, dv, (int)M, 0, 26, st));
        void *tmp = scratch(SLOT_SORT_TEMP, temp > 0 ? temp : 1, &status);
        if (!tmp) return status;
        CK_CUDA(cub::DeviceRadixSort::SortPairsDescending(tmp, temp, dk, dv, (int)M, 0, 26, st));
        int32_t wmax = 0;
        CK_TRY(widest_band(in, st, &wmax));
        const uint32_t *order = dv.Current();
        // narrow bands: a strip's ramps (R - 1 masked columns at each end) weigh
        // against 2w + 1 interior columns, so fewer rows per strip win there
        int32_t rows = g_rows_per_strip ? g_rows_per_strip : (wmax <= 64 ? 8 : 16);
        // A call that routes every pair one warp per pair (at most
        // CK_CFG_WAVE_ALL_BELOW pairs, a band narrow enough for every pair to
        // rotate) never runs lane-per-pair strips: the 8-row kernel's larger
        // CTA gives its warp-per-pair phase 20 warps per SM instead of 16
        // (search-shaped calls of 8 k and 32 k pairs: 9-18 % faster), unless
        // the call has no more pairs than 16 warps per SM -- one pair per warp,
        // where the 512-thread CTA's unspilled code is the faster.
        const bool wave_only = !g_rows_per_strip && M <= (int64_t)g_wave_all_below && in.band_width >= 1 &&
                               2 * in.band_width < 31 * 16 + 32;
        if (wave_only) rows = 8;
        int32_t nt = strip_threads(rows);
        if (wave_only && !g_strip_threads && M <= 16 * (int64_t)sm_count()) nt = 512;
        wave_split_kernel<<<1, 32, 0, st>>>(dk.Current(), cnt, in.band_width, g_wave_all_below,
                                            g_wave_min_rows, g_wave_adaptive, (int64_t)sm_count() * nt);
        CK_CUDA(cudaGetLastError());
        // profiling events bracket the alignment kernel
        cudaEvent_t ev0 = nullptr, ev1 = nullptr;
        if (profile_events(&ev0, &ev1)) CK_CUDA(cudaEventRecord(ev0, st));
        switch (rows) {
            case 8:
                CK_TRY(launch_strips_v<8>(in, out, order, cnt, inc, wmax, cnt + 2, fb, cnt + 1, d_err, st, ctr, nt));
                break;
            case 24:
                CK_TRY(launch_strips_v<24>(in, out, order, cnt, inc, wmax, cnt + 2, fb, cnt + 1, d_err, st, ctr, nt));
                break;
            case 32:
                CK_TRY(launch_strips_v<32>(in, out, order, cnt, inc, wmax, cnt + 2, fb, cnt + 1, d_err, st, ctr, nt));
                break;
            default:
                CK_TRY(launch_strips_v<16>(in, out, order, cnt, inc, wmax, cnt + 2, fb, cnt + 1, d_err, st, ctr, nt));
                break;
        }
        if (ev1) CK_CUDA(cudaEventRecord(ev1, st));
        if (ctr) ctr->launches += 1;
    }
    // plain kernel over the fallback list (its length is read on the device)
    CK_TRY(sw_plain_launch(in, out, M, fb, cnt + 1, d_err, st, ctr));
    if (read_counters && ctr) {
        int32_t hcnt[8];
        CK_CUDA(cudaMemcpyAsync(hcnt, cnt, 32, cudaMemcpyDeviceToHost, st));
        // hcnt[6]: pairs the warp-per-pair kernel took (part of hcnt[0])
        CK_CUDA(cudaStreamSynchronize(st));
        unsigned long long c = 0;
        memcpy(&c, hcnt + 4, sizeof(c));
        ctr->batched += hcnt[0];
        ctr->plain += hcnt[1];
        ctr->rerun += hcnt[3];
        ctr->wave += hcnt[6];
        ctr->cells += (int64_t)c;
    }
    return CK_OK;
}

}  // namespace ck
