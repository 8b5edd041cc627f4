/*
 * oracle.c -- CPU restatement of clustkit's Align-phase and sketch arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path: it
 * is linked by tests/, by __graft_entry__.smoke() and by the cpu_baseline /
 * reference leg of bench.py, and by nothing in the product library.
 *
 * Every function restates one reference function (paths are relative to the
 * clustkit project root):
 *
 *   or_sw_one      clustkit/csrc/sw_align.c:25-177   (sw_align_one)
 *   or_sw_batch    clustkit/csrc/sw_align.c:182-266  (batch_sw_align_c)
 *   or_fmix64      clustkit/sketch.py:17-26          (_murmurhash3_fmix)
 *   or_sketch      clustkit/sketch.py:29-80, 97-109  (_sketch_one,
 *                                                     _compute_sketches_compact)
 *   or_jaccard     clustkit/pairwise.py:1564-1612    (_jaccard_sorted,
 *                                                     _batch_jaccard)
 *
 * The SW restatement keeps one row of (H, E, Hm, Em) per column and updates it
 * in place (the reference toggles two rows); the band semantics are the
 * reference's: every cell outside row i's band [i+h-w, i+h+w] n [1, lb] acts
 * as H = 0, E = F = -inf with zero match counts.  The sketch restatement
 * hashes every k-mer and keeps the s smallest (multiset) with a bounded max
 * heap, which is the set the reference's online replace-the-maximum loop
 * keeps.  Both formulations are pinned against the reference itself by the
 * golden fixtures and by oracle/_ref (the reference C built from source).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_NEG_INF (-1000000)
#define OR_GAP_OPEN (-11)
#define OR_GAP_EXTEND (-1)

/* clustkit/csrc/sw_align.c:19-21 */
void or_set_num_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int32_t or_max_threads(void) {
#ifdef _OPENMP
    return (int32_t)omp_get_max_threads();
#else
    return 1;
#endif
}

/*
 * Banded local alignment of a (rows, la <= lb) against b (columns).
 * clustkit/csrc/sw_align.c:25-177.  Workspace arrays hold lb + 2 entries.
 * Writes the best score (0 when no positive cell) and the match count of the
 * first cell, in row-major order, that reaches it (sw_align.c:156-159).
 */
static void or_sw_one(const uint8_t *a, int32_t la, const uint8_t *b, int32_t lb,
                      int32_t band_width, int32_t hint, const int8_t *sub,
                      int32_t *H, int32_t *E, int32_t *Hm, int32_t *Em,
                      int32_t *score_out, int32_t *matches_out) {
    *score_out = 0;
    *matches_out = 0;
    if (la == 0 || lb == 0) return;

    /* sw_align.c:55-58: full matrix when bw <= 0 or the longer side <= 50 */
    int32_t longer = la > lb ? la : lb;
    int32_t w = (band_width <= 0 || longer <= 50) ? longer : band_width;

    for (int32_t j = 0; j <= lb + 1; j++) {
        H[j] = 0; E[j] = OR_NEG_INF; Hm[j] = 0; Em[j] = 0;
    }

    int32_t best_score = 0, best_matches = 0;

    for (int32_t i = 1; i <= la; i++) {
        int64_t lo = (int64_t)i + hint - w;
        int64_t hi = (int64_t)i + hint + w;
        int32_t js = lo < 1 ? 1 : (int32_t)lo;
        int32_t je = hi > lb ? lb : (int32_t)hi;
        if (hi < 1) continue;          /* band entirely left of column 1 */
        if (js > lb) break;            /* band entirely right of column lb */

        const uint8_t ai = a[i - 1];
        /* H(i-1, js-1): column 0 is 0, otherwise it lies in row i-1's band */
        int32_t hd = H[js - 1], hmd = Hm[js - 1];
        /* H(i, js-1) is outside row i's band: 0, and F starts at -inf */
        int32_t hl = 0, hml = 0;
        int32_t f = OR_NEG_INF, fm = 0;

        for (int32_t j = js; j <= je; j++) {
            const uint8_t bj = b[j - 1];
            int32_t s = (ai < 20 && bj < 20) ? (int32_t)sub[ai * 20 + bj] : -4;
            int32_t diag = hd + s;
            int32_t diag_m = hmd + (ai == bj ? 1 : 0);

            /* values of row i-1 at column j, read before the in-place write */
            int32_t hu = H[j], hmu = Hm[j];
            int32_t eu = E[j], emu = Em[j];

            int32_t e, em;
            if (eu + OR_GAP_EXTEND >= hu + OR_GAP_OPEN) { e = eu + OR_GAP_EXTEND; em = emu; }
            else { e = hu + OR_GAP_OPEN; em = hmu; }

            int32_t fx = (j > js) ? f + OR_GAP_EXTEND : OR_NEG_INF;
            if (fx >= hl + OR_GAP_OPEN) { f = fx; /* fm unchanged */ }
            else { f = hl + OR_GAP_OPEN; fm = hml; }

            int32_t h = 0, hm = 0;
            if (diag > h) { h = diag; hm = diag_m; }
            if (e > h) { h = e; hm = em; }
            if (f > h) { h = f; hm = fm; }

            if (h > best_score) { best_score = h; best_matches = hm; }

            H[j] = h; Hm[j] = hm; E[j] = e; Em[j] = em;
            hd = hu; hmd = hmu;
            hl = h; hml = hm;
        }
        /* the cell right of row i's band reads as the out-of-band boundary */
        if (je + 1 <= lb) {
            H[je + 1] = 0; Hm[je + 1] = 0; E[je + 1] = OR_NEG_INF; Em[je + 1] = 0;
        }
    }
    *score_out = best_score;
    *matches_out = best_matches;
}

/*
 * clustkit/csrc/sw_align.c:182-266 (batch_sw_align_c) with the raw integer
 * outputs exposed: out_matches is the identity numerator, out_shorter the
 * denominator.  out_sims = matches/shorter in float32 when score > 0, else 0.
 * out_mask = score > 0 (sw_align.c:260).  Any output pointer may be NULL.
 */
void or_sw_batch(const int32_t *pairs, const uint8_t *flat, const int64_t *offsets,
                 const int32_t *lengths, int64_t M, int32_t band_width,
                 const int8_t *sub, const int32_t *diag_hints,
                 float *out_sims, int32_t *out_scores, int32_t *out_matches,
                 int32_t *out_shorter, uint8_t *out_mask) {
    int32_t max_len = 0;
    for (int64_t p = 0; p < M; p++) {
        int32_t li = lengths[pairs[2 * p]], lj = lengths[pairs[2 * p + 1]];
        int32_t ml = li > lj ? li : lj;
        if (ml > max_len) max_len = ml;
    }
    const int64_t cols = (int64_t)max_len + 2;

#pragma omp parallel
    {
        int32_t *ws = (int32_t *)malloc(sizeof(int32_t) * 4 * cols);
        int32_t *H = ws, *E = ws + cols, *Hm = ws + 2 * cols, *Em = ws + 3 * cols;
#pragma omp for schedule(dynamic, 64)
        for (int64_t p = 0; p < M; p++) {
            int32_t ii = pairs[2 * p], jj = pairs[2 * p + 1];
            int32_t li = lengths[ii], lj = lengths[jj];
            int32_t shorter = li < lj ? li : lj;
            int32_t score = 0, matches = 0;
            if (li != 0 && lj != 0) {
                int32_t hint = diag_hints ? diag_hints[p] : 0;
                if (hint > shorter || hint < -shorter) hint = 0;  /* sw_align.c:240-242 */
                const uint8_t *si = flat + offsets[ii], *sj = flat + offsets[jj];
                if (li <= lj)
                    or_sw_one(si, li, sj, lj, band_width, hint, sub, H, E, Hm, Em, &score, &matches);
                else
                    or_sw_one(sj, lj, si, li, band_width, -hint, sub, H, E, Hm, Em, &score, &matches);
            }
            if (out_scores) out_scores[p] = score;
            if (out_matches) out_matches[p] = matches;
            if (out_shorter) out_shorter[p] = shorter;
            if (out_sims) out_sims[p] = score > 0 ? (float)matches / (float)shorter : 0.0f;
            if (out_mask) out_mask[p] = score > 0 ? 1 : 0;
        }
        free(ws);
    }
}

/* clustkit/sketch.py:17-26 */
static inline uint64_t or_fmix64(uint64_t key, uint64_t seed) {
    uint64_t h = key ^ seed;
    h ^= h >> 33;
    h *= 0xFF51AFD7ED558CCDULL;
    h ^= h >> 33;
    h *= 0xC4CEB9FE1A85EC53ULL;
    h ^= h >> 33;
    return h;
}

uint64_t or_fmix64_export(uint64_t key, uint64_t seed) { return or_fmix64(key, seed); }

static void heap_sift_down(uint64_t *hp, int32_t n, int32_t i) {
    for (;;) {
        int32_t l = 2 * i + 1, r = l + 1, m = i;
        if (l < n && hp[l] > hp[m]) m = l;
        if (r < n && hp[r] > hp[m]) m = r;
        if (m == i) return;
        uint64_t t = hp[i]; hp[i] = hp[m]; hp[m] = t;
        i = m;
    }
}

static int cmp_u64(const void *x, const void *y) {
    uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
    return (a > b) - (a < b);
}

/*
 * Bottom-s MinHash sketch of every sequence.  clustkit/sketch.py:29-80:
 * len < k gives s zeros; otherwise the k-mer value is the base-`alphabet`
 * number of the k codes (uint64 arithmetic, codes used as they are), hashed
 * by fmix64(value ^ seed); the sketch is the sorted multiset of the s
 * smallest hashes, padded with UINT64_MAX.
 */
void or_sketch(const uint8_t *flat, const int64_t *offsets, const int32_t *lengths,
               int64_t N, int32_t k, int32_t s, int32_t alphabet, uint64_t seed,
               uint64_t *out) {
#pragma omp parallel
    {
        uint64_t *heap = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(s > 0 ? s : 1));
#pragma omp for schedule(dynamic, 16)
        for (int64_t q = 0; q < N; q++) {
            uint64_t *o = out + q * (int64_t)s;
            int32_t len = lengths[q];
            if (len < k) {
                for (int32_t t = 0; t < s; t++) o[t] = 0ULL;
                continue;
            }
            const uint8_t *seq = flat + offsets[q];
            int32_t nk = len - k + 1, n = 0;
            for (int32_t i = 0; i < nk; i++) {
                uint64_t v = 0;
                for (int32_t m = 0; m < k; m++) v = v * (uint64_t)alphabet + (uint64_t)seq[i + m];
                uint64_t h = or_fmix64(v, seed);
                if (n < s) {
                    /* sift up */
                    int32_t c = n++;
                    heap[c] = h;
                    while (c > 0) {
                        int32_t p = (c - 1) / 2;
                        if (heap[p] >= heap[c]) break;
                        uint64_t t = heap[p]; heap[p] = heap[c]; heap[c] = t;
                        c = p;
                    }
                } else if (s > 0 && h < heap[0]) {
                    heap[0] = h;
                    heap_sift_down(heap, n, 0);
                }
            }
            qsort(heap, (size_t)n, sizeof(uint64_t), cmp_u64);
            for (int32_t t = 0; t < s; t++) o[t] = t < n ? heap[t] : UINT64_MAX;
        }
        free(heap);
    }
}

/*
 * Merge-walk Jaccard of two sorted sketches, clustkit/pairwise.py:1564-1595:
 * at most s steps; stop when both heads are UINT64_MAX; equal heads count as
 * shared and advance both.  J = shared / steps in float32 (0 when no step).
 */
static float or_jaccard_one(const uint64_t *A, const uint64_t *B, int32_t s) {
    int32_t i = 0, j = 0, shared = 0, uni = 0;
    while (uni < s && i < s && j < s) {
        uint64_t a = A[i], b = B[j];
        if (a == UINT64_MAX && b == UINT64_MAX) break;
        if (a == b) { shared++; i++; j++; }
        else if (a < b) i++;
        else j++;
        uni++;
    }
    if (uni == 0) return 0.0f;
    return (float)((double)shared / (double)uni);
}

/* clustkit/pairwise.py:1598-1612 (_batch_jaccard) */
void or_jaccard(const int32_t *pairs, const uint64_t *sketches, int64_t M, int32_t s,
                float *out_sims) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < M; p++) {
        const uint64_t *A = sketches + (int64_t)pairs[2 * p] * s;
        const uint64_t *B = sketches + (int64_t)pairs[2 * p + 1] * s;
        out_sims[p] = or_jaccard_one(A, B, s);
    }
}
