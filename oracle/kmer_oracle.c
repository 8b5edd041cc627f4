/*
 * kmer_oracle.c -- CPU restatement of clustkit's C k-mer scorer.
 *
 * TEST INFRASTRUCTURE ONLY: linked into liboracle.so beside oracle.c, used by
 * tests/ and by bench.py's CPU baseline of the search path; nothing in the
 * product library links it.
 *
 *   or_kmer_candidates   clustkit/csrc/kmer_score.c:195-470
 *                        (score_query_full, batch_score_queries_c)
 *   or_similar_candidates clustkit/kmer_index.py:1187-1328
 *                        (_score_query_similar_k5: BLOSUM62 similar 5-mers)
 *
 * Per query: Phase A counts the hits of every valid k-mer (all codes below
 * alpha) whose frequency is at most freq_thresh, per database sequence,
 * saturating at 32767; survivors have at least min_total_hits.  With
 * min_diag_hits <= 1 the survivors are the candidates.  Otherwise the top
 * phase_a_topk survivors by (hits desc, id asc) are rescored by their hits'
 * diagonal bins (tpos - qpos + qlen) / diag_bin_width: each keeps its longest
 * bin, the first on ties, and is kept when that run reaches min_diag_hits,
 * with the hint bin * width - qlen + width / 2 (zero hints in the other mode).
 * Candidates are written in id order when at most max_cands, else the best
 * max_cands by (score desc, id asc) in that order.  The hits of the selected
 * targets are gathered as (target, bin) keys, sorted and run-length counted.
 * OpenMP over queries, per-thread dense count rows.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

static int cmp_i32(const void *x, const void *y) {
    const int32_t a = *(const int32_t *)x, b = *(const int32_t *)y;
    return (a > b) - (a < b);
}

static int cmp_u64k(const void *x, const void *y) {
    const uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
    return (a > b) - (a < b);
}

/* Order ids[0..n) (with their scores) so that the first k are the best by
 * (score desc, id asc) in that order; returns min(n, k).  When n <= k the
 * given order stays. */
static int32_t top_by_score(int32_t *ids, int32_t *sc, int32_t *aux_d, int32_t n, int32_t k, uint64_t *tmp) {
    if (n <= k) return n;
    if (k <= 0) return 0;
    for (int32_t i = 0; i < n; ++i)
        tmp[i] = ((uint64_t)(uint32_t)(0x7fffffff - sc[i]) << 32) | (uint32_t)i;
    qsort(tmp, (size_t)n, 8, cmp_u64k);
    /* gather through the original positions (ties: ids ascending, as the
     * positions are in id order) */
    int32_t *oi = (int32_t *)malloc((size_t)k * 4), *os = (int32_t *)malloc((size_t)k * 4);
    int32_t *od = aux_d ? (int32_t *)malloc((size_t)k * 4) : NULL;
    for (int32_t j = 0; j < k; ++j) {
        const int32_t p = (int32_t)(tmp[j] & 0xffffffffu);
        oi[j] = ids[p];
        os[j] = sc[p];
        if (od) od[j] = aux_d[p];
    }
    memcpy(ids, oi, (size_t)k * 4);
    memcpy(sc, os, (size_t)k * 4);
    if (od) memcpy(aux_d, od, (size_t)k * 4);
    free(oi);
    free(os);
    free(od);
    return k;
}

void or_kmer_candidates(const uint8_t *q_flat, const int64_t *q_offsets, const int32_t *q_lengths, int32_t nq,
                        int32_t k, int32_t alpha, const int64_t *kmer_offsets, const int64_t *kmer_entries,
                        const int32_t *kmer_freqs, int32_t freq_thresh, int32_t num_db, int32_t min_total_hits,
                        int32_t min_diag_hits, int32_t diag_bin_width, int32_t max_cands, int32_t phase_a_topk,
                        int32_t *out_targets, int32_t *out_scores, int32_t *out_diags, int32_t *out_n) {
#pragma omp parallel
    {
        int32_t *counts = (int32_t *)calloc((size_t)num_db + 1, 4);
        int32_t *touched = (int32_t *)malloc(((size_t)num_db + 1) * 4);
        uint8_t *mark = (uint8_t *)calloc((size_t)num_db + 1, 1);
        int32_t *ids = (int32_t *)malloc(((size_t)num_db + 1) * 4);
        int32_t *sc = (int32_t *)malloc(((size_t)num_db + 1) * 4);
        int32_t *dg = (int32_t *)malloc(((size_t)num_db + 1) * 4);
        uint64_t *tmp = (uint64_t *)malloc(((size_t)num_db + 1) * 8);
        size_t hcap = 1 << 16;
        uint64_t *hits = (uint64_t *)malloc(hcap * 8);
#pragma omp for schedule(dynamic, 1)
        for (int32_t qi = 0; qi < nq; ++qi) {
            const uint8_t *s = q_flat + q_offsets[qi];
            const int32_t L = q_lengths[qi];
            int32_t nt = 0;
            for (int32_t p = 0; p + k <= L; ++p) {
                uint32_t v = 0;
                int ok = 1;
                for (int32_t m = 0; m < k; ++m) {
                    ok &= s[p + m] < alpha;
                    v = v * (uint32_t)alpha + s[p + m];
                }
                if (!ok || kmer_freqs[v] > freq_thresh) continue;
                for (int64_t h = kmer_offsets[v]; h < kmer_offsets[v + 1]; ++h) {
                    const int32_t t = (int32_t)(kmer_entries[h] >> 32);
                    if (counts[t] == 0) touched[nt++] = t;
                    if (counts[t] < 32767) counts[t]++;
                }
            }
            int32_t n = 0;
            if (min_total_hits <= 0) {
                for (int32_t t = 0; t < num_db; ++t) { ids[n] = t; sc[n] = counts[t]; ++n; }
            } else {
                qsort(touched, (size_t)nt, 4, cmp_i32);
                for (int32_t i = 0; i < nt; ++i)
                    if (counts[touched[i]] >= min_total_hits) { ids[n] = touched[i]; sc[n] = counts[touched[i]]; ++n; }
            }
            for (int32_t i = 0; i < nt; ++i) counts[touched[i]] = 0;
            if (min_diag_hits <= 1) {
                n = top_by_score(ids, sc, NULL, n, max_cands, tmp);
                for (int32_t j = 0; j < n; ++j) dg[j] = 0;
            } else {
                const int32_t ns = top_by_score(ids, sc, NULL, n, phase_a_topk, tmp);
                for (int32_t j = 0; j < ns; ++j) mark[ids[j]] = 1;
                size_t nh = 0;
                for (int32_t p = 0; p + k <= L; ++p) {
                    uint32_t v = 0;
                    int ok = 1;
                    for (int32_t m = 0; m < k; ++m) {
                        ok &= s[p + m] < alpha;
                        v = v * (uint32_t)alpha + s[p + m];
                    }
                    if (!ok || kmer_freqs[v] > freq_thresh) continue;
                    for (int64_t h = kmer_offsets[v]; h < kmer_offsets[v + 1]; ++h) {
                        const int64_t e = kmer_entries[h];
                        const int32_t t = (int32_t)(e >> 32);
                        if (!mark[t]) continue;
                        const int64_t bin = ((int64_t)(int32_t)(e & 0xffffffff) - p + L) / diag_bin_width;
                        if (nh == hcap) {
                            hcap *= 2;
                            hits = (uint64_t *)realloc(hits, hcap * 8);
                        }
                        hits[nh++] = ((uint64_t)(uint32_t)t << 32) | (uint32_t)bin;
                    }
                }
                for (int32_t j = 0; j < ns; ++j) mark[ids[j]] = 0;
                qsort(hits, nh, 8, cmp_u64k);
                n = 0;
                for (size_t i = 0; i < nh;) {
                    const uint32_t t = (uint32_t)(hits[i] >> 32);
                    int32_t best = 0, best_bin = 0;
                    size_t j = i;
                    while (j < nh && (uint32_t)(hits[j] >> 32) == t) {
                        const uint64_t key = hits[j];
                        size_t r = j;
                        while (r < nh && hits[r] == key) ++r;
                        if ((int32_t)(r - j) > best) { best = (int32_t)(r - j); best_bin = (int32_t)(key & 0xffffffffu); }
                        j = r;
                    }
                    if (best >= min_diag_hits) {
                        ids[n] = (int32_t)t;
                        sc[n] = best;
                        dg[n] = best_bin * diag_bin_width - L + diag_bin_width / 2;
                        ++n;
                    }
                    i = j;
                }
                n = top_by_score(ids, sc, dg, n, max_cands, tmp);
            }
            out_n[qi] = n;
            if (n > 0) {
                memcpy(out_targets + (int64_t)qi * max_cands, ids, (size_t)n * 4);
                memcpy(out_scores + (int64_t)qi * max_cands, sc, (size_t)n * 4);
                if (out_diags) memcpy(out_diags + (int64_t)qi * max_cands, dg, (size_t)n * 4);
            }
        }
        free(counts);
        free(touched);
        free(mark);
        free(ids);
        free(sc);
        free(dg);
        free(tmp);
        free(hits);
    }
}

/* clustkit's similar-k-mer scoring (k = 5, alphabet 20): for every query
 * 5-mer of codes below 20, every 5-mer whose column-sum score under sub
 * (int8 [20][20], row = query residue) reaches T, and whose frequency is in
 * (0, freq_thresh], adds that score to each target of its posting list.
 * The neighbours are enumerated by branch and bound on the best remaining
 * row scores (the same set as a full scan).  Survivors have a sum of at
 * least min_total_hits (every target when it is <= 0); written in id order
 * when at most max_cands, else the best max_cands by (score desc, id asc) in
 * that order.  T >= 1 (as clustkit's threshold), so a touched target's sum
 * is positive.  Sums in int64 (written as int32).  OpenMP over queries. */
void or_similar_candidates(const uint8_t *q_flat, const int64_t *q_offsets, const int32_t *q_lengths, int32_t nq,
                           const int8_t *sub, int32_t T, const int64_t *kmer_offsets, const int64_t *kmer_entries,
                           const int32_t *kmer_freqs, int32_t freq_thresh, int32_t num_db, int32_t min_total_hits,
                           int32_t max_cands, int32_t *out_targets, int32_t *out_scores, int32_t *out_n) {
    int32_t S[400], mx[20];
    for (int i = 0; i < 400; ++i) S[i] = sub[i];
    for (int a = 0; a < 20; ++a) {
        int32_t m = S[a * 20];
        for (int b = 1; b < 20; ++b) m = S[a * 20 + b] > m ? S[a * 20 + b] : m;
        mx[a] = m;
    }
#pragma omp parallel
    {
        int64_t *counts = (int64_t *)calloc((size_t)num_db + 1, 8);
        int32_t *touched = (int32_t *)malloc(((size_t)num_db + 1) * 4);
        int32_t *ids = (int32_t *)malloc(((size_t)num_db + 1) * 4);
        int32_t *sc = (int32_t *)malloc(((size_t)num_db + 1) * 4);
        uint64_t *tmp = (uint64_t *)malloc(((size_t)num_db + 1) * 8);
#pragma omp for schedule(dynamic, 1)
        for (int32_t qi = 0; qi < nq; ++qi) {
            const uint8_t *s = q_flat + q_offsets[qi];
            const int32_t L = q_lengths[qi];
            int32_t nt = 0;
            for (int32_t p = 0; p + 5 <= L; ++p) {
                const int32_t q0 = s[p], q1 = s[p + 1], q2 = s[p + 2], q3 = s[p + 3], q4 = s[p + 4];
                if (q0 >= 20 || q1 >= 20 || q2 >= 20 || q3 >= 20 || q4 >= 20) continue;
                const int32_t m4 = mx[q4], m34 = mx[q3] + m4, m234 = mx[q2] + m34, m1234 = mx[q1] + m234;
                for (int32_t a0 = 0; a0 < 20; ++a0) {
                    const int32_t s0 = S[q0 * 20 + a0];
                    if (s0 + m1234 < T) continue;
                    for (int32_t a1 = 0; a1 < 20; ++a1) {
                        const int32_t s1 = s0 + S[q1 * 20 + a1];
                        if (s1 + m234 < T) continue;
                        for (int32_t a2 = 0; a2 < 20; ++a2) {
                            const int32_t s2 = s1 + S[q2 * 20 + a2];
                            if (s2 + m34 < T) continue;
                            for (int32_t a3 = 0; a3 < 20; ++a3) {
                                const int32_t s3 = s2 + S[q3 * 20 + a3];
                                if (s3 + m4 < T) continue;
                                for (int32_t a4 = 0; a4 < 20; ++a4) {
                                    const int32_t s4 = s3 + S[q4 * 20 + a4];
                                    if (s4 < T) continue;
                                    const int32_t v = (((a0 * 20 + a1) * 20 + a2) * 20 + a3) * 20 + a4;
                                    const int32_t f = kmer_freqs[v];
                                    if (f == 0 || f > freq_thresh) continue;
                                    for (int64_t h = kmer_offsets[v]; h < kmer_offsets[v + 1]; ++h) {
                                        const int32_t t = (int32_t)(kmer_entries[h] >> 32);
                                        if (counts[t] == 0) touched[nt++] = t;
                                        counts[t] += s4;
                                    }
                                }
                            }
                        }
                    }
                }
            }
            int32_t n = 0;
            if (min_total_hits <= 0) {
                for (int32_t t = 0; t < num_db; ++t) { ids[n] = t; sc[n] = (int32_t)counts[t]; ++n; }
            } else {
                qsort(touched, (size_t)nt, 4, cmp_i32);
                for (int32_t i = 0; i < nt; ++i)
                    if (counts[touched[i]] >= min_total_hits) {
                        ids[n] = touched[i];
                        sc[n] = (int32_t)counts[touched[i]];
                        ++n;
                    }
            }
            for (int32_t i = 0; i < nt; ++i) counts[touched[i]] = 0;
            n = top_by_score(ids, sc, NULL, n, max_cands, tmp);
            out_n[qi] = n;
            if (n > 0) {
                memcpy(out_targets + (int64_t)qi * max_cands, ids, (size_t)n * 4);
                memcpy(out_scores + (int64_t)qi * max_cands, sc, (size_t)n * 4);
            }
        }
        free(counts);
        free(touched);
        free(ids);
        free(sc);
        free(tmp);
    }
}
