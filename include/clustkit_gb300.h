/*
 * clustkit_gb300.h -- C ABI of libckgpu.so, the GB300 (sm_103a) engine for
 * clustkit's Align phase (banded SW, sketches, Jaccard pre-filter) and the
 * steps either side of it: LSH candidates, the k-mer search path (index,
 * Phase A / similar k-mers / Phase B, hinted SW) and the similarity graph
 * with its connected components.
 *
 * Conventions
 *   - Every ck_* entry point returns an int status (CK_OK on success) and
 *     never aborts; ck_last_error() returns a message for the calling thread.
 *   - Host-buffer entry points copy inputs to the GPU, run, copy outputs back
 *     and return after the results are in the caller's buffers.
 *   - *_device entry points take device pointers and a cudaStream_t (passed as
 *     void*, NULL = the legacy default stream) and return once the work is
 *     enqueued; results are ready when that stream is synchronised.  Input
 *     errors found on the GPU are reported through ck_sw_status_device() (or
 *     ck_ctx_status() for a library context).  The ones that must size a
 *     buffer from a device-side count first say "Blocking" and synchronise
 *     their stream.
 *   - Pair lists are int32 [M][2]; sequences use clustkit's compact layout
 *     (clustkit/io.py:35-131): uint8 codes `flat`, int64 `offsets[N]`,
 *     int32 `lengths[N]`.  Protein codes are 0..19, unknown residues 20.
 *   - Reference paths are relative to the clustkit project root.
 */
#ifndef CLUSTKIT_GB300_H
#define CLUSTKIT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define CK_OK                    0
#define CK_ERR_INVALID_ARGUMENT  1  /* NULL pointer, negative size, bad enum value   */
#define CK_ERR_OUT_OF_RANGE      2  /* pair index, offset or length outside the inputs */
#define CK_ERR_CUDA              3  /* CUDA runtime failure (message in ck_last_error) */
#define CK_ERR_OUT_OF_MEMORY     4
#define CK_ERR_UNSUPPORTED       5  /* parameter outside what the kernels implement   */
#define CK_ERR_NO_DEVICE         6
#define CK_ERR_CAPACITY          7  /* a caller-bounded device buffer (Phase-B bins,
                                       neighbour list) was too small: the call's
                                       results are incomplete; run it again with
                                       a larger bound (reported at the next
                                       status check of the context)            */

/* --------------------------------------------------- pass / fail rules
 * clustkit decides pass/fail differently on each of its three SW paths; the
 * rule is chosen per call so every one of them can be reproduced exactly.
 * identity = (float)matches / (float)shorter, 0 when score <= 0.            */
#define CK_PASS_CPU    0  /* identity >= t           (clustkit/pairwise.py:107, C path)     */
#define CK_PASS_NUMBA  1  /* score > 0 && identity>=t (clustkit/pairwise.py:679 and :1182)  */
#define CK_PASS_CUPY   2  /* shorter/longer >= t (else not aligned) && identity >= t
                             (clustkit/pairwise.py:1246-1252, :1393-1400)                   */
#define CK_PASS_SCORE  3  /* score > 0                (clustkit/csrc/sw_align.c:260)        */

/* --------------------------------------------------------- SW engines */
#define CK_SW_BATCHED  0  /* length-binned persistent strip kernel + work queue (default);
                             pairs it cannot take run on the plain kernel                  */
#define CK_SW_PLAIN    1  /* one unbinned launch per chunk, one thread per pair             */

int32_t ck_version(void);
const char *ck_last_error(void);
/* status of the last call made through the clustkit-compatible entry points
 * below (they return void, as clustkit's own C functions do) */
int32_t ck_last_status(void);
int32_t ck_device_count(void);

/* ------------------------------------------------ clustkit-compatible ABI
 * Same symbol names, argument lists and output meaning as clustkit's C
 * extension, so clustkit's ctypes loader (clustkit/pairwise.py:41-66) can
 * bind this library in place of csrc/sw_align.so unchanged.
 *
 * batch_sw_align_c: replaces clustkit/csrc/sw_align.c:182-195.  Host buffers.
 *   out_sims = identity, out_scores = best local score, out_mask = score > 0.
 *   The GPU path is always used; on failure the outputs are zeroed and
 *   ck_last_status()/ck_last_error() describe the error.
 * sw_set_num_threads: replaces clustkit/csrc/sw_align.c:19-21.  Accepted and
 *   ignored (the work runs on the GPU).                                      */
void batch_sw_align_c(const int32_t *pairs, const uint8_t *flat_sequences,
                      const int64_t *offsets, const int32_t *lengths, int32_t M,
                      int32_t band_width, const int8_t *sub_matrix, float threshold,
                      const int32_t *diag_hints, float *out_sims, int32_t *out_scores,
                      uint8_t *out_mask);
void sw_set_num_threads(int32_t n);

/* ------------------------------------------------------------- SW batch
 * ck_sw_batch: banded Smith-Waterman over a candidate-pair list
 * (clustkit/csrc/sw_align.c:25-266, same recurrence, tie rules and band as
 * clustkit).  Host buffers.
 *   n_seqs, flat_len  sizes of lengths/offsets and flat (bounds are checked)
 *   band_width        half-width; <= 0, or a longer side <= 50, means full matrix
 *   sub_matrix        20x20 int8, row = residue of the shorter sequence
 *   diag_hints        NULL, or per-pair band-centre offsets (sw_align.c:237-256)
 *   pass_rule         CK_PASS_*; engine CK_SW_*
 *   outputs           any may be NULL: out_sims (float identity), out_scores,
 *                     out_matches (identity numerator), out_shorter
 *                     (denominator), out_mask (uint8 pass/fail under pass_rule) */
int32_t ck_sw_batch(const int32_t *pairs, int64_t M, const uint8_t *flat, int64_t flat_len,
                    const int64_t *offsets, const int32_t *lengths, int64_t n_seqs,
                    int32_t band_width, const int8_t *sub_matrix, float threshold,
                    const int32_t *diag_hints, int32_t pass_rule, int32_t engine,
                    float *out_sims, int32_t *out_scores, int32_t *out_matches,
                    int32_t *out_shorter, uint8_t *out_mask);

/* Device-pointer form of ck_sw_batch.  Scratch memory is managed by the
 * library per device.  Errors detected on the GPU (pair index or sequence
 * extent out of range) are latched in a per-device flag read by
 * ck_sw_status_device(). */
int32_t ck_sw_batch_device(const int32_t *d_pairs, int64_t M, const uint8_t *d_flat,
                           int64_t flat_len, const int64_t *d_offsets,
                           const int32_t *d_lengths, int64_t n_seqs, int32_t band_width,
                           const int8_t *sub_matrix_host, float threshold,
                           const int32_t *d_diag_hints, int32_t pass_rule, int32_t engine,
                           float *d_sims, int32_t *d_scores, int32_t *d_matches,
                           int32_t *d_shorter, uint8_t *d_mask, void *stream);
/* Allocation-free form of ck_sw_batch_device.  No counterpart in clustkit:
 * it is for callers that cannot let a library allocate GPU memory -- a host
 * system that owns the device's memory through its own pre-sized pool, or a
 * latency-bound serving loop where an allocation could stall or fail
 * mid-request.  It calls no cudaMalloc/cudaFree and no allocating library
 * routine: the caller passes device buffers for inputs and outputs, and the
 * kernel's workspace is a 32 MiB static device array inside this library,
 * held on every GPU that loads it until the process exits.
 *   - Runs the plain kernel (one thread per pair); results equal
 *     ck_sw_batch_device's.
 *   - band_width must be 1..8191 (the workspace per thread grows with the
 *     band); larger, or <= 0 (full matrix), returns CK_ERR_UNSUPPORTED.
 *   - Blocking: enqueues on `stream`, waits for it, and returns
 *     CK_ERR_OUT_OF_RANGE if a pair index or sequence extent was bad.
 *   - The first call on a device looks up the static arrays' device
 *     addresses; make that first call before any stream capture.  Not for
 *     use on a device after cudaDeviceReset in the same process.
 *   - Every call on a device shares that device's static arrays (which keep
 *     the last call's contents).  Calls on one device are serialised by a
 *     lock held until the kernel has finished, so calls from several threads
 *     or streams of this process never overlap on them; calls on different
 *     devices do not wait for each other. */
int32_t ck_sw_batch_device_noalloc(const int32_t *d_pairs, int64_t M, const uint8_t *d_flat,
                                   int64_t flat_len, const int64_t *d_offsets,
                                   const int32_t *d_lengths, int64_t n_seqs, int32_t band_width,
                                   const int8_t *sub_matrix_host, float threshold,
                                   const int32_t *d_diag_hints, int32_t pass_rule, float *d_sims,
                                   int32_t *d_scores, int32_t *d_matches, int32_t *d_shorter,
                                   uint8_t *d_mask, void *stream);

/* Synchronises `stream`, returns CK_OK, CK_ERR_OUT_OF_RANGE or
 * CK_ERR_CAPACITY for the GPU checks of the ck_*_device calls since the
 * previous ck_sw_status_device on this device, and clears the flag. */
int32_t ck_sw_status_device(void *stream);

/* Work counters of the last ck_sw_batch / ck_sw_batch_device call on this
 * thread: out[0] pairs, out[1] DP cells (the band cells clustkit computes),
 * out[2] pairs taken by the batched kernel, out[3] pairs run on the plain
 * kernel, out[4] pairs re-run after a score overflowed the packed lane,
 * out[5] kernel launches issued. */
int32_t ck_sw_last_counters(int64_t *out6);
/* Of the batched pairs of the same call, how many ran one warp per pair
 * (long pairs, or every pair of a small call; see CK_CFG_WAVE_*). */
int32_t ck_sw_last_wave_pairs(int64_t *out);

/* Kernel timing for measurement: after ck_sw_profile(1), every SW call
 * records CUDA events on its stream around its dominant kernel (the strip
 * kernel for CK_SW_BATCHED, the plain kernel for CK_SW_PLAIN);
 * ck_sw_last_kernel_ms waits for the last one and returns its duration in
 * milliseconds (-1 if none was recorded). */
int32_t ck_sw_profile(int32_t enable);
int32_t ck_sw_last_kernel_ms(float *out_ms);

/* Tunables of the batched engine, process-wide (the autotuner in
 * clustkit_gb300/tune.py picks them per workload):
 *   CK_CFG_ROWS_PER_STRIP  rows a lane keeps in registers per strip: 8, 16, 24,
 *                          32, or 0 (default) for 8 when the band half-width
 *                          is <= 64, else 16
 *   CK_CFG_STRIP_VARIANT   0..3: bit 1 runs interior columns in groups of
 *                          four (else two), with one first-maximum vote per
 *                          group; bit 0 aligns the groups, addresses each
 *                          group's window slots and residues from one base
 *                          pointer per run and prefetches four columns ahead
 *                          (else each column its own addresses, two ahead);
 *                          -1 (default): 3 for strips of 8 rows, else 1
 *   CK_CFG_WAVE_ALL_BELOW  calls with at most this many pairs to align (the
 *                          count is taken on the device, after empty and
 *                          skipped pairs) run every pair one warp per pair
 *                          (default 40960)
 *   CK_CFG_WAVE_MIN_ROWS   in larger calls with band_width > 0, pairs with at
 *                          least this many rows (shorter side) run one warp
 *                          per pair instead of one lane per pair (default 512)
 *   CK_CFG_WAVE_ADAPTIVE   1 (default): raise that row bound to where a pair's
 *                          one-lane time would pass the call's expected
 *                          kernel time, from the call's cell count; 0:
 *                          use CK_CFG_WAVE_MIN_ROWS as given
 *   CK_CFG_WAVE_STREAM     1 (default): when a call has more warp-per-pair
 *                          pairs than the kernel has warps, a warp streams the
 *                          row strips of consecutive pairs through its lanes;
 *                          2: always; 0: never (one pair per warp at a time)
 *   CK_CFG_WAVE_ROWS       rows per strip of that streamed schedule: 0
 *                          (default) the smallest of 4/8/16 whose strips can
 *                          rotate through the lanes at the call's band width;
 *                          4, 8 or 16: at least that many
 *                          (key 7, a cluster-shared-memory form of the
 *                          similar-k-mer posting walk, is retired: it
 *                          measured 2.6x slower than the L2-atomic walk)
 *   CK_CFG_STRIP_THREADS   threads of the strip kernel's one persistent CTA
 *                          per SM for strips of 8 rows: 512 (16 warps, up to
 *                          128 registers), 640 (20 warps, 96) or 768 (24, 80);
 *                          0 (default): 640.  Strips of 16 rows always run
 *                          512 threads, of 24 or 32 rows 256.  With the
 *                          default rows per strip, a call whose pairs all run
 *                          one warp per pair runs the 8-row kernel.  (Key 8,
 *                          CTAs of 256 threads per SM, is retired: one CTA of
 *                          512 threads measured at least as fast in every case.)
 *   CK_CFG_STRIP_KEY       0 (default): the strip kernel packs pairs of at
 *                          most 2047 rows in the compact key (11-bit match
 *                          count, a gap-extension counter in place of a tie
 *                          bit: fewer logic ops a cell), longer ones in the
 *                          wide key (13-bit match count); 1: the wide key for
 *                          every pair.  Results are the same either way. */
#define CK_CFG_ROWS_PER_STRIP 0
#define CK_CFG_STRIP_VARIANT 1
#define CK_CFG_WAVE_MIN_ROWS 2
#define CK_CFG_WAVE_ALL_BELOW 3
#define CK_CFG_WAVE_ADAPTIVE 4
#define CK_CFG_WAVE_STREAM 5
#define CK_CFG_WAVE_ROWS 6
#define CK_CFG_STRIP_KEY 9
#define CK_CFG_STRIP_THREADS 10
int32_t ck_sw_set_config(int32_t key, int32_t value);
int32_t ck_sw_get_config(int32_t key, int32_t *value);

/* ------------------------------------------------------------- sketches
 * Bottom-s MinHash sketches (clustkit/sketch.py:17-183): k-mer value in base
 * `alphabet` (20 protein, 4 nucleotide), hash fmix64(value ^ seed), the s
 * smallest hashes sorted, UINT64_MAX padding, s zeros when length < k.
 * out is uint64 [N][s].  1 <= k <= 32, 1 <= s <= 4096. */
int32_t ck_sketch(const uint8_t *flat, int64_t flat_len, const int64_t *offsets,
                  const int32_t *lengths, int64_t N, int32_t k, int32_t s,
                  int32_t alphabet, uint64_t seed, uint64_t *out);
int32_t ck_sketch_device(const uint8_t *d_flat, int64_t flat_len, const int64_t *d_offsets,
                         const int32_t *d_lengths, int64_t N, int32_t k, int32_t s,
                         int32_t alphabet, uint64_t seed, uint64_t *d_out, void *stream);

/* -------------------------------------------------------------- Jaccard
 * Merge-walk Jaccard of sorted sketches (clustkit/pairwise.py:1564-1612) and
 * the pre-filter mask sims >= floor (clustkit/pairwise.py:949-1001, float32
 * comparison).  sketches uint64 [N][s]; out_sims float [M]; out_mask uint8
 * [M] (may be NULL). */
int32_t ck_jaccard(const int32_t *pairs, int64_t M, const uint64_t *sketches, int64_t N,
                   int32_t s, float floor, float *out_sims, uint8_t *out_mask);
int32_t ck_jaccard_device(const int32_t *d_pairs, int64_t M, const uint64_t *d_sketches,
                          int64_t N, int32_t s, float floor, float *d_sims,
                          uint8_t *d_mask, void *stream);

/* ------------------------------------------------------------ contexts
 * A context owns its own scratch buffers and error word, so that calls
 * enqueued on different streams (e.g. overlapping search batches) never share
 * scratch.  Handles are small positive integers; 0 names the device's default
 * scratch used by the entry points without a context argument.  A context is
 * bound to the device current at creation. */
int32_t ck_ctx_create(int32_t *out_handle);
int32_t ck_ctx_destroy(int32_t handle);
/* Freeze (1) or thaw (0) a context's scratch: while frozen, a call that would
 * need to grow a scratch buffer fails with CK_ERR_UNSUPPORTED instead of
 * reallocating it, so the buffers stay valid inside CUDA graphs captured from
 * calls on this context (size them with one uncaptured call of the largest
 * shape first). */
int32_t ck_ctx_freeze(int32_t handle, int32_t frozen);
/* Synchronises `stream` and returns CK_OK, CK_ERR_OUT_OF_RANGE (GPU-side
 * input checks) or CK_ERR_CAPACITY (a caller-bounded buffer too small) for
 * the context's calls since its last status read. */
int32_t ck_ctx_status(int32_t handle, void *stream);
/* ck_sw_batch_device with the scratch of context `ctx`. */
int32_t ck_sw_batch_device_ctx(int32_t ctx, const int32_t *d_pairs, int64_t M, const uint8_t *d_flat,
                               int64_t flat_len, const int64_t *d_offsets,
                               const int32_t *d_lengths, int64_t n_seqs, int32_t band_width,
                               const int8_t *sub_matrix_host, float threshold,
                               const int32_t *d_diag_hints, int32_t pass_rule, int32_t engine,
                               float *d_sims, int32_t *d_scores, int32_t *d_matches,
                               int32_t *d_shorter, uint8_t *d_mask, void *stream);

/* Resident database and asynchronous submit/poll on a context, for hosts
 * that drive batches without a Python runtime.  Replaces, for such hosts,
 * clustkit's synchronous ctypes call into batch_sw_align_c
 * (clustkit/pairwise.py:50-58, :69-108 -> csrc/sw_align.c:182-266): the
 * sequences go to the device once, then each batch is only its pairs.
 *
 * ck_ctx_upload_db copies flat / offsets / lengths (host buffers, clustkit's
 * compact layout) into device memory owned by the context, replacing any
 * earlier database; synchronous.
 *
 * ck_ctx_submit enqueues on `stream` (NULL: the default stream): the copy of
 * the batch's pairs (and hints) to the device, the alignment against the
 * resident database, and the copies of the outputs into the caller's host
 * buffers (any of them NULL to skip), then returns without waiting.  One
 * submission per context may be in flight; another submit or an upload
 * before it completes returns CK_ERR_INVALID_ARGUMENT.  Every host buffer of
 * the call must stay valid and unmodified until ck_ctx_poll reports it done.
 * With page-locked host buffers (cudaHostAlloc / cudaHostRegister) the call
 * returns at once; with pageable ones the CUDA runtime copies synchronously
 * and the call returns when the outputs have landed.
 *
 * ck_ctx_poll sets *out_done to 0 while the submission runs; once it has
 * finished (or when none is in flight) it sets 1 and returns the
 * submission's status: CK_OK, or CK_ERR_OUT_OF_RANGE when a pair index or a
 * sequence extent was outside the database.  ck_ctx_wait blocks until the
 * submission has finished and returns the same status.
 * Results are those of ck_sw_batch with the same arguments. */
int32_t ck_ctx_upload_db(int32_t ctx, const uint8_t *flat, int64_t flat_len, const int64_t *offsets,
                         const int32_t *lengths, int64_t n_seqs);
int32_t ck_ctx_submit(int32_t ctx, const int32_t *pairs, int64_t M, int32_t band_width,
                      const int8_t *sub_matrix, float threshold, const int32_t *diag_hints,
                      int32_t pass_rule, int32_t engine, float *out_sims, int32_t *out_scores,
                      int32_t *out_matches, int32_t *out_shorter, uint8_t *out_mask, void *stream);
int32_t ck_ctx_poll(int32_t ctx, int32_t *out_done);
int32_t ck_ctx_wait(int32_t ctx);

/* ------------------------------------------------------ search: k-mer index
 * CSR inverted index in clustkit's layout (clustkit/kmer_index.py:117-166),
 * built on the GPU: kmer_offsets int64[alpha^k + 1], kmer_freqs
 * int32[alpha^k], kmer_entries int64 (sequence << 32 | position), grouped by
 * k-mer value and in (sequence, position) order within a k-mer.  k-mers with a
 * code >= alpha are skipped.  entries_capacity must be at least
 * sum(max(0, length - k + 1)) (the buffer also serves as sort space); the
 * number of entries written is returned in *out_total.  Synchronous. */
int32_t ck_kmer_index_build_device(int32_t ctx, const uint8_t *d_flat, int64_t flat_len,
                                   const int64_t *d_offsets, const int32_t *d_lengths,
                                   int64_t n_seqs, int32_t k, int32_t alpha, int64_t *d_kmer_offsets,
                                   int64_t *d_kmer_entries, int64_t entries_capacity,
                                   int32_t *d_kmer_freqs, int64_t *out_total, void *stream);

/* The compact Phase-A index (clustkit's kmer_entries_compact,
 * clustkit/database.py:128-135): d_kmer_targets int32[n_entries] = the
 * sequence ids of d_kmer_entries.  The Phase-A walks below read it instead of
 * the full entries when given (half the bytes per posting); the entries stay
 * needed for Phase B. */
int32_t ck_kmer_targets_device(int32_t ctx, const int64_t *d_kmer_entries, int64_t n_entries,
                               int32_t *d_kmer_targets, void *stream);

/* LSH candidate pairs on the device (clustkit/lsh.py:20-178): d_sketches is
 * uint64 [n][s]; band_idx_host int32 [num_tables][num_bands] and seeds_host
 * uint64 [num_tables] are the per-table band positions and seeds (clustkit
 * draws them with np.random.RandomState(seed), lsh.py:116-123; the caller
 * passes them in).  Writes the de-duplicated pairs (i < j), sorted by
 * (i, j), as int32 [count][2] to d_out_pairs and their number to *out_count;
 * when count > capacity nothing is written, *out_count holds the count and the
 * call returns CK_ERR_OUT_OF_MEMORY.  Identical to clustkit whenever no bucket
 * has more than 1000 members; in a larger bucket the 1000 lowest sequence ids
 * are kept (clustkit keeps the first 1000 of numpy's unstable argsort).
 * Blocking; scratch ~ n*s*8 + 16*(pairs over all tables) bytes. */
int32_t ck_lsh_candidates_device(int32_t ctx, const uint64_t *d_sketches, int64_t n, int32_t s,
                                 int32_t num_tables, int32_t num_bands, const int32_t *band_idx_host,
                                 const uint64_t *seeds_host, int32_t *d_out_pairs, int64_t capacity,
                                 int64_t *out_count, void *stream);

/* The same with clustkit's BLOSUM62 similar-k-mer scoring (k = 5,
 * clustkit/kmer_index.py:1187-1328, its default search mode with
 * kmer_score_thresh = 13): every 5-mer whose column-sum score under
 * sub_matrix_host (int8 [20][20], row = query residue) against a query 5-mer
 * is >= kmer_score_thresh adds that score to each target of its posting list
 * (k-mers with frequency 0 or above freq_thresh skipped); sums are int32, not
 * saturated; survivors and cap as above.  d_kmer_targets (may be NULL) as
 * in ck_search_phase_a_device.
 * The (query, 5-mer, score) triples are listed once into a device list that
 * the posting walk then reads.  list_capacity < 0: the library sizes that
 * list from its scratch, reads the count on the host (blocking) and, when it
 * was too small, grows it and lists again.  list_capacity >= 0: at most that
 * many triples (8 bytes each in the context's scratch), no host
 * synchronisation (the call can be captured in a CUDA graph); a call that
 * lists more walks only the first list_capacity and the next status check
 * reports CK_ERR_CAPACITY. */
int32_t ck_search_phase_a_similar_device(int32_t ctx, const uint8_t *d_qflat, int64_t qflat_len,
                                         const int64_t *d_qoffsets, const int32_t *d_qlengths, int32_t nq,
                                         int32_t max_qlen, const int8_t *sub_matrix_host,
                                         int32_t kmer_score_thresh, const int64_t *d_kmer_offsets,
                                         const int64_t *d_kmer_entries, const int32_t *d_kmer_targets,
                                         const int32_t *d_kmer_freqs, int32_t freq_thresh, int32_t num_db,
                                         int32_t min_total_hits, int32_t top_k, int32_t *d_out_targets,
                                         int32_t *d_out_scores, int32_t *d_out_n, int64_t list_capacity,
                                         void *stream);

/* The k-mer scorer of clustkit's C/OpenMP search path (batch_score_queries_c,
 * clustkit/csrc/kmer_score.c:420-470, bound at clustkit/kmer_index.py:
 * 1600-1656), on the device.  Phase A as ck_search_phase_a_device (hits from
 * the query's valid k-mers with frequency <= freq_thresh, saturating at
 * 32767, survivors with >= min_total_hits).  min_diag_hits <= 1: the survivors
 * capped at max_cands (kmer_score.c:244-262), d_out_diags zeroed (the C scorer
 * leaves them unset there).  Otherwise Phase B (kmer_score.c:264-415): the top
 * phase_a_topk survivors by (hits desc, id asc) are rescored by their hits'
 * diagonal bins (tpos - qpos + qlen) / diag_bin_width -- per target its
 * longest bin, the first on ties -- those with a bin of >= min_diag_hits hits
 * kept with that count as score and the hint bin * diag_bin_width - qlen +
 * diag_bin_width / 2 in d_out_diags (may be NULL), capped at max_cands.
 * Output rows [nq x max_cands]: targets id ascending when not capped, else the
 * max_cands best by (score desc, id asc) in that order; d_out_n [nq].
 * d_db_lengths int32 [num_db] (the target lengths size each target's bins; the
 * C scorer sorts its hits instead) is needed only for Phase B.  The k-mer
 * entries are the full (target << 32 | position) ones (needed for Phase B);
 * d_kmer_targets (may be NULL) is the compact Phase-A index, which Phase A
 * then reads, as the C scorer reads its compact_entries.  Phase B keeps a
 * diagonal-bin counter per (query, selected target, bin): sum over the
 * selected targets of (qlen + tlen) / diag_bin_width + 1.  bins_capacity >= 0
 * is the caller's bound on that number (for a batch: phase_a_topk x
 * ((total query residues + nq x longest target) / diag_bin_width + nq)); the
 * call then runs without host synchronisation, so it can be captured in a
 * CUDA graph, and bins past the bound are skipped and reported as
 * CK_ERR_CAPACITY by ck_ctx_status.  bins_capacity < 0: the bins are
 * sized from a device count read back on the host (blocking). */
int32_t ck_search_kmer_candidates_device(int32_t ctx, const uint8_t *d_qflat, int64_t qflat_len,
                                         const int64_t *d_qoffsets, const int32_t *d_qlengths, int32_t nq,
                                         int32_t max_qlen, int32_t k, int32_t alpha,
                                         const int64_t *d_kmer_offsets, const int64_t *d_kmer_entries,
                                         const int32_t *d_kmer_targets, const int32_t *d_kmer_freqs,
                                         int32_t freq_thresh, int32_t num_db,
                                         const int32_t *d_db_lengths, int32_t min_total_hits,
                                         int32_t min_diag_hits, int32_t diag_bin_width, int32_t max_cands,
                                         int32_t phase_a_topk, int32_t *d_out_targets, int32_t *d_out_scores,
                                         int32_t *d_out_diags, int32_t *d_out_n, int64_t bins_capacity,
                                         void *stream);

/* ---------------------------------------------------- graph + components
 * The step after Align.  ck_graph_csr_device: the symmetric similarity graph
 * of clustkit/graph.py:7-39 -- edges (i, j) and (j, i) of every pair with
 * weight d_sims[e] (1.0 when NULL), columns ascending within a row, repeated
 * entries summed (scipy's canonical CSR) -- into d_indptr int64 [N + 1],
 * d_indices int32 and d_data float32 (room for 2K entries); *out_nnz = the
 * number of entries.  ck_connected_components_device: component labels of
 * the undirected graph on the pairs, numbered in order of each component's
 * smallest node as scipy's connected_components does (clustkit/cluster.py:
 * 43-55); *out_n_components, *out_rounds (may be NULL) the union-find rounds.
 * Both blocking. */
int32_t ck_graph_csr_device(int32_t ctx, const int32_t *d_pairs, const float *d_sims, int64_t K, int64_t N,
                            int64_t *d_indptr, int32_t *d_indices, float *d_data, int64_t *out_nnz,
                            void *stream);
int32_t ck_connected_components_device(int32_t ctx, const int32_t *d_pairs, int64_t K, int64_t N,
                                       int32_t *d_labels, int64_t *out_n_components, int32_t *out_rounds,
                                       void *stream);

/* The dense pair list of a search batch, for ck_sw_batch_device_ctx: entry
 * q * max_cands + c of d_pairs (int32 [nq * max_cands][2]) becomes
 * (seq0 + q, d_targets[q * max_cands + c]) for the query's first d_n[q]
 * candidates and (empty_idx, empty_idx) after them -- empty_idx names a
 * sequence of length 0, which aligns to nothing.  The candidate lists are
 * the ones the search scorers write (d_targets int32 [nq][max_cands], d_n
 * int32 [nq]).  Replaces the per-query loop of clustkit/kmer_index.py:
 * 2230-2266 that gathers (query, target) pairs for the SW call.
 * Asynchronous on `stream`. */
int32_t ck_search_pairs_device(int32_t nq, int32_t max_cands, int32_t seq0, int32_t empty_idx,
                               const int32_t *d_n, const int32_t *d_targets, int32_t *d_pairs,
                               void *stream);
/* Phase-A k-mer scoring of a query batch (clustkit/kmer_index.py:470-534 with
 * the per-query cap of :858-902): hits per database sequence from the query's
 * valid k-mers with frequency <= freq_thresh, saturating at 32767; targets with
 * at least min_total_hits hits survive; at most top_k per query, chosen by hit
 * count with ties to the lower target id, are written in target-id order to
 * d_out_targets[q * top_k ...] (hit counts to d_out_scores, may be NULL) and
 * their number to d_out_n[q].  Every query's extent is checked against
 * qflat_len on the device (CK_ERR_OUT_OF_RANGE, reported by ck_ctx_status);
 * max_qlen sizes the grid only.  Uses nq * num_db * 4 bytes of context
 * scratch.  When more than top_k survive, the top_k are written in descending
 * count order (ties: lower id first), as clustkit's argsort(-scores) orders
 * them; otherwise in id order.  The posting walk reads d_kmer_targets (the
 * compact index of ck_kmer_targets_device) when it is not NULL, else the
 * targets of d_kmer_entries; one of the two must be given. */
int32_t ck_search_phase_a_device(int32_t ctx, const uint8_t *d_qflat, int64_t qflat_len,
                                 const int64_t *d_qoffsets,
                                 const int32_t *d_qlengths, int32_t nq, int32_t max_qlen, int32_t k,
                                 int32_t alpha, const int64_t *d_kmer_offsets,
                                 const int64_t *d_kmer_entries, const int32_t *d_kmer_targets,
                                 const int32_t *d_kmer_freqs, int32_t freq_thresh, int32_t num_db,
                                 int32_t min_total_hits, int32_t top_k, int32_t *d_out_targets,
                                 int32_t *d_out_scores, int32_t *d_out_n, void *stream);

/* ---------------------------------------------------- measurement probe
 * Sustained lane-operation rate of one integer instruction class on the
 * current device, used as the roofline denominator of the SW kernels.
 * which: 0 = __viaddmax_s32, 1 = __vimax3_s32, 2 = 3-input 32-bit add,
 * 3 = __viaddmax_s16x2 (2 lane-ops per instruction), 4 = 3-input logic op,
 * 5 = 32-bit multiply-add.  Writes lane-ops/s. */
int32_t ck_probe_int_rate(int32_t which, double *out_ops_per_s);
/* DP cells per second of three forms of the Smith-Waterman cell, each run as
 * the strip kernel runs it (16 rows a lane, register state, increments from
 * shared memory) but without the kernel's window, residue stream and
 * first-maximum tracking: form 0 = the exact int32 packed key this library
 * uses; 1 = int16x2 score only (two pairs a lane; no match count, so not
 * usable for clustkit's identity); 2 = int16x2 with match counts carried in
 * a second int16x2 register and picked by compare masks (what exact tracking
 * at two pairs a lane costs); 3 = form 0 with the strip's lower half one
 * column behind its upper half (two independent row chains a column); 4 = a
 * compact key with an 11-bit match count and a 3-bit gap-extension counter
 * cleared every few cells in place of a tie bit set at every cell.  A
 * measurement of the cell arithmetic, no counterpart in clustkit. */
int32_t ck_probe_cell_rate(int32_t form, double *out_cells_per_s);

#ifdef __cplusplus
}
#endif

#endif /* CLUSTKIT_GB300_H */
