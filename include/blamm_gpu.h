/*
 * blamm_gpu.h -- C ABI of the GB300 (sm_103a) PWM scan library, libblamm_gpu.so.
 *
 * The library replaces the compute seam of biointec/blamm's scan module:
 *   - Matrix::sgemm_batch / sgemm_batch_cuda (src/matrix.h:292-323), the
 *     batched S x P products, one per column offset,
 *   - kernel_wrapper / filterScore (src/kernel.cu:21-45), the threshold filter
 *     and hit compaction, and
 *   - PWMScan::extractOccurrences / extractOccurrences2 (src/pwmscan.cpp:104-163),
 *     the threshold and run-length checks,
 * with one fused call that takes the filtered base stream of a species and
 * returns its occurrences.  The one-hot S matrix and the score matrix R never
 * exist in memory.  Scores are bit-identical to the reference's FP32 sgemm
 * sums (sequential in motif position), and so is the hit set.
 *
 * Conventions: plain pointers and sizes, no C++ types; every call returns a
 * status (0 = ok, negative = error; blamm_last_error() has the message).  A
 * context belongs to one host thread at a time (the reference runs one host
 * thread per device, src/pwmscan.cpp:439-453); contexts are independent.
 */
#ifndef BLAMM_GPU_H
#define BLAMM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define BLAMM_OK 0
#define BLAMM_ERR_ARG (-1)         /* invalid argument */
#define BLAMM_ERR_CUDA (-2)        /* CUDA runtime error */
#define BLAMM_ERR_OVERFLOW (-3)    /* hit buffer too small; *n_hits holds the total */
#define BLAMM_ERR_TIMEOUT (-4)     /* a bounded device-side wait gave up */
#define BLAMM_ERR_NOMEM (-5)       /* device allocation failed */
#define BLAMM_ERR_UNSUPPORTED (-6) /* e.g. no sm_100-class GPU, motif too long */
#define BLAMM_ERR_STATE (-7)       /* call order (e.g. scan before set_motifs) */

/* longest motifs: the tensor-core modes take motifs up to BLAMM_MAX_TC_MOTIF_LEN
 * positions (longer ones need BLAMM_MODE_FP32); every mode up to BLAMM_MAX_MOTIF_LEN */
#define BLAMM_MAX_TC_MOTIF_LEN 256
#define BLAMM_MAX_MOTIF_LEN 1024

/* arithmetic of the contraction (the emitted scores are FP32-exact in all modes) */
#define BLAMM_MODE_FP32 0   /* plain SIMT FP32 sums: the straightforward GPU form */
#define BLAMM_MODE_BF16 1   /* tcgen05, P as one BF16 term, wide guard band */
#define BLAMM_MODE_BF16X2 2 /* tcgen05, P split hi+lo BF16 (two MMAs), narrow guard band */
#define BLAMM_MODE_AUTO 3   /* tcgen05 with one or two BF16 terms or E4M3, whichever
                               blamm_autotune measured faster on its sample (one BF16 term
                               until then) */
#define BLAMM_MODE_E4M3 4   /* tcgen05 kind::f8f6f4: P x 2^k (max |P| 2^k in (32, 64]) as one
                               E4M3 term, 8 motif positions per MMA, widest guard band;
                               motifs up to 64 positions */

typedef struct blamm_ctx blamm_ctx;

/* One occurrence (the fields of MotifOccurrence, src/motif.h:557-641, before
 * the stream position is mapped to (sequence, position)). */
typedef struct {
    int64_t pos;  /* stream position of the first motif base */
    int32_t col;  /* column of P (motif index in the MotifContainer) */
    float score;  /* FP32 score, equal to the reference's R(i, j) */
} blamm_hit;

/* Statistics of the last scan on a context. */
typedef struct {
    int64_t positions;   /* stream positions scanned */
    int64_t columns;     /* motif columns scanned */
    int64_t candidates;  /* positions x columns that passed the guard band */
    int64_t hits;        /* occurrences found */
    int32_t tiles;       /* motif tiles (tcgen05 N tiles) */
    int32_t launches;    /* kernels launched by the last scan */
    float kernel_ms;     /* device time of all kernels of the call (CUDA events) */
    float total_ms;      /* time of the whole call incl. copies (device events; wall time
                            when blamm_scan pipelines a long stream in chunks) */
    float scan_ms;       /* device time of the scan kernel alone (tcgen05 or plain FP32) */
    float rescore_ms;    /* device time of the rescoring kernel (tcgen05 modes) */
} blamm_stats;

/* Library version (major*10000 + minor*100 + patch). */
int blamm_version(void);

/* Create a context on a CUDA device (own stream, own device buffers).
 * Replaces the per-thread set-up of PWMScan::scanThreadCUBLAS
 * (src/pwmscan.cpp:297-360): cudaSetDevice, cublasCreate, cudaMalloc. */
int blamm_ctx_create(int device, blamm_ctx **out);
void blamm_ctx_destroy(blamm_ctx *ctx);
const char *blamm_last_error(const blamm_ctx *ctx);

/* Select the arithmetic (BLAMM_MODE_*).  Default BLAMM_MODE_AUTO.  Every mode
 * emits the same hits and bit-identical scores; they differ in speed only. */
int blamm_set_mode(blamm_ctx *ctx, int mode);

/* Upload the motif bank.  P is MotifContainer's matrix (src/motif.cpp:542-564):
 * column-major FP32, p_rows x ncols, p_rows = 4 * (longest motif), column c
 * holding motif c's PWM as P(4j+b, c) (b = A,C,G,T) and zeros below 4*len[c].
 * thr[c] is the score threshold of column c (Motif::getThreshold; set at
 * src/pwmscan.cpp:599-616).  Replaces the d_P / d_threshold uploads of
 * src/pwmscan.cpp:317-342 and the P tiling of MotifContainer::generateMatrixTiles
 * (src/motif.cpp:482-540), which the library re-plans for the tensor cores. */
int blamm_set_motifs(blamm_ctx *ctx, const float *P, int p_rows, int ncols,
                     const int32_t *col_len, const float *thr);

/* Replace the thresholds only (per species / per p-value), keeping the bank. */
int blamm_set_thresholds(blamm_ctx *ctx, const float *thr);

/* Scan only the n bank columns cols[0..n-1] (distinct, each in [0, ncols));
 * n = 0 scans every column again.  Hits keep the bank's column numbers.  The
 * reference always scans its whole bank; a subset serves requests that ask
 * for some motifs only.  blamm_set_motifs resets the subset. */
int blamm_set_columns(blamm_ctx *ctx, const int32_t *cols, int n);

/* Scan a filtered base stream held in host memory.
 * bases: n characters from {A,C,G,T,a,c,g,t} -- the content of the reference's
 *   SeqBlock stream (src/sequence.cpp:181-250).  Lowercase bases are scanned
 *   positions but add nothing to a score, as in the one-hot S of
 *   src/sequence.cpp:306-337.
 * run_start: nruns ascending stream positions, run_start[0] == 0, one per
 *   maximal contiguous run (the SeqBlock markers, src/sequence.cpp:81-88).
 *   A window that crosses into the next run is not a hit (src/pwmscan.cpp:122-126).
 * Writes up to hit_cap hits (unordered) and their number to *n_hits.
 * Returns BLAMM_ERR_OVERFLOW, with *n_hits = the total, when hit_cap is too small.
 * A stream longer than 32 Mi positions is scanned in chunks of 16 Mi positions
 * (plus the longest motif - 1 bases of overlap): each chunk's bases are copied
 * in on a second stream while the previous chunk is scanned, and its hits are
 * copied out while the next one is scanned (pinned host buffers let the copies
 * run beside the scan). */
int blamm_scan(blamm_ctx *ctx, const char *bases, int64_t n, const int64_t *run_start,
               int64_t nruns, blamm_hit *hits, int64_t hit_cap, int64_t *n_hits);

/* The same on device-resident data (device pointers, the context's stream):
 * nothing is copied between host and device except the hit count. */
int blamm_scan_device(blamm_ctx *ctx, const char *d_bases, int64_t n,
                      const int64_t *d_run_start, int64_t nruns, blamm_hit *d_hits,
                      int64_t hit_cap, int64_t *n_hits);

/* Drop-in for the reference's kernel_wrapper (src/kernel.cu:36-45): for the
 * column-major m x n matrix d_R, append every entry R(i,j) >= d_threshold[j]
 * to d_occScore / d_occIdx (index j*m+i) at atomically reserved slots of
 * *d_nOcc.  Device pointers; runs on the context's stream and synchronises.
 * Like kernel_wrapper it writes without a capacity check: one call appends at
 * most m*n entries, so buffers of 2*m*n entries (the reference's, allocated at
 * src/pwmscan.cpp:346-352) hold a call's output while *d_nOcc <= m*n. */
int blamm_filter_score(blamm_ctx *ctx, float *d_R, int m, int n, const float *d_threshold,
                       int *d_occIdx, float *d_occScore, int *d_nOcc);

/* Batched and graph launches (no counterpart in the reference, which
 * synchronises after every sgemm batch, src/pwmscan.cpp:386-412).
 *
 * blamm_reserve sizes the context's buffers for scans of up to max_positions
 * positions and max_candidates tensor-core candidates and builds the tile plan
 * of the current bank, columns, thresholds and mode.  After it,
 * blamm_scan_enqueue needs no allocation and no host synchronisation: it
 * enqueues packing, the scan and the rescoring on the context's stream and
 * returns.  counts is device memory of 4 uint64, set when the stream gets
 * there: [0] candidate record slots used (a record holds the candidates of one
 * position in a 32-column chunk; each CTA's warps take slots in blocks), [1]
 * hits, [2] status (non-zero: a device wait timed out), [3] candidates.  Hits
 * beyond hit_cap and records beyond the reservation (max_candidates plus the
 * blocks the warps hold) are counted but not stored; the caller compares counts
 * with its capacities and scans again with more room.  BLAMM_ERR_STATE when the reservation or plan does not
 * cover the call.
 *
 * blamm_scan_graph_create captures one blamm_scan_enqueue into an executable
 * CUDA graph (opaque handle) that blamm_scan_graph_launch replays on the
 * context's stream.  The graph holds the buffer addresses of its capture: it
 * stays valid until the bank, columns, thresholds, mode or reservation change
 * or the context is destroyed. */
int blamm_reserve(blamm_ctx *ctx, int64_t max_positions, int64_t max_candidates);
int blamm_scan_enqueue(blamm_ctx *ctx, const char *d_bases, int64_t n, const int64_t *d_run_start,
                       int64_t nruns, blamm_hit *d_hits, int64_t hit_cap, uint64_t *d_counts);
int blamm_scan_graph_create(blamm_ctx *ctx, const char *d_bases, int64_t n,
                            const int64_t *d_run_start, int64_t nruns, blamm_hit *d_hits,
                            int64_t hit_cap, uint64_t *d_counts, void **graph);
int blamm_scan_graph_launch(blamm_ctx *ctx, void *graph);
void blamm_scan_graph_destroy(void *graph);

/* Autotuner: time the tensor-core scan of the first min(n, 16 Mi) positions
 * (device data) under several tile plans -- widest N tile 128 / 192 / 256 x
 * the planner's fixed cost per job, and in BLAMM_MODE_AUTO one and two BF16
 * terms and one E4M3 term (motifs up to 64 positions) -- and keep the fastest
 * for later scans of this context (the time of
 * all kernels of the call: packing, scan, rescoring; median of three).
 * *best_ms (optional) receives that time.  Nothing to tune in BLAMM_MODE_FP32.
 * The chosen term count: blamm_get_terms. */
int blamm_autotune(blamm_ctx *ctx, const char *d_bases, int64_t n, const int64_t *d_run_start,
                   int64_t nruns, float *best_ms);

/* The planner's knobs that the autotuner sets: the widest N tile (32..256
 * columns; at most 128 gives four TMEM accumulators instead of two) and the
 * fixed cycles per job of its cost model.  Setting them replans. */
int blamm_set_plan_options(blamm_ctx *ctx, int max_tile_columns, float job_cost);
/* The tensor-core form of the current mode: 1 or 2 BF16 terms, 8 for one E4M3 term
 * (BLAMM_MODE_E4M3, or BLAMM_MODE_AUTO after the autotuner chose it); 0 for FP32. */
int blamm_get_terms(const blamm_ctx *ctx);
int blamm_get_plan_options(const blamm_ctx *ctx, int *max_tile_columns, float *job_cost);

/* The hist module's theoretical histograms and p-value thresholds on the GPU
 * (Motif::computeTheoreticalSpectrum src/motif.cpp:151-192,
 * Histogram::generateTheoreticalHist src/hist.cpp:162-175,
 * ScoreHistogram::getScoreCutoff src/motif.cpp:47-69), one CTA per column.
 * Column c's distribution is that of column hist_of[c]'s PWM (NULL: its own;
 * the reference gives a reverse-complement or permuted motif the histogram of
 * its forward motif); bg_prob are the background probabilities, nbins <= 4096
 * bins of max_length observations.  fp64_dp = 0 follows the reference's FP32
 * dynamic programme operation for operation (same counts, same thresholds bit
 * for bit); 1 runs it in FP64.  The inversion is FP64 as in the reference.
 * Outputs (host memory, either may be NULL): thr, npv x ncols thresholds (row v
 * for pvalues[v]); counts, ncols x nbins histogram counts. */
int blamm_theoretical_hist(blamm_ctx *ctx, const float *P, int p_rows, int ncols, const int32_t *col_len,
                           const int32_t *hist_of, const float bg_prob[4], int nbins, uint64_t max_length,
                           int fp64_dp, const float *pvalues, int npv, float *thr, uint64_t *counts);

/* FASTA ingest on the GPU: the filtered base stream and run table that
 * FastaBatch builds (src/sequence.cpp:142-293) from raw FASTA text in device
 * memory (several files concatenated, each ending with a newline).  Outputs,
 * device memory sized for the worst case (nraw entries each): the stream
 * bases (A/C/G/T/a/c/g/t), per run its stream start, sequence index and
 * position in the sequence (the SeqBlock markers, src/sequence.cpp:35-50),
 * and per sequence the byte offset of its '>' header line (names stay with
 * the caller).  Counts come back in *n_bases, *nruns, *nseqs, and (optional,
 * host memory) the A/C/G/T counts of the stream in nucl_counts[4] -- the
 * dict module's nucleotide composition (src/species.cpp:31-61).  Sequence
 * data before the first header gives BLAMM_ERR_ARG, as the reference rejects it. */
int blamm_fasta_parse_device(blamm_ctx *ctx, const char *d_raw, int64_t nraw, char *d_bases, int64_t *n_bases,
                             int64_t *d_run_start, int64_t *d_run_seq, int64_t *d_run_seqpos, int64_t *nruns,
                             int64_t *d_header_pos, int64_t *nseqs, uint64_t *nucl_counts);

/* The resident stream: FASTA text parsed on the device and kept in the context, so that
 * the bases never pass through host memory between the file and the scan.
 *
 * blamm_stream_load_fasta: raw (host memory, nraw bytes: one or more files' text, each
 * ending in a newline) is copied to the device and parsed as blamm_fasta_parse_device does
 * (FastaBatch's filtered stream, src/sequence.cpp:142-293); the stream, its run table and
 * the header offsets replace the context's previous resident stream.  *n_bases, *nruns,
 * *nseqs and nucl_counts[4] (may be NULL) as blamm_fasta_parse_device returns them.
 * Device memory: nraw + n_bases + 8 x (3 nruns + nseqs) bytes kept, plus ~56 bytes per raw
 * byte during the call.  blamm_release_buffers drops the resident stream.
 *
 * blamm_stream_tables: the run table (stream position, sequence index, position inside
 * the sequence; nruns entries each) and the header offsets (byte offset of each '>' in
 * raw; nseqs entries) copied to host arrays; a NULL pointer skips that array.
 *
 * blamm_scan_stream: blamm_scan over positions [begin, begin + n) of the resident stream:
 * run_start (host, nruns entries) relative to begin with run_start[0] == 0, hits (host)
 * with positions relative to begin, BLAMM_ERR_OVERFLOW as blamm_scan.  The reference has
 * no counterpart: its FastaBatch reads on the host (src/sequence.cpp:142-293) and each
 * block's S is built on the host (src/sequence.cpp:299-340). */
int blamm_stream_load_fasta(blamm_ctx *ctx, const char *raw, int64_t nraw, int64_t *n_bases, int64_t *nruns,
                            int64_t *nseqs, uint64_t *nucl_counts);
int blamm_stream_tables(blamm_ctx *ctx, int64_t *run_start, int64_t *run_seq, int64_t *run_seqpos,
                        int64_t *header_pos);
int blamm_scan_stream(blamm_ctx *ctx, int64_t begin, int64_t n, const int64_t *run_start, int64_t nruns,
                      blamm_hit *hits, int64_t hit_cap, int64_t *n_hits);

/* Number of CUDA devices (0 when there is no driver or device). */
int blamm_device_count(int *n);

/* Free and total device memory of a device (cudaMemGetInfo). */
int blamm_device_memory(int device, int64_t *free_bytes, int64_t *total_bytes);

/* Soft-masked (lowercase) bases: 0 (default) = they add nothing to a score,
 * as in the reference's BLAS/cuBLAS scan (src/sequence.cpp:312-318);
 * 1 = they score like uppercase, as in its simple scan (`scan -s`,
 * Motif::getScore, src/motif.cpp:225-239). */
int blamm_set_softmask(blamm_ctx *ctx, int lowercase_scores);

/* Empirical score histograms (the `hist -e` module, src/hist.cpp:70-140):
 * for every position whose window fits inside its run, add the FP32 score of
 * each column c to bin int((score - min_score[c]) / width[c]) clamped to
 * [0, nbins-1] (ScoreHistogram::addObservation, src/motif.h:96-102).
 * counts is ncols x nbins, row-major, and is accumulated into. */
int blamm_score_histograms(blamm_ctx *ctx, const char *bases, int64_t n, const int64_t *run_start,
                           int64_t nruns, const float *min_score, const float *width, int nbins,
                           uint64_t *counts);
/* The same over positions [begin, begin + n) of the resident stream
 * (blamm_stream_load_fasta); run_start (host) relative to begin, run_start[0] == 0. */
int blamm_score_histograms_stream(blamm_ctx *ctx, int64_t begin, int64_t n, const int64_t *run_start,
                                  int64_t nruns, const float *min_score, const float *width, int nbins,
                                  uint64_t *counts);

/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or events around the library's. */
int blamm_ctx_stream(const blamm_ctx *ctx, void **stream);

/* Statistics of the last scan. */
int blamm_last_stats(const blamm_ctx *ctx, blamm_stats *out);

/* Test and measurement hooks.
 * blamm_debug_scores: for positions [p0, p0+npos) of a host stream, the raw
 * tensor-core score of every column (row-major npos x ncols) -- the value the
 * guard band is applied to -- in the current tcgen05 mode. */
int blamm_debug_scores(blamm_ctx *ctx, const char *bases, int64_t n, int64_t p0, int64_t npos,
                       float *out);
/* The guard band of each column in the current mode (ncols floats). */
int blamm_guard_band(const blamm_ctx *ctx, float *out);
/* Role timing of the tensor-core scan kernel: enable (1) / disable (0) it for
 * later scans; read the last scan's counters (32 int64 per CTA, clock cycles:
 * 0 / 1 the even / odd issuer's waits for a free accumulator, 2 issuers' waits
 * for B tiles, 3 MMA loop, 4 loader waits for a free E stage, 5 loader waits at
 * tile changes, 7 drain warp 0's waits for an accumulator, 8 its loop, 9 its
 * drain (full accumulator to hand-back), 10 jobs, 11 even issuer's waits for E
 * windows, 12 drain warp 0's rounds with candidates, 13 its record block
 * changes, 15 its candidate test and record writing).  *nctas receives the
 * CTA count.  The timing variant of the kernel is slower than the scan itself. */
int blamm_debug_profile(blamm_ctx *ctx, int enable);
/* Failure-path test hook: with enable = 1 the tensor-core scan kernel first
 * waits on a barrier that nothing completes; every wait of the kernel gives up
 * after wait_limit_cycles (0 = the default, about 2 s of clock64 cycles), the
 * CTAs drain their copies and MMAs, free their tensor memory and the call
 * returns BLAMM_ERR_TIMEOUT; the context stays usable.  enable = 0 restores
 * normal scans (with the given limit). */
int blamm_debug_stall(blamm_ctx *ctx, int enable, long long wait_limit_cycles);
int blamm_debug_profile_read(const blamm_ctx *ctx, int64_t *out, int max_ctas, int *nctas);

/* Device memory held for scans (no counterpart in the reference, whose threads allocate
 * per run): a context keeps the per-call buffers of its largest scan so far (stream, packed
 * stream, one-hot window, run table, candidate records, hits).  blamm_ctx_call_bytes reports
 * their size; blamm_release_buffers frees them (the motif bank and its plan stay) after the
 * context's stream has drained, and trims the device's stream-ordered memory pool. */
int blamm_ctx_call_bytes(const blamm_ctx *ctx, int64_t *bytes);
int blamm_release_buffers(blamm_ctx *ctx);

/* blamm_scan_device without allocation.  It has no counterpart in the
 * reference; it is for callers that may not allocate device or host memory
 * during a scan (a memory pool that must not grow, a host thread that must not
 * block in the allocator).  Same arguments, results and status codes as
 * blamm_scan_device, but the packed stream, candidate list, counters and
 * status word live in one fixed array of device memory that this library
 * declares (about 97 MiB per device, reserved when the library's device code
 * is loaded there).  Limits: n <= 4 Mi positions per call (more gives
 * BLAMM_ERR_ARG) and at most 2 Mi tensor-core candidate record slots per call
 * (a record holds one position's candidates in a 32-column chunk; each CTA's
 * warps take slots in blocks, about 0.6 Mi of them on a full GPU; more gives
 * BLAMM_ERR_OVERFLOW: scan fewer positions per call).  The counters and the
 * status word are set to zero at the start of every call.  Preconditions are
 * checked before the size: an unprepared context fails the same way for an
 * empty stream as for a non-empty one.
 * Preconditions: a bank (blamm_set_motifs) and, in the tensor-core modes, a
 * plan for the current bank, mode and thresholds, which the first
 * blamm_scan / blamm_scan_device after a change builds (otherwise
 * BLAMM_ERR_STATE).  The first call on a device looks up the array's device
 * address and keeps it for the life of the process; make it before any stream
 * capture, and do not use this entry point on a device after cudaDeviceReset
 * (the module is reloaded and the kept address is stale).
 * The array is shared by every context on a device: calls that overlap in
 * time on one device (from two host threads, or on two streams) race on it
 * and corrupt each other's results.  Serialise them. */
int blamm_scan_device_static(blamm_ctx *ctx, const char *d_bases, int64_t n,
                             const int64_t *d_run_start, int64_t nruns, blamm_hit *d_hits,
                             int64_t hit_cap, int64_t *n_hits);

#ifdef __cplusplus
}
#endif
#endif
