/*
 * blamm_oracle.h -- CPU restatement of biointec/blamm's PWM scan path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU product is compared
 * against; it is never linked into, or called by, the product.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs use it.
 *
 * Parity pin: the oracle CLI (oracle/oracle_main.c) is run on the same inputs
 * as the compiled reference binary (oracle/build_ref.sh -> oracle/_ref/blamm)
 * and must produce byte-identical .dict and hist_*.dat files, identical
 * PWMthresholds.txt and the identical occurrence set with identical printed
 * scores (tests/test_oracle_pin.py, fixtures in tests/golden/).
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the blamm source tree).
 */
#ifndef BLAMM_ORACLE_H
#define BLAMM_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One occurrence: stream position of the motif start, P column, FP32 score. */
typedef struct {
    int64_t pos;
    int32_t col;
    float score;
} orc_hit;

/* A filtered base stream: the concatenation of all runs of A/C/G/T/a/c/g/t
 * characters of a set of FASTA files (sequence.cpp:142-250), with one marker
 * per maximal contiguous run (SeqBlock::append/isContiguous, sequence.cpp:35-88). */
typedef struct {
    char *bases;          /* n filtered bases (ACGTacgt) */
    int64_t n;
    int64_t *run_start;   /* stream position where run r starts (ascending, run_start[0] == 0) */
    int64_t *run_seq;     /* sequence index of run r */
    int64_t *run_seqpos;  /* 0-based position of the run start inside its sequence */
    int64_t nruns;
    char **names;         /* sequence names in reading order */
    int64_t nseq;
    int64_t tot_seq_len;  /* total characters on sequence lines (FastaBatch::_totSeqLen) */
} orc_stream;

/* sequence.cpp:142-250 + species.cpp:32-61.  max_filt truncates the stream
 * like FastaBatch's _maxFiltSeqLen (pass -1 for no limit).  Returns 0 on
 * success, nonzero (and a message in err) on error. */
int orc_stream_read(const char *const *files, int nfiles, int64_t max_filt,
                    orc_stream *out, char *err, int errlen);
void orc_stream_free(orc_stream *s);

/* Motif::PFM2PWM, motif.cpp:194-223.  pfm and pwm are L x 4 (ACGT).
 * revcomp swaps the background (A<->T, C<->G) as motif.cpp:204-207. */
void orc_pfm2pwm(const uint64_t *pfm, int L, const uint64_t bg_counts[4],
                 float pseudo, int revcomp, float *pwm);
/* Motif::revCompl on a PFM, motif.cpp:267-276. */
void orc_revcompl_pfm(const uint64_t *pfm, int L, uint64_t *out);
/* Motif::getMaxScore / getMinScore, motif.cpp:241-265. */
float orc_max_score(const float *pwm, int L);
float orc_min_score(const float *pwm, int L);

/* ScoreHistogram::getScoreCutoff, motif.cpp:47-69. */
float orc_score_cutoff(const uint64_t *counts, int64_t nbins, float min_score,
                       float width, float max_score, float pvalue);

/* Histogram::generateTheoreticalHist + Motif::computeTheoreticalSpectrum +
 * ScoreHistogram::setNumObservations (hist.cpp:162-175, motif.cpp:151-192,
 * motif.h:109-115).  counts must hold nbins zeros on entry. */
int orc_theoretical_hist(const float *pwm, int L, const float bg_prob[4],
                         int64_t nbins, uint64_t max_length, uint64_t *counts);

/* Species::getNuclProbabilities, species.cpp:63-71. */
void orc_nucl_prob(const uint64_t counts[4], float pseudo, float prob[4]);

/* Scan: every stream position p and P column c with
 *   score = sequential FP32 sum over j < len[c] of P(4j + base(p+j), c),
 *           uppercase bases only (sequence.cpp:312-318: lowercase rows of S stay 0),
 *   hit   iff score >= thr[c] (pwmscan.cpp:118) and the window fits inside its
 *           run (pwmscan.cpp:122-126).
 * P is column-major with p_rows rows (matrix.h:252-264).  This is the order in
 * which the reference's BLAS sgemm accumulates the one-hot products (and the
 * naive scorer's order, motif.cpp:225-239).  hits may be NULL to count only.
 * Returns the number of hits found (which can exceed cap; only cap are
 * written), or -1 on error. */
int64_t orc_scan(const char *bases, int64_t n, const int64_t *run_start,
                 int64_t nruns, const float *P, int p_rows, int ncols,
                 const int32_t *col_len, const float *thr, int nthreads,
                 orc_hit *hits, int64_t cap);

/* orc_scan with the simple scan's case handling (PWMScan::scanThreadNaive,
 * pwmscan.cpp:165-206): lower_scores = 1 scores lowercase bases like uppercase
 * (Motif::getScore, motif.cpp:225-239). */
int64_t orc_scan_ex(const char *bases, int64_t n, const int64_t *run_start,
                    int64_t nruns, const float *P, int p_rows, int ncols,
                    const int32_t *col_len, const float *thr, int nthreads,
                    int lower_scores, orc_hit *hits, int64_t cap);

/* Same hit set, computed the reference's way: per block of h*w payload bases
 * (+ overlap), a one-hot S matrix, one BLAS sgemm per P tile per column offset,
 * then a threshold scan of R (pwmscan.cpp:223-278, matrix.h:292-306,
 * sequence.cpp:299-340, pwmscan.cpp:104-133).  Needs orc_set_blas() first.
 * tiles: ntiles x (colStart, colEnd, rowEnd) as MotifContainer's MatrixTile. */
int orc_set_blas(const char *libpath);
int64_t orc_scan_blas(const char *bases, int64_t n, const int64_t *run_start,
                      int64_t nruns, const float *P, int p_rows, int ncols,
                      const int32_t *col_len, const float *thr,
                      const int32_t *tiles, int ntiles, int h, int w,
                      int nthreads, orc_hit *hits, int64_t cap);

/* MotifContainer::generateMatrixTiles, motif.cpp:451-540.  lens: column
 * lengths (sorted ascending as in the reference).  Writes up to max_tiles
 * (colStart, colEnd, rowEnd) triples; returns the tile count. */
int orc_matrix_tiles(const int32_t *lens, int ncols, int64_t min_zero_area,
                     int32_t *tiles, int max_tiles);

/* Scores as PWMScan::writeOccToDisk prints them (src/pwmscan.cpp:88-95): the
 * default std::ostream float output, i.e. printf("%g"); value i goes to
 * out + i * stride. */
void orc_format_scores(const float *values, int64_t n, char *out, int stride);

#ifdef __cplusplus
}
#endif
#endif
