/*
 * blamm_host.h -- C ABI of the host library libblamm_host.so: the motif-bank
 * side of biointec/blamm's scan path (MotifContainer, Motif, ScoreHistogram;
 * src/motif.h, src/motif.cpp), for callers that drive libblamm_gpu.so
 * without the `blamm` command line (language bindings, benchmarks, services).
 *
 * A bank is a MotifContainer: motifs sorted by length, optionally with their
 * reverse complements interleaved ([m0, rc(m0), m1, rc(m1), ...]); column c
 * of its matrix P is motif c.  Every call returns 0 on success, negative on
 * error (blamm_host_last_error() has the message, per thread).
 */
#ifndef BLAMM_HOST_H
#define BLAMM_HOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct blamm_bank blamm_bank;

const char *blamm_host_last_error(void);

/* MotifContainer::load (src/motif.cpp:323-338) + addReverseComplements (:439-449).
 * motif_file: JASPAR when it ends in ".jaspar", Cluster-Buster otherwise. */
int blamm_bank_load(const char *motif_file, int load_permutations, int revcompl, blamm_bank **out);

/* A bank from in-memory PFMs: pfm holds the motifs' L x 4 (A,C,G,T) counts
 * back to back, lengths[i] their lengths; names are "M<i>".  Sorted by length
 * like a loaded file. */
int blamm_bank_from_pfms(const uint64_t *pfm, const int32_t *lengths, int nmotifs, int revcompl,
                         blamm_bank **out);
void blamm_bank_free(blamm_bank *bank);

int blamm_bank_columns(const blamm_bank *bank);  /* motifs in the container */
int blamm_bank_max_len(const blamm_bank *bank);

/* MotifContainer::generateMatrix (src/motif.cpp:542-564): PWMs for the
 * background counts (A,C,G,T) and pseudocount, and the matrix P. */
int blamm_bank_generate(blamm_bank *bank, const uint64_t bg_counts[4], float pseudo);

/* P as column-major floats (columns x 4*max_len), lengths, strands (1 = rc). */
int blamm_bank_matrix(const blamm_bank *bank, float *P, int32_t *lengths, int32_t *revcompl);

/* Motif::getMinScore / getMaxScore per column (src/motif.cpp:241-265). */
int blamm_bank_min_max(const blamm_bank *bank, float *min_score, float *max_score);

/* p-value thresholds from theoretical histograms: per column, the histogram of
 * `hist` (src/hist.cpp:162-175; nbins bins, max_length observations, iid
 * background probabilities bg_prob) of the forward motif of the same name,
 * inverted at pvalue (ScoreHistogram::getScoreCutoff, src/motif.cpp:47-69).
 * Histograms are kept in memory (no text round trip of the .dat files). */
int blamm_bank_pvalue_thresholds(const blamm_bank *bank, const float bg_prob[4], int nbins,
                                 uint64_t max_length, float pvalue, float *thr);

/* For every column, the column of the forward motif whose histogram gives
 * its p-value threshold (the same base name, src/motif.h:256-267): the
 * hist_of argument of blamm_theoretical_hist. */
int blamm_bank_hist_columns(const blamm_bank *bank, int32_t *hist_of);

/* Scores as the occurrence file prints them (the reference's default ostream
 * output, printf %g: 6 significant digits): value i goes to out + i * stride as a
 * zero-terminated string (stride >= 16). */
int blamm_format_scores(const float *values, int64_t n, char *out, int stride);

/* Name of column c (valid until the bank is freed). */
const char *blamm_bank_name(const blamm_bank *bank, int c);

/* FASTA streaming (FastaBatch, src/sequence.cpp:123-293): the files' runs of
 * A/C/G/T/a/c/g/t concatenated into one stream, cut into chunks of `payload`
 * positions plus `overlap` bases that reappear at the start of the next chunk.
 * max_filt truncates the stream (FastaBatch's maximum filtered length; -1 =
 * no limit).  Each chunk comes with its markers: chunk position, sequence index
 * and position inside the sequence of every run start (the first marker is at
 * chunk position 0).  Chunk pointers stay valid until the next call. */
typedef struct blamm_fasta blamm_fasta;
int blamm_fasta_open(const char *const *files, int nfiles, int64_t max_filt, blamm_fasta **out);
/* returns 1 and fills the outputs when a chunk was read, 0 at the end, <0 on error */
int blamm_fasta_next(blamm_fasta *f, int64_t payload, int64_t overlap, const char **bases, int64_t *size,
                     int64_t *chunk_payload, int64_t *offset, const int64_t **marker_pos,
                     const int64_t **marker_seq, const int64_t **marker_seqpos, int64_t *nmarkers);
/* sequences named so far (all of them once the stream is exhausted) */
int64_t blamm_fasta_num_sequences(const blamm_fasta *f);
const char *blamm_fasta_sequence_name(const blamm_fasta *f, int64_t i);
void blamm_fasta_close(blamm_fasta *f);

/* FASTA text in pieces for a device parser (the command line's GPU reader,
 * blamm_stream_load_fasta): the files' text in order, a newline added to a file
 * that lacks a final one, cut only where a header line starts, each piece at least
 * piece_bytes long (the last may be shorter).  No sequence spans two pieces.
 * _next returns 1 and the piece (valid until the next call), 0 at the end, <0 on
 * error (a file that cannot be opened: blamm_host_last_error). */
typedef struct blamm_fasta_pieces blamm_fasta_pieces;
int blamm_fasta_pieces_open(const char *const *files, int nfiles, int64_t piece_bytes, blamm_fasta_pieces **out);
int blamm_fasta_pieces_next(blamm_fasta_pieces *p, const char **text, int64_t *size);
void blamm_fasta_pieces_close(blamm_fasta_pieces *p);
/* The sequence name of the header line at byte offset header_pos of text (the first
 * whitespace-delimited token after '>', as the reference reads it), zero-terminated
 * into out (cap bytes); returns its length, or -1 if it does not fit. */
int blamm_fasta_header_name(const char *text, int64_t size, int64_t header_pos, char *out, int cap);

#ifdef __cplusplus
}
#endif
#endif
