/*
 * blamm_serve.h -- a scan service over one GPU (part of libblamm_host.so).
 *
 * No counterpart in the reference, which scans one fixed motif set per run
 * (src/pwmscan.cpp:439-453).  The service keeps a motif bank and several
 * threshold sets (one per p-value) resident on the device and scans requests
 * -- a base stream with its run table, a subset of the bank's columns and a
 * threshold set -- as they arrive:
 *
 *   - continuous batching: `slots` requests are in flight at once, each on its
 *     own context (CUDA stream + device buffers) driven by its own host thread.
 *     A slot takes the next queued request as soon as its previous one is done,
 *     so requests that arrive while others run are admitted without waiting for
 *     a batch boundary, and their copies and kernels overlap on the device
 *     (a small request occupies only the SMs its jobs need);
 *   - admission by device memory: a request is admitted when the device bytes
 *     it needs (stream, packed stream, candidates, hits, tile plan; an estimate
 *     made at submission) fit in what the requests in flight and the buffers the
 *     slots keep leave of the budget.  Admission is first in, first out.  A
 *     slot's context keeps the device buffers of the largest request it has run
 *     (they are reused: the slot's own kept bytes count toward its next request);
 *     their size is measured after every request, and a slot whose kept
 *     buffers no longer fit beside the others' commitments releases them
 *     (blamm_release_buffers).  When the queue's head does not fit and nothing
 *     is in flight, every slot releases its kept buffers, so a request that fits
 *     the budget alone always runs;
 *   - results: the hits of a request are the same alone and in any mix (each
 *     request has its own context; scores are exact FP32, see blamm_gpu.h).
 *
 * Latency is measured per request from submission to completion.
 */
#ifndef BLAMM_SERVE_H
#define BLAMM_SERVE_H

#include <stdint.h>

#include "blamm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct blamm_server blamm_server;

typedef struct {
    int device;          /* CUDA device */
    int slots;           /* requests in flight at once (1..64) */
    int mode;            /* BLAMM_MODE_* of every scan */
    int64_t hbm_budget;  /* device bytes the requests in flight may hold; 0 = 80% of the free memory */
} blamm_server_config;

typedef struct {
    int64_t submitted, completed, failed;
    int64_t queued;           /* waiting for a slot or for memory */
    int64_t bases;            /* positions scanned by completed requests */
    double bp_columns;        /* sum over completed requests of positions x columns */
    int64_t bytes_in_flight;  /* admitted estimate */
    int64_t bytes_held;       /* device bytes the slots' contexts keep between requests */
    int64_t peak_committed;   /* largest commitment at an admission: per slot the larger of its kept
                                 bytes and its request's estimate */
    int64_t budget;
} blamm_server_stats;

/* The bank is the matrix of blamm_set_motifs (column-major P, p_rows x ncols,
 * lengths); thr_sets holds nsets threshold sets of ncols floats each, back to
 * back.  Creates `slots` contexts and their threads. */
int blamm_server_create(const blamm_server_config *cfg, const float *P, int p_rows, int ncols,
                        const int32_t *col_len, const float *thr_sets, int nsets, blamm_server **out);

/* Queue a request and return at once.  The inputs are copied.  cols lists
 * the bank columns to scan (ncols_sel of them; 0 = all); thr_set picks the
 * threshold set.  *id identifies the request.  BLAMM_ERR_NOMEM when the request
 * alone needs more than the budget. */
int blamm_server_submit(blamm_server *s, const char *bases, int64_t n, const int64_t *run_start,
                        int64_t nruns, const int32_t *cols, int ncols_sel, int thr_set, int64_t *id);

/* Block until request id is done (timeout_ms < 0: no limit; BLAMM_ERR_TIMEOUT
 * when it runs out).  Gives its hit count and latency (submission to
 * completion, and submission to admission) in milliseconds; returns the
 * request's own status. */
int blamm_server_wait(blamm_server *s, int64_t id, int64_t timeout_ms, int64_t *n_hits, double *latency_ms,
                      double *queue_ms);

/* Copy the hits of a finished request (up to cap) and release it. */
int blamm_server_take(blamm_server *s, int64_t id, blamm_hit *hits, int64_t cap, int64_t *n_hits);

int blamm_server_stats_get(blamm_server *s, blamm_server_stats *out);

/* Message of the last failed call or request on this server. */
const char *blamm_server_last_error(blamm_server *s);

/* Finish the requests in flight, drop the queued ones, free everything. */
void blamm_server_destroy(blamm_server *s);

#ifdef __cplusplus
}
#endif
#endif
