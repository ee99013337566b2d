/*
 * blamm_oracle.c -- CPU restatement of biointec/blamm's PWM scan path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): see blamm_oracle.h.  Compiled with
 * -ffp-contract=off so that every float expression rounds exactly as the
 * reference's x86-64 build does (no FMA contraction).
 */
#define _GNU_SOURCE
#include "blamm_oracle.h"

#include <dlfcn.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* small growable arrays                                                     */
/* ------------------------------------------------------------------------ */

static int grow(void **p, int64_t *cap, int64_t need, size_t elem)
{
    if (need <= *cap) return 0;
    int64_t nc = *cap ? *cap : 64;
    while (nc < need) nc *= 2;
    void *q = realloc(*p, (size_t)nc * elem);
    if (!q) return -1;
    *p = q;
    *cap = nc;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* FASTA streaming: sequence.cpp:142-250 (getNextLine, filterLine,           */
/* appendNextBlock) and the run markers of SeqBlock::append (:81-88)         */
/* ------------------------------------------------------------------------ */

static int is_valid_base(unsigned char c)
{
    /* sequence.cpp:190-193 */
    return c == 'A' || c == 'a' || c == 'C' || c == 'c' || c == 'G' ||
           c == 'g' || c == 'T' || c == 't';
}

static int is_ws(unsigned char c)
{
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

typedef struct {
    orc_stream *s;
    int64_t cap_bases, cap_runs, cap_names;
    int64_t max_filt;
} stream_builder;

static int sb_append_run(stream_builder *b, const char *data, int64_t len,
                         int64_t seq, int64_t seqpos)
{
    orc_stream *s = b->s;
    if (b->max_filt >= 0) {
        int64_t room = b->max_filt - s->n;
        if (room <= 0) return 0;
        if (len > room) len = room;
    }
    if (len <= 0) return 0;
    /* SeqBlock::isContiguous (sequence.cpp:35-50): continue the last marker
     * when it is the same sequence and the position deltas agree. */
    int contiguous = 0;
    if (s->nruns > 0) {
        int64_t r = s->nruns - 1;
        contiguous = s->run_seq[r] == seq &&
                     (s->n - s->run_start[r]) == (seqpos - s->run_seqpos[r]);
    }
    if (!contiguous) {
        int64_t c1 = b->cap_runs, c2 = b->cap_runs, c3 = b->cap_runs;
        if (grow((void **)&s->run_start, &c1, s->nruns + 1, sizeof(int64_t)) ||
            grow((void **)&s->run_seq, &c2, s->nruns + 1, sizeof(int64_t)) ||
            grow((void **)&s->run_seqpos, &c3, s->nruns + 1, sizeof(int64_t)))
            return -1;
        b->cap_runs = c1;
        s->run_start[s->nruns] = s->n;
        s->run_seq[s->nruns] = seq;
        s->run_seqpos[s->nruns] = seqpos;
        s->nruns++;
    }
    if (grow((void **)&s->bases, &b->cap_bases, s->n + len + 1, 1)) return -1;
    memcpy(s->bases + s->n, data, (size_t)len);
    s->n += len;
    s->bases[s->n] = 0;
    return 0;
}

void orc_stream_free(orc_stream *s)
{
    if (!s) return;
    free(s->bases);
    free(s->run_start);
    free(s->run_seq);
    free(s->run_seqpos);
    for (int64_t i = 0; i < s->nseq; i++) free(s->names[i]);
    free(s->names);
    memset(s, 0, sizeof(*s));
}

int orc_stream_read(const char *const *files, int nfiles, int64_t max_filt,
                    orc_stream *out, char *err, int errlen)
{
    memset(out, 0, sizeof(*out));
    stream_builder b = {out, 0, 0, 0, max_filt};
    int64_t cur_seq_len = 0;
    char *line = NULL;
    size_t lcap = 0;
    for (int f = 0; f < nfiles; f++) {
        FILE *fp = fopen(files[f], "rb");
        if (!fp) {
            snprintf(err, (size_t)errlen, "Could not open file: %s", files[f]);
            free(line);
            return 1;
        }
        ssize_t len;
        while ((len = getline(&line, &lcap, fp)) >= 0) {
            if (len > 0 && line[len - 1] == '\n') len--; /* std::getline drops '\n' only */
            if (len == 0) continue;
            if (line[0] == '>') {
                /* sequence.cpp:155-161: name = first whitespace token after '>' */
                int64_t i = 1;
                while (i < len && is_ws((unsigned char)line[i])) i++;
                int64_t j = i;
                while (j < len && !is_ws((unsigned char)line[j])) j++;
                if (grow((void **)&out->names, &b.cap_names, out->nseq + 1, sizeof(char *)))
                    goto oom;
                char *nm = (char *)malloc((size_t)(j - i + 1));
                if (!nm) goto oom;
                memcpy(nm, line + i, (size_t)(j - i));
                nm[j - i] = 0;
                out->names[out->nseq++] = nm;
                cur_seq_len = 0;
                continue;
            }
            if (out->nseq == 0) {
                snprintf(err, (size_t)errlen, "Input file does not appear to be in fasta format\n");
                fclose(fp);
                free(line);
                return 2;
            }
            int64_t seq = out->nseq - 1, pos0 = cur_seq_len;
            cur_seq_len += len;
            out->tot_seq_len += len;
            /* filterLine, sequence.cpp:181-214 */
            int64_t i = 0;
            while (i < len) {
                while (i < len && !is_valid_base((unsigned char)line[i])) i++;
                int64_t j = i;
                while (j < len && is_valid_base((unsigned char)line[j])) j++;
                if (j > i && sb_append_run(&b, line + i, j - i, seq, pos0 + i)) {
                    fclose(fp);
                    goto oom;
                }
                i = j;
            }
        }
        fclose(fp);
    }
    free(line);
    if (!out->bases) {
        out->bases = (char *)calloc(1, 1);
        if (!out->bases) goto oom;
    }
    return 0;
oom:
    free(line);
    snprintf(err, (size_t)errlen, "out of memory");
    return 3;
}

/* ------------------------------------------------------------------------ */
/* PWM construction: motif.cpp:194-223, 241-286; species.cpp:63-71           */
/* ------------------------------------------------------------------------ */

void orc_nucl_prob(const uint64_t counts[4], float pseudo, float prob[4])
{
    unsigned long long tot = 0;
    for (int i = 0; i < 4; i++) tot += counts[i];
    float t = (float)tot;
    t += 4.0f * pseudo;
    for (int i = 0; i < 4; i++) prob[i] = ((float)counts[i] + pseudo) / t;
}

void orc_pfm2pwm(const uint64_t *pfm, int L, const uint64_t bg_counts[4],
                 float pseudo, int revcomp, float *pwm)
{
    float bg[4];
    orc_nucl_prob(bg_counts, pseudo, bg);
    if (revcomp) {
        float t = bg[0]; bg[0] = bg[3]; bg[3] = t;
        t = bg[1]; bg[1] = bg[2]; bg[2] = t;
    }
    for (int i = 0; i < L; i++) {
        unsigned long long tot = 0;
        for (int j = 0; j < 4; j++) tot += pfm[4 * i + j];
        float totc = (float)tot;
        totc += 4.0f * pseudo;
        for (int j = 0; j < 4; j++) {
            float ppm = ((float)pfm[4 * i + j] + pseudo) / totc;
            pwm[4 * i + j] = log2f(ppm / bg[j]);
        }
    }
}

void orc_revcompl_pfm(const uint64_t *pfm, int L, uint64_t *out)
{
    for (int i = 0; i < L; i++)
        for (int j = 0; j < 4; j++) out[4 * i + j] = pfm[4 * (L - 1 - i) + (3 - j)];
}

static float fmaxf_ref(float a, float b) { return (a < b) ? b : a; } /* std::max */
static float fminf_ref(float a, float b) { return (b < a) ? b : a; } /* std::min */

float orc_max_score(const float *pwm, int L)
{
    float s = 0.0f;
    for (int i = 0; i < L; i++) {
        float ac = fmaxf_ref(pwm[4 * i + 0], pwm[4 * i + 1]);
        float gt = fmaxf_ref(pwm[4 * i + 2], pwm[4 * i + 3]);
        s += fmaxf_ref(ac, gt);
    }
    return s;
}

float orc_min_score(const float *pwm, int L)
{
    float s = 0.0f;
    for (int i = 0; i < L; i++) {
        float ac = fminf_ref(pwm[4 * i + 0], pwm[4 * i + 1]);
        float gt = fminf_ref(pwm[4 * i + 2], pwm[4 * i + 3]);
        s += fminf_ref(ac, gt);
    }
    return s;
}

/* ------------------------------------------------------------------------ */
/* Histograms: motif.cpp:47-69, 151-192; motif.h:109-115; hist.cpp:162-175  */
/* ------------------------------------------------------------------------ */

float orc_score_cutoff(const uint64_t *counts, int64_t nbins, float min_score,
                       float width, float max_score, float pvalue)
{
    double tot = 0.0;
    for (int64_t i = 0; i < nbins; i++) tot += (double)counts[i];
    double best = (double)pvalue * tot;
    double curr = best;
    for (int64_t i = nbins - 1; i >= 0; i--) {
        if ((double)counts[i] < curr) {
            curr -= (double)counts[i];
        } else {
            double frac = curr / (double)counts[i];
            float cutoffi = (float)(frac * (double)i + (1.0 - frac) * (double)(i + 1));
            return cutoffi * width + min_score;
        }
    }
    return max_score;
}

int orc_theoretical_hist(const float *pwm, int L, const float bg_prob[4],
                         int64_t nbins, uint64_t max_length, uint64_t *counts)
{
    if (L <= 0 || nbins <= 0) return -1;
    float mn = orc_min_score(pwm, L), mx = orc_max_score(pwm, L);
    float range = mx - mn;
    float a = (float)nbins / range;
    float b = -a * mn / (float)L;
    int *q = (int *)malloc(sizeof(int) * 4 * (size_t)L);
    if (!q) return -1;
    /* bounds of every reachable prefix sum, over all positions */
    int64_t plo = 0, phi = 0, qmin = 0, qmax = 0;
    for (int p = 0; p < L; p++) {
        int lo = 0, hi = 0;
        for (int k = 0; k < 4; k++) {
            q[4 * p + k] = (int)roundf(a * pwm[4 * p + k] + b);
            if (k == 0 || q[4 * p + k] < lo) lo = q[4 * p + k];
            if (k == 0 || q[4 * p + k] > hi) hi = q[4 * p + k];
        }
        plo += lo;
        phi += hi;
        if (p == 0 || plo < qmin) qmin = plo;
        if (p == 0 || phi > qmax) qmax = phi;
    }
    /* The reference keeps a std::map<int,float> per position; iterating the
     * present keys in ascending order is reproduced with a dense array plus a
     * presence flag (absent keys must not be created: their zero entries
     * would later overwrite histogram bins). */
    int64_t width = (int64_t)qmax - qmin + 1;
    float *cur = (float *)calloc((size_t)width, sizeof(float));
    float *nxt = (float *)calloc((size_t)width, sizeof(float));
    unsigned char *pc = (unsigned char *)calloc((size_t)width, 1);
    unsigned char *pn = (unsigned char *)calloc((size_t)width, 1);
    if (!cur || !nxt || !pc || !pn) {
        free(q); free(cur); free(nxt); free(pc); free(pn);
        return -1;
    }
    /* running offset: keys of position p live in [lo_p, hi_p] */
    int64_t base = qmin; /* array index = key - base */
    for (int k = 0; k < 4; k++) {
        int64_t key = q[k];
        cur[key - base] += bg_prob[k];
        pc[key - base] = 1;
    }
    for (int p = 1; p < L; p++) {
        memset(nxt, 0, sizeof(float) * (size_t)width);
        memset(pn, 0, (size_t)width);
        for (int64_t idx = 0; idx < width; idx++) {
            if (!pc[idx]) continue;
            int64_t key = idx + base;
            for (int k = 0; k < 4; k++) {
                int64_t t = key + q[4 * p + k] - base;
                nxt[t] += cur[idx] * bg_prob[k];
                pn[t] = 1;
            }
        }
        float *tf = cur; cur = nxt; nxt = tf;
        unsigned char *tp = pc; pc = pn; pn = tp;
    }
    /* spectrum: map<float,float>::insert keeps the first value of a key;
     * keys arrive ascending (a > 0), so a duplicate float key is skipped. */
    float hw = (mx - mn) / (float)nbins;
    int have_prev = 0;
    float prev = 0.0f;
    for (int64_t idx = 0; idx < width; idx++) {
        if (!pc[idx]) continue;
        int64_t key = idx + base;
        float score = ((float)key - (float)L * b) / a;
        if (have_prev && score == prev) continue;
        have_prev = 1;
        prev = score;
        float cntf = (float)max_length * cur[idx];
        uint64_t cnt = (uint64_t)cntf;
        int bin = (int)((score - mn) / hw);
        if (bin < 0) bin = 0;
        if (bin > (int)(nbins - 1)) bin = (int)(nbins - 1);
        counts[bin] = cnt; /* setNumObservations overwrites */
    }
    free(q); free(cur); free(nxt); free(pc); free(pn);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* P tiling: motif.cpp:451-540                                              */
/* ------------------------------------------------------------------------ */

int orc_matrix_tiles(const int32_t *lens, int ncols, int64_t min_zero_area,
                     int32_t *tiles, int max_tiles)
{
    if (ncols <= 0) return 0;
    int64_t maxlen = 0;
    for (int i = 0; i < ncols; i++) if (lens[i] > maxlen) maxlen = lens[i];
    int cap = ncols * 2 + 4, n = 1;
    int64_t *cs = malloc(sizeof(int64_t) * cap), *ce = malloc(sizeof(int64_t) * cap),
            *re = malloc(sizeof(int64_t) * cap);
    int64_t *ncs = malloc(sizeof(int64_t) * cap), *nce = malloc(sizeof(int64_t) * cap),
            *nre = malloc(sizeof(int64_t) * cap);
    cs[0] = 0; ce[0] = ncols; re[0] = 4 * maxlen;
    for (;;) {
        int nn = 0, did = 0;
        for (int t = 0; t < n; t++) {
            int64_t best_area = 0, best_j = cs[t] + 1;
            for (int64_t j = cs[t] + 1; j < ce[t]; j++) {
                int64_t area = (j - cs[t]) * (re[t] - 4 * (int64_t)lens[j - 1]);
                if (area > best_area) { best_area = area; best_j = j; }
            }
            int64_t lre = 4 * (int64_t)lens[best_j - 1];
            int64_t keep_area = (re[t] - lre) * (best_j - cs[t]);
            if (keep_area >= min_zero_area && nn + 2 <= cap) {
                did = 1;
                ncs[nn] = cs[t]; nce[nn] = best_j; nre[nn] = lre; nn++;
                ncs[nn] = best_j; nce[nn] = ce[t]; nre[nn] = re[t]; nn++;
            } else {
                ncs[nn] = cs[t]; nce[nn] = ce[t]; nre[nn] = re[t]; nn++;
            }
        }
        memcpy(cs, ncs, sizeof(int64_t) * nn);
        memcpy(ce, nce, sizeof(int64_t) * nn);
        memcpy(re, nre, sizeof(int64_t) * nn);
        n = nn;
        if (!did) break;
    }
    int out = n < max_tiles ? n : max_tiles;
    for (int t = 0; t < out; t++) {
        tiles[3 * t + 0] = (int32_t)cs[t];
        tiles[3 * t + 1] = (int32_t)ce[t];
        tiles[3 * t + 2] = (int32_t)re[t];
    }
    free(cs); free(ce); free(re); free(ncs); free(nce); free(nre);
    return n;
}

/* ------------------------------------------------------------------------ */
/* scan (sequential FP32 scores)                                            */
/* ------------------------------------------------------------------------ */

static inline int base_code(char c)
{
    /* sequence.cpp:312-318: only uppercase bases set a 1 in S */
    switch (c) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    default: return 4;
    }
}

/* index of the run containing stream position p (run_start ascending) */
static int64_t run_of(const int64_t *run_start, int64_t nruns, int64_t p)
{
    int64_t lo = 0, hi = nruns; /* first run_start > p */
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        if (run_start[mid] <= p) lo = mid + 1; else hi = mid;
    }
    return lo - 1;
}

typedef struct {
    const char *bases;
    const unsigned char *code;
    int64_t n, p0, p1;
    const int64_t *run_start;
    int64_t nruns;
    const float *P;
    int p_rows, ncols;
    const int32_t *len;
    const float *thr;
    orc_hit *hits;
    int64_t nhits, cap;
    int failed;
} scan_job;

static void push_hit(scan_job *j, int64_t p, int32_t c, float s)
{
    if (j->nhits >= j->cap) {
        if (grow((void **)&j->hits, &j->cap, j->nhits + 1, sizeof(orc_hit))) { j->failed = 1; return; }
    }
    j->hits[j->nhits].pos = p;
    j->hits[j->nhits].col = c;
    j->hits[j->nhits].score = s;
    j->nhits++;
}

static void *scan_worker(void *arg)
{
    scan_job *j = (scan_job *)arg;
    if (j->p0 >= j->p1) return NULL;
    int64_t r = run_of(j->run_start, j->nruns, j->p0);
    for (int64_t p = j->p0; p < j->p1; p++) {
        while (r + 1 < j->nruns && j->run_start[r + 1] <= p) r++;
        int64_t run_end = (r + 1 < j->nruns) ? j->run_start[r + 1] : j->n;
        int64_t rem = run_end - p;
        for (int c = 0; c < j->ncols; c++) {
            int L = j->len[c];
            if (L > rem) continue;
            const float *col = j->P + (size_t)c * (size_t)j->p_rows;
            float s = 0.0f;
            for (int k = 0; k < L; k++) {
                int b = j->code[p + k];
                if (b < 4) s = s + col[4 * k + b];
            }
            if (s >= j->thr[c]) push_hit(j, p, c, s);
        }
    }
    return NULL;
}

static int64_t collect(scan_job *jobs, int nt, orc_hit *hits, int64_t cap)
{
    int64_t tot = 0;
    for (int t = 0; t < nt; t++) {
        if (jobs[t].failed) tot = -1;
    }
    if (tot < 0) {
        for (int t = 0; t < nt; t++) free(jobs[t].hits);
        return -1;
    }
    for (int t = 0; t < nt; t++) {
        for (int64_t i = 0; i < jobs[t].nhits; i++, tot++)
            if (hits && tot < cap) hits[tot] = jobs[t].hits[i];
        free(jobs[t].hits);
    }
    return tot;
}

static unsigned char *make_codes(const char *bases, int64_t n, int lower_scores)
{
    unsigned char *code = (unsigned char *)malloc((size_t)n + 1);
    if (!code) return NULL;
    for (int64_t i = 0; i < n; i++) {
        char c = bases[i];
        /* Motif::getScore / char2idx (motif.cpp:138-149, 225-239) is case-insensitive */
        if (lower_scores && c >= 'a' && c <= 'z') c = (char)(c - 32);
        code[i] = (unsigned char)base_code(c);
    }
    code[n] = 4;
    return code;
}

int64_t orc_scan(const char *bases, int64_t n, const int64_t *run_start,
                 int64_t nruns, const float *P, int p_rows, int ncols,
                 const int32_t *col_len, const float *thr, int nthreads,
                 orc_hit *hits, int64_t cap)
{
    return orc_scan_ex(bases, n, run_start, nruns, P, p_rows, ncols, col_len, thr,
                       nthreads, 0, hits, cap);
}

int64_t orc_scan_ex(const char *bases, int64_t n, const int64_t *run_start,
                    int64_t nruns, const float *P, int p_rows, int ncols,
                    const int32_t *col_len, const float *thr, int nthreads,
                    int lower_scores, orc_hit *hits, int64_t cap)
{
    if (n < 0 || ncols < 0 || (n > 0 && nruns <= 0)) return -1;
    if (nthreads < 1) nthreads = 1;
    if (n == 0 || ncols == 0) return 0;
    unsigned char *code = make_codes(bases, n, lower_scores);
    if (!code) return -1;
    scan_job *jobs = (scan_job *)calloc((size_t)nthreads, sizeof(scan_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    int64_t per = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        scan_job *j = &jobs[t];
        j->bases = bases; j->code = code; j->n = n;
        j->p0 = (int64_t)t * per; j->p1 = j->p0 + per < n ? j->p0 + per : n;
        if (j->p0 > n) j->p0 = n;
        j->run_start = run_start; j->nruns = nruns;
        j->P = P; j->p_rows = p_rows; j->ncols = ncols; j->len = col_len; j->thr = thr;
        pthread_create(&th[t], NULL, scan_worker, j);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    int64_t tot = collect(jobs, nthreads, hits, cap);
    free(jobs); free(th); free(code);
    return tot;
}

/* ------------------------------------------------------------------------ */
/* scan, the reference's BLAS way (for the CPU baseline)                    */
/* ------------------------------------------------------------------------ */

typedef void (*sgemm_fn)(const char *, const char *, const int *, const int *,
                         const int *, const float *, const float *, const int *,
                         const float *, const int *, const float *, float *,
                         const int *);
static sgemm_fn g_sgemm = NULL;

int orc_set_blas(const char *libpath)
{
    /* the reference is run with OPENBLAS_NUM_THREADS=1: one BLAS thread per scan thread */
    setenv("OPENBLAS_NUM_THREADS", "1", 1);
    void *h = dlopen(libpath, RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    g_sgemm = (sgemm_fn)dlsym(h, "scipy_sgemm_");
    if (!g_sgemm) g_sgemm = (sgemm_fn)dlsym(h, "sgemm_");
    void (*setnt)(int) = (void (*)(int))dlsym(h, "scipy_openblas_set_num_threads");
    if (!setnt) setnt = (void (*)(int))dlsym(h, "openblas_set_num_threads");
    if (setnt) setnt(1);
    return g_sgemm ? 0 : -2;
}

typedef struct {
    scan_job base;
    const int32_t *tiles;
    int ntiles, h, w, overlap;
    int64_t nblocks;
    int64_t *next_block; /* shared counter */
    pthread_mutex_t *mu;
} blas_job;

static void *blas_worker(void *arg)
{
    blas_job *bj = (blas_job *)arg;
    scan_job *j = &bj->base;
    const int h = bj->h, w = bj->w, ov = bj->overlap;
    const int scols = 4 * (w + ov);
    float *S = (float *)malloc(sizeof(float) * (size_t)h * (size_t)scols);
    float *R = (float *)malloc(sizeof(float) * (size_t)h * (size_t)(j->ncols > 0 ? j->ncols : 1));
    if (!S || !R) { j->failed = 1; free(S); free(R); return NULL; }
    const float one = 1.0f, zero = 0.0f;
    for (;;) {
        pthread_mutex_lock(bj->mu);
        int64_t blk = (*bj->next_block)++;
        pthread_mutex_unlock(bj->mu);
        if (blk >= bj->nblocks) break;
        int64_t start = blk * (int64_t)h * w;
        int64_t end = start + (int64_t)h * w + ov;
        if (end > j->n) end = j->n;
        int64_t bs = end - start;
        /* SeqMatrix::getNextSeqMatrix, sequence.cpp:299-340 */
        memset(S, 0, sizeof(float) * (size_t)h * (size_t)scols);
        int64_t occ_rows = (bs + w - 1) / w;
        if (occ_rows > h) occ_rows = h;
        for (int i = 0; i < occ_rows; i++)
            for (int c = 0; c < w + ov; c++) {
                int64_t bp = (int64_t)i * w + c;
                if (bp >= bs) break;
                int b = j->code[start + bp];
                if (b < 4) S[(size_t)(4 * c + b) * h + i] = 1.0f;
            }
        for (int off = 0; off < w; off++) {
            /* Matrix::sgemm_batch, matrix.h:292-306 (one sgemm per tile) */
            for (int t = 0; t < bj->ntiles; t++) {
                int c0 = bj->tiles[3 * t], c1 = bj->tiles[3 * t + 1], k = bj->tiles[3 * t + 2];
                int m = h, nn = c1 - c0, lda = h, ldb = j->p_rows, ldc = h;
                if (nn <= 0) continue;
                g_sgemm("N", "N", &m, &nn, &k, &one, S + (size_t)4 * off * h, &lda,
                        j->P + (size_t)c0 * ldb, &ldb, &zero, R + (size_t)c0 * h, &ldc);
            }
            /* PWMScan::extractOccurrences, pwmscan.cpp:104-133 */
            for (int c = 0; c < j->ncols; c++) {
                const float th = j->thr[c];
                for (int i = 0; i < occ_rows; i++) {
                    float v = R[(size_t)c * h + i];
                    if (v < th) continue;
                    int64_t bp = (int64_t)i * w + off;
                    if (bp >= bs) continue; /* getRemainingSeqLen == 0 */
                    int64_t p = start + bp;
                    int64_t r = run_of(j->run_start, j->nruns, p);
                    int64_t re = (r + 1 < j->nruns) ? j->run_start[r + 1] : j->n;
                    if (re > end) re = end;
                    if (j->len[c] > re - p) continue;
                    push_hit(j, p, c, v);
                }
            }
        }
    }
    free(S);
    free(R);
    return NULL;
}

int64_t orc_scan_blas(const char *bases, int64_t n, const int64_t *run_start,
                      int64_t nruns, const float *P, int p_rows, int ncols,
                      const int32_t *col_len, const float *thr,
                      const int32_t *tiles, int ntiles, int h, int w,
                      int nthreads, orc_hit *hits, int64_t cap)
{
    if (!g_sgemm || h <= 0 || w <= 0 || n < 0 || (n > 0 && nruns <= 0)) return -1;
    if (nthreads < 1) nthreads = 1;
    if (n == 0 || ncols == 0) return 0;
    int maxlen = 0;
    for (int c = 0; c < ncols; c++) if (col_len[c] > maxlen) maxlen = col_len[c];
    unsigned char *code = make_codes(bases, n, 0);
    if (!code) return -1;
    int64_t payload = (int64_t)h * w;
    int64_t nblocks = (n + payload - 1) / payload;
    int64_t next = 0;
    pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
    blas_job *jobs = (blas_job *)calloc((size_t)nthreads, sizeof(blas_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        blas_job *bj = &jobs[t];
        scan_job *j = &bj->base;
        j->bases = bases; j->code = code; j->n = n;
        j->run_start = run_start; j->nruns = nruns;
        j->P = P; j->p_rows = p_rows; j->ncols = ncols; j->len = col_len; j->thr = thr;
        bj->tiles = tiles; bj->ntiles = ntiles; bj->h = h; bj->w = w;
        bj->overlap = maxlen - 1; bj->nblocks = nblocks; bj->next_block = &next; bj->mu = &mu;
        pthread_create(&th[t], NULL, blas_worker, bj);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    scan_job *sj = (scan_job *)calloc((size_t)nthreads, sizeof(scan_job));
    for (int t = 0; t < nthreads; t++) sj[t] = jobs[t].base;
    int64_t tot = collect(sj, nthreads, hits, cap);
    free(sj); free(jobs); free(th); free(code);
    return tot;
}

void orc_format_scores(const float *values, int64_t n, char *out, int stride)
{
    for (int64_t i = 0; i < n; i++) snprintf(out + i * stride, (size_t)stride, "%g", (double)values[i]);
}
