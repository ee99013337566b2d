/*
 * oracle_main.c -- command-line driver of the CPU oracle (TEST INFRASTRUCTURE).
 *
 * Mirrors `blamm dict|hist|scan` (blstools.cpp:113-166) closely enough that its
 * output files can be compared with the compiled reference's on the same
 * inputs: <manifest>.dict (dict.cpp:53-115, species.cpp:149-207),
 * hist_<group>_<motif>.dat/.gnu (hist.cpp:177-266, motif.cpp:71-107),
 * PWMthresholds.txt and the occurrence file (pwmscan.cpp:456-648, 81-102).
 * Only the theoretical histogram is restated (the hist default).  The scan
 * writes occurrences sorted by (sequence stream position, P column); the
 * reference's order is thread-dependent, so comparisons use sorted sets.
 */
#define _GNU_SOURCE
#include "blamm_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static void die(const char *msg)
{
    fprintf(stderr, "%s\n", msg);
    exit(EXIT_FAILURE);
}

/* ---------------- text input helpers (istream >> / getline semantics) ---- */

typedef struct {
    char *buf;
    size_t n, pos;
    int fail;
} text;

static int text_load(const char *fn, text *t)
{
    FILE *fp = fopen(fn, "rb");
    if (!fp) return -1;
    fseek(fp, 0, SEEK_END);
    long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    t->buf = (char *)malloc((size_t)sz + 1);
    t->n = fread(t->buf, 1, (size_t)sz, fp);
    t->buf[t->n] = 0;
    t->pos = 0;
    t->fail = 0;
    fclose(fp);
    return 0;
}

static int ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

/* operator>>(string): skip whitespace, read a token; empty + fail at EOF */
static char *text_tok(text *t)
{
    if (t->fail) return strdup("");
    while (t->pos < t->n && ws(t->buf[t->pos])) t->pos++;
    size_t s = t->pos;
    while (t->pos < t->n && !ws(t->buf[t->pos])) t->pos++;
    if (t->pos == s) { t->fail = 1; return strdup(""); }
    return strndup(t->buf + s, t->pos - s);
}

/* std::getline: up to '\n' (consumed); fail when nothing is left */
static char *text_line(text *t)
{
    if (t->fail || t->pos >= t->n) { t->fail = 1; return strdup(""); }
    size_t s = t->pos;
    while (t->pos < t->n && t->buf[t->pos] != '\n') t->pos++;
    char *r = strndup(t->buf + s, t->pos - s);
    if (t->pos < t->n) t->pos++;
    return r;
}

/* operator>>(unsigned integer) on a string cursor; returns 0 on failure */
static int parse_u64(const char **p, unsigned long long *v)
{
    const char *s = *p;
    while (*s && ws(*s)) s++;
    if (*s == '+') s++;
    if (*s < '0' || *s > '9') return 0;
    unsigned long long x = 0;
    while (*s >= '0' && *s <= '9') x = x * 10 + (unsigned long long)(*s++ - '0');
    *v = x;
    *p = s;
    return 1;
}

/* operator>>(string) on a string cursor */
static int skip_tok(const char **p)
{
    const char *s = *p;
    while (*s && ws(*s)) s++;
    if (!*s) return 0;
    while (*s && !ws(*s)) s++;
    *p = s;
    return 1;
}

/* ---------------- settings.cnf (settings.cpp:481-521) ------------------- */

typedef struct {
    long long s_w, s_h, tile_min_zero_area, flush;
    float pseudo;
} settings;

static void settings_load(settings *st)
{
    st->s_w = 250; st->s_h = 1000; st->tile_min_zero_area = 64 * 64; st->flush = 100000;
    st->pseudo = 0.25f;
    text t;
    if (text_load("settings.cnf", &t)) return;
    while (!t.fail) {
        char *line = text_line(&t);
        if (!line[0] || line[0] == '#') { free(line); continue; }
        char key[256] = {0}, val[256] = {0};
        sscanf(line, "%255s %255s", key, val);
        if (!strcmp(key, "MATRIX_S_W")) st->s_w = atoll(val);
        else if (!strcmp(key, "MATRIX_S_H")) st->s_h = atoll(val);
        else if (!strcmp(key, "MATRIX_P_TILE_MIN_ZERO_AREA")) st->tile_min_zero_area = atoll(val);
        else if (!strcmp(key, "PSEUDOCOUNT")) st->pseudo = strtof(val, NULL);
        else if (!strcmp(key, "FLUSHOUTPUT")) st->flush = atoll(val);
        else fprintf(stderr, "WARNING: settings.cnf contains unknown key: %s\n", key);
        free(line);
    }
    free(t.buf);
}

/* ---------------- motifs (motif.cpp:323-449) ----------------------------- */

typedef struct {
    char *name;
    int L;
    uint64_t *pfm; /* L x 4 */
    int revcomp;
} motif;

typedef struct {
    motif *m;
    int n, cap;
} motif_set;

static void ms_push(motif_set *s, motif m)
{
    if (s->n == s->cap) {
        s->cap = s->cap ? 2 * s->cap : 16;
        s->m = (motif *)realloc(s->m, sizeof(motif) * (size_t)s->cap);
    }
    s->m[s->n++] = m;
}

static void add_char(motif *m, const unsigned long long c[4])
{
    m->pfm = (uint64_t *)realloc(m->pfm, sizeof(uint64_t) * 4 * (size_t)(m->L + 1));
    for (int k = 0; k < 4; k++) m->pfm[4 * m->L + k] = c[k];
    m->L++;
}

static void load_jaspar(const char *fn, motif_set *out)
{
    text t;
    if (text_load(fn, &t)) {
        char msg[4096];
        snprintf(msg, sizeof msg, "Could not open file: %s", fn);
        die(msg);
    }
    for (;;) {
        char *name = text_tok(&t);
        char *rest = text_line(&t);
        free(rest);
        if (t.fail) { free(name); break; }
        unsigned long long *freq[4] = {0};
        int nf[4] = {0};
        for (int i = 0; i < 4; i++) {
            char *line = text_line(&t);
            const char *p = line;
            if (skip_tok(&p) && skip_tok(&p)) {
                unsigned long long v;
                while (parse_u64(&p, &v)) {
                    freq[i] = realloc(freq[i], sizeof(unsigned long long) * (size_t)(nf[i] + 1));
                    freq[i][nf[i]++] = v;
                }
            }
            free(line);
        }
        motif m = {strdup(name[0] ? name + 1 : ""), 0, NULL, 0};
        free(name);
        for (int j = 0; j < nf[0]; j++) {
            unsigned long long c[4];
            for (int k = 0; k < 4; k++) c[k] = j < nf[k] ? freq[k][j] : 0;
            add_char(&m, c);
        }
        for (int k = 0; k < 4; k++) free(freq[k]);
        ms_push(out, m);
        t.fail = 0;
        if (t.pos >= t.n) break;
    }
    free(t.buf);
}

static void load_cb(const char *fn, motif_set *out)
{
    text t;
    if (text_load(fn, &t)) {
        char msg[4096];
        snprintf(msg, sizeof msg, "Could not open file: %s", fn);
        die(msg);
    }
    while (!t.fail) {
        char *line = text_line(&t);
        if (!line[0]) { free(line); continue; }
        if (line[0] == '>') {
            motif m = {strdup(line + 1), 0, NULL, 0};
            ms_push(out, m);
            free(line);
            continue;
        }
        if (out->n == 0) {
            char msg[4096];
            snprintf(msg, sizeof msg, "Incorrect motif file format: %s", fn);
            die(msg);
        }
        const char *p = line;
        unsigned long long c[4] = {0, 0, 0, 0};
        for (int k = 0; k < 4; k++)
            if (!parse_u64(&p, &c[k])) break;
        add_char(&out->m[out->n - 1], c);
        free(line);
    }
    free(t.buf);
}

static int motif_cmp_len(const void *a, const void *b)
{
    const motif *x = (const motif *)a, *y = (const motif *)b;
    return (x->L > y->L) - (x->L < y->L);
}

/* Motif::isPermutation / getBaseName, motif.h:256-281 */
static int perm_split(const char *name)
{
    long i = (long)strlen(name) - 1;
    for (; i >= 0; i--)
        if (!(name[i] >= '0' && name[i] <= '9')) break;
    if (i < 1) return -1;
    if (name[i - 1] == '_' && name[i] == '_') return (int)(i - 1);
    return -1;
}

static void load_motifs(const char *fn, int with_perm, motif_set *out)
{
    motif_set all = {0};
    size_t l = strlen(fn);
    if (l > 7 && !strcmp(fn + l - 7, ".jaspar")) load_jaspar(fn, &all);
    else load_cb(fn, &all);
    /* stable by length; the reference's std::sort may order equal lengths
     * differently, which changes no hit and no threshold */
    for (int i = 1; i < all.n; i++) {
        motif key = all.m[i];
        int j = i - 1;
        while (j >= 0 && motif_cmp_len(&all.m[j], &key) > 0) { all.m[j + 1] = all.m[j]; j--; }
        all.m[j + 1] = key;
    }
    for (int i = 0; i < all.n; i++) {
        if (with_perm || perm_split(all.m[i].name) < 0) ms_push(out, all.m[i]);
        else { free(all.m[i].name); free(all.m[i].pfm); }
    }
    free(all.m);
}

static void add_revcompl(motif_set *s)
{
    motif_set out = {0};
    for (int i = 0; i < s->n; i++) {
        ms_push(&out, s->m[i]);
        motif rc = {strdup(s->m[i].name), s->m[i].L, NULL, !s->m[i].revcomp};
        rc.pfm = (uint64_t *)malloc(sizeof(uint64_t) * 4 * (size_t)(rc.L ? rc.L : 1));
        orc_revcompl_pfm(s->m[i].pfm, rc.L, rc.pfm);
        ms_push(&out, rc);
    }
    free(s->m);
    *s = out;
}

/* ---------------- species / dictionary (species.cpp) --------------------- */

typedef struct {
    char *name;
    char **files;
    int nfiles;
    unsigned long long tot;
    uint64_t counts[4];
    char **seqnames;
    long long nseq;
} species;

static int strptrcmp(const void *a, const void *b)
{
    return strcmp(*(char *const *)a, *(char *const *)b);
}

static void dict_load(const char *fn, species **out, int *nout)
{
    text t;
    if (text_load(fn, &t)) {
        char msg[4096];
        snprintf(msg, sizeof msg, "Cannot open file: %s", fn);
        die(msg);
    }
    char *tok = text_tok(&t);
    free(tok);
    tok = text_tok(&t);
    int n = atoi(tok);
    free(tok);
    species *sp = (species *)calloc((size_t)(n > 0 ? n : 1), sizeof(species));
    for (int i = 0; i < n; i++) {
        free(text_tok(&t));
        sp[i].name = text_tok(&t);
        free(text_tok(&t));
        tok = text_tok(&t);
        sp[i].nfiles = atoi(tok);
        free(tok);
        sp[i].files = (char **)calloc((size_t)sp[i].nfiles + 1, sizeof(char *));
        for (int f = 0; f < sp[i].nfiles; f++) sp[i].files[f] = text_tok(&t);
        qsort(sp[i].files, (size_t)sp[i].nfiles, sizeof(char *), strptrcmp);
        free(text_tok(&t));
        tok = text_tok(&t);
        sp[i].tot = strtoull(tok, NULL, 10);
        free(tok);
        free(text_tok(&t));
        for (int k = 0; k < 4; k++) {
            tok = text_tok(&t);
            sp[i].counts[k] = strtoull(tok, NULL, 10);
            free(tok);
        }
        free(text_tok(&t));
        tok = text_tok(&t);
        sp[i].nseq = atoll(tok);
        free(tok);
        sp[i].seqnames = (char **)calloc((size_t)sp[i].nseq + 1, sizeof(char *));
        for (long long s = 0; s < sp[i].nseq; s++) sp[i].seqnames[s] = text_tok(&t);
    }
    free(t.buf);
    *out = sp;
    *nout = n;
}

static int run_dict(int argc, char **argv)
{
    if (argc < 3) die("Usage: blamm dict [options] sequences.input");
    const char *manifest = argv[argc - 1];
    text t;
    if (text_load(manifest, &t)) {
        char msg[4096];
        snprintf(msg, sizeof msg, "Could not open file: %s", manifest);
        die(msg);
    }
    species sp[256];
    int nsp = 0;
    while (!t.fail) {
        char *line = text_line(&t);
        if (!line[0]) { free(line); continue; }
        char g[4096] = {0}, f[4096] = {0};
        sscanf(line, "%4095s %4095s", g, f);
        free(line);
        if (!g[0] || !f[0]) die("File has incorrect format.");
        FILE *fp = fopen(f, "rb");
        if (!fp) {
            char msg[8192];
            snprintf(msg, sizeof msg, "Could not open fasta file: %s", f);
            die(msg);
        }
        fclose(fp);
        int idx = -1;
        for (int i = 0; i < nsp; i++) if (!strcmp(sp[i].name, g)) idx = i;
        if (idx < 0) {
            idx = nsp++;
            memset(&sp[idx], 0, sizeof(species));
            sp[idx].name = strdup(g);
            sp[idx].files = (char **)calloc(1024, sizeof(char *));
        }
        int dup = 0;
        for (int i = 0; i < sp[idx].nfiles; i++) if (!strcmp(sp[idx].files[i], f)) dup = 1;
        if (!dup) sp[idx].files[sp[idx].nfiles++] = strdup(f);
    }
    free(t.buf);
    char dictfn[4096];
    snprintf(dictfn, sizeof dictfn, "%s.dict", manifest);
    FILE *out = fopen(dictfn, "wb");
    if (!out) die("Cannot write to file");
    fprintf(out, "NUM_SPECIES\t%d\n", nsp);
    for (int i = 0; i < nsp; i++) {
        qsort(sp[i].files, (size_t)sp[i].nfiles, sizeof(char *), strptrcmp);
        orc_stream s;
        char err[512];
        if (orc_stream_read((const char *const *)sp[i].files, sp[i].nfiles, -1, &s, err, sizeof err))
            die(err);
        uint64_t c[4] = {0, 0, 0, 0};
        for (int64_t p = 0; p < s.n; p++) {
            switch (s.bases[p]) {
            case 'A': case 'a': c[0]++; break;
            case 'C': case 'c': c[1]++; break;
            case 'G': case 'g': c[2]++; break;
            default: c[3]++; break;
            }
        }
        fprintf(out, "SPECIES\t%s\n", sp[i].name);
        fprintf(out, "NUM_FASTA_FILES\t%d\n", sp[i].nfiles);
        for (int f = 0; f < sp[i].nfiles; f++) fprintf(out, "%s\n", sp[i].files[f]);
        fprintf(out, "TOT_SEQ_LENGTH\t%llu\n",
                (unsigned long long)(c[0] + c[1] + c[2] + c[3]));
        fprintf(out, "NUCL_COUNT_ACGT\t%llu\t%llu\t%llu\t%llu\n", (unsigned long long)c[0],
                (unsigned long long)c[1], (unsigned long long)c[2], (unsigned long long)c[3]);
        fprintf(out, "NUM_SEQUENCES\t%lld\n", (long long)s.nseq);
        for (int64_t q = 0; q < s.nseq; q++) fprintf(out, "%s\n", s.names[q]);
        orc_stream_free(&s);
    }
    fclose(out);
    return 0;
}

/* ---------------- hist (theoretical), hist.cpp:177-266 ------------------- */

static int run_hist(int argc, char **argv)
{
    if (argc < 4) die("Usage: blamm hist [options] motifs.input sequences.input");
    unsigned long long max_len = 10000000ULL, nbins = 250;
    char histdir[4096] = "";
    for (int i = 2; i < argc - 2; i++) {
        if ((!strcmp(argv[i], "-l") || !strcmp(argv[i], "--length")) && i + 1 < argc - 2) {
            max_len = strtoull(argv[++i], NULL, 10);
        } else if ((!strcmp(argv[i], "-b") || !strcmp(argv[i], "--numbins")) && i + 1 < argc - 2) {
            nbins = strtoull(argv[++i], NULL, 10);
            if (nbins < 2) nbins = 2;
        } else if ((!strcmp(argv[i], "-t") || !strcmp(argv[i], "--numthreads")) && i + 1 < argc - 2) {
            i++;
        } else if ((!strcmp(argv[i], "-H") || !strcmp(argv[i], "--histdir")) && i + 1 < argc - 2) {
            snprintf(histdir, sizeof histdir, "%s", argv[++i]);
            size_t l = strlen(histdir);
            if (l == 0 || histdir[l - 1] != '/') strcat(histdir, "/");
        } else {
            die("unsupported hist option in the oracle");
        }
    }
    settings st;
    settings_load(&st);
    char dictfn[4096];
    snprintf(dictfn, sizeof dictfn, "%s.dict", argv[argc - 1]);
    species *sp;
    int nsp;
    dict_load(dictfn, &sp, &nsp);
    motif_set ms = {0};
    load_motifs(argv[argc - 2], 0, &ms);
    for (int s = 0; s < nsp; s++) {
        float bg[4];
        orc_nucl_prob(sp[s].counts, st.pseudo, bg);
        for (int i = 0; i < ms.n; i++) {
            motif *m = &ms.m[i];
            float *pwm = (float *)malloc(sizeof(float) * 4 * (size_t)(m->L ? m->L : 1));
            orc_pfm2pwm(m->pfm, m->L, sp[s].counts, st.pseudo, 0, pwm);
            float mn = orc_min_score(pwm, m->L), mx = orc_max_score(pwm, m->L);
            float width = (mx - mn) / (float)nbins;
            uint64_t *cnt = (uint64_t *)calloc((size_t)nbins, sizeof(uint64_t));
            orc_theoretical_hist(pwm, m->L, bg, (int64_t)nbins, max_len, cnt);
            char fn[8192];
            snprintf(fn, sizeof fn, "%shist_%s_%s.dat", histdir, sp[s].name, m->name);
            FILE *o = fopen(fn, "wb");
            if (!o) die("Error: cannot write to file");
            fprintf(o, "%llu\t%g\t%g\n", nbins, (double)mn, (double)mx);
            unsigned long long maxy = 0;
            for (unsigned long long b = 0; b < nbins; b++) {
                fprintf(o, "%g\t%llu\n", (0.5 + (double)b) * (double)width + (double)mn,
                        (unsigned long long)cnt[b]);
                if (cnt[b] > maxy) maxy = cnt[b];
            }
            fclose(o);
            maxy = (unsigned long long)((double)maxy * 1.1);
            snprintf(fn, sizeof fn, "%shist_%s_%s.gnu", histdir, sp[s].name, m->name);
            o = fopen(fn, "wb");
            if (!o) die("Error: cannot write to file");
            fprintf(o, "set output \"hist_%s_%s.ps\"\n", sp[s].name, m->name);
            fprintf(o, "set key autotitle columnhead\n");
            fprintf(o, "set terminal postscript landscape\n");
            fprintf(o, "set terminal postscript noenhanced\n");
            fprintf(o, "set xrange [%g:%g]\n", (double)mn, (double)mx);
            fprintf(o, "set yrange [0:%llu]\n", maxy);
            fprintf(o, "set xlabel 'PWM score'\n");
            fprintf(o, "set ylabel 'count'\n");
            fprintf(o, "plot \"hist_%s_%s.dat\" using 1:2 title '%s (%s)' with boxes\n",
                    sp[s].name, m->name, m->name, sp[s].name);
            fclose(o);
            free(cnt);
            free(pwm);
        }
    }
    return 0;
}

/* ---------------- scan, pwmscan.cpp:456-648 ------------------------------ */

static float hist_cutoff(const char *histdir, const char *spname, const char *motif_name,
                         float pvalue)
{
    char base[4096];
    snprintf(base, sizeof base, "%s", motif_name);
    int cut = perm_split(base);
    if (cut >= 0) base[cut] = 0;
    char fn[8192];
    snprintf(fn, sizeof fn, "%shist_%s_%s.dat", histdir, spname, base);
    text t;
    if (text_load(fn, &t)) {
        char msg[9000];
        snprintf(msg, sizeof msg, "Error: cannot read file %s. Did you run the hist module?", fn);
        die(msg);
    }
    char *tok = text_tok(&t);
    long long nb = atoll(tok);
    free(tok);
    tok = text_tok(&t);
    float mn = strtof(tok, NULL);
    free(tok);
    tok = text_tok(&t);
    float mx = strtof(tok, NULL);
    free(tok);
    float width = (mx - mn) / (float)nb;
    uint64_t *cnt = (uint64_t *)calloc((size_t)(nb > 0 ? nb : 1), sizeof(uint64_t));
    for (long long b = 0; b < nb; b++) {
        free(text_tok(&t));
        tok = text_tok(&t);
        cnt[b] = strtoull(tok, NULL, 10);
        free(tok);
    }
    if (t.fail) die("Unexpected end-of-file reached");
    float c = orc_score_cutoff(cnt, nb, mn, width, mx, pvalue);
    free(cnt);
    free(t.buf);
    return c;
}

static int run_scan(int argc, char **argv)
{
    if (argc < 4) die("Usage: blamm scan [options] motifs.input sequences.input");
    int rc = 0, nthreads = 8, abs_set = 0, rel_set = 0, p_set = 0, simple = 0;
    float abs_t = 0.0f, rel_t = 0.95f, pval = 0.0001f;
    char histdir[4096] = "", outfn[4096] = "occurrences.txt";
    for (int i = 2; i < argc - 2; i++) {
        const char *a = argv[i];
        if (!strcmp(a, "-rc") || !strcmp(a, "--revcompl")) rc = 1;
        else if (!strcmp(a, "-s") || !strcmp(a, "--simple")) simple = 1;
        else if (!strcmp(a, "-c") || !strcmp(a, "--cuda")) {}
        else if ((!strcmp(a, "-at") || !strcmp(a, "--absthreshold")) && i + 1 < argc - 2) { abs_set = 1; abs_t = (float)atof(argv[++i]); }
        else if ((!strcmp(a, "-rt") || !strcmp(a, "--relthreshold")) && i + 1 < argc - 2) {
            rel_set = 1; rel_t = (float)atof(argv[++i]);
            if (rel_t < 0.0 || rel_t > 1.0) die("The relative threshold should be in range [0..1].");
        } else if ((!strcmp(a, "-pt") || !strcmp(a, "--pthreshold")) && i + 1 < argc - 2) {
            p_set = 1; pval = (float)atof(argv[++i]);
            if (pval < 0.0 || pval > 1.0) die("The p-value should be in range [0..1].");
        } else if ((!strcmp(a, "-t") || !strcmp(a, "--numthreads")) && i + 1 < argc - 2) {
            nthreads = atoi(argv[++i]);
            if (nthreads < 1) die("Number of threads must be a non-zero positive number");
        } else if ((!strcmp(a, "-H") || !strcmp(a, "--histdir")) && i + 1 < argc - 2) {
            snprintf(histdir, sizeof histdir, "%s", argv[++i]);
            size_t l = strlen(histdir);
            if (l == 0 || histdir[l - 1] != '/') strcat(histdir, "/");
        } else if ((!strcmp(a, "-o") || !strcmp(a, "--output")) && i + 1 < argc - 2) {
            snprintf(outfn, sizeof outfn, "%s", argv[++i]);
        } else die("unknown scan option");
    }
    if (!(abs_set || rel_set || p_set)) rel_set = 1;
    if (abs_set && rel_set) die("Specify either the absolute or relative threshold, not both.");
    if (abs_set && p_set) die("Specify either the absolute or p-value threshold, not both.");
    if (rel_set && p_set) die("Specify either the relative or p-value threshold, not both.");
    settings st;
    settings_load(&st);
    char dictfn[4096];
    snprintf(dictfn, sizeof dictfn, "%s.dict", argv[argc - 1]);
    species *sp;
    int nsp;
    dict_load(dictfn, &sp, &nsp);
    motif_set ms = {0};
    load_motifs(argv[argc - 2], 1, &ms);
    if (rc) add_revcompl(&ms);
    int maxlen = 0;
    for (int i = 0; i < ms.n; i++) if (ms.m[i].L > maxlen) maxlen = ms.m[i].L;
    int rows = 4 * maxlen, ncols = ms.n;
    FILE *cut = fopen("PWMthresholds.txt", "wb");
    FILE *out = fopen(outfn, "wb");
    if (!cut || !out) die("cannot open output files");
    long long total = 0;
    float *P = (float *)calloc((size_t)rows * (size_t)(ncols ? ncols : 1), sizeof(float));
    int32_t *len = (int32_t *)calloc((size_t)(ncols ? ncols : 1), sizeof(int32_t));
    float *thr = (float *)calloc((size_t)(ncols ? ncols : 1), sizeof(float));
    for (int s = 0; s < nsp; s++) {
        memset(P, 0, sizeof(float) * (size_t)rows * (size_t)ncols);
        for (int c = 0; c < ncols; c++) {
            motif *m = &ms.m[c];
            float *pwm = (float *)malloc(sizeof(float) * 4 * (size_t)(m->L ? m->L : 1));
            orc_pfm2pwm(m->pfm, m->L, sp[s].counts, st.pseudo, m->revcomp, pwm);
            memcpy(P + (size_t)c * rows, pwm, sizeof(float) * 4 * (size_t)m->L);
            len[c] = m->L;
            float mn = orc_min_score(pwm, m->L), mx = orc_max_score(pwm, m->L);
            if (abs_set) thr[c] = abs_t;
            else if (rel_set) thr[c] = rel_t * (mx - mn) + mn;
            else thr[c] = hist_cutoff(histdir, sp[s].name, m->name, pval);
            if (m->L <= 15)
                fprintf(cut, "%s\t%s\t%g\t%g\t%g\n", sp[s].name, m->name, (double)mn,
                        (double)thr[c], (double)mx);
            free(pwm);
        }
        orc_stream str;
        char err[1024];
        if (orc_stream_read((const char *const *)sp[s].files, sp[s].nfiles, (int64_t)sp[s].tot,
                            &str, err, sizeof err))
            die(err);
        /* The reference's default scan is its BLAS block loop (pwmscan.cpp:223-278); it runs
         * here when BLAMM_ORACLE_BLAS names an LP64 BLAS library with sgemm_, else the
         * sequential scorer, which gives the same hits (motif.cpp:225-239). */
        const char *blas = getenv("BLAMM_ORACLE_BLAS");
        int use_blas = !simple && blas && *blas;
        if (use_blas && orc_set_blas(blas)) die("BLAMM_ORACLE_BLAS: cannot load sgemm");
        int32_t *tiles = NULL;
        int ntiles = 0;
        if (use_blas) {
            tiles = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(2 * ncols + 4));
            ntiles = orc_matrix_tiles(len, ncols, st.tile_min_zero_area, tiles, 2 * ncols + 4);
        }
        int64_t nh = use_blas ? orc_scan_blas(str.bases, str.n, str.run_start, str.nruns, P, rows, ncols,
                                              len, thr, tiles, ntiles, (int)st.s_h, (int)st.s_w,
                                              nthreads, NULL, 0)
                              : orc_scan_ex(str.bases, str.n, str.run_start, str.nruns, P, rows, ncols, len,
                                            thr, nthreads, simple, NULL, 0);
        if (nh < 0) die("oracle scan failed");
        orc_hit *hits = (orc_hit *)malloc(sizeof(orc_hit) * (size_t)(nh ? nh : 1));
        if (use_blas)
            orc_scan_blas(str.bases, str.n, str.run_start, str.nruns, P, rows, ncols, len, thr, tiles,
                          ntiles, (int)st.s_h, (int)st.s_w, nthreads, hits, nh);
        else
            orc_scan_ex(str.bases, str.n, str.run_start, str.nruns, P, rows, ncols, len, thr, nthreads,
                        simple, hits, nh);
        free(tiles);
        int64_t r = 0;
        for (int64_t h = 0; h < nh; h++) {
            int64_t p = hits[h].pos;
            while (r + 1 < str.nruns && str.run_start[r + 1] <= p) r++;
            while (r > 0 && str.run_start[r] > p) r--;
            int64_t seq = str.run_seq[r];
            int64_t seqpos = str.run_seqpos[r] + (p - str.run_start[r]);
            const motif *m = &ms.m[hits[h].col];
            const char *nm = seq < sp[s].nseq ? sp[s].seqnames[seq] : "";
            fprintf(out, "%s\tblamm\t%s\t%lld\t%lld\t%g\t%c\t.\t.\n", nm, m->name,
                    (long long)seqpos, (long long)(seqpos + m->L), (double)hits[h].score,
                    m->revcomp ? '-' : '+');
        }
        total += nh;
        free(hits);
        orc_stream_free(&str);
    }
    fclose(out);
    fclose(cut);
    printf("\nWrote %lld matches to %s.\n", total, outfn);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 2) die("Usage: blamm_oracle dict|hist|scan [options]");
    if (!strcmp(argv[1], "dict")) return run_dict(argc, argv);
    if (!strcmp(argv[1], "hist")) return run_hist(argc, argv);
    if (!strcmp(argv[1], "scan")) return run_scan(argc, argv);
    die("unknown command");
    return 1;
}
