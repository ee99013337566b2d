// blamm_gpu.cu -- libblamm_gpu.so: the C ABI declared in include/blamm_gpu.h.
//
// Host half of the GB300 scan: motif-bank planning (length-sorted N tiles,
// fixed-point BF16 hi/lo split, per-column guard band), device buffers, and
// the drivers that chain pack -> fused tcgen05 scan -> FP32 rescoring (or the
// plain FP32 kernel) on the context's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include "blamm_gpu.h"
#include "scan_kernels.cuh"
#include "scan_tc.cuh"
#include "hist_kernels.cuh"
#include "ingest_kernels.cuh"

#include <nvtx3/nvToolsExt.h>

// A named range on the profiler timeline (nsys, ncu --nvtx) around each entry point;
// NVTX calls do nothing unless a tool is attached.
namespace {
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
}  // namespace

using namespace blamm;

static_assert(sizeof(blamm_hit) == sizeof(HitRec), "hit record layout");

// Default scan window (positions): see launch_tc_windows.
constexpr int64_t kEWindowDefault = int64_t(16) << 20;

struct blamm_ctx {
    int device = 0;
    int sm_count = 0;
    int max_smem = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    std::string err;
    int mode = BLAMM_MODE_AUTO;
    int auto_terms = 1;  // BLAMM_MODE_AUTO: the form in use, 1 or 2 BF16 terms or kE4M3 (1 until tuned)
    bool plain_timed = false, rescore_timed = false;
    int lower_scores = 0;  // soft-masked bases add their PWM value (simple scan) when 1
    long long wait_limit = 4000000000LL;  // clock64 cycles (about 2 s)
    int debug_stall = 0;                  // test hook: make the scan kernel's first wait run out
    int64_t ewindow = 0;                  // positions per tensor-core scan window (one-hot entry array)

    // motif bank (host copy); `active` lists the columns scanned (all when empty)
    int ncols = 0, p_rows = 0, lmax = 0;
    std::vector<int32_t> active;
    int32_t *d_active = nullptr;
    size_t cap_active = 0;
    bool active_dirty = false;
    std::vector<float> P;
    std::vector<int32_t> len;
    std::vector<float> thr;
    float *d_P = nullptr;
    int32_t *d_len = nullptr;
    float *d_thr = nullptr;

    // tensor-core plan (valid for plan_terms; rebuilt on mode/threshold change)
    int plan_terms = 0;
    bool plan_valid = false;
    std::vector<TileDesc> tiles;
    std::vector<float> guard;    // per column
    std::vector<double> bias_T;  // per column: threshold - guard on the column grid
    int erows = 0;  // one-hot pair entries per E stage
    uint32_t b_term_max = 0, tmem_cols = 0;
    int acc_stages = 2;
    TileDesc *d_tiles = nullptr;
    uint8_t *d_bbuf = nullptr;
    int32_t *d_slot_col = nullptr;
    size_t cap_tiles = 0, cap_bbuf = 0, cap_slot_col = 0;
    // per-column fixed-point BF16 terms and guard bands of the bank (for colq_terms terms)
    bool colq_valid = false;
    int colq_terms = 0;
    std::vector<int> colq_k;
    std::vector<double> colq_guard;
    std::vector<uint32_t> colq_off;  // column c's 4L values start at colq_off[c]
    std::vector<uint16_t> colq_hi, colq_lo;
    std::vector<uint8_t> colq_e8;  // E4M3 codes of P(c) x 2^colq_k[c] (the E4M3 form)
    // planner knobs (the autotuner sets them): widest N tile, fixed cycles per job
    int plan_nmax = 256;
    double plan_job_cost = 700.0;

    // stream buffers
    char *d_bases = nullptr;
    size_t cap_bases = 0;
    uint32_t *d_seq2 = nullptr, *d_zmask = nullptr;
    size_t cap_words32 = 0, cap_zmask = 0;
    uint4 *d_e16 = nullptr;  // one-hot entries of the packed stream (tensor-core A operand windows)
    size_t cap_e16 = 0;
    int64_t *d_runs = nullptr;
    size_t cap_runs = 0;
    uint4 *d_cand = nullptr;  // candidate record slots (scan_tc.cuh: blocks of kRecBlock)
    int64_t cand_cap = 0;     // record slots
    blamm_hit *d_hits = nullptr;
    int64_t hits_cap = 0;
    unsigned long long *d_counters = nullptr;  // [0] candidates, [1] hits
    int *d_status = nullptr;
    // hit filtering of one chunk of a pipelined blamm_scan: hits at chunk positions >=
    // keep_below are dropped (0: none), pos_base is added to the positions written
    int64_t keep_below = 0, pos_base = 0;
    // blamm_scan's copy pipeline: a second stream and double-buffered chunk inputs
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t chunk_ev[2] = {nullptr, nullptr};
    char *d_chunk_bases[2] = {nullptr, nullptr};
    size_t cap_chunk_bases[2] = {0, 0};
    int64_t *d_chunk_runs[2] = {nullptr, nullptr};
    size_t cap_chunk_runs[2] = {0, 0};
    int64_t *h_chunk_runs[2] = {nullptr, nullptr};  // pinned: their copies stay asynchronous
    size_t cap_h_chunk_runs = 0;
    cudaEvent_t done_ev[2] = {nullptr, nullptr};  // per input buffer: its chunk's kernels are done
    unsigned long long *h_chunk_counts = nullptr;  // pinned, 4 per chunk: candidates, hits, status
    size_t cap_h_chunk_counts = 0;
    // resident stream (blamm_stream_load_fasta): FASTA text, filtered bases, run table
    // (stream position, sequence index, position in the sequence), header offsets
    char *d_raw = nullptr, *d_stream = nullptr;
    size_t cap_raw = 0, cap_stream = 0;
    int64_t *d_srun[3] = {nullptr, nullptr, nullptr}, *d_shdr = nullptr;
    size_t cap_srun[3] = {0, 0, 0}, cap_shdr = 0;
    int64_t stream_n = 0, stream_nruns = 0, stream_nseqs = 0;
    bool prof_on = false;
    long long *d_prof = nullptr;
    std::vector<long long> prof;  // last scan's role timing, 32 counters per CTA
    int prof_ctas = 0;

    blamm_stats stats{};
    int64_t rec_slots = 0;  // record slots the last tensor-core scan reserved
};

// ------------------------------------------------------------------ errors
static int fail(blamm_ctx *c, int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? BLAMM_ERR_NOMEM : BLAMM_ERR_CUDA, \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

// Grow a context buffer to at least `need` elements.  The stream-ordered
// allocator keeps a growing buffer from synchronising the whole device (other
// contexts' work keeps running); every use of these buffers is on ctx->stream.
template <typename T>
static int ensure(blamm_ctx *ctx, T **ptr, size_t *cap, size_t need)
{
    if (need <= *cap && *ptr) return BLAMM_OK;
    if (*ptr) CK(cudaFreeAsync(*ptr, ctx->stream));
    *ptr = nullptr;
    *cap = 0;
    size_t n = std::max<size_t>(need, 1);
    CK(cudaMallocAsync((void **)ptr, n * sizeof(T), ctx->stream));
    *cap = n;
    return BLAMM_OK;
}

static int scanned_columns(const blamm_ctx *ctx)
{
    return ctx->active.empty() ? ctx->ncols : (int)ctx->active.size();
}

// ------------------------------------------------------------------ planning
namespace {

// Fixed-point BF16 split of one column: hi on the grid 2^-k, lo on 2^-(k+8),
// with k chosen so |hi| <= 128 * 2^-k.  Every partial sum of such values over
// up to 256 motif positions is an integer multiple of 2^-(k+8) below 2^24 of
// those units, i.e. exactly representable in FP32: the tensor-core
// accumulation is exact, whatever its internal rounding.
struct ColQuant {
    int k;
};

int column_exponent(const float *col, int L)
{
    double mx = 0.0;
    for (int r = 0; r < 4 * L; ++r) mx = std::max(mx, (double)std::fabs(col[r]));
    if (!(mx > 0.0) || !std::isfinite(mx)) return -30;
    int e;
    double f = std::frexp(mx, &e);  // mx = f * 2^e, f in [0.5, 1)
    if (f == 0.5) e -= 1;           // mx is a power of two: mx <= 2^(e-1)
    return std::max(-30, std::min(40, e));
}

inline double q_hi(double v, int k) { return std::nearbyint(std::ldexp(v, k)) * std::ldexp(1.0, -k); }
inline double q_lo(double r, int k) { return std::nearbyint(std::ldexp(r, k + 8)) * std::ldexp(1.0, -(k + 8)); }

inline uint16_t bf16_bits_exact(double v)
{
    float f = (float)v;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return (uint16_t)(u >> 16);  // exact: v has <= 8 significant bits
}

// A tile whose longest motif has length L = 4g-3 or 4g-2 leaves motif positions 4g-2 and
// 4g-1 (the second K core of its last k-step) unused: the bias rides there.
inline bool bias_folds(int L) { return L % 4 == 1 || L % 4 == 2; }

// E4M3 (sign, 4 exponent bits with bias 7, 3 mantissa bits; exponent 0 subnormal, largest
// finite 448).  In units of 2^-9 every E4M3 value is an integer: m (subnormal, m < 8) or
// (8 + m) 2^(e-1).
constexpr int64_t kE4M3MaxUnits = 448 * 512;

// The E4M3 value nearest to v (ties to even mantissa), as its code; |v| <= 448.
inline uint8_t e4m3_round(double v)
{
    const uint8_t sign = v < 0 ? 0x80 : 0;
    const double a = std::fabs(v) * 512.0;  // in units of 2^-9
    if (a < 7.5) {  // subnormal: nearest integer, 8 rounds up to the smallest normal
        const double r = std::nearbyint(a);
        return (uint8_t)(sign | (r >= 8.0 ? 0x08 : (uint8_t)r));
    }
    int e = 1;
    while (e < 15 && a >= 16.0 * std::ldexp(1.0, e - 1)) ++e;  // (8+m) 2^(e-1) with m < 8
    double m = std::nearbyint(a / std::ldexp(1.0, e - 1)) - 8.0;  // ties to even (FE_TONEAREST)
    if (m >= 8.0) {  // carried into the next binade
        m = 0.0;
        ++e;
    }
    if (e > 15 || (e == 15 && m > 6.0)) {  // beyond 448 (callers keep |v| <= 256)
        e = 15;
        m = 6.0;
    }
    return (uint8_t)(sign | (uint8_t)(e << 3) | (uint8_t)m);
}

// value of an E4M3 code in units of 2^-9
inline int64_t e4m3_units(uint8_t code)
{
    const int e = (code >> 3) & 15, m = code & 7;
    const int64_t a = e == 0 ? m : (int64_t)(8 + m) << (e - 1);
    return code & 0x80 ? -a : a;
}

// Split an integer number of 2^-9 units into E4M3 values that add up to it exactly, the
// largest first (each step leaves less than an eighth of the rest).  Returns the count,
// or -1 if more than `cap` pieces would be needed.
inline int e4m3_pieces(int64_t t, uint8_t *out, int cap)
{
    int n = 0;
    while (t != 0) {
        if (n == cap) return -1;
        const int64_t a = t < 0 ? -t : t;
        uint8_t code;
        if (a >= kE4M3MaxUnits) {
            code = 0x7E;  // 448
        } else if (a < 8) {
            code = (uint8_t)a;
        } else {
            int e = 1;
            while (e < 15 && a >= ((int64_t)16 << (e - 1))) ++e;
            const int64_t m = (a >> (e - 1)) - 8;  // rounded down: the piece never exceeds a
            code = (uint8_t)((e << 3) | (int)m);
        }
        if (t < 0) code |= 0x80;
        out[n++] = code;
        t -= e4m3_units(code);
    }
    return n;
}

}  // namespace

static int build_plan(blamm_ctx *ctx, int terms)
{
    // the scanned columns, sorted by length (the reference's order already is, fwd/rc interleaved)
    std::vector<int> order;
    if (ctx->active.empty()) {
        order.resize(ctx->ncols);
        for (int i = 0; i < ctx->ncols; ++i) order[i] = i;
    } else {
        order.assign(ctx->active.begin(), ctx->active.end());
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ctx->len[a] < ctx->len[b]; });
    const int nsel = (int)order.size();
    const int lmax_sel = nsel ? ctx->len[order.back()] : 1;
    if (lmax_sel > kMaxTcLen)
        return fail(ctx, BLAMM_ERR_UNSUPPORTED,
                    "motif length %d exceeds the tensor-core limit %d (use BLAMM_MODE_FP32)", lmax_sel,
                    kMaxTcLen);

    // the E4M3 form: one B term, 8 motif positions per k-step (K = 32); BF16: 4 (K = 16)
    const bool e8 = terms == kE4M3;
    const int kpos = e8 ? 8 : 4, nterm = e8 ? 1 : terms;
    if (e8 && lmax_sel > kMaxE4M3Len)
        return fail(ctx, BLAMM_ERR_UNSUPPORTED, "motif length %d exceeds the E4M3 form's limit %d", lmax_sel,
                    kMaxE4M3Len);
    const int gmax_all = std::max(1, (lmax_sel + kpos - 1) / kpos);
    const int erows_all = kBM + kpos * gmax_all + 8;
    const long long smem_limit = (long long)ctx->max_smem;
    // everything but the B tiles (E stages, bias A tile, candidate staging, ...)
    const long long other = (long long)tc_smem_layout(0u, terms, erows_all, 256).total;
    const long long b_term_cap = (smem_limit - other) / nterm;
    const int ncap = std::max(32, std::min(256, ctx->plan_nmax / 32 * 32));
    // widest tile whose B terms (g motif k-steps + 1 bias k-step) fit shared memory
    auto nmax_for = [&](int g) {
        long long n = b_term_cap / (32LL * (g + 1));
        n = n / 32 * 32;
        return (int)std::min<long long>(ncap, n);
    };
    if (nmax_for(gmax_all) < 32)
        return fail(ctx, BLAMM_ERR_UNSUPPORTED, "motif bank does not fit shared memory");

    // DP over sorted columns: tile = contiguous run of sorted columns.
    // Per-job cycle model: MMA = (terms*g + bias)*N/2, epilogue ~ N, plus a fixed cost per
    // job (hand-offs); the bias MMA is folded into the last k-step when the tile's longest
    // motif leaves that k-step's second K core unused.
    const double kInf = 1e300;
    std::vector<double> f(nsel + 1, kInf);
    std::vector<int> from(nsel + 1, -1);
    f[0] = 0.0;
    // A tile's cost depends only on its padded width N and its last (longest) column, and
    // f is non-decreasing, so for each N the tile that starts as far left as N allows is
    // the best: 8 candidates per end column instead of 256, same optimum.
    for (int j = 1; j <= nsel; ++j) {
        const int L = ctx->len[order[j - 1]];
        const int g = std::max(1, (L + kpos - 1) / kpos);
        const int bias = !e8 && bias_folds(L) ? 0 : 1;
        for (int N = 32; N <= 256; N += 32) {
            if (N > nmax_for(g)) break;
            const int i = std::max(0, j - N);
            const double mma = (nterm * g + bias) * N / 2.0, epi = 1.0 * N;
            const double cost = std::max(std::max(mma, epi), 300.0) + ctx->plan_job_cost;
            if (f[i] + cost < f[j]) {
                f[j] = f[i] + cost;
                from[j] = i;
            }
            if (i == 0) break;
        }
        if (from[j] < 0) return fail(ctx, BLAMM_ERR_UNSUPPORTED, "tile planning failed");
    }
    std::vector<std::pair<int, int>> spans;
    for (int j = nsel; j > 0; j = from[j]) spans.push_back({from[j], j});
    std::reverse(spans.begin(), spans.end());
    const int ncols = ctx->ncols;

    // per-column quantisation and guard band: computed once per bank and number of terms
    // (thresholds only move the bias), reused by every later plan (column subsets,
    // threshold sets of the scan service)
    if (!(ctx->colq_valid && ctx->colq_terms == terms)) {
        ctx->colq_k.assign(ncols, 0);
        ctx->colq_guard.assign(ncols, 0.0);
        ctx->colq_off.assign(ncols + 1, 0);
        for (int c = 0; c < ncols; ++c) ctx->colq_off[c + 1] = ctx->colq_off[c] + 4 * (uint32_t)ctx->len[c];
        ctx->colq_hi.assign(e8 ? 0 : ctx->colq_off[ncols], 0);
        ctx->colq_lo.assign(terms == 2 ? ctx->colq_off[ncols] : 0, 0);
        ctx->colq_e8.assign(e8 ? ctx->colq_off[ncols] : 0, 0);
        for (int c = 0; c < ncols; ++c) {
            const float *col = &ctx->P[(size_t)c * ctx->p_rows];
            const int L = ctx->len[c];
            // BF16: grid 2^-k with |P| <= 128 * 2^-k; E4M3: scale 2^k with max|P| 2^k in (32, 64]
            const int k = (e8 ? 6 : 7) - column_exponent(col, L);
            ctx->colq_k[c] = k;
            double eq = 0.0, a = 0.0;
            for (int j = 0; j < L; ++j) {
                double mres = 0.0, mabs = 0.0;
                for (int b = 0; b < 4; ++b) {
                    const double v = col[4 * j + b];
                    double q;
                    if (e8) {
                        const uint8_t code = e4m3_round(std::ldexp(v, k));
                        ctx->colq_e8[ctx->colq_off[c] + 4 * j + b] = code;
                        q = std::ldexp((double)e4m3_units(code), -9 - k);
                    } else {
                        const double hi = q_hi(v, k);
                        const double lo = terms == 2 ? q_lo(v - hi, k) : 0.0;
                        ctx->colq_hi[ctx->colq_off[c] + 4 * j + b] = bf16_bits_exact(hi);
                        if (terms == 2) ctx->colq_lo[ctx->colq_off[c] + 4 * j + b] = bf16_bits_exact(lo);
                        q = hi + lo;
                    }
                    // only P > q can put a reference hit below T: sum(q) = sum(P) - sum(P - q)
                    mres = std::max(mres, v - q);
                    mabs = std::max(mabs, std::fabs(v));
                }
                eq += mres;
                a += mabs;
            }
            // guard = sum_j max_b (P - q)^+ (mres starts at 0) + the bound on the reference's
            // own rounding, |fl(sequential sum) - exact sum| <= gamma_{L-1} * sum|terms|
            const double u = std::ldexp(1.0, -24);
            const double nl = std::max(0, L - 1);
            const double gamma = nl * u / (1.0 - nl * u);
            ctx->colq_guard[c] = (eq + gamma * a) * (1.0 + 1e-9) + std::ldexp(1.0, -60);
        }
        ctx->colq_terms = terms;
        ctx->colq_valid = true;
    }
    const std::vector<int> &kcol = ctx->colq_k;
    const std::vector<double> &guard_d = ctx->colq_guard;
    ctx->guard.assign(ncols, 0.0f);
    for (const int c : order) ctx->guard[c] = (float)guard_d[c];

    // tiles, slots, B buffer.  B term layout (canonical no-swizzle K-major):
    // element (column i, K index kk) of a tile with g motif k-steps sits at
    // ((i/8 * 2(g+1) + kk/8) * 8 + i%8) * 8 + kk%8.  The hi term holds the bias,
    // -T split into three BF16-exact pieces on the column's grid, in K indices
    // 16g..16g+2 (the bias MMA's k-step) or, in a folded tile, 16g-8..16g-6 (the
    // second K core of k-step g-1, which no motif of the tile reaches).  The E4M3 form
    // (1 byte per element, 16 per core row): byte ((i/8 * 2(g+1) + kk/16) * 8 + i%8) * 16
    // + kk%16, K index 4j + b for position j, base b; the bias k-step (K 32g..32g+31)
    // holds -T x 2^k (T on the grid 2^-(9+k)) as up to 32 E4M3 pieces.
    std::vector<TileDesc> tiles;
    std::vector<int32_t> slot_col;
    std::vector<uint8_t> bbuf;
    ctx->bias_T.assign(ncols, 0.0);
    int gmax = 1;
    uint32_t btmax = 0;
    int nmax = 0;
    for (auto &sp : spans) {
        const int cnt = sp.second - sp.first;
        const int L = ctx->len[order[sp.second - 1]];
        const int g = std::max(1, (L + kpos - 1) / kpos);
        const int N = (cnt + 31) / 32 * 32;
        TileDesc td{};
        td.slot0 = (int32_t)slot_col.size();
        td.n = N;
        td.g = g;
        td.b_bytes = N * 32 * (g + 1);  // 32 bytes per column and k-step in both forms
        td.fold = !e8 && bias_folds(L) ? 1 : 0;
        const int kb = td.fold ? 16 * g - 8 : 16 * g;  // K index of the first bias piece
        size_t off = (bbuf.size() + 1023) / 1024 * 1024;
        td.b_off = (int64_t)off;
        bbuf.resize(off + (size_t)td.b_bytes * nterm, 0);
        if (e8) {
            uint8_t *b8 = bbuf.data() + off;
            auto at = [&](int i, int kk) {
                return ((size_t)((i / 8) * 2 * (g + 1) + kk / 16) * 8 + i % 8) * 16 + kk % 16;
            };
            for (int i = 0; i < N; ++i) {
                const int c = i < cnt ? order[sp.first + i] : -1;
                slot_col.push_back(c);
                // T x 2^k in units of 2^-9, kept within the scores a window can reach
                // (|sum q| x 2^k <= 64 L): below it every window is a candidate, above it none
                // is (a padding column: T = 1.0, never a candidate)
                int64_t Tint = 512;
                if (c >= 0) {
                    const int k = kcol[c];
                    const double lim = (double)(64 * ctx->len[c] + 1) * 512.0;
                    const double t = ((double)ctx->thr[c] - guard_d[c]) * std::ldexp(1.0, 9 + k);
                    Tint = std::isnan(t) ? (int64_t)lim : (int64_t)std::floor(std::max(-lim, std::min(lim, t)));
                    ctx->bias_T[c] = std::ldexp((double)Tint, -9 - k);
                }
                uint8_t pcs[32];
                const int np = e4m3_pieces(-Tint, pcs, 32);
                if (np < 0) return fail(ctx, BLAMM_ERR_UNSUPPORTED, "E4M3 bias of column %d needs over 32 pieces", c);
                for (int q = 0; q < np; ++q) b8[at(i, 32 * g + q)] = pcs[q];
                if (c < 0) continue;
                const uint32_t o = ctx->colq_off[c], nk = ctx->colq_off[c + 1] - o;
                for (uint32_t kk = 0; kk < nk; ++kk) b8[at(i, (int)kk)] = ctx->colq_e8[o + kk];
            }
            tiles.push_back(td);
            gmax = std::max(gmax, g);
            btmax = std::max<uint32_t>(btmax, (uint32_t)td.b_bytes);
            nmax = std::max(nmax, N);
            continue;
        }
        uint16_t *b_hi = reinterpret_cast<uint16_t *>(bbuf.data() + off);
        uint16_t *b_lo = terms == 2 ? reinterpret_cast<uint16_t *>(bbuf.data() + off + td.b_bytes) : nullptr;
        auto elem = [&](int i, int kk) {
            return ((size_t)((i / 8) * 2 * (g + 1) + kk / 8) * 8 + i % 8) * 8 + kk % 8;
        };
        for (int i = 0; i < N; ++i) {
            const int c = i < cnt ? order[sp.first + i] : -1;
            slot_col.push_back(c);
            // bias: T on the grid u = 2^-(k+8), clamped to +-2^23 u (a padding column
            // gets T = 2^22 u at k = 0: never a candidate)
            int k = 0;
            int64_t Tint = (int64_t)1 << 22;
            if (c >= 0) {
                k = kcol[c];
                const double t = ((double)ctx->thr[c] - guard_d[c]) * std::ldexp(1.0, k + 8);
                const double lim = std::ldexp(1.0, 23);
                Tint = std::isnan(t) ? (int64_t)lim : (int64_t)std::floor(std::max(-lim, std::min(lim, t)));
                ctx->bias_T[c] = (double)Tint * std::ldexp(1.0, -(k + 8));
            }
            const int64_t pa = (int64_t)std::llround((double)Tint / 65536.0);
            const int64_t rem = Tint - pa * 65536;
            const int64_t pb = (int64_t)std::llround((double)rem / 256.0);
            const int64_t pc = rem - pb * 256;
            const int64_t pieces[3] = {pa * 65536, pb * 256, pc};
            for (int s = 0; s < 3; ++s)
                if (pieces[s] != 0) b_hi[elem(i, kb + s)] = bf16_bits_exact(-std::ldexp((double)pieces[s], -(k + 8)));
            if (c < 0) continue;
            const uint32_t o = ctx->colq_off[c], nk = ctx->colq_off[c + 1] - o;
            for (uint32_t kk = 0; kk < nk; ++kk) {
                b_hi[elem(i, (int)kk)] = ctx->colq_hi[o + kk];
                if (b_lo) b_lo[elem(i, (int)kk)] = ctx->colq_lo[o + kk];
            }
        }
        tiles.push_back(td);
        gmax = std::max(gmax, g);
        btmax = std::max<uint32_t>(btmax, (uint32_t)td.b_bytes);
        nmax = std::max(nmax, N);
    }

    // upload (buffers are reused; the copies are ordered on the context's stream)
    int rc = ensure(ctx, &ctx->d_tiles, &ctx->cap_tiles, tiles.size());
    if (!rc) rc = ensure(ctx, &ctx->d_bbuf, &ctx->cap_bbuf, bbuf.size());
    if (!rc) rc = ensure(ctx, &ctx->d_slot_col, &ctx->cap_slot_col, slot_col.size());
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->d_tiles, tiles.data(), sizeof(TileDesc) * tiles.size(), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_bbuf, bbuf.data(), bbuf.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_slot_col, slot_col.data(), sizeof(int32_t) * slot_col.size(),
                       cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));  // the host vectors go out of scope
    ctx->tiles = tiles;
    ctx->erows = kBM + kpos * gmax + 8;
    ctx->b_term_max = btmax;
    ctx->tmem_cols = 512u;  // the whole TMEM: 4 accumulators of <= 128 columns or 2 of <= 256
    ctx->acc_stages = nmax <= 128 ? 4 : 2;
    ctx->plan_terms = terms;
    ctx->plan_valid = true;
    return BLAMM_OK;
}

// ------------------------------------------------------------------ API
extern "C" {

int blamm_version(void) { return 10000; }

int blamm_ctx_create(int device, blamm_ctx **out)
{
    if (!out) return BLAMM_ERR_ARG;
    *out = nullptr;
    blamm_ctx *ctx = new blamm_ctx();
    ctx->device = device;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || device < 0 || device >= ndev) {
        delete ctx;
        return BLAMM_ERR_CUDA;
    }
    int rc = BLAMM_OK;
    auto init = [&]() -> int {
        CK(cudaSetDevice(device));
        cudaDeviceProp prop;
        CK(cudaGetDeviceProperties(&prop, device));
        if (prop.major != 10)
            return fail(ctx, BLAMM_ERR_UNSUPPORTED, "compute capability %d.%d is not sm_100-class",
                        prop.major, prop.minor);
        ctx->sm_count = prop.multiProcessorCount;
        // scan window (positions, a multiple of 128): BLAMM_SCAN_WINDOW overrides the default
        ctx->ewindow = kEWindowDefault;
        if (const char *w = std::getenv("BLAMM_SCAN_WINDOW"))
            ctx->ewindow = std::max<int64_t>(kBM, std::atoll(w) / kBM * kBM);
        ctx->max_smem = (int)prop.sharedMemPerBlockOptin;
        cudaFuncAttributes fa;
        // fails if no sm_103a image fits
        for (const void *k : {(const void *)scan_tc_kernel<false, false, 1>,
                              (const void *)scan_tc_kernel<false, false, 2>,
                              (const void *)scan_tc_kernel<true, false, 1>,
                              (const void *)scan_tc_kernel<true, false, 2>,
                              (const void *)scan_tc_kernel<false, true, 1>,
                              (const void *)scan_tc_kernel<false, true, 2>,
                              (const void *)scan_tc_kernel<false, false, kE4M3>,
                              (const void *)scan_tc_kernel<true, false, kE4M3>,
                              (const void *)scan_tc_kernel<false, true, kE4M3>}) {
            CK(cudaFuncGetAttributes(&fa, k));
            if (fa.maxThreadsPerBlock < kTcThreads)
                return fail(ctx, BLAMM_ERR_UNSUPPORTED,
                            "scan kernel: %d registers allow only %d threads per block (< %d)", fa.numRegs,
                            fa.maxThreadsPerBlock, kTcThreads);
            CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->max_smem));
        }
        CK(cudaFuncSetAttribute(scan_plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                ctx->max_smem));
        CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        for (auto &ev : ctx->ev) CK(cudaEventCreate(&ev));
        CK(cudaMalloc(&ctx->d_counters, 4 * sizeof(unsigned long long)));
        CK(cudaMalloc(&ctx->d_status, sizeof(int)));
        return BLAMM_OK;
    };
    rc = init();
    if (rc != BLAMM_OK) {
        fprintf(stderr, "blamm_ctx_create: %s\n", ctx->err.c_str());
        blamm_ctx_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return BLAMM_OK;
}

void blamm_ctx_destroy(blamm_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    void *bufs[] = {ctx->d_P,      ctx->d_len,   ctx->d_thr,      ctx->d_tiles, ctx->d_bbuf,
                    ctx->d_slot_col, ctx->d_prof, ctx->d_bases, ctx->d_seq2, ctx->d_zmask, ctx->d_e16,
                    ctx->d_runs,   ctx->d_cand,  ctx->d_hits,     ctx->d_counters, ctx->d_status,
                    ctx->d_active, ctx->d_chunk_bases[0], ctx->d_chunk_bases[1], ctx->d_chunk_runs[0],
                    ctx->d_chunk_runs[1], ctx->d_raw, ctx->d_stream, ctx->d_srun[0], ctx->d_srun[1],
                    ctx->d_srun[2], ctx->d_shdr};
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    for (void *b : bufs)
        if (b) cudaFree(b);
    for (auto &ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto &ev : ctx->chunk_ev)
        if (ev) cudaEventDestroy(ev);
    for (auto &ev : ctx->done_ev)
        if (ev) cudaEventDestroy(ev);
    for (auto &h : ctx->h_chunk_runs)
        if (h) cudaFreeHost(h);
    if (ctx->h_chunk_counts) cudaFreeHost(ctx->h_chunk_counts);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

// Device bytes of the per-call buffers (stream, packed stream, one-hot window, run table,
// candidate records, hits, pipeline chunks, resident stream); the motif bank and its plan
// are not counted.
static int64_t call_buffer_bytes(const blamm_ctx *ctx)
{
    return (int64_t)(ctx->cap_bases + 4 * ctx->cap_words32 + 4 * ctx->cap_zmask + 16 * ctx->cap_e16 +
                     8 * ctx->cap_runs + 8 * (ctx->cap_chunk_runs[0] + ctx->cap_chunk_runs[1]) +
                     ctx->cap_chunk_bases[0] + ctx->cap_chunk_bases[1] + ctx->cap_raw + ctx->cap_stream +
                     8 * (ctx->cap_srun[0] + ctx->cap_srun[1] + ctx->cap_srun[2] + ctx->cap_shdr)) +
           16 * ctx->cand_cap + (int64_t)sizeof(blamm_hit) * ctx->hits_cap;
}

int blamm_ctx_call_bytes(const blamm_ctx *ctx, int64_t *bytes)
{
    if (!ctx || !bytes) return BLAMM_ERR_ARG;
    *bytes = call_buffer_bytes(ctx);
    return BLAMM_OK;
}

int blamm_release_buffers(blamm_ctx *ctx)
{
    if (!ctx) return BLAMM_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->copy_stream) CK(cudaStreamSynchronize(ctx->copy_stream));
    auto drop = [&](auto **ptr, auto *cap) {
        if (*ptr) cudaFreeAsync(*ptr, ctx->stream);
        *ptr = nullptr;
        *cap = 0;
    };
    drop(&ctx->d_bases, &ctx->cap_bases);
    drop(&ctx->d_seq2, &ctx->cap_words32);
    drop(&ctx->d_zmask, &ctx->cap_zmask);
    drop(&ctx->d_e16, &ctx->cap_e16);
    drop(&ctx->d_runs, &ctx->cap_runs);
    for (int b = 0; b < 2; ++b) {
        drop(&ctx->d_chunk_bases[b], &ctx->cap_chunk_bases[b]);
        drop(&ctx->d_chunk_runs[b], &ctx->cap_chunk_runs[b]);
    }
    drop(&ctx->d_raw, &ctx->cap_raw);
    drop(&ctx->d_stream, &ctx->cap_stream);
    for (int k = 0; k < 3; ++k) drop(&ctx->d_srun[k], &ctx->cap_srun[k]);
    drop(&ctx->d_shdr, &ctx->cap_shdr);
    ctx->stream_n = ctx->stream_nruns = ctx->stream_nseqs = 0;
    if (ctx->d_cand) cudaFreeAsync(ctx->d_cand, ctx->stream);
    ctx->d_cand = nullptr;
    ctx->cand_cap = 0;
    if (ctx->d_hits) cudaFreeAsync(ctx->d_hits, ctx->stream);
    ctx->d_hits = nullptr;
    ctx->hits_cap = 0;
    CK(cudaStreamSynchronize(ctx->stream));
    // give the freed memory back to the device: the stream-ordered pool would keep it
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
    return BLAMM_OK;
}

const char *blamm_last_error(const blamm_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int blamm_set_mode(blamm_ctx *ctx, int mode)
{
    if (!ctx) return BLAMM_ERR_ARG;
    if (mode != BLAMM_MODE_FP32 && mode != BLAMM_MODE_BF16 && mode != BLAMM_MODE_BF16X2 && mode != BLAMM_MODE_AUTO &&
        mode != BLAMM_MODE_E4M3)
        return fail(ctx, BLAMM_ERR_ARG, "unknown mode %d", mode);
    ctx->mode = mode;
    return BLAMM_OK;
}

int blamm_set_motifs(blamm_ctx *ctx, const float *P, int p_rows, int ncols, const int32_t *col_len,
                     const float *thr)
{
    const NvtxRange nvtx_range("blamm_set_motifs");
    if (!ctx) return BLAMM_ERR_ARG;
    if (!P || !col_len || !thr || ncols <= 0 || p_rows <= 0 || p_rows % 4)
        return fail(ctx, BLAMM_ERR_ARG, "invalid motif bank arguments");
    if (ncols >= (1 << kColBits)) return fail(ctx, BLAMM_ERR_ARG, "too many motif columns");
    int lmax = 0;
    for (int c = 0; c < ncols; ++c) {
        if (col_len[c] <= 0 || 4 * col_len[c] > p_rows)
            return fail(ctx, BLAMM_ERR_ARG, "column %d: length %d does not fit %d rows", c, col_len[c],
                        p_rows);
        if (col_len[c] > kMaxMotifLen)
            return fail(ctx, BLAMM_ERR_UNSUPPORTED, "column %d: length %d > %d", c, col_len[c], kMaxMotifLen);
        lmax = std::max(lmax, (int)col_len[c]);
    }
    CK(cudaSetDevice(ctx->device));
    ctx->ncols = ncols;
    ctx->p_rows = p_rows;
    ctx->lmax = lmax;
    ctx->P.assign(P, P + (size_t)p_rows * ncols);
    ctx->len.assign(col_len, col_len + ncols);
    ctx->thr.assign(thr, thr + ncols);
    ctx->active.clear();
    ctx->colq_valid = false;
    if (ctx->d_P) cudaFree(ctx->d_P);
    if (ctx->d_len) cudaFree(ctx->d_len);
    if (ctx->d_thr) cudaFree(ctx->d_thr);
    ctx->d_P = nullptr;
    ctx->d_len = nullptr;
    ctx->d_thr = nullptr;
    CK(cudaMalloc(&ctx->d_P, sizeof(float) * ctx->P.size()));
    CK(cudaMalloc(&ctx->d_len, sizeof(int32_t) * ncols));
    CK(cudaMalloc(&ctx->d_thr, sizeof(float) * ncols));
    CK(cudaMemcpy(ctx->d_P, ctx->P.data(), sizeof(float) * ctx->P.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_len, ctx->len.data(), sizeof(int32_t) * ncols, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_thr, ctx->thr.data(), sizeof(float) * ncols, cudaMemcpyHostToDevice));
    ctx->plan_valid = false;
    return BLAMM_OK;
}

int blamm_set_columns(blamm_ctx *ctx, const int32_t *cols, int n)
{
    if (!ctx || n < 0 || (n > 0 && !cols)) return BLAMM_ERR_ARG;
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "no motif bank");
    if (n > ctx->ncols) return fail(ctx, BLAMM_ERR_ARG, "%d columns > bank size %d", n, ctx->ncols);
    std::vector<int32_t> act;
    if (n > 0) {
        std::vector<char> seen(ctx->ncols, 0);
        act.reserve(n);
        for (int i = 0; i < n; ++i) {
            const int c = cols[i];
            if (c < 0 || c >= ctx->ncols) return fail(ctx, BLAMM_ERR_ARG, "column %d is not in the bank", c);
            if (seen[c]) return fail(ctx, BLAMM_ERR_ARG, "column %d is listed twice", c);
            seen[c] = 1;
            act.push_back(c);
        }
    }
    CK(cudaSetDevice(ctx->device));
    ctx->active.swap(act);
    if (!ctx->active.empty()) {
        int rc = ensure(ctx, &ctx->d_active, &ctx->cap_active, ctx->active.size());
        if (rc) return rc;
        CK(cudaMemcpyAsync(ctx->d_active, ctx->active.data(), sizeof(int32_t) * ctx->active.size(),
                           cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    ctx->plan_valid = false;
    return BLAMM_OK;
}

int blamm_set_thresholds(blamm_ctx *ctx, const float *thr)
{
    if (!ctx || !thr) return BLAMM_ERR_ARG;
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "no motif bank");
    CK(cudaSetDevice(ctx->device));
    ctx->thr.assign(thr, thr + ctx->ncols);
    CK(cudaMemcpy(ctx->d_thr, ctx->thr.data(), sizeof(float) * ctx->ncols, cudaMemcpyHostToDevice));
    ctx->plan_valid = false;
    return BLAMM_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ drivers
// BF16 terms of the tensor-core modes
static int mode_terms(const blamm_ctx *ctx)
{
    return ctx->mode == BLAMM_MODE_BF16X2 ? 2
           : ctx->mode == BLAMM_MODE_E4M3  ? kE4M3
           : ctx->mode == BLAMM_MODE_AUTO  ? ctx->auto_terms
                                           : 1;
}

static int ensure_plan(blamm_ctx *ctx)
{
    const int terms = mode_terms(ctx);
    if (ctx->plan_valid && ctx->plan_terms == terms) return BLAMM_OK;
    return build_plan(ctx, terms);
}

// The tensor-core scan runs over windows of at most ctx->ewindow positions (16 Mi by
// default): per window the one-hot entries of its positions (e16_kernel or e8_kernel, 16 B
// each) and one scan launch, so the entry array holds one window (256 MB) whatever the stream
// length.  A window's scan reads up to entry (its positions) + 127 + 4 * 64 + 2 (BF16) or
// + 127 + 8 * 32 + 3 (E4M3), and the entry kernels read up to base i + 3 of the padded
// stream: entries = positions + kStreamPad - 64 stay inside both.
static int64_t e16_entries(const blamm_ctx *ctx, int64_t n) { return std::min(n, ctx->ewindow) + kStreamPad - 64; }

static int launch_pack(blamm_ctx *ctx, const char *d_bases, int64_t n)
{
    const int64_t nwords32 = (n + kStreamPad + 31) / 32;
    int rc = ensure(ctx, &ctx->d_seq2, &ctx->cap_words32, (size_t)(2 * nwords32));
    if (rc) return rc;
    rc = ensure(ctx, &ctx->d_zmask, &ctx->cap_zmask, (size_t)nwords32);
    if (rc) return rc;
    const int threads = 256;
    const int64_t blocks = (nwords32 + threads - 1) / threads;
    pack_kernel<<<(unsigned)blocks, threads, 0, ctx->stream>>>(d_bases, n, ctx->d_seq2, ctx->d_zmask,
                                                               nwords32, ctx->lower_scores);
    CK(cudaGetLastError());
    if (ctx->mode != BLAMM_MODE_FP32) {
        rc = ensure(ctx, &ctx->d_e16, &ctx->cap_e16, (size_t)e16_entries(ctx, n));
        if (rc) return rc;
    }
    return BLAMM_OK;
}

// Kernel parameters of the current plan over a packed stream of n positions
// (the caller adds candidates, counters, status and the test hooks).
static TcParams tc_params(const blamm_ctx *ctx, int64_t n)
{
    TcParams p{};
    p.n = n;
    p.n_mtiles = (n + kBM - 1) / kBM;
    p.tiles = ctx->d_tiles;
    p.ntiles = (int32_t)ctx->tiles.size();
    p.terms = ctx->plan_terms;
    p.bbuf = ctx->d_bbuf;
    p.slot_col = ctx->d_slot_col;
    p.erows = ctx->erows;
    p.b_term_max = ctx->b_term_max;
    p.tmem_cols = ctx->tmem_cols;
    p.acc_stages = ctx->acc_stages;
    p.wait_limit = ctx->wait_limit;
    p.dump_ncols = ctx->ncols;
    return p;
}

// The scan kernel counts jobs and record slots in 32 bits.
constexpr int64_t kMaxJobs = 0x7fffffff;
constexpr int64_t kMaxRecordSlots = (int64_t(1) << 31) - 1024;

static int check_jobs(blamm_ctx *ctx, long long njobs)
{
    return njobs > kMaxJobs ? fail(ctx, BLAMM_ERR_UNSUPPORTED,
                                   "%lld scan jobs (tiles x 128-position blocks) exceed one launch's %lld; "
                                   "scan the stream in parts", njobs, (long long)kMaxJobs)
                            : BLAMM_OK;
}

// Record slots a scan with this grid reserves beyond its records: every drain warp holds
// one block it fills and one reserved ahead.
static int64_t record_slots_reserved(int grid) { return (int64_t)grid * kEpiWarps * 2 * kRecBlock; }

// Record slots for a first scan of n positions (about one candidate per 1000 position x
// column pairs, the thresholds' p-values being small) on a full grid.
static int64_t record_slots_guess(const blamm_ctx *ctx, int64_t n, double per = 1000.0)
{
    const double est = (double)n * scanned_columns(ctx) / per + (double)record_slots_reserved(ctx->sm_count);
    return (int64_t)std::min(std::max(est, (double)(1 << 20)), 512.0 * 1024 * 1024);
}

// Rescoring of the candidate records of one scan: the context's bank and chunk filter.
static RescoreParams rescore_params(const blamm_ctx *ctx, const uint4 *cand, const unsigned long long *cand_count,
                                    int64_t cand_cap, const uint32_t *seq2,
                                    const uint32_t *zmask, int64_t n, const int64_t *d_runs, int64_t nruns,
                                    blamm_hit *d_hits, unsigned long long *hit_count, int64_t hit_cap)
{
    RescoreParams r{};
    r.cand = cand;
    r.slot_col = ctx->d_slot_col;
    r.cand_count = cand_count;
    r.cand_cap = cand_cap;
    r.seq2 = seq2;
    r.zmask = zmask;
    r.n = n;
    r.run_start = d_runs;
    r.nruns = nruns;
    r.P = ctx->d_P;
    r.p_rows = ctx->p_rows;
    r.col_len = ctx->d_len;
    r.thr = ctx->d_thr;
    r.hits = d_hits;
    r.hit_count = hit_count;
    r.hit_cap = hit_cap;
    r.keep_below = ctx->keep_below;
    r.pos_base = ctx->pos_base;
    return r;
}

// One launch of the scan kernel instance that p asks for.
template <bool kDump, bool kProf>
static void launch_tc_as(const TcParams &p, int grid, uint32_t smem, cudaStream_t st)
{
    if (p.terms == 2) scan_tc_kernel<kDump, kProf, 2><<<grid, kTcThreads, smem, st>>>(p);
    else if (p.terms == kE4M3) scan_tc_kernel<kDump, kProf, kE4M3><<<grid, kTcThreads, smem, st>>>(p);
    else scan_tc_kernel<kDump, kProf, 1><<<grid, kTcThreads, smem, st>>>(p);
}

static void launch_tc(const TcParams &p, bool dump, int grid, uint32_t smem, cudaStream_t st)
{
    if (dump) launch_tc_as<true, false>(p, grid, smem, st);
    else if (p.prof) launch_tc_as<false, true>(p, grid, smem, st);
    else launch_tc_as<false, false>(p, grid, smem, st);
}

// The scan of n positions of a packed stream (p: the plan, candidates, counters, status),
// window by window: the window's one-hot entries into e16, then its scan launch.  Returns the
// largest grid used; adds the launches to *launches.
static int launch_tc_windows(blamm_ctx *ctx, TcParams p, const uint32_t *seq2, const uint32_t *zmask, uint4 *e16,
                             int64_t n, bool dump, uint32_t smem, int *launches, int *grid_out)
{
    const int64_t n_mtiles = (n + kBM - 1) / kBM, wt = std::max<int64_t>(1, ctx->ewindow / kBM);
    int gmax = 0;
    for (int64_t m0 = 0; m0 < n_mtiles; m0 += wt) {
        const int64_t mt = std::min(wt, n_mtiles - m0), base = m0 * kBM;
        const int64_t ne = std::min(mt * kBM, n - base) + kStreamPad - 64;
        if (p.terms == kE4M3) e8_kernel<<<(unsigned)((ne + 255) / 256), 256, 0, ctx->stream>>>(seq2, zmask, base, ne, e16);
        else e16_kernel<<<(unsigned)((ne + 255) / 256), 256, 0, ctx->stream>>>(seq2, zmask, base, ne, e16);
        CK(cudaGetLastError());
        p.e16 = e16;
        p.n_mtiles = mt;
        p.m0 = (int32_t)m0;
        const int grid = (int)std::min<long long>(ctx->sm_count, (long long)ctx->tiles.size() * mt);
        launch_tc(p, dump, grid, smem, ctx->stream);
        CK(cudaGetLastError());
        gmax = std::max(gmax, grid);
        if (launches) *launches += 2;
    }
    if (grid_out) *grid_out = gmax;
    return BLAMM_OK;
}

// tcgen05 scan + rescoring; candidates buffer grows (and the scan re-runs) on overflow
static int run_tc(blamm_ctx *ctx, int64_t n, const int64_t *d_runs, int64_t nruns, blamm_hit *d_hits,
                  int64_t hit_cap, float *dump, int64_t dump_p0, int64_t dump_npos, int *launches)
{
    int rc = ensure_plan(ctx);
    if (rc) return rc;
    const int64_t n_mtiles = (n + kBM - 1) / kBM;
    const long long njobs = (long long)ctx->tiles.size() * n_mtiles;
    if ((rc = check_jobs(ctx, njobs))) return rc;
    if (ctx->cand_cap == 0) {
        size_t cap = 0;
        rc = ensure(ctx, &ctx->d_cand, &cap, (size_t)record_slots_guess(ctx, n));
        if (rc) return rc;
        ctx->cand_cap = (int64_t)cap;
    }
    const TcSmem L = tc_smem_layout(ctx->b_term_max, ctx->plan_terms, ctx->erows,
                                    (int)ctx->tiles.size());
    if ((int)L.total > ctx->max_smem)
        return fail(ctx, BLAMM_ERR_UNSUPPORTED, "shared memory plan %u > %d", L.total, ctx->max_smem);
    // at least ~116 KB so that two CTAs never share an SM (each allocates TMEM)
    const uint32_t smem = std::max<uint32_t>(L.total, 116 * 1024);
    for (int attempt = 0; attempt < 3; ++attempt) {
        CK(cudaMemsetAsync(ctx->d_counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
        TcParams p = tc_params(ctx, n);
        p.cand = ctx->d_cand;
        p.cand_count = ctx->d_counters;
        p.ncand = ctx->d_counters + 3;
        p.cand_cap = ctx->cand_cap;
        p.status = ctx->d_status;
        p.wait_limit = ctx->wait_limit;
        p.debug_stall = ctx->debug_stall;
        p.dump = dump;
        p.dump_p0 = dump_p0;
        p.dump_npos = dump_npos;
        p.dump_ncols = ctx->ncols;
        p.prof = nullptr;
        if (ctx->prof_on) {
            if (!ctx->d_prof) CK(cudaMalloc(&ctx->d_prof, sizeof(long long) * 32 * ctx->sm_count));
            CK(cudaMemsetAsync(ctx->d_prof, 0, sizeof(long long) * 32 * ctx->sm_count, ctx->stream));
            p.prof = ctx->d_prof;
        }
        int grid = 0;
        if (njobs > 0) {
            CK(cudaEventRecord(ctx->ev[4], ctx->stream));
            if ((rc = launch_tc_windows(ctx, p, ctx->d_seq2, ctx->d_zmask, ctx->d_e16, n, dump != nullptr, smem,
                                        launches, &grid)))
                return rc;
            CK(cudaEventRecord(ctx->ev[5], ctx->stream));
        }
        unsigned long long ncand = 0;
        int status = 0;
        CK(cudaMemcpyAsync(&ncand, ctx->d_counters, sizeof ncand, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(&status, ctx->d_status, sizeof status, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if (status) return fail(ctx, BLAMM_ERR_TIMEOUT, "scan kernel: a device wait timed out");
        if (njobs > 0) cudaEventElapsedTime(&ctx->stats.scan_ms, ctx->ev[4], ctx->ev[5]);
        if (ctx->prof_on && njobs > 0) {
            ctx->prof.resize((size_t)32 * grid);
            CK(cudaMemcpy(ctx->prof.data(), ctx->d_prof, sizeof(long long) * 32 * grid, cudaMemcpyDeviceToHost));
            ctx->prof_ctas = grid;
        }
        ctx->stats.candidates = 0;  // counted by the rescoring
        ctx->rec_slots = (int64_t)ncand;
        if ((int64_t)ncand <= ctx->cand_cap) break;
        // grow and re-run
        size_t cap = 0;
        CK(cudaFreeAsync(ctx->d_cand, ctx->stream));
        ctx->d_cand = nullptr;
        ctx->cand_cap = 0;
        if ((int64_t)ncand >= kMaxRecordSlots)
            return fail(ctx, BLAMM_ERR_OVERFLOW, "%llu candidate records exceed one launch's %lld", ncand,
                        (long long)kMaxRecordSlots);
        rc = ensure(ctx, &ctx->d_cand, &cap,
                    (size_t)std::min<int64_t>((int64_t)(ncand + ncand / 4 + 1024), kMaxRecordSlots));
        if (rc) return rc;
        ctx->cand_cap = (int64_t)cap;
        if (attempt == 2) return fail(ctx, BLAMM_ERR_OVERFLOW, "candidate buffer overflow");
    }
    const RescoreParams r = rescore_params(ctx, ctx->d_cand, ctx->d_counters, ctx->cand_cap,
                                           ctx->d_seq2, ctx->d_zmask, n, d_runs, nruns, d_hits,
                                           ctx->d_counters + 1, hit_cap);
    const int64_t nc = ctx->rec_slots;
    if (nc > 0) {
        const int threads = 256;
        const int64_t blocks = std::min<int64_t>((nc + threads - 1) / threads, (int64_t)ctx->sm_count * 16);
        CK(cudaEventRecord(ctx->ev[6], ctx->stream));
        rescore_kernel<<<(unsigned)blocks, threads, 0, ctx->stream>>>(r);
        CK(cudaGetLastError());
        CK(cudaEventRecord(ctx->ev[7], ctx->stream));
        ctx->rescore_timed = true;
        ++*launches;
    }
    return BLAMM_OK;
}

// The plain FP32 scan of n positions of the packed stream (seq2/zmask) on the context's
// stream: parameters of the current bank and columns, hits appended through hit_count.
static PlainParams plain_params(const blamm_ctx *ctx, const uint32_t *seq2, const uint32_t *zmask, int64_t n,
                                const int64_t *d_runs, int64_t nruns, blamm_hit *d_hits, int64_t hit_cap,
                                unsigned long long *hit_count)
{
    PlainParams p{};
    p.seq2 = seq2;
    p.zmask = zmask;
    p.n = n;
    p.run_start = d_runs;
    p.nruns = nruns;
    p.P = ctx->d_P;
    p.p_rows = ctx->p_rows;
    p.ncols = scanned_columns(ctx);
    p.lmax = ctx->lmax;
    p.col_len = ctx->d_len;
    p.thr = ctx->d_thr;
    p.cols = ctx->active.empty() ? nullptr : ctx->d_active;
    p.hits = d_hits;
    p.hit_count = hit_count;
    p.hit_cap = hit_cap;
    p.keep_below = ctx->keep_below;
    p.pos_base = ctx->pos_base;
    return p;
}

// Launch it: a block's columns staged in shared memory (as many as fit, at most 32).
static int launch_plain(blamm_ctx *ctx, PlainParams &p)
{
    const int threads = 256;
    int cpb = 32;
    while (cpb > 1 && (size_t)cpb * (p.p_rows + 2) * 4 + threads + p.lmax + 64 > (size_t)ctx->max_smem) cpb /= 2;
    p.cols_per_block = cpb;
    const size_t smem = (size_t)cpb * (p.p_rows + 2) * 4 + threads + p.lmax + 64;
    const int64_t bx = (p.n + threads - 1) / threads;
    const int by = (p.ncols + cpb - 1) / cpb;
    if (bx > 0x7fffffff || by > 65535) return fail(ctx, BLAMM_ERR_UNSUPPORTED, "grid too large");
    if (bx > 0) {
        scan_plain_kernel<<<dim3((unsigned)bx, (unsigned)by), threads, smem, ctx->stream>>>(p);
        CK(cudaGetLastError());
    }
    return BLAMM_OK;
}

static int run_plain(blamm_ctx *ctx, int64_t n, const int64_t *d_runs, int64_t nruns, blamm_hit *d_hits,
                     int64_t hit_cap, int *launches)
{
    CK(cudaMemsetAsync(ctx->d_counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
    PlainParams p = plain_params(ctx, ctx->d_seq2, ctx->d_zmask, n, d_runs, nruns, d_hits, hit_cap,
                                 ctx->d_counters + 1);
    if (n == 0) return BLAMM_OK;
    CK(cudaEventRecord(ctx->ev[4], ctx->stream));
    const int rc = launch_plain(ctx, p);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->ev[5], ctx->stream));
    ctx->plain_timed = true;
    ++*launches;
    return BLAMM_OK;
}

static int scan_core(blamm_ctx *ctx, const char *d_bases, int64_t n, const int64_t *d_runs, int64_t nruns,
                     blamm_hit *d_hits, int64_t hit_cap, int64_t *n_hits)
{
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "blamm_set_motifs was not called");
    int launches = 0;
    ctx->stats = blamm_stats{};
    ctx->plain_timed = ctx->rescore_timed = false;
    ctx->stats.positions = n;
    ctx->stats.columns = scanned_columns(ctx);
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    int rc = launch_pack(ctx, d_bases, n);
    if (rc) return rc;
    launches += 1;  // packing (the tensor-core scan adds its windows' one-hot entries)
    if (ctx->mode == BLAMM_MODE_FP32) rc = run_plain(ctx, n, d_runs, nruns, d_hits, hit_cap, &launches);
    else rc = run_tc(ctx, n, d_runs, nruns, d_hits, hit_cap, nullptr, 0, 0, &launches);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    unsigned long long cnt[4] = {0, 0, 0, 0};  // record slots, hits, -, candidates
    CK(cudaMemcpyAsync(cnt, ctx->d_counters, sizeof cnt, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const unsigned long long nh = cnt[1];
    if (ctx->mode != BLAMM_MODE_FP32) ctx->stats.candidates = (int64_t)cnt[3];
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
    ctx->stats.kernel_ms = ms;
    if (ctx->plain_timed) cudaEventElapsedTime(&ctx->stats.scan_ms, ctx->ev[4], ctx->ev[5]);
    if (ctx->rescore_timed) cudaEventElapsedTime(&ctx->stats.rescore_ms, ctx->ev[6], ctx->ev[7]);
    ctx->stats.hits = (int64_t)nh;
    ctx->stats.tiles = (int32_t)(ctx->mode == BLAMM_MODE_FP32 ? 0 : ctx->tiles.size());
    ctx->stats.launches = launches;
    *n_hits = (int64_t)nh;
    return (int64_t)nh > hit_cap ? fail(ctx, BLAMM_ERR_OVERFLOW, "%lld hits > capacity %lld",
                                        (long long)nh, (long long)hit_cap)
                                 : BLAMM_OK;
}

extern "C" {

int blamm_scan_device(blamm_ctx *ctx, const char *d_bases, int64_t n, const int64_t *d_run_start,
                      int64_t nruns, blamm_hit *d_hits, int64_t hit_cap, int64_t *n_hits)
{
    const NvtxRange nvtx_range("blamm_scan_device");
    if (!ctx || !n_hits || n < 0 || hit_cap < 0) return BLAMM_ERR_ARG;
    *n_hits = 0;
    if (n == 0) return BLAMM_OK;
    if (!d_bases || !d_run_start || nruns <= 0 || (hit_cap > 0 && !d_hits))
        return fail(ctx, BLAMM_ERR_ARG, "null buffer");
    CK(cudaSetDevice(ctx->device));
    return scan_core(ctx, d_bases, n, d_run_start, nruns, d_hits, hit_cap, n_hits);
}

// blamm_scan on a long stream: chunks of kPipeChunk positions (plus the longest motif - 1
// bases of overlap, whose window starts belong to the next chunk), each chunk's bases
// copied in on a second stream while the previous chunk is scanned, and its hits copied
// out there while the next one is scanned.
constexpr int64_t kPipeChunk = int64_t(16) << 20;

static int scan_host_pipelined_steps(blamm_ctx *ctx, const char *bases, int64_t n, const int64_t *run_start,
                                     int64_t nruns, blamm_hit *hits, int64_t hit_cap, int64_t *n_hits)
{
    const int64_t ov = std::max(ctx->lmax - 1, 0);
    const int64_t nchunks = (n + kPipeChunk - 1) / kPipeChunk;
    int rc = BLAMM_OK;
    for (int b = 0; b < 2; ++b) {
        if ((rc = ensure(ctx, &ctx->d_chunk_bases[b], &ctx->cap_chunk_bases[b], (size_t)(kPipeChunk + ov))))
            return rc;
        if ((rc = ensure(ctx, &ctx->d_chunk_runs[b], &ctx->cap_chunk_runs[b], (size_t)nruns + 1))) return rc;
    }
    size_t hc = (size_t)ctx->hits_cap;
    if ((rc = ensure(ctx, &ctx->d_hits, &hc, (size_t)std::max<int64_t>(hit_cap, 1)))) return rc;
    ctx->hits_cap = (int64_t)hc;
    if (!ctx->copy_stream) {
        CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        for (auto &ev : ctx->chunk_ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    CK(cudaStreamSynchronize(ctx->stream));  // the buffers exist before the copy stream uses them
    if (ctx->cap_h_chunk_runs < (size_t)nruns + 1) {
        for (auto &h : ctx->h_chunk_runs) {
            if (h) CK(cudaFreeHost(h));
            h = nullptr;
        }
        ctx->cap_h_chunk_runs = 0;
        for (auto &h : ctx->h_chunk_runs) CK(cudaHostAlloc((void **)&h, sizeof(int64_t) * ((size_t)nruns + 1), 0));
        ctx->cap_h_chunk_runs = (size_t)nruns + 1;
    }
    int64_t kruns[2] = {0, 0};  // per buffer: run starts of its chunk (in h_chunk_runs)
    auto issue_in = [&](int64_t k) -> int {
        const int b = (int)(k & 1);
        const int64_t c0 = k * kPipeChunk, end = std::min(n, c0 + kPipeChunk + ov);
        int64_t *hr = ctx->h_chunk_runs[b];  // its previous copy (chunk k - 2) has landed
        int64_t m = 0;
        hr[m++] = 0;  // c0 lies inside some run
        for (const int64_t *r = std::upper_bound(run_start, run_start + nruns, c0); r < run_start + nruns && *r < end;
             ++r)
            hr[m++] = *r - c0;
        kruns[b] = m;
        CK(cudaMemcpyAsync(ctx->d_chunk_bases[b], bases + c0, (size_t)(end - c0), cudaMemcpyHostToDevice,
                           ctx->copy_stream));
        CK(cudaMemcpyAsync(ctx->d_chunk_runs[b], hr, sizeof(int64_t) * (size_t)m, cudaMemcpyHostToDevice,
                           ctx->copy_stream));
        CK(cudaEventRecord(ctx->chunk_ev[b], ctx->copy_stream));
        return BLAMM_OK;
    };
    blamm_stats total{};
    total.positions = n;
    int64_t nh_total = 0;
    if ((rc = issue_in(0))) return rc;
    for (int64_t k = 0; k < nchunks; ++k) {
        const int b = (int)(k & 1);
        // the next chunk's input buffer served chunk k - 1, whose scan has returned
        if (k + 1 < nchunks && (rc = issue_in(k + 1))) return rc;
        CK(cudaStreamWaitEvent(ctx->stream, ctx->chunk_ev[b], 0));
        const int64_t c0 = k * kPipeChunk, c1 = std::min(n, c0 + kPipeChunk), end = std::min(n, c1 + ov);
        ctx->keep_below = end > c1 ? c1 - c0 : 0;
        ctx->pos_base = c0;
        const int64_t at = std::min(nh_total, hit_cap), cap_k = hit_cap - at;
        int64_t nh = 0;
        rc = scan_core(ctx, ctx->d_chunk_bases[b], end - c0, ctx->d_chunk_runs[b], kruns[b], ctx->d_hits + at,
                       cap_k, &nh);
        if (rc && rc != BLAMM_ERR_OVERFLOW) return rc;
        // scan_core returned after its stream drained: copy this chunk's hits out beside the next scan
        const int64_t ncopy = std::min(nh, cap_k);
        if (ncopy > 0)
            CK(cudaMemcpyAsync(hits + at, ctx->d_hits + at, sizeof(blamm_hit) * ncopy, cudaMemcpyDeviceToHost,
                               ctx->copy_stream));
        nh_total += nh;
        total.columns = ctx->stats.columns;
        total.candidates += ctx->stats.candidates;
        total.tiles = ctx->stats.tiles;
        total.launches += ctx->stats.launches;
        total.kernel_ms += ctx->stats.kernel_ms;
        total.scan_ms += ctx->stats.scan_ms;
        total.rescore_ms += ctx->stats.rescore_ms;
    }
    CK(cudaStreamSynchronize(ctx->copy_stream));  // the hits are in host memory
    total.hits = nh_total;
    ctx->stats = total;
    *n_hits = nh_total;
    return nh_total > hit_cap
               ? fail(ctx, BLAMM_ERR_OVERFLOW, "%lld hits > capacity %lld", (long long)nh_total, (long long)hit_cap)
               : BLAMM_OK;
}

// One chunk's kernels, enqueued without host synchronisation (the blamm_scan_enqueue
// sequence): candidates beyond the candidate buffer are only counted, and the rescoring
// reads their number on the device.
static int enqueue_chunk(blamm_ctx *ctx, const char *d_bases, int64_t n, const int64_t *d_runs, int64_t nruns,
                         blamm_hit *d_hits, int64_t hit_cap)
{
    unsigned long long *cnt = ctx->d_counters;  // [0] candidates of this chunk, [1] hits of the call
    const int64_t nwords32 = (n + kStreamPad + 31) / 32;
    pack_kernel<<<(unsigned)((nwords32 + 255) / 256), 256, 0, ctx->stream>>>(d_bases, n, ctx->d_seq2, ctx->d_zmask,
                                                                          nwords32, ctx->lower_scores);
    CK(cudaGetLastError());
    if (ctx->mode == BLAMM_MODE_FP32) {
        PlainParams p = plain_params(ctx, ctx->d_seq2, ctx->d_zmask, n, d_runs, nruns, d_hits, hit_cap, cnt + 1);
        return launch_plain(ctx, p);
    }
    CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), ctx->stream));      // record slots of this chunk
    CK(cudaMemsetAsync(cnt + 3, 0, sizeof(unsigned long long), ctx->stream));  // its candidates
    const int64_t n_mtiles = (n + kBM - 1) / kBM;
    const long long njobs = (long long)ctx->tiles.size() * n_mtiles;
    int rc = check_jobs(ctx, njobs);
    if (rc) return rc;
    const TcSmem L = tc_smem_layout(ctx->b_term_max, ctx->plan_terms, ctx->erows, (int)ctx->tiles.size());
    if ((int)L.total > ctx->max_smem)
        return fail(ctx, BLAMM_ERR_UNSUPPORTED, "shared memory plan %u > %d", L.total, ctx->max_smem);
    TcParams p = tc_params(ctx, n);
    p.cand = ctx->d_cand;
    p.cand_count = cnt;
    p.ncand = cnt + 3;
    p.cand_cap = ctx->cand_cap;
    p.status = ctx->d_status;
    p.wait_limit = ctx->wait_limit;
    p.dump_ncols = ctx->ncols;
    if ((rc = launch_tc_windows(ctx, p, ctx->d_seq2, ctx->d_zmask, ctx->d_e16, n, false,
                                std::max<uint32_t>(L.total, 116 * 1024), nullptr, nullptr)))
        return rc;
    const RescoreParams r = rescore_params(ctx, ctx->d_cand, cnt, ctx->cand_cap, ctx->d_seq2, ctx->d_zmask,
                                           n, d_runs, nruns, d_hits, cnt + 1, hit_cap);
    rescore_kernel<<<(unsigned)(ctx->sm_count * 8), 256, 0, ctx->stream>>>(r);
    CK(cudaGetLastError());
    return BLAMM_OK;
}

// The copy pipeline without host synchronisation inside a chunk: the host only waits for
// chunk k - 1 to finish (while chunk k runs) to learn how many hits to copy out.  Returns
// BLAMM_ERR_OVERFLOW with *cand_overflow set when a chunk had more candidates than the
// candidate buffer holds (its hits are then incomplete: the caller rescans).
static int scan_host_async_steps(blamm_ctx *ctx, const char *bases, int64_t n, const int64_t *run_start,
                                 int64_t nruns, blamm_hit *hits, int64_t hit_cap, int64_t *n_hits,
                                 int64_t *cand_overflow)
{
    *cand_overflow = 0;
    const int64_t ov = std::max(ctx->lmax - 1, 0);
    const int64_t nchunks = (n + kPipeChunk - 1) / kPipeChunk;
    const int64_t span = kPipeChunk + ov;  // positions of the longest chunk
    const bool tc = ctx->mode != BLAMM_MODE_FP32;
    int rc = BLAMM_OK;
    for (int b = 0; b < 2; ++b) {
        if ((rc = ensure(ctx, &ctx->d_chunk_bases[b], &ctx->cap_chunk_bases[b], (size_t)span))) return rc;
        if ((rc = ensure(ctx, &ctx->d_chunk_runs[b], &ctx->cap_chunk_runs[b], (size_t)nruns + 1))) return rc;
    }
    const int64_t nwords32 = (span + kStreamPad + 31) / 32;
    if ((rc = ensure(ctx, &ctx->d_seq2, &ctx->cap_words32, (size_t)(2 * nwords32)))) return rc;
    if ((rc = ensure(ctx, &ctx->d_zmask, &ctx->cap_zmask, (size_t)nwords32))) return rc;
    if (tc) {
        if ((rc = ensure_plan(ctx))) return rc;
        if ((rc = ensure(ctx, &ctx->d_e16, &ctx->cap_e16, (size_t)e16_entries(ctx, span)))) return rc;
        // candidates: four times the usual first guess for a chunk (a chunk that still
        // overflows sends the whole call to the synchronous path)
        const double want = (double)record_slots_guess(ctx, span, 250.0);
        if ((double)ctx->cand_cap < want) {
            size_t cap = ctx->cand_cap > 0 ? (size_t)ctx->cand_cap : 0;
            if ((rc = ensure(ctx, &ctx->d_cand, &cap, (size_t)want))) return rc;
            ctx->cand_cap = (int64_t)cap;
        }
    }
    size_t hc = (size_t)ctx->hits_cap;
    if ((rc = ensure(ctx, &ctx->d_hits, &hc, (size_t)std::max<int64_t>(hit_cap, 1)))) return rc;
    ctx->hits_cap = (int64_t)hc;
    if (!ctx->copy_stream) {
        CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        for (auto &ev : ctx->chunk_ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    if (!ctx->done_ev[0])
        for (auto &ev : ctx->done_ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    if (ctx->cap_h_chunk_runs < (size_t)nruns + 1) {
        for (auto &h : ctx->h_chunk_runs) {
            if (h) CK(cudaFreeHost(h));
            h = nullptr;
        }
        ctx->cap_h_chunk_runs = 0;
        for (auto &h : ctx->h_chunk_runs) CK(cudaHostAlloc((void **)&h, sizeof(int64_t) * ((size_t)nruns + 1), 0));
        ctx->cap_h_chunk_runs = (size_t)nruns + 1;
    }
    if (ctx->cap_h_chunk_counts < (size_t)(4 * nchunks)) {
        if (ctx->h_chunk_counts) CK(cudaFreeHost(ctx->h_chunk_counts));
        ctx->h_chunk_counts = nullptr;
        ctx->cap_h_chunk_counts = 0;
        CK(cudaHostAlloc((void **)&ctx->h_chunk_counts, sizeof(unsigned long long) * 4 * (size_t)nchunks, 0));
        ctx->cap_h_chunk_counts = (size_t)(4 * nchunks);
    }
    CK(cudaMemsetAsync(ctx->d_counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));  // the buffers exist before the copy stream uses them
    int64_t kruns[2] = {0, 0};
    auto issue_in = [&](int64_t k) -> int {
        const int b = (int)(k & 1);
        const int64_t c0 = k * kPipeChunk, end = std::min(n, c0 + kPipeChunk + ov);
        // the staging and device buffers served chunk k - 2: its run copy has landed, and the
        // copy stream waits for its kernels (packing reads the bases, the scans the runs)
        if (k >= 2) {
            CK(cudaEventSynchronize(ctx->chunk_ev[b]));
            CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->done_ev[b], 0));
        }
        int64_t *hr = ctx->h_chunk_runs[b];
        int64_t m = 0;
        hr[m++] = 0;  // c0 lies inside some run
        for (const int64_t *r = std::upper_bound(run_start, run_start + nruns, c0); r < run_start + nruns && *r < end;
             ++r)
            hr[m++] = *r - c0;
        kruns[b] = m;
        CK(cudaMemcpyAsync(ctx->d_chunk_bases[b], bases + c0, (size_t)(end - c0), cudaMemcpyHostToDevice,
                           ctx->copy_stream));
        CK(cudaMemcpyAsync(ctx->d_chunk_runs[b], hr, sizeof(int64_t) * (size_t)m, cudaMemcpyHostToDevice,
                           ctx->copy_stream));
        CK(cudaEventRecord(ctx->chunk_ev[b], ctx->copy_stream));
        return BLAMM_OK;
    };
    unsigned long long *hc_k = ctx->h_chunk_counts;
    int64_t copied = 0;  // hits already sent to host memory
    // copy out the hits chunk k added, once it has finished (the host waits for that chunk)
    auto drain_out = [&](int64_t k) -> int {
        CK(cudaEventSynchronize(ctx->done_ev[k & 1]));
        const int64_t upto = std::min<int64_t>((int64_t)hc_k[4 * k + 1], hit_cap);
        if (upto > copied) {
            CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->done_ev[k & 1], 0));
            CK(cudaMemcpyAsync(hits + copied, ctx->d_hits + copied, sizeof(blamm_hit) * (size_t)(upto - copied),
                               cudaMemcpyDeviceToHost, ctx->copy_stream));
            copied = upto;
        }
        return BLAMM_OK;
    };
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    if ((rc = issue_in(0))) return rc;
    for (int64_t k = 0; k < nchunks; ++k) {
        const int b = (int)(k & 1);
        if (k + 1 < nchunks && (rc = issue_in(k + 1))) return rc;
        CK(cudaStreamWaitEvent(ctx->stream, ctx->chunk_ev[b], 0));
        const int64_t c0 = k * kPipeChunk, c1 = std::min(n, c0 + kPipeChunk), end = std::min(n, c1 + ov);
        ctx->keep_below = end > c1 ? c1 - c0 : 0;
        ctx->pos_base = c0;
        rc = enqueue_chunk(ctx, ctx->d_chunk_bases[b], end - c0, ctx->d_chunk_runs[b], kruns[b], ctx->d_hits,
                           hit_cap);
        ctx->keep_below = ctx->pos_base = 0;
        if (rc) return rc;
        // this chunk's record slots, the running hit count, its candidates and the status, to
        // host memory
        CK(cudaMemcpyAsync(hc_k + 4 * k, ctx->d_counters, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           ctx->stream));
        CK(cudaMemcpyAsync(hc_k + 4 * k + 2, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaEventRecord(ctx->done_ev[b], ctx->stream));
        if (k >= 1 && (rc = drain_out(k - 1))) return rc;
    }
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    if ((rc = drain_out(nchunks - 1))) return rc;
    CK(cudaStreamSynchronize(ctx->copy_stream));  // the hits are in host memory
    blamm_stats total{};
    total.positions = n;
    total.columns = scanned_columns(ctx);
    total.tiles = (int32_t)(tc ? ctx->tiles.size() : 0);
    total.launches = 0;
    for (int64_t k = 0; k < nchunks; ++k) {  // packing + scan (+ rescoring and a one-hot build per window)
        const int64_t len = std::min(n, (k + 1) * kPipeChunk + ov) - k * kPipeChunk;
        total.launches += (int32_t)(tc ? 2 + 2 * ((len + ctx->ewindow - 1) / ctx->ewindow) : 2);
    }
    int status = 0;
    for (int64_t k = 0; k < nchunks; ++k) {
        const int64_t nc = (int64_t)hc_k[4 * k];
        if (tc) total.candidates += (int64_t)hc_k[4 * k + 3];
        if (tc && nc > ctx->cand_cap) *cand_overflow = std::max(*cand_overflow, nc);
        status |= (int)(hc_k[4 * k + 2] & 0xffffffffu);
    }
    cudaEventElapsedTime(&total.kernel_ms, ctx->ev[1], ctx->ev[2]);
    const int64_t nh_total = (int64_t)hc_k[4 * (nchunks - 1) + 1];
    total.hits = nh_total;
    ctx->stats = total;
    *n_hits = nh_total;
    if (status) return fail(ctx, BLAMM_ERR_TIMEOUT, "scan kernel: a device wait timed out");
    if (*cand_overflow) return BLAMM_ERR_OVERFLOW;
    return nh_total > hit_cap
               ? fail(ctx, BLAMM_ERR_OVERFLOW, "%lld hits > capacity %lld", (long long)nh_total, (long long)hit_cap)
               : BLAMM_OK;
}

// Whatever way the steps end, the chunk filter is reset and no copy into the caller's
// buffers is still in flight.  A chunk whose candidates overflowed the buffer sends the
// call to the synchronous chunked path, which grows the buffer and rescans.
static int scan_host_pipelined(blamm_ctx *ctx, const char *bases, int64_t n, const int64_t *run_start,
                               int64_t nruns, blamm_hit *hits, int64_t hit_cap, int64_t *n_hits)
{
    int64_t cand_overflow = 0;
    int rc = scan_host_async_steps(ctx, bases, n, run_start, nruns, hits, hit_cap, n_hits, &cand_overflow);
    ctx->keep_below = ctx->pos_base = 0;
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamSynchronize(ctx->stream);
    if (rc == BLAMM_ERR_OVERFLOW && cand_overflow > 0) {
        rc = scan_host_pipelined_steps(ctx, bases, n, run_start, nruns, hits, hit_cap, n_hits);
        ctx->keep_below = ctx->pos_base = 0;
        if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    }
    return rc;
}

int blamm_scan(blamm_ctx *ctx, const char *bases, int64_t n, const int64_t *run_start, int64_t nruns,
               blamm_hit *hits, int64_t hit_cap, int64_t *n_hits)
{
    const NvtxRange nvtx_range("blamm_scan");
    if (!ctx || !n_hits || n < 0 || hit_cap < 0) return BLAMM_ERR_ARG;
    *n_hits = 0;
    if (n == 0) return BLAMM_OK;
    if (!bases || !run_start || nruns <= 0 || (hit_cap > 0 && !hits))
        return fail(ctx, BLAMM_ERR_ARG, "null buffer");
    if (run_start[0] != 0) return fail(ctx, BLAMM_ERR_ARG, "run_start[0] must be 0");
    for (int64_t r = 1; r < nruns; ++r)
        if (run_start[r] <= run_start[r - 1] || run_start[r] >= n)
            return fail(ctx, BLAMM_ERR_ARG, "run_start must ascend strictly inside [0, n)");
    CK(cudaSetDevice(ctx->device));
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "blamm_set_motifs was not called");
    if (n > 2 * kPipeChunk) {
        const auto t0 = std::chrono::steady_clock::now();
        const int rc = scan_host_pipelined(ctx, bases, n, run_start, nruns, hits, hit_cap, n_hits);
        ctx->stats.total_ms =
            std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return rc;
    }
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    int rc = ensure(ctx, &ctx->d_bases, &ctx->cap_bases, (size_t)n);
    if (rc) return rc;
    rc = ensure(ctx, &ctx->d_runs, &ctx->cap_runs, (size_t)nruns);
    if (rc) return rc;
    size_t hc = (size_t)ctx->hits_cap;
    rc = ensure(ctx, &ctx->d_hits, &hc, (size_t)std::max<int64_t>(hit_cap, 1));
    if (rc) return rc;
    ctx->hits_cap = (int64_t)hc;
    CK(cudaMemcpyAsync(ctx->d_bases, bases, (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_runs, run_start, sizeof(int64_t) * nruns, cudaMemcpyHostToDevice, ctx->stream));
    rc = scan_core(ctx, ctx->d_bases, n, ctx->d_runs, nruns, ctx->d_hits, hit_cap, n_hits);
    if (rc && rc != BLAMM_ERR_OVERFLOW) return rc;
    const int64_t ncopy = std::min<int64_t>(*n_hits, hit_cap);
    if (ncopy > 0)
        CK(cudaMemcpyAsync(hits, ctx->d_hits, sizeof(blamm_hit) * ncopy, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[3]);
    ctx->stats.total_ms = ms;
    return rc;
}

int blamm_filter_score(blamm_ctx *ctx, float *d_R, int m, int n, const float *d_threshold, int *d_occIdx,
                       float *d_occScore, int *d_nOcc)
{
    if (!ctx || m < 0 || n < 0) return BLAMM_ERR_ARG;
    if ((long long)m * n == 0) return BLAMM_OK;
    if (!d_R || !d_threshold || !d_occIdx || !d_occScore || !d_nOcc)
        return fail(ctx, BLAMM_ERR_ARG, "null buffer");
    CK(cudaSetDevice(ctx->device));
    const long long total = (long long)m * n;
    const int threads = 256;
    const long long blocks = std::min<long long>((total + threads - 1) / threads, (long long)ctx->sm_count * 32);
    filter_score_kernel<<<(unsigned)blocks, threads, 0, ctx->stream>>>(d_R, m, n, d_threshold, d_occIdx,
                                                                      d_occScore, d_nOcc);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    return BLAMM_OK;
}

int blamm_device_count(int *n)
{
    if (!n) return BLAMM_ERR_ARG;
    *n = 0;
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        return BLAMM_OK;
    }
    *n = c;
    return BLAMM_OK;
}

int blamm_device_memory(int device, int64_t *free_bytes, int64_t *total_bytes)
{
    if (!free_bytes || !total_bytes) return BLAMM_ERR_ARG;
    *free_bytes = *total_bytes = 0;
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) return BLAMM_ERR_CUDA;
    if (cudaSetDevice(device) != cudaSuccess) return BLAMM_ERR_CUDA;
    size_t f = 0, t = 0;
    const cudaError_t e = cudaMemGetInfo(&f, &t);
    cudaSetDevice(cur);
    if (e != cudaSuccess) return BLAMM_ERR_CUDA;
    *free_bytes = (int64_t)f;
    *total_bytes = (int64_t)t;
    return BLAMM_OK;
}

int blamm_set_softmask(blamm_ctx *ctx, int lowercase_scores)
{
    if (!ctx) return BLAMM_ERR_ARG;
    ctx->lower_scores = lowercase_scores ? 1 : 0;
    return BLAMM_OK;
}

// The empirical histograms of n bases already on the device (run starts on the host).
static int score_histograms_on(blamm_ctx *ctx, const char *d_bases, int64_t n, const int64_t *run_start,
                               int64_t nruns, const float *min_score, const float *width, int nbins,
                               uint64_t *counts)
{
    int rc = ensure(ctx, &ctx->d_runs, &ctx->cap_runs, (size_t)nruns);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->d_runs, run_start, sizeof(int64_t) * nruns, cudaMemcpyHostToDevice, ctx->stream));
    rc = launch_pack(ctx, d_bases, n);
    if (rc) return rc;
    const size_t nc = (size_t)ctx->ncols;
    float *d_min = nullptr, *d_w = nullptr;
    unsigned long long *d_counts = nullptr;
    auto cleanup = [&]() {
        if (d_min) cudaFree(d_min);
        if (d_w) cudaFree(d_w);
        if (d_counts) cudaFree(d_counts);
    };
    cudaError_t e = cudaMalloc(&d_min, sizeof(float) * nc);
    if (e == cudaSuccess) e = cudaMalloc(&d_w, sizeof(float) * nc);
    if (e == cudaSuccess) e = cudaMalloc(&d_counts, sizeof(unsigned long long) * nc * nbins);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_min, min_score, sizeof(float) * nc, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_w, width, sizeof(float) * nc, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_counts, 0, sizeof(unsigned long long) * nc * nbins, ctx->stream);
    if (e != cudaSuccess) {
        cleanup();
        return fail(ctx, BLAMM_ERR_CUDA, "%s", cudaGetErrorString(e));
    }
    HistParams p{};
    p.seq2 = ctx->d_seq2;
    p.zmask = ctx->d_zmask;
    p.n = n;
    p.run_start = ctx->d_runs;
    p.nruns = nruns;
    p.P = ctx->d_P;
    p.p_rows = ctx->p_rows;
    p.ncols = ctx->ncols;
    p.lmax = ctx->lmax;
    p.col_len = ctx->d_len;
    p.min_score = d_min;
    p.width = d_w;
    p.nbins = nbins;
    p.counts = d_counts;
    const int threads = 256;
    int cpb = 32;
    auto need = [&](int c) { return (size_t)c * (p.p_rows + nbins) * 4 + threads + p.lmax + 64; };
    while (cpb > 1 && need(cpb) > (size_t)ctx->max_smem) cpb /= 2;
    if (need(cpb) > (size_t)ctx->max_smem) {
        cleanup();
        return fail(ctx, BLAMM_ERR_UNSUPPORTED, "too many bins for shared memory");
    }
    p.cols_per_block = cpb;
    const int64_t bx = (n + threads - 1) / threads;
    const int by = (ctx->ncols + cpb - 1) / cpb;
    e = cudaFuncSetAttribute(score_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->max_smem);
    if (e == cudaSuccess) {
        score_hist_kernel<<<dim3((unsigned)bx, (unsigned)by), threads, need(cpb), ctx->stream>>>(p);
        e = cudaGetLastError();
    }
    std::vector<unsigned long long> host(nc * nbins);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host.data(), d_counts, sizeof(unsigned long long) * nc * nbins, cudaMemcpyDeviceToHost,
                            ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cleanup();
    if (e != cudaSuccess) return fail(ctx, BLAMM_ERR_CUDA, "%s", cudaGetErrorString(e));
    for (size_t i = 0; i < nc * (size_t)nbins; ++i) counts[i] += host[i];
    return BLAMM_OK;
}

int blamm_score_histograms(blamm_ctx *ctx, const char *bases, int64_t n, const int64_t *run_start,
                           int64_t nruns, const float *min_score, const float *width, int nbins,
                           uint64_t *counts)
{
    const NvtxRange nvtx_range("blamm_score_histograms");
    if (!ctx || n < 0 || nbins <= 0 || !min_score || !width || !counts) return BLAMM_ERR_ARG;
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "no motif bank");
    if (n == 0) return BLAMM_OK;
    if (!bases || !run_start || nruns <= 0) return fail(ctx, BLAMM_ERR_ARG, "null buffer");
    CK(cudaSetDevice(ctx->device));
    int rc = ensure(ctx, &ctx->d_bases, &ctx->cap_bases, (size_t)n);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->d_bases, bases, (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    return score_histograms_on(ctx, ctx->d_bases, n, run_start, nruns, min_score, width, nbins, counts);
}

int blamm_score_histograms_stream(blamm_ctx *ctx, int64_t begin, int64_t n, const int64_t *run_start,
                                  int64_t nruns, const float *min_score, const float *width, int nbins,
                                  uint64_t *counts)
{
    const NvtxRange nvtx_range("blamm_score_histograms_stream");
    if (!ctx || n < 0 || begin < 0 || nbins <= 0 || !min_score || !width || !counts) return BLAMM_ERR_ARG;
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "no motif bank");
    if (begin > ctx->stream_n || n > ctx->stream_n - begin)
        return fail(ctx, BLAMM_ERR_ARG, "positions [%lld, %lld) outside the resident stream of %lld bases",
                    (long long)begin, (long long)(begin + n), (long long)ctx->stream_n);
    if (n == 0) return BLAMM_OK;
    if (!run_start || nruns <= 0) return fail(ctx, BLAMM_ERR_ARG, "null buffer");
    if (run_start[0] != 0) return fail(ctx, BLAMM_ERR_ARG, "run_start[0] must be 0");
    for (int64_t r = 1; r < nruns; ++r)
        if (run_start[r] <= run_start[r - 1] || run_start[r] >= n)
            return fail(ctx, BLAMM_ERR_ARG, "run_start must ascend strictly inside [0, n)");
    CK(cudaSetDevice(ctx->device));
    return score_histograms_on(ctx, ctx->d_stream + begin, n, run_start, nruns, min_score, width, nbins, counts);
}

int blamm_debug_stall(blamm_ctx *ctx, int enable, long long wait_limit_cycles)
{
    if (!ctx || wait_limit_cycles < 0) return BLAMM_ERR_ARG;
    ctx->debug_stall = enable ? 1 : 0;
    ctx->wait_limit = wait_limit_cycles > 0 ? wait_limit_cycles : 4000000000LL;
    return BLAMM_OK;
}

int blamm_debug_profile(blamm_ctx *ctx, int enable)
{
    if (!ctx) return BLAMM_ERR_ARG;
    ctx->prof_on = enable != 0;
    return BLAMM_OK;
}

int blamm_debug_profile_read(const blamm_ctx *ctx, int64_t *out, int max_ctas, int *nctas)
{
    if (!ctx || !nctas) return BLAMM_ERR_ARG;
    *nctas = ctx->prof_ctas;
    if (out)
        for (int i = 0; i < 32 * std::min(max_ctas, ctx->prof_ctas); ++i) out[i] = ctx->prof[(size_t)i];
    return BLAMM_OK;
}

int blamm_ctx_stream(const blamm_ctx *ctx, void **stream)
{
    if (!ctx || !stream) return BLAMM_ERR_ARG;
    *stream = (void *)ctx->stream;
    return BLAMM_OK;
}

int blamm_last_stats(const blamm_ctx *ctx, blamm_stats *out)
{
    if (!ctx || !out) return BLAMM_ERR_ARG;
    *out = ctx->stats;
    return BLAMM_OK;
}

int blamm_guard_band(const blamm_ctx *ctx, float *out)
{
    if (!ctx || !out) return BLAMM_ERR_ARG;
    blamm_ctx *c = const_cast<blamm_ctx *>(ctx);
    if (c->mode == BLAMM_MODE_FP32) {
        std::fill(out, out + c->ncols, 0.0f);
        return BLAMM_OK;
    }
    int rc = ensure_plan(c);
    if (rc) return rc;
    std::copy(c->guard.begin(), c->guard.end(), out);
    return BLAMM_OK;
}

int blamm_debug_scores(blamm_ctx *ctx, const char *bases, int64_t n, int64_t p0, int64_t npos, float *out)
{
    if (!ctx || !bases || !out || n <= 0 || p0 < 0 || npos <= 0 || p0 + npos > n) return BLAMM_ERR_ARG;
    if (ctx->mode == BLAMM_MODE_FP32) return fail(ctx, BLAMM_ERR_STATE, "debug scores need a tcgen05 mode");
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "no motif bank");
    CK(cudaSetDevice(ctx->device));
    int rc = ensure(ctx, &ctx->d_bases, &ctx->cap_bases, (size_t)n);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->d_bases, bases, (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    rc = launch_pack(ctx, ctx->d_bases, n);
    if (rc) return rc;
    int64_t runs0 = 0;
    rc = ensure(ctx, &ctx->d_runs, &ctx->cap_runs, 1);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->d_runs, &runs0, sizeof runs0, cudaMemcpyHostToDevice, ctx->stream));
    float *d_dump = nullptr;
    CK(cudaMalloc(&d_dump, sizeof(float) * (size_t)npos * ctx->ncols));
    CK(cudaMemsetAsync(d_dump, 0, sizeof(float) * (size_t)npos * ctx->ncols, ctx->stream));
    int launches = 0;
    size_t hc = (size_t)ctx->hits_cap;
    rc = ensure(ctx, &ctx->d_hits, &hc, 1);
    if (rc) { cudaFree(d_dump); return rc; }
    ctx->hits_cap = (int64_t)hc;
    rc = run_tc(ctx, n, ctx->d_runs, 1, ctx->d_hits, 0, d_dump, p0, npos, &launches);
    if (rc == BLAMM_OK) {
        cudaError_t e = cudaMemcpyAsync(out, d_dump, sizeof(float) * (size_t)npos * ctx->ncols,
                                        cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = fail(ctx, BLAMM_ERR_CUDA, "%s", cudaGetErrorString(e));
        // the accumulator holds sum(q) - T; report sum(q) (exact: both are on the column grid)
        for (int64_t i = 0; rc == BLAMM_OK && i < npos; ++i)
            for (int c = 0; c < ctx->ncols; ++c) {
                float &v = out[i * ctx->ncols + c];
                // the E4M3 form's accumulator is scaled by 2^k (exact: a power of two)
                const double sv = ctx->plan_terms == kE4M3 ? std::ldexp((double)v, -ctx->colq_k[c]) : (double)v;
                v = (float)(sv + ctx->bias_T[c]);
            }
    }
    cudaFree(d_dump);
    return rc;
}

}  // extern "C"

// ------------------------------------------------------------------ allocation-free scan
//
// blamm_scan_device_static keeps every per-call buffer of a scan (the packed
// stream, the candidate list, the counters and the status word) in one
// file-scope __device__ array instead of the context's cudaMalloc'd buffers,
// so the call itself allocates no device or host memory.  The array is part of
// this library's device image: each device gets its own copy when the module
// is loaded there.  Its device address is looked up once per device with
// cudaGetSymbolAddress (the host-side name of a __device__ array is not a
// device address) with that device current.

namespace {

constexpr int64_t kStaticMaxBases = int64_t(4) << 20;  // positions per call
constexpr int64_t kStaticWords32 = (kStaticMaxBases + kStreamPad + 31) / 32;
constexpr int64_t kStaticCandCap = int64_t(2) << 20;   // tensor-core candidate record slots per call
constexpr size_t round256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kStaticSeq2Off = 0;
constexpr size_t kStaticZmaskOff = round256(kStaticSeq2Off + sizeof(uint32_t) * 2 * kStaticWords32);
constexpr size_t kStaticE16Off = round256(kStaticZmaskOff + sizeof(uint32_t) * kStaticWords32);
constexpr size_t kStaticCandOff = round256(kStaticE16Off + sizeof(uint4) * (kStaticMaxBases + kStreamPad));
constexpr size_t kStaticCountOff = round256(kStaticCandOff + sizeof(uint4) * kStaticCandCap);
constexpr size_t kStaticStatusOff = round256(kStaticCountOff + sizeof(unsigned long long) * 4);
constexpr size_t kStaticBytes = round256(kStaticStatusOff + sizeof(int));  // about 97 MiB

constexpr int kStaticMaxDevices = 64;

}  // namespace

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

static std::mutex g_static_mu;
static unsigned char *g_static_ptr[kStaticMaxDevices] = {};

// Device address of this device's scratch copy; the first call on a device
// looks it up (the current device must be ctx->device).
static int static_scratch(blamm_ctx *ctx, unsigned char **out)
{
    if (ctx->device < 0 || ctx->device >= kStaticMaxDevices)
        return fail(ctx, BLAMM_ERR_UNSUPPORTED, "device %d: no static scratch slot", ctx->device);
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[ctx->device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            return fail(ctx, BLAMM_ERR_CUDA, "cudaGetSymbolAddress(static scratch): %s", cudaGetErrorString(e));
        g_static_ptr[ctx->device] = static_cast<unsigned char *>(p);
    }
    *out = g_static_ptr[ctx->device];
    return BLAMM_OK;
}

extern "C" {

int blamm_scan_device_static(blamm_ctx *ctx, const char *d_bases, int64_t n, const int64_t *d_run_start,
                             int64_t nruns, blamm_hit *d_hits, int64_t hit_cap, int64_t *n_hits)
{
    const NvtxRange nvtx_range("blamm_scan_device_static");
    if (!ctx || !n_hits || n < 0 || hit_cap < 0) return BLAMM_ERR_ARG;
    *n_hits = 0;
    if (n > kStaticMaxBases)
        return fail(ctx, BLAMM_ERR_ARG, "blamm_scan_device_static: %lld positions > the static limit %lld",
                    (long long)n, (long long)kStaticMaxBases);
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "blamm_set_motifs was not called");
    const bool tc = ctx->mode != BLAMM_MODE_FP32;
    const int terms = mode_terms(ctx);
    if (tc && !(ctx->plan_valid && ctx->plan_terms == terms))
        return fail(ctx, BLAMM_ERR_STATE,
                    "blamm_scan_device_static: no tensor-core plan for this bank, mode and thresholds "
                    "(one blamm_scan or blamm_scan_device call builds it)");
    if (n == 0) return BLAMM_OK;
    if (!d_bases || !d_run_start || nruns <= 0 || (hit_cap > 0 && !d_hits))
        return fail(ctx, BLAMM_ERR_ARG, "null buffer");
    CK(cudaSetDevice(ctx->device));
    unsigned char *base = nullptr;
    int rc = static_scratch(ctx, &base);
    if (rc) return rc;
    uint32_t *seq2 = reinterpret_cast<uint32_t *>(base + kStaticSeq2Off);
    uint32_t *zmask = reinterpret_cast<uint32_t *>(base + kStaticZmaskOff);
    uint4 *e16 = reinterpret_cast<uint4 *>(base + kStaticE16Off);
    uint4 *cand = reinterpret_cast<uint4 *>(base + kStaticCandOff);
    unsigned long long *counters = reinterpret_cast<unsigned long long *>(base + kStaticCountOff);
    int *status = reinterpret_cast<int *>(base + kStaticStatusOff);

    ctx->stats = blamm_stats{};
    ctx->stats.positions = n;
    ctx->stats.columns = scanned_columns(ctx);
    int launches = 0;
    // the counters (candidates, hits) and the status word start at zero on every call
    CK(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
    CK(cudaMemsetAsync(status, 0, sizeof(int), ctx->stream));
    const int64_t nwords32 = (n + kStreamPad + 31) / 32;
    pack_kernel<<<(unsigned)((nwords32 + 255) / 256), 256, 0, ctx->stream>>>(d_bases, n, seq2, zmask, nwords32,
                                                                          ctx->lower_scores);
    CK(cudaGetLastError());
    ++launches;

    if (!tc) {
        PlainParams p = plain_params(ctx, seq2, zmask, n, d_run_start, nruns, d_hits, hit_cap, counters + 1);
        if ((rc = launch_plain(ctx, p))) return rc;
        ++launches;
    } else {
        const int64_t n_mtiles = (n + kBM - 1) / kBM;
        const long long njobs = (long long)ctx->tiles.size() * n_mtiles;
        const TcSmem L = tc_smem_layout(ctx->b_term_max, ctx->plan_terms, ctx->erows, (int)ctx->tiles.size());
        if ((int)L.total > ctx->max_smem)
            return fail(ctx, BLAMM_ERR_UNSUPPORTED, "shared memory plan %u > %d", L.total, ctx->max_smem);
        const uint32_t smem = std::max<uint32_t>(L.total, 116 * 1024);
        TcParams p = tc_params(ctx, n);
        p.cand = cand;
        p.cand_count = counters;
        p.ncand = counters + 3;
        p.cand_cap = kStaticCandCap;
        p.status = status;
        p.wait_limit = ctx->wait_limit;
        p.dump_ncols = ctx->ncols;
        (void)njobs;
        if ((rc = launch_tc_windows(ctx, p, seq2, zmask, e16, n, false, smem, &launches, nullptr))) return rc;
        unsigned long long ncand = 0;
        int st = 0;
        CK(cudaMemcpyAsync(&ncand, counters, sizeof ncand, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(&st, status, sizeof st, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if (st) return fail(ctx, BLAMM_ERR_TIMEOUT, "scan kernel: a device wait timed out");
        if ((int64_t)ncand > kStaticCandCap)
            return fail(ctx, BLAMM_ERR_OVERFLOW,
                        "blamm_scan_device_static: %llu candidate record slots > the static limit %lld (scan "
                        "fewer positions per call)", ncand, (long long)kStaticCandCap);
        if (ncand > 0) {
            const RescoreParams r = rescore_params(ctx, cand, counters, kStaticCandCap, seq2, zmask, n,
                                                   d_run_start, nruns, d_hits, counters + 1, hit_cap);
            const int threads = 256;
            const int64_t blocks = std::min<int64_t>(((int64_t)ncand + threads - 1) / threads,
                                                     (int64_t)ctx->sm_count * 16);
            rescore_kernel<<<(unsigned)blocks, threads, 0, ctx->stream>>>(r);
            CK(cudaGetLastError());
            ++launches;
        }
    }
    unsigned long long cnt[4] = {0, 0, 0, 0};  // record slots, hits, -, candidates
    CK(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const unsigned long long nh = cnt[1];
    if (tc) ctx->stats.candidates = (int64_t)cnt[3];
    ctx->stats.hits = (int64_t)nh;
    ctx->stats.tiles = (int32_t)(tc ? ctx->tiles.size() : 0);
    ctx->stats.launches = launches;
    *n_hits = (int64_t)nh;
    return (int64_t)nh > hit_cap ? fail(ctx, BLAMM_ERR_OVERFLOW, "%lld hits > capacity %lld", (long long)nh,
                                        (long long)hit_cap)
                                 : BLAMM_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ enqueued scans, graphs, autotuning

extern "C" {

int blamm_reserve(blamm_ctx *ctx, int64_t max_positions, int64_t max_candidates)
{
    const NvtxRange nvtx_range("blamm_reserve");
    if (!ctx || max_positions < 0 || max_candidates < 0) return BLAMM_ERR_ARG;
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "blamm_set_motifs was not called");
    CK(cudaSetDevice(ctx->device));
    const int64_t nwords32 = (max_positions + kStreamPad + 31) / 32;
    int rc = ensure(ctx, &ctx->d_seq2, &ctx->cap_words32, (size_t)(2 * nwords32));
    if (!rc) rc = ensure(ctx, &ctx->d_zmask, &ctx->cap_zmask, (size_t)nwords32);
    if (rc) return rc;
    if (ctx->mode != BLAMM_MODE_FP32) {
        if ((rc = ensure_plan(ctx))) return rc;
        if ((rc = ensure(ctx, &ctx->d_e16, &ctx->cap_e16, (size_t)e16_entries(ctx, max_positions)))) return rc;
        // record slots: at most one record per candidate, plus the blocks the warps reserve
        const int64_t slots = std::min(max_candidates + record_slots_reserved(ctx->sm_count), kMaxRecordSlots);
        if (slots > ctx->cand_cap) {
            size_t cap = ctx->cand_cap > 0 ? (size_t)ctx->cand_cap : 0;
            rc = ensure(ctx, &ctx->d_cand, &cap, (size_t)slots);
            if (rc) return rc;
            ctx->cand_cap = (int64_t)cap;
        }
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return BLAMM_OK;
}

int blamm_scan_enqueue(blamm_ctx *ctx, const char *d_bases, int64_t n, const int64_t *d_run_start, int64_t nruns,
                       blamm_hit *d_hits, int64_t hit_cap, uint64_t *d_counts)
{
    const NvtxRange nvtx_range("blamm_scan_enqueue");
    if (!ctx || !d_counts || n < 0 || hit_cap < 0) return BLAMM_ERR_ARG;
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "blamm_set_motifs was not called");
    const int64_t nwords32 = (n + kStreamPad + 31) / 32;
    if ((size_t)(2 * nwords32) > ctx->cap_words32 || (size_t)nwords32 > ctx->cap_zmask)
        return fail(ctx, BLAMM_ERR_STATE, "blamm_scan_enqueue: %lld positions exceed the reservation",
                    (long long)n);
    const bool tc = ctx->mode != BLAMM_MODE_FP32;
    const int terms = mode_terms(ctx);
    if (tc && (!(ctx->plan_valid && ctx->plan_terms == terms) || ctx->cand_cap <= 0 ||
               (size_t)e16_entries(ctx, n) > ctx->cap_e16))
        return fail(ctx, BLAMM_ERR_STATE, "blamm_scan_enqueue: call blamm_reserve after changing the bank, "
                                          "columns, thresholds or mode");
    if (n > 0 && (!d_bases || !d_run_start || nruns <= 0 || (hit_cap > 0 && !d_hits)))
        return fail(ctx, BLAMM_ERR_ARG, "null buffer");
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemsetAsync(d_counts, 0, 4 * sizeof(uint64_t), ctx->stream));
    if (n == 0) return BLAMM_OK;
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(d_counts);
    pack_kernel<<<(unsigned)((nwords32 + 255) / 256), 256, 0, ctx->stream>>>(d_bases, n, ctx->d_seq2, ctx->d_zmask,
                                                                          nwords32, ctx->lower_scores);
    CK(cudaGetLastError());
    if (!tc) {
        PlainParams p = plain_params(ctx, ctx->d_seq2, ctx->d_zmask, n, d_run_start, nruns, d_hits, hit_cap, cnt + 1);
        return launch_plain(ctx, p);
    }
    const int64_t n_mtiles = (n + kBM - 1) / kBM;
    const long long njobs = (long long)ctx->tiles.size() * n_mtiles;
    if (int rc = check_jobs(ctx, njobs)) return rc;
    const TcSmem L = tc_smem_layout(ctx->b_term_max, ctx->plan_terms, ctx->erows, (int)ctx->tiles.size());
    if ((int)L.total > ctx->max_smem)
        return fail(ctx, BLAMM_ERR_UNSUPPORTED, "shared memory plan %u > %d", L.total, ctx->max_smem);
    TcParams p = tc_params(ctx, n);
    p.cand = ctx->d_cand;
    p.cand_count = cnt;
    p.ncand = cnt + 3;
    p.cand_cap = ctx->cand_cap;
    p.status = reinterpret_cast<int *>(cnt + 2);
    p.wait_limit = ctx->wait_limit;
    p.dump_ncols = ctx->ncols;
    if (int rc = launch_tc_windows(ctx, p, ctx->d_seq2, ctx->d_zmask, ctx->d_e16, n, false,
                                   std::max<uint32_t>(L.total, 116 * 1024), nullptr, nullptr))
        return rc;
    const RescoreParams r = rescore_params(ctx, ctx->d_cand, cnt, ctx->cand_cap, ctx->d_seq2, ctx->d_zmask,
                                           n, d_run_start, nruns, d_hits, cnt + 1, hit_cap);
    // a fixed grid: the candidate count is only known on the device
    rescore_kernel<<<(unsigned)(ctx->sm_count * 8), 256, 0, ctx->stream>>>(r);
    CK(cudaGetLastError());
    return BLAMM_OK;
}

int blamm_scan_graph_create(blamm_ctx *ctx, const char *d_bases, int64_t n, const int64_t *d_run_start,
                            int64_t nruns, blamm_hit *d_hits, int64_t hit_cap, uint64_t *d_counts, void **graph)
{
    if (!ctx || !graph) return BLAMM_ERR_ARG;
    *graph = nullptr;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = blamm_scan_enqueue(ctx, d_bases, n, d_run_start, nruns, d_hits, hit_cap, d_counts);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(ctx, BLAMM_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e));
    cudaGraphExec_t ge = nullptr;
    const cudaError_t e2 = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) return fail(ctx, BLAMM_ERR_CUDA, "graph instantiation: %s", cudaGetErrorString(e2));
    *graph = ge;
    return BLAMM_OK;
}

int blamm_scan_graph_launch(blamm_ctx *ctx, void *graph)
{
    const NvtxRange nvtx_range("blamm_scan_graph_launch");
    if (!ctx || !graph) return BLAMM_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaGraphLaunch(static_cast<cudaGraphExec_t>(graph), ctx->stream));
    return BLAMM_OK;
}

void blamm_scan_graph_destroy(void *graph)
{
    if (graph) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(graph));
}

int blamm_set_plan_options(blamm_ctx *ctx, int max_tile_columns, float job_cost)
{
    if (!ctx || max_tile_columns < 32 || max_tile_columns > 256 || !(job_cost >= 0.0f)) return BLAMM_ERR_ARG;
    ctx->plan_nmax = max_tile_columns;
    ctx->plan_job_cost = job_cost;
    ctx->plan_valid = false;
    return BLAMM_OK;
}

int blamm_get_terms(const blamm_ctx *ctx)
{
    if (!ctx) return 0;
    return ctx->mode == BLAMM_MODE_FP32 ? 0 : mode_terms(ctx);
}

int blamm_get_plan_options(const blamm_ctx *ctx, int *max_tile_columns, float *job_cost)
{
    if (!ctx || !max_tile_columns || !job_cost) return BLAMM_ERR_ARG;
    *max_tile_columns = ctx->plan_nmax;
    *job_cost = (float)ctx->plan_job_cost;
    return BLAMM_OK;
}

int blamm_autotune(blamm_ctx *ctx, const char *d_bases, int64_t n, const int64_t *d_run_start, int64_t nruns,
                   float *best_ms)
{
    const NvtxRange nvtx_range("blamm_autotune");
    if (!ctx || n < 0) return BLAMM_ERR_ARG;
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "blamm_set_motifs was not called");
    if (best_ms) *best_ms = 0.0f;
    if (ctx->mode == BLAMM_MODE_FP32 || n == 0) return BLAMM_OK;
    if (!d_bases || !d_run_start || nruns <= 0) return fail(ctx, BLAMM_ERR_ARG, "null buffer");
    CK(cudaSetDevice(ctx->device));
    // a sample of up to 16 Mi positions (the runs that start inside it)
    const int64_t ns = std::min<int64_t>(n, int64_t(16) << 20);
    std::vector<int64_t> runs((size_t)nruns);
    CK(cudaMemcpy(runs.data(), d_run_start, sizeof(int64_t) * nruns, cudaMemcpyDeviceToHost));
    const int64_t nrs = std::max<int64_t>(1, std::lower_bound(runs.begin(), runs.end(), ns) - runs.begin());
    size_t hc = (size_t)ctx->hits_cap;
    int rc = ensure(ctx, &ctx->d_hits, &hc, (size_t)1 << 20);
    if (rc) return rc;
    ctx->hits_cap = (int64_t)hc;
    const int nmax_opts[] = {128, 192, 256};
    const double cost_opts[] = {200.0, 700.0, 1500.0};
    const int keep_nmax = ctx->plan_nmax, keep_terms = ctx->auto_terms;
    const double keep_cost = ctx->plan_job_cost;
    // BLAMM_MODE_AUTO also chooses the form: one BF16 term halves the MMAs of two and
    // widens the guard band (more candidates to rescore), one E4M3 term (motifs up to 64
    // positions) halves them again with a still wider band, so the whole call's kernel
    // time (packing, scan, rescoring) decides
    int lmax_sel = 1;
    if (ctx->active.empty())
        for (int c = 0; c < ctx->ncols; ++c) lmax_sel = std::max(lmax_sel, ctx->len[c]);
    else
        for (const int c : ctx->active) lmax_sel = std::max(lmax_sel, ctx->len[c]);
    int term_opts[3] = {1, 2, kE4M3};
    const int nterm_opts = ctx->mode == BLAMM_MODE_AUTO ? (lmax_sel <= kMaxE4M3Len ? 3 : 2) : 1;
    float best = std::numeric_limits<float>::infinity();
    int bn = keep_nmax, bt = keep_terms;
    double bc = keep_cost;
    for (int ti = 0; ti < nterm_opts; ++ti)
        for (int nm : nmax_opts)
            for (double jc : cost_opts) {
                if (ctx->mode == BLAMM_MODE_AUTO) ctx->auto_terms = term_opts[ti];
                ctx->plan_nmax = nm;
                ctx->plan_job_cost = jc;
                ctx->plan_valid = false;
                float t[3];
                for (int rep = 0; rep < 3; ++rep) {
                    int64_t nh = 0;
                    rc = scan_core(ctx, d_bases, ns, d_run_start, nrs, ctx->d_hits, ctx->hits_cap, &nh);
                    if (rc && rc != BLAMM_ERR_OVERFLOW) {
                        ctx->plan_nmax = keep_nmax;
                        ctx->plan_job_cost = keep_cost;
                        ctx->auto_terms = keep_terms;
                        ctx->plan_valid = false;
                        return rc;
                    }
                    t[rep] = ctx->stats.kernel_ms;
                }
                std::sort(t, t + 3);
                if (t[1] < best) {
                    best = t[1];
                    bn = nm;
                    bc = jc;
                    bt = ctx->auto_terms;
                }
            }
    ctx->plan_nmax = bn;
    ctx->plan_job_cost = bc;
    ctx->auto_terms = bt;
    ctx->plan_valid = false;
    if ((rc = ensure_plan(ctx))) return rc;
    if (best_ms) *best_ms = best;
    return BLAMM_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ theoretical histograms, thresholds

extern "C" {

int blamm_theoretical_hist(blamm_ctx *ctx, const float *P, int p_rows, int ncols, const int32_t *col_len,
                           const int32_t *hist_of, const float bg_prob[4], int nbins, uint64_t max_length,
                           int fp64_dp, const float *pvalues, int npv, float *thr, uint64_t *counts)
{
    const NvtxRange nvtx_range("blamm_theoretical_hist");
    if (!ctx || !P || !col_len || !bg_prob || ncols <= 0 || p_rows <= 0 || nbins < 1 || nbins > 4096 ||
        npv < 0 || (npv > 0 && (!pvalues || !thr)))
        return BLAMM_ERR_ARG;
    for (int c = 0; c < ncols; ++c) {
        const int h = hist_of ? hist_of[c] : c;
        if (h < 0 || h >= ncols) return fail(ctx, BLAMM_ERR_ARG, "hist_of[%d] = %d is not a column", c, h);
        if (col_len[h] <= 0 || col_len[h] > kMaxMotifLen || 4 * col_len[h] > p_rows)
            return fail(ctx, BLAMM_ERR_ARG, "column %d: bad length %d", h, col_len[h]);
    }
    CK(cudaSetDevice(ctx->device));
    const int kmax = 8192;
    const size_t smem = theo_smem_bytes(kmax, nbins, fp64_dp);
    if (smem > (size_t)ctx->max_smem) return fail(ctx, BLAMM_ERR_UNSUPPORTED, "histogram does not fit");
    std::vector<int32_t> hof(ncols);
    for (int c = 0; c < ncols; ++c) hof[c] = hist_of ? hist_of[c] : c;
    float *d_P = nullptr, *d_pv = nullptr, *d_thr = nullptr;
    int32_t *d_len = nullptr, *d_hof = nullptr;
    unsigned long long *d_counts = nullptr;
    int *d_status = nullptr;
    const size_t pbytes = sizeof(float) * (size_t)p_rows * ncols;
    cudaError_t e = cudaMallocAsync(&d_P, pbytes, ctx->stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_len, sizeof(int32_t) * ncols, ctx->stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_hof, sizeof(int32_t) * ncols, ctx->stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_status, sizeof(int), ctx->stream);
    if (e == cudaSuccess && npv > 0) e = cudaMallocAsync(&d_pv, sizeof(float) * npv, ctx->stream);
    if (e == cudaSuccess && npv > 0) e = cudaMallocAsync(&d_thr, sizeof(float) * (size_t)npv * ncols, ctx->stream);
    if (e == cudaSuccess && counts)
        e = cudaMallocAsync(&d_counts, sizeof(unsigned long long) * (size_t)ncols * nbins, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_P, P, pbytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_len, col_len, sizeof(int32_t) * ncols, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_hof, hof.data(), sizeof(int32_t) * ncols, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && npv > 0)
        e = cudaMemcpyAsync(d_pv, pvalues, sizeof(float) * npv, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, sizeof(int), ctx->stream);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(theoretical_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int status = 0;
    if (e == cudaSuccess) {
        TheoHistParams p{};
        p.P = d_P;
        p.p_rows = p_rows;
        p.ncols = ncols;
        p.col_len = d_len;
        p.hist_of = d_hof;
        for (int k = 0; k < 4; ++k) p.bg[k] = bg_prob[k];
        p.nbins = nbins;
        p.max_length = max_length;
        p.fp64_dp = fp64_dp ? 1 : 0;
        p.kmax = kmax;
        p.pvalues = d_pv;
        p.npv = npv;
        p.thr = d_thr;
        p.counts = d_counts;
        p.status = d_status;
        theoretical_hist_kernel<<<ncols, 256, smem, ctx->stream>>>(p);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && npv > 0)
        e = cudaMemcpyAsync(thr, d_thr, sizeof(float) * (size_t)npv * ncols, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && counts)
        e = cudaMemcpyAsync(counts, d_counts, sizeof(unsigned long long) * (size_t)ncols * nbins,
                            cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    void *bufs[] = {d_P, d_len, d_hof, d_status, d_pv, d_thr, d_counts};
    for (void *b : bufs)
        if (b) cudaFreeAsync(b, ctx->stream);
    const cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return fail(ctx, BLAMM_ERR_CUDA, "theoretical histograms: %s", cudaGetErrorString(e));
    if (status) return fail(ctx, BLAMM_ERR_UNSUPPORTED, "a score range exceeds %d keys (fewer bins)", kmax);
    return BLAMM_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ FASTA ingest on the GPU

// In-place inclusive scan of v[0..n) with Op; `scratch` holds at least
// scan_scratch_words(n) values.
static size_t scan_scratch_words(int64_t n)
{
    size_t w = 0;
    for (int64_t t = (n + kScanTile - 1) / kScanTile; t > 1; t = (t + kScanTile - 1) / kScanTile) w += (size_t)t;
    return w + 1;
}

template <class Op>
static cudaError_t device_scan(cudaStream_t st, int64_t *v, int64_t n, int64_t *scratch)
{
    if (n <= 0) return cudaSuccess;
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    scan_tiles_kernel<Op><<<(unsigned)tiles, kScanThreads, 0, st>>>(v, n, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || tiles == 1) return e;
    e = device_scan<Op>(st, scratch, tiles, scratch + tiles);
    if (e != cudaSuccess) return e;
    scan_add_kernel<Op><<<(unsigned)tiles, kScanThreads, 0, st>>>(v, n, scratch);
    return cudaGetLastError();
}

// FASTA text on the device -> filtered stream, run table and header offsets.  Outputs go
// to the caller's buffers, or (resident: the caller's pointers are null) into the
// context's resident-stream buffers, sized once the counts are known.
static int fasta_parse(blamm_ctx *ctx, const char *d_raw, int64_t nraw, bool resident, char *d_bases,
                       int64_t *d_run_start, int64_t *d_run_seq, int64_t *d_run_seqpos, int64_t *d_header_pos,
                       int64_t *n_bases, int64_t *nruns, int64_t *nseqs, uint64_t *nucl_counts)
{
    cudaStream_t st = ctx->stream;
    const size_t n = (size_t)nraw, sw = scan_scratch_words(nraw);
    // four per-byte arrays (line starts, header count, sequence characters, stream bases),
    // the per-sequence character offsets, scan scratch and a status word
    int64_t *A = nullptr, *B = nullptr, *Cc = nullptr, *D = nullptr, *sc0 = nullptr, *scr = nullptr;
    int *bad = nullptr;
    unsigned long long *nucl = nullptr;
    int64_t *bseq = nullptr, *bpos = nullptr;
    int rc = BLAMM_OK;
    cudaError_t e = cudaMallocAsync(&A, 8 * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&B, 8 * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&Cc, 8 * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&D, 8 * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&sc0, 8 * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&scr, 8 * sw, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&bad, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&nucl, 4 * sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(nucl, 0, 4 * sizeof(unsigned long long), st);
    const unsigned grid = (unsigned)std::min<int64_t>((nraw + 255) / 256, (int64_t)ctx->sm_count * 32);
    if (e == cudaSuccess) {
        ingest_lines_kernel<<<grid, 256, 0, st>>>(d_raw, nraw, A, B);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = device_scan<MaxOp>(st, A, nraw, scr);
    if (e == cudaSuccess) e = device_scan<SumOp>(st, B, nraw, scr);
    if (e == cudaSuccess) {
        ingest_chars_kernel<<<grid, 256, 0, st>>>(d_raw, nraw, A, B, Cc, D, bad);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = device_scan<SumOp>(st, Cc, nraw, scr);
    if (e == cudaSuccess) e = device_scan<SumOp>(st, D, nraw, scr);
    int64_t tot[2] = {0, 0};
    int badh = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tot[0], B + nraw - 1, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tot[1], D + nraw - 1, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&badh, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    const int64_t ns = tot[0], nb = tot[1];
    const bool go = e == cudaSuccess && !badh;
    if (go && resident) {
        rc = ensure(ctx, &ctx->d_shdr, &ctx->cap_shdr, (size_t)std::max<int64_t>(ns, 1));
        if (!rc) rc = ensure(ctx, &ctx->d_stream, &ctx->cap_stream, (size_t)std::max<int64_t>(nb, 1));
        d_header_pos = ctx->d_shdr;
        d_bases = ctx->d_stream;
    }
    if (go && !rc) {
        ingest_headers_kernel<<<grid, 256, 0, st>>>(d_raw, nraw, B, Cc, sc0, d_header_pos);
        e = cudaGetLastError();
    }
    const bool have = go && !rc && nb > 0;
    if (have && e == cudaSuccess) e = cudaMallocAsync(&bseq, 8 * (size_t)nb, st);
    if (have && e == cudaSuccess) e = cudaMallocAsync(&bpos, 8 * (size_t)nb, st);
    if (have && e == cudaSuccess) {
        ingest_bases_kernel<<<grid, 256, 0, st>>>(d_raw, nraw, A, B, Cc, D, sc0, d_bases, bseq, bpos, nucl);
        e = cudaGetLastError();
    }
    unsigned long long nh[4] = {0, 0, 0, 0};
    if (have && e == cudaSuccess && nucl_counts) e = cudaMemcpyAsync(nh, nucl, sizeof nh, cudaMemcpyDeviceToHost, st);
    int64_t nr = 0;
    const unsigned g2 = (unsigned)std::min<int64_t>((nb + 255) / 256, (int64_t)ctx->sm_count * 32);
    if (have && e == cudaSuccess) {
        // run flags into A (no longer needed), scanned in place
        ingest_runflags_kernel<<<g2, 256, 0, st>>>(bseq, bpos, nb, A);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = device_scan<SumOp>(st, A, nb, scr);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&nr, A + nb - 1, 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (have && e == cudaSuccess && resident) {
        for (int k = 0; k < 3 && !rc; ++k)
            rc = ensure(ctx, &ctx->d_srun[k], &ctx->cap_srun[k], (size_t)std::max<int64_t>(nr, 1));
        d_run_start = ctx->d_srun[0];
        d_run_seq = ctx->d_srun[1];
        d_run_seqpos = ctx->d_srun[2];
    }
    if (have && e == cudaSuccess && !rc) {
        ingest_runs_kernel<<<g2, 256, 0, st>>>(bseq, bpos, nb, A, d_run_start, d_run_seq, d_run_seqpos);
        e = cudaGetLastError();
    }
    void *bufs[] = {A, B, Cc, D, sc0, scr, bad, bseq, bpos, nucl};
    for (void *b : bufs)
        if (b) cudaFreeAsync(b, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess)
        return fail(ctx, e == cudaErrorMemoryAllocation ? BLAMM_ERR_NOMEM : BLAMM_ERR_CUDA, "FASTA ingest: %s",
                    cudaGetErrorString(e));
    if (rc) return rc;
    if (badh) return fail(ctx, BLAMM_ERR_ARG, "Input file does not appear to be in fasta format");
    *n_bases = nb;
    *nruns = nr;
    *nseqs = ns;
    if (nucl_counts)
        for (int b = 0; b < 4; ++b) nucl_counts[b] = nh[b];
    return BLAMM_OK;
}

extern "C" {

int blamm_fasta_parse_device(blamm_ctx *ctx, const char *d_raw, int64_t nraw, char *d_bases, int64_t *n_bases,
                             int64_t *d_run_start, int64_t *d_run_seq, int64_t *d_run_seqpos, int64_t *nruns,
                             int64_t *d_header_pos, int64_t *nseqs, uint64_t *nucl_counts)
{
    const NvtxRange nvtx_range("blamm_fasta_parse_device");
    if (!ctx || nraw < 0 || !n_bases || !nruns || !nseqs) return BLAMM_ERR_ARG;
    *n_bases = *nruns = *nseqs = 0;
    if (nucl_counts)
        for (int b = 0; b < 4; ++b) nucl_counts[b] = 0;
    if (nraw == 0) return BLAMM_OK;
    if (!d_raw || !d_bases || !d_run_start || !d_run_seq || !d_run_seqpos || !d_header_pos)
        return fail(ctx, BLAMM_ERR_ARG, "null buffer");
    CK(cudaSetDevice(ctx->device));
    return fasta_parse(ctx, d_raw, nraw, false, d_bases, d_run_start, d_run_seq, d_run_seqpos, d_header_pos,
                       n_bases, nruns, nseqs, nucl_counts);
}

int blamm_stream_load_fasta(blamm_ctx *ctx, const char *raw, int64_t nraw, int64_t *n_bases, int64_t *nruns,
                            int64_t *nseqs, uint64_t *nucl_counts)
{
    const NvtxRange nvtx_range("blamm_stream_load_fasta");
    if (!ctx || nraw < 0 || !n_bases || !nruns || !nseqs || (nraw > 0 && !raw)) return BLAMM_ERR_ARG;
    *n_bases = *nruns = *nseqs = 0;
    if (nucl_counts)
        for (int b = 0; b < 4; ++b) nucl_counts[b] = 0;
    ctx->stream_n = ctx->stream_nruns = ctx->stream_nseqs = 0;
    if (nraw == 0) return BLAMM_OK;
    CK(cudaSetDevice(ctx->device));
    int rc = ensure(ctx, &ctx->d_raw, &ctx->cap_raw, (size_t)nraw);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->d_raw, raw, (size_t)nraw, cudaMemcpyHostToDevice, ctx->stream));
    rc = fasta_parse(ctx, ctx->d_raw, nraw, true, nullptr, nullptr, nullptr, nullptr, nullptr, n_bases, nruns,
                     nseqs, nucl_counts);
    if (rc) return rc;
    ctx->stream_n = *n_bases;
    ctx->stream_nruns = *nruns;
    ctx->stream_nseqs = *nseqs;
    return BLAMM_OK;
}

int blamm_stream_tables(blamm_ctx *ctx, int64_t *run_start, int64_t *run_seq, int64_t *run_seqpos,
                        int64_t *header_pos)
{
    if (!ctx) return BLAMM_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    int64_t *dst[4] = {run_start, run_seq, run_seqpos, header_pos};
    const int64_t *src[4] = {ctx->d_srun[0], ctx->d_srun[1], ctx->d_srun[2], ctx->d_shdr};
    const int64_t cnt[4] = {ctx->stream_nruns, ctx->stream_nruns, ctx->stream_nruns, ctx->stream_nseqs};
    for (int k = 0; k < 4; ++k)
        if (dst[k] && cnt[k] > 0)
            CK(cudaMemcpyAsync(dst[k], src[k], 8 * (size_t)cnt[k], cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return BLAMM_OK;
}

int blamm_scan_stream(blamm_ctx *ctx, int64_t begin, int64_t n, const int64_t *run_start, int64_t nruns,
                      blamm_hit *hits, int64_t hit_cap, int64_t *n_hits)
{
    const NvtxRange nvtx_range("blamm_scan_stream");
    if (!ctx || !n_hits || n < 0 || hit_cap < 0 || begin < 0) return BLAMM_ERR_ARG;
    *n_hits = 0;
    if (begin > ctx->stream_n || n > ctx->stream_n - begin)
        return fail(ctx, BLAMM_ERR_ARG, "positions [%lld, %lld) outside the resident stream of %lld bases",
                    (long long)begin, (long long)(begin + n), (long long)ctx->stream_n);
    if (n == 0) return BLAMM_OK;
    if (!run_start || nruns <= 0 || (hit_cap > 0 && !hits)) return fail(ctx, BLAMM_ERR_ARG, "null buffer");
    if (run_start[0] != 0) return fail(ctx, BLAMM_ERR_ARG, "run_start[0] must be 0");
    for (int64_t r = 1; r < nruns; ++r)
        if (run_start[r] <= run_start[r - 1] || run_start[r] >= n)
            return fail(ctx, BLAMM_ERR_ARG, "run_start must ascend strictly inside [0, n)");
    CK(cudaSetDevice(ctx->device));
    if (ctx->ncols == 0) return fail(ctx, BLAMM_ERR_STATE, "blamm_set_motifs was not called");
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    int rc = ensure(ctx, &ctx->d_runs, &ctx->cap_runs, (size_t)nruns);
    if (rc) return rc;
    size_t hc = (size_t)ctx->hits_cap;
    rc = ensure(ctx, &ctx->d_hits, &hc, (size_t)std::max<int64_t>(hit_cap, 1));
    if (rc) return rc;
    ctx->hits_cap = (int64_t)hc;
    CK(cudaMemcpyAsync(ctx->d_runs, run_start, sizeof(int64_t) * nruns, cudaMemcpyHostToDevice, ctx->stream));
    rc = scan_core(ctx, ctx->d_stream + begin, n, ctx->d_runs, nruns, ctx->d_hits, hit_cap, n_hits);
    if (rc && rc != BLAMM_ERR_OVERFLOW) return rc;
    const int64_t ncopy = std::min<int64_t>(*n_hits, hit_cap);
    if (ncopy > 0)
        CK(cudaMemcpyAsync(hits, ctx->d_hits, sizeof(blamm_hit) * ncopy, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[3]);
    ctx->stats.total_ms = ms;
    return rc;
}

}  // extern "C"
