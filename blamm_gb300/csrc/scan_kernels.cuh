// scan_kernels.cuh -- device code of the GB300 PWM scan.
//
// Data layout in HBM (one species' filtered base stream of n positions):
//   seq2[]  : 2-bit base codes, 16 per uint32 (A=0 C=1 G=2 T=3), base i at
//             bits 2*(i%16) of word i/16;
//   zmask[] : 1 bit per base, bit i%32 of word i/32 set when the base adds
//             nothing to a score (lowercase, or past the end of the stream);
//   both padded by kStreamPad bases so that tile loads need no bounds checks.
// Motif bank: the reference's column-major FP32 P (4*Lmax rows), per-column
// lengths and thresholds; for the tensor-core path also the B tiles (one per
// N tile of columns sorted by length), pre-laid-out in the canonical
// no-swizzle K-major UMMA layout so that one TMA bulk copy stages a tile.
#pragma once
#include <cstdint>

#include "ptx_sm100.cuh"

namespace blamm {

constexpr int kStreamPad = 2048;   // padding bases after the stream end
constexpr int kBM = 128;           // positions per M tile (= UMMA M)
constexpr int kWinBases = 8;       // bases per row of the one-hot window W
constexpr int kWRowBytes = 64;     // 8 bases x 4 channels x bf16
constexpr int kMaxTcLen = 256;     // longest motif on the tensor-core path
constexpr int kCandBuf = 256;      // per-warp staging of candidates in SMEM
constexpr int kColBits = 20;       // candidate = pos << 20 | column
constexpr int kTcThreads = 192;    // 4 epilogue warps, 1 MMA warp, 1 W-builder warp

// Per-N-tile description (host-built, staged in SMEM by the kernel).
struct TileDesc {
    int32_t slot0;    // first column slot of the tile (slots: tile-local padded columns)
    int32_t n;        // UMMA N: columns of the tile, padded to a multiple of 32 (<= 256)
    int32_t g;        // k-steps: ceil(max motif length in the tile / 4)
    int32_t b_bytes;  // bytes of one B term (n * 16 * g * 2)
    int64_t b_off;    // byte offset of the tile's first B term in the B buffer
    int64_t pad;
};

struct TcParams {
    const uint32_t *seq2;
    const uint32_t *zmask;
    int64_t n;           // stream positions
    int64_t n_mtiles;    // ceil(n / 128)
    const TileDesc *tiles;
    int32_t ntiles;
    int32_t terms;       // 1 (hi) or 2 (hi + lo)
    const uint8_t *bbuf; // B tiles
    const float *thr_adj;   // per slot: threshold minus guard band (+inf for padding)
    const int32_t *slot_col;  // per slot: motif column, -1 for padding
    int32_t nslots;
    int32_t wrows;       // rows of one W stage (max over tiles)
    uint32_t b_term_max; // bytes reserved per B term in SMEM
    uint32_t tmem_cols;  // TMEM columns allocated (2 accumulators)
    unsigned long long *cand;
    unsigned long long *cand_count;
    int64_t cand_cap;
    int *status;         // bit 0: device wait timed out
    long long wait_limit;  // clock64 cycles a wait may last
    // debug dump of raw accumulator values (positions [dump_p0, dump_p0+dump_npos))
    float *dump;
    int64_t dump_p0, dump_npos;
    int32_t dump_ncols;
};

// ------------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------------
__device__ __forceinline__ int base_code_at(const uint32_t *seq2, const uint32_t *zmask, int64_t i)
{
    uint32_t z = (zmask[i >> 5] >> (i & 31)) & 1u;
    uint32_t b = (seq2[i >> 4] >> (2 * (i & 15))) & 3u;
    return z ? 4 : (int)b;
}

// end (exclusive) of the run that contains position p
__device__ __forceinline__ int64_t run_end_of(const int64_t *run_start, int64_t nruns, int64_t n,
                                              int64_t p)
{
    int64_t lo = 0, hi = nruns;  // first run_start > p
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (__ldg(run_start + mid) <= p) lo = mid + 1;
        else hi = mid;
    }
    return lo < nruns ? __ldg(run_start + lo) : n;
}

// ------------------------------------------------------------------------
// 1. pack: filtered ASCII bases -> 2-bit codes + zero mask
// ------------------------------------------------------------------------
__global__ void pack_kernel(const char *__restrict__ bases, int64_t n, uint32_t *__restrict__ seq2,
                            uint32_t *__restrict__ zmask, int64_t nwords32, int lower_scores)
{
    int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords32) return;
    uint32_t lo = 0, hi = 0, z = 0;
    int64_t p0 = w * 32;
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
        int64_t p = p0 + i;
        uint32_t code = 0, zero = 1;
        if (p < n) {
            uint32_t c = (unsigned char)bases[p];
            uint32_t u = c & 0xDFu;
            bool valid = (u == 'A') | (u == 'C') | (u == 'G') | (u == 'T');
            code = ((c >> 1) ^ (c >> 2)) & 3u;  // A/a=0 C/c=1 G/g=2 T/t=3
            zero = (!valid) | (!lower_scores && (c & 0x20u) != 0);
        }
        if (i < 16) lo |= code << (2 * i);
        else hi |= code << (2 * (i - 16));
        z |= zero << i;
    }
    seq2[2 * w] = lo;
    seq2[2 * w + 1] = hi;
    zmask[w] = z;
}

// ------------------------------------------------------------------------
// 2. plain FP32 scan: one thread per position, sequential FP32 sums
//    (the straightforward GPU form of PWMScan::scanThreadBLAS + extractOccurrences)
// ------------------------------------------------------------------------
struct PlainParams {
    const uint32_t *seq2;
    const uint32_t *zmask;
    int64_t n;
    const int64_t *run_start;
    int64_t nruns;
    const float *P;
    int32_t p_rows;
    int32_t ncols;
    int32_t cols_per_block;
    int32_t lmax;
    const int32_t *col_len;
    const float *thr;
    void *hits;  // blamm_hit*
    unsigned long long *hit_count;
    int64_t hit_cap;
};

struct HitRec {
    int64_t pos;
    int32_t col;
    float score;
};

__device__ __forceinline__ void emit_hits_warp(bool hit, int64_t pos, int32_t col, float score,
                                               HitRec *hits, unsigned long long *count,
                                               int64_t cap)
{
    unsigned m = __ballot_sync(0xffffffffu, hit);
    if (!m) return;
    int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == __ffs(m) - 1) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
    if (hit) {
        unsigned long long idx = base + __popc(m & ((1u << lane) - 1u));
        if ((int64_t)idx < cap) {
            HitRec h;
            h.pos = pos;
            h.col = col;
            h.score = score;
            hits[idx] = h;
        }
    }
}

__global__ void __launch_bounds__(256) scan_plain_kernel(PlainParams p)
{
    extern __shared__ __align__(16) uint8_t smem_plain[];
    const int cpb = p.cols_per_block;
    float *sP = reinterpret_cast<float *>(smem_plain);
    int32_t *sLen = reinterpret_cast<int32_t *>(sP + (size_t)cpb * p.p_rows);
    float *sThr = reinterpret_cast<float *>(sLen + cpb);
    uint8_t *sCode = reinterpret_cast<uint8_t *>(sThr + cpb);

    const int64_t p0 = (int64_t)blockIdx.x * blockDim.x;
    const int c0 = blockIdx.y * cpb;
    const int nc = min(cpb, p.ncols - c0);
    for (int i = threadIdx.x; i < nc * p.p_rows; i += blockDim.x)
        sP[i] = p.P[(size_t)c0 * p.p_rows + i];
    for (int i = threadIdx.x; i < nc; i += blockDim.x) {
        sLen[i] = p.col_len[c0 + i];
        sThr[i] = p.thr[c0 + i];
    }
    const int nwin = blockDim.x + p.lmax;
    for (int i = threadIdx.x; i < nwin; i += blockDim.x)
        sCode[i] = (uint8_t)base_code_at(p.seq2, p.zmask, p0 + i);
    __syncthreads();

    const int64_t pos = p0 + threadIdx.x;
    int64_t rem = 0;
    if (pos < p.n) rem = run_end_of(p.run_start, p.nruns, p.n, pos) - pos;
    const uint8_t *code = sCode + threadIdx.x;
    for (int cc = 0; cc < nc; ++cc) {
        const int L = sLen[cc];
        bool hit = false;
        float s = 0.0f;
        if (L <= rem) {
            const float *col = sP + (size_t)cc * p.p_rows;
            for (int j = 0; j < L; ++j) {
                int b = code[j];
                if (b < 4) s = __fadd_rn(s, col[4 * j + b]);
            }
            hit = s >= sThr[cc];
        }
        emit_hits_warp(hit, pos, c0 + cc, s, reinterpret_cast<HitRec *>(p.hits), p.hit_count,
                       p.hit_cap);
    }
}

// ------------------------------------------------------------------------
// 2b. empirical score histograms: the plain scan with a histogram epilogue
//     (Histogram::histThread / extractObsScore, hist.cpp:70-140)
// ------------------------------------------------------------------------
struct HistParams {
    const uint32_t *seq2;
    const uint32_t *zmask;
    int64_t n;
    const int64_t *run_start;
    int64_t nruns;
    const float *P;
    int32_t p_rows;
    int32_t ncols;
    int32_t cols_per_block;
    int32_t lmax;
    const int32_t *col_len;
    const float *min_score;
    const float *width;
    int32_t nbins;
    unsigned long long *counts;  // ncols x nbins
};

__global__ void __launch_bounds__(256) score_hist_kernel(HistParams p)
{
    extern __shared__ __align__(16) uint8_t smem_hist[];
    const int cpb = p.cols_per_block;
    float *sP = reinterpret_cast<float *>(smem_hist);
    unsigned int *sH = reinterpret_cast<unsigned int *>(sP + (size_t)cpb * p.p_rows);
    uint8_t *sCode = reinterpret_cast<uint8_t *>(sH + (size_t)cpb * p.nbins);
    const int64_t p0 = (int64_t)blockIdx.x * blockDim.x;
    const int c0 = blockIdx.y * cpb;
    const int nc = min(cpb, p.ncols - c0);
    for (int i = threadIdx.x; i < nc * p.p_rows; i += blockDim.x) sP[i] = p.P[(size_t)c0 * p.p_rows + i];
    for (int i = threadIdx.x; i < nc * p.nbins; i += blockDim.x) sH[i] = 0;
    const int nwin = blockDim.x + p.lmax;
    for (int i = threadIdx.x; i < nwin; i += blockDim.x)
        sCode[i] = (uint8_t)base_code_at(p.seq2, p.zmask, p0 + i);
    __syncthreads();
    const int64_t pos = p0 + threadIdx.x;
    int64_t rem = 0;
    if (pos < p.n) rem = run_end_of(p.run_start, p.nruns, p.n, pos) - pos;
    const uint8_t *code = sCode + threadIdx.x;
    for (int cc = 0; cc < nc; ++cc) {
        const int L = __ldg(p.col_len + c0 + cc);
        if (L > rem) continue;
        const float *col = sP + (size_t)cc * p.p_rows;
        float s = 0.0f;
        for (int j = 0; j < L; ++j) {
            const int b = code[j];
            if (b < 4) s = __fadd_rn(s, col[4 * j + b]);
        }
        int bin = (int)__fdiv_rn(__fsub_rn(s, __ldg(p.min_score + c0 + cc)), __ldg(p.width + c0 + cc));
        bin = max(0, min(p.nbins - 1, bin));
        atomicAdd(&sH[cc * p.nbins + bin], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nc * p.nbins; i += blockDim.x)
        if (sH[i]) atomicAdd(&p.counts[(size_t)c0 * p.nbins + i], (unsigned long long)sH[i]);
}

// ------------------------------------------------------------------------
// 3. rescoring of tensor-core candidates: run check + exact FP32 score
// ------------------------------------------------------------------------
struct RescoreParams {
    const unsigned long long *cand;
    const unsigned long long *cand_count;
    int64_t cand_cap;
    const uint32_t *seq2;
    const uint32_t *zmask;
    int64_t n;
    const int64_t *run_start;
    int64_t nruns;
    const float *P;
    int32_t p_rows;
    const int32_t *col_len;
    const float *thr;
    void *hits;
    unsigned long long *hit_count;
    int64_t hit_cap;
};

__global__ void __launch_bounds__(256) rescore_kernel(RescoreParams p)
{
    unsigned long long nc = *p.cand_count;
    if ((int64_t)nc > p.cand_cap) nc = (unsigned long long)p.cand_cap;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < nc;
         base += stride) {
        unsigned long long i = base + threadIdx.x;
        bool hit = false;
        int64_t pos = 0;
        int32_t col = 0;
        float s = 0.0f;
        if (i < nc) {
            unsigned long long c = p.cand[i];
            pos = (int64_t)(c >> kColBits);
            col = (int32_t)(c & ((1u << kColBits) - 1u));
            const int L = __ldg(p.col_len + col);
            if (pos + L <= run_end_of(p.run_start, p.nruns, p.n, pos)) {
                const float *pc = p.P + (size_t)col * p.p_rows;
                for (int j = 0; j < L; ++j) {
                    int b = base_code_at(p.seq2, p.zmask, pos + j);
                    if (b < 4) s = __fadd_rn(s, __ldg(pc + 4 * j + b));
                }
                hit = s >= __ldg(p.thr + col);
            }
        }
        emit_hits_warp(hit, pos, col, s, reinterpret_cast<HitRec *>(p.hits), p.hit_count,
                       p.hit_cap);
    }
}

// ------------------------------------------------------------------------
// 4. the reference's filterScore (kernel.cu:21-34), for the drop-in entry point
// ------------------------------------------------------------------------
__global__ void filter_score_kernel(const float *R, int m, int n, const float *threshold,
                                    int *occIdx, float *occScore, int *nOcc)
{
    const long long total = (long long)m * n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < total; base += stride) {
        long long idx = base + threadIdx.x;
        bool hit = false;
        float v = 0.0f;
        if (idx < total) {
            int j = (int)(idx / m);
            v = R[idx];
            hit = v >= threshold[j];
        }
        unsigned msk = __ballot_sync(0xffffffffu, hit);
        if (!msk) continue;
        int lane = threadIdx.x & 31, leader = __ffs(msk) - 1;
        int b = 0;
        if (lane == leader) b = atomicAdd(nOcc, __popc(msk));
        b = __shfl_sync(0xffffffffu, b, leader);
        if (hit) {
            int slot = b + __popc(msk & ((1u << lane) - 1u));
            occScore[slot] = v;
            occIdx[slot] = (int)idx;
        }
    }
}

// ------------------------------------------------------------------------
// 5. the fused tensor-core scan (tcgen05 + TMA + TMEM), persistent
// ------------------------------------------------------------------------
//
// Score of motif column c at position p:  sum_j P(4j + base(p+j), c).
// With W the one-hot window matrix, W[r][4i+b] = [base(m0 + r + i) == b] for
// i < 8, the 128 x N tile of scores of M tile m0 is
//     D = sum_g  W[8*(g/2) : 8*(g/2)+128, 16*(g%2) : 16*(g%2)+16] * B_g
// where B_g holds rows 16g..16g+15 of P (motif bases 4g..4g+3): the shift of
// the motif's k-th 4-base group is a row offset of the A descriptor, so W is
// built once per M tile and never expanded further.  P enters as one or two
// fixed-point BF16 terms (hi, lo) whose partial sums are exactly
// representable in FP32, so the tensor-core accumulation is exact; the guard
// band bounds only the quantisation and the reference's own FP32 rounding.
//
// Roles (192 threads): warps 0-3 drain TMEM (lane quarter = warp), compare
// against the guard-banded thresholds and stage candidates; warp 4 allocates
// TMEM and one lane issues the MMAs and the TMA bulk copies of B tiles;
// warp 5 builds the one-hot W tiles from the 2-bit stream.  Two W stages and
// two TMEM accumulators keep the roles overlapped.  Jobs (N tile, M tile) are
// statically interleaved over the persistent CTAs, N-tile major, so each CTA
// reloads B only when its N tile changes.

struct TcSmem {
    // offsets (bytes) into dynamic shared memory
    uint32_t b_hi, b_lo, w0, w1, thr, cand, codes, tiles, pairtab, bars, misc, total;
};

__host__ __device__ inline TcSmem tc_smem_layout(uint32_t b_term_max, int terms, int wrows,
                                                 int nslots, int ntiles)
{
    TcSmem L;
    uint32_t o = 0;
    auto take = [&](uint32_t bytes, uint32_t align) {
        o = (o + align - 1) / align * align;
        uint32_t r = o;
        o += bytes;
        return r;
    };
    L.b_hi = take(b_term_max, 1024);
    L.b_lo = take(terms == 2 ? b_term_max : 0, 1024);
    L.w0 = take((uint32_t)wrows * kWRowBytes, 1024);
    L.w1 = take((uint32_t)wrows * kWRowBytes, 1024);
    L.thr = take((uint32_t)nslots * 4, 16);
    L.cand = take(4 * kCandBuf * 8, 16);
    L.codes = take((uint32_t)(wrows + 64), 16);
    L.tiles = take((uint32_t)ntiles * sizeof(TileDesc), 16);
    L.pairtab = take(25 * 16, 16);
    L.bars = take(16 * 8, 8);
    L.misc = take(64, 16);
    L.total = take(0, 1024) + 1024;  // + slack for runtime base alignment
    return L;
}

enum { BAR_WFULL = 0, BAR_WEMPTY = 2, BAR_AFULL = 4, BAR_AEMPTY = 6, BAR_BFULL = 8, BAR_DRAIN = 9 };

__global__ void __launch_bounds__(kTcThreads, 1) scan_tc_kernel(TcParams p)
{
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte aligned base
    uint8_t *smem = smem_raw + ((1024 - (ptx::smem_addr(smem_raw) & 1023)) & 1023);
    const TcSmem L = tc_smem_layout(p.b_term_max, p.terms, p.wrows, p.nslots, p.ntiles);
    const uint32_t sbase = ptx::smem_addr(smem);
    float *s_thr = reinterpret_cast<float *>(smem + L.thr);
    unsigned long long *s_cand = reinterpret_cast<unsigned long long *>(smem + L.cand);
    uint8_t *s_codes = smem + L.codes;
    TileDesc *s_tiles = reinterpret_cast<TileDesc *>(smem + L.tiles);
    uint4 *s_pair = reinterpret_cast<uint4 *>(smem + L.pairtab);
    const uint32_t bars = sbase + L.bars;
    volatile int *s_abort = reinterpret_cast<volatile int *>(smem + L.misc);
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(smem + L.misc + 4);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // ---- set-up
    for (int i = threadIdx.x; i < p.nslots; i += blockDim.x) s_thr[i] = p.thr_adj[i];
    for (int i = threadIdx.x; i < p.ntiles * (int)(sizeof(TileDesc) / 4); i += blockDim.x)
        reinterpret_cast<int32_t *>(s_tiles)[i] = reinterpret_cast<const int32_t *>(p.tiles)[i];
    if (threadIdx.x < 25) {
        // one-hot of a base pair (b0, b1), 4 bf16 channels each; code 4 = zero
        int b0 = threadIdx.x / 5, b1 = threadIdx.x % 5;
        uint32_t w[4] = {0, 0, 0, 0};
        if (b0 < 4) w[b0 >> 1] |= 0x3F80u << (16 * (b0 & 1));
        if (b1 < 4) w[2 + (b1 >> 1)] |= 0x3F80u << (16 * (b1 & 1));
        s_pair[threadIdx.x] = make_uint4(w[0], w[1], w[2], w[3]);
    }
    if (threadIdx.x == 0) {
        *s_abort = 0;
        ptx::mbar_init(bars + 8 * (BAR_WFULL + 0), 1);
        ptx::mbar_init(bars + 8 * (BAR_WFULL + 1), 1);
        ptx::mbar_init(bars + 8 * (BAR_WEMPTY + 0), 1);
        ptx::mbar_init(bars + 8 * (BAR_WEMPTY + 1), 1);
        ptx::mbar_init(bars + 8 * (BAR_AFULL + 0), 1);
        ptx::mbar_init(bars + 8 * (BAR_AFULL + 1), 1);
        ptx::mbar_init(bars + 8 * (BAR_AEMPTY + 0), 4);
        ptx::mbar_init(bars + 8 * (BAR_AEMPTY + 1), 4);
        ptx::mbar_init(bars + 8 * BAR_BFULL, 1);
        ptx::mbar_init(bars + 8 * BAR_DRAIN, 1);
        ptx::fence_mbar_init();
    }
    if (warp == 4) {
        ptx::tmem_alloc(ptx::smem_addr(s_tmem), p.tmem_cols);
        ptx::tmem_relinquish();
        ptx::tc_fence_before();
    }
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem_base = *s_tmem;
    const long long njobs = (long long)p.ntiles * p.n_mtiles;

    if (warp == 4) {
        // =========================== MMA issuer ===========================
        if (lane == 0) {
            int cur_tile = -1;
            uint32_t bphase = 0, dphase = 0, idesc = 0, g_steps = 0, sbo_b = 0;
            uint32_t jc = 0;
            bool ok = true;
            for (long long job = blockIdx.x; job < njobs && ok; job += gridDim.x, ++jc) {
                const int tile = (int)(job / p.n_mtiles);
                if (tile != cur_tile) {
                    if (cur_tile >= 0) {  // every MMA reading the old B must be done
                        ptx::mma_commit(bars + 8 * BAR_DRAIN);
                        ok = ptx::mbar_wait(bars + 8 * BAR_DRAIN, dphase, s_abort, p.wait_limit);
                        dphase ^= 1;
                        if (!ok) break;
                    }
                    const TileDesc td = s_tiles[tile];
                    ptx::mbar_arrive_expect_tx(bars + 8 * BAR_BFULL, (uint32_t)td.b_bytes * p.terms);
                    ptx::bulk_g2s(sbase + L.b_hi, p.bbuf + td.b_off, (uint32_t)td.b_bytes,
                                  bars + 8 * BAR_BFULL);
                    if (p.terms == 2)
                        ptx::bulk_g2s(sbase + L.b_lo, p.bbuf + td.b_off + td.b_bytes,
                                      (uint32_t)td.b_bytes, bars + 8 * BAR_BFULL);
                    ok = ptx::mbar_wait(bars + 8 * BAR_BFULL, bphase, s_abort, p.wait_limit);
                    bphase ^= 1;
                    if (!ok) break;
                    cur_tile = tile;
                    g_steps = (uint32_t)td.g;
                    idesc = ptx::idesc_bf16_f32(kBM, (uint32_t)td.n);
                    sbo_b = 256u * g_steps;  // bytes between 8-column groups of B
                }
                const uint32_t s = jc & 1u, ph = (jc >> 1) & 1u;
                ok = ptx::mbar_wait(bars + 8 * (BAR_AEMPTY + s), ph ^ 1u, s_abort, p.wait_limit) &&
                     ptx::mbar_wait(bars + 8 * (BAR_WFULL + s), ph, s_abort, p.wait_limit);
                if (!ok) break;
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem_base + s * (p.tmem_cols >> 1);
                const uint32_t w_addr = sbase + (s ? L.w1 : L.w0);
                for (uint32_t g = 0; g < g_steps; ++g) {
                    // A: W rows shifted by 8*(g/2), channels of bases 4*(g%2)..+3
                    const uint64_t adesc =
                        ptx::smem_desc(w_addr + (g >> 1) * 512u + (g & 1u) * 256u, 128u, 512u);
                    const uint64_t bdesc_hi = ptx::smem_desc(sbase + L.b_hi + g * 256u, 128u, sbo_b);
                    ptx::mma_bf16(d_tmem, adesc, bdesc_hi, idesc, g > 0);
                    if (p.terms == 2) {
                        const uint64_t bdesc_lo =
                            ptx::smem_desc(sbase + L.b_lo + g * 256u, 128u, sbo_b);
                        ptx::mma_bf16(d_tmem, adesc, bdesc_lo, idesc, 1u);
                    }
                }
                ptx::mma_commit(bars + 8 * (BAR_WEMPTY + s));
                ptx::mma_commit(bars + 8 * (BAR_AFULL + s));
            }
            // drain: nothing may still write TMEM when it is freed
            ptx::mma_commit(bars + 8 * BAR_DRAIN);
            if (!ptx::mbar_wait(bars + 8 * BAR_DRAIN, dphase, s_abort, p.wait_limit)) *s_abort = 1;
        }
        __syncwarp();
    } else if (warp == 5) {
        // ========================== W builder =============================
        uint32_t jc = 0;
        for (long long job = blockIdx.x; job < njobs; job += gridDim.x, ++jc) {
            const int tile = (int)(job / p.n_mtiles);
            const int64_t m = job % p.n_mtiles;
            const int g = s_tiles[tile].g;
            const int rows = kBM + 8 * (((g + 1) >> 1) - 1);
            const uint32_t s = jc & 1u, ph = (jc >> 1) & 1u;
            if (!ptx::mbar_wait(bars + 8 * (BAR_WEMPTY + s), ph ^ 1u, s_abort, p.wait_limit)) break;
            // decode bases [m*128, m*128 + rows + 8) into byte codes
            const int64_t b0 = m * kBM;
            const int nchunks = (rows + kWinBases + 31) >> 5;
            for (int c = lane; c < nchunks; c += 32) {
                const int64_t q = b0 + 32 * c;  // multiple of 32
                const uint32_t lo = __ldg(p.seq2 + (q >> 4)), hi = __ldg(p.seq2 + (q >> 4) + 1);
                const uint32_t z = __ldg(p.zmask + (q >> 5));
                uint32_t packed[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    uint32_t v = 0;
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const int i = 4 * k + t;
                        uint32_t code = ((i < 16 ? (lo >> (2 * i)) : (hi >> (2 * (i - 16)))) & 3u);
                        if ((z >> i) & 1u) code = 4;
                        v |= code << (8 * t);
                    }
                    packed[k] = v;
                }
                uint4 *dst = reinterpret_cast<uint4 *>(s_codes + 32 * c);
                dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
            }
            __syncwarp();
            uint8_t *w = smem + (s ? L.w1 : L.w0);
            for (int r = lane; r < rows; r += 32) {
                uint8_t *row = w + (r >> 3) * 512 + (r & 7) * 16;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int c0 = s_codes[r + 2 * k], c1 = s_codes[r + 2 * k + 1];
                    *reinterpret_cast<uint4 *>(row + k * 128) = s_pair[c0 * 5 + c1];
                }
            }
            ptx::fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(bars + 8 * (BAR_WFULL + s));
        }
    } else {
        // ===================== epilogue (warps 0-3) =======================
        const int q = warp;  // TMEM lanes 32q .. 32q+31
        unsigned long long *buf = s_cand + q * kCandBuf;
        int fill = 0;
        auto flush = [&]() {
            __syncwarp();
            unsigned long long gb = 0;
            if (lane == 0 && fill > 0) gb = atomicAdd(p.cand_count, (unsigned long long)fill);
            gb = __shfl_sync(0xffffffffu, gb, 0);
            for (int i = lane; i < fill; i += 32)
                if ((int64_t)(gb + i) < p.cand_cap) p.cand[gb + i] = buf[i];
            __syncwarp();
            fill = 0;
        };
        uint32_t jc = 0;
        for (long long job = blockIdx.x; job < njobs; job += gridDim.x, ++jc) {
            const int tile = (int)(job / p.n_mtiles);
            const int64_t m = job % p.n_mtiles;
            const TileDesc td = s_tiles[tile];
            const uint32_t s = jc & 1u, ph = (jc >> 1) & 1u;
            if (!ptx::mbar_wait(bars + 8 * (BAR_AFULL + s), ph, s_abort, p.wait_limit)) break;
            ptx::tc_fence_after();
            const int64_t pos = m * kBM + q * 32 + lane;
            const bool valid = pos < p.n;
            const uint32_t taddr = tmem_base + ((uint32_t)(q * 32) << 16) + s * (p.tmem_cols >> 1);
            const bool dump_row =
                p.dump != nullptr && pos >= p.dump_p0 && pos < p.dump_p0 + p.dump_npos;
            for (int ch = 0; ch < td.n / 32; ++ch) {
                uint32_t v[32];
                ptx::tmem_ld_32x32b_x32(taddr + ch * 32, v);
                ptx::tmem_wait_ld();
                const float4 *th4 = reinterpret_cast<const float4 *>(s_thr + td.slot0 + ch * 32);
                uint32_t mask = 0;
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const float4 t = th4[k];
                    mask |= (__uint_as_float(v[4 * k + 0]) >= t.x ? 1u : 0u) << (4 * k + 0);
                    mask |= (__uint_as_float(v[4 * k + 1]) >= t.y ? 1u : 0u) << (4 * k + 1);
                    mask |= (__uint_as_float(v[4 * k + 2]) >= t.z ? 1u : 0u) << (4 * k + 2);
                    mask |= (__uint_as_float(v[4 * k + 3]) >= t.w ? 1u : 0u) << (4 * k + 3);
                }
                if (!valid) mask = 0;
                if (dump_row) {
                    for (int i = 0; i < 32; ++i) {
                        const int col = __ldg(p.slot_col + td.slot0 + ch * 32 + i);
                        if (col >= 0)
                            p.dump[(pos - p.dump_p0) * p.dump_ncols + col] = __uint_as_float(v[i]);
                    }
                }
                if (__any_sync(0xffffffffu, mask != 0)) {
                    const int cnt = __popc(mask);
                    int incl = cnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int t = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= o) incl += t;
                    }
                    const int total = __shfl_sync(0xffffffffu, incl, 31);
                    int at = incl - cnt;
                    if (fill + total > kCandBuf) flush();
                    if (total > kCandBuf) {
                        unsigned long long gb = 0;
                        if (lane == 0) gb = atomicAdd(p.cand_count, (unsigned long long)total);
                        gb = __shfl_sync(0xffffffffu, gb, 0);
                        while (mask) {
                            const int i = __ffs(mask) - 1;
                            mask &= mask - 1;
                            const unsigned long long c =
                                ((unsigned long long)pos << kColBits) |
                                (unsigned long long)__ldg(p.slot_col + td.slot0 + ch * 32 + i);
                            if ((int64_t)(gb + at) < p.cand_cap) p.cand[gb + at] = c;
                            ++at;
                        }
                    } else {
                        while (mask) {
                            const int i = __ffs(mask) - 1;
                            mask &= mask - 1;
                            buf[fill + at] =
                                ((unsigned long long)pos << kColBits) |
                                (unsigned long long)__ldg(p.slot_col + td.slot0 + ch * 32 + i);
                            ++at;
                        }
                        fill += total;
                    }
                    __syncwarp();
                }
            }
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(bars + 8 * (BAR_AEMPTY + s));
        }
        flush();
    }

    // ---- teardown
    __syncthreads();
    if (threadIdx.x == 0 && *s_abort) atomicOr(p.status, 1);
    if (warp == 4) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem_base, p.tmem_cols);
    }
}

}  // namespace blamm
