// scan_kernels.cuh -- SIMT device code of the GB300 PWM scan: stream packing,
// the plain FP32 scan, empirical histograms, candidate rescoring and the
// reference-compatible threshold filter.  The tensor-core scan is scan_tc.cuh.
//
// Data layout in HBM (one species' filtered base stream of n positions):
//   seq2[]  : 2-bit base codes, 16 per uint32 (A=0 C=1 G=2 T=3), base i at
//             bits 2*(i%16) of word i/16;
//   zmask[] : 1 bit per base, bit i%32 of word i/32 set when the base adds
//             nothing to a score (lowercase, or past the end of the stream);
//   both padded by kStreamPad bases so that tile loads need no bounds checks.
// Motif bank: the reference's column-major FP32 P (4*Lmax rows), per-column
// lengths and thresholds.
#pragma once
#include <cstdint>

#include "blamm_gpu.h"

#include "ptx_sm100.cuh"

namespace blamm {

constexpr int kStreamPad = 2048;   // padding bases after the stream end
constexpr int kMaxMotifLen = BLAMM_MAX_MOTIF_LEN;  // the plain kernel reads up to 255 + L bases past a block
constexpr int kColBits = 20;       // tensor-core candidate = pos << 20 | tile slot

// ------------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------------
__device__ __forceinline__ int base_code_at(const uint32_t *seq2, const uint32_t *zmask, int64_t i)
{
    uint32_t z = (zmask[i >> 5] >> (i & 31)) & 1u;
    uint32_t b = (seq2[i >> 4] >> (2 * (i & 15))) & 3u;
    return z ? 4 : (int)b;
}

// Sequential FP32 score of the window at pos (motif position order, __fadd_rn: the
// reference's sum), zero-masked bases adding nothing.  The 2-bit codes and mask bits of
// 16 positions come from two words of each array (the padded stream covers the reads).
__device__ __forceinline__ float window_score(const uint32_t *seq2, const uint32_t *zmask, const float *pc,
                                              int64_t pos, int L)
{
    float s = 0.0f;
    for (int j = 0; j < L; j += 16) {
        const int64_t q = pos + j;
        const int64_t w = q >> 4, wz = q >> 5;
        const uint64_t cw = (uint64_t)__ldg(seq2 + w) | ((uint64_t)__ldg(seq2 + w + 1) << 32);
        const uint64_t zw = (uint64_t)__ldg(zmask + wz) | ((uint64_t)__ldg(zmask + wz + 1) << 32);
        const uint32_t codes = (uint32_t)(cw >> (2 * (q & 15)));
        const uint32_t zero = (uint32_t)(zw >> (q & 31));
        const int cnt = min(16, L - j);
        for (int k = 0; k < cnt; ++k)
            if (!((zero >> k) & 1u)) s = __fadd_rn(s, __ldg(pc + 4 * (j + k) + ((codes >> (2 * k)) & 3u)));
    }
    return s;
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

// One-hot entries for the tensor-core scan: E[i] = onehot(base i) ++ onehot(base i+1),
// 4 bf16 channels per base (1.0 = 0x3F80 in channel code, zeros for a zero-masked base).
__device__ __forceinline__ uint2 onehot_bf16(uint32_t code, uint32_t zero)
{
    const uint32_t h = zero ? 0u : (0x3F80u << ((code & 1u) << 4));
    return make_uint2((code & 2u) ? 0u : h, (code & 2u) ? h : 0u);
}

// E4M3 one-hot of one base: byte `code` of the 4 is 1.0 (0x38), zeros for a zero-masked base.
__device__ __forceinline__ uint32_t onehot_e4m3(uint32_t code, uint32_t zero)
{
    return zero ? 0u : 0x38u << (8 * code);
}

// E4M3 entries of one window: e8[i] = one-hot of bases base + i .. base + i + 3 (4 bytes
// each, in that order: K slots 4u + code), i < ne.
__global__ void e8_kernel(const uint32_t *__restrict__ seq2, const uint32_t *__restrict__ zmask, int64_t base,
                          int64_t ne, uint4 *__restrict__ e8)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ne) return;
    uint32_t w[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int64_t i = base + t + u;
        w[u] = onehot_e4m3((seq2[i >> 4] >> (2 * (i & 15))) & 3u, (zmask[i >> 5] >> (i & 31)) & 1u);
    }
    e8[t] = make_uint4(w[0], w[1], w[2], w[3]);
}

// Entries of one window of the stream: e16[i] = entry of position base + i, i < ne.
__global__ void e16_kernel(const uint32_t *__restrict__ seq2, const uint32_t *__restrict__ zmask, int64_t base,
                           int64_t ne, uint4 *__restrict__ e16)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ne) return;
    const int64_t i = base + t, j = i + 1;
    const uint2 a = onehot_bf16((seq2[i >> 4] >> (2 * (i & 15))) & 3u, (zmask[i >> 5] >> (i & 31)) & 1u);
    const uint2 b = onehot_bf16((seq2[j >> 4] >> (2 * (j & 15))) & 3u, (zmask[j >> 5] >> (j & 31)) & 1u);
    e16[t] = make_uint4(a.x, a.y, b.x, b.y);
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
    const int32_t *cols;  // the ncols bank columns to scan (nullptr: columns 0 .. ncols-1)
    void *hits;  // blamm_hit*
    unsigned long long *hit_count;
    int64_t hit_cap;
    int64_t keep_below;  // hits at positions >= keep_below are dropped (0: none are)
    int64_t pos_base;    // added to the positions written
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
    for (int i = threadIdx.x; i < nc * p.p_rows; i += blockDim.x) {
        const int cc = i / p.p_rows;
        const int col = p.cols ? p.cols[c0 + cc] : c0 + cc;
        sP[i] = p.P[(size_t)col * p.p_rows + (i - cc * p.p_rows)];
    }
    for (int i = threadIdx.x; i < nc; i += blockDim.x) {
        const int col = p.cols ? p.cols[c0 + i] : c0 + i;
        sLen[i] = p.col_len[col];
        sThr[i] = p.thr[col];
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
            hit = s >= sThr[cc] && (p.keep_below == 0 || pos < p.keep_below);
        }
        emit_hits_warp(hit, pos + p.pos_base, p.cols ? p.cols[c0 + cc] : c0 + cc, s,
                       reinterpret_cast<HitRec *>(p.hits), p.hit_count, p.hit_cap);
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
// Candidates come as 16-byte records {M tile m, row | slot << 7, mask, 0}: the position is
// m * 128 + row, slot the first tile slot of a 32-column chunk, bit i of mask = slot + i is a
// candidate.  The scan
// writes them in blocks of kRecBlockSlots slots; slot 0 of a block holds the number of
// records that follow it (the rest of the block is unused).
constexpr int kRecBlockSlots = 128;

struct RescoreParams {
    const uint4 *cand;                // record slots
    const int32_t *slot_col;          // tile slot -> motif column
    const unsigned long long *cand_count;  // record slots reserved
    int64_t cand_cap;                 // record slots available
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
    int64_t keep_below;  // hits at positions >= keep_below are dropped (0: none are)
    int64_t pos_base;    // added to the positions written
};

// One thread per record slot; the candidates of a warp's 32 records are then shared out
// over its lanes (a prefix sum of the masks' bit counts), 32 at a time, so that a record
// with several candidates does not leave the other lanes idle.
__global__ void __launch_bounds__(256) rescore_kernel(RescoreParams p)
{
    unsigned long long ns = *p.cand_count;
    if ((int64_t)ns > p.cand_cap) ns = (unsigned long long)p.cand_cap;
    const int lane = threadIdx.x & 31;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < ns; base += stride) {
        const unsigned long long i = base + threadIdx.x;
        uint32_t mask = 0u, mt = 0u, ry = 0u;
        const unsigned long long b = i & ~(unsigned long long)(kRecBlockSlots - 1);
        const uint32_t k = (uint32_t)(i & (kRecBlockSlots - 1));
        if (i < ns && k != 0u && k <= __ldg(&p.cand[b].x)) {
            const uint4 r = p.cand[i];
            mt = r.x;
            ry = r.y;
            mask = r.z;
        }
        const int c = __popc(mask);
        int incl = c;  // inclusive prefix sum of the lanes' candidate counts
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        for (int t0 = 0; t0 < total; t0 += 32) {
            const int t = t0 + lane;
            // the lane r whose record holds candidate t: the first with incl[r] > t
            int r = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int v = __shfl_sync(0xffffffffu, incl, r + step - 1);
                if (v <= t) r += step;
            }
            const uint32_t rmask = __shfl_sync(0xffffffffu, mask, r);
            const uint32_t rmt = __shfl_sync(0xffffffffu, mt, r);
            const uint32_t rry = __shfl_sync(0xffffffffu, ry, r);
            const int before = __shfl_sync(0xffffffffu, incl, r) - __shfl_sync(0xffffffffu, c, r);
            bool hit = false;
            int64_t pos = 0;
            int32_t col = 0;
            float s = 0.0f;
            if (t < total) {
                const int bit = (int)__fns(rmask, 0u, t - before + 1);  // its (t - before)-th set bit
                pos = (int64_t)rmt * 128 + (rry & 127u);
                col = __ldg(p.slot_col + (int32_t)(rry >> 7) + bit);
                const int L = __ldg(p.col_len + col);
                if (pos + L <= run_end_of(p.run_start, p.nruns, p.n, pos)) {
                    s = window_score(p.seq2, p.zmask, p.P + (size_t)col * p.p_rows, pos, L);
                    hit = s >= __ldg(p.thr + col) && (p.keep_below == 0 || pos < p.keep_below);
                }
            }
            emit_hits_warp(hit, pos + p.pos_base, col, s, reinterpret_cast<HitRec *>(p.hits), p.hit_count,
                           p.hit_cap);
        }
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

}  // namespace blamm
