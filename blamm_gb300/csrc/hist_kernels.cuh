// hist_kernels.cuh -- the hist module's theoretical score distributions and
// their p-value inversion on the GPU (one CTA per motif column).
//
// Follows, operation for operation in FP32 (no contraction: __fmul_rn /
// __fadd_rn), the reference's
//   Motif::computeTheoreticalSpectrum  src/motif.cpp:151-192
//     a = nbins / (max - min), b = -a*min / L, q = round(a*PWM + b),
//     DP over positions with std::map<int, float> (a key exists once touched;
//     each key's float sum takes its terms in ascending source key, then base);
//   Histogram::generateTheoreticalHist src/hist.cpp:162-175
//     spectrum map<float, float>: score = (key - L*b) / a, insert keeps the
//     first of equal scores; setNumObservations overwrites the bin with
//     (size_t)(maxLength * probability) (src/motif.h:109-115);
//   ScoreHistogram::getScoreCutoff src/motif.cpp:47-69, in FP64.
// so thresholds equal the host's (and the reference's) bit for bit.  With
// fp64_dp the DP runs in FP64 instead (a more accurate distribution; not the
// reference's numbers).
#pragma once
#include <cstdint>

namespace blamm {

struct TheoHistParams {
    const float *P;         // column-major, p_rows x ncols
    int32_t p_rows;
    int32_t ncols;
    const int32_t *col_len;
    const int32_t *hist_of;  // column whose PWM gives column c's distribution
    float bg[4];
    int32_t nbins;
    uint64_t max_length;
    int32_t fp64_dp;
    int32_t kmax;            // capacity of the key arrays (entries)
    const float *pvalues;
    int32_t npv;
    float *thr;              // npv x ncols (or nullptr)
    unsigned long long *counts;  // ncols x nbins (or nullptr)
    int *status;             // set to 1 when a column's key range exceeds kmax
};

// Shared memory: q[4 * 1024] ints, two value arrays of kmax (float or double),
// two presence arrays of kmax bytes, nbins counts.
__host__ __device__ inline size_t theo_smem_bytes(int kmax, int nbins, int fp64)
{
    const size_t v = fp64 ? 8 : 4;
    return 4 * 1024 * 4 + 2 * (size_t)kmax * v + 2 * (size_t)kmax + 8 * (size_t)nbins + 64;
}

template <typename T>
__device__ __forceinline__ T theo_mul(T a, T b);
template <>
__device__ __forceinline__ float theo_mul<float>(float a, float b) { return __fmul_rn(a, b); }
template <>
__device__ __forceinline__ double theo_mul<double>(double a, double b) { return __dmul_rn(a, b); }
template <typename T>
__device__ __forceinline__ T theo_add(T a, T b);
template <>
__device__ __forceinline__ float theo_add<float>(float a, float b) { return __fadd_rn(a, b); }
template <>
__device__ __forceinline__ double theo_add<double>(double a, double b) { return __dadd_rn(a, b); }

template <typename T>
__device__ void theo_column(const TheoHistParams &p, int c, uint8_t *smem)
{
    const int h = p.hist_of[c];
    const int L = p.col_len[h];
    const float *pwm = p.P + (size_t)h * p.p_rows;
    int *q = reinterpret_cast<int *>(smem);
    T *cur = reinterpret_cast<T *>(smem + 4 * 1024 * 4);
    T *nxt = cur + p.kmax;
    uint8_t *pc = reinterpret_cast<uint8_t *>(nxt + p.kmax);
    uint8_t *pn = pc + p.kmax;
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(
        (reinterpret_cast<uintptr_t>(pn + p.kmax) + 15) & ~uintptr_t(15));
    __shared__ float s_min, s_max, s_a, s_b;
    __shared__ int s_base, s_w;
    __shared__ int8_t s_ord[1024][4];

    if (threadIdx.x == 0) {
        // Motif::getMinScore / getMaxScore: sequential float sums of the row extremes
        float mn = 0.0f, mx = 0.0f;
        for (int j = 0; j < L; ++j) {
            const float *r = pwm + 4 * j;
            mn = __fadd_rn(mn, fminf(fminf(r[0], r[1]), fminf(r[2], r[3])));
            mx = __fadd_rn(mx, fmaxf(fmaxf(r[0], r[1]), fmaxf(r[2], r[3])));
        }
        const float range = __fadd_rn(mx, -mn);
        const float a = __fdiv_rn((float)p.nbins, range);
        const float b = __fdiv_rn(__fmul_rn(-a, mn), (float)L);
        s_min = mn;
        s_max = mx;
        s_a = a;
        s_b = b;
    }
    __syncthreads();
    const float a = s_a, b = s_b;
    for (int i = threadIdx.x; i < 4 * L; i += blockDim.x) q[i] = (int)roundf(__fadd_rn(__fmul_rn(a, pwm[i]), b));
    __syncthreads();
    if (threadIdx.x == 0) {
        // bounds of every reachable key, and per position the order in which a key's
        // terms arrive: ascending source key = descending q, ties by base
        long long plo = 0, phi = 0, qmin = 0, qmax = 0;
        for (int j = 0; j < L; ++j) {
            int lo = q[4 * j], hi = q[4 * j];
            for (int k = 1; k < 4; ++k) {
                lo = min(lo, q[4 * j + k]);
                hi = max(hi, q[4 * j + k]);
            }
            plo += lo;
            phi += hi;
            if (j == 0 || plo < qmin) qmin = plo;
            if (j == 0 || phi > qmax) qmax = phi;
            int8_t o[4] = {0, 1, 2, 3};
            for (int x = 1; x < 4; ++x)
                for (int y = x; y > 0 && q[4 * j + o[y]] > q[4 * j + o[y - 1]]; --y) {
                    const int8_t t = o[y];
                    o[y] = o[y - 1];
                    o[y - 1] = t;
                }
            for (int k = 0; k < 4; ++k) s_ord[j][k] = o[k];
        }
        const long long w = qmax - qmin + 1;
        s_base = (int)qmin;
        s_w = w > p.kmax ? -1 : (int)w;
    }
    __syncthreads();
    const int W = s_w, base = s_base;
    if (W < 0) {
        if (threadIdx.x == 0) atomicOr(p.status, 1);
        return;
    }
    for (int i = threadIdx.x; i < W; i += blockDim.x) {
        cur[i] = T(0);
        pc[i] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; ++k) {  // position 0, bases in order
            const int t = q[k] - base;
            cur[t] = theo_add<T>(cur[t], (T)p.bg[k]);
            pc[t] = 1;
        }
    __syncthreads();
    for (int j = 1; j < L; ++j) {
        for (int t = threadIdx.x; t < W; t += blockDim.x) {
            T s = T(0);
            uint8_t present = 0;
#pragma unroll
            for (int x = 0; x < 4; ++x) {
                const int k = s_ord[j][x];
                const int src = t - q[4 * j + k];
                if (src >= 0 && src < W && pc[src]) {
                    s = theo_add<T>(s, theo_mul<T>(cur[src], (T)p.bg[k]));
                    present = 1;
                }
            }
            nxt[t] = s;
            pn[t] = present;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < W; t += blockDim.x) {
            cur[t] = nxt[t];
            pc[t] = pn[t];
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < p.nbins; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        const float mn = s_min, mx = s_max;
        const float width = __fdiv_rn(__fadd_rn(mx, -mn), (float)p.nbins);
        const float lb = __fmul_rn((float)L, b);
        const float maxlen = (float)p.max_length;
        bool have_prev = false;
        float prev = 0.0f;
        for (int t = 0; t < W; ++t) {
            if (!pc[t]) continue;
            const float score = __fdiv_rn(__fadd_rn((float)(t + base), -lb), a);
            if (have_prev && score == prev) continue;  // map::insert keeps the first
            have_prev = true;
            prev = score;
            unsigned long long n;
            if (sizeof(T) == 4) n = (unsigned long long)__fmul_rn(maxlen, (float)cur[t]);
            else n = (unsigned long long)__dmul_rn((double)p.max_length, (double)cur[t]);
            int bin = (int)__fdiv_rn(__fadd_rn(score, -mn), width);
            bin = max(0, min(p.nbins - 1, bin));
            cnt[bin] = n;
        }
        if (p.counts)
            for (int i = 0; i < p.nbins; ++i) p.counts[(size_t)c * p.nbins + i] = cnt[i];
        if (p.thr) {
            double tot = 0.0;
            for (int i = 0; i < p.nbins; ++i) tot = __dadd_rn(tot, (double)cnt[i]);
            for (int v = 0; v < p.npv; ++v) {
                double curr = __dmul_rn((double)p.pvalues[v], tot);
                float cut = mx;
                for (int i = p.nbins - 1; i >= 0; --i) {
                    const double ci = (double)cnt[i];
                    if (ci < curr) {
                        curr = __dadd_rn(curr, -ci);
                    } else {
                        const double frac = __ddiv_rn(curr, ci);
                        const float cutoffi = (float)__dadd_rn(__dmul_rn(frac, (double)i),
                                                               __dmul_rn(__dadd_rn(1.0, -frac), (double)(i + 1)));
                        cut = __fadd_rn(__fmul_rn(cutoffi, width), mn);
                        break;
                    }
                }
                p.thr[(size_t)v * p.ncols + c] = cut;
            }
        }
    }
}

__global__ void __launch_bounds__(256) theoretical_hist_kernel(TheoHistParams p)
{
    extern __shared__ __align__(16) uint8_t smem_theo[];
    if (p.fp64_dp) theo_column<double>(p, blockIdx.x, smem_theo);
    else theo_column<float>(p, blockIdx.x, smem_theo);
}

}  // namespace blamm
