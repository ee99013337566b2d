// ingest_kernels.cuh -- FASTA text -> filtered base stream + run table on the GPU.
//
// The same stream and markers the host's FastaStream builds (FastaBatch,
// src/sequence.cpp:142-293): lines split at '\n'; a line starting with '>'
// opens a sequence; every other character of a sequence line (including 'N',
// '\r' and other non-bases) advances the position in the sequence; the
// stream holds the A/C/G/T/a/c/g/t characters; a run (SeqBlock marker,
// src/sequence.cpp:35-50) starts where the stream position and the sequence
// position stop advancing together.
//
// Data-parallel form: per-byte flags, prefix scans (line starts by a max scan,
// header count, sequence characters and stream bases by sum scans), scatter of
// the bases with their (sequence, position), then run flags and their scan.
// Every pass is a coalesced streaming pass over HBM.
#pragma once
#include <cstdint>

namespace blamm {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;  // per thread
constexpr int kScanTile = kScanThreads * kScanItems;
// shared-memory index with one pad word per 32 (a thread's items are consecutive)
__device__ __forceinline__ int scan_pad(int k) { return k + (k >> 5); }

struct SumOp {
    __device__ __forceinline__ static int64_t identity() { return 0; }
    __device__ __forceinline__ static int64_t apply(int64_t a, int64_t b) { return a + b; }
};
struct MaxOp {
    __device__ __forceinline__ static int64_t identity() { return INT64_MIN; }
    __device__ __forceinline__ static int64_t apply(int64_t a, int64_t b) { return a > b ? a : b; }
};

// Inclusive scan of each tile of kScanTile values in place; the tile's total
// goes to partial[tile].
template <class Op>
__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(int64_t *v, int64_t n, int64_t *partial)
{
    __shared__ int64_t tile[kScanTile + kScanTile / 32];
    __shared__ int64_t warp_tot[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    for (int k = threadIdx.x; k < kScanTile; k += kScanThreads)
        tile[scan_pad(k)] = base + k < n ? v[base + k] : Op::identity();
    __syncthreads();
    int64_t run = Op::identity();
    const int first = threadIdx.x * kScanItems;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        run = Op::apply(run, tile[scan_pad(first + k)]);
        tile[scan_pad(first + k)] = run;
    }
    // exclusive scan of the threads' totals
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl = Op::apply(t, incl);
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    int64_t before = Op::identity();
    for (int w = 0; w < warp; ++w) before = Op::apply(before, warp_tot[w]);
    int64_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = Op::identity();
    const int64_t off = Op::apply(before, excl);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) tile[scan_pad(first + k)] = Op::apply(off, tile[scan_pad(first + k)]);
    __syncthreads();
    for (int k = threadIdx.x; k < kScanTile; k += kScanThreads)
        if (base + k < n) v[base + k] = tile[scan_pad(k)];
    if (threadIdx.x == kScanThreads - 1) partial[blockIdx.x] = tile[scan_pad(kScanTile - 1)];
}

// v[i] = op(prefix of the earlier tiles, v[i]), partial holding the inclusive
// scan of the tile totals.
template <class Op>
__global__ void scan_add_kernel(int64_t *v, int64_t n, const int64_t *partial)
{
    const int64_t t = blockIdx.x;
    if (t == 0) return;
    const int64_t pre = partial[t - 1];
    const int64_t base = t * kScanTile;
    for (int k = threadIdx.x; k < kScanTile; k += blockDim.x)
        if (base + k < n) v[base + k] = Op::apply(pre, v[base + k]);
}

__device__ __forceinline__ bool ingest_base(unsigned char c)
{
    const unsigned char u = c & 0xDFu;
    return u == 'A' || u == 'C' || u == 'G' || u == 'T';
}

// pass 1: line starts (as their index, for a max scan) and header starts (for a sum scan)
__global__ void ingest_lines_kernel(const char *raw, int64_t n, int64_t *ls, int64_t *hs)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const bool start = i == 0 || raw[i - 1] == '\n';
        ls[i] = start ? i : -1;
        hs[i] = start && raw[i] == '>';
    }
}

// pass 2: sequence characters and stream bases (flags for sum scans); sequence data
// before the first header sets *bad
__global__ void ingest_chars_kernel(const char *raw, int64_t n, const int64_t *LS, const int64_t *HC, int64_t *sc,
                                    int64_t *vb, int *bad)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const char c = raw[i];
        const bool in_header = raw[LS[i]] == '>';
        const bool seqchar = c != '\n' && !in_header;
        if (seqchar && HC[i] == 0) *bad = 1;
        sc[i] = seqchar;
        vb[i] = seqchar && ingest_base((unsigned char)c);
    }
}

// pass 3a: per sequence its header offset and the count of sequence characters before it
// (SC is the inclusive scan; a header byte is no sequence character)
__global__ void ingest_headers_kernel(const char *raw, int64_t n, const int64_t *HC, const int64_t *SC,
                                      int64_t *seq_sc0, int64_t *header_pos)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if ((i == 0 || raw[i - 1] == '\n') && raw[i] == '>') {
            const int64_t k = HC[i] - 1;
            header_pos[k] = i;
            seq_sc0[k] = SC[i];
        }
    }
}

// pass 3b: every stream base with its sequence and position in the sequence, and the
// A/C/G/T counts of the stream (Species::computeNucleotideComposition,
// src/species.cpp:31-61: case-insensitive), one atomic per warp and base
__global__ void ingest_bases_kernel(const char *raw, int64_t n, const int64_t *LS, const int64_t *HC,
                                    const int64_t *SC, const int64_t *VX, const int64_t *seq_sc0, char *bases,
                                    int64_t *bseq, int64_t *bpos, unsigned long long *nucl)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t start = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long cnt[4] = {0, 0, 0, 0};
    for (int64_t i = start; i < n; i += stride) {
        const char c = raw[i];
        if (c == '\n' || raw[LS[i]] == '>' || !ingest_base((unsigned char)c)) continue;
        const int64_t o = VX[i] - 1, s = HC[i] - 1;
        bases[o] = c;
        bseq[o] = s;
        bpos[o] = SC[i] - 1 - seq_sc0[s];
        const unsigned char u = (unsigned char)c;
        ++cnt[((u >> 1) ^ (u >> 2)) & 3u];  // A/a=0 C/c=1 G/g=2 T/t=3
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        unsigned long long v = cnt[b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(nucl + b, v);
    }
}

__device__ __forceinline__ bool ingest_run_start(const int64_t *bseq, const int64_t *bpos, int64_t k)
{
    return k == 0 || bseq[k] != bseq[k - 1] || bpos[k] != bpos[k - 1] + 1;
}

// pass 4: run-start flags over the stream (for a sum scan)
__global__ void ingest_runflags_kernel(const int64_t *bseq, const int64_t *bpos, int64_t nb, int64_t *f)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += (int64_t)gridDim.x * blockDim.x)
        f[k] = ingest_run_start(bseq, bpos, k);
}

// pass 5: the run table (R is the inclusive scan of the flags)
__global__ void ingest_runs_kernel(const int64_t *bseq, const int64_t *bpos, int64_t nb, const int64_t *R,
                                   int64_t *run_start, int64_t *run_seq, int64_t *run_seqpos)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += (int64_t)gridDim.x * blockDim.x) {
        if (!ingest_run_start(bseq, bpos, k)) continue;
        const int64_t r = R[k] - 1;
        run_start[r] = k;
        run_seq[r] = bseq[k];
        run_seqpos[r] = bpos[k];
    }
}

}  // namespace blamm
