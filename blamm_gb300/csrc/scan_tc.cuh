// scan_tc.cuh -- the fused tensor-core PWM scan (tcgen05 + TMA bulk + TMEM),
// one persistent CTA per SM.
//
// Score of motif column c at position p:  sum_j P(4j + base(p+j), c).
// After packing, e16_kernel writes one 16-byte entry per stream position of a
// window of at most 16 Mi positions (the scan runs once per window, so the entry
// array stays 256 MB whatever the stream length),
// E[i] = onehot(base i) ++ onehot(base i+1) (2 bases x 4 channels x bf16).
// For an M tile of 128 positions starting at m0, a bulk copy brings entries
// m0 .. m0+128+4g+1 into shared memory; read with row stride 16 B, 8-row group
// stride (SBO) 128 B and K-core stride (LBO) 32 B, the entries starting at
// E[4g] form exactly the A operand of motif bases 4g..4g+3 for all 128
// positions -- the overlapping one-hot windows of the reference's S matrix
// (src/sequence.cpp:299-340) without materialising them: each k-step is a
// shifted A descriptor over the same ~150 entries.  B_g holds rows
// 16g..16g+15 of P for the tile's columns.
//
// Arithmetic.  Column c's P enters as fixed-point BF16 terms: hi on the grid
// 2^-k, lo on 2^-(k+8), k = 7 - ceil(log2 max|P_c|), so |hi| <= 128 * 2^-k.
// The accumulator starts at -T (one extra "bias" MMA: a constant A tile with
// 1.0 in K slots 0-2 times three BF16 pieces of T), where T is the column's
// threshold minus its guard band, rounded down to the grid u = 2^-(k+8).
// Every partial sum is then an integer multiple of u below 2^24 u in
// magnitude (motifs up to 256 long), i.e. exactly representable in FP32, so an
// accumulation that keeps 24 significant bits holds sum(q) - T exactly (the
// raw-score dump instance compares the accumulator with the exact sum on
// every position and column of a test bank), and a position is a candidate
// iff its sign bit is clear.  The
// guard band bounds |sum(q) - sum(P)| plus the reference's own FP32 rounding
// of sum(P), so every reference hit is a candidate; candidates are rescored
// in exact FP32 (rescore_kernel).
//
// The E4M3 form (kTerms == kE4M3, kind::f8f6f4, K = 32 per MMA) scores 8 motif
// positions per k-step: e8_kernel's entries hold 4 bases (4 x 4 E4M3 bytes), the
// A cores of a k-step are 4 entries apart (LBO 64 B) and k-steps 8 entries (128 B)
// apart; B holds P(c) x 2^s_c rounded to E4M3 (s_c puts max|P_c| 2^s_c in
// (32, 64]), so every product and partial sum is a multiple of 2^-9 below 2^13
// in magnitude (motifs up to 64 positions), exact in FP32 when the tensor cores
// add exactly -- which the lane check in the tests shows for these operands.  The bias MMA's A rows are 32
// ones and its B column the pieces of T x 2^s_c.
//
// Roles (640 threads, warp w on SM sub-partition w % 4): warps 0-15 drain TMEM
// (lane quarter = warp % 4, column group = warp / 4) and test for candidates;
// warps 16 and 17 issue the MMAs of the even and the odd jobs (the whole warp
// runs the loop, one elected lane issues), so that one issuer's waits, commits
// and loop overhead overlap the other's MMAs (a job's result reaches the drain
// warps several hundred cycles after its last MMA is accepted); their
// waits spin instead of sleeping, since a sleeping issuer wakes late; warp 18
// (one lane) loads B tiles and E windows with TMA bulk copies up to kEStages
// jobs ahead; warp 16 also allocates TMEM.
// kEStages E stages and 2 or 4 TMEM accumulator stages (4 when the plan's N
// tiles are at most 128 wide) keep the roles overlapped.  A drain warp hands
// its accumulator back right after its TMEM loads; a chunk holds a candidate
// iff the maximum that the load returns is >= 0, and only then (rare) are the
// sign masks built and one 16-byte record (M tile, row and first column slot, mask)
// per lane with candidates written to global memory, into a block of record
// slots the warp reserved (kRecBlock slots per atomic, the next block reserved
// one block ahead; slot 0 of a block counts its records).  The rescoring kernel
// expands the masks.  The drain of every job gates the next MMAs on its
// accumulator and all 16 drain warps take part in it, so their rare path is kept
// to registers and fire-and-forget stores: shared-memory traffic from the SIMT
// warps queues behind the tensor cores' operand reads.  Jobs (N tile, M tile) are statically
// interleaved over the CTAs, N-tile major, so a CTA reloads B only when its
// tile changes: both issuers commit their old-tile MMAs to a tile-done
// barrier, the loader then copies the new B, and both wait for it.  Every wait
// is bounded (the issuers poll with test_wait, the drain warps wait with try_wait
// without a suspend hint, the loader's try_wait sleeps): on a timeout the CTA
// raises an abort flag, every role stops, copies and MMAs in flight are
// drained, TMEM is freed and the status word tells the host.
#pragma once
#include <cstdint>

#include "blamm_gpu.h"
#include "ptx_sm100.cuh"
#include "scan_kernels.cuh"

namespace blamm {

constexpr int kBM = 128;         // positions per M tile (= UMMA M)
constexpr int kMaxTcLen = BLAMM_MAX_TC_MOTIF_LEN;  // longest motif on the tensor-core path
constexpr int kEpiWarps = 16;    // TMEM drain warps (4 per lane quarter)
constexpr int kMmaWarp = 16;     // issuer of the even jobs; TMEM allocation
constexpr int kMmaWarp2 = 17;    // issuer of the odd jobs
constexpr int kLoadWarp = 18;    // TMA bulk copies of B tiles and E windows
constexpr int kRecBlock = kRecBlockSlots;  // candidate record slots a drain warp reserves at a time
constexpr int kTcThreads = 640;  // 20 warps (registers are allocated per 4 warps)
constexpr int kEStages = 6;      // E windows in flight
constexpr int kE4M3 = 8;         // kTerms of the E4M3 form (one term, K = 32 per MMA)
constexpr int kMaxE4M3Len = 64;  // longest motif of the E4M3 form (its bias needs <= 32 pieces)
constexpr int kMaxAcc = 4;       // TMEM accumulator stages (at most)

// Per-N-tile description (host-built, staged in SMEM by the kernel).
struct TileDesc {
    int32_t slot0;    // first column slot of the tile (slots: tile-local padded columns)
    int32_t n;        // UMMA N: columns of the tile, padded to a multiple of 32 (<= 256)
    int32_t g;        // k-steps of motif data: ceil(max motif length in the tile / 4)
    int32_t b_bytes;  // bytes of one B term: n x 16 x (g + 1) bf16 (last k-step: bias)
    int64_t b_off;    // byte offset of the tile's first B term in the B buffer
    // 1: the tile's longest motif leaves motif positions 4g-2 and 4g-1 unused (length
    // 4g-3 or 4g-2), so the bias pieces sit in K slots 8-10 of k-step g-1 and that
    // k-step reads its second K core from the constant A rows: no bias MMA
    int32_t fold;
    int32_t pad;
};

struct TcParams {
    const uint4 *e16;    // one-hot entries of this launch's window (16 B per position, padded)
    int64_t n;           // stream positions
    int64_t n_mtiles;    // M tiles of this launch's window
    int32_t m0;          // the window's first M tile in the stream
    const TileDesc *tiles;
    int32_t ntiles;
    int32_t terms;       // 1 (hi) or 2 (hi + lo)
    const uint8_t *bbuf; // B tiles
    const int32_t *slot_col;  // per slot: motif column, -1 for padding
    int32_t erows;       // E entries per stage (128 + 4 * max k-steps + 8)
    uint32_t b_term_max; // bytes reserved per B term in SMEM
    uint32_t tmem_cols;  // TMEM columns allocated (acc_stages accumulators)
    int32_t acc_stages;  // 2 (N <= 256) or 4 (N <= 128)
    uint4 *cand;                      // candidate record slots: blocks of kRecBlock (see scan_tc.cuh)
    unsigned long long *cand_count;   // record slots reserved
    unsigned long long *ncand;        // candidates (set mask bits), added up per drain warp
    int64_t cand_cap;                 // record slots available
    int *status;         // bit 0: a device wait timed out
    long long wait_limit;  // clock64 cycles a wait may last
    int32_t debug_stall;   // test hook: the MMA warp first waits on a barrier nobody completes
    // debug dump of the accumulator, sum(q) - T (positions [dump_p0, dump_p0+dump_npos))
    float *dump;
    int64_t dump_p0, dump_npos;
    int32_t dump_ncols;
    // optional per-CTA role timing (32 counters per CTA, clock64 cycles): see tc_prof_fields
    long long *prof;
};

// tc_prof_fields: 0/1 issuers' waits for a drained accumulator, 2 issuers' waits for B
// tiles, 3 MMA loop, 4 loader waits for free E stages, 5 loader waits at tile changes,
// 7 drain warp 0's accumulator waits, 8 its loop, 9 its drain (full accumulator -> hand-back),
// 10 jobs, 11 issuers' waits for E, 12 drain warp 0's rounds with a candidate, 13 its record
// block changes, 15 its candidate test and record writing

struct TcSmem {
    // byte offsets into dynamic shared memory
    uint32_t b_hi, b_lo, e0, abias, tiles, bars, ctl, total;
};

// control words in shared memory
enum {
    CTL_ABORT = 0,     // set by the first wait that times out
    CTL_TMEM = 1,      // TMEM base address
    CTL_WORDS = 4
};

__host__ __device__ inline TcSmem tc_smem_layout(uint32_t b_term_max, int terms, int erows, int ntiles)
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
    L.e0 = take((uint32_t)kEStages * erows * 16, 128);  // kEStages stages of erows entries
    L.abias = take(16 * 256, 128);  // 128 rows x 16 K-elements, canonical K-major layout
    L.tiles = take((uint32_t)ntiles * sizeof(TileDesc), 16);
    L.bars = take(32 * 8, 8);  // BAR_COUNT <= 32
    L.ctl = take(CTL_WORDS * 4, 16);
    L.total = take(0, 1024) + 1024;  // + slack for aligning the runtime base
    return L;
}

enum {
    BAR_WFULL = 0,                       // E window landed       (kEStages)
    BAR_WEMPTY = BAR_WFULL + kEStages,   // E window consumed     (kEStages)
    BAR_AFULL = BAR_WEMPTY + kEStages,   // accumulator ready     (kMaxAcc)
    BAR_AEMPTY = BAR_AFULL + kMaxAcc,    // accumulator drained   (kMaxAcc)
    BAR_BFULL = BAR_AEMPTY + kMaxAcc,    // B tile landed
    BAR_TILE = BAR_BFULL + 1,            // both issuers done with the old B tile
    BAR_DRAIN = BAR_TILE + 1,            // an issuer's MMAs drained (2)
    BAR_NEVER = BAR_DRAIN + 2,           // never completed (the stall test hook)
    BAR_COUNT = BAR_NEVER + 1
};
static_assert(BAR_COUNT <= 32, "the barrier area holds 32 mbarriers");

// Bit i set <=> word i is non-negative (sign bit clear), i.e. column i is a candidate.
// One funnel shift per word ((m << 1) | (v >> 31)), in four independent chains.
__device__ __forceinline__ uint32_t sign_mask(const uint32_t (&v)[32])
{
    uint32_t m0 = 0, m1 = 0, m2 = 0, m3 = 0;
#pragma unroll
    for (int i = 7; i >= 0; --i) {
        m0 = __funnelshift_l(v[i], m0, 1);
        m1 = __funnelshift_l(v[8 + i], m1, 1);
        m2 = __funnelshift_l(v[16 + i], m2, 1);
        m3 = __funnelshift_l(v[24 + i], m3, 1);
    }
    return ~(m0 | (m1 << 8) | (m2 << 16) | (m3 << 24));
}

// The jobs of one CTA: job = blockIdx.x + k * gridDim.x, tile = job / n_mtiles,
// m = job % n_mtiles, advanced without 64-bit divisions after the first.
// Job and M tile indices are 32-bit (the host launches at most 2^31 - 1 jobs): fewer
// registers on the drain warps' path.
struct JobIter {
    int job;
    int tile;
    int m;
    __device__ __forceinline__ void init(int j, int n_mtiles)
    {
        job = j;
        tile = j / n_mtiles;
        m = j - tile * n_mtiles;
    }
    __device__ __forceinline__ void next(int stride, int n_mtiles)
    {
        job += stride;
        m += stride;
        while (m >= n_mtiles) {
            m -= n_mtiles;
            ++tile;
        }
    }
};

template <bool kProf>
__device__ __forceinline__ long long tick()
{
    if constexpr (kProf) return clock64();
    else return 0;
}

// kDump: also write the raw accumulator of some positions (test hook);
// kProf: role timing into p.prof; kTerms: p.terms (1 or 2 BF16 terms, or kE4M3,
// one E4M3 term; B terms loaded: 2 for kTerms == 2, else 1).  The scan itself
// is <false, false, p.terms>.  The issuing threads run once per MMA and per
// job, so every branch taken out of their loops at compile time shows in the
// scan time (runtime mode switches cost 2-4 %).
template <bool kDump, bool kProf, int kTerms>
__global__ void __launch_bounds__(kTcThreads, 1) scan_tc_kernel(TcParams p)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = smem_raw + ((1024 - (ptx::smem_addr(smem_raw) & 1023)) & 1023);
    const TcSmem L = tc_smem_layout(p.b_term_max, kTerms, p.erows, p.ntiles);
    const uint32_t sbase = ptx::smem_addr(smem);
    TileDesc *s_tiles = reinterpret_cast<TileDesc *>(smem + L.tiles);
    const uint32_t bars = sbase + L.bars;
    volatile int *ctl = reinterpret_cast<volatile int *>(smem + L.ctl);
    volatile int *s_abort = ctl + CTL_ABORT;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // ---- set-up
    for (int i = threadIdx.x; i < p.ntiles * (int)(sizeof(TileDesc) / 4); i += blockDim.x)
        reinterpret_cast<int32_t *>(s_tiles)[i] = reinterpret_cast<const int32_t *>(p.tiles)[i];
    for (int i = threadIdx.x; i < CTL_WORDS; i += blockDim.x)
        if (i != CTL_TMEM) ctl[i] = 0;  // the TMEM word is written by the allocation below
    {
        // constant A rows: 128 rows of 8 K slots [1, 1, 1, 0, ...], 16 B apart, then 128
        // zero rows. With 8-row groups 128 B apart, the first block is a K core for any
        // descriptor that points its second core there (LBO = block - start), and the bias
        // MMA reads [ones | zeros] (start = block, LBO = 2048 B)
        uint4 *ab = reinterpret_cast<uint4 *>(smem + L.abias);
        for (int i = threadIdx.x; i < 256; i += blockDim.x)
            ab[i] = kTerms == kE4M3 ? make_uint4(0x38383838u, 0x38383838u, 0x38383838u, 0x38383838u)
                    : i < 128      ? make_uint4(0x3F803F80u, 0x00003F80u, 0u, 0u)
                                   : make_uint4(0u, 0u, 0u, 0u);
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < kEStages; ++s) {
            ptx::mbar_init(bars + 8 * (BAR_WFULL + s), 1);
            ptx::mbar_init(bars + 8 * (BAR_WEMPTY + s), 1);
        }
        for (int s = 0; s < kMaxAcc; ++s) {
            ptx::mbar_init(bars + 8 * (BAR_AFULL + s), 1);
            ptx::mbar_init(bars + 8 * (BAR_AEMPTY + s), kEpiWarps);
        }
        ptx::mbar_init(bars + 8 * BAR_BFULL, 1);
        ptx::mbar_init(bars + 8 * BAR_TILE, 2);
        ptx::mbar_init(bars + 8 * (BAR_DRAIN + 0), 1);
        ptx::mbar_init(bars + 8 * (BAR_DRAIN + 1), 1);
        ptx::mbar_init(bars + 8 * BAR_NEVER, 1);
        ptx::fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        ptx::tmem_alloc(sbase + L.ctl + 4 * CTL_TMEM, p.tmem_cols);
        ptx::tmem_relinquish();
        ptx::tc_fence_before();
    }
    ptx::fence_proxy_async_smem();  // the bias A tile is read by the tensor cores
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem_base = (uint32_t)ctl[CTL_TMEM];
    const uint32_t acc_stride = p.tmem_cols / (uint32_t)p.acc_stages;
    const uint32_t acc_shift = p.acc_stages == 4 ? 2u : 1u, acc_mask = (uint32_t)p.acc_stages - 1u;
    const int njobs = p.ntiles * (int)p.n_mtiles;  // < 2^31 (host-checked)
    const int n_mt = (int)p.n_mtiles;

    if (warp == kMmaWarp || warp == kMmaWarp2) {
        // ============ MMA issuers: warp 16 the even jobs, warp 17 the odd ones ============
        // Both walk every job of the CTA, so that both take part in every B tile change.
        // The whole warp runs the loop (warp-uniform descriptors, one vote per wait); one
        // elected lane issues each MMA and commit.
        const uint32_t mine = warp == kMmaWarp ? 0u : 1u;
        int cur_tile = -1;
        uint32_t bphase = 0, idesc = 0, g_steps = 0, es = 0, eph = 0, fold = 0;
        uint64_t bdesc_hi0 = 0, bdesc_lo0 = 0;  // k-step 0 of the current tile's B terms
        long long t_acc = 0, t_w = 0, t_b = 0;
        const long long t_start = tick<kProf>();
        const uint64_t adesc_bias = ptx::smem_desc(sbase + L.abias, 2048u, 128u);
        // A of a k-step: its two K cores 2 (BF16) or 4 (E4M3) entries apart; k-steps 4 or 8
        // entries apart (a_step, in 16 B units)
        const uint64_t adesc_e = ptx::smem_desc(sbase + L.e0, kTerms == kE4M3 ? 64u : 32u, 128u);
        const uint32_t a_step = kTerms == kE4M3 ? 8u : 4u;
        auto mma = [&](uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
            if constexpr (kTerms == kE4M3) ptx::mma_e4m3_elect(d, a, b, idesc, acc);
            else ptx::mma_bf16_elect(d, a, b, idesc, acc);
        };
        const uint32_t e_step = (uint32_t)p.erows;  // one E stage in 16 B units
        uint32_t jc = 0;
        bool ok = true;
        if (p.debug_stall) ok = ptx::mbar_wait(bars + 8 * BAR_NEVER, 0, s_abort, p.wait_limit);
        ok = __all_sync(0xffffffffu, ok);
        JobIter it;
        for (it.init(blockIdx.x, n_mt); it.job < njobs && ok; it.next(gridDim.x, n_mt), ++jc) {
            const int tile = it.tile;
            if (tile != cur_tile) {
                const long long tb = tick<kProf>();
                // this issuer is done with the old tile once its MMAs so far are complete
                if (cur_tile >= 0) ptx::mma_commit_elect(bars + 8 * BAR_TILE);
                ok = __all_sync(0xffffffffu, ptx::mbar_wait(bars + 8 * BAR_BFULL, bphase, s_abort, p.wait_limit));
                bphase ^= 1;
                if (!ok) break;
                ptx::tc_fence_after();
                cur_tile = tile;
                if (kProf) t_b += tick<kProf>() - tb;
                const TileDesc td = s_tiles[tile];
                g_steps = (uint32_t)td.g;
                fold = (uint32_t)td.fold;
                idesc = kTerms == kE4M3 ? ptx::idesc_e4m3_f32(kBM, (uint32_t)td.n)
                                        : ptx::idesc_bf16_f32(kBM, (uint32_t)td.n);
                const uint32_t sbo_b = 256u * (g_steps + 1);  // bytes between 8-column groups of B
                bdesc_hi0 = ptx::smem_desc(sbase + L.b_hi, 128u, sbo_b);
                bdesc_lo0 = ptx::smem_desc(sbase + L.b_lo, 128u, sbo_b);
            }
            if ((jc & 1u) == mine) {
                const uint32_t s = jc & acc_mask, ph = (jc >> acc_shift) & 1u;  // accumulator
                const long long t0 = tick<kProf>();
                ok = ptx::mbar_wait_spin(bars + 8 * (BAR_AEMPTY + s), ph ^ 1u, s_abort, p.wait_limit);
                const long long t1 = tick<kProf>();
                ok = ok && ptx::mbar_wait_spin(bars + 8 * (BAR_WFULL + es), eph, s_abort, p.wait_limit);
                ok = __all_sync(0xffffffffu, ok);
                if (kProf) {
                    t_acc += t1 - t0;
                    t_w += tick<kProf>() - t1;
                }
                if (!ok) break;
                ptx::tc_fence_after();
                const uint32_t d_tmem = tmem_base + s * acc_stride;
                // A of k-step g starts 4g entries (64 B) into the E stage, B_g 256 B into each
                // term: the descriptors' address fields (bits 0-13, in 16 B units) advance by
                // 4 and 16
                const uint64_t adesc0 = adesc_e + es * e_step;
                uint32_t acc = 1u, g_plain = g_steps;
                if (fold) {
                    g_plain = g_steps - 1u;  // the last k-step carries the bias
                    acc = g_plain > 0u ? 1u : 0u;
                } else {
                    // D = -T (bias pieces in the extra k-step g of the hi term)
                    mma(d_tmem, adesc_bias, bdesc_hi0 + 16u * g_steps, 0u);
                }
                for (uint32_t g = 0; g < g_plain; ++g) {
                    const uint32_t a = (g == 0u && fold) ? 0u : 1u;  // a folded tile starts at D = A B
                    mma(d_tmem, adesc0 + a_step * g, bdesc_hi0 + 16u * g, a);
                    if (kTerms == 2) mma(d_tmem, adesc0 + a_step * g, bdesc_lo0 + 16u * g, 1u);
                }
                if (fold) {
                    // k-step g-1: first K core = entries m0 + 4(g-1) + r, second K core = the
                    // constant rows (the hi term's B holds the bias pieces there)
                    const uint32_t a_last = sbase + L.e0 + es * e_step * 16u + 16u * a_step * g_plain;
                    const uint64_t adesc_last = ptx::smem_desc(a_last, sbase + L.abias - a_last, 128u);
                    mma(d_tmem, adesc_last, bdesc_hi0 + 16u * g_plain, acc);
                    if (kTerms == 2) mma(d_tmem, adesc_last, bdesc_lo0 + 16u * g_plain, 1u);
                }
                ptx::mma_commit_elect(bars + 8 * (BAR_WEMPTY + es));
                ptx::mma_commit_elect(bars + 8 * (BAR_AFULL + s));
            }
            if (++es == (uint32_t)kEStages) {
                es = 0;
                eph ^= 1u;
            }
        }
        // drain: nothing may still write TMEM or shared memory when they are freed
        ptx::mma_commit_elect(bars + 8 * (BAR_DRAIN + mine));
        if (!ptx::mbar_wait_drain(bars + 8 * (BAR_DRAIN + mine), 0, p.wait_limit)) *s_abort = 1;
        if (kProf && lane == 0) {
            long long *pr = p.prof + 32 * blockIdx.x;
            pr[mine] += t_acc;
            if (mine == 0) {
                pr[2] += t_b;
                pr[3] += tick<kProf>() - t_start;
                pr[10] += jc;
                pr[11] += t_w;
            }
        }
    } else if (warp == kLoadWarp && lane == 0) {
        // ============ loader: B tiles at tile changes, E windows kEStages jobs ahead ============
        int cur_tile = -1;
        uint32_t tphase = 0, bphase = 0, es = 0, eph = 0, jc = 0;
        uint32_t issued[kEStages];  // per E stage: 1 + the phase of its last copy, 0 = none
        for (int k = 0; k < kEStages; ++k) issued[k] = 0;
        bool b_pending = false, ok = true;
        long long t_we = 0, t_tile = 0;
        JobIter it;
        for (it.init(blockIdx.x, n_mt); it.job < njobs; it.next(gridDim.x, n_mt), ++jc) {
            const int tile = it.tile;
            const TileDesc &td = s_tiles[tile];
            if (tile != cur_tile) {
                if (cur_tile >= 0) {  // both issuers' MMAs on the old B are complete
                    const long long t0 = tick<kProf>();
                    ok = ptx::mbar_wait(bars + 8 * BAR_TILE, tphase, s_abort, p.wait_limit);
                    tphase ^= 1;
                    if (kProf) t_tile += tick<kProf>() - t0;
                    if (!ok) break;
                    // the previous B copy has landed (both issuers waited for it)
                }
                ptx::mbar_arrive_expect_tx(bars + 8 * BAR_BFULL, (uint32_t)td.b_bytes * (kTerms == 2 ? 2u : 1u));
                ptx::bulk_g2s(sbase + L.b_hi, p.bbuf + td.b_off, (uint32_t)td.b_bytes, bars + 8 * BAR_BFULL);
                if (kTerms == 2)
                    ptx::bulk_g2s(sbase + L.b_lo, p.bbuf + td.b_off + td.b_bytes, (uint32_t)td.b_bytes,
                                  bars + 8 * BAR_BFULL);
                b_pending = true;
                bphase ^= 1;
                cur_tile = tile;
            }
            // E window of this job (16 B entries)
            const long long t0 = tick<kProf>();
            ok = ptx::mbar_wait(bars + 8 * (BAR_WEMPTY + es), eph ^ 1u, s_abort, p.wait_limit);
            if (kProf) t_we += tick<kProf>() - t0;
            if (!ok) break;
            // entries m0 .. m0 + 128 + 4g + 1 (BF16) or m0 + 128 + 8g + 3 (E4M3)
            const uint32_t bytes = 16u * (uint32_t)(kTerms == kE4M3 ? kBM + 8 * td.g + 4 : kBM + 4 * td.g + 2);
            ptx::mbar_arrive_expect_tx(bars + 8 * (BAR_WFULL + es), bytes);
            ptx::bulk_g2s(sbase + L.e0 + es * (uint32_t)p.erows * 16u, p.e16 + (int64_t)it.m * kBM, bytes,
                          bars + 8 * (BAR_WFULL + es));
            issued[es] = 1u + eph;
            if (++es == (uint32_t)kEStages) {
                es = 0;
                eph ^= 1u;
            }
        }
        // on an abort, copies still in flight must land before the CTA frees its memory
        if (*s_abort) {
            for (int k = 0; k < kEStages; ++k)
                if (issued[k]) ptx::mbar_wait_drain(bars + 8 * (BAR_WFULL + k), issued[k] - 1u, p.wait_limit);
            if (b_pending) ptx::mbar_wait_drain(bars + 8 * BAR_BFULL, bphase ^ 1u, p.wait_limit);
        }
        if (kProf) {
            long long *pr = p.prof + 32 * blockIdx.x;
            pr[4] += t_we;
            pr[5] += t_tile;
        }
    } else if (warp < kEpiWarps) {
        // ===================== epilogue (warps 0-15) ======================
        const int q = warp & 3;     // TMEM lanes 32q .. 32q+31
        const int grp = warp >> 2;  // 32-column chunks grp, grp + 4
        const uint32_t lt = (1u << lane) - 1u;
        // record blocks (slot indices): the current one and, in lane 0, the next one, reserved
        // one block ahead so that the atomic's latency stays off the drain path
        // (32-bit slot indices: the host keeps the capacity below 2^31; a block reserved
        // beyond the capacity becomes slot index cap, whose stores are dropped)
        const uint32_t cap = (uint32_t)p.cand_cap;
        auto reserve = [&]() -> uint32_t {
            const unsigned long long b = atomicAdd(p.cand_count, (unsigned long long)kRecBlock);
            return b < (unsigned long long)cap ? (uint32_t)b : cap;
        };
        uint32_t blk = 0xFFFFFFFFu, nxt_blk = 0;
        uint32_t bfill = 0;  // slots used in the current block (slot 0 is its count)
        if (lane == 0) nxt_blk = reserve();
        auto put = [&](uint32_t slot, uint4 v) {
            if (slot < cap) p.cand[slot] = v;
        };
        auto close_block = [&]() {  // slot 0 of a block: its number of records
            if (blk != 0xFFFFFFFFu && lane == 0) put(blk, make_uint4(bfill - 1u, 0u, 0u, 0u));
        };
        long long t_af = 0, t_dr = 0, n_rare = 0, t_red = 0, t_full = 0;
        uint32_t my_cand = 0;  // this lane's candidates
        const long long t_start = tick<kProf>();
        uint32_t jc = 0;
        JobIter it;
        for (it.init(blockIdx.x, n_mt); it.job < njobs; it.next(gridDim.x, n_mt), ++jc) {
            const int tile = it.tile;
            const int m = p.m0 + it.m;  // M tile in the stream
            const int slot0 = s_tiles[tile].slot0, nch = s_tiles[tile].n >> 5;
            const uint32_t s = jc & acc_mask, ph = (jc >> acc_shift) & 1u;
            const long long t0 = tick<kProf>();
            if (!ptx::mbar_wait_nohint(bars + 8 * (BAR_AFULL + s), ph, s_abort, p.wait_limit)) break;
            const long long t1 = tick<kProf>();
            if (kProf) t_af += t1 - t0;
            ptx::tc_fence_after();
            const uint32_t row = (uint32_t)(q * 32 + lane);  // this lane's position: m * 128 + row
            const bool valid = (int64_t)m * kBM + row < p.n;
            const uint32_t taddr = tmem_base + ((uint32_t)(q * 32) << 16) + s * acc_stride;
            // This warp's 32-column chunks grp and grp+4 (N <= 256): two TMEM loads that
            // also return each lane's maximum over the chunk, after which the accumulator
            // is handed back at once; the candidate test on the maxima and the rare mask
            // building run on the registers.
            const int ca = grp, cb = grp + 4;
            const bool has_a = ca < nch, has_b = cb < nch;  // warp-uniform
            uint32_t va[32], vb[32];
            float max_a = -1.f, max_b = -1.f;  // each chunk's maximum, from the loads themselves
            if (has_a) {
                ptx::tmem_ld_max_32x32b_x32(taddr + ca * 32, va, max_a);
                if (has_b) ptx::tmem_ld_max_32x32b_x32(taddr + cb * 32, vb, max_b);
                ptx::tmem_wait_ld();
                ptx::reg_fence(va);
                ptx::reg_fence(vb);
                asm volatile("" : "+f"(max_a), "+f"(max_b));  // the same fence for the maxima
            }
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(bars + 8 * (BAR_AEMPTY + s));
            if (kProf) t_dr += tick<kProf>() - t1;
            if (has_a) {
                const long long tr0 = tick<kProf>();
                // maximum >= 0 <=> some column of the chunk is a candidate (a -0.0 passes
                // here and is dropped by the sign mask)
                const bool any_a = valid && max_a >= 0.f;
                const bool any_b = has_b && valid && max_b >= 0.f;
                if (__any_sync(0xffffffffu, any_a || any_b)) {  // rare: publish records
                    ++n_rare;
                    const uint32_t ma = any_a ? sign_mask(va) : 0u, mb = any_b ? sign_mask(vb) : 0u;
                    const uint32_t ba = __ballot_sync(0xffffffffu, ma != 0u);
                    const uint32_t bb = __ballot_sync(0xffffffffu, mb != 0u);
                    const uint32_t na = (uint32_t)__popc(ba), cnt = na + (uint32_t)__popc(bb);
                    if (cnt > 0) {
                        if (blk == 0xFFFFFFFFu || bfill + cnt > (uint32_t)kRecBlock) {  // next block
                            const long long tw = tick<kProf>();
                            close_block();
                            blk = __shfl_sync(0xffffffffu, nxt_blk, 0);
                            bfill = 1;
                            if (lane == 0) nxt_blk = reserve();
                            if (kProf) t_full += tick<kProf>() - tw;
                        }
                        // record: M tile, row | first slot of the chunk << 7, mask
                        if (ma)
                            put(blk + bfill + __popc(ba & lt),
                                make_uint4((uint32_t)m, row | (uint32_t)(slot0 + ca * 32) << 7, ma, 0u));
                        if (mb)
                            put(blk + bfill + na + __popc(bb & lt),
                                make_uint4((uint32_t)m, row | (uint32_t)(slot0 + cb * 32) << 7, mb, 0u));
                        bfill += cnt;
                        my_cand += (uint32_t)(__popc(ma) + __popc(mb));
                    }
                }
                const int64_t pos = (int64_t)m * kBM + row;
                if (kDump && pos >= p.dump_p0 && pos < p.dump_p0 + p.dump_npos) {
                    // debug instantiation only: raw accumulator of some positions
                    float *drow = p.dump + (pos - p.dump_p0) * p.dump_ncols;
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        int col = __ldg(p.slot_col + slot0 + ca * 32 + i);
                        if (col >= 0) drow[col] = __uint_as_float(va[i]);
                        if (has_b && (col = __ldg(p.slot_col + slot0 + cb * 32 + i)) >= 0)
                            drow[col] = __uint_as_float(vb[i]);
                    }
                }
                if (kProf) t_red += tick<kProf>() - tr0;
            }
        }
        // every reserved block states its count: the current one and the one reserved ahead
        close_block();
        if (lane == 0) put(nxt_blk, make_uint4(0u, 0u, 0u, 0u));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) my_cand += __shfl_xor_sync(0xffffffffu, my_cand, o);
        if (lane == 0 && my_cand) atomicAdd(p.ncand, (unsigned long long)my_cand);
        if (kProf && lane == 0 && warp == 0) {
            long long *pr = p.prof + 32 * blockIdx.x;
            pr[7] += t_af;
            pr[8] += tick<kProf>() - t_start;
            pr[9] += t_dr;
            pr[12] += n_rare;
            pr[13] += t_full;
            pr[15] += t_red;
        }
    }


    // ---- teardown
    __syncthreads();
    if (threadIdx.x == 0 && *s_abort) atomicOr(p.status, 1);
    if (warp == kMmaWarp) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem_base, p.tmem_cols);
    }
}

}  // namespace blamm
