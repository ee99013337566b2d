// fp8_lane_check.cu -- test source: one tcgen05.mma of kind::f8f6f4 (E4M3 x E4M3, FP32
// accumulate), M = 128, N = 32, K = 32, on operands the host chooses, with D copied out.
// It checks how the tensor cores place and sum 8-bit operands: the operand layout (one-hot
// rows select single B entries) and the rounding of sums whose terms span many binades.
//
// Built by tests/test_gpu_fp8_lanes.py with
//   nvcc -gencode arch=compute_103a,code=sm_103a -shared -Xcompiler -fPIC -o <lib> fp8_lane_check.cu
#include <cstdint>
#include <cuda_runtime.h>

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, no swizzle: start, K-core stride (LBO), 8-row group
// stride (SBO), all in 16-byte units; bit 46: the descriptor version of sm_100-class parts
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

}  // namespace

// A: 128 rows x 32 K bytes (row-major), B: 32 columns x 32 K bytes; D: 128 x 32 floats.
// status[0]: 1 if the wait for the MMA ran out (then D is not written).
__global__ void fp8_mma_kernel(const uint8_t *A, const uint8_t *B, float *D, int *status)
{
    __shared__ __align__(1024) uint8_t sA[128 * 32];
    __shared__ __align__(1024) uint8_t sB[32 * 32];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    const int t = threadIdx.x, warp = t >> 5;
    // canonical K-major layout without swizzle: a core is 8 rows x 16 bytes; the two K cores
    // of an 8-row group are 128 B apart, 8-row groups 256 B apart
    for (int i = t; i < 128 * 32; i += blockDim.x) {
        const int r = i / 32, k = i % 32;
        sA[((r / 8) * 2 + k / 16) * 128 + (r % 8) * 16 + (k % 16)] = A[i];
    }
    for (int i = t; i < 32 * 32; i += blockDim.x) {
        const int c = i / 32, k = i % 32;
        sB[((c / 8) * 2 + k / 16) * 128 + (c % 8) * 16 + (k % 16)] = B[i];
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(smem_u32(&tmem_base))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tm = tmem_base;
    if (t == 0) {
        const uint64_t ad = smem_desc(smem_u32(sA), 128u, 256u), bd = smem_desc(smem_u32(sB), 128u, 256u);
        // D format F32 (bits 4-5 = 1), A and B format E4M3 (0), both K-major, N >> 3 at bit 17,
        // M >> 4 at bit 24
        const uint32_t idesc = (1u << 4) | ((32u >> 3) << 17) | ((128u >> 4) << 24);
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tm),
            "l"(ad), "l"(bd), "r"(idesc), "r"(0)
            : "memory");
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&bar))
                     : "memory");
    }
    // bounded wait for the MMA (a few microseconds; the limit is ~0.5 s)
    bool done = false;
    const long long t0 = clock64();
    while (!done && clock64() - t0 < (1LL << 30)) done = mbar_try_wait(smem_u32(&bar), 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (done) {
        uint32_t v[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
            "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
            "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
              "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
              "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
              "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
            : "r"(tm + ((uint32_t)(warp * 32) << 16)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        for (int c = 0; c < 32; ++c) D[t * 32 + c] = __uint_as_float(v[c]);
    } else if (t == 0) {
        status[0] = 1;
        // the MMA must land before its memory is released
        const long long t1 = clock64();
        while (!mbar_try_wait(smem_u32(&bar), 0) && clock64() - t1 < (1LL << 30)) {
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tm) : "memory");
    }
}

// Host entry: copies A (4096 B) and B (1024 B) in, runs the kernel, copies D (128 x 32
// floats) out.  Returns 0, 1 if the device wait ran out, or a CUDA error code + 100.
extern "C" int fp8_lane_check(const uint8_t *A, const uint8_t *B, float *D)
{
    uint8_t *dA = nullptr, *dB = nullptr;
    float *dD = nullptr;
    int *dS = nullptr, st = 0;
    cudaError_t e = cudaMalloc(&dA, 128 * 32);
    if (e == cudaSuccess) e = cudaMalloc(&dB, 32 * 32);
    if (e == cudaSuccess) e = cudaMalloc(&dD, 128 * 32 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dS, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(dA, A, 128 * 32, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dB, B, 32 * 32, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dS, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(dD, 0, 128 * 32 * sizeof(float));
    if (e == cudaSuccess) {
        fp8_mma_kernel<<<1, 128>>>(dA, dB, dD, dS);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(D, dD, 128 * 32 * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&st, dS, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dS);
    return e != cudaSuccess ? 100 + (int)e : st;
}
