// Peak-rate measurement kernels: the TF32 tensor-core rate (tcgen05.mma
// kind::tf32, M = 128, N = 256, K = 8, operands in shared memory, one CTA per
// SM) and the FP32 / FP64 FMA rates of the SIMT pipes.  They give the
// denominators of the roofline fractions that the copy and bf16 GEMM figures
// do not cover: the fast Legendre contraction runs in TF32 and its λ
// production in FP32; the plain form runs in FP64.  Operand values are
// constants, so the work is the same on every call.

#include <cstdint>

#include "glg_internal.cuh"
#include "tc_ptx.cuh"

using namespace glg_tc;

namespace {

constexpr int PK_N = 256;
constexpr uint32_t PK_LIMIT = 1u << 26;

// One CTA per SM (the dynamic shared memory forbids a second): thread 0
// issues `iters` MMAs into one 128 x 256 FP32 accumulator, then waits for
// their completion with a bounded wait.  A = 128 x 8 and B = 256 x 8 TF32
// tiles of 1.0 in the no-swizzle K-major layout (core matrices of 8 rows x
// 16 bytes, 128 bytes apart along K, 256 bytes apart along M / N).
__global__ void __launch_bounds__(128) k_peak_tf32(int iters, unsigned int *err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    const int warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < 48 * 1024 / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(sm)[i] = 0x3f800000u;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(&tbase, PK_N);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tb = tbase;
    if (threadIdx.x == 0) {
        fence_proxy_async_smem();
        constexpr uint32_t IDESC = idesc_tf32(128, PK_N);
        const uint64_t bd = sdesc_noswz(smem_u32(sm), 128, 256);
        const uint64_t ad = sdesc_noswz(smem_u32(sm + 32 * 1024), 128, 256);
        for (int i = 0; i < iters; ++i) {
            const uint32_t acc = i > 0 ? 1u : 0u;
            asm volatile(
                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tb),
                "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                : "memory");
        }
        mma_commit(&bar);
        if (!mbar_wait(&bar, 0, PK_LIMIT)) {
            atomicExch(err, 1u);
            mbar_wait(&bar, 0, PK_LIMIT);  // the MMAs still own the accumulator
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        tmem_dealloc(tb, PK_N);
    }
}

// Eight independent FMA chains per thread; the sum is stored so that the
// chains are live.
template <typename T>
__global__ void __launch_bounds__(256) k_peak_fma(int iters, T *sink) {
    T a[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) a[c] = (T)(threadIdx.x + c) * (T)1e-3;
    const T b = (T)0.999999, d = (T)1e-6;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) a[c] = fma(a[c], b, d);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += a[c];
    if (s == (T)-1) sink[blockIdx.x] = s;  // never true; keeps the chains
}

}  // namespace

extern "C" int glg_peak_tf32(int ctas, int iters, unsigned int *err, void *stream) {
    GLG_REQUIRE(ctas >= 1 && ctas <= 4096 && iters >= 1 && iters <= (1 << 24), "glg_peak_tf32: bad size");
    GLG_REQUIRE(err, "glg_peak_tf32: null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    const int smem = 160 * 1024;  // one CTA per SM
    cudaFuncSetAttribute(k_peak_tf32, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_peak_tf32<<<ctas, 128, smem, st>>>(iters, err);
    GLG_CHECK_LAUNCH("k_peak_tf32");
    return GLG_OK;
}

extern "C" int glg_peak_fma(int dtype, int blocks, int iters, void *sink, void *stream) {
    GLG_REQUIRE(dtype == GLG_F64 || dtype == GLG_F32, "glg_peak_fma: bad dtype");
    GLG_REQUIRE(blocks >= 1 && blocks <= (1 << 20) && iters >= 1, "glg_peak_fma: bad size");
    GLG_REQUIRE(sink, "glg_peak_fma: null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == GLG_F64) k_peak_fma<double><<<blocks, 256, 0, st>>>(iters, (double *)sink);
    else k_peak_fma<float><<<blocks, 256, 0, st>>>(iters, (float *)sink);
    GLG_CHECK_LAUNCH("k_peak_fma");
    return GLG_OK;
}
