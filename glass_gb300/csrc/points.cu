// Per-pixel Poisson galaxy counts (GLASS glass/points.py:252-348: the
// expected count n = (b delta - <b delta> + 1) (ARCMIN2_SPHERE / npix) ngal,
// times the visibility, clipped at zero, then one Poisson draw per pixel).
//
// The draw is reproducible bit for bit by a host restatement: every
// floating-point step is an explicitly rounded FP64 add, multiply or divide
// (no contraction into fma), and e^{-x} comes from a fixed polynomial rather
// than a math library.  A Poisson(lam) variate is the sum of Poisson pieces
// of mean <= 256 (Poisson additivity), each drawn by sequential inversion
// from one 53-bit uniform: k = min{k : u <= F(k)}, F accumulated from
// p_0 = e^{-lam}, p_k = (p_{k-1} lam) (1/k), 1/k the correctly rounded
// reciprocal (a per-block table in shared memory: FP64 division is a long
// instruction sequence on this GPU, a table load is one).  Piece c of pixel e uses words
// (2 (c & 1), 2 (c & 1) + 1) of the Philox block with counter
// (e, sid, c >> 1) and key = seed.
#include <cuda_runtime.h>
#include <math.h>

#include "glg_internal.cuh"
#include "philox.cuh"

namespace {

constexpr double PIECE = 256.0;
constexpr int64_t KMAX = 1 << 20;  // far beyond any piece's support

// e^{-x}, 0 <= x <= 256: Cody-Waite reduction x = k ln2 + r (ln2 split into
// a 32-bit head and a tail, so k ln2_hi is exact), |r| <= ln2 / 2, then the
// degree-13 Taylor polynomial of e^{-r} (truncation < 4e-18) by Horner, and
// an exact scaling by 2^-k.
__device__ __forceinline__ double exp_neg(double x) {
    const double inv_ln2 = 0x1.71547652b82fep+0;
    const double ln2_hi = 0x1.62e42fee00000p-1, ln2_lo = 0x1.a39ef35793c76p-33;
    const double c[14] = {0x1.0000000000000p+0, 0x1.0000000000000p+0, 0x1.0000000000000p-1,
                          0x1.5555555555555p-3, 0x1.5555555555555p-5, 0x1.1111111111111p-7,
                          0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16,
                          0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
                          0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33};
    const double kd = floor(__dadd_rn(__dmul_rn(x, inv_ln2), 0.5));
    const double r = __dsub_rn(__dsub_rn(x, __dmul_rn(kd, ln2_hi)), __dmul_rn(kd, ln2_lo));
    const double y = -r;
    double p = c[13];
#pragma unroll
    for (int i = 12; i >= 0; --i) p = __dadd_rn(__dmul_rn(p, y), c[i]);
    return ldexp(p, -(int)kd);
}

constexpr int NINV = 512;  // reciprocals 1/k, k < NINV, in shared memory

__device__ __forceinline__ int64_t poisson_piece(double lam, double u, const double *__restrict__ inv) {
    double p = exp_neg(lam), F = p;
    int64_t k = 0;
    while (u > F && p > 0.0 && k < KMAX) {
        k += 1;
        const double rk = k < NINV ? inv[k] : __drcp_rn((double)k);
        p = __dmul_rn(__dmul_rn(p, lam), rk);
        F = __dadd_rn(F, p);
    }
    return k;
}

template <typename T>
__global__ void k_poisson_counts(const T *__restrict__ delta, int64_t npix, double bias, double offset,
                                 double scale, const double *__restrict__ vis, uint64_t seed, uint32_t sid,
                                 int64_t *__restrict__ counts) {
    __shared__ double inv[NINV];
    for (int k = threadIdx.x; k < NINV; k += blockDim.x) inv[k] = k > 0 ? __drcp_rn((double)k) : 0.0;
    __syncthreads();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < npix;
         e += (int64_t)gridDim.x * blockDim.x) {
        const double d = (double)delta[e];
        double n = __dadd_rn(__dsub_rn(__dmul_rn(bias, d), offset), 1.0);
        n = __dmul_rn(n, scale);
        if (vis) n = __dmul_rn(n, vis[e]);
        double rest = n > 0.0 ? n : 0.0;  // clip (NaN -> 0)
        int64_t total = 0;
        glg_rng::U4 x = {0u, 0u, 0u, 0u};
        for (uint32_t c = 0; rest > 0.0; ++c) {
            const double lam = rest > PIECE ? PIECE : rest;
            rest = __dsub_rn(rest, lam);
            if ((c & 1u) == 0u)
                x = glg_rng::philox4x32_10((uint32_t)e, (uint32_t)(e >> 32), sid, c >> 1, (uint32_t)seed,
                                           (uint32_t)(seed >> 32));
            const double u = (c & 1u) ? glg_rng::u53(x.z, x.w) : glg_rng::u53(x.x, x.y);
            total += poisson_piece(lam, u, inv);
        }
        counts[e] = total;
    }
}

}  // namespace

extern "C" int glg_poisson_counts(const void *delta, int dtype, int64_t npix, double bias, double offset,
                                  double scale, const double *vis, uint64_t seed, uint64_t sid,
                                  int64_t *counts, void *stream) {
    GLG_REQUIRE(dtype == GLG_F64 || dtype == GLG_F32, "glg_poisson_counts: bad dtype");
    GLG_REQUIRE(npix >= 0, "glg_poisson_counts: negative size");
    GLG_REQUIRE(sid <= 0xFFFFFFFFull, "glg_poisson_counts: stream id must fit in 32 bits");
    if (npix == 0) return GLG_OK;
    GLG_REQUIRE(delta && counts, "glg_poisson_counts: null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    int64_t blocks = (npix + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    GLG_LAUNCH_SCOPE("k_poisson_counts", st);
    if (dtype == GLG_F64)
        k_poisson_counts<double><<<(unsigned)blocks, 256, 0, st>>>((const double *)delta, npix, bias, offset,
                                                                    scale, vis, seed, (uint32_t)sid, counts);
    else
        k_poisson_counts<float><<<(unsigned)blocks, 256, 0, st>>>((const float *)delta, npix, bias, offset,
                                                                   scale, vis, seed, (uint32_t)sid, counts);
    GLG_CHECK_LAUNCH("k_poisson_counts");
    return GLG_OK;
}
