// glg_alm2map_noalloc: spin-0 synthesis for callers that cannot allocate
// device memory.
//
// Some callers cannot call cudaMalloc at the point where they need a map:
// real-time or embedded loops whose device memory is fixed at start-up (an
// allocation there can fail or stall the loop), or host programs whose device
// memory is owned by another allocator (a framework's caching pool, a memory
// budget enforced per process) that must not be bypassed.  This entry point serves them: it needs no plan and no workspace
// and calls no allocating routine.  Ring geometry, Legendre coefficients and
// Fourier phases are computed on the fly in FP64, and the per-ring Legendre
// sums go into one fixed scratch array that lives in the library's own
// device memory (GLG_NOALLOC_SCRATCH_BYTES, held by every GPU that loads the
// library until the process exits).
//
// Limits: nside <= 256 (ring length <= 1024), lmax + 1 <= 65535 and
// nmaps <= 65535 (the grid's y dimensions) and
// nmaps * (4 nside - 1) * (lmax + 1) * 16 bytes <= GLG_NOALLOC_SCRATCH_BYTES;
// larger requests are rejected with GLG_ERR_UNSUPPORTED.  All calls share the
// scratch array, so calls whose kernels overlap on the GPU (different
// streams, or different host threads) race; serialise them.  Every scratch
// entry a call reads is written earlier in the same call, so nothing has to
// start at zero.  The first call on a device looks up the array's device
// address (cudaGetSymbolAddress); make that first call before any stream
// capture begins.  The address is kept per device index, so the entry point
// assumes the CUDA runtime's primary context of each device (the context
// every runtime-API caller shares).
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

#include "glg_internal.cuh"

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GLG_NOALLOC_SCRATCH_BYTES];

constexpr int NA_THREADS = 128;
constexpr int NA_MAX_NSIDE = 256;

std::mutex g_na_mu;
void *g_na_ptr[64] = {nullptr};

// Ring p (0-based, north) of an nside map: cos theta, sin theta, nph, phi0 = pi/nph flag.
__device__ void na_ring(int nside, int p, double &z, double &s, int &nph, int &half) {
    const int ir = p + 1;
    const double ns = nside;
    if (ir < nside) {
        const double t = (double)ir * ir / (3.0 * ns * ns);
        z = 1.0 - t;
        s = sqrt(t * (2.0 - t));
        nph = 4 * ir;
        half = 1;
    } else {
        z = (2.0 * ns - ir) * 2.0 / (3.0 * ns);
        s = sqrt((1.0 - z) * (1.0 + z));
        nph = 4 * nside;
        half = ((ir - nside) % 2 == 0) ? 1 : 0;
    }
}

// F[map][ring][m] = sum_l a_lm lambda_lm(z_ring), north and south ring of pair p.
__global__ void __launch_bounds__(NA_THREADS)
k_na_leg(int nside, int lmax, const double2 *__restrict__ alm, int nmaps, double2 *__restrict__ F) {
    const int npairs = 2 * nside, nrings = 4 * nside - 1;
    const int p = blockIdx.x * NA_THREADS + threadIdx.x;
    const int m = blockIdx.y;
    if (p >= npairs) return;
    double x, s;
    int nph, half;
    na_ring(nside, p, x, s, nph, half);
    // lambda_mm with an exponent scale of 2^800 steps
    double l1 = 0.28209479177387814;  // 1 / sqrt(4 pi)
    int sc = 0;
    for (int k = 1; k <= m; ++k) {
        l1 *= -s * sqrt((2.0 * k + 1.0) / (2.0 * k));
        if (fabs(l1) < GLG_TWO_M400) {
            l1 *= GLG_TWO_P800;
            sc -= 1;
        }
    }
    double l0 = 0.0;
    const int64_t nalm = glg_nalm(lmax);
    const int64_t base = (int64_t)m * (2 * lmax + 3 - m) / 2;  // index of (l = m, m)
    for (int mp = 0; mp < nmaps; ++mp) {
        double er = 0, ei = 0, orr = 0, oi = 0;
        double a0 = l0, a1 = l1;
        int asc = sc;
        for (int l = m; l <= lmax; ++l) {
            if (l > m) {
                double nl;
                if (l == m + 1) {
                    nl = sqrt(2.0 * m + 3.0) * x * a1;
                } else {
                    const double l2 = (double)l * l, m2 = (double)m * m, lm1 = l - 1.0;
                    const double A = sqrt((4.0 * l2 - 1.0) / (l2 - m2));
                    const double B = sqrt((4.0 * l2 - 1.0) * (lm1 * lm1 - m2) / ((l2 - m2) * (4.0 * lm1 * lm1 - 1.0)));
                    nl = A * (x * a1) - B * a0;
                }
                a0 = a1;
                a1 = nl;
                if (asc < 0 && fabs(nl) > GLG_TWO_P400) {
                    a0 *= GLG_TWO_M800;
                    a1 *= GLG_TWO_M800;
                    asc += 1;
                }
            }
            if (asc == 0) {
                const double2 a = alm[(int64_t)mp * nalm + base + (l - m)];
                if ((l - m) & 1) {
                    orr += a.x * a1;
                    oi += a.y * a1;
                } else {
                    er += a.x * a1;
                    ei += a.y * a1;
                }
            }
        }
        double2 *Fm = F + (int64_t)mp * nrings * (lmax + 1);
        const int rn = p, rs = nrings - 1 - p;
        Fm[(int64_t)rn * (lmax + 1) + m] = make_double2(er + orr, ei + oi);
        if (rs != rn) Fm[(int64_t)rs * (lmax + 1) + m] = make_double2(er - orr, ei - oi);
    }
}

// Ring values by direct Fourier sums: f_j = sum_m c_m Re(F_m e^{i m (phi0 + 2 pi j / n)}),
// c_0 = 1, c_m = 2; one block per (ring, map).
__global__ void __launch_bounds__(NA_THREADS)
k_na_ring(int nside, int lmax, const double2 *__restrict__ F, double *__restrict__ maps) {
    __shared__ double2 w[4 * NA_MAX_NSIDE];  // omega_n^t = e^{2 pi i t / n}
    const int nrings = 4 * nside - 1;
    const int r = blockIdx.x, mp = blockIdx.y;
    const int p = r < 2 * nside ? r : nrings - 1 - r;
    double x, s;
    int n, half;
    na_ring(nside, p, x, s, n, half);
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        double sn, cs;
        sincospi(2.0 * t / n, &sn, &cs);
        w[t] = make_double2(cs, sn);
    }
    __syncthreads();
    // first pixel of ring r (RING scheme)
    const int64_t npix = 12LL * nside * nside;
    const int ir = r + 1;
    int64_t start;
    if (ir < nside)
        start = 2LL * ir * (ir - 1);
    else if (ir <= 3 * nside)
        start = 2LL * nside * (nside - 1) + (int64_t)(ir - nside) * 4 * nside;
    else {
        const int irs = 4 * nside - ir;
        start = npix - 2LL * irs * (irs + 1);
    }
    const double2 *Fr = F + ((int64_t)mp * nrings + r) * (lmax + 1);
    double *out = maps + (int64_t)mp * npix + start;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        double acc = 0.0;
        for (int m = 0; m <= lmax; ++m) {
            // phase m (phi0 + 2 pi j / n) = 2 pi (m j + half m / 2) / n
            const int64_t t2 = 2LL * m * j + (int64_t)half * m;  // in units of pi / n
            const int64_t tt = t2 % (2LL * n);
            double2 e;
            if ((tt & 1) == 0) {
                e = w[tt >> 1];
            } else {
                double sn, cs;
                sincospi((double)tt / n, &sn, &cs);
                e = make_double2(cs, sn);
            }
            const double2 f = Fr[m];
            const double re = f.x * e.x - f.y * e.y;
            acc += (m == 0 ? 1.0 : 2.0) * re;
        }
        out[j] = acc;
    }
}

int na_scratch(void **ptr) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_alm2map_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= 64) {
        glg_set_error("glg_alm2map_noalloc: device index out of range");
        return GLG_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return glg_cuda_status(e, "glg_alm2map_noalloc: cudaGetSymbolAddress");
        g_na_ptr[dev] = p;
    }
    *ptr = g_na_ptr[dev];
    return GLG_OK;
}

}  // namespace

extern "C" int glg_alm2map_noalloc(int nside, int lmax, const void *alm, int nmaps, void *maps,
                                   void *stream) {
    GLG_REQUIRE(alm && maps, "glg_alm2map_noalloc: null pointer");
    GLG_REQUIRE(nside >= 1 && (nside & (nside - 1)) == 0, "glg_alm2map_noalloc: nside must be a power of two");
    GLG_REQUIRE(lmax >= 0 && nmaps >= 1, "glg_alm2map_noalloc: bad lmax or nmaps");
    if (nside > NA_MAX_NSIDE) {
        glg_set_error("glg_alm2map_noalloc: nside above 256 (the fixed-size path's limit)");
        return GLG_ERR_UNSUPPORTED;
    }
    if (lmax + 1 > 65535 || nmaps > 65535) {
        glg_set_error("glg_alm2map_noalloc: lmax + 1 and nmaps must each be at most 65535 (grid y limit)");
        return GLG_ERR_UNSUPPORTED;
    }
    const size_t need = sizeof(double2) * (size_t)nmaps * (4 * nside - 1) * (size_t)(lmax + 1);
    if (need > GLG_NOALLOC_SCRATCH_BYTES) {
        glg_set_error("glg_alm2map_noalloc: nmaps * (4 nside - 1) * (lmax + 1) * 16 bytes exceeds the "
                      "16 MiB scratch array");
        return GLG_ERR_UNSUPPORTED;
    }
    void *scratch = nullptr;
    int rc = na_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    double2 *F = (double2 *)scratch;
    dim3 g1((2 * nside + NA_THREADS - 1) / NA_THREADS, lmax + 1);
    k_na_leg<<<g1, NA_THREADS, 0, st>>>(nside, lmax, (const double2 *)alm, nmaps, F);
    GLG_CHECK_LAUNCH("k_na_leg");
    dim3 g2(4 * nside - 1, nmaps);
    k_na_ring<<<g2, NA_THREADS, 0, st>>>(nside, lmax, F, (double *)maps);
    GLG_CHECK_LAUNCH("k_na_ring");
    return GLG_OK;
}
