// HEALPix pixel window functions, computed on the device from their
// definition (replaces healpy.pixwin, called at glass/healpix.py:351 and used
// by glass/lensing.py:360-362 for discretized shear).  healpy reads the
// windows from data files; here they are evaluated directly:
//
//   pw0_l^2 = mean over pixels of << P_l(cos gamma) >>_p
//   pw2_l^2 = mean over pixels of << d^l_22(gamma) >>_p      (l >= 2; 0 below)
//
// where << >>_p averages over two independent uniform points of pixel p and
// gamma is their separation (the addition theorem turns the pixel-averaged
// harmonics' power (4 pi / (2l+1)) sum_m |<Y_lm>_p|^2 into this pair average;
// for spin 2 the frames of both points are carried to the pixel centre, which
// leaves a phase of twice the spherical excess of a triangle inside the
// pixel, below 1e-12 in its cosine for nside >= 512, neglected).
//
// With t = sin^2(gamma/2) = |n - n'|^2 / 4 both kernels are power series in t:
//   P_l(1 - 2t)      = sum_k (-1)^k C(l,k) C(l+k,k) t^k
//   d^l_22(gamma)    = (1 - t)^2 sum_k (-1)^k C(l-2,k) C(l+k+2,k) t^k,
// so one pass over the pixels accumulates the pair moments M_k = <<t^k>> of
// all pixels, and every l follows from the same moments (t <= ~2 / nside^2
// inside a pixel, so for l <= 4 nside the terms peak near 3e3 at k ~ 5 and
// fall below 1e-30 by k = 40).
//
// Pixel quadrature: each pixel is the diamond |x - xc| + |y - yc| <= pi/(4 nside)
// of the equal-area HEALPix projection (x = phi, y = 3 pi z / 8 in the
// belt; y = (pi/4)(2 - s), x = phic + (phi - phic) s, s = sqrt(3(1 - |z|))
// in the caps).  It is cut at y = yc (the second derivative of the projection
// jumps there for the rings next to |z| = 2/3) and each half takes an 8 x 8
// Gauss-Legendre rule, 128 equal-area nodes per pixel (converged to ~1e-12
// against 12 x 12).  One pixel per congruence class is evaluated: a
// quadrant of each polar ring 1..nside (weight 8: four quadrants, both
// hemispheres) and one pixel of each belt ring nside+1..2 nside (weight
// 2 nph; nph for the equator).
#include <cuda_runtime.h>
#include <math.h>

#include "glg_internal.cuh"

namespace {

constexpr int PW_Q = 8;
constexpr int PW_NODES = 2 * PW_Q * PW_Q;  // 128 = threads per block
constexpr int PW_K = 43;                   // moments k = 0 .. 42 (the spin-2 series reads k + 2)
constexpr int PW_TERMS = PW_K - 2;         // series terms

struct PwRule {
    double u[PW_Q], w[PW_Q];  // Gauss-Legendre nodes and weights on [-1, 1]
};

// Gauss-Legendre rule of PW_Q points by Newton's method on P_Q (host, FP64).
PwRule gauss_rule() {
    PwRule r;
    const int n = PW_Q;
    for (int i = 0; i < n; ++i) {
        double x = cos(M_PI * (i + 0.75) / (n + 0.5));
        double dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = x;
            for (int k = 2; k <= n; ++k) {
                const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (x * p1 - p0) / (x * x - 1.0);
            const double dx = p1 / dp;
            x -= dx;
            if (fabs(dx) < 1e-16) break;
        }
        r.u[i] = x;
        r.w[i] = 2.0 / ((1.0 - x * x) * dp * dp);
    }
    return r;
}

__device__ __forceinline__ void pw_class(int nside, int64_t c, int &ring, int &jj, double &wgt) {
    const int64_t T = (int64_t)nside * (nside + 1) / 2;
    if (c < T) {
        int i = (int)((1.0 + sqrt(1.0 + 8.0 * (double)c)) * 0.5);
        while ((int64_t)i * (i - 1) / 2 > c) --i;
        while ((int64_t)(i + 1) * i / 2 <= c) ++i;
        ring = i;
        jj = (int)(c - (int64_t)i * (i - 1) / 2);
        wgt = 8.0;
    } else {
        ring = nside + 1 + (int)(c - T);
        jj = 0;
        wgt = (ring < 2 * nside ? 8.0 : 4.0) * nside;
    }
}

// Pair moments of the pixel classes [c0, c1) of this block, weighted by the
// class weights, into part[blockIdx.x][0 .. PW_K-1] (scaled: t * nside^2).
__global__ void __launch_bounds__(PW_NODES) k_pixwin_moments(int nside, int64_t nclass, PwRule g, double *part) {
    __shared__ double nx[PW_NODES], ny[PW_NODES], nz[PW_NODES], nw[PW_NODES];
    __shared__ double red[PW_NODES];
    const int a = threadIdx.x;
    const int64_t c0 = nclass * blockIdx.x / gridDim.x, c1 = nclass * (blockIdx.x + 1) / gridDim.x;
    const double PI = 3.14159265358979323846;
    const double h = PI / (4.0 * nside), s2 = (double)nside * nside;
    double acc[PW_K];
#pragma unroll
    for (int k = 0; k < PW_K; ++k) acc[k] = 0.0;
    for (int64_t c = c0; c < c1; ++c) {
        int ring, jj;
        double wgt;
        pw_class(nside, c, ring, jj, wgt);
        double xc, yc;
        const double phic = PI / 4;
        if (ring <= nside) {
            yc = (PI / 4) * (2.0 - (double)ring / nside);
            xc = phic + (PI / (2.0 * nside)) * (jj - 0.5 * (ring - 1));
        } else {
            yc = PI / 2 - ring * PI / (4.0 * nside);
            const int half = ((ring - nside) % 2 == 0) ? 1 : 0;
            xc = (PI / (2.0 * nside)) * (jj + 0.5 * half);
        }
        {  // node a of the pixel
            const int up = a / (PW_Q * PW_Q), ia = (a / PW_Q) % PW_Q, ib = a % PW_Q;
            const double yp = (up ? 1.0 : -1.0) * (h * 0.5) * (1.0 + g.u[ia]);
            const double width = h - fabs(yp);
            const double x = xc + width * g.u[ib], y = yc + yp;
            double z, phi;
            if (fabs(y) <= PI / 4) {
                z = 8.0 * y / (3.0 * PI);
                phi = x;
            } else {
                const double s = 2.0 - 4.0 * fabs(y) / PI;
                z = (y > 0 ? 1.0 : -1.0) * (1.0 - s * s / 3.0);
                phi = phic + (x - phic) / s;
            }
            const double st = sqrt((1.0 - z) * (1.0 + z));
            double sp, cp;
            sincos(phi, &sp, &cp);
            nx[a] = st * cp;
            ny[a] = st * sp;
            nz[a] = z;
            nw[a] = g.w[ia] * g.w[ib] * width / (4.0 * h);
        }
        __syncthreads();
        const double xa = nx[a], ya = ny[a], za = nz[a], wa = nw[a];
        acc[0] += wgt * wa * wa;  // the pair (a, a): t = 0
        // every unordered pair once: partner a + d (mod 128), d = 1 .. 64
        // (d = 64 by the lower half only)
        for (int d = 1; d <= PW_NODES / 2; ++d) {
            if (d == PW_NODES / 2 && a >= PW_NODES / 2) break;
            const int b = (a + d) & (PW_NODES - 1);
            const double dx = xa - nx[b], dy = ya - ny[b], dz = za - nz[b];
            const double t = 0.25 * s2 * (dx * dx + dy * dy + dz * dz);
            double tk = 2.0 * wgt * wa * nw[b];
#pragma unroll
            for (int k = 0; k < PW_K; ++k) {
                acc[k] += tk;
                tk *= t;
            }
        }
        __syncthreads();
    }
    // fixed-order tree reduction over the block's threads
    for (int k = 0; k < PW_K; ++k) {
        red[a] = acc[k];
        __syncthreads();
        for (int s = PW_NODES / 2; s > 0; s >>= 1) {
            if (a < s) red[a] += red[a + s];
            __syncthreads();
        }
        if (a == 0) part[(int64_t)blockIdx.x * PW_K + k] = red[0];
        __syncthreads();
    }
}

// M[k] = sum over blocks (fixed order) / the same sum of the pair weights
// (= npix up to rounding; dividing by the sum itself makes pw0_0 exactly 1).
__global__ void k_pixwin_sum(const double *part, int nblk, double *M) {
    const int k = threadIdx.x;
    double s = 0.0, s0 = 0.0;
    if (k < PW_K)
        for (int b = 0; b < nblk; ++b) {
            s += part[(int64_t)b * PW_K + k];
            s0 += part[(int64_t)b * PW_K];
        }
    if (k < PW_K) M[k] = s / s0;
}

// pw0[l], pw2[l] from the scaled moments (t scaled by nside^2).
__global__ void k_pixwin_series(const double *M, int nside, int lmax, double *pw0, double *pw2) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l > lmax) return;
    const double s = 1.0 / ((double)nside * nside);
    double c = 1.0, acc = 0.0;
    for (int k = 0; k < PW_TERMS && k <= l; ++k) {
        acc += c * M[k];
        c *= -(double)(l - k) * (double)(l + k + 1) / ((double)(k + 1) * (k + 1)) * s;
    }
    pw0[l] = sqrt(acc);
    if (pw2) {
        double v = 0.0;
        if (l >= 2) {
            const int n = l - 2;
            c = 1.0;
            acc = 0.0;
            for (int k = 0; k < PW_TERMS && k <= n; ++k) {
                acc += c * (M[k] - 2.0 * s * M[k + 1] + s * s * M[k + 2]);
                c *= -(double)(n - k) * (double)(n + k + 5) / ((double)(k + 1) * (k + 1)) * s;
            }
            v = sqrt(acc > 0.0 ? acc : 0.0);
        }
        pw2[l] = v;
    }
}

int pw_blocks(int nside) {
    const int64_t nclass = (int64_t)nside * (nside + 1) / 2 + nside;
    return (int)(nclass < 1216 ? nclass : 1216);
}

}  // namespace

extern "C" size_t glg_pixwin_workspace(int nside) {
    if (nside < 1 || nside > 8192) return 0;
    return sizeof(double) * ((size_t)pw_blocks(nside) * PW_K + PW_K);
}

extern "C" int glg_pixwin(int nside, int lmax, double *pw0, double *pw2, void *ws, size_t ws_bytes,
                          void *stream) {
    GLG_REQUIRE(nside >= 1 && nside <= 8192, "glg_pixwin: nside must be in [1, 8192]");
    GLG_REQUIRE(lmax >= 0 && lmax <= 4 * nside, "glg_pixwin: lmax must be in [0, 4 nside]");
    GLG_REQUIRE(pw0 != nullptr, "glg_pixwin: null pw0");
    GLG_REQUIRE(ws && ws_bytes >= glg_pixwin_workspace(nside), "glg_pixwin: workspace too small");
    static const PwRule rule = gauss_rule();
    cudaStream_t st = (cudaStream_t)stream;
    const int nblk = pw_blocks(nside);
    const int64_t nclass = (int64_t)nside * (nside + 1) / 2 + nside;
    double *part = (double *)ws;
    double *M = part + (size_t)nblk * PW_K;
    {
        GLG_LAUNCH_SCOPE("k_pixwin_moments", st);
        k_pixwin_moments<<<nblk, PW_NODES, 0, st>>>(nside, nclass, rule, part);
        GLG_CHECK_LAUNCH("k_pixwin_moments");
    }
    {
        GLG_LAUNCH_SCOPE("k_pixwin_sum", st);
        k_pixwin_sum<<<1, 64, 0, st>>>(part, nblk, M);
        GLG_CHECK_LAUNCH("k_pixwin_sum");
    }
    {
        GLG_LAUNCH_SCOPE("k_pixwin_series", st);
        k_pixwin_series<<<(lmax + 128) / 128, 128, 0, st>>>(M, nside, lmax, pw0, pw2);
        GLG_CHECK_LAUNCH("k_pixwin_series");
    }
    return GLG_OK;
}
