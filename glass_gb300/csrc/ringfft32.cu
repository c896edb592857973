// FP32 ring FFTs of the fast form (inside healpy.alm2map, glass/healpix.py:71).
//
// Input: Legendre sums F[map][m][ring] from the tensor-core contraction.  A
// tiled transpose makes every ring's m-vector contiguous; then one block per
// (ring pair, map) folds m onto the ring's n pixels, packs the north ring and
// its mirror as one complex sequence Z_k = B^N_k + i B^S_k, runs one complex
// inverse DFT of length n and stores both rings with the fused field
// transform (glass/grf/_transformations.py:83-89).
//
// Fold.  With G_m = F_m e^{i m phi0} and phi0 = h pi / n (h = 1 on rings
// whose first pixel sits half a step off phi = 0),
//   B_k = sum_{m = k mod n} c_m G_m + sum_{m = -k mod n} c_m conj(G_m),
// c_0 = 1/2, c_m = 1 otherwise.  Since e^{i pi (k + n j) / n} =
// e^{i pi k / n} (-1)^j, both sums come from one signed fold per residue,
//   S_k = sum_j (-1)^{h j} c_{k+nj} F_{k+nj},
//   B_k = w_k S_k + conj(w_k' S_k'),  w_k = e^{i pi h k / n}, k' = -k mod n,
// so every F_m is read once and the phases cost one table value per k.
//
// Transforms.  Lengths n = 4 i whose prime factors are all <= 13 use an
// in-place mixed-radix decimation-in-frequency FFT (radix 16 and 8
// butterflies in registers, then 4 or 2, then odd primes); the output order is
// undone through a per-length position table.  Lengths with a larger prime
// factor use Bluestein's algorithm: the DFT becomes a cyclic convolution of
// power-of-two length M >= 2n - 1 with the chirp h_t = e^{-i pi t^2 / n},
// computed as a forward DIF FFT, a product with the chirp spectrum (stored in
// DIF output order) and the adjoint of the DIF FFT, so no permutation pass is
// needed.  Shared-memory buffers are padded (glg_zi) so that the strides of
// the passes and of the digit-reversed output gather are free of bank
// conflicts.
//
// Rings are launched in size buckets built with the plan (one launch per
// bucket, all maps of the call in one grid with the map index fastest, so the
// blocks that share a ring's tables run together).
#include <cuda_runtime.h>
#include <type_traits>

#include <math.h>

#include <algorithm>

#include "glg_internal.cuh"
#include "tc_ptx.cuh"

namespace {

constexpr int TMAX = 512;        // block size limit of the kernel with odd radices (125 registers)
constexpr int TMAX_POW2 = 1024;  // power-of-two transforms (64 registers): up to 1024 threads
constexpr int EPI_MAX = 40;

struct c32 {
    float x, y;
};
__device__ __forceinline__ c32 cmul(c32 a, c32 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ c32 cadd(c32 a, c32 b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ c32 csub(c32 a, c32 b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ c32 cconj(c32 a) { return {a.x, -a.y}; }
__device__ __forceinline__ c32 cscale(c32 a, float s) { return {a.x * s, a.y * s}; }
__device__ __forceinline__ c32 ldg(const float2 *p) {
    const float2 v = __ldg(p);
    return {v.x, v.y};
}
__device__ __forceinline__ int zi(int e) { return glg_zi(e); }

// e^{DIR 2 pi i t / n}, 0 <= t < n, from the half table wh[zi(t)] = e^{2 pi i t / n},
// t <= n/2 (padded like the data, so strided twiddle reads rarely share a bank).
template <int DIR>
__device__ __forceinline__ c32 tw(const c32 *wh, int n, int t) {
    const bool lo = t <= (n >> 1);
    c32 w = wh[zi(lo ? t : n - t)];
    if (lo != (DIR > 0)) w.y = -w.y;
    return w;
}

// ------------------------------------------------------- register DFTs
// y_k = sum_j v_j e^{DIR 2 pi i j k / R}, natural order in and out.

template <int DIR>
__device__ __forceinline__ c32 mul_i(c32 a) {  // a * (DIR i)
    return DIR > 0 ? c32{-a.y, a.x} : c32{a.y, -a.x};
}

template <int DIR>
__device__ __forceinline__ void dft4(c32 &v0, c32 &v1, c32 &v2, c32 &v3) {
    const c32 a = cadd(v0, v2), b = csub(v0, v2), c = cadd(v1, v3), d = mul_i<DIR>(csub(v1, v3));
    v0 = cadd(a, c);
    v2 = csub(a, c);
    v1 = cadd(b, d);
    v3 = csub(b, d);
}

constexpr float R2 = 0.70710678118654752440f;   // cos(pi/4)
constexpr float C8 = 0.92387953251128675613f;   // cos(pi/8)
constexpr float S8 = 0.38268343236508977173f;   // sin(pi/8)

// Radix constants as FP32 (hi, lo) pairs: hi the float nearest to the exact
// value, lo the float nearest to the remainder.  Products with them are taken
// as fma(x, hi, x * lo), one rounding of the full product: the constants'
// own rounding (cos(pi/4), cos(pi/8) and sin(pi/8) all round down in FP32)
// would otherwise shrink every output of every radix-8/16 butterfly by the
// same 2-3e-8, a bias that accumulates over the passes of a transform.
constexpr float R2L = 1.21016175e-08f, C8L = 2.83074897e-08f, S8L = 6.22335072e-09f;
// e^{2 pi i j / R} for the odd radices R = 3, 5, 7, 11, 13 (j = 0 .. R-1),
// from odd_ofs(R) on in the tables.
__constant__ float2 kOddHi[] = {
    {1.0f, 0.0f}, {-0.5f, 0.866025388f}, {-0.5f, -0.866025388f},  // R = 3
    {1.0f, 0.0f}, {0.309017003f, 0.95105654f}, {-0.809017003f, 0.587785244f}, {-0.809017003f, -0.587785244f}, {0.309017003f, -0.95105654f},  // R = 5
    {1.0f, 0.0f}, {0.623489797f, 0.781831503f}, {-0.222520933f, 0.974927902f}, {-0.90096885f, 0.433883727f}, {-0.90096885f, -0.433883727f}, {-0.222520933f, -0.974927902f}, {0.623489797f, -0.781831503f},  // R = 7
    {1.0f, 0.0f}, {0.841253519f, 0.540640831f}, {0.415415019f, 0.909631968f}, {-0.142314836f, 0.989821434f}, {-0.654860735f, 0.755749583f}, {-0.959492981f, 0.281732559f}, {-0.959492981f, -0.281732559f}, {-0.654860735f, -0.755749583f}, {-0.142314836f, -0.989821434f}, {0.415415019f, -0.909631968f}, {0.841253519f, -0.540640831f},  // R = 11
    {1.0f, 0.0f}, {0.885456026f, 0.46472317f}, {0.568064749f, 0.822983861f}, {0.120536678f, 0.992708862f}, {-0.3546049f, 0.935016215f}, {-0.748510778f, 0.663122654f}, {-0.970941842f, 0.239315659f}, {-0.970941842f, -0.239315659f}, {-0.748510778f, -0.663122654f}, {-0.3546049f, -0.935016215f}, {0.120536678f, -0.992708862f}, {0.568064749f, -0.822983861f}, {0.885456026f, -0.46472317f},  // R = 13
};
__constant__ float2 kOddLo[] = {
    {0.0f, 0.0f}, {0.0f, 1.55436251e-08f}, {0.0f, -1.55436251e-08f},  // R = 3
    {0.0f, 0.0f}, {-8.2076026e-09f, -2.3717206e-08f}, {8.2076026e-09f, 8.30443625e-09f}, {8.2076026e-09f, -8.30443625e-09f}, {-8.2076026e-09f, 2.3717206e-08f},  // R = 5
    {0.0f, 0.0f}, {4.74340744e-09f, -2.04463984e-08f}, {-1.40111578e-09f, 9.96014382e-09f}, {-1.8243453e-08f, 1.25207258e-08f}, {-1.8243453e-08f, -1.25207258e-08f}, {-1.40111578e-09f, -9.96014382e-09f}, {4.74340744e-09f, 2.04463984e-08f},  // R = 7
    {0.0f, 0.0f}, {1.37729534e-08f, -1.35380551e-08f}, {-5.79503423e-09f, 2.78099623e-08f}, {-1.89041915e-09f, 7.8599367e-09f}, {9.94290095e-10f, -8.89006557e-09f}, {7.81937093e-09f, -2.36267184e-09f}, {7.81937093e-09f, 2.36267184e-09f}, {9.94290095e-10f, 8.89006557e-09f}, {-1.89041915e-09f, -7.8599367e-09f}, {-5.79503423e-09f, -2.78099623e-08f}, {1.37729534e-08f, 1.35380551e-08f},  // R = 11
    {0.0f, 0.0f}, {5.2776547e-11f, 2.24014918e-09f}, {-2.50971954e-09f, 4.92411312e-09f}, {2.71597456e-09f, 1.22702035e-08f}, {1.28407347e-08f, 2.78378494e-08f}, {2.97791853e-08f, 4.27961355e-09f}, {2.41762734e-08f, 5.47980328e-09f}, {2.41762734e-08f, -5.47980328e-09f}, {2.97791853e-08f, -4.27961355e-09f}, {1.28407347e-08f, -2.78378494e-08f}, {2.71597456e-09f, -1.22702035e-08f}, {-2.50971954e-09f, -4.92411312e-09f}, {5.2776547e-11f, -2.24014918e-09f},  // R = 13
};
__device__ __forceinline__ int odd_ofs(int R) {
    return R == 3 ? 0 : R == 5 ? 3 : R == 7 ? 8 : R == 11 ? 15 : 26;
}
__device__ __forceinline__ float mulc(float x, float h, float l) { return fmaf(x, h, x * l); }
// a * (wh + wl) with one rounding per component
__device__ __forceinline__ c32 cmulc(c32 a, c32 wh, c32 wl) {
    const float pr = fmaf(a.x, wl.x, -(a.y * wl.y)), pi = fmaf(a.x, wl.y, a.y * wl.x);
    return {fmaf(a.x, wh.x, fmaf(-a.y, wh.y, pr)), fmaf(a.x, wh.y, fmaf(a.y, wh.x, pi))};
}

template <int DIR>
__device__ __forceinline__ void dft8(c32 *v) {
    c32 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    c32 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<DIR>(e0, e1, e2, e3);
    dft4<DIR>(o0, o1, o2, o3);
    // o_k *= e^{DIR 2 pi i k / 8}
    o1 = c32{mulc(o1.x - DIR * o1.y, R2, R2L), mulc(o1.y + DIR * o1.x, R2, R2L)};
    o2 = mul_i<DIR>(o2);
    o3 = c32{mulc(-o3.x - DIR * o3.y, R2, R2L), mulc(DIR * o3.x - o3.y, R2, R2L)};
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
}

template <int DIR>
__device__ __forceinline__ void dft16(c32 *v) {
    // j = j2 + 4 j1: length-4 DFTs over j1, twiddles w16^(j2 k1), length-4
    // DFTs over j2; y[k1 + 4 k2] lands in u[4 k1 + k2].
    c32 u[16];
#pragma unroll
    for (int j2 = 0; j2 < 4; ++j2) {
        c32 a = v[j2], b = v[j2 + 4], c = v[j2 + 8], d = v[j2 + 12];
        dft4<DIR>(a, b, c, d);
        u[4 * 0 + j2] = a;
        u[4 * 1 + j2] = b;
        u[4 * 2 + j2] = c;
        u[4 * 3 + j2] = d;
    }
    const float D = (float)DIR;
    // u[4 k1 + j2] *= e^{DIR 2 pi i j2 k1 / 16}
    const c32 w1 = {C8, D * S8}, w2 = {R2, D * R2}, w3 = {S8, D * C8};
    const c32 w6 = {-R2, D * R2}, w9 = {-C8, -D * S8};
    const c32 l1 = {C8L, D * S8L}, l2 = {R2L, D * R2L}, l3 = {S8L, D * C8L};
    const c32 l6 = {-R2L, D * R2L}, l9 = {-C8L, -D * S8L};
    u[5] = cmulc(u[5], w1, l1);
    u[6] = cmulc(u[6], w2, l2);
    u[7] = cmulc(u[7], w3, l3);
    u[9] = cmulc(u[9], w2, l2);
    u[10] = mul_i<DIR>(u[10]);
    u[11] = cmulc(u[11], w6, l6);
    u[13] = cmulc(u[13], w3, l3);
    u[14] = cmulc(u[14], w6, l6);
    u[15] = cmulc(u[15], w9, l9);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4<DIR>(u[4 * k1], u[4 * k1 + 1], u[4 * k1 + 2], u[4 * k1 + 3]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = u[4 * k1 + k2];
}

// Odd prime radix with the constant twiddles e^{DIR 2 pi i (j k mod R) / R}.
template <int R, int DIR>
__device__ __forceinline__ void dft_odd(c32 *v) {
    c32 y[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        c32 acc = v[0];
#pragma unroll
        for (int j = 1; j < R; ++j) {
            const int q = odd_ofs(R) + (j * k) % R;
            c32 h = {kOddHi[q].x, kOddHi[q].y}, l = {kOddLo[q].x, kOddLo[q].y};
            if (DIR < 0) {
                h.y = -h.y;
                l.y = -l.y;
            }
            acc = cadd(acc, cmulc(v[j], h, l));
        }
        y[k] = acc;
    }
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = y[k];
}

template <int R, int DIR>
__device__ __forceinline__ void dft(c32 *v, const c32 *wh, int n) {
    if constexpr (R == 2) {
        const c32 a = v[0];
        v[0] = cadd(a, v[1]);
        v[1] = csub(a, v[1]);
    } else if constexpr (R == 4) {
        dft4<DIR>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R == 8) {
        dft8<DIR>(v);
    } else if constexpr (R == 16) {
        dft16<DIR>(v);
    } else {
        dft_odd<R, DIR>(v);
    }
}

// One in-place DIF pass of radix R (sub-length L) of a length-n transform,
// or its adjoint.  DIF: y = DFT_R(v), then y_k *= w_L^(DIR j1 k).  Adjoint:
// v_k *= w_L^(-DIR j1 k), then y = DFT_R^(-DIR)(v).
// P2: n is a power of two, so the butterfly's sub-transform and position
// come from shifts and masks instead of integer divisions.
// ZV: elements at or beyond nv are zero and not read (the zero padding of a
// Bluestein input, on its first pass).
template <int R, int DIR, bool ADJ, bool P2, bool ZV = false>
__device__ __forceinline__ void pass(c32 *Z, const c32 *wh, int n, int L, int nv = 0) {
    const int msub = L / R, nbf = n / R, tsc = n / L;
    // with 32 or more sub-transforms, neighbouring threads take neighbouring
    // sub-transforms (same twiddles: one broadcast read); otherwise
    // neighbouring butterflies of one sub-transform
    const bool by_blk = tsc >= 32;
    const int lg_tsc = __ffs(tsc) - 1, lg_msub = __ffs(msub) - 1;
    for (int bf = threadIdx.x; bf < nbf; bf += blockDim.x) {
        int blk, j1;
        if constexpr (P2) {
            blk = by_blk ? bf & (tsc - 1) : bf >> lg_msub;
            j1 = by_blk ? bf >> lg_tsc : bf & (msub - 1);
        } else {
            blk = by_blk ? bf % tsc : bf / msub;
            j1 = by_blk ? bf / tsc : bf - blk * msub;
        }
        const int base = blk * L + j1;
        const int ts = tsc * j1;
        c32 v[R];
        if constexpr (!ADJ) {
#pragma unroll
            for (int j = 0; j < R; ++j) {
                if constexpr (ZV) v[j] = base + msub * j < nv ? Z[zi(base + msub * j)] : c32{0.f, 0.f};
                else v[j] = Z[zi(base + msub * j)];
            }
            dft<R, DIR>(v, wh, n);
            Z[zi(base)] = v[0];
#pragma unroll
            for (int k = 1; k < R; ++k) Z[zi(base + msub * k)] = cmul(v[k], tw<DIR>(wh, n, ts * k));
        } else {
            v[0] = Z[zi(base)];
#pragma unroll
            for (int k = 1; k < R; ++k) v[k] = cmul(Z[zi(base + msub * k)], tw<-DIR>(wh, n, ts * k));
            dft<R, -DIR>(v, wh, n);
#pragma unroll
            for (int j = 0; j < R; ++j) Z[zi(base + msub * j)] = v[j];
        }
    }
    __syncthreads();
}

template <int DIR, bool ADJ, bool POW2>
__device__ __forceinline__ void pass_any(c32 *Z, const c32 *wh, int n, int R, int L) {
    switch (R) {
        case 16: pass<16, DIR, ADJ, POW2>(Z, wh, n, L); break;
        case 8: pass<8, DIR, ADJ, POW2>(Z, wh, n, L); break;
        case 4: pass<4, DIR, ADJ, POW2>(Z, wh, n, L); break;
        case 2: pass<2, DIR, ADJ, POW2>(Z, wh, n, L); break;
        default:
            if constexpr (!POW2) {
                switch (R) {
                    case 3: pass<3, DIR, ADJ, POW2>(Z, wh, n, L); break;
                    case 5: pass<5, DIR, ADJ, POW2>(Z, wh, n, L); break;
                    case 7: pass<7, DIR, ADJ, POW2>(Z, wh, n, L); break;
                    case 11: pass<11, DIR, ADJ, POW2>(Z, wh, n, L); break;
                    case 13: pass<13, DIR, ADJ, POW2>(Z, wh, n, L); break;
                    default: break;
                }
            }
            break;
    }
}

// First forward pass of a power-of-two transform whose input is zero at and
// beyond nv.
template <int DIR>
__device__ __forceinline__ void pass_first_zv(c32 *Z, const c32 *wh, int n, int R, int L, int nv) {
    switch (R) {
        case 16: pass<16, DIR, false, true, true>(Z, wh, n, L, nv); break;
        case 8: pass<8, DIR, false, true, true>(Z, wh, n, L, nv); break;
        case 4: pass<4, DIR, false, true, true>(Z, wh, n, L, nv); break;
        case 2: pass<2, DIR, false, true, true>(Z, wh, n, L, nv); break;
        default: break;
    }
}

// nv < n: the input is zero at and beyond nv (power-of-two n only).
// skip_last: leave out the last pass (the caller folds it into its reads).
template <int DIR, bool POW2>
__device__ void fft_dif(c32 *Z, const c32 *wh, int n, int nv = -1, bool skip_last = false) {
    int r[GLG_MAX_FFT_STAGES];
    const int ns = glg_fft32_radices(n, r) - (skip_last ? 1 : 0);
    int L = n;
    for (int s = 0; s < ns; ++s) {
        if (POW2 && s == 0 && nv >= 0) pass_first_zv<DIR>(Z, wh, n, r[s], L, nv);
        else pass_any<DIR, false, POW2>(Z, wh, n, r[s], L);
        L /= r[s];
    }
}

template <int DIR, bool POW2>
__device__ void fft_dif_adjoint(c32 *Z, const c32 *wh, int n) {
    int r[GLG_MAX_FFT_STAGES], Ls[GLG_MAX_FFT_STAGES];
    const int ns = glg_fft32_radices(n, r);
    int L = n;
    for (int s = 0; s < ns; ++s) {
        Ls[s] = L;
        L /= r[s];
    }
    for (int s = ns - 1; s >= 0; --s) pass_any<DIR, true, POW2>(Z, wh, n, r[s], Ls[s]);
}

// Power-of-two transforms of a compile-time length N: the same passes (16s,
// then one 8, 4 or 2) with every index, shift and mask a constant.
// The passes of a compile-time length: 3 * 2^k lengths take their radix-3
// pass first (the rest is a power of two), then 16s, then one 8, 4 or 2.
template <int L>
struct RadixOf {
    static constexpr int value = L % 3 == 0 ? 3 : (L % 16 == 0 ? 16 : L);
};

// Per-pass twiddle tables of a compile-time length N: for every DIF pass
// below the first (sub-length L < N) with more than one butterfly column
// (msub = L / R > 1), the R - 1 rows [k - 1][j1] of e^{2 pi i j1 k / L},
// j1 < msub, so that a thread's twiddles sit at constant offsets from its
// column and neighbouring threads read neighbouring words.  WTab<N, L>:
// offset of pass L's rows, and the total size of the passes from L down.
template <int N, int L>
struct WTab {
    static constexpr int R = L > 1 ? RadixOf<L>::value : 1;
    static constexpr int own = (L < N && L > 1 && L / R > 1) ? (R - 1) * (L / R) : 0;
    static constexpr int below = L > 1 ? WTab<N, L / R>::total : 0;
    static constexpr int total = own + below;
};
template <int N>
struct WTab<N, 1> {
    static constexpr int R = 1, own = 0, below = 0, total = 0;
};
// offset of pass L's rows when the passes from N down are laid out in order
template <int N, int L>
struct WOfs {
    static constexpr int value = WTab<N, N>::total - WTab<N, L>::total;
};

// Fill the per-pass tables from the padded half table wh (the same values
// tw() gives, so the transforms are unchanged); ends with __syncthreads().
template <int N, int L>
__device__ __forceinline__ void wtab_fill_rec(c32 *wp, const c32 *wh) {
    if constexpr (L > 1) {
        constexpr int R = RadixOf<L>::value, msub = L / R, own = WTab<N, L>::own;
        if constexpr (own > 0) {
            c32 *w = wp + WOfs<N, L>::value;
            for (int q = threadIdx.x; q < own; q += blockDim.x) {
                const int k = q / msub + 1, j1 = q % msub;
                w[q] = tw<1>(wh, N, (N / L) * j1 * k);
            }
        }
        wtab_fill_rec<N, L / R>(wp, wh);
    }
}
template <int N>
__device__ __forceinline__ void wtab_fill(c32 *wp, const c32 *wh) {
    wtab_fill_rec<N, N>(wp, wh);
    __syncthreads();
}

template <int E>
struct ZiC {  // glg_zi(E) as a constant
    static constexpr int value = E + (E >> 4) + (E >> 8);
};

// cmul by w (DIR > 0) or by conj(w) (DIR < 0)
template <int DIR>
__device__ __forceinline__ c32 cmul_dir(c32 a, c32 w) {
    return cmul(a, DIR > 0 ? w : cconj(w));
}

// Host copy of WTab<N, N>::total (entries of the per-pass tables of N).
static int wtab_total_host(int N) {
    int tot = 0;
    for (int L = N; L > 1;) {
        const int R = L % 3 == 0 ? 3 : (L % 16 == 0 ? 16 : L), msub = L / R;
        if (L < N && msub > 1) tot += (R - 1) * msub;
        L /= R;
    }
    return tot;
}

// One DIF pass (or its adjoint) of radix R, sub-length L, length N.  wp:
// the per-pass tables of wtab_fill (null: twiddles from wh).  For msub >=
// 16 the padded offsets of a butterfly's elements are constants from its
// first (the column j1 < msub adds no carry into bits 4 and 8); for msub
// == 1 every twiddle is 1.
template <int R, int DIR, bool ADJ, bool ZV, int N, int L>
__device__ __forceinline__ void pass_ct(c32 *Z, const c32 *wh, const c32 *wp, int nv) {
    constexpr int msub = L / R, nbf = N / R, tsc = N / L;
    constexpr bool by_blk = tsc >= 32;
    constexpr bool cidx = msub >= 16;
    constexpr bool unit = msub == 1;
    const bool table = wp != nullptr && L < N && !unit;
    const c32 *wl = table ? wp + WOfs<N, L>::value : nullptr;
    for (int bf = threadIdx.x; bf < nbf; bf += blockDim.x) {
        // divisions by constants (shifts and masks for powers of two)
        const int blk = by_blk ? bf % tsc : bf / msub;
        const int j1 = by_blk ? bf / tsc : bf % msub;
        const int base = blk * L + j1;
        const int ts = tsc * j1;
        const int zb = zi(base);
        c32 *zp = Z + zb;
        // element j of the butterfly (j a constant once unrolled)
        auto el = [&](int j) -> c32 & {
            return cidx ? zp[msub * j + ((msub * j) >> 4) + ((msub * j) >> 8)] : Z[zi(base + msub * j)];
        };
        // a * e^{D 2 pi i ts k / N}
        auto twm = [&](c32 a, int k, auto dtag) -> c32 {
            constexpr int D = decltype(dtag)::value;
            if (table) return cmul_dir<D>(a, wl[(k - 1) * msub + j1]);
            return cmul(a, tw<D>(wh, N, ts * k));
        };
        c32 v[R];
        if constexpr (!ADJ) {
#pragma unroll
            for (int j = 0; j < R; ++j) {
                if constexpr (ZV) v[j] = base + msub * j < nv ? el(j) : c32{0.f, 0.f};
                else v[j] = el(j);
            }
            dft<R, DIR>(v, wh, N);
            el(0) = v[0];
#pragma unroll
            for (int k = 1; k < R; ++k) el(k) = unit ? v[k] : twm(v[k], k, std::integral_constant<int, DIR>{});
        } else {
            v[0] = el(0);
#pragma unroll
            for (int k = 1; k < R; ++k) v[k] = unit ? el(k) : twm(el(k), k, std::integral_constant<int, -DIR>{});
            dft<R, -DIR>(v, wh, N);
#pragma unroll
            for (int j = 0; j < R; ++j) el(j) = v[j];
        }
    }
    __syncthreads();
}

// DIF passes from sub-length L down; the first pass reads zeros at and
// beyond nv when ZV; SKIP2: a last radix-2 pass is left to the caller.
template <int DIR, int N, int L, bool ZV, bool SKIP2>
__device__ __forceinline__ void dif_ct(c32 *Z, const c32 *wh, int nv, const c32 *wp = nullptr) {
    if constexpr (L > 1) {
        constexpr int R = RadixOf<L>::value;
        if constexpr (!(SKIP2 && L == 2 && R == 2 && N > 2)) {
            pass_ct<R, DIR, false, ZV, N, L>(Z, wh, wp, nv);
            dif_ct<DIR, N, L / R, false, SKIP2>(Z, wh, nv, wp);
        }
    }
}

// The adjoint of dif_ct<DIR, N, L>: its passes in reverse order.
template <int DIR, int N, int L>
__device__ __forceinline__ void adj_ct(c32 *Z, const c32 *wh, const c32 *wp = nullptr) {
    if constexpr (L > 1) {
        constexpr int R = RadixOf<L>::value;
        adj_ct<DIR, N, L / R>(Z, wh, wp);
        pass_ct<R, DIR, true, false, N, L>(Z, wh, wp, 0);
    }
}

// ------------------------------------------------------------- epilogue

__device__ __forceinline__ float epi(float v, int kind, float hv, float lam) {
    if (kind == GLG_EPI_LOGNORMAL) {
        v = expm1f(v - hv);
        if (lam != 1.0f) v = lam * v;
    }
    return v;
}

struct Epi32 {
    int kind[EPI_MAX];
    float hvar[EPI_MAX], lam[EPI_MAX];  // var / 2 and lambda per map
    float thr[EPI_MAX];                 // tail-refinement threshold on the Gaussian value (+inf: none)
    int *rcount;                        // tail-refinement list: entries appended, capacity, items
    int rcap;
    int4 *ritems;
};

// Tail refinement.  The lognormal map's relative RMS error is dominated by
// its largest pixels (weight y^2 ~ e^{2 g}); at sigma^2 ~ 7 the top few
// thousand of 50 M pixels carry ~90% of it, and there the FP32 transform's
// rounding (~1.4e-7 of sigma, plus the rounding of g itself before the
// exponential) is what is left.  The output loops list every pixel whose
// Gaussian value exceeds thr = var/2 + log1p(sqrt(KAPPA expm1(var))), i.e.
// whose lognormal value exceeds sqrt(KAPPA) times the map's RMS, on maps
// whose variance reaches REFINE_MIN_VAR; k_refine then recomputes those
// pixels from the Legendre sums by a direct FP64 sum over m and the FP64
// transform.  Below REFINE_MIN_VAR the FP32 pipeline's error stays well
// inside 1e-6 without it.
constexpr double REFINE_KAPPA = 1000.0;
constexpr double REFINE_MIN_VAR = 4.0;

__device__ __forceinline__ void refine_note(const Epi32 &e, float thr, int map, float g, int ring, int k) {
    if (g > thr) {
        const int slot = atomicAdd(e.rcount, 1);
        if (slot < e.rcap) e.ritems[slot] = make_int4(map, ring, k, 0);
    }
}

struct RingArgs {
    int nrings, mmax, nmaps;
    const int *pairs;  // ring pairs of this launch
    const int *nph, *half;
    const int64_t *startN, *startS;
    const int64_t *tw_ofs;
    const float2 *tw32;  // e^{i pi t / n}, t < 2n, per length
    const int64_t *pos_ofs;
    const uint16_t *pos16;
    const int64_t *blu_ofs, *chirp_ofs;
    const int *blu_M;
    const float2 *blu_H, *chirp, *twM;
    int Mmax;
    const float2 *twMp;  // padded twiddles of Mmax (class 3)
    float2 *gz;          // global transform buffers of class 3, glg_zsize(Mmax) per block
    const float2 *Ft;  // [map][ring][m]
    float *maps;
    int64_t npix;
    const float2 *twp;   // padded half twiddle tables by log2 length (staged kernels)
    int64_t twp_ofs[16];
    int64_t twp3_ofs[16];  // the same for lengths 3 * 2^k, by k
    int *err;            // status word for a staged copy that never arrived (or null)
    const glg_epi_dev *edev;  // epilogue in device memory (graph-captured calls), or null
};

// Offset of the padded half twiddle table of length M (2^k or 3 * 2^k) in twp.
__device__ __forceinline__ int64_t twp_offset(const RingArgs &a, int M) {
    return (M % 3 == 0) ? a.twp3_ofs[__ffs(M / 3) - 1] : a.twp_ofs[__ffs(M) - 1];
}

// The epilogue of one map: from the device epilogue when the call has one.
struct EpiMap {
    int kind;
    float hv, lam, thr;
};
__device__ __forceinline__ EpiMap epi_map(const RingArgs &a, const Epi32 &e, int map) {
    if (a.edev) return {a.edev->kind[map], a.edev->hvar[map], a.edev->lam[map], a.edev->thr[map]};
    return {e.kind[map], e.hvar[map], e.lam[map], e.thr[map]};
}

__device__ __forceinline__ c32 pack(c32 bn, c32 bs) { return {bn.x - bs.y, bn.y + bs.x}; }

// Z[zi(k)] = B^N_k + i B^S_k for k < n (times chirp[k] when chirp != null).
// SS: scratch of the south fold, element k at SS[zi(soff + k)] (may alias Z
// beyond n); X: 2 x blockDim partial sums.  Ends with __syncthreads().
__device__ void fold(const float2 *FN, const float2 *FS, bool equator, int n, int mmax, int h,
                     const float2 *w2n, const float2 *chirp, c32 *Z, c32 *SS, int soff, c32 *X) {
    const int T = blockDim.x, t = threadIdx.x;
    const c32 one = {1.f, 0.f};
    if (n > mmax) {
        // at most one term per residue: read F directly; the residues k and
        // n - k use the same two values of F, so one thread makes both
#pragma unroll 2
        for (int k = t; k <= (n >> 1); k += T) {
            const int k2 = k ? n - k : 0;
            const float ck = k ? 1.f : 0.5f;
            c32 fn = {0.f, 0.f}, fs = fn, gn = fn, gs = fn;  // F at k and at k2
            if (k <= mmax) {
                fn = ldg(FN + k);
                fs = ldg(FS + k);
            }
            if (k2 <= mmax) {
                gn = ldg(FN + k2);
                gs = ldg(FS + k2);
            }
            const c32 wk = h ? ldg(w2n + k) : one, wk2 = h ? ldg(w2n + k2) : one;
            const c32 an = cscale(fn, ck), as = cscale(fs, ck), bn = cscale(gn, ck), bs = cscale(gs, ck);
            const c32 BN = cadd(cmul(wk, an), cconj(cmul(wk2, bn)));
            c32 BS = cadd(cmul(wk, as), cconj(cmul(wk2, bs)));
            if (equator) BS = {0.f, 0.f};
            c32 z = pack(BN, BS);
            if (chirp) z = cmul(z, ldg(chirp + k));
            Z[zi(k)] = z;
            if (k2 != k) {  // residue n - k: the roles of the two values swap
                const c32 BN2 = cadd(cmul(wk2, gn), cconj(cmul(wk, fn)));
                c32 BS2 = cadd(cmul(wk2, gs), cconj(cmul(wk, fs)));
                if (equator) BS2 = {0.f, 0.f};
                c32 z2 = pack(BN2, BS2);
                if (chirp) z2 = cmul(z2, ldg(chirp + k2));
                Z[zi(k2)] = z2;
            }
        }
        __syncthreads();
        return;
    }
    // signed fold S_k: one thread per residue, or C threads per residue
    // (fixed slices, summed in order) when n < blockDim
    const float sgn = h ? -1.f : 1.f;
    if (n >= T) {
        for (int k = t; k < n; k += T) {
            c32 sn = {0.f, 0.f}, ss = sn;
            float s = 1.f;
            for (int m = k; m <= mmax; m += n, s *= sgn) {
                const float c = m ? s : 0.5f * s;
                const c32 fn = ldg(FN + m), fs = ldg(FS + m);
                sn = {fmaf(c, fn.x, sn.x), fmaf(c, fn.y, sn.y)};
                ss = {fmaf(c, fs.x, ss.x), fmaf(c, fs.y, ss.y)};
            }
            Z[zi(k)] = sn;
            SS[zi(soff + k)] = ss;
        }
    } else {
        const int C = T / n;
        if (t < C * n) {
            const int k = t % n, c = t / n;
            c32 sn = {0.f, 0.f}, ss = sn;
            const float sC = (h && (C & 1)) ? -1.f : 1.f;  // sign step over C folds
            float s = (h && (c & 1)) ? -1.f : 1.f;
            for (int m = k + c * n; m <= mmax; m += C * n, s *= sC) {
                const float cc = m ? s : 0.5f * s;
                const c32 fn = ldg(FN + m), fs = ldg(FS + m);
                sn = {fmaf(cc, fn.x, sn.x), fmaf(cc, fn.y, sn.y)};
                ss = {fmaf(cc, fs.x, ss.x), fmaf(cc, fs.y, ss.y)};
            }
            X[t] = sn;
            X[T + t] = ss;
        }
        __syncthreads();
        if (t < n) {
            c32 sn = X[t], ss = X[T + t];
            for (int c = 1; c < C; ++c) {
                sn = cadd(sn, X[c * n + t]);
                ss = cadd(ss, X[T + c * n + t]);
            }
            Z[zi(t)] = sn;
            SS[zi(soff + t)] = ss;
        }
    }
    __syncthreads();
    // combine the residue pair (k, n - k)
    for (int k = t; k <= (n >> 1); k += T) {
        const int k2 = k ? n - k : 0;
        const c32 an = Z[zi(k)], bn = Z[zi(k2)];
        c32 as = SS[zi(soff + k)], bs = SS[zi(soff + k2)];
        if (equator) as = bs = {0.f, 0.f};
        const c32 wk = h ? ldg(w2n + k) : one, wk2 = h ? ldg(w2n + k2) : one;
        const c32 pa = cmul(wk, an), pb = cmul(wk2, bn), qa = cmul(wk, as), qb = cmul(wk2, bs);
        c32 z = pack(cadd(pa, cconj(pb)), cadd(qa, cconj(qb)));
        if (chirp) z = cmul(z, ldg(chirp + k));
        Z[zi(k)] = z;
        if (k2 != k) {
            c32 z2 = pack(cadd(pb, cconj(pa)), cadd(qb, cconj(qa)));
            if (chirp) z2 = cmul(z2, ldg(chirp + k2));
            Z[zi(k2)] = z2;
        }
    }
    __syncthreads();
}

// Class 0 (any n) and class 2 (power-of-two equatorial n, POW2: radices
// 16/8/4/2 only):
// mixed-radix DIF.  smem: Z | SS (n <= mmax) | X[2T] | wh[zi(n/2) + 1].
// LOGN > 0 (class 2 only): the ring length is 2^LOGN, a compile-time constant.
template <bool POW2, int LOGN = 0>
__global__ void __launch_bounds__(POW2 ? TMAX_POW2 : TMAX) k_ring32(const RingArgs a, const Epi32 e) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int map = blockIdx.x % a.nmaps;
    const int p = a.pairs[blockIdx.x / a.nmaps];
    const int n = a.nph[p], i4 = n / 4, T = blockDim.x;
    const bool folds = n <= a.mmax;
    const int zs = glg_zsize(n);
    c32 *Z = reinterpret_cast<c32 *>(smem_raw);
    c32 *SS = Z + zs;
    c32 *X = SS + (folds ? zs : 0);
    c32 *wh = X + 2 * T;
    const float2 *w2n = a.tw32 + a.tw_ofs[i4];  // e^{i pi t / n}, t < 2n
    for (int t = threadIdx.x; t <= n / 2; t += T) wh[zi(t)] = ldg(w2n + 2 * t);
    const int rn = p, rs = a.nrings - 1 - p;
    const bool equator = rn == rs;
    const float2 *FN = a.Ft + ((int64_t)map * a.nrings + rn) * (a.mmax + 1);
    const float2 *FS = a.Ft + ((int64_t)map * a.nrings + rs) * (a.mmax + 1);
    fold(FN, FS, equator, n, a.mmax, a.half[p], w2n, nullptr, Z, SS, 0, X);
    // a last DIF pass of radix 2 (L = 2: no twiddles) is folded into the
    // output gather: frequency at storage slot s is Z[s & ~1] +- Z[s | 1]
    bool last2;
    if constexpr (LOGN > 0) {
        constexpr int N = 1 << LOGN;
        // the passes are 16s then one 8/4/2: the last is radix 2 when log2(N) % 4 == 1
        last2 = LOGN > 1 && LOGN % 4 == 1;
        dif_ct<1, N, N, false, true>(Z, wh, 0);
    } else {
        int rr[GLG_MAX_FFT_STAGES];
        const int nst = glg_fft32_radices(n, rr);
        last2 = POW2 && nst > 1 && rr[nst - 1] == 2;
        fft_dif<1, POW2>(Z, wh, n, -1, last2);
    }
    const uint16_t *pos = a.pos16 + a.pos_ofs[i4];
    float *mp = a.maps + (int64_t)map * a.npix;
    const int64_t sN = a.startN[p], sS = a.startS[p];
    const EpiMap em = epi_map(a, e, map);
    const int kind = em.kind;
    const float hv = em.hv, lam = em.lam;
    // four consecutive pixels per thread, stored as one 16-byte vector (ring
    // starts and lengths are multiples of 4 pixels): fewer, larger stores,
    // which the CPU-GPU link takes better when the maps are host memory
#pragma unroll 2
    for (int q = threadIdx.x; q < (n >> 2); q += T) {
        const ushort4 ps = *reinterpret_cast<const ushort4 *>(pos + 4 * q);
        auto at = [&](int sl) -> c32 {
            if (!last2) return Z[zi(sl)];
            const c32 u0 = Z[zi(sl & ~1)], u1 = Z[zi(sl | 1)];
            return (sl & 1) ? csub(u0, u1) : cadd(u0, u1);
        };
        const c32 v0 = at(ps.x), v1 = at(ps.y), v2 = at(ps.z), v3 = at(ps.w);
        if (kind == GLG_EPI_LOGNORMAL) {
            refine_note(e, em.thr, map, v0.x, rn, 4 * q);
            refine_note(e, em.thr, map, v1.x, rn, 4 * q + 1);
            refine_note(e, em.thr, map, v2.x, rn, 4 * q + 2);
            refine_note(e, em.thr, map, v3.x, rn, 4 * q + 3);
            if (!equator) {
                refine_note(e, em.thr, map, v0.y, rs, 4 * q);
                refine_note(e, em.thr, map, v1.y, rs, 4 * q + 1);
                refine_note(e, em.thr, map, v2.y, rs, 4 * q + 2);
                refine_note(e, em.thr, map, v3.y, rs, 4 * q + 3);
            }
        }
        *reinterpret_cast<float4 *>(mp + sN + 4 * q) =
            make_float4(epi(v0.x, kind, hv, lam), epi(v1.x, kind, hv, lam), epi(v2.x, kind, hv, lam),
                        epi(v3.x, kind, hv, lam));
        if (!equator)
            *reinterpret_cast<float4 *>(mp + sS + 4 * q) =
                make_float4(epi(v0.y, kind, hv, lam), epi(v1.y, kind, hv, lam), epi(v2.y, kind, hv, lam),
                            epi(v3.y, kind, hv, lam));
    }
}

template <int CNT>
struct ZSize {  // glg_zsize(CNT) as a constant
    static constexpr int value = (CNT - 1) + ((CNT - 1) >> 4) + ((CNT - 1) >> 8) + 1;
};
constexpr uint32_t STAGE_WAIT_LIMIT = 1u << 24;  // polls of a staged copy (its data is plain HBM reads)

// Class 2 (power-of-two equatorial rings, n = 2^LOGN > mmax) with staged
// inputs: one thread bulk-copies the ring pair's two rows of Legendre sums
// (mmax + 1 values each, from the 16-byte boundary at or below each row
// start) into the raw bytes of the transform buffer and the padded half
// twiddle table of n into its own slot, all on one mbarrier; the threads
// then form the folded sequence in registers from shared memory (every
// staged value is read before the first write) and run the compile-time DIF
// passes.  T threads, n / 2 + 1 residue pairs in ceil((n/2+1)/T) per thread.
// smem: Z[zsize(n)] | wh[zsize(n/2+1)], 16-byte aligned.
template <int LOGN, int T>
__global__ void __launch_bounds__(T, T <= 512 ? 2 : 1) k_ring32eq(const RingArgs a, const Epi32 e) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int N = 1 << LOGN, NZ = ZSize<N>::value, NW = ZSize<N / 2 + 1>::value;
    constexpr int NI = (N / 2 + 1 + T - 1) / T;
    constexpr uint32_t BW = (uint32_t)(((NW * 8) + 15) & ~15);
    __shared__ __align__(8) uint64_t bar;
    const int map = blockIdx.x % a.nmaps;
    const int p = a.pairs[blockIdx.x / a.nmaps];
    const int rn = p, rs = a.nrings - 1 - p;
    const bool equator = rn == rs;
    const int mm = a.mmax + 1;
    c32 *Z = reinterpret_cast<c32 *>(smem_raw);
    c32 *wh = Z + ((NZ + 1) & ~1);
    c32 *wp = wh + ((NW + 1) & ~1);  // per-pass twiddle tables
    const float2 *FN = a.Ft + ((int64_t)map * a.nrings + rn) * mm;
    const float2 *FS = a.Ft + ((int64_t)map * a.nrings + rs) * mm;
    const int oN = (int)((reinterpret_cast<uintptr_t>(FN) >> 3) & 1);
    const int oS = (int)((reinterpret_cast<uintptr_t>(FS) >> 3) & 1);
    const uint32_t bN = (uint32_t)(((oN + mm) * 8 + 15) & ~15);
    const uint32_t bS = equator ? 0u : (uint32_t)(((oS + mm) * 8 + 15) & ~15);
    const float2 *stN = reinterpret_cast<const float2 *>(smem_raw) + oN;
    const float2 *stS = reinterpret_cast<const float2 *>(smem_raw + bN) + oS;
    if (threadIdx.x == 0) {
        glg_tc::mbar_init(&bar, 1);
        glg_tc::fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        glg_tc::mbar_arrive_expect_tx(&bar, bN + bS + BW);
        glg_tc::bulk_g2s(smem_raw, FN - oN, bN, &bar);
        if (!equator) glg_tc::bulk_g2s(smem_raw + bN, FS - oS, bS, &bar);
        glg_tc::bulk_g2s(wh, a.twp + a.twp_ofs[LOGN], BW, &bar);
    }
    if (!glg_tc::mbar_wait(&bar, 0, STAGE_WAIT_LIMIT)) {
        if (threadIdx.x == 0 && a.err) atomicExch(a.err, GLG_ERR_TIMEOUT);
        glg_tc::mbar_wait(&bar, 0, STAGE_WAIT_LIMIT);  // the copies in flight land before the block exits
        return;
    }
    wtab_fill_rec<N, N>(wp, wh);  // the barrier before the transform's first pass publishes it
    // residue pairs (k, n - k): Z_k and Z_{n-k} from F_k and F_{n-k} (one term each, n > mmax)
    const float2 *w2n = a.tw32 + a.tw_ofs[N / 4];  // e^{i pi t / n}
    const bool h = a.half[p] != 0;
    const c32 one = {1.f, 0.f}, zero = {0.f, 0.f};
    c32 z1[NI], z2[NI];
#pragma unroll
    for (int i = 0; i < NI; ++i) {
        const int k = threadIdx.x + i * T;
        z1[i] = z2[i] = zero;
        if (k <= N / 2) {
            const int k2 = k ? N - k : 0;
            const float ck = k ? 1.f : 0.5f;
            c32 fn = zero, fs = zero, gn = zero, gs = zero;
            if (k < mm) {
                fn = {stN[k].x, stN[k].y};
                if (!equator) fs = {stS[k].x, stS[k].y};
            }
            if (k2 < mm) {
                gn = {stN[k2].x, stN[k2].y};
                if (!equator) gs = {stS[k2].x, stS[k2].y};
            }
            const c32 wk = h ? ldg(w2n + k) : one, wk2 = h ? ldg(w2n + k2) : one;
            const c32 an = cscale(fn, ck), as = cscale(fs, ck), bn = cscale(gn, ck), bs = cscale(gs, ck);
            const c32 BN = cadd(cmul(wk, an), cconj(cmul(wk2, bn)));
            const c32 BS = cadd(cmul(wk, as), cconj(cmul(wk2, bs)));
            z1[i] = pack(BN, BS);
            if (k2 != k)
                z2[i] = pack(cadd(cmul(wk2, gn), cconj(cmul(wk, fn))), cadd(cmul(wk2, gs), cconj(cmul(wk, fs))));
        }
    }
    __syncthreads();  // every staged value is in registers
#pragma unroll
    for (int i = 0; i < NI; ++i) {
        const int k = threadIdx.x + i * T;
        if (k <= N / 2) {
            Z[zi(k)] = z1[i];
            if (k && k != N / 2) Z[zi(N - k)] = z2[i];
        }
    }
    __syncthreads();
    constexpr bool last2 = LOGN > 1 && LOGN % 4 == 1;
    dif_ct<1, N, N, false, true>(Z, wh, 0, wp);
    const int i4 = N / 4;
    const uint16_t *pos = a.pos16 + a.pos_ofs[i4];
    float *mp = a.maps + (int64_t)map * a.npix;
    const int64_t sN = a.startN[p], sS = a.startS[p];
    const EpiMap em = epi_map(a, e, map);
    const int kind = em.kind;
    const float hv = em.hv, lam = em.lam;
#pragma unroll 2
    for (int q = threadIdx.x; q < N / 4; q += T) {
        const ushort4 ps = *reinterpret_cast<const ushort4 *>(pos + 4 * q);
        auto at = [&](int sl) -> c32 {
            if (!last2) return Z[zi(sl)];
            const c32 u0 = Z[zi(sl & ~1)], u1 = Z[zi(sl | 1)];
            return (sl & 1) ? csub(u0, u1) : cadd(u0, u1);
        };
        const c32 v0 = at(ps.x), v1 = at(ps.y), v2 = at(ps.z), v3 = at(ps.w);
        if (kind == GLG_EPI_LOGNORMAL) {
            refine_note(e, em.thr, map, v0.x, rn, 4 * q);
            refine_note(e, em.thr, map, v1.x, rn, 4 * q + 1);
            refine_note(e, em.thr, map, v2.x, rn, 4 * q + 2);
            refine_note(e, em.thr, map, v3.x, rn, 4 * q + 3);
            if (!equator) {
                refine_note(e, em.thr, map, v0.y, rs, 4 * q);
                refine_note(e, em.thr, map, v1.y, rs, 4 * q + 1);
                refine_note(e, em.thr, map, v2.y, rs, 4 * q + 2);
                refine_note(e, em.thr, map, v3.y, rs, 4 * q + 3);
            }
        }
        *reinterpret_cast<float4 *>(mp + sN + 4 * q) =
            make_float4(epi(v0.x, kind, hv, lam), epi(v1.x, kind, hv, lam), epi(v2.x, kind, hv, lam),
                        epi(v3.x, kind, hv, lam));
        if (!equator)
            *reinterpret_cast<float4 *>(mp + sS + 4 * q) =
                make_float4(epi(v0.y, kind, hv, lam), epi(v1.y, kind, hv, lam), epi(v2.y, kind, hv, lam),
                            epi(v3.y, kind, hv, lam));
    }
}

// Bluestein transform of ring pair p, map `map`, in buffer Z (shared or
// global memory) with the padded twiddle table wh of its length M and the
// partial-sum scratch X (2 x blockDim).  Ends with the stores.
template <int MC = 0>  // compile-time transform length (0: the ring's, at run time)
__device__ __forceinline__ void blu_ring(const RingArgs &a, const Epi32 &e, int map, int p, c32 *Z, c32 *X,
                                         const c32 *wh, bool folded = false, const c32 *wp = nullptr) {
    const int n = a.nph[p], i4 = n / 4, T = blockDim.x;
    const int M = a.blu_M[i4];
    const float2 *w2n = a.tw32 + a.tw_ofs[i4];
    const float2 *chirp = a.chirp + a.chirp_ofs[i4];  // e^{i pi k^2 / n}
    const int rn = p, rs = a.nrings - 1 - p;
    const bool equator = rn == rs;
    const float2 *FN = a.Ft + ((int64_t)map * a.nrings + rn) * (a.mmax + 1);
    const float2 *FS = a.Ft + ((int64_t)map * a.nrings + rs) * (a.mmax + 1);
    if (!folded) fold(FN, FS, equator, n, a.mmax, a.half[p], w2n, chirp, Z, Z, n, X);
    if constexpr (MC > 0)  // the padding beyond n is zero: not written, not read
        dif_ct<-1, MC, MC, true, false>(Z, wh, n, wp);
    else
        fft_dif<-1, true>(Z, wh, M, n);
    const float2 *H = a.blu_H + a.blu_ofs[i4];
#pragma unroll 8
    for (int k = threadIdx.x; k < M; k += T) Z[zi(k)] = cmul(Z[zi(k)], ldg(H + k));  // 8 loads in flight
    __syncthreads();
    if constexpr (MC > 0)
        adj_ct<-1, MC, MC>(Z, wh, wp);
    else
        fft_dif_adjoint<-1, true>(Z, wh, M);
    float *mp = a.maps + (int64_t)map * a.npix;
    const int64_t sN = a.startN[p], sS = a.startS[p];
    const EpiMap em = epi_map(a, e, map);
    const int kind = em.kind;
    const float hv = em.hv, lam = em.lam;
    const float invM = 1.0f / (float)M;
#pragma unroll 1
    for (int q = threadIdx.x; q < (n >> 2); q += T) {  // four pixels per thread, 16-byte stores
        const float4 ca = __ldg(reinterpret_cast<const float4 *>(chirp + 4 * q));
        const float4 cb = __ldg(reinterpret_cast<const float4 *>(chirp + 4 * q) + 1);
        const c32 v0 = cscale(cmul(Z[zi(4 * q)], c32{ca.x, ca.y}), invM);
        const c32 v1 = cscale(cmul(Z[zi(4 * q + 1)], c32{ca.z, ca.w}), invM);
        const c32 v2 = cscale(cmul(Z[zi(4 * q + 2)], c32{cb.x, cb.y}), invM);
        const c32 v3 = cscale(cmul(Z[zi(4 * q + 3)], c32{cb.z, cb.w}), invM);
        if (kind == GLG_EPI_LOGNORMAL) {
            refine_note(e, em.thr, map, v0.x, rn, 4 * q);
            refine_note(e, em.thr, map, v1.x, rn, 4 * q + 1);
            refine_note(e, em.thr, map, v2.x, rn, 4 * q + 2);
            refine_note(e, em.thr, map, v3.x, rn, 4 * q + 3);
            if (!equator) {
                refine_note(e, em.thr, map, v0.y, rs, 4 * q);
                refine_note(e, em.thr, map, v1.y, rs, 4 * q + 1);
                refine_note(e, em.thr, map, v2.y, rs, 4 * q + 2);
                refine_note(e, em.thr, map, v3.y, rs, 4 * q + 3);
            }
        }
        *reinterpret_cast<float4 *>(mp + sN + 4 * q) =
            make_float4(epi(v0.x, kind, hv, lam), epi(v1.x, kind, hv, lam), epi(v2.x, kind, hv, lam),
                        epi(v3.x, kind, hv, lam));
        if (!equator)
            *reinterpret_cast<float4 *>(mp + sS + 4 * q) =
                make_float4(epi(v0.y, kind, hv, lam), epi(v1.y, kind, hv, lam), epi(v2.y, kind, hv, lam),
                            epi(v3.y, kind, hv, lam));
    }
}

// The Bluestein fold of blu_ring (chirp included) from rows staged in
// shared memory (stN, stS: element m of the north / south row; they occupy
// the raw bytes of Z): every staged value is read into registers before Z
// is written.  n >= blockDim.x.  NI, NK: register slots of the one-term
// residue pairs (n > mmax) and of the signed multi-term fold (n <= mmax).
template <int NI, int NK>
__device__ __forceinline__ void fold_staged(const float2 *stN, const float2 *stS, bool equator, int n, int mmax,
                                            int h, const float2 *w2n, const float2 *chirp, c32 *Z) {
    const int T = blockDim.x, t = threadIdx.x;
    const c32 one = {1.f, 0.f}, zero = {0.f, 0.f};
    auto ld = [](const float2 *q, int m) -> c32 { return {q[m].x, q[m].y}; };
    if (n > mmax) {  // at most one term per residue: pairs (k, n - k) from the same two values
        c32 z1[NI], z2[NI];
#pragma unroll
        for (int i = 0; i < NI; ++i) {
            const int k = t + i * T;
            z1[i] = z2[i] = zero;
            if (k <= (n >> 1)) {
                const int k2 = k ? n - k : 0;
                const float ck = k ? 1.f : 0.5f;
                c32 fn = zero, fs = zero, gn = zero, gs = zero;
                if (k <= mmax) {
                    fn = ld(stN, k);
                    if (!equator) fs = ld(stS, k);
                }
                if (k2 <= mmax) {
                    gn = ld(stN, k2);
                    if (!equator) gs = ld(stS, k2);
                }
                const c32 wk = h ? ldg(w2n + k) : one, wk2 = h ? ldg(w2n + k2) : one;
                const c32 an = cscale(fn, ck), as = cscale(fs, ck), bn = cscale(gn, ck), bs = cscale(gs, ck);
                const c32 BN = cadd(cmul(wk, an), cconj(cmul(wk2, bn)));
                const c32 BS = cadd(cmul(wk, as), cconj(cmul(wk2, bs)));
                z1[i] = cmul(pack(BN, BS), ldg(chirp + k));
                if (k2 != k)
                    z2[i] = cmul(pack(cadd(cmul(wk2, gn), cconj(cmul(wk, fn))), cadd(cmul(wk2, gs), cconj(cmul(wk, fs)))),
                                 ldg(chirp + k2));
            }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < NI; ++i) {
            const int k = t + i * T;
            if (k <= (n >> 1)) {
                Z[zi(k)] = z1[i];
                if (k && 2 * k != n) Z[zi(n - k)] = z2[i];
            }
        }
        __syncthreads();
        return;
    }
    // signed fold S_k, one thread per residue (the order of fold's sums)
    const float sgn = h ? -1.f : 1.f;
    c32 sn[NK], ss[NK];
#pragma unroll
    for (int i = 0; i < NK; ++i) {
        const int k = t + i * T;
        sn[i] = ss[i] = zero;
        if (k < n) {
            float s = 1.f;
            for (int m = k; m <= mmax; m += n, s *= sgn) {
                const float c = m ? s : 0.5f * s;
                const c32 fn = ld(stN, m), fs = ld(equator ? stN : stS, m);
                sn[i] = {fmaf(c, fn.x, sn[i].x), fmaf(c, fn.y, sn[i].y)};
                ss[i] = {fmaf(c, fs.x, ss[i].x), fmaf(c, fs.y, ss[i].y)};
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NK; ++i) {
        const int k = t + i * T;
        if (k < n) {
            Z[zi(k)] = sn[i];
            Z[zi(n + k)] = ss[i];
        }
    }
    __syncthreads();
    // combine the residue pair (k, n - k), as fold does
    for (int k = t; k <= (n >> 1); k += T) {
        const int k2 = k ? n - k : 0;
        const c32 an = Z[zi(k)], bn = Z[zi(k2)];
        c32 as = Z[zi(n + k)], bs = Z[zi(n + k2)];
        if (equator) as = bs = zero;
        const c32 wk = h ? ldg(w2n + k) : one, wk2 = h ? ldg(w2n + k2) : one;
        const c32 pa = cmul(wk, an), pb = cmul(wk2, bn), qa = cmul(wk, as), qb = cmul(wk2, bs);
        const c32 z = cmul(pack(cadd(pa, cconj(pb)), cadd(qa, cconj(qb))), ldg(chirp + k));
        Z[zi(k)] = z;
        if (k2 != k) Z[zi(k2)] = cmul(pack(cadd(pb, cconj(pa)), cadd(qb, cconj(qa))), ldg(chirp + k2));
    }
    __syncthreads();
}

// Class 1 for M = 2^13, 2^14 with staged inputs (as k_ring32eq): the ring
// pair's rows of Legendre sums and the padded half twiddle table of M
// bulk-copied into shared memory on one mbarrier, then the fold from shared
// memory and blu_ring's transforms.  smem: Z[zsize(M)] | wh[zsize(M/2+1)].
template <int M, int T>
__global__ void __launch_bounds__(T, T <= 512 ? 2 : 1) k_ring32_blus(const RingArgs a, const Epi32 e) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NZ = ZSize<M>::value, NW = ZSize<M / 2 + 1>::value;
    constexpr int NI = (M / 4 + 1 + T - 1) / T, NK = (M / 2 + T - 1) / T;
    constexpr uint32_t BW = (uint32_t)(((NW * 8) + 15) & ~15);
    __shared__ __align__(8) uint64_t bar;
    const int map = blockIdx.x % a.nmaps;
    const int p = a.pairs[blockIdx.x / a.nmaps];
    const int rn = p, rs = a.nrings - 1 - p;
    const bool equator = rn == rs;
    const int mm = a.mmax + 1, n = a.nph[p], i4 = n / 4;
    c32 *Z = reinterpret_cast<c32 *>(smem_raw);
    c32 *wh = Z + ((NZ + 1) & ~1);
    c32 *wp = wh + ((NW + 1) & ~1);  // per-pass twiddle tables
    const float2 *FN = a.Ft + ((int64_t)map * a.nrings + rn) * mm;
    const float2 *FS = a.Ft + ((int64_t)map * a.nrings + rs) * mm;
    const int oN = (int)((reinterpret_cast<uintptr_t>(FN) >> 3) & 1);
    const int oS = (int)((reinterpret_cast<uintptr_t>(FS) >> 3) & 1);
    const uint32_t bN = (uint32_t)(((oN + mm) * 8 + 15) & ~15);
    const uint32_t bS = equator ? 0u : (uint32_t)(((oS + mm) * 8 + 15) & ~15);
    if (threadIdx.x == 0) {
        glg_tc::mbar_init(&bar, 1);
        glg_tc::fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        glg_tc::mbar_arrive_expect_tx(&bar, bN + bS + BW);
        glg_tc::bulk_g2s(smem_raw, FN - oN, bN, &bar);
        if (!equator) glg_tc::bulk_g2s(smem_raw + bN, FS - oS, bS, &bar);
        glg_tc::bulk_g2s(wh, a.twp + twp_offset(a, M), BW, &bar);
    }
    if (!glg_tc::mbar_wait(&bar, 0, STAGE_WAIT_LIMIT)) {
        if (threadIdx.x == 0 && a.err) atomicExch(a.err, GLG_ERR_TIMEOUT);
        glg_tc::mbar_wait(&bar, 0, STAGE_WAIT_LIMIT);  // the copies in flight land before the block exits
        return;
    }
    wtab_fill_rec<M, M>(wp, wh);  // published by the fold's barriers
    fold_staged<NI, NK>(reinterpret_cast<const float2 *>(smem_raw) + oN,
                        reinterpret_cast<const float2 *>(smem_raw + bN) + oS, equator, n, a.mmax, a.half[p],
                        a.tw32 + a.tw_ofs[i4], a.chirp + a.chirp_ofs[i4], Z);
    blu_ring<M>(a, e, map, p, Z, nullptr, wh, true, wp);
}

// Class 1: Bluestein.  smem: Z[M] (the south fold scratch sits at n..2n-1) |
// X[2T] | wh[zi(M/2) + 1].
template <int LOGM>
__global__ void __launch_bounds__(TMAX_POW2) k_ring32_blu(const RingArgs a, const Epi32 e) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int map = blockIdx.x % a.nmaps;
    const int p = a.pairs[blockIdx.x / a.nmaps];
    const int M = a.blu_M[a.nph[p] / 4], T = blockDim.x;
    c32 *Z = reinterpret_cast<c32 *>(smem_raw);
    c32 *X = Z + glg_zsize(M);
    c32 *wh = X + 2 * T;
    const int stride = a.Mmax / M;
    for (int t = threadIdx.x; t <= M / 2; t += T) wh[zi(t)] = ldg(a.twM + (int64_t)t * stride);
    blu_ring<(1 << LOGM)>(a, e, map, p, Z, X, wh);
}

// Class 3: Bluestein lengths too large for shared memory (M = 32768, the
// polar rings of nside 4096 with a large prime factor): the same transform
// with Z in a global slice per block of a persistent grid (the slices of
// the blocks in flight, 2 per SM x 275 KB, stay in L2) and the padded
// twiddles of M = Mmax from a global table; only X is in shared memory.
__global__ void __launch_bounds__(TMAX_POW2) k_ring32_blug(const RingArgs a, const Epi32 e, int nitems) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    c32 *X = reinterpret_cast<c32 *>(smem_raw);
    c32 *Z = reinterpret_cast<c32 *>(a.gz) + (int64_t)blockIdx.x * glg_zsize(a.Mmax);
    const c32 *wh = reinterpret_cast<const c32 *>(a.twMp);
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        blu_ring<0>(a, e, item % a.nmaps, a.pairs[item / a.nmaps], Z, X, wh);
        __syncthreads();  // the buffer is reused by the block's next item
    }
}

// F[map][m][ring] -> Ft[map][ring][m] for rings rb .. re-1, 32 x 32 tiles.
__global__ void k_transpose32(const float2 *__restrict__ F, float2 *__restrict__ Ft, int nm, int nr, int rb,
                              int re) {
    __shared__ float2 tile[32][33];
    const int map = blockIdx.z;
    const int r0 = rb + blockIdx.x * 32, m0 = blockIdx.y * 32;
    const float2 *src = F + (int64_t)map * nm * nr;
    float2 *dst = Ft + (int64_t)map * nm * nr;
    float2 v[4];  // blockDim.y == 8: four loads in flight per thread
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int y = threadIdx.y + 8 * i, m = m0 + y, r = r0 + threadIdx.x;
        v[i] = (m < nm && r < re) ? src[(int64_t)m * nr + r] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) tile[threadIdx.y + 8 * i][threadIdx.x] = v[i];
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, m = m0 + threadIdx.x;
        if (m < nm && r < re) dst[(int64_t)r * nm + m] = tile[threadIdx.x][y];
    }
}

struct RefineArgs {
    int nrings, npairs, mmax;
    int64_t npix;
    const int *nph, *half;
    const int64_t *startN, *startS;
    const float2 *Ft;  // [map][ring][m]
    float *maps;
    const int *hdr;    // [0] entries appended, [1] entries already refined
    int cap;
    const int4 *items;  // (map, ring, pixel within the ring, -)
    double hv[EPI_MAX], lam[EPI_MAX];
    const glg_epi_dev *edev;  // when set: hv, lam from device memory
};

// Float-float ("double-single") arithmetic: a value hi + lo with |lo| <=
// half an ulp of hi, about 48 significant bits, from FP32 operations only
// (error-free sums and FMA products, Dekker 1971 / Knuth TAOCP 4.2.2): on
// this GPU the FP32 pipe issues some 64 times the FP64 one.  The _rn
// intrinsics keep the compiler from fusing a product into a sum, which
// would break the error-free transformations.
struct f2f {
    float hi, lo;
};
__device__ __forceinline__ f2f ff_of(double d) {
    const float h = (float)d;
    return {h, (float)(d - (double)h)};
}
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// x * c - y * d + f (c, d float-float, f an exact float)
__device__ __forceinline__ f2f ff_rot(f2f x, f2f c, f2f y, f2f d, float f) {
    const float p1 = __fmul_rn(x.hi, c.hi), e1 = fmaf(x.hi, c.hi, -p1);
    const float p2 = __fmul_rn(-y.hi, d.hi), e2 = fmaf(-y.hi, d.hi, -p2);
    float s1, t1, s2, t2;
    two_sum(p1, p2, s1, t1);
    two_sum(s1, f, s2, t2);
    float lo = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(t1, t2));
    lo = fmaf(x.hi, c.lo, lo);
    lo = fmaf(x.lo, c.hi, lo);
    lo = fmaf(-y.hi, d.lo, lo);
    lo = fmaf(-y.lo, d.hi, lo);
    const float hi = __fadd_rn(s2, lo);
    return {hi, __fsub_rn(lo, __fsub_rn(hi, s2))};
}

// One warp per listed pixel: g = F_0 + 2 Re sum_{m>0} F_m e^{i m phi} from
// the FP32 Legendre sums of its ring (lane L takes m = L + 32 j, summed by
// Horner in z^32 from the top, then times z^L; angles reduced exactly as
// integer multiples of pi / nph) in float-float arithmetic, a fixed-order
// FP64 warp sum, and the lognormal value in FP64 stored over the FP32 one.
// Lane 0 evaluates z^32 (its own z^L is 1) and hands it to the warp.
__global__ void __launch_bounds__(256) k_refine(const RefineArgs r) {
    const int lane = threadIdx.x & 31;
    const int n0 = r.hdr[1];
    const int n1 = r.hdr[0] < r.cap ? r.hdr[0] : r.cap;
    for (int it = n0 + blockIdx.x * 8 + (threadIdx.x >> 5); it < n1; it += gridDim.x * 8) {
        const int4 e = r.items[it];
        const int map = e.x, ring = e.y, k = e.z;
        const int p = ring < r.npairs ? ring : r.nrings - 1 - ring;
        const int64_t nph = r.nph[p], a1 = 2LL * k + r.half[p];  // phi = pi a1 / nph
        const float2 *F = r.Ft + ((int64_t)map * r.nrings + ring) * (r.mmax + 1);
        double c, sn;
        sincospi((double)(((lane ? lane : 32) * a1) % (2 * nph)) / (double)nph, &sn, &c);
        const double zc64 = __shfl_sync(0xffffffffu, c, 0), zs64 = __shfl_sync(0xffffffffu, sn, 0);
        const double lc = lane ? c : 1.0, ls = lane ? sn : 0.0;  // z^L
        const f2f zc = ff_of(zc64), zs = ff_of(zs64);
        f2f sr = {0.f, 0.f}, si = {0.f, 0.f};
        const int jt = (r.mmax - lane) >= 0 ? (r.mmax - lane) / 32 : -1;
        for (int j = jt; j >= 0; --j) {
            const int m = lane + 32 * j;
            const float2 f = F[m];
            const float cm = m ? 2.f : 1.f;  // exact scalings
            const f2f tr = ff_rot(sr, zc, si, zs, cm * f.x);
            si = ff_rot(sr, zs, si, {-zc.hi, -zc.lo}, cm * f.y);  // sr zs + si zc + cm f.y
            sr = tr;
        }
        double v = ((double)sr.hi + (double)sr.lo) * lc - ((double)si.hi + (double)si.lo) * ls;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) {
            const int64_t start = ring < r.npairs ? r.startN[p] : r.startS[p];
            const double hv = r.edev ? r.edev->hv64[map] : r.hv[map];
            const double lam = r.edev ? r.edev->lam64[map] : r.lam[map];
            r.maps[(int64_t)map * r.npix + start + k] = (float)(lam * expm1(v - hv));
        }
    }
}

__global__ void k_refine_done(int *hdr, int cap) { hdr[1] = hdr[0] < cap ? hdr[0] : cap; }

}  // namespace

static void ring_args(const glg_plan *P, const float2 *Ft, int nmaps, float *maps, RingArgs &a) {
    a.nrings = P->nrings;
    a.mmax = P->mmax;
    a.nmaps = nmaps;
    a.nph = P->nph;
    a.half = P->half;
    a.startN = P->startN;
    a.startS = P->startS;
    a.tw_ofs = P->tw_ofs;
    a.tw32 = P->tw32;
    a.pos_ofs = P->pos_ofs;
    a.pos16 = P->pos16;
    a.blu_ofs = P->blu_ofs;
    a.chirp_ofs = P->chirp_ofs;
    a.blu_M = P->blu_M;
    a.blu_H = P->blu_H;
    a.chirp = P->chirp;
    a.twM = P->twM;
    a.Mmax = P->blu_Mmax;
    a.twMp = P->twMp;
    a.gz = nullptr;
    a.Ft = Ft;
    a.maps = maps;
    a.npix = P->npix;
    a.twp = P->twp;
    for (int k = 0; k < 16; ++k) {
        a.twp_ofs[k] = P->twp_ofs[k];
        a.twp3_ofs[k] = P->twp3_ofs[k];
    }
    a.err = nullptr;
    a.edev = nullptr;
}

typedef void (*RingKernel)(const RingArgs, const Epi32);
// Bluestein kernels by log2 M (3 .. 14) and equatorial kernels by log2 n (2 .. 14).
static const RingKernel kBlu[15] = {nullptr,           nullptr,           nullptr,           k_ring32_blu<3>,
                                    k_ring32_blu<4>,   k_ring32_blu<5>,   k_ring32_blu<6>,   k_ring32_blu<7>,
                                    k_ring32_blu<8>,   k_ring32_blu<9>,   k_ring32_blu<10>,  k_ring32_blu<11>,
                                    k_ring32_blu<12>,  k_ring32_blu<13>,  k_ring32_blu<14>};
static const RingKernel kEq[15] = {nullptr,            nullptr,            k_ring32<true, 2>,  k_ring32<true, 3>,
                                   k_ring32<true, 4>,  k_ring32<true, 5>,  k_ring32<true, 6>,  k_ring32<true, 7>,
                                   k_ring32<true, 8>,  k_ring32<true, 9>,  k_ring32<true, 10>, k_ring32<true, 11>,
                                   k_ring32<true, 12>, k_ring32<true, 13>, k_ring32<true, 14>};

// Staged equatorial kernels by log2 n (10 .. 14): 512 threads, 1024 at 2^14.
static const RingKernel kEqStaged[15] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                         nullptr, nullptr, k_ring32eq<10, 512>, k_ring32eq<11, 512>,
                                         k_ring32eq<12, 512>, k_ring32eq<13, 512>, k_ring32eq<14, 1024>};
static size_t eq_staged_smem(int n) {
    return sizeof(float2) *
           (size_t)(((glg_zsize(n) + 1) & ~1) + ((glg_zsize(n / 2 + 1) + 1) & ~1) + wtab_total_host(n) + 2);
}
// The staged kernel takes a power-of-two bucket of 2^10 .. 2^14 when n > mmax
// and the two staged rows fit the transform buffer.
static bool staged_eq_ok(const glg_plan *P, const glg_ring_bucket &B) {
    const int n = B.size, lg = __builtin_ctz((unsigned)n);
    if (n != (1 << lg) || lg < 10 || lg > 14 || n <= P->mmax || !P->twp || P->twp_ofs[lg] < 0) return false;
    const size_t rows = 2 * (((size_t)(P->mmax + 2) * 8 + 15) & ~(size_t)15);
    return rows <= sizeof(float2) * (size_t)glg_zsize(n) && eq_staged_smem(n) <= 227 * 1024;
}

// The staged Bluestein kernels take M = 6144, 8192 (512 threads), 12288, 16384 (1024)
// when the two staged rows fit the transform buffer and every ring of the
// bucket has at least as many pixels as the block has threads.
static bool staged_blu_ok(const glg_plan *P, const glg_ring_bucket &B, int count) {
    const int M = B.size;
    if ((M != 6144 && M != 8192 && M != 12288 && M != 16384) || !P->twp || count <= 0) return false;
    if ((M % 3 == 0 ? P->twp3_ofs[__builtin_ctz((unsigned)(M / 3))] : P->twp_ofs[__builtin_ctz((unsigned)M)]) < 0)
        return false;
    const int T = M >= 12288 ? 1024 : 512;
    const int *bp = P->bucket_pairs_host + B.first;
    for (int i = 0; i < B.count; ++i) {
        const int p = bp[i];
        const int ring = p + 1 < P->nside ? p + 1 : P->nside;  // north ring p + 1 has 4 min(p + 1, nside) pixels
        if (4 * ring < T) return false;
    }
    const size_t rows = 2 * (((size_t)(P->mmax + 2) * 8 + 15) & ~(size_t)15);
    return rows <= sizeof(float2) * (size_t)glg_zsize(M) && eq_staged_smem(M) <= 227 * 1024;
}

// Pairs lo .. lo+count-1 of bucket B (the whole bucket by default).
static int launch_bucket(const glg_plan *P, const glg_ring_bucket &B, int threads, RingArgs a, const Epi32 &e,
                         cudaStream_t st, int lo = 0, int count = -1) {
    if (count < 0) count = B.count;
    if (count == 0) return GLG_OK;
    a.pairs = P->bucket_pairs + B.first + lo;
    const size_t smem = glg_ring32_smem(B.kind, B.size, threads, B.fold != 0);
    const unsigned grid = (unsigned)count * (unsigned)a.nmaps;
    if (B.kind == 3) {
        if (!a.gz || B.size != P->blu_Mmax) {
            glg_set_error("fast ring FFT: no global transform buffers for the largest Bluestein length");
            return GLG_ERR_UNSUPPORTED;
        }
        const unsigned g3 = grid < GLG_RING_GSLOTS ? grid : GLG_RING_GSLOTS;
        cudaFuncSetAttribute(k_ring32_blug, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        GLG_LAUNCH_SCOPE("k_ring32_blug", st);
        k_ring32_blug<<<g3, threads, smem, st>>>(a, e, (int)grid);
        GLG_CHECK_LAUNCH("k_ring32_blug");
    } else if (B.kind == 1 && staged_blu_ok(P, B, count)) {
        RingKernel kern;
        int T;
        switch (B.size) {
            case 16384: kern = k_ring32_blus<16384, 1024>; T = 1024; break;
            case 12288: kern = k_ring32_blus<12288, 1024>; T = 1024; break;
            case 8192: kern = k_ring32_blus<8192, 512>; T = 512; break;
            default: kern = k_ring32_blus<6144, 512>; T = 512; break;
        }
        const size_t sm = eq_staged_smem(B.size);
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        GLG_LAUNCH_SCOPE("k_ring32_blu", st);
        kern<<<grid, T, sm, st>>>(a, e);
        GLG_CHECK_LAUNCH("k_ring32_blu");
    } else if (B.kind == 1) {
        const int lg = __builtin_ctz((unsigned)B.size);
        if (B.size != (1 << lg) || lg < 3 || lg > 14) {
            glg_set_error("fast ring FFT: Bluestein length outside 2^3 .. 2^14");
            return GLG_ERR_UNSUPPORTED;
        }
        const RingKernel kern = kBlu[lg];
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        GLG_LAUNCH_SCOPE("k_ring32_blu", st);
        kern<<<grid, threads, smem, st>>>(a, e);
        GLG_CHECK_LAUNCH("k_ring32_blu");
    } else if (B.kind == 2 && staged_eq_ok(P, B)) {
        const int lg = __builtin_ctz((unsigned)B.size);
        const int T = lg >= 14 ? 1024 : 512;
        const RingKernel kern = kEqStaged[lg];
        const size_t sm = eq_staged_smem(B.size);
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        GLG_LAUNCH_SCOPE("k_ring32", st);
        kern<<<grid, T, sm, st>>>(a, e);
        GLG_CHECK_LAUNCH("k_ring32");
    } else if (B.kind == 2) {
        const int lg = __builtin_ctz((unsigned)B.size);
        const RingKernel kern = (B.size == (1 << lg) && lg >= 2 && lg <= 14) ? kEq[lg] : k_ring32<true, 0>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        GLG_LAUNCH_SCOPE("k_ring32", st);
        kern<<<grid, threads, smem, st>>>(a, e);
        GLG_CHECK_LAUNCH("k_ring32");
    } else {
        cudaFuncSetAttribute(k_ring32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        GLG_LAUNCH_SCOPE("k_ring32", st);
        k_ring32<false><<<grid, threads, smem, st>>>(a, e);
        GLG_CHECK_LAUNCH("k_ring32");
    }
    return GLG_OK;
}

static int launch_transpose(const float2 *F, float2 *Ft, int nm, int nr, int rb, int re, int nmaps,
                            cudaStream_t st) {
    if (re <= rb) return GLG_OK;
    dim3 grid((re - rb + 31) / 32, (nm + 31) / 32, nmaps);
    GLG_LAUNCH_SCOPE("k_transpose32", st);
    k_transpose32<<<grid, dim3(32, 8), 0, st>>>(F, Ft, nm, nr, rb, re);
    GLG_CHECK_LAUNCH("k_transpose32");
    return GLG_OK;
}

int glg_launch_ring_syn_f32(const glg_plan *P, const float2 *F, float2 *Ft, int nmaps, float *maps,
                            const glg_epilogue *epi_in, const glg_refine_list *rl, cudaStream_t st) {
    return glg_launch_ring_syn_f32_range(P, F, Ft, nmaps, maps, epi_in, 0, P->npairs, rl, st);
}

// Lognormal threshold of the tail refinement of map k (+inf: none).
static float refine_threshold(const glg_epilogue *epi, int k, int kind) {
    if (kind != GLG_EPI_LOGNORMAL || !epi || !epi->var || epi->var[k] < REFINE_MIN_VAR) return INFINITY;
    const double v = epi->var[k];
    return (float)(0.5 * v + log1p(sqrt(REFINE_KAPPA * expm1(v))));
}

bool glg_refine_wanted(const glg_epilogue *epi, int nmaps) {
    for (int k = 0; k < nmaps && epi; ++k) {
        const int kind = epi->kinds ? epi->kinds[k] : epi->kind;
        if (refine_threshold(epi, k, kind) < INFINITY) return true;
    }
    return false;
}

void glg_epi_dev_fill(const glg_epilogue *epi, int nmaps, glg_epi_dev *out) {
    for (int k = 0; k < GLG_EPI_MAPS; ++k) {
        const bool on = epi && k < nmaps;
        const int kind = !on ? GLG_EPI_NONE : (epi->kinds ? epi->kinds[k] : epi->kind);
        const double var = (on && epi->var) ? epi->var[k] : 0.0;
        const double lam = (on && epi->lamda) ? epi->lamda[k] : 1.0;
        out->kind[k] = kind;
        out->hvar[k] = (float)(0.5 * var);
        out->lam[k] = (float)lam;
        out->thr[k] = on ? refine_threshold(epi, k, kind) : INFINITY;
        out->hv64[k] = 0.5 * var;
        out->lam64[k] = lam;
    }
}

int glg_launch_refine(const glg_plan *P, const float2 *Ft, int nmaps, float *maps, const glg_epilogue *epi,
                      const glg_refine_list &rl, cudaStream_t st) {
    // a device epilogue is read at run time: the (possibly empty) list is always processed
    if (!rl.edev && !glg_refine_wanted(epi, nmaps)) return GLG_OK;
    RefineArgs r;
    r.nrings = P->nrings;
    r.npairs = P->npairs;
    r.mmax = P->mmax;
    r.npix = P->npix;
    r.nph = P->nph;
    r.half = P->half;
    r.startN = P->startN;
    r.startS = P->startS;
    r.Ft = Ft;
    r.maps = maps;
    r.hdr = rl.hdr;
    r.cap = rl.cap;
    r.items = rl.items;
    for (int k = 0; k < EPI_MAX; ++k) {
        r.hv[k] = epi && k < nmaps && epi->var ? 0.5 * epi->var[k] : 0.0;
        r.lam[k] = epi && k < nmaps && epi->lamda ? epi->lamda[k] : 1.0;
    }
    r.edev = rl.edev;
    {
        GLG_LAUNCH_SCOPE("k_refine", st);
        k_refine<<<608, 256, 0, st>>>(r);
        GLG_CHECK_LAUNCH("k_refine");
    }
    k_refine_done<<<1, 1, 0, st>>>(rl.hdr, rl.cap);
    GLG_CHECK_LAUNCH("k_refine_done");
    return GLG_OK;
}

int glg_launch_ring_syn_f32_range(const glg_plan *P, const float2 *F, float2 *Ft, int nmaps, float *maps,
                                  const glg_epilogue *epi_in, int p0, int p1, const glg_refine_list *rl,
                                  cudaStream_t st) {
    if (nmaps > EPI_MAX) {
        glg_set_error("fast ring FFT: at most 40 maps per call");
        return GLG_ERR_UNSUPPORTED;
    }
    if (p0 < 0 || p1 > P->npairs || p0 >= p1) {
        glg_set_error("fast ring FFT: empty or out-of-range ring-pair range");
        return GLG_ERR_INVALID;
    }
    const int nm = P->mmax + 1, nr = P->nrings;
    for (int b = 0; b < P->nbuckets; ++b)
        if (P->buckets[b].smem > 227 * 1024) {
            glg_set_error("fast ring FFT: ring length too large for shared memory (nside <= 4096)");
            return GLG_ERR_UNSUPPORTED;
        }
    // north rings p0 .. p1-1 and their south partners nr-p1 .. nr-1-p0 (the
    // equator ring, pair npairs-1, is its own partner)
    if (F) {
        int rc = launch_transpose(F, Ft, nm, nr, p0, p1, nmaps, st);
        if (!rc) rc = launch_transpose(F, Ft, nm, nr, nr - p1 > p1 ? nr - p1 : p1, nr - p0, nmaps, st);
        if (rc) return rc;
    }
    RingArgs a;
    ring_args(P, Ft, nmaps, maps, a);
    Epi32 e;
    for (int k = 0; k < EPI_MAX; ++k) {
        const bool on = epi_in && k < nmaps;
        e.kind[k] = !on ? GLG_EPI_NONE : (epi_in->kinds ? epi_in->kinds[k] : epi_in->kind);
        e.hvar[k] = (on && epi_in->var) ? (float)(0.5 * epi_in->var[k]) : 0.f;
        e.lam[k] = (on && epi_in->lamda) ? (float)epi_in->lamda[k] : 1.f;
        e.thr[k] = (on && rl) ? refine_threshold(epi_in, k, e.kind[k]) : INFINITY;
    }
    e.rcount = rl ? rl->hdr : nullptr;
    e.rcap = rl ? rl->cap : 0;
    e.ritems = rl ? rl->items : nullptr;
    a.gz = rl ? rl->gz : nullptr;
    a.err = rl ? rl->err : nullptr;
    a.edev = rl ? rl->edev : nullptr;
    const bool whole = p0 == 0 && p1 == P->npairs;
    for (int b = 0; b < P->nbuckets; ++b) {
        const glg_ring_bucket &B = P->buckets[b];
        int lo = 0, hi = B.count;
        if (!whole) {  // a bucket's pairs ascend: the range is one slice of them
            const int *bp = P->bucket_pairs_host + B.first;
            lo = (int)(std::lower_bound(bp, bp + B.count, p0) - bp);
            hi = (int)(std::lower_bound(bp, bp + B.count, p1) - bp);
        }
        const int rc = launch_bucket(P, B, B.threads, a, e, st, lo, hi - lo);
        if (rc) return rc;
    }
    return GLG_OK;
}

size_t glg_ring_gz_bytes(int nside) {
    if (nside <= 2048) return 0;
    int M = 1;
    while (M < 8 * nside - 1) M <<= 1;
    return sizeof(float2) * (size_t)GLG_RING_GSLOTS * glg_zsize(M);
}

int glg_launch_ring_bucket_f32(const glg_plan *P, int bucket, int threads, const float2 *Ft, int nmaps,
                               float *maps, float2 *gz, cudaStream_t st) {
    const glg_ring_bucket &B = P->buckets[bucket];
    if (glg_ring32_smem(B.kind, B.size, threads, B.fold != 0) > 227 * 1024) {
        glg_set_error("fast ring FFT: block size does not fit shared memory");
        return GLG_ERR_UNSUPPORTED;
    }
    RingArgs a;
    ring_args(P, Ft, nmaps, maps, a);
    a.gz = gz;
    Epi32 e;
    for (int k = 0; k < EPI_MAX; ++k) {
        e.kind[k] = GLG_EPI_NONE;
        e.hvar[k] = 0.f;
        e.lam[k] = 1.f;
        e.thr[k] = INFINITY;
    }
    e.rcount = nullptr;
    e.rcap = 0;
    e.ritems = nullptr;
    return launch_bucket(P, B, threads, a, e, st);
}
