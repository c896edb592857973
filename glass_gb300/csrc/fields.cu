// Field-generation kernels before the transform: iternorm, Philox normals,
// correlated alm assembly, multalm and almxfl.
#include <cuda_runtime.h>
#include <math.h>

#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "glg_internal.cuh"
#include "philox.cuh"

using glg_rng::U4;
using glg_rng::philox4x32_10;

namespace {

// ---------------------------------------------------------------- iternorm

// One warp per angular mode l (glass/fields.py:101-188).  The matrix m
// (k x k, double buffered), a and atm live in shared memory.  Every sum
// runs in the same fixed order, with explicit fma, as orc_iternorm in the
// CPU oracle, so both give identical bits.  After row i only the trailing
// z = min(i, k) rows and columns of m (and entries of a) can be non-zero, so
// the sums start at index k - z: the terms skipped are exact zeros.
__global__ void __launch_bounds__(32)
k_iternorm(const double *__restrict__ cov, const int64_t nrows, const int64_t nl, const int k,
           double *__restrict__ w, int64_t *__restrict__ bad) {
    extern __shared__ double sm[];
    const int64_t l = blockIdx.x;
    const int lane = threadIdx.x;
    const int kp = k + 1;
    const int kk = k > 0 ? k * k : 1;
    double *m = sm;
    double *mn = sm + kk;
    double *a = mn + kk;
    double *atm = a + (k > 0 ? k : 1);
    for (int t = lane; t < kk; t += 32) m[t] = 0.0;
    for (int t = lane; t < k; t += 32) a[t] = 0.0;
    double s = 1.0;
    __syncwarp();
    for (int64_t i = 0; i < nrows; ++i) {
        const double *row = cov + ((size_t)i * nl + l) * kp;
        const int z = i < k ? (int)i : k, zp = i - 1 < k ? (int)(i - 1) : k;
        const int lo = k - z, lop = k - (zp > 0 ? zp : 0);
        if (i > 0 && k > 0) {
            // lanes over the non-zero columns first (one pass while z <= 32)
            for (int j = lop + lane; j < k; j += 32) {
                double acc = 0.0;
                for (int q = lop; q < k; ++q) acc = fma(a[q], m[q * k + j], acc);
                atm[j] = acc;
            }
            for (int j = lane; j < lop; j += 32) atm[j] = 0.0;
            __syncwarp();
            const double u = s > 0 ? 1.0 : 0.0;
            const double sd = s > 0 ? s : 1.0;
            // only the new non-zero block [lo, k) x [lo, k) of m is written
            // (nothing reads outside it); its z x z entries are split into
            // (row, column) with an FP32 reciprocal, exact for z <= 127
            const float inv_z = 1.0f / (float)z;
            for (int t = lane; t < z * z; t += 32) {
                const int rr = (int)(((float)t + 0.5f) * inv_z);
                const int r = lo + rr, cc = lo + (t - rr * z);
                double v;
                if (r < k - 1)
                    v = (cc + 1 < k) ? m[(r + 1) * k + (cc + 1)] : 0.0;
                else
                    v = ((cc + 1 < k) ? -atm[cc + 1] : u) / sd;
                mn[r * k + cc] = v;
            }
            __syncwarp();
            double *tmp = m;
            m = mn;
            mn = tmp;
        }
        for (int r = lo + lane; r < k; r += 32) {
            double acc = 0.0;
            for (int cc = lo; cc < k; ++cc) acc = fma(m[r * k + cc], row[k - cc], acc);
            a[r] = acc;
        }
        for (int r = lane; r < lo; r += 32) a[r] = 0.0;
        __syncwarp();
        double sv = 0.0;
        if (lane == 0) {
            double aa = 0.0;
            for (int r = lo; r < k; ++r) aa = fma(a[r], a[r], aa);
            sv = row[0] - aa;
            if (sv < 0) {
                atomicMin((unsigned long long *)bad, (unsigned long long)i);
                sv = 0.0;
            }
            sv = sqrt(sv);
        }
        s = __shfl_sync(0xffffffffu, sv, 0);
        double *wo = w + ((size_t)i * nl + l) * kp;
        for (int r = lane; r < k; r += 32) wo[r] = a[r];
        if (lane == 0) wo[k] = s;
        __syncwarp();
    }
}

// ----------------------------------------------------------------- cls2cov

// cov[j][l][i] = C^{j,j-i}_l / 2 for i <= min(j, nc) and l < len(C^{j,j-i}),
// else 0 (glass/fields.py:191-236); spectra in GLASS order, concatenated in
// `flat` with offsets `offs` (spectrum q = offs[q] .. offs[q+1]-1).
__global__ void k_cls2cov(const double *__restrict__ flat, const int64_t *__restrict__ offs, int nf,
                          int nl, int nc, double *__restrict__ cov) {
    const int j = blockIdx.y;
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nl) return;
    double *row = cov + ((int64_t)j * nl + l) * (nc + 1);
    const int64_t base = (int64_t)j * (j + 1) / 2;
    for (int i = 0; i <= nc; ++i) {
        double v = 0.0;
        if (i <= j) {
            const int64_t o = offs[base + i], len = offs[base + i + 1] - o;
            if (l < len) v = flat[o + l] / 2;
        }
        row[i] = v;
    }
}

// var[j] = sum_l (2l+1)/(4 pi) C^{jj}_l (the variance transformcl.cltovar
// gives, glass/fields.py:890); *status = first field whose auto-spectrum has a
// negative value ("negative values in cl", glass/fields.py:229-231).
__global__ void k_cltovar(const double *__restrict__ flat, const int64_t *__restrict__ offs,
                          double *__restrict__ var, unsigned long long *__restrict__ status) {
    __shared__ double part[256];
    const int j = blockIdx.x;
    const int64_t q = (int64_t)j * (j + 1) / 2;
    const int64_t o = offs[q], len = offs[q + 1] - o;
    double s = 0.0;
    bool neg = false;
    for (int64_t l = threadIdx.x; l < len; l += blockDim.x) {
        const double c = flat[o + l];
        neg |= c < 0;
        s += (2.0 * l + 1.0) * c;
    }
    if (neg) atomicMin(status, (unsigned long long)j);
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) var[j] = part[0] / (4.0 * 3.14159265358979323846);
}

// ------------------------------------------------------------------ philox

// Complex standard normal: element e of stream sid (see orc_philox_normals).
__device__ __forceinline__ double2 philox_cnormal_f64(uint64_t seed, uint64_t sid, uint64_t e) {
    const U4 x = philox4x32_10((uint32_t)e, (uint32_t)(e >> 32), (uint32_t)sid,
                               (uint32_t)(sid >> 32), (uint32_t)seed, (uint32_t)(seed >> 32));
    const double u1 = ((double)(x.x >> 5) * 67108864.0 + (double)(x.y >> 6) + 0.5) * 1.1102230246251565e-16;
    const double u2 = ((double)(x.z >> 5) * 67108864.0 + (double)(x.w >> 6) + 0.5) * 1.1102230246251565e-16;
    const double r = sqrt(-2.0 * log(u1));
    double sn, cs;
    sincospi(2.0 * u2, &sn, &cs);
    return make_double2(r * cs, r * sn);
}

__device__ __forceinline__ float2 philox_cnormal_f32(uint64_t seed, uint64_t sid, uint64_t e) {
    const U4 x = philox4x32_10((uint32_t)e, (uint32_t)(e >> 32), (uint32_t)sid,
                               (uint32_t)(sid >> 32), (uint32_t)seed, (uint32_t)(seed >> 32));
    // The FP64 form's 53-bit uniforms u = (K + 1/2) 2^-53, K = a 2^26 + b, held
    // as an exact FP32 head h = (a >> 3) 2^-24 plus a small tail t, so that
    // the FP32 normals track the FP64 ones to about one FP32 ulp.
    const float s24 = 5.9604644775390625e-08f, s53 = 1.1102230246251565e-16f;
    const uint32_t a1 = x.x >> 5, b1 = x.y >> 6, a2 = x.z >> 5, b2 = x.w >> 6;
    const float h1 = (float)(a1 >> 3) * s24, t1 = ((float)((a1 & 7u) << 26 | b1) + 0.5f) * s53;
    const float h2 = (float)(a2 >> 3) * s24, t2 = ((float)((a2 & 7u) << 26 | b2) + 0.5f) * s53;
    // log(u1), without divergence: logf(A) + log1pf(P) + C with
    //   u1 >= 1/2: A = 1, P = -vh, C = -vt / (1 - vh)   (v = 1 - u1 = vh + vt
    //              from the complemented bits, so log(u1) = log1p(-v));
    //   0 < h1 < 1/2: A = h1, P = t1 / h1, C = 0       (log(h1) + log1p(t1 / h1));
    //   h1 = 0 (u1 < 2^-24): A = t1, P = C = 0.
    const bool up = h1 >= 0.5f;
    const uint32_t ca = 0x7FFFFFFu - a1, cb = 0x3FFFFFFu - b1;
    const float vh = (float)(ca >> 3) * s24, vt = ((float)((ca & 7u) << 26 | cb) + 0.5f) * s53;
    const float num = up ? -vt : t1, den = up ? 1.0f - vh : (h1 > 0.0f ? h1 : 1.0f);
    const float qd = num / den;
    const float A = up ? 1.0f : (h1 > 0.0f ? h1 : t1);
    const float P = up ? -vh : (h1 > 0.0f ? qd : 0.0f);
    const float C = up ? qd : 0.0f;
    const float lg = (logf(A) + log1pf(P)) + C;
    const float r = sqrtf(-2.0f * lg);
    float sn, cs;
    sincospif(2.0f * h2, &sn, &cs);
    const float dphi = 6.283185307179586f * t2;  // rotate by the tail of the angle
    return make_float2(r * (cs - sn * dphi), r * (sn + cs * dphi));
}

__global__ void k_philox_normals(uint64_t seed, uint64_t sid, int64_t offset, int64_t n, int dtype,
                                 void *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t e = (uint64_t)(offset + i);
        if (dtype == GLG_F64)
            reinterpret_cast<double2 *>(out)[i] = philox_cnormal_f64(seed, sid, e);
        else
            reinterpret_cast<float2 *>(out)[i] = philox_cnormal_f32(seed, sid, e);
    }
}

// ------------------------------------------------------- alm correlation

// Element (l, m) of shells t0..t0+nshell-1, written in HEALPix order.  A
// block covers a tile of 16 consecutive l by (blockDim / 16) consecutive m:
// the w rows of its 16 l values are staged in shared memory once per shell
// and shared by all m of the tile, and the 16 l of one m are 16 consecutive
// HEALPix indices, so stores stay coalesced.  Each thread keeps the window of
// variates z_{t-k..t} of its element in shared memory, so every variate is
// read or generated once per element.  The sum runs oldest variate first,
// like the reference's sum over the deque (glass/fields.py:420); the fast
// form (FP32) accumulates in FP32, the plain form in FP64.
constexpr int CT_L = 16;

template <typename T2, typename T>
__global__ void k_alm_correlate(const T *__restrict__ w, const int nshell, const int lmax,
                                const int k, const int64_t t0, const T2 *__restrict__ z,
                                const int64_t z_first, const uint64_t seed, const uint64_t sid_base,
                                T2 *__restrict__ alm, const int window) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    const int kp = k + 1;
    const int wst = kp | 1;  // odd row stride: the 16 l rows sit in distinct banks
    // q / kp as a multiply-high by ceil(2^32 / kp): exact for q < 17 kp, kp <= 127
    const uint32_t kmagic = kp > 1 ? (uint32_t)((0x100000000ull + (uint64_t)kp - 1) / (uint64_t)kp) : 0u;
    T *ws = reinterpret_cast<T *>(sm_raw);  // [CT_L][wst]
    const size_t ws_bytes = ((sizeof(T) * CT_L * wst) + 15) & ~(size_t)15;
    // variate window, slot-major ([slot][thread]) so a warp's accesses are contiguous
    T2 *zs = reinterpret_cast<T2 *>(sm_raw + ws_bytes) + threadIdx.x;
    const int B = blockDim.x;
    const int ctm = B / CT_L;
    const int l0 = blockIdx.x * CT_L, m0 = blockIdx.y * ctm;
    if (m0 > l0 + CT_L - 1 || m0 > lmax) return;  // tile entirely above m = l
    const int l = l0 + (int)(threadIdx.x % CT_L), m = m0 + (int)(threadIdx.x / CT_L);
    const bool valid = l <= lmax && m <= l;
    const int64_t nalm = glg_nalm(lmax);
    const int64_t g = (int64_t)l * (l + 1) / 2 + m;                // GLASS index
    const int64_t ix = (int64_t)m * (2 * lmax + 1 - m) / 2 + l;    // HEALPix index
    const int L = lmax + 1;
    const int64_t zlo = t0 - k > 0 ? t0 - k : 0;
    auto fetch = [&](int64_t t) -> T2 {
        if (z != nullptr) return z[(t - z_first) * nalm + g];
        if constexpr (sizeof(T) == 8) {
            return philox_cnormal_f64(seed, sid_base + (uint64_t)t, (uint64_t)g);
        } else {
            return philox_cnormal_f32(seed, sid_base + (uint64_t)t, (uint64_t)g);
        }
    };
    // shell t lives in slot t mod window; head = slot of the current shell
    int head = (int)(t0 % window);
    if (valid) {
        int slot = (int)(zlo % window);
        for (int64_t t = zlo; t < t0; ++t) {
            zs[slot * B] = fetch(t);
            if (++slot == window) slot = 0;
        }
    }
    for (int s = 0; s < nshell; ++s) {
        const int64_t t = t0 + s;
        __syncthreads();
        for (int q = threadIdx.x; q < CT_L * kp; q += B) {
            const int r = kp > 1 ? (int)__umulhi((uint32_t)q, kmagic) : q, c = q - r * kp;
            const int lg = l0 + r;
            ws[r * wst + c] = lg <= lmax ? w[((size_t)s * L + lg) * kp + c] : (T)0;
        }
        __syncthreads();
        if (valid) {
            zs[head * B] = fetch(t);
            T re = 0, im = 0;
            const int dmax = t < k ? (int)t : k;
            // the window z_{t-dmax} .. z_t, oldest first, in at most two
            // contiguous runs of slots (j0 .. window-1, then 0 .. head);
            // coefficient of slot j: w_t[k - dmax + (j - j0) mod window]
            int j0 = head - dmax;
            if (j0 < 0) j0 += window;
            const int run1 = j0 + dmax + 1 <= window ? dmax + 1 : window - j0;
            const T *wc = ws + (l - l0) * wst + (k - dmax) - j0;
            const T2 *zp = zs;
#pragma unroll 8
            for (int j = j0; j < j0 + run1; ++j) {
                const T2 zz = zp[j * B];
                const T c = wc[j];
                re += c * zz.x;
                im += c * zz.y;
            }
            wc += window;
#pragma unroll 4
            for (int j = 0; j < dmax + 1 - run1; ++j) {
                const T2 zz = zp[j * B];
                const T c = wc[j];
                re += c * zz.x;
                im += c * zz.y;
            }
            if (m == 0) {
                re = re + im;
                im = 0;
            }
            T2 o;
            o.x = re;
            o.y = im;
            alm[(int64_t)s * nalm + ix] = o;
        }
        if (++head == window) head = 0;
    }
}

// The fast form's window sum (glass/fields.py:401-425) with the variate
// window in registers: the same elements, sums and summation order as
// k_alm_correlate<float2, float>, for windows k + 1 <= WT <= 40.  One warp
// per l and 32 consecutive m (a block: 8 l x 32 m), so the warp's lanes
// share every w coefficient: per group of CR_SB shells the warp stages its
// l's w rows (loaded into registers one group ahead) into its own shared memory,
// right-aligned in rows of WT coefficients (slot j holds the coefficient of
// z_{t-(WT-1-j)}, zero where that variate is absent or older than the
// window: adding 0 * z leaves the running sum's bits unchanged), and each
// lane draws its CR_SB variates into its own column; the sum then reads the
// coefficients as 16-byte broadcasts.  No block-wide barrier.
// The window is a ring of WT registers and the shell loop is unrolled WT
// times, so every ring slot is a constant.
constexpr int CR_SB = 8, CR_WARPS = 8;

template <int WT>
__global__ void __launch_bounds__(32 * CR_WARPS, 2)
    k_alm_correlate_rw(const float *__restrict__ w, const int nshell, const int lmax, const int k, const int64_t t0,
                       const float2 *__restrict__ z, const int64_t z_first, const uint64_t seed,
                       const uint64_t sid_base, float2 *__restrict__ alm) {
    static_assert(WT % CR_SB == 0 && WT % 4 == 0 && WT <= 40, "window slots");
    __shared__ __align__(16) float wsm[CR_WARPS][CR_SB][WT];
    __shared__ __align__(16) float2 zsm[CR_WARPS][CR_SB][32];
    const int kp = k + 1;
    const int wi = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
    const int l = blockIdx.x * CR_WARPS + wi, m0 = blockIdx.y * 32;
    if (l > lmax || m0 > l) return;  // the warp's whole row lies outside m <= l <= lmax
    const int m = m0 + lane;
    const bool valid = m <= l;
    const int64_t nalm = glg_nalm(lmax);
    const int64_t g = (int64_t)l * (l + 1) / 2 + m;              // GLASS index
    const int64_t ix = (int64_t)m * (2 * lmax + 1 - m) / 2 + l;  // HEALPix index
    const int L = lmax + 1;
    const int64_t zlo = t0 - k > 0 ? t0 - k : 0;
    auto fetch = [&](int64_t t) -> float2 {
        if (z != nullptr) return z[(t - z_first) * nalm + g];
        return philox_cnormal_f32(seed, sid_base + (uint64_t)t, (uint64_t)g);
    };
    float2 *zc = &zsm[wi][0][lane];  // this lane's column: zc[sb * 32]
    float(*wr)[WT] = wsm[wi];
    // the window before t0: z_{t0-d} in register WT - d (d = 1 .. WT - 1),
    // drawn CR_SB at a time through the column
    float2 zr[WT];
#pragma unroll
    for (int i = 0; i < WT; ++i) zr[i] = make_float2(0.f, 0.f);
    if (valid && t0 > zlo) {
#pragma unroll
        for (int q = 0; q < WT / CR_SB; ++q) {
#pragma unroll 1
            for (int s = 0; s < CR_SB; ++s) {
                const int d = q * CR_SB + s + 1;
                zc[s * 32] = (d < WT && t0 - d >= zlo) ? fetch(t0 - d) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int s = 0; s < CR_SB; ++s) {
                const int d = q * CR_SB + s + 1;
                if (d < WT) zr[WT - d] = zc[s * 32];
            }
        }
    }
    // w rows of shells ub .. ub + CR_SB - 1 (lanes over the slots) into
    // registers, zero where absent: loaded one group ahead, so that the
    // loads are in flight while the current group's variates and sums run
    constexpr int NH = (WT + 31) / 32;
    float pre[CR_SB][NH];
    auto load_rows = [&](int ub) {
#pragma unroll
        for (int sb = 0; sb < CR_SB; ++sb) {
            const int64_t t = t0 + ub + sb;
            const int dmax = t < k ? (int)t : k;
            const float *row = w + ((size_t)(ub + sb) * L + l) * kp + k;
#pragma unroll
            for (int h = 0; h < NH; ++h) {
                const int j = lane + 32 * h, d = WT - 1 - j;
                pre[sb][h] = (ub + sb < nshell && j < WT && d <= dmax) ? row[-d] : 0.f;
            }
        }
    };
    // the staged rows and the variates of shells ub .. ub + nsb - 1
    auto stage = [&](int ub, int nsb) {
        __syncwarp();  // the previous group's rows and variates are read
#pragma unroll
        for (int sb = 0; sb < CR_SB; ++sb) {
#pragma unroll
            for (int h = 0; h < NH; ++h)
                if (lane + 32 * h < WT) wr[sb][lane + 32 * h] = pre[sb][h];
        }
        load_rows(ub + CR_SB);
        if (valid) {
#pragma unroll 1
            for (int sb = 0; sb < nsb; ++sb) zc[sb * 32] = fetch(t0 + ub + sb);
        }
        __syncwarp();
    };
    load_rows(0);
    // shell u, row sb: the window sum, oldest variate first; slot(j) is the
    // register of the variate whose coefficient sits in row slot j
    auto shell = [&](int u, int sb, auto slot) {
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int j = 0; j < WT; j += 4) {
            const float4 c4 = *reinterpret_cast<const float4 *>(&wr[sb][j]);
            const float2 z0 = zr[slot(j)], z1 = zr[slot(j + 1)], z2 = zr[slot(j + 2)], z3 = zr[slot(j + 3)];
            re = fmaf(c4.x, z0.x, re);
            im = fmaf(c4.x, z0.y, im);
            re = fmaf(c4.y, z1.x, re);
            im = fmaf(c4.y, z1.y, im);
            re = fmaf(c4.z, z2.x, re);
            im = fmaf(c4.z, z2.y, im);
            re = fmaf(c4.w, z3.x, re);
            im = fmaf(c4.w, z3.y, im);
        }
        if (m == 0) {
            re = re + im;
            im = 0.f;
        }
        if (valid) alm[(int64_t)u * nalm + ix] = make_float2(re, im);
    };
    for (int c0 = 0; c0 < nshell; c0 += WT) {
#pragma unroll
        for (int q = 0; q < WT / CR_SB; ++q) {
            const int ub = c0 + q * CR_SB;
            if (ub >= nshell) break;
            const int nsb = nshell - ub < CR_SB ? nshell - ub : CR_SB;
            stage(ub, nsb);
#pragma unroll
            for (int sb = 0; sb < CR_SB; ++sb) {
                if (sb >= nsb) break;
                const int uu = q * CR_SB + sb;  // a constant once unrolled: shell t0 + c0 + uu sits in register uu
                zr[uu] = valid ? zc[sb * 32] : make_float2(0.f, 0.f);
                shell(ub + sb, sb, [uu](int j) { return (uu + j + 1) % WT; });
            }
        }
    }
}

// ----------------------------------------------------------- multalm etc.

template <typename T2>
__global__ void k_multalm(const T2 *__restrict__ alm, const double *__restrict__ bl, int lmax,
                          T2 *__restrict__ out) {
    const int64_t n = glg_nalm(lmax);
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
         g += (int64_t)gridDim.x * blockDim.x) {
        int l = (int)((sqrt(8.0 * (double)g + 1.0) - 1.0) * 0.5);
        while ((int64_t)l * (l + 1) / 2 > g) --l;
        while ((int64_t)(l + 1) * (l + 2) / 2 <= g) ++l;
        const double f = bl[l];
        T2 a = alm[g];
        a.x = a.x * f;
        a.y = a.y * f;
        out[g] = a;
    }
}

template <typename T2>
__global__ void k_almxfl(const T2 *__restrict__ alm, const double *__restrict__ fl, int nfl,
                         int lmax, int nmaps, T2 *__restrict__ out) {
    const int64_t n = glg_nalm(lmax);
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n * nmaps;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ix = q % n;
        const double L2 = 2.0 * lmax + 3.0;
        int m = (int)floor((L2 - sqrt(L2 * L2 - 8.0 * (double)ix)) * 0.5);
        while ((int64_t)m * (2 * lmax + 3 - m) / 2 > ix) --m;
        while ((int64_t)(m + 1) * (2 * lmax + 3 - (m + 1)) / 2 <= ix) ++m;
        const int l = (int)(ix - (int64_t)m * (2 * lmax + 3 - m) / 2) + m;
        const double f = l < nfl ? fl[l] : 0.0;
        T2 a = alm[q];
        a.x = a.x * f;
        a.y = a.y * f;
        out[q] = a;
    }
}

int grid_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    if (b > 152 * 64) b = 152 * 64;
    return (int)(b > 0 ? b : 1);
}

}  // namespace

extern "C" int glg_iternorm(const double *cov, int64_t nrows, int64_t nl, int k, double *w,
                            uint64_t *status, void *stream) {
    GLG_REQUIRE(cov && w && status, "glg_iternorm: null pointer");
    GLG_REQUIRE(nrows >= 0 && nl >= 0, "glg_iternorm: negative size");
    // two k x k FP64 matrices and two k-vectors of one mode in shared memory: k <= 120
    GLG_REQUIRE(k >= 0 && k <= 120, "glg_iternorm: k must be in [0, 120] (shared memory of one mode)");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(status, 0xff, sizeof(uint64_t), st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_iternorm: status reset");
    if (nrows == 0 || nl == 0) return GLG_OK;
    const int kk = k > 0 ? k * k : 1;
    const size_t smem = sizeof(double) * (2 * (size_t)kk + 2 * (size_t)(k > 0 ? k : 1));
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_iternorm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    GLG_LAUNCH_SCOPE("k_iternorm", st);
    k_iternorm<<<(unsigned)nl, 32, smem, st>>>(cov, nrows, nl, k, w, (int64_t *)status);
    GLG_CHECK_LAUNCH("k_iternorm");
    return GLG_OK;
}

extern "C" int glg_cls2cov(const double *flat, const int64_t *offs, int nf, int nl, int nc,
                           double *cov, double *var, uint64_t *status, void *stream) {
    GLG_REQUIRE(flat && offs && cov && var && status, "glg_cls2cov: null pointer");
    GLG_REQUIRE(nf >= 0 && nl >= 0 && nc >= 0, "glg_cls2cov: negative size");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(status, 0xff, sizeof(uint64_t), st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_cls2cov: status reset");
    if (nf == 0) return GLG_OK;
    if (nl > 0) {
        GLG_LAUNCH_SCOPE("k_cls2cov", st);
        k_cls2cov<<<dim3((nl + 255) / 256, nf), 256, 0, st>>>(flat, offs, nf, nl, nc, cov);
        GLG_CHECK_LAUNCH("k_cls2cov");
    }
    {
        GLG_LAUNCH_SCOPE("k_cltovar", st);
        k_cltovar<<<nf, 256, 0, st>>>(flat, offs, var, (unsigned long long *)status);
        GLG_CHECK_LAUNCH("k_cltovar");
    }
    return GLG_OK;
}

extern "C" int glg_philox_normals(uint64_t seed, uint64_t sid, int64_t offset, int64_t n, int dtype,
                                  void *out, void *stream) {
    GLG_REQUIRE(out || n == 0, "glg_philox_normals: null output");
    GLG_REQUIRE(dtype == GLG_F64 || dtype == GLG_F32, "glg_philox_normals: bad dtype");
    GLG_REQUIRE(n >= 0 && offset >= 0, "glg_philox_normals: negative size");
    if (n == 0) return GLG_OK;
    GLG_LAUNCH_SCOPE("k_philox_normals", (cudaStream_t)stream);
    k_philox_normals<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(seed, sid, offset, n, dtype, out);
    GLG_CHECK_LAUNCH("k_philox_normals");
    return GLG_OK;
}

extern "C" int glg_gather_host(const void *const *src, const int64_t *bytes, int n, void *dst, int nthreads) {
    GLG_REQUIRE(n >= 0, "glg_gather_host: negative count");
    if (n == 0) return GLG_OK;
    GLG_REQUIRE(src && bytes && dst, "glg_gather_host: null pointer");
    std::vector<int64_t> off(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        GLG_REQUIRE(bytes[i] >= 0 && (bytes[i] == 0 || src[i]), "glg_gather_host: bad buffer");
        off[i + 1] = off[i] + bytes[i];
    }
    const int64_t total = off[n];
    // at least 2 MB a thread: below that, starting a thread costs more than it copies
    int nt = nthreads < 1 ? 1 : (nthreads > 32 ? 32 : nthreads);
    while (nt > 1 && total / nt < ((int64_t)2 << 20)) --nt;
    // thread t copies destination bytes [total t / nt, total (t + 1) / nt)
    auto run = [&](int t) {
        const int64_t b0 = total * t / nt, b1 = total * (t + 1) / nt;
        int i = (int)(std::upper_bound(off.begin(), off.end(), b0) - off.begin()) - 1;
        for (int64_t b = b0; b < b1; ++i) {
            const int64_t e = off[i + 1] < b1 ? off[i + 1] : b1;
            if (e > b) memcpy((char *)dst + b, (const char *)src[i] + (b - off[i]), (size_t)(e - b));
            b = e;
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(run, t);
    run(0);
    for (auto &th : pool) th.join();
    return GLG_OK;
}

extern "C" int glg_alm_correlate(const void *w, int nshell, int lmax, int k, int64_t t0,
                                 const void *z, int64_t z_first, uint64_t seed, uint64_t sid_base,
                                 int dtype, void *alm, void *stream) {
    GLG_REQUIRE(w && alm, "glg_alm_correlate: null pointer");
    GLG_REQUIRE(nshell >= 0 && lmax >= 0 && k >= 0 && t0 >= 0, "glg_alm_correlate: bad size");
    GLG_REQUIRE(dtype == GLG_F64 || dtype == GLG_F32, "glg_alm_correlate: bad dtype");
    GLG_REQUIRE(k <= 126, "glg_alm_correlate: k must be <= 126");
    if (z) GLG_REQUIRE(z_first == (t0 - k > 0 ? t0 - k : 0), "glg_alm_correlate: z must start at max(0, t0-k)");
    if (nshell == 0) return GLG_OK;
    const int window = k + 1;
    const size_t esz = dtype == GLG_F64 ? sizeof(double2) : sizeof(float2);
    const size_t rsz = dtype == GLG_F64 ? sizeof(double) : sizeof(float);
    int threads = 128;  // 16 l x 8 m; fewer m per tile when the variate window is long
    auto smem_for = [&](int th) {
        return (((rsz * CT_L * (size_t)(window | 1)) + 15) & ~(size_t)15) + esz * (size_t)window * th;
    };
    while (threads > CT_L && smem_for(threads) > 200 * 1024) threads /= 2;
    const size_t smem = smem_for(threads);
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == GLG_F32 && window <= 40) {  // the fast form's register window
        const dim3 g2((lmax + CR_WARPS) / CR_WARPS, (lmax + 32) / 32);
        using KR = void (*)(const float *, int, int, int, int64_t, const float2 *, int64_t, uint64_t, uint64_t, float2 *);
        static const KR kr[5] = {k_alm_correlate_rw<8>, k_alm_correlate_rw<16>, k_alm_correlate_rw<24>,
                                 k_alm_correlate_rw<32>, k_alm_correlate_rw<40>};
        GLG_LAUNCH_SCOPE("k_alm_correlate", st);
        kr[(window + 7) / 8 - 1]<<<g2, 32 * CR_WARPS, 0, st>>>((const float *)w, nshell, lmax, k, t0,
                                                                  (const float2 *)z, z_first, seed, sid_base,
                                                                  (float2 *)alm);
        GLG_CHECK_LAUNCH("k_alm_correlate");
        return GLG_OK;
    }
    dim3 grid((lmax + CT_L) / CT_L, (lmax + threads / CT_L) / (threads / CT_L));
    GLG_LAUNCH_SCOPE("k_alm_correlate", st);
    if (dtype == GLG_F64) {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(k_alm_correlate<double2, double>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_alm_correlate<double2, double><<<grid, threads, smem, st>>>(
            (const double *)w, nshell, lmax, k, t0, (const double2 *)z, z_first, seed, sid_base, (double2 *)alm, window);
    } else {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(k_alm_correlate<float2, float>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_alm_correlate<float2, float><<<grid, threads, smem, st>>>(
            (const float *)w, nshell, lmax, k, t0, (const float2 *)z, z_first, seed, sid_base, (float2 *)alm, window);
    }
    GLG_CHECK_LAUNCH("k_alm_correlate");
    return GLG_OK;
}

extern "C" int glg_multalm(const void *alm, const double *bl, int lmax, int dtype, void *out,
                           void *stream) {
    GLG_REQUIRE((alm && bl && out) || lmax < 0, "glg_multalm: null pointer");
    GLG_REQUIRE(dtype == GLG_F64 || dtype == GLG_F32, "glg_multalm: bad dtype");
    if (lmax < 0) return GLG_OK;
    const int64_t n = glg_nalm(lmax);
    cudaStream_t st = (cudaStream_t)stream;
    GLG_LAUNCH_SCOPE("k_multalm", st);
    if (dtype == GLG_F64)
        k_multalm<double2><<<grid_for(n, 256), 256, 0, st>>>((const double2 *)alm, bl, lmax, (double2 *)out);
    else
        k_multalm<float2><<<grid_for(n, 256), 256, 0, st>>>((const float2 *)alm, bl, lmax, (float2 *)out);
    GLG_CHECK_LAUNCH("k_multalm");
    return GLG_OK;
}

extern "C" int glg_almxfl(const void *alm, const double *fl, int nfl, int lmax, int nmaps, int dtype,
                          void *out, void *stream) {
    GLG_REQUIRE(alm && out, "glg_almxfl: null pointer");
    GLG_REQUIRE(fl || nfl == 0, "glg_almxfl: null fl");
    GLG_REQUIRE(lmax >= 0 && nmaps >= 0 && nfl >= 0, "glg_almxfl: bad size");
    GLG_REQUIRE(dtype == GLG_F64 || dtype == GLG_F32, "glg_almxfl: bad dtype");
    const int64_t n = glg_nalm(lmax) * nmaps;
    if (n == 0) return GLG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    GLG_LAUNCH_SCOPE("k_almxfl", st);
    if (dtype == GLG_F64)
        k_almxfl<double2><<<grid_for(n, 256), 256, 0, st>>>((const double2 *)alm, fl, nfl, lmax, nmaps, (double2 *)out);
    else
        k_almxfl<float2><<<grid_for(n, 256), 256, 0, st>>>((const float2 *)alm, fl, nfl, lmax, nmaps, (float2 *)out);
    GLG_CHECK_LAUNCH("k_almxfl");
    return GLG_OK;
}
