// Ring FFTs of the HEALPix ring SHT, FP64 (plain form) and FP32 (fast form).
//
// Synthesis (inside healpy.alm2map, glass/healpix.py:71): for every ring
// pair, the Legendre sums F_m of the north and the south ring are folded
// onto the ring's n = nph pixels (m aliased modulo n, phase e^{i m phi0},
// Hermitian symmetrised) and packed as Z_k = B^N_k + i B^S_k, so that one
// complex inverse DFT of length n yields both real rings:
//   f^N_j + i f^S_j = sum_k Z_k e^{+2 pi i jk/n}.
// The DFT is an in-place mixed-radix decimation-in-frequency FFT in shared
// memory (radices 4, 2, then odd primes; primes above 13 use a cooperative
// O(n p) pass).  The map store fuses the field transform
// (glass/grf/_transformations.py:83-89, lambda * expm1(x - var/2)).
//
// Analysis (inside healpy.map2alm, glass/healpix.py:270) runs the forward
// transform of f^N + i f^S and unpacks the two spectra.
#include <cuda_runtime.h>

#include "glg_internal.cuh"

namespace {

constexpr int FFT_THREADS = 256;
constexpr int SMALL_RADIX_MAX = 13;

template <typename R>
struct cplx {
    R x, y;
};
template <typename R>
struct vec2;
template <>
struct vec2<double> {
    using type = double2;
};
template <>
struct vec2<float> {
    using type = float2;
};
template <typename R>
using V2 = typename vec2<R>::type;

template <typename R>
__device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename R>
__device__ __forceinline__ cplx<R> cadd(cplx<R> a, cplx<R> b) {
    return {a.x + b.x, a.y + b.y};
}
template <typename R>
__device__ __forceinline__ cplx<R> csub(cplx<R> a, cplx<R> b) {
    return {a.x - b.x, a.y - b.y};
}
template <typename R>
__device__ __forceinline__ cplx<R> cconj(cplx<R> a) {
    return {a.x, -a.y};
}
template <typename R>
__device__ __forceinline__ cplx<R> ld(const V2<R> *p) {
    V2<R> v = *p;
    return {v.x, v.y};
}

template <typename R>
struct RingCtx {
    int n;
    const V2<R> *tw;  // omega_{2n}^t, t < 2n (synthesis direction e^{+i})
    const int *radix;
    int nst;
    int dir;  // +1 synthesis (e^{+2 pi i/n}), -1 analysis
};

// omega_n^t in direction dir, 0 <= t < n
template <typename R>
__device__ __forceinline__ cplx<R> wn(const RingCtx<R> &c, int t) {
    cplx<R> w = ld<R>(c.tw + 2 * t);
    if (c.dir < 0) w.y = -w.y;
    return w;
}

template <typename R, int RD>
__device__ __forceinline__ void bfly_small(cplx<R> *Z, const RingCtx<R> &c, int base, int msub,
                                           int L, int j1) {
    cplx<R> v[RD];
#pragma unroll
    for (int j = 0; j < RD; ++j) v[j] = Z[base + msub * j];
    cplx<R> y[RD];
    if (RD == 2) {
        y[0] = cadd(v[0], v[1]);
        y[1] = csub(v[0], v[1]);
    } else if (RD == 4) {
        // omega_4 = dir * i
        cplx<R> a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
        cplx<R> cc = cadd(v[1], v[3]), d = csub(v[1], v[3]);
        cplx<R> id = c.dir > 0 ? cplx<R>{-d.y, d.x} : cplx<R>{d.y, -d.x};
        y[0] = cadd(a, cc);
        y[2] = csub(a, cc);
        y[1] = cadd(b, id);
        y[3] = csub(b, id);
    } else {
        const int step = c.n / RD;
#pragma unroll
        for (int k = 0; k < RD; ++k) {
            cplx<R> acc = v[0];
#pragma unroll
            for (int j = 1; j < RD; ++j) acc = cadd(acc, cmul(v[j], wn(c, ((j * k) % RD) * step)));
            y[k] = acc;
        }
    }
    // twiddle omega_L^{j1 k} = omega_n^{(n/L) j1 k}
    const int tstep = (c.n / L) * j1;
    Z[base] = y[0];
#pragma unroll
    for (int k = 1; k < RD; ++k) Z[base + msub * k] = cmul(y[k], wn(c, tstep * k));
}

// In-place DIF mixed-radix FFT of Z[0..n) in shared memory.
template <typename R>
__device__ void fft_dif(cplx<R> *Z, cplx<R> *scratch, const RingCtx<R> &c) {
    int L = c.n;
    for (int s = 0; s < c.nst; ++s) {
        const int RD = c.radix[s];
        const int msub = L / RD;
        const int nbf = c.n / RD;
        if (RD <= SMALL_RADIX_MAX) {
            for (int bf = threadIdx.x; bf < nbf; bf += blockDim.x) {
                const int blk = bf / msub, j1 = bf - blk * msub;
                const int base = blk * L + j1;
                switch (RD) {
                    case 2: bfly_small<R, 2>(Z, c, base, msub, L, j1); break;
                    case 3: bfly_small<R, 3>(Z, c, base, msub, L, j1); break;
                    case 4: bfly_small<R, 4>(Z, c, base, msub, L, j1); break;
                    case 5: bfly_small<R, 5>(Z, c, base, msub, L, j1); break;
                    case 7: bfly_small<R, 7>(Z, c, base, msub, L, j1); break;
                    case 11: bfly_small<R, 11>(Z, c, base, msub, L, j1); break;
                    case 13: bfly_small<R, 13>(Z, c, base, msub, L, j1); break;
                    default: break;
                }
            }
            __syncthreads();
        } else {
            // large prime radix: one butterfly at a time, threads over outputs
            const int step = c.n / RD;
            for (int bf = 0; bf < nbf; ++bf) {
                const int blk = bf / msub, j1 = bf - blk * msub;
                const int base = blk * L + j1;
                const int tstep = (c.n / L) * j1;
                for (int k = threadIdx.x; k < RD; k += blockDim.x) {
                    cplx<R> acc = {R(0), R(0)};
                    int t = 0;  // (j k) mod RD
                    for (int j = 0; j < RD; ++j) {
                        acc = cadd(acc, cmul(Z[base + msub * j], wn(c, t * step)));
                        t += k;
                        if (t >= RD) t -= RD;
                    }
                    scratch[k] = k == 0 ? acc : cmul(acc, wn(c, tstep * k));
                }
                __syncthreads();
                for (int k = threadIdx.x; k < RD; k += blockDim.x) Z[base + msub * k] = scratch[k];
                __syncthreads();
            }
        }
        L = msub;
    }
}

// Position of output k after the in-place DIF passes (mixed-radix digit reversal).
template <typename R>
__device__ __forceinline__ int dif_pos(const RingCtx<R> &c, int k) {
    int pos = 0, span = c.n;
    for (int s = 0; s < c.nst; ++s) {
        const int RD = c.radix[s];
        span /= RD;
        const int d = k % RD;
        k /= RD;
        pos += d * span;
    }
    return pos;
}

__device__ __forceinline__ double apply_epi(double v, int kind, double var, double lam) {
    if (kind == GLG_EPI_LOGNORMAL) {
        v = expm1(v - var * 0.5);
        if (lam != 1.0) v = lam * v;
    }
    return v;
}

struct EpiArgs {
    int kind[8];  // per map of this launch chunk
    double var[8], lam[8];
};

// Strides of the Legendre-sum array F (in complex elements).
struct FLayout {
    int64_t map, ring, m;
};

// grid (npairs, nmaps): F -> maps [nmaps][npix].  GB: rings too long for
// shared memory (nside > 2048 in FP64): a persistent grid over the items
// (ring pair, map), each block's ring buffer a slice of gbuf (gstride
// complex values per block; the slices of the blocks in flight stay in L2).
template <typename R, bool GB>
__global__ void __launch_bounds__(FFT_THREADS)
k_ring_syn(const int nrings, const int mmax, const int *__restrict__ nph, const int *__restrict__ half,
           const int64_t *__restrict__ startN, const int64_t *__restrict__ startS,
           const int *__restrict__ fft_radix, const int *__restrict__ fft_nst,
           const int64_t *__restrict__ tw_ofs, const V2<R> *__restrict__ tw,
           const V2<R> *__restrict__ F, const FLayout fl, R *__restrict__ maps, const int64_t npix,
           const int map0, const EpiArgs epi, cplx<R> *gbuf, const int64_t gstride, const int nitems,
           const int cnt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int radix_s[GLG_MAX_FFT_STAGES];
    for (int it = GB ? blockIdx.x : 0; it < (GB ? nitems : 1); it += (GB ? gridDim.x : 1)) {
    const int p = GB ? it / cnt : blockIdx.x;
    const int slot = GB ? it % cnt : blockIdx.y;
    const int map = map0 + slot;
    const int n = nph[p];
    const int i4 = n / 4;
    cplx<R> *Z = GB ? gbuf + (int64_t)blockIdx.x * gstride : reinterpret_cast<cplx<R> *>(smem_raw);
    cplx<R> *scratch = Z + n;
    if (threadIdx.x < GLG_MAX_FFT_STAGES)
        radix_s[threadIdx.x] = fft_radix[i4 * GLG_MAX_FFT_STAGES + threadIdx.x];
    RingCtx<R> c;
    c.n = n;
    c.tw = tw + tw_ofs[i4];
    c.radix = radix_s;
    c.nst = fft_nst[i4];
    c.dir = 1;
    const int h = half[p];
    const int rn = p, rs = nrings - 1 - p;
    const bool equator = rn == rs;
    const V2<R> *FN = F + (int64_t)map * fl.map + (int64_t)rn * fl.ring;
    const V2<R> *FS = F + (int64_t)map * fl.map + (int64_t)rs * fl.ring;
    // fold: B_k = 1/2 sum_{m = k mod n} c_m G_m + 1/2 sum_{m = -k mod n} c_m conj(G_m)
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        cplx<R> bn = {R(0), R(0)}, bs = {R(0), R(0)};
        for (int m = k; m <= mmax; m += n) {
            const R cm = m == 0 ? R(0.5) : R(1);
            cplx<R> ph = h ? ld<R>(c.tw + (m % (2 * n))) : cplx<R>{R(1), R(0)};
            cplx<R> gn = cmul(ld<R>(FN + m * fl.m), ph);
            cplx<R> gs = cmul(ld<R>(FS + m * fl.m), ph);
            bn = cadd(bn, cplx<R>{cm * gn.x, cm * gn.y});
            bs = cadd(bs, cplx<R>{cm * gs.x, cm * gs.y});
        }
        for (int m = (n - k) % n; m <= mmax; m += n) {
            const R cm = m == 0 ? R(0.5) : R(1);
            cplx<R> ph = h ? ld<R>(c.tw + (m % (2 * n))) : cplx<R>{R(1), R(0)};
            cplx<R> gn = cconj(cmul(ld<R>(FN + m * fl.m), ph));
            cplx<R> gs = cconj(cmul(ld<R>(FS + m * fl.m), ph));
            bn = cadd(bn, cplx<R>{cm * gn.x, cm * gn.y});
            bs = cadd(bs, cplx<R>{cm * gs.x, cm * gs.y});
        }
        if (equator) bs = {R(0), R(0)};
        Z[k] = {bn.x - bs.y, bn.y + bs.x};  // B^N + i B^S
    }
    __syncthreads();
    fft_dif<R>(Z, scratch, c);
    const double var = epi.var[slot], lam = epi.lam[slot];
    const int ekind = epi.kind[slot];
    R *mp = maps + (int64_t)map * npix;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const cplx<R> v = Z[dif_pos(c, j)];
        mp[startN[p] + j] = apply_epi(v.x, ekind, var, lam);
        if (!equator) mp[startS[p] + j] = apply_epi(v.y, ekind, var, lam);
    }
    __syncthreads();  // the buffer and the radix table are reused by the block's next item
    }
}

// grid (npairs, nmaps): maps -> G [nmaps][nrings][mmax+1],
// G_m = (4 pi / npix) e^{-i m phi0} sum_j f_j e^{-2 pi i m j / n}.
template <bool GB>
__global__ void __launch_bounds__(FFT_THREADS)
k_ring_ana(const int nrings, const int mmax, const int *__restrict__ nph, const int *__restrict__ half,
           const int64_t *__restrict__ startN, const int64_t *__restrict__ startS,
           const int *__restrict__ fft_radix, const int *__restrict__ fft_nst,
           const int64_t *__restrict__ tw_ofs, const double2 *__restrict__ tw,
           const double *__restrict__ maps, const int64_t npix, double2 *__restrict__ G,
           cplx<double> *gbuf, const int64_t gstride, const int nitems, const int nmaps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int radix_s[GLG_MAX_FFT_STAGES];
    for (int it = GB ? blockIdx.x : 0; it < (GB ? nitems : 1); it += (GB ? gridDim.x : 1)) {
    const int p = GB ? it / nmaps : blockIdx.x;
    const int map = GB ? it % nmaps : blockIdx.y;
    const int n = nph[p];
    const int i4 = n / 4;
    cplx<double> *Z = GB ? gbuf + (int64_t)blockIdx.x * gstride : reinterpret_cast<cplx<double> *>(smem_raw);
    cplx<double> *scratch = Z + n;
    if (threadIdx.x < GLG_MAX_FFT_STAGES)
        radix_s[threadIdx.x] = fft_radix[i4 * GLG_MAX_FFT_STAGES + threadIdx.x];
    RingCtx<double> c;
    c.n = n;
    c.tw = tw + tw_ofs[i4];
    c.radix = radix_s;
    c.nst = fft_nst[i4];
    c.dir = -1;
    const int h = half[p];
    const int rn = p, rs = nrings - 1 - p;
    const bool equator = rn == rs;
    const double *mp = maps + (int64_t)map * npix;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double fn = mp[startN[p] + j];
        const double fs = equator ? 0.0 : mp[startS[p] + j];
        Z[j] = {fn, fs};
    }
    __syncthreads();
    fft_dif<double>(Z, scratch, c);
    const double w = 4.0 * 3.14159265358979323846 / (double)npix;
    double2 *GN = G + ((int64_t)map * nrings + rn) * (mmax + 1);
    double2 *GS = G + ((int64_t)map * nrings + rs) * (mmax + 1);
    for (int m = threadIdx.x; m <= mmax; m += blockDim.x) {
        const int k = m % n;
        const int kc = (n - k) % n;
        const cplx<double> X = Z[dif_pos(c, k)];
        const cplx<double> Xc = cconj(Z[dif_pos(c, kc)]);
        // spectra of the real parts: N = (X + conj X_{-k})/2, S = (X - conj X_{-k})/(2i)
        cplx<double> sn = {0.5 * (X.x + Xc.x), 0.5 * (X.y + Xc.y)};
        cplx<double> ss = {0.5 * (X.y - Xc.y), -0.5 * (X.x - Xc.x)};
        cplx<double> ph = h ? cconj(ld<double>(c.tw + (m % (2 * n)))) : cplx<double>{1.0, 0.0};
        sn = cmul(sn, ph);
        ss = cmul(ss, ph);
        GN[m] = make_double2(w * sn.x, w * sn.y);
        if (!equator) GS[m] = make_double2(w * ss.x, w * ss.y);
    }
    __syncthreads();  // the buffer and the radix table are reused by the block's next item
    }
}

template <typename R>
size_t ring_smem_bytes(int nmax) {
    // data + large-radix scratch (a prime radix is at most n / 4)
    return sizeof(cplx<R>) * ((size_t)nmax + (size_t)nmax / 4 + 1);
}

constexpr int GB_SLOTS = 304;  // blocks of the persistent global-buffer grid

template <typename R>
int launch_ring_syn(const glg_plan *P, const V2<R> *tw, const V2<R> *F, FLayout fl, int nmaps,
                    R *maps, const glg_epilogue *epi, void *gbuf, cudaStream_t st) {
    const size_t smem = ring_smem_bytes<R>(4 * P->nside);
    const bool gb = smem > 227 * 1024;
    if (gb && !gbuf) {
        glg_set_error("ring FFT: rings too long for shared memory and no global ring buffers given");
        return GLG_ERR_UNSUPPORTED;
    }
    const int64_t gstride = (int64_t)(smem / sizeof(cplx<R>));
    if (!gb) cudaFuncSetAttribute(k_ring_syn<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    for (int m0 = 0; m0 < nmaps; m0 += 8) {
        const int cnt = nmaps - m0 < 8 ? nmaps - m0 : 8;
        EpiArgs ea;
        for (int k = 0; k < 8; ++k) {
            ea.kind[k] = !epi || k >= cnt ? GLG_EPI_NONE : (epi->kinds ? epi->kinds[m0 + k] : epi->kind);
            ea.var[k] = (epi && epi->var && k < cnt) ? epi->var[m0 + k] : 0.0;
            ea.lam[k] = (epi && epi->lamda && k < cnt) ? epi->lamda[m0 + k] : 1.0;
        }
        GLG_LAUNCH_SCOPE("k_ring_syn", st);
        if (gb) {
            const int nitems = P->npairs * cnt;
            k_ring_syn<R, true><<<nitems < GB_SLOTS ? nitems : GB_SLOTS, FFT_THREADS, 0, st>>>(
                P->nrings, P->mmax, P->nph, P->half, P->startN, P->startS, P->fft_radix, P->fft_nst, P->tw_ofs,
                tw, F, fl, maps, P->npix, m0, ea, (cplx<R> *)gbuf, gstride, nitems, cnt);
        } else {
            dim3 grid(P->npairs, cnt);
            k_ring_syn<R, false><<<grid, FFT_THREADS, smem, st>>>(
                P->nrings, P->mmax, P->nph, P->half, P->startN, P->startS, P->fft_radix, P->fft_nst, P->tw_ofs,
                tw, F, fl, maps, P->npix, m0, ea, nullptr, 0, 0, cnt);
        }
        GLG_CHECK_LAUNCH("k_ring_syn");
    }
    return GLG_OK;
}

}  // namespace

size_t glg_ring64_gbuf_bytes(const glg_plan *P) {
    const size_t smem = ring_smem_bytes<double>(4 * P->nside);
    return smem > 227 * 1024 ? (size_t)GB_SLOTS * smem : 0;
}

int glg_launch_ring_syn(const glg_plan *P, const double2 *F, int nmaps, double *maps,
                        const glg_epilogue *epi, void *gbuf, cudaStream_t st) {
    const FLayout fl{(int64_t)P->nrings * (P->mmax + 1), (int64_t)(P->mmax + 1), 1};
    return launch_ring_syn<double>(P, P->tw, F, fl, nmaps, maps, epi, gbuf, st);
}


int glg_launch_ring_ana(const glg_plan *P, const double *maps, int nmaps, double2 *G, void *gbuf,
                        cudaStream_t st) {
    const size_t smem = ring_smem_bytes<double>(4 * P->nside);
    const bool gb = smem > 227 * 1024;
    if (gb && !gbuf) {
        glg_set_error("ring FFT: rings too long for shared memory and no global ring buffers given");
        return GLG_ERR_UNSUPPORTED;
    }
    GLG_LAUNCH_SCOPE("k_ring_ana", st);
    if (gb) {
        const int nitems = P->npairs * nmaps;
        k_ring_ana<true><<<nitems < GB_SLOTS ? nitems : GB_SLOTS, FFT_THREADS, 0, st>>>(
            P->nrings, P->mmax, P->nph, P->half, P->startN, P->startS, P->fft_radix, P->fft_nst, P->tw_ofs, P->tw,
            maps, P->npix, G, (cplx<double> *)gbuf, (int64_t)(smem / sizeof(cplx<double>)), nitems, nmaps);
    } else {
        cudaFuncSetAttribute(k_ring_ana<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        dim3 grid(P->npairs, nmaps);
        k_ring_ana<false><<<grid, FFT_THREADS, smem, st>>>(P->nrings, P->mmax, P->nph, P->half, P->startN,
                                                          P->startS, P->fft_radix, P->fft_nst, P->tw_ofs,
                                                          P->tw, maps, P->npix, G, nullptr, 0, 0, nmaps);
    }
    GLG_CHECK_LAUNCH("k_ring_ana");
    return GLG_OK;
}
