// FP32 ring FFTs of the fast form (inside healpy.alm2map, glass/healpix.py:71).
//
// Input: Legendre sums F[map][m][ring] from the tensor-core contraction.  A
// tiled transpose makes every ring's m-vector contiguous; then one block per
// (ring pair, map) folds m onto the ring's n pixels, packs the north ring and
// its mirror as one complex sequence Z_k = B^N_k + i B^S_k, runs one complex
// inverse DFT of length n and stores both rings with the fused field
// transform (glass/grf/_transformations.py:83-89).
//
// Ring lengths n = 4 i whose prime factors are all <= 13 use an in-place
// mixed-radix decimation-in-frequency FFT whose twiddles come from a
// shared-memory table.  Lengths with a larger prime factor use Bluestein's
// algorithm: the DFT becomes a cyclic convolution of length M (a power of
// two, M >= 2n - 1) with the chirp h_t = e^{-i pi t^2 / n}, computed as a
// forward DIF FFT, a product with the precomputed chirp spectrum (stored in
// the DIF output order) and the adjoint of the DIF FFT, so that no
// permutation pass is needed.
#include <cuda_runtime.h>

#include "glg_internal.cuh"

namespace {

constexpr int T32 = 256;

struct c32 {
    float x, y;
};
__device__ __forceinline__ c32 cmul(c32 a, c32 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ c32 cadd(c32 a, c32 b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ c32 csub(c32 a, c32 b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ c32 cconj(c32 a) { return {a.x, -a.y}; }
__device__ __forceinline__ c32 ld(const float2 *p) {
    const float2 v = *p;
    return {v.x, v.y};
}

// e^{dir 2 pi i t / n} from a half table wh[t] = e^{2 pi i t / n}, t <= n/2.
__device__ __forceinline__ c32 tw(const c32 *wh, int n, int t, int dir) {
    c32 w = t <= (n >> 1) ? wh[t] : cconj(wh[n - t]);
    if (dir < 0) w.y = -w.y;
    return w;
}

struct FftDesc {
    int n, nst, dir;
    int radix[GLG_MAX_FFT_STAGES];
    const c32 *wh;
};

// One radix-RD DIF butterfly: y_k = sum_j v_j w_RD^{jk}, then twiddle w_L^{j1 k}.
template <int RD>
__device__ __forceinline__ void dif_bfly(c32 *Z, const FftDesc &f, int base, int msub, int L, int j1) {
    c32 v[RD], y[RD];
#pragma unroll
    for (int j = 0; j < RD; ++j) v[j] = Z[base + msub * j];
    if (RD == 2) {
        y[0] = cadd(v[0], v[1]);
        y[1] = csub(v[0], v[1]);
    } else if (RD == 4) {
        const c32 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
        const c32 cc = cadd(v[1], v[3]), d = csub(v[1], v[3]);
        const c32 id = f.dir > 0 ? c32{-d.y, d.x} : c32{d.y, -d.x};
        y[0] = cadd(a, cc);
        y[2] = csub(a, cc);
        y[1] = cadd(b, id);
        y[3] = csub(b, id);
    } else {
        const int step = f.n / RD;
#pragma unroll
        for (int k = 0; k < RD; ++k) {
            c32 acc = v[0];
#pragma unroll
            for (int j = 1; j < RD; ++j) acc = cadd(acc, cmul(v[j], tw(f.wh, f.n, ((j * k) % RD) * step, f.dir)));
            y[k] = acc;
        }
    }
    const int ts = (f.n / L) * j1;
    Z[base] = y[0];
#pragma unroll
    for (int k = 1; k < RD; ++k) Z[base + msub * k] = cmul(y[k], tw(f.wh, f.n, ts * k, f.dir));
}

// Adjoint of dif_bfly: undo the twiddle (conjugate), then the opposite-direction DFT_RD.
template <int RD>
__device__ __forceinline__ void adj_bfly(c32 *Z, const FftDesc &f, int base, int msub, int L, int j1) {
    c32 v[RD], y[RD];
    const int ts = (f.n / L) * j1;
    v[0] = Z[base];
#pragma unroll
    for (int k = 1; k < RD; ++k) v[k] = cmul(Z[base + msub * k], tw(f.wh, f.n, ts * k, -f.dir));
    if (RD == 2) {
        y[0] = cadd(v[0], v[1]);
        y[1] = csub(v[0], v[1]);
    } else if (RD == 4) {
        const c32 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
        const c32 cc = cadd(v[1], v[3]), d = csub(v[1], v[3]);
        const c32 id = f.dir > 0 ? c32{d.y, -d.x} : c32{-d.y, d.x};
        y[0] = cadd(a, cc);
        y[2] = csub(a, cc);
        y[1] = cadd(b, id);
        y[3] = csub(b, id);
    } else {
        const int step = f.n / RD;
#pragma unroll
        for (int j = 0; j < RD; ++j) {
            c32 acc = v[0];
#pragma unroll
            for (int k = 1; k < RD; ++k) acc = cadd(acc, cmul(v[k], tw(f.wh, f.n, ((j * k) % RD) * step, -f.dir)));
            y[j] = acc;
        }
    }
#pragma unroll
    for (int j = 0; j < RD; ++j) Z[base + msub * j] = y[j];
}

template <bool ADJ, bool POW2>
__device__ __forceinline__ void stage(c32 *Z, const FftDesc &f, int RD, int L) {
    const int msub = L / RD, nbf = f.n / RD;
    for (int bf = threadIdx.x; bf < nbf; bf += blockDim.x) {
        const int blk = bf / msub, j1 = bf - blk * msub;
        const int base = blk * L + j1;
        switch (RD) {
#define GLG_CASE(R)                                          \
    case R:                                                  \
        if (ADJ) adj_bfly<R>(Z, f, base, msub, L, j1);       \
        else dif_bfly<R>(Z, f, base, msub, L, j1);           \
        break;
            GLG_CASE(2) GLG_CASE(4)
            default:
                if constexpr (!POW2) {
                    switch (RD) { GLG_CASE(3) GLG_CASE(5) GLG_CASE(7) GLG_CASE(11) GLG_CASE(13) default: break; }
                }
                break;
#undef GLG_CASE
        }
    }
    __syncthreads();
}

template <bool POW2>
__device__ void fft_dif(c32 *Z, const FftDesc &f) {
    int L = f.n;
    for (int s = 0; s < f.nst; ++s) {
        stage<false, POW2>(Z, f, f.radix[s], L);
        L /= f.radix[s];
    }
}

template <bool POW2>
__device__ void fft_dif_adjoint(c32 *Z, const FftDesc &f) {
    int Ls[GLG_MAX_FFT_STAGES];
    int L = f.n;
    for (int s = 0; s < f.nst; ++s) {
        Ls[s] = L;
        L /= f.radix[s];
    }
    for (int s = f.nst - 1; s >= 0; --s) stage<true, POW2>(Z, f, f.radix[s], Ls[s]);
}

__device__ __forceinline__ float epi(float v, int kind, float hv, float lam) {
    if (kind == GLG_EPI_LOGNORMAL) {
        v = expm1f(v - hv);
        if (lam != 1.0f) v = lam * v;
    }
    return v;
}

struct Epi32 {
    int kind[8];
    float hvar[8], lam[8];  // var / 2 and lambda per map of the launch
};

struct RingArgs {
    int nrings, mmax, nside;
    const int *pairs;
    const int *nph, *half;
    const int64_t *startN, *startS;
    const int *fft_radix, *fft_nst;
    const int64_t *tw_ofs;
    const float2 *tw32;
    const int64_t *pos_ofs;
    const uint16_t *pos16;
    const int64_t *blu_ofs;
    const int *blu_M;
    const float2 *blu_H;
    const float2 *twM;
    int Mmax;
    const float2 *Ft;  // [map][ring][m]
    float *maps;
    int64_t npix;
    int map0;
};

// Fold F_m (m = 0..mmax) of both rings onto n bins, packed as B^N + i B^S:
// B_k = 1/2 sum_{m = k} c_m G_m + 1/2 sum_{m = -k} c_m conj(G_m), G_m = F_m e^{i m phi0}.
__device__ __forceinline__ c32 fold(const RingArgs &a, const float2 *FN, const float2 *FS, const float2 *tw2n,
                                    int n, int h, bool equator, int k) {
    c32 bn = {0.f, 0.f}, bs = {0.f, 0.f};
    for (int m = k; m <= a.mmax; m += n) {
        const float cm = m == 0 ? 0.5f : 1.0f;
        const c32 ph = h ? ld(tw2n + (m % (2 * n))) : c32{1.f, 0.f};
        const c32 gn = cmul(ld(FN + m), ph), gs = cmul(ld(FS + m), ph);
        bn = cadd(bn, c32{cm * gn.x, cm * gn.y});
        bs = cadd(bs, c32{cm * gs.x, cm * gs.y});
    }
    for (int m = (n - k) % n; m <= a.mmax; m += n) {
        const float cm = m == 0 ? 0.5f : 1.0f;
        const c32 ph = h ? ld(tw2n + (m % (2 * n))) : c32{1.f, 0.f};
        const c32 gn = cconj(cmul(ld(FN + m), ph)), gs = cconj(cmul(ld(FS + m), ph));
        bn = cadd(bn, c32{cm * gn.x, cm * gn.y});
        bs = cadd(bs, c32{cm * gs.x, cm * gs.y});
    }
    if (equator) bs = {0.f, 0.f};
    return {bn.x - bs.y, bn.y + bs.x};
}

// Class 0: mixed-radix DIF in shared memory.  smem: Z[n], wh[n/2 + 1].
__global__ void __launch_bounds__(T32) k_ring32(const RingArgs a, const Epi32 e) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int p = a.pairs[blockIdx.x];
    const int slot = blockIdx.y, map = a.map0 + slot;
    const int n = a.nph[p], i4 = n / 4;
    c32 *Z = reinterpret_cast<c32 *>(smem_raw);
    c32 *wh = Z + n;
    const float2 *tw2n = a.tw32 + a.tw_ofs[i4];  // e^{i pi t / n}, t < 2n
    for (int t = threadIdx.x; t <= n / 2; t += blockDim.x) wh[t] = ld(tw2n + 2 * t);
    FftDesc f;
    f.n = n;
    f.nst = a.fft_nst[i4];
    f.dir = 1;
    f.wh = wh;
    for (int s = 0; s < GLG_MAX_FFT_STAGES; ++s) f.radix[s] = a.fft_radix[i4 * GLG_MAX_FFT_STAGES + s];
    const int rn = p, rs = a.nrings - 1 - p;
    const bool equator = rn == rs;
    const float2 *FN = a.Ft + ((int64_t)map * a.nrings + rn) * (a.mmax + 1);
    const float2 *FS = a.Ft + ((int64_t)map * a.nrings + rs) * (a.mmax + 1);
    const int h = a.half[p];
    for (int k = threadIdx.x; k < n; k += blockDim.x) Z[k] = fold(a, FN, FS, tw2n, n, h, equator, k);
    __syncthreads();
    fft_dif<false>(Z, f);
    const uint16_t *pos = a.pos16 + a.pos_ofs[i4];
    float *mp = a.maps + (int64_t)map * a.npix;
    const int64_t sN = a.startN[p], sS = a.startS[p];
    const int kind = e.kind[slot];
    const float hv = e.hvar[slot], lam = e.lam[slot];
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const c32 v = Z[pos[j]];
        mp[sN + j] = epi(v.x, kind, hv, lam);
        if (!equator) mp[sS + j] = epi(v.y, kind, hv, lam);
    }
}

// Class 1: Bluestein.  smem: Z[M], wh[M/2 + 1].
__global__ void __launch_bounds__(T32) k_ring32_blu(const RingArgs a, const Epi32 e) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int p = a.pairs[blockIdx.x];
    const int slot = blockIdx.y, map = a.map0 + slot;
    const int n = a.nph[p], i4 = n / 4;
    const int M = a.blu_M[i4];
    c32 *Z = reinterpret_cast<c32 *>(smem_raw);
    c32 *wh = Z + M;
    const int stride = a.Mmax / M;
    for (int t = threadIdx.x; t <= M / 2; t += blockDim.x) wh[t] = ld(a.twM + (int64_t)t * stride);
    FftDesc f;
    f.n = M;
    f.dir = -1;
    f.wh = wh;
    {
        int r = M, s = 0;
        while (r % 4 == 0 && r > 1) { f.radix[s++] = 4; r /= 4; }
        while (r % 2 == 0) { f.radix[s++] = 2; r /= 2; }
        f.nst = s;
    }
    const float2 *tw2n = a.tw32 + a.tw_ofs[i4];  // e^{i pi t / n}: the chirp b_t = tw2n[t^2 mod 2n]
    const int rn = p, rs = a.nrings - 1 - p;
    const bool equator = rn == rs;
    const float2 *FN = a.Ft + ((int64_t)map * a.nrings + rn) * (a.mmax + 1);
    const float2 *FS = a.Ft + ((int64_t)map * a.nrings + rs) * (a.mmax + 1);
    const int h = a.half[p];
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        c32 v = {0.f, 0.f};
        if (k < n) {
            const c32 x = fold(a, FN, FS, tw2n, n, h, equator, k);
            v = cmul(x, ld(tw2n + (int)(((int64_t)k * k) % (2 * n))));
        }
        Z[k] = v;
    }
    __syncthreads();
    fft_dif<true>(Z, f);
    const float2 *H = a.blu_H + a.blu_ofs[i4];
    for (int k = threadIdx.x; k < M; k += blockDim.x) Z[k] = cmul(Z[k], ld(H + k));
    __syncthreads();
    fft_dif_adjoint<true>(Z, f);
    float *mp = a.maps + (int64_t)map * a.npix;
    const int64_t sN = a.startN[p], sS = a.startS[p];
    const int kind = e.kind[slot];
    const float hv = e.hvar[slot], lam = e.lam[slot];
    const float invM = 1.0f / (float)M;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        c32 v = cmul(Z[j], ld(tw2n + (int)(((int64_t)j * j) % (2 * n))));
        v.x *= invM;
        v.y *= invM;
        mp[sN + j] = epi(v.x, kind, hv, lam);
        if (!equator) mp[sS + j] = epi(v.y, kind, hv, lam);
    }
}

// F[map][m][ring] -> Ft[map][ring][m], 32 x 32 tiles.
__global__ void k_transpose32(const float2 *__restrict__ F, float2 *__restrict__ Ft, int nm, int nr) {
    __shared__ float2 tile[32][33];
    const int map = blockIdx.z;
    const int r0 = blockIdx.x * 32, m0 = blockIdx.y * 32;
    const float2 *src = F + (int64_t)map * nm * nr;
    float2 *dst = Ft + (int64_t)map * nm * nr;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int m = m0 + y, r = r0 + threadIdx.x;
        if (m < nm && r < nr) tile[y][threadIdx.x] = src[(int64_t)m * nr + r];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, m = m0 + threadIdx.x;
        if (m < nm && r < nr) dst[(int64_t)r * nm + m] = tile[threadIdx.x][y];
    }
}

}  // namespace

int glg_launch_ring_syn_f32(const glg_plan *P, const float2 *F, float2 *Ft, int nmaps, float *maps,
                            const glg_epilogue *epi_in, cudaStream_t st) {
    const int nm = P->mmax + 1, nr = P->nrings;
    {
        dim3 grid((nr + 31) / 32, (nm + 31) / 32, nmaps);
        GLG_LAUNCH_SCOPE("k_transpose32", st);
        k_transpose32<<<grid, dim3(32, 8), 0, st>>>(F, Ft, nm, nr);
        GLG_CHECK_LAUNCH("k_transpose32");
    }
    const size_t smem0 = sizeof(c32) * ((size_t)4 * P->nside + 2 * P->nside + 1);
    const size_t smem1 = sizeof(c32) * ((size_t)P->blu_Mmax + P->blu_Mmax / 2 + 1);
    if (smem0 > 227 * 1024 || (P->ncls1 > 0 && smem1 > 227 * 1024)) {
        glg_set_error("fast ring FFT: ring length too large for shared memory (nside <= 2048)");
        return GLG_ERR_UNSUPPORTED;
    }
    cudaFuncSetAttribute(k_ring32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0);
    cudaFuncSetAttribute(k_ring32_blu, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
    RingArgs a;
    a.nrings = nr;
    a.mmax = P->mmax;
    a.nside = P->nside;
    a.nph = P->nph;
    a.half = P->half;
    a.startN = P->startN;
    a.startS = P->startS;
    a.fft_radix = P->fft_radix;
    a.fft_nst = P->fft_nst;
    a.tw_ofs = P->tw_ofs;
    a.tw32 = P->tw32;
    a.pos_ofs = P->pos_ofs;
    a.pos16 = P->pos16;
    a.blu_ofs = P->blu_ofs;
    a.blu_M = P->blu_M;
    a.blu_H = P->blu_H;
    a.twM = P->twM;
    a.Mmax = P->blu_Mmax;
    a.Ft = Ft;
    a.maps = maps;
    a.npix = P->npix;
    for (int m0 = 0; m0 < nmaps; m0 += 8) {
        const int cnt = nmaps - m0 < 8 ? nmaps - m0 : 8;
        Epi32 e;
        for (int k = 0; k < 8; ++k) {
            const bool on = epi_in && k < cnt;
            e.kind[k] = !on ? GLG_EPI_NONE : (epi_in->kinds ? epi_in->kinds[m0 + k] : epi_in->kind);
            e.hvar[k] = (on && epi_in->var) ? (float)(0.5 * epi_in->var[m0 + k]) : 0.f;
            e.lam[k] = (on && epi_in->lamda) ? (float)epi_in->lamda[m0 + k] : 1.f;
        }
        a.map0 = m0;
        if (P->ncls1 > 0) {
            a.pairs = P->cls1_pairs;
            GLG_LAUNCH_SCOPE("k_ring32_blu", st);
            k_ring32_blu<<<dim3(P->ncls1, cnt), T32, smem1, st>>>(a, e);
            GLG_CHECK_LAUNCH("k_ring32_blu");
        }
        if (P->ncls0 > 0) {
            a.pairs = P->cls0_pairs;
            GLG_LAUNCH_SCOPE("k_ring32", st);
            k_ring32<<<dim3(P->ncls0, cnt), T32, smem0, st>>>(a, e);
            GLG_CHECK_LAUNCH("k_ring32");
        }
    }
    return GLG_OK;
}
