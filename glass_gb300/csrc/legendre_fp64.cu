// Plain FP64 Legendre sums of the HEALPix ring SHT (the drop-in form).
//
// Synthesis (inside healpy.alm2map, called at glass/healpix.py:71 from
// glass/fields.py:429):  F_m(ring) = sum_l a_lm lambda_lm(cos theta_ring),
// evaluated for a north ring and its mirror at once through
// lambda_lm(-x) = (-1)^(l+m) lambda_lm(x): E_m = sum over l-m even,
// O_m = sum over l-m odd, north = E + O, south = E - O.
//
// lambda_lm follows the normalised three-term recurrence in FP64 with an
// exponent scale of 2^800 steps (values whose scale is below zero are
// smaller than 2^-400 and contribute nothing), so lmax up to 16384 works.
#include <cuda_runtime.h>

#include "glg_internal.cuh"

namespace {

constexpr int LEG_THREADS = 128;  // ring pairs per block
constexpr int LEG_CHUNK = 64;     // l values staged per pass

struct RecState {
    double l0, l1;  // lambda_{l-1}, lambda_l
    int sc;         // exponent scale (0: values are exact)
};

__device__ __forceinline__ void rec_init(RecState &r, double mant, int sc) {
    r.l0 = 0.0;
    r.l1 = mant;
    r.sc = sc;
}

// Advance from l-1 to l (l >= m+1). Returns lambda_l (0 while negligible).
__device__ __forceinline__ double rec_step(RecState &r, int l, int m, double x, double2 ab) {
    double nl;
    if (l == m + 1)
        nl = sqrt(2.0 * m + 3.0) * x * r.l1;
    else
        nl = ab.x * (x * r.l1) - ab.y * r.l0;
    r.l0 = r.l1;
    r.l1 = nl;
    if (r.sc < 0 && fabs(nl) > GLG_TWO_P400) {
        r.l0 *= GLG_TWO_M800;
        r.l1 *= GLG_TWO_M800;
        r.sc += 1;
    }
    return r.sc == 0 ? r.l1 : 0.0;
}

// ------------------------------------------------------------ spin 0 synth

template <int NS>
__global__ void __launch_bounds__(LEG_THREADS)
k_leg_syn(const int npairs, const int nrings, const int lmax, const int64_t nalm,
          const double *__restrict__ cth, const int64_t *__restrict__ mofs,
          const double2 *__restrict__ coef, const double *__restrict__ lmm,
          const int *__restrict__ lmm_scale, const double2 *__restrict__ alm, const int nmaps,
          double2 *__restrict__ F) {
    const int m = blockIdx.y;
    const int map0 = blockIdx.z * NS;
    const int p = blockIdx.x * LEG_THREADS + threadIdx.x;
    const bool active = p < npairs;
    __shared__ double2 a_s[LEG_CHUNK][NS];
    __shared__ double2 c_s[LEG_CHUNK];

    const int pp = active ? p : npairs - 1;
    const double x = cth[pp];
    RecState r;
    rec_init(r, lmm[(int64_t)m * npairs + pp], lmm_scale[(int64_t)m * npairs + pp]);
    double2 E[NS], O[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) E[s] = O[s] = make_double2(0.0, 0.0);

    const int64_t base = mofs[m];
    for (int l0 = m; l0 <= lmax; l0 += LEG_CHUNK) {
        const int cnt = min(LEG_CHUNK, lmax + 1 - l0);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt * NS; t += LEG_THREADS) {
            const int j = t / NS, s = t % NS;
            const int mp = map0 + s;
            a_s[j][s] = mp < nmaps ? alm[(int64_t)mp * nalm + base + (l0 - m) + j]
                                   : make_double2(0.0, 0.0);
        }
        for (int t = threadIdx.x; t < cnt; t += LEG_THREADS) c_s[t] = coef[base + (l0 - m) + t];
        __syncthreads();
        for (int j = 0; j < cnt; ++j) {
            const int l = l0 + j;
            double lam;
            if (l == m)
                lam = r.sc == 0 ? r.l1 : 0.0;
            else
                lam = rec_step(r, l, m, x, c_s[j]);
            if (((l - m) & 1) == 0) {
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    E[s].x = fma(a_s[j][s].x, lam, E[s].x);
                    E[s].y = fma(a_s[j][s].y, lam, E[s].y);
                }
            } else {
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    O[s].x = fma(a_s[j][s].x, lam, O[s].x);
                    O[s].y = fma(a_s[j][s].y, lam, O[s].y);
                }
            }
        }
    }
    if (!active) return;
    const int rn = p, rs = nrings - 1 - p;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const int mp = map0 + s;
        if (mp >= nmaps) break;
        double2 *Fm = F + (int64_t)mp * nrings * (lmax + 1);
        Fm[(int64_t)rn * (lmax + 1) + m] = make_double2(E[s].x + O[s].x, E[s].y + O[s].y);
        if (rs != rn)
            Fm[(int64_t)rs * (lmax + 1) + m] = make_double2(E[s].x - O[s].x, E[s].y - O[s].y);
    }
}

// ------------------------------------------------------------ spin-s synth

// Per ring and m: Q_m = -sum lp E - i sum lm B, U_m = i sum lm E - sum lp B,
// with lambda^+ (lp) and lambda^- (lm) from lambda_l, lambda_{l-1}:
//   s = 1: N lp = -dlam, N lm = m lam / sin;                N = sqrt(l(l+1))
//   s = 2: N lp = -2 cot dlam + (2 m^2 / sin^2 - l(l+1)) lam,
//          N lm = (2 m / sin)(cot lam - dlam);              N = sqrt((l-1)l(l+1)(l+2))
//   dlam = (l x lam - sqrt((2l+1)/(2l-1) (l^2-m^2)) lam_{l-1}) / sin.
// Mirror ring: lp(pi-t) = (-1)^(l+m+s) lp(t), lm(pi-t) = -(-1)^(l+m+s) lm(t).
template <bool HASB>
__global__ void __launch_bounds__(LEG_THREADS)
k_leg_syn_spin(const int npairs, const int nrings, const int lmax, const int spin,
               const double *__restrict__ cth, const double *__restrict__ sth,
               const int64_t *__restrict__ mofs, const double2 *__restrict__ coef,
               const double *__restrict__ lmm, const int *__restrict__ lmm_scale,
               const double2 *__restrict__ elm, const double2 *__restrict__ blm,
               double2 *__restrict__ F) {
    const int m = blockIdx.y;
    const int p = blockIdx.x * LEG_THREADS + threadIdx.x;
    const bool active = p < npairs;
    // per l of the chunk: alm, recurrence coefficients, and the l-only
    // factors of lambda^+- (sqrt((2l+1)/(2l-1) (l^2-m^2)), 1/N, l(l+1)),
    // computed once per block instead of per ring (FP64 sqrt and division
    // are slow)
    __shared__ double2 e_s[LEG_CHUNK], b_s[HASB ? LEG_CHUNK : 1], c_s[LEG_CHUNK];
    __shared__ double f_s[LEG_CHUNK], n_s[LEG_CHUNK], ll_s[LEG_CHUNK];
    const int pp = active ? p : npairs - 1;
    const double x = cth[pp], sn = sth[pp];
    const double isn = 1.0 / sn, cot = x * isn;
    RecState r;
    rec_init(r, lmm[(int64_t)m * npairs + pp], lmm_scale[(int64_t)m * npairs + pp]);
    // accumulators [parity][+/-][E/B]
    double2 acc[2][2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int c = 0; c < 2; ++c) acc[a][b][c] = make_double2(0.0, 0.0);
    const int64_t base = mofs[m];
    const double fm = m;
    const double m2i2 = 2.0 * fm * fm * isn * isn, m2i = 2.0 * fm * isn, mi = fm * isn;
    double lam_prev = 0.0;
    for (int l0 = m; l0 <= lmax; l0 += LEG_CHUNK) {
        const int cnt = min(LEG_CHUNK, lmax + 1 - l0);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt; t += LEG_THREADS) {
            e_s[t] = elm[base + (l0 - m) + t];
            if constexpr (HASB) b_s[t] = blm[base + (l0 - m) + t];
            c_s[t] = coef[base + (l0 - m) + t];
            const double fl = l0 + t;
            f_s[t] = fl >= 1.0 ? sqrt((2.0 * fl + 1.0) / (2.0 * fl - 1.0) * (fl * fl - fm * fm)) : 0.0;
            n_s[t] = fl < spin ? 0.0
                     : spin == 1 ? 1.0 / sqrt(fl * (fl + 1.0))
                                 : 1.0 / sqrt((fl - 1.0) * fl * (fl + 1.0) * (fl + 2.0));
            ll_s[t] = fl * (fl + 1.0);
        }
        __syncthreads();
        for (int j = 0; j < cnt; ++j) {
            const int l = l0 + j;
            double lam;
            if (l == m) {
                lam = r.sc == 0 ? r.l1 : 0.0;
            } else {
                lam = rec_step(r, l, m, x, c_s[j]);
            }
            if (l >= spin && l >= 1) {
                const double dlam = ((double)l * x * lam - f_s[j] * lam_prev) * isn;
                const double nrm = n_s[j];
                double lp, lmv;
                if (spin == 1) {
                    lp = -dlam * nrm;
                    lmv = mi * lam * nrm;
                } else {
                    lp = (-2.0 * cot * dlam + (m2i2 - ll_s[j]) * lam) * nrm;
                    lmv = m2i * (cot * lam - dlam) * nrm;
                }
                const int par = (l - m) & 1;
                const double2 e = e_s[j];
                acc[par][0][0].x += lp * e.x;  acc[par][0][0].y += lp * e.y;
                acc[par][1][0].x += lmv * e.x; acc[par][1][0].y += lmv * e.y;
                if constexpr (HASB) {
                    const double2 b = b_s[j];
                    acc[par][0][1].x += lp * b.x;  acc[par][0][1].y += lp * b.y;
                    acc[par][1][1].x += lmv * b.x; acc[par][1][1].y += lmv * b.y;
                }
            }
            lam_prev = lam;
        }
    }
    if (!active) return;
    const int rn = p, rs = nrings - 1 - p;
    const double sg = (spin & 1) ? -1.0 : 1.0;  // (-1)^s
    for (int h = 0; h < 2; ++h) {
        if (h == 1 && rs == rn) break;
        const int ring = h == 0 ? rn : rs;
        // north: sum = even + odd ; south: lp -> (-1)^s (even - odd), lm -> -(-1)^s (even - odd)
        double2 pE, mE, pB, mB;
        if (h == 0) {
            pE = make_double2(acc[0][0][0].x + acc[1][0][0].x, acc[0][0][0].y + acc[1][0][0].y);
            mE = make_double2(acc[0][1][0].x + acc[1][1][0].x, acc[0][1][0].y + acc[1][1][0].y);
            pB = make_double2(acc[0][0][1].x + acc[1][0][1].x, acc[0][0][1].y + acc[1][0][1].y);
            mB = make_double2(acc[0][1][1].x + acc[1][1][1].x, acc[0][1][1].y + acc[1][1][1].y);
        } else {
            pE = make_double2(sg * (acc[0][0][0].x - acc[1][0][0].x), sg * (acc[0][0][0].y - acc[1][0][0].y));
            mE = make_double2(-sg * (acc[0][1][0].x - acc[1][1][0].x), -sg * (acc[0][1][0].y - acc[1][1][0].y));
            pB = make_double2(sg * (acc[0][0][1].x - acc[1][0][1].x), sg * (acc[0][0][1].y - acc[1][0][1].y));
            mB = make_double2(-sg * (acc[0][1][1].x - acc[1][1][1].x), -sg * (acc[0][1][1].y - acc[1][1][1].y));
        }
        // Q_m = -pE - i mB ; U_m = i mE - pB
        const double2 q = make_double2(-pE.x + mB.y, -pE.y - mB.x);
        const double2 u = make_double2(-mE.y - pB.x, mE.x - pB.y);
        F[(int64_t)ring * (lmax + 1) + m] = q;
        F[((int64_t)nrings + ring) * (lmax + 1) + m] = u;
    }
}

// ------------------------------------------------------------ spin 0 anal

// alm[l, m] (+)= sum_pairs lambda_lm(x_p) (G^N_m + (-1)^(l+m) G^S_m).
// One block per m owns alm[:, m]; ring pairs are looped in groups of
// LEG_THREADS, contributions are warp-reduced in a fixed order.
constexpr int ANA_THREADS = 128;
constexpr int ANA_WARPS = ANA_THREADS / 32;

__global__ void __launch_bounds__(ANA_THREADS)
k_leg_ana(const int npairs, const int nrings, const int lmax, const int64_t nalm,
          const double *__restrict__ cth, const int64_t *__restrict__ mofs,
          const double2 *__restrict__ coef, const double *__restrict__ lmm,
          const int *__restrict__ lmm_scale, const double2 *__restrict__ G, const int map,
          double2 *__restrict__ alm, const int accumulate) {
    const int m = blockIdx.x;
    const int64_t base = mofs[m];
    const int nl = lmax + 1 - m;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ double2 part[ANA_WARPS][LEG_CHUNK];
    __shared__ double2 c_s[LEG_CHUNK];
    double2 *out = alm + (int64_t)map * nalm + base;
    const double2 *Gm = G + (int64_t)map * nrings * (lmax + 1);
    for (int g0 = 0; g0 < npairs; g0 += ANA_THREADS) {
        const int p = g0 + threadIdx.x;
        const bool active = p < npairs;
        const int pp = active ? p : npairs - 1;
        const double x = cth[pp];
        RecState r;
        rec_init(r, lmm[(int64_t)m * npairs + pp], lmm_scale[(int64_t)m * npairs + pp]);
        double2 gE = make_double2(0.0, 0.0), gO = gE;
        if (active) {
            const int rn = p, rs = nrings - 1 - p;
            const double2 gn = Gm[(int64_t)rn * (lmax + 1) + m];
            const double2 gs = rs != rn ? Gm[(int64_t)rs * (lmax + 1) + m] : make_double2(0.0, 0.0);
            gE = make_double2(gn.x + gs.x, gn.y + gs.y);
            gO = make_double2(gn.x - gs.x, gn.y - gs.y);
        }
        for (int l0 = m; l0 <= lmax; l0 += LEG_CHUNK) {
            const int cnt = min(LEG_CHUNK, lmax + 1 - l0);
            __syncthreads();
            for (int t = threadIdx.x; t < cnt; t += ANA_THREADS) c_s[t] = coef[base + (l0 - m) + t];
            __syncthreads();
            // 16 l at a time: every lane forms its ring pair's 16 products,
            // then one butterfly reduction across the warp sums all 16 (each
            // step keeps half of the values and trades the other half with
            // the partner lane): 16 shuffles per 16 l and per component,
            // instead of 5 per l.  Lane 2k ends with the sum of l0 + j0 + k.
            for (int j0 = 0; j0 < cnt; j0 += 16) {
                double vr[16], vi[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int j = j0 + i, l = l0 + j;
                    double lam = 0.0;
                    if (j < cnt) lam = (l == m) ? (r.sc == 0 ? r.l1 : 0.0) : rec_step(r, l, m, x, c_s[j]);
                    if (!active) lam = 0.0;
                    const double2 g = (i & 1) ? gO : gE;  // l0 - m and j0 are even
                    vr[i] = lam * g.x;
                    vi[i] = lam * g.y;
                }
#pragma unroll
                for (int h = 8; h >= 1; h >>= 1) {  // lane bit 4, 3, 2, 1
                    const bool up = lane & (2 * h);
#pragma unroll
                    for (int i = 0; i < h; ++i) {
                        const double kr = up ? vr[i + h] : vr[i], ki = up ? vi[i + h] : vi[i];
                        const double sr = up ? vr[i] : vr[i + h], si = up ? vi[i] : vi[i + h];
                        vr[i] = kr + __shfl_xor_sync(0xffffffffu, sr, 2 * h);
                        vi[i] = ki + __shfl_xor_sync(0xffffffffu, si, 2 * h);
                    }
                }
                const double tr = vr[0] + __shfl_xor_sync(0xffffffffu, vr[0], 1);
                const double ti = vi[0] + __shfl_xor_sync(0xffffffffu, vi[0], 1);
                const int k = lane >> 1;
                if (!(lane & 1) && j0 + k < cnt) part[warp][j0 + k] = make_double2(tr, ti);
            }
            __syncthreads();
            for (int t = threadIdx.x; t < cnt; t += ANA_THREADS) {
                double2 s = part[0][t];
#pragma unroll
                for (int w = 1; w < ANA_WARPS; ++w) {
                    s.x += part[w][t].x;
                    s.y += part[w][t].y;
                }
                const int64_t ix = (l0 - m) + t;
                if (g0 == 0 && !accumulate) {
                    out[ix] = s;
                } else {
                    double2 o = out[ix];
                    out[ix] = make_double2(o.x + s.x, o.y + s.y);
                }
            }
        }
    }
    (void)nl;
}

}  // namespace

template <int NS>
static int launch_leg_syn(const glg_plan *P, const double2 *alm, int nmaps, double2 *F, cudaStream_t st) {
    dim3 grid((P->npairs + LEG_THREADS - 1) / LEG_THREADS, P->mmax + 1, (nmaps + NS - 1) / NS);
    GLG_LAUNCH_SCOPE("k_leg_syn", st);
    k_leg_syn<NS><<<grid, LEG_THREADS, 0, st>>>(P->npairs, P->nrings, P->lmax, P->nalm, P->cth,
                                                P->mofs, P->coef, P->lmm, P->lmm_scale, alm,
                                                nmaps, F);
    GLG_CHECK_LAUNCH("k_leg_syn");
    return GLG_OK;
}

// Maps per pass: the FP64 recurrence (~4 operations per lambda) is shared by
// the NS maps of a pass (2 FMA per lambda and map, also for empty slots of
// the last pass): NS in {1, 2, 4, 8} minimising passes x (2 NS + 4).
int glg_launch_leg_syn(const glg_plan *P, const double2 *alm, int nmaps, double2 *F,
                       cudaStream_t st) {
    int best = 1;
    long best_cost = -1;
    for (int ns : {8, 4, 2, 1}) {
        const long cost = (long)((nmaps + ns - 1) / ns) * (2 * ns + 4);
        if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            best = ns;
        }
    }
    switch (best) {
        case 8: return launch_leg_syn<8>(P, alm, nmaps, F, st);
        case 4: return launch_leg_syn<4>(P, alm, nmaps, F, st);
        case 2: return launch_leg_syn<2>(P, alm, nmaps, F, st);
        default: return launch_leg_syn<1>(P, alm, nmaps, F, st);
    }
}

int glg_launch_leg_syn_spin(const glg_plan *P, const double2 *elm, const double2 *blm, int spin,
                            double2 *F, cudaStream_t st) {
    dim3 grid((P->npairs + LEG_THREADS - 1) / LEG_THREADS, P->mmax + 1);
    GLG_LAUNCH_SCOPE("k_leg_syn_spin", st);
    if (blm)
        k_leg_syn_spin<true><<<grid, LEG_THREADS, 0, st>>>(P->npairs, P->nrings, P->lmax, spin, P->cth, P->sth,
                                                           P->mofs, P->coef, P->lmm, P->lmm_scale, elm, blm, F);
    else
        k_leg_syn_spin<false><<<grid, LEG_THREADS, 0, st>>>(P->npairs, P->nrings, P->lmax, spin, P->cth, P->sth,
                                                            P->mofs, P->coef, P->lmm, P->lmm_scale, elm, blm, F);
    GLG_CHECK_LAUNCH("k_leg_syn_spin");
    return GLG_OK;
}

int glg_launch_leg_ana(const glg_plan *P, const double2 *G, int nmaps, double2 *alm,
                       int accumulate, cudaStream_t st) {
    for (int k = 0; k < nmaps; ++k) {
        GLG_LAUNCH_SCOPE("k_leg_ana", st);
        k_leg_ana<<<P->mmax + 1, ANA_THREADS, 0, st>>>(P->npairs, P->nrings, P->lmax, P->nalm,
                                                       P->cth, P->mofs, P->coef, P->lmm,
                                                       P->lmm_scale, G, k, alm, accumulate);
        GLG_CHECK_LAUNCH("k_leg_ana");
    }
    return GLG_OK;
}
