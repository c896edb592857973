// Plan creation: HEALPix ring geometry, FP64 Legendre recurrence tables and
// ring-FFT tables, built on the device once per (nside, lmax).
//
// Geometry follows the HEALPix RING scheme (Gorski et al. 2005), which the
// reference reaches through healpy/healpix (glass/healpix.py:38-78,
// :293-310).
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <math.h>

#include <algorithm>
#include <complex>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "glg_internal.cuh"

static thread_local std::string g_last_error;

void glg_set_error(const std::string &msg) { g_last_error = msg; }

int glg_cuda_status(cudaError_t err, const char *where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(err);
    return err == cudaErrorMemoryAllocation ? GLG_ERR_NOMEM : GLG_ERR_CUDA;
}

extern "C" const char *glg_version(void) { return "glass_gb300 0.1 (sm_103a)"; }
extern "C" const char *glg_last_error(void) { return g_last_error.c_str(); }

// ------------------------------------------------------- launch accounting

namespace {
struct TimingRecord {
    std::string name;
    cudaEvent_t ev0, ev1;
};
std::mutex g_timing_mu;
std::vector<TimingRecord> g_records;
bool g_timing_on = false;
long long g_launches = 0;
}  // namespace

glg_launch_scope::glg_launch_scope(const char *n, cudaStream_t s)
    : name(n), st(s), ev0(nullptr), ev1(nullptr), timed(false) {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    ++g_launches;
    if (g_timing_on && cudaEventCreate(&ev0) == cudaSuccess && cudaEventCreate(&ev1) == cudaSuccess) {
        timed = cudaEventRecord(ev0, st) == cudaSuccess;
    }
}

glg_launch_scope::~glg_launch_scope() {
    if (!timed) return;
    cudaEventRecord(ev1, st);
    std::lock_guard<std::mutex> lk(g_timing_mu);
    g_records.push_back({name, ev0, ev1});
}

extern "C" int glg_timing_enable(int on) {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    g_timing_on = on != 0;
    return GLG_OK;
}

extern "C" int glg_timing_reset(void) {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    for (auto &r : g_records) {
        cudaEventDestroy(r.ev0);
        cudaEventDestroy(r.ev1);
    }
    g_records.clear();
    g_launches = 0;
    return GLG_OK;
}

extern "C" int64_t glg_launch_count(void) {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    return g_launches;
}

extern "C" int glg_timing_query(const char *name, double *total_ms, int64_t *launches) {
    GLG_REQUIRE(name && total_ms && launches, "glg_timing_query: null pointer");
    std::lock_guard<std::mutex> lk(g_timing_mu);
    double tot = 0.0;
    int64_t cnt = 0;
    for (auto &r : g_records) {
        if (r.name != name) continue;
        cudaError_t e = cudaEventSynchronize(r.ev1);
        if (e != cudaSuccess) return glg_cuda_status(e, "glg_timing_query");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.ev0, r.ev1);
        tot += ms;
        ++cnt;
    }
    *total_ms = tot;
    *launches = cnt;
    return GLG_OK;
}

// ---------------------------------------------------------------- kernels

__global__ void k_plan_rings(int nside, int npairs, double *cth, double *sth, int *nph, int *half,
                             int64_t *startN, int64_t *startS) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const int ir = p + 1;  // 1-based ring index counted from the north pole
    const double ns = nside;
    const int64_t npix = 12LL * nside * nside;
    const int64_t ncap = 2LL * nside * (nside - 1);
    double z, s;
    if (ir < nside) {
        double t = (double)ir * ir / (3.0 * ns * ns);
        z = 1.0 - t;
        s = sqrt(t * (2.0 - t));
        nph[p] = 4 * ir;
        half[p] = 1;
        startN[p] = 2LL * ir * (ir - 1);
        startS[p] = npix - 2LL * ir * (ir + 1);
    } else {
        z = (2.0 * ns - ir) * 2.0 / (3.0 * ns);
        s = sqrt((1.0 - z) * (1.0 + z));
        nph[p] = 4 * nside;
        half[p] = ((ir - nside) % 2 == 0) ? 1 : 0;
        startN[p] = ncap + (int64_t)(ir - nside) * 4 * nside;
        const int irs = 4 * nside - ir;  // south partner
        startS[p] = ncap + (int64_t)(irs - nside) * 4 * nside;
    }
    cth[p] = z;
    sth[p] = s;
}

// (A, B) per (l, m) for l >= m+2; entries l = m, m+1 are unused (0).
__global__ void k_plan_coef(int lmax, const int64_t *mofs, double2 *coef) {
    const int m = blockIdx.y;
    const int64_t base = mofs[m];
    for (int l = m + blockIdx.x * blockDim.x + threadIdx.x; l <= lmax; l += gridDim.x * blockDim.x) {
        double2 c = make_double2(0.0, 0.0);
        if (l >= m + 2) {
            double l2 = (double)l * l, m2 = (double)m * m, lm1 = l - 1.0;
            c.x = sqrt((4.0 * l2 - 1.0) / (l2 - m2));
            c.y = sqrt((4.0 * l2 - 1.0) * (lm1 * lm1 - m2) / ((l2 - m2) * (4.0 * lm1 * lm1 - 1.0)));
        }
        coef[base + l - m] = c;
    }
}

// lambda_mm at every ring pair, as mantissa * 2^(800 * scale), scale <= 0.
__global__ void k_plan_lmm(int mmax, int npairs, const double *sth, double *lmm, int *lmm_scale) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const double s = sth[p];
    double v = 0.28209479177387814;  // 1 / sqrt(4 pi)
    int sc = 0;
    lmm[p] = v;
    lmm_scale[p] = 0;
    for (int m = 1; m <= mmax; ++m) {
        v *= -s * sqrt((2.0 * m + 1.0) / (2.0 * m));
        if (fabs(v) < GLG_TWO_M400) {
            v *= GLG_TWO_P800;
            sc -= 1;
        }
        lmm[(int64_t)m * npairs + p] = v;
        lmm_scale[(int64_t)m * npairs + p] = sc;
    }
}

// tw[ofs_i + t] = exp(i pi t / (4 i)) for t < 8 i (= omega_{2n}^t, n = 4 i).
__global__ void k_plan_tw(int nside, const int64_t *tw_ofs, double2 *tw) {
    const int i = blockIdx.y + 1;
    const int n2 = 8 * i;
    const int64_t base = tw_ofs[i];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n2; t += gridDim.x * blockDim.x) {
        double s, c;
        sincospi((double)t / (4.0 * i), &s, &c);
        tw[base + t] = make_double2(c, s);
    }
}

// ------------------------------------------------------------------- host

static void factor_ring(int n, int *radix, int *nst) {
    // DIF order: radix-4 passes first, then 2, then odd primes ascending.
    int k = 0;
    while (n % 4 == 0 && n > 1) { radix[k++] = 4; n /= 4; }
    while (n % 2 == 0) { radix[k++] = 2; n /= 2; }
    for (int p = 3; n > 1; p += 2) {
        while (n % p == 0) { radix[k++] = p; n /= p; }
        if ((int64_t)p * p > n && n > 1) { radix[k++] = n; n = 1; }
    }
    *nst = k;
}

// Device bytes a plan's P_lm table may take (glg_set_plm_table_budget).
static std::atomic<size_t> g_plm_budget{(size_t)160 << 30};

extern "C" int glg_set_plm_table_budget(size_t bytes) {
    g_plm_budget.store(bytes);
    return GLG_OK;
}

// Failure injection for tests: the n-th plan allocation from now (1 = the
// next) reports cudaErrorMemoryAllocation without calling cudaMalloc.
static std::atomic<int> g_fail_alloc{0};

extern "C" int glg_test_fail_plan_alloc(int nth) {
    GLG_REQUIRE(nth >= 0, "glg_test_fail_plan_alloc: negative count");
    g_fail_alloc.store(nth);
    return GLG_OK;
}

template <typename T>
static int dalloc(glg_plan *P, T **ptr, size_t count) {
    const int f = g_fail_alloc.load();
    if (f > 0 && g_fail_alloc.fetch_sub(1) == 1) {
        *ptr = nullptr;
        return glg_cuda_status(cudaErrorMemoryAllocation, "glg_plan_create: cudaMalloc (injected failure)");
    }
    cudaError_t e = cudaMalloc((void **)ptr, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_plan_create: cudaMalloc");
    P->bytes += sizeof(T) * count;
    return GLG_OK;
}

extern "C" void glg_plan_destroy(glg_plan *P) {
    if (!P) return;
    void *ptrs[] = {P->cth,   P->sth,       P->nph,     P->half,   P->startN, P->startS,
                    P->mofs,  P->coef,      P->lmm,     P->lmm_scale, P->fft_radix,
                    P->fft_nst, P->tw_ofs,  P->tw,      P->cth32,  P->tw32,   P->coef32,
                    P->goff,  P->seeds,     P->lstart,  P->tfirst, P->bucket_pairs, P->chirp_ofs,
                    P->chirp, P->pos_ofs, P->pos16,   P->blu_ofs, P->blu_M,  P->blu_H,  P->twM,
                    P->plm,   P->twMp, P->twp, P->plm_spin[0][0], P->plm_spin[0][1], P->plm_spin[1][0],
                    P->plm_spin[1][1], P->tfirst_spin[0], P->tfirst_spin[1]};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    delete[] P->bucket_pairs_host;
    delete P;
}

// ------------------------------------------------------- fast-form tables

// FP64 recurrence per (m, ring pair) that records, for every group of 16 l
// values starting at l0 = m + 16 j, the seed pair (mu_s0, mu_s0+1) with
// s0 = max(l0, ls), ls the first l whose |lambda| reaches 2^-40 and
// mu_l = lambda_l / d_l the group-scaled values of the fast contraction (d = 1
// at l0 and l0 + 1, d_l = B_l d_{l-2} after).  The FP32 recurrence of the
// fast contraction restarts from these seeds, so its rounding error never
// accumulates over more than 16 steps.
__global__ void k_plan_seeds(int lmax, int npairs, const double *__restrict__ cth,
                             const int64_t *__restrict__ mofs, const double2 *__restrict__ coef,
                             const double *__restrict__ lmm, const int *__restrict__ lmm_scale,
                             const int64_t *__restrict__ goff, float2 *__restrict__ seeds,
                             int64_t sstride, int *__restrict__ lstart) {
    const int m = blockIdx.y;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const double x = cth[p];
    const double thr = 9.094947017729282e-13;  // 2^-40, ~1e-12 of the O(1) normalised lambda
    double l0 = 0.0, l1 = lmm[(int64_t)m * npairs + p];
    int sc = lmm_scale[(int64_t)m * npairs + p];
    int ls = -1;
    float sx = 0.f;
    int64_t pend = -1;  // group whose seed still needs lambda_{s0+1}
    const int64_t base = mofs[m];
    const int64_t g0 = goff[m];
    double d1 = 1.0, d2 = 1.0;  // d_{l-1}, d_{l-2} of the group scale
    for (int l = m; l <= lmax; ++l) {
        const double dl = (l - m) % GLG_GROUP < 2 ? 1.0 : coef[base + l - m].y * d2;
        d2 = d1;
        d1 = dl;
        if (l > m) {
            double nl;
            if (l == m + 1) {
                nl = sqrt(2.0 * m + 3.0) * x * l1;
            } else {
                const double2 ab = coef[base + l - m];
                nl = ab.x * (x * l1) - ab.y * l0;
            }
            l0 = l1;
            l1 = nl;
            if (sc < 0 && fabs(nl) > GLG_TWO_P400) {
                l0 *= GLG_TWO_M800;
                l1 *= GLG_TWO_M800;
                sc += 1;
            }
        }
        const double lam = sc == 0 ? l1 : 0.0;
        if (ls < 0 && fabs(lam) >= thr) ls = l;
        const double tv = lam / dl;  // the seed value mu_l
        const int j = (l - m) / GLG_GROUP;
        const int lg0 = m + j * GLG_GROUP;
        if (pend >= 0) {  // l == s0 + 1 of the pending seed
            if (seeds) seeds[pend * sstride + p] = make_float2(sx, (float)tv);
            pend = -1;
        }
        if (ls >= 0 && l == (lg0 > ls ? lg0 : ls)) {
            sx = (float)tv;
            pend = g0 + j;
        }
        const bool group_end = ((l - m) % GLG_GROUP == GLG_GROUP - 1) || l == lmax;
        if (group_end && ls < 0 && seeds) seeds[(g0 + j) * sstride + p] = make_float2(0.f, 0.f);
    }
    if (pend >= 0 && seeds) seeds[pend * sstride + p] = make_float2(sx, 0.f);
    lstart[(int64_t)m * npairs + p] = ls < 0 ? lmax + 1 : ls;
}

__global__ void k_plan_f32(int64_t n, const double2 *__restrict__ src, float2 *__restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = make_float2((float)src[i].x, (float)src[i].y);
}

// FP64 -> FP32 (hi, lo) pairs: hi = fl32(v), lo = fl32(v - hi).
__device__ __forceinline__ float2 split_f64(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}

__global__ void k_plan_cth32(int n, const double *__restrict__ src, float2 *__restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = split_f64(src[i]);
}

// Coefficients of the fast contraction's scaled recurrence, per (l, m):
// (alpha_hi, alpha_lo, d, 0), d the group scale (1 at the group's first two
// l, d_l = B_l d_{l-2} after) and alpha_l = A_l d_{l-1} / d_l (0 at the
// group's first two l, which are seeds).  One thread per (m, group).
__global__ void k_plan_coef32(int lmax, const int64_t *__restrict__ mofs, const double2 *__restrict__ coef,
                              float4 *__restrict__ dst) {
    const int m = blockIdx.y;
    const int G = (lmax - m + GLG_GROUP) / GLG_GROUP;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= G) return;
    const int64_t base = mofs[m];
    double d1 = 1.0, d2 = 1.0;  // d_{l-1}, d_{l-2}
    for (int t = 0; t < GLG_GROUP; ++t) {
        const int l = m + j * GLG_GROUP + t;
        if (l > lmax) break;
        if (t < 2) {
            dst[base + l - m] = make_float4(0.f, 0.f, 1.f, 0.f);
            continue;
        }
        const double2 ab = coef[base + l - m];
        const double d = ab.y * d2;
        const float2 al = split_f64(ab.x * d1 / d);
        dst[base + l - m] = make_float4(al.x, al.y, (float)d, 0.f);
        d2 = d1;
        d1 = d;
    }
}

// P_lm table of the fast contraction: for every (m, group g, ring tile) one
// tile [l quad q][ring pair r][4] of mu_l = lambda_l / d_l, l = m + 16 g +
// 4 q + i, d_l the FP32 group scale of coef32 (the B operand carries d_l),
// from the FP64 extended-range recurrence rounded once to FP32; zero beyond
// lmax and for ring pairs beyond the last.  One thread per (m, ring pair of
// a whole tile), float4 stores coalesced across the tile's ring pairs.
__global__ void k_plan_plm(int lmax, int npairs, int ntiles, const double *__restrict__ cth,
                           const int64_t *__restrict__ mofs, const double2 *__restrict__ coef,
                           const double *__restrict__ lmm, const int *__restrict__ lmm_scale,
                           const int64_t *__restrict__ goff, const float4 *__restrict__ coef32,
                           float4 *__restrict__ plm) {
    const int m = blockIdx.y;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;  // < ntiles * 128
    const bool live = p < npairs;
    const int pp = live ? p : npairs - 1;
    const double x = cth[pp];
    double l0 = 0.0, l1 = lmm[(int64_t)m * npairs + pp];
    int sc = lmm_scale[(int64_t)m * npairs + pp];
    const int64_t base = mofs[m];
    const int G = (lmax - m + GLG_GROUP) / GLG_GROUP;
    float4 q4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float *qv = &q4.x;
    for (int t = 0; t < G * GLG_GROUP; ++t) {
        const int l = m + t;
        float v = 0.f;
        if (l <= lmax) {
            if (l > m) {
                double nl;
                if (l == m + 1) {
                    nl = sqrt(2.0 * m + 3.0) * x * l1;
                } else {
                    const double2 ab = coef[base + t];
                    nl = ab.x * (x * l1) - ab.y * l0;
                }
                l0 = l1;
                l1 = nl;
                if (sc < 0 && fabs(nl) > GLG_TWO_P400) {
                    l0 *= GLG_TWO_M800;
                    l1 *= GLG_TWO_M800;
                    sc += 1;
                }
            }
            if (live && sc == 0) v = (float)(l1 / (double)coef32[base + t].z);
        }
        qv[t & 3] = v;
        if ((t & 3) == 3) {
            const int64_t gt = (goff[m] + t / GLG_GROUP) * ntiles + p / 128;
            plm[(gt * 4 + (t % GLG_GROUP) / 4) * 128 + p % 128] = q4;
        }
    }
}

// Spin-s tables (s = 1, 2) of the fast spin synthesis: the same tiles as
// k_plan_plm holding lambda^+_l / d_l (tab_p) and lambda^-_l / d_l (tab_m),
// with lambda^+- from lambda_l and lambda_{l-1} of the FP64 extended-range
// recurrence (the formulas of the FP64 spin synthesis, evaluated in FP64 and
// rounded once):
//   dlam = (l x lam_l - sqrt((2l+1)/(2l-1) (l^2 - m^2)) lam_{l-1}) / sin,
//   s = 1: lambda^+ = -dlam / N, lambda^- = m lam / (sin N),  N = sqrt(l(l+1));
//   s = 2: lambda^+ = (-2 cot dlam + (2 m^2 / sin^2 - l(l+1)) lam) / N,
//          lambda^- = (2 m / sin)(cot lam - dlam) / N,        N = sqrt((l-1)l(l+1)(l+2)).
// One block of 128 threads per (ring tile, m); the block also writes the
// tile's first group where |lambda^+| or |lambda^-| reaches 2^-40 (the
// number of groups when none does).
__global__ void k_plan_plm_spin(int lmax, int npairs, int ntiles, int spin, const double *__restrict__ cth,
                                const double *__restrict__ sth, const int64_t *__restrict__ mofs,
                                const double2 *__restrict__ coef, const double *__restrict__ lmm,
                                const int *__restrict__ lmm_scale, const int64_t *__restrict__ goff,
                                const float4 *__restrict__ coef32, float4 *__restrict__ tab_p,
                                float4 *__restrict__ tab_m, int *__restrict__ tfirst) {
    const int m = blockIdx.y;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;  // < ntiles * 128
    const bool live = p < npairs;
    const int pp = live ? p : npairs - 1;
    const double x = cth[pp], isn = 1.0 / sth[pp], cot = x * isn, fm = m;
    double l0 = 0.0, l1 = lmm[(int64_t)m * npairs + pp];
    int sc = lmm_scale[(int64_t)m * npairs + pp];
    const int64_t base = mofs[m];
    const int G = (lmax - m + GLG_GROUP) / GLG_GROUP;
    int first = G;
    float4 qp = make_float4(0.f, 0.f, 0.f, 0.f), qm = qp;
    float *vp = &qp.x, *vm = &qm.x;
    for (int t = 0; t < G * GLG_GROUP; ++t) {
        const int l = m + t;
        float a = 0.f, b = 0.f;
        if (l <= lmax) {
            if (l > m) {
                double nl;
                if (l == m + 1) {
                    nl = sqrt(2.0 * m + 3.0) * x * l1;
                } else {
                    const double2 ab = coef[base + t];
                    nl = ab.x * (x * l1) - ab.y * l0;
                }
                l0 = l1;
                l1 = nl;
                if (sc < 0 && fabs(nl) > GLG_TWO_P400) {
                    l0 *= GLG_TWO_M800;
                    l1 *= GLG_TWO_M800;
                    sc += 1;
                }
            }
            if (live && sc == 0 && l >= spin) {
                const double fl = l, lam = l1, lprev = l > m ? l0 : 0.0;
                const double dlam =
                    (fl * x * lam - sqrt((2.0 * fl + 1.0) / (2.0 * fl - 1.0) * (fl * fl - fm * fm)) * lprev) * isn;
                double lp, lmv;
                if (spin == 1) {
                    const double nrm = 1.0 / sqrt(fl * (fl + 1.0));
                    lp = -dlam * nrm;
                    lmv = fm * lam * isn * nrm;
                } else {
                    const double nrm = 1.0 / sqrt((fl - 1.0) * fl * (fl + 1.0) * (fl + 2.0));
                    lp = (-2.0 * cot * dlam + (2.0 * fm * fm * isn * isn - fl * (fl + 1.0)) * lam) * nrm;
                    lmv = (2.0 * fm * isn) * (cot * lam - dlam) * nrm;
                }
                if (first == G && fmax(fabs(lp), fabs(lmv)) >= 0x1p-40) first = t / GLG_GROUP;
                const double d = (double)coef32[base + t].z;
                a = (float)(lp / d);
                b = (float)(lmv / d);
            }
        }
        vp[t & 3] = a;
        vm[t & 3] = b;
        if ((t & 3) == 3) {
            const int64_t gt = (goff[m] + t / GLG_GROUP) * ntiles + p / 128;
            const int64_t ix = (gt * 4 + (t % GLG_GROUP) / 4) * 128 + p % 128;
            tab_p[ix] = qp;
            tab_m[ix] = qm;
        }
    }
    __shared__ int fmin_s;
    if (threadIdx.x == 0) fmin_s = G;
    __syncthreads();
    atomicMin(&fmin_s, first);
    __syncthreads();
    if (threadIdx.x == 0) tfirst[(int64_t)m * ntiles + blockIdx.x] = fmin_s;
}

// Output position of frequency k after in-place DIF passes with `radix`.
static int dif_pos_host(const int *radix, int nst, int n, int k) {
    int pos = 0, span = n;
    for (int s = 0; s < nst; ++s) {
        span /= radix[s];
        pos += (k % radix[s]) * span;
        k /= radix[s];
    }
    return pos;
}

// In-place iterative radix-2 FFT, sum_t x_t e^{-2 pi i k t / M}, FP64 (host).
static void fft_pow2_host(std::vector<std::complex<double>> &x) {
    const size_t M = x.size();
    for (size_t i = 1, j = 0; i < M; ++i) {
        size_t bit = M >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(x[i], x[j]);
    }
    for (size_t len = 2; len <= M; len <<= 1) {
        const double ang = -2.0 * M_PI / (double)len;
        for (size_t i = 0; i < M; i += len)
            for (size_t k = 0; k < len / 2; ++k) {
                const std::complex<double> w(cos(ang * (double)k), sin(ang * (double)k));
                const std::complex<double> u = x[i + k], v = x[i + k + len / 2] * w;
                x[i + k] = u + v;
                x[i + k + len / 2] = u - v;
            }
    }
}

// First 16-l group of every (m, ring tile) that holds a lambda above
// 2^-40 on some ring of the tile: tfirst = (min_p lstart[m][p] - m) / 16
// (G when no ring of the tile reaches it).  Every group before it is zero
// on the whole tile, so the contraction skips it.
__global__ void k_plan_tfirst(int lmax, int npairs, int ntiles, const int *__restrict__ lstart,
                              int *__restrict__ tfirst) {
    const int m = blockIdx.y, tile = blockIdx.x;
    const int p = tile * 128 + threadIdx.x;
    int ls = p < npairs ? lstart[(int64_t)m * npairs + p] : lmax + 1;
    for (int o = 16; o > 0; o >>= 1) ls = min(ls, __shfl_xor_sync(0xffffffffu, ls, o));
    __shared__ int wmin[4];
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = ls;
    __syncthreads();
    if (threadIdx.x == 0) {
        const int v = min(min(wmin[0], wmin[1]), min(wmin[2], wmin[3]));
        const int G = (lmax - m + GLG_GROUP) / GLG_GROUP;
        tfirst[(int64_t)m * ntiles + tile] = v > lmax ? G : (v - m) / GLG_GROUP;
    }
}

// Host-built tables of the FP32 ring FFTs: launch buckets, DIF output
// orders, the Bluestein chirps c_k = e^{i pi k^2 / n} and chirp spectra
// H = DFT_M(h), h_t = e^{-i pi t^2 / n} for |t| < n (indices mod M), stored
// in the DIF output order of M.
size_t glg_ring32_smem(int kind, int n_or_M, int threads, bool fold) {
    if (kind == 3) return 2 * (size_t)threads * sizeof(float2);  // the buffer is in global memory
    const size_t zs = (size_t)glg_zsize(n_or_M);
    size_t slots = zs + 2 * (size_t)threads + glg_zi(n_or_M / 2) + 1;
    if (kind != 1 && fold) slots += zs;
    return slots * sizeof(float2);
}

// Bluestein length of a ring of n pixels: the smallest power of two M >=
// 2n - 1, or 3 * 2^k when that is smaller and the staged kernels take it
// (M = 6144 or 12288, the ring pair's two rows of Legendre sums fitting the
// transform buffer): 13.5 % fewer butterflies over the rings of nside 2048.
static int blu_length(int n, int mmax) {
    int M = 1;
    while (M < 2 * n - 1) M <<= 1;
    int M3 = 3;
    while (M3 < 2 * n - 1) M3 <<= 1;
    const size_t rows = 2 * (((size_t)(mmax + 2) * 8 + 15) & ~(size_t)15);
    if (M3 < M && (M3 == 6144 || M3 == 12288) && rows <= sizeof(float2) * (size_t)glg_zsize(M3)) return M3;
    return M;
}

// Radix passes of a Bluestein length in the device's order: 3 * 2^k lengths
// start with their radix-3 pass, then as glg_fft32_radices.
static int blu_radices(int M, int *r) {
    if (M % 3 != 0) return glg_fft32_radices(M, r);
    r[0] = 3;
    return 1 + glg_fft32_radices(M / 3, r + 1);
}

// Forward DFT (e^{-2 pi i k t / M}) of a length 2^k or 3 * 2^k, FP64 (host).
static void fft_host(std::vector<std::complex<double>> &x) {
    const size_t M = x.size();
    if (M % 3 != 0) {
        fft_pow2_host(x);
        return;
    }
    const size_t Q = M / 3;
    std::vector<std::complex<double>> y[3];
    for (int r = 0; r < 3; ++r) {
        y[r].resize(Q);
        for (size_t j = 0; j < Q; ++j) y[r][j] = x[3 * j + r];
        fft_pow2_host(y[r]);
    }
    for (size_t k = 0; k < M; ++k) {
        std::complex<double> acc = y[0][k % Q];
        for (int r = 1; r < 3; ++r) {
            const double ang = -2.0 * M_PI * (double)(((int64_t)r * (int64_t)k) % (int64_t)M) / (double)M;
            acc += std::complex<double>(cos(ang), sin(ang)) * y[r][k % Q];
        }
        x[k] = acc;
    }
}

static int build_fft32_tables(glg_plan *P, cudaStream_t st) {
    const int nside = P->nside, mmax = P->mmax;
    std::vector<int64_t> pos_ofs(nside + 2, 0), blu_ofs(nside + 1, -1), chirp_ofs(nside + 1, -1);
    std::vector<int> blu_M(nside + 1, 0);
    int64_t nblu = 0, nchirp = 0;
    int Mmax = 4;
    for (int i = 1; i <= nside; ++i) {
        int r[GLG_MAX_FFT_STAGES];
        pos_ofs[i + 1] = pos_ofs[i] + 4LL * i;
        if (glg_fft32_radices(4 * i, r) < 0) {
            const int M = blu_length(4 * i, mmax);
            blu_M[i] = M;
            blu_ofs[i] = nblu;
            nblu += M;
            chirp_ofs[i] = nchirp;
            nchirp += 4 * i;
            if (M > Mmax && M % 3 != 0) Mmax = M;
        }
    }
    std::vector<uint16_t> pos16(pos_ofs[nside + 1]);
    for (int i = 1; i <= nside; ++i) {
        int r[GLG_MAX_FFT_STAGES];
        const int ns = glg_fft32_radices(4 * i, r);
        if (ns < 0) continue;
        for (int k = 0; k < 4 * i; ++k) pos16[pos_ofs[i] + k] = (uint16_t)dif_pos_host(r, ns, 4 * i, k);
    }
    std::vector<float2> H((size_t)(nblu > 0 ? nblu : 1)), chirp((size_t)(nchirp > 0 ? nchirp : 1));
    // chirps and chirp spectra of every Bluestein length, ring lengths dealt
    // out to the host's threads (each writes its own table ranges)
    auto chirp_tables = [&](int i) {
        const int M = blu_M[i];
        if (!M) return;
        const int n = 4 * i;
        std::vector<std::complex<double>> h(M, 0.0);
        for (int t = 0; t < n; ++t) {
            const double ph = M_PI * (double)(((int64_t)t * t) % (2LL * n)) / n;
            chirp[chirp_ofs[i] + t] = make_float2((float)cos(ph), (float)sin(ph));
            h[t] = std::complex<double>(cos(ph), -sin(ph));
            if (t > 0) h[M - t] = h[t];
        }
        fft_host(h);
        int mr[GLG_MAX_FFT_STAGES];
        const int mns = blu_radices(M, mr);
        for (int k = 0; k < M; ++k) {
            const int q = dif_pos_host(mr, mns, M, k);
            H[blu_ofs[i] + q] = make_float2((float)h[k].real(), (float)h[k].imag());
        }
    };
    {
        const unsigned hw = std::thread::hardware_concurrency();
        const int nth = nside < 256 ? 1 : (int)(hw > 0 ? (hw < 32 ? hw : 32) : 4);
        std::atomic<int> next{1};
        std::vector<std::thread> pool;
        for (int t = 1; t < nth; ++t)
            pool.emplace_back([&] {
                for (int i = next++; i <= nside; i = next++) chirp_tables(i);
            });
        for (int i = next++; i <= nside; i = next++) chirp_tables(i);
        for (auto &th : pool) th.join();
    }
    std::vector<float2> twM(Mmax / 2 + 1);
    for (int t = 0; t <= Mmax / 2; ++t)
        twM[t] = make_float2((float)cos(2.0 * M_PI * t / Mmax), (float)sin(2.0 * M_PI * t / Mmax));
    // padded half tables of every power of two up to the largest transform
    int lgmax = 3;
    while ((1 << lgmax) < Mmax || (1 << lgmax) < 4 * nside) ++lgmax;
    std::vector<float2> twp;
    for (int lg = 0; lg < 16; ++lg) P->twp_ofs[lg] = P->twp3_ofs[lg] = -1;
    for (int lg = 3; lg <= lgmax && lg < 16; ++lg) {
        const int L = 1 << lg;
        P->twp_ofs[lg] = (int64_t)twp.size();
        twp.resize(twp.size() + ((glg_zsize(L / 2 + 1) + 1) & ~1) + 2, make_float2(0.f, 0.f));  // 16-byte sizes, slack
        for (int t = 0; t <= L / 2; ++t)
            twp[P->twp_ofs[lg] + glg_zi(t)] = make_float2((float)cos(2.0 * M_PI * t / L), (float)sin(2.0 * M_PI * t / L));
    }
    for (int k = 0; k < 16; ++k) {  // the 3 * 2^k Bluestein lengths in use
        const int L = 3 << k;
        if (std::find(blu_M.begin(), blu_M.end(), L) == blu_M.end()) continue;
        P->twp3_ofs[k] = (int64_t)twp.size();
        twp.resize(twp.size() + ((glg_zsize(L / 2 + 1) + 1) & ~1) + 2, make_float2(0.f, 0.f));
        for (int t = 0; t <= L / 2; ++t)
            twp[P->twp3_ofs[k] + glg_zi(t)] = make_float2((float)cos(2.0 * M_PI * t / L), (float)sin(2.0 * M_PI * t / L));
    }
    std::vector<float2> twMp;  // padded copy for class 3 (read from global memory)
    if (Mmax > 16384) {
        twMp.assign((size_t)glg_zsize(Mmax / 2 + 1), make_float2(0.f, 0.f));
        for (int t = 0; t <= Mmax / 2; ++t) twMp[glg_zi(t)] = twM[t];
    }

    // buckets: Bluestein rings by M, mixed-radix rings by (next power of two
    // of n, power-of-two n or not, whether m folds onto the ring); largest
    // work first
    struct Key {
        int kind, size, fold;
        bool operator<(const Key &o) const {
            if (size != o.size) return size > o.size;
            if (kind != o.kind) return kind > o.kind;
            return fold > o.fold;
        }
    };
    std::map<Key, std::vector<int>> groups;
    for (int p = 0; p < P->npairs; ++p) {
        const int i = p + 1 < nside ? p + 1 : nside;
        const int n = 4 * i;
        if (blu_M[i]) {  // class 3 when the transform buffer exceeds shared memory
            groups[{blu_M[i] > 16384 ? 3 : 1, blu_M[i], 0}].push_back(p);
        } else {
            int nb = 1;
            while (nb < n) nb <<= 1;
            // power-of-two equatorial rings get their own launch (kind 2): a
            // kernel built for radices 16/8/4/2 only needs half the registers
            // (a lone polar ring of that length stays with its size class)
            groups[{nb == n && i == nside ? 2 : 0, nb, n <= mmax ? 1 : 0}].push_back(p);
        }
    }
    GLG_REQUIRE((int)groups.size() <= GLG_MAX_RING_BUCKETS, "fast ring FFT: too many ring buckets");
    std::vector<int> bpairs;
    P->nbuckets = 0;
    for (auto &kv : groups) {
        glg_ring_bucket &b = P->buckets[P->nbuckets++];
        b.kind = kv.first.kind;
        b.size = kv.first.size;
        b.fold = kv.first.fold;
        b.threads = kv.first.size >= 4096 ? 512 : 256;  // until glg_autotune_fast picks
        b.smem = glg_ring32_smem(b.kind, kv.first.size, b.threads, kv.first.fold != 0);
        b.ms = 0.f;
        b.count = (int)kv.second.size();
        b.first = (int64_t)bpairs.size();
        bpairs.insert(bpairs.end(), kv.second.begin(), kv.second.end());
    }
    P->blu_Mmax = Mmax;
    int rc;
    if ((rc = dalloc(P, &P->bucket_pairs, bpairs.size())) ||
        (rc = dalloc(P, &P->pos_ofs, pos_ofs.size())) || (rc = dalloc(P, &P->pos16, pos16.size())) ||
        (rc = dalloc(P, &P->blu_ofs, blu_ofs.size())) || (rc = dalloc(P, &P->blu_M, blu_M.size())) ||
        (rc = dalloc(P, &P->blu_H, H.size())) || (rc = dalloc(P, &P->twM, twM.size())) ||
        (!twMp.empty() && (rc = dalloc(P, &P->twMp, twMp.size()))) || (rc = dalloc(P, &P->twp, twp.size())) ||
        (rc = dalloc(P, &P->chirp_ofs, chirp_ofs.size())) || (rc = dalloc(P, &P->chirp, chirp.size())))
        return rc;
    cudaError_t e = cudaSuccess;
    auto up = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    up(P->bucket_pairs, bpairs.data(), sizeof(int) * bpairs.size());
    delete[] P->bucket_pairs_host;
    P->bucket_pairs_host = new int[bpairs.size() ? bpairs.size() : 1];
    std::copy(bpairs.begin(), bpairs.end(), P->bucket_pairs_host);
    up(P->pos_ofs, pos_ofs.data(), sizeof(int64_t) * pos_ofs.size());
    up(P->pos16, pos16.data(), sizeof(uint16_t) * pos16.size());
    up(P->blu_ofs, blu_ofs.data(), sizeof(int64_t) * blu_ofs.size());
    up(P->blu_M, blu_M.data(), sizeof(int) * blu_M.size());
    up(P->blu_H, H.data(), sizeof(float2) * H.size());
    up(P->twM, twM.data(), sizeof(float2) * twM.size());
    if (!twMp.empty()) up(P->twMp, twMp.data(), sizeof(float2) * twMp.size());
    up(P->twp, twp.data(), sizeof(float2) * twp.size());
    up(P->chirp_ofs, chirp_ofs.data(), sizeof(int64_t) * chirp_ofs.size());
    up(P->chirp, chirp.data(), sizeof(float2) * chirp.size());
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // host vectors go out of scope
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_plan_prepare_fast: FFT tables");
    return GLG_OK;
}

int glg_plan_prepare_fast(glg_plan *P, cudaStream_t st) {
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (P->fast_ready) return GLG_OK;
    const int np = P->npairs, lmax = P->lmax;
    std::vector<int64_t> goff(lmax + 2, 0);
    for (int m = 0; m <= lmax; ++m)
        goff[m + 1] = goff[m] + (lmax - m + 1 + GLG_GROUP - 1) / GLG_GROUP;
    P->ngroups = goff[lmax + 1];
    const int64_t ntw = 4LL * P->nside * (P->nside + 1);
    // seed rows padded to whole 128-pair tiles, and 16 spare coefficient
    // entries: the contraction copies whole tiles / whole groups per stage
    P->seed_stride = (int64_t)((np + 127) / 128) * 128;
    int rc;
    if ((rc = dalloc(P, &P->cth32, np)) || (rc = dalloc(P, &P->tw32, ntw)) ||
        (rc = dalloc(P, &P->coef32, P->nalm + GLG_GROUP)) || (rc = dalloc(P, &P->goff, lmax + 2)) ||
        (rc = dalloc(P, &P->lstart, (size_t)(lmax + 1) * np)) ||
        (rc = dalloc(P, &P->tfirst, (size_t)(lmax + 1) * ((np + 127) / 128))))
        return rc;
    // the P_lm table when it fits the budget and the free device memory
    // (with 4 GiB to spare), else the seeds of the FP32 recurrence
    const int ntiles = (np + 127) / 128;
    const size_t tbytes = (size_t)GLG_PLM_TILE_BYTES * (size_t)P->ngroups * ntiles;
    size_t free_b = 0, total_b = 0;
    bool table = tbytes <= g_plm_budget.load() && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
                 tbytes + ((size_t)4 << 30) <= free_b;
    if (table && cudaMalloc((void **)&P->plm, tbytes) != cudaSuccess) {
        cudaGetLastError();  // not enough room after all: recurrence path
        P->plm = nullptr;
        table = false;
    }
    if (table) {
        P->plm_bytes = tbytes;
        P->bytes += tbytes;
    } else if ((rc = dalloc(P, &P->seeds, (size_t)P->ngroups * P->seed_stride))) {
        return rc;
    }
    cudaError_t e = cudaMemcpyAsync(P->goff, goff.data(), sizeof(int64_t) * goff.size(),
                                    cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !table)
        e = cudaMemsetAsync(P->seeds, 0, sizeof(float2) * (size_t)P->ngroups * P->seed_stride, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(P->coef32, 0, sizeof(float4) * (size_t)(P->nalm + GLG_GROUP), st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_plan_prepare_fast: upload");
    k_plan_cth32<<<(np + 255) / 256, 256, 0, st>>>(np, P->cth, P->cth32);
    k_plan_f32<<<1024, 256, 0, st>>>(ntw, P->tw, P->tw32);
    k_plan_coef32<<<dim3((lmax / GLG_GROUP + 128) / 128, lmax + 1), 128, 0, st>>>(lmax, P->mofs, P->coef,
                                                                                 P->coef32);
    dim3 gs((np + 127) / 128, lmax + 1);
    k_plan_seeds<<<gs, 128, 0, st>>>(lmax, np, P->cth, P->mofs, P->coef, P->lmm, P->lmm_scale,
                                     P->goff, P->seeds, P->seed_stride, P->lstart);
    k_plan_tfirst<<<dim3((np + 127) / 128, lmax + 1), 128, 0, st>>>(lmax, np, (np + 127) / 128, P->lstart,
                                                                   P->tfirst);
    if (table)
        k_plan_plm<<<dim3(ntiles, lmax + 1), 128, 0, st>>>(lmax, np, ntiles, P->cth, P->mofs, P->coef, P->lmm,
                                                          P->lmm_scale, P->goff, P->coef32, P->plm);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_plan_prepare_fast");
    if ((rc = build_fft32_tables(P, st))) return rc;
    P->fast_ready = true;
    return GLG_OK;
}

int glg_plan_prepare_spin(glg_plan *P, int spin, cudaStream_t st) {
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    GLG_REQUIRE(spin == 1 || spin == 2, "fast spin synthesis: spin must be 1 or 2");
    GLG_REQUIRE(P->fast_ready, "fast spin synthesis: fast tables not prepared");
    const int k = spin - 1;
    if (P->plm_spin[k][0]) return GLG_OK;
    const int np = P->npairs, lmax = P->lmax, ntiles = (np + 127) / 128;
    const size_t tbytes = (size_t)GLG_PLM_TILE_BYTES * (size_t)P->ngroups * ntiles;
    const size_t used = P->plm_bytes + P->spin_bytes;
    size_t free_b = 0, total_b = 0;
    if (used + 2 * tbytes > g_plm_budget.load() || cudaMemGetInfo(&free_b, &total_b) != cudaSuccess ||
        2 * tbytes + ((size_t)4 << 30) > free_b) {
        cudaGetLastError();
        char msg[200];
        snprintf(msg, sizeof msg,
                 "fast spin synthesis: its lambda+- tables (2 x %.2f GB) do not fit the table budget or the "
                 "free device memory; use the FP64 form", (double)tbytes / 1e9);
        glg_set_error(msg);
        return GLG_ERR_UNSUPPORTED;
    }
    int rc;
    if ((rc = dalloc(P, &P->plm_spin[k][0], tbytes / sizeof(float4))) ||
        (rc = dalloc(P, &P->plm_spin[k][1], tbytes / sizeof(float4))) ||
        (rc = dalloc(P, &P->tfirst_spin[k], (size_t)(lmax + 1) * ntiles)))
        return rc;
    P->spin_bytes += 2 * tbytes;
    k_plan_plm_spin<<<dim3(ntiles, lmax + 1), 128, 0, st>>>(lmax, np, ntiles, spin, P->cth, P->sth, P->mofs,
                                                           P->coef, P->lmm, P->lmm_scale, P->goff, P->coef32,
                                                           P->plm_spin[k][0], P->plm_spin[k][1],
                                                           P->tfirst_spin[k]);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_plan_prepare_spin");
    return GLG_OK;
}

extern "C" int glg_plan_create(int nside, int lmax, void *stream, glg_plan **out) {
    GLG_REQUIRE(out != nullptr, "glg_plan_create: null output pointer");
    *out = nullptr;
    GLG_REQUIRE(nside >= 1 && nside <= 8192 && (nside & (nside - 1)) == 0,
                "glg_plan_create: nside must be a power of two in [1, 8192]");
    GLG_REQUIRE(lmax >= 0 && lmax <= 16384, "glg_plan_create: lmax must be in [0, 16384]");
    cudaStream_t st = (cudaStream_t)stream;
    glg_plan *P = new glg_plan();
    P->nside = nside;
    P->lmax = lmax;
    P->mmax = lmax;
    P->nrings = 4 * nside - 1;
    P->npairs = 2 * nside;
    P->npix = 12LL * nside * nside;
    P->nalm = glg_nalm(lmax);
    cudaGetDevice(&P->device);
    int rc;
#define ALLOC(ptr, n)                          \
    if ((rc = dalloc(P, &P->ptr, (n))) != 0) { \
        glg_plan_destroy(P);                   \
        return rc;                             \
    }
    const int np = P->npairs;
    ALLOC(cth, np); ALLOC(sth, np); ALLOC(nph, np); ALLOC(half, np);
    ALLOC(startN, np); ALLOC(startS, np);
    ALLOC(mofs, lmax + 2);
    ALLOC(coef, P->nalm);
    ALLOC(lmm, (size_t)(lmax + 1) * np);
    ALLOC(lmm_scale, (size_t)(lmax + 1) * np);
    ALLOC(fft_radix, (size_t)(nside + 1) * GLG_MAX_FFT_STAGES);
    ALLOC(fft_nst, nside + 1);
    ALLOC(tw_ofs, nside + 2);
    std::vector<int64_t> tw_ofs(nside + 2, 0);
    for (int i = 1; i <= nside; ++i) tw_ofs[i + 1] = tw_ofs[i] + 8LL * i;
    ALLOC(tw, tw_ofs[nside + 1]);
#undef ALLOC

    std::vector<int64_t> mofs(lmax + 2);
    for (int m = 0; m <= lmax + 1; ++m) mofs[m] = (int64_t)m * (2 * lmax + 3 - m) / 2;
    std::vector<int> radix((size_t)(nside + 1) * GLG_MAX_FFT_STAGES, 0), nst(nside + 1, 0);
    for (int i = 1; i <= nside; ++i)
        factor_ring(4 * i, &radix[(size_t)i * GLG_MAX_FFT_STAGES], &nst[i]);

    cudaError_t e;
    if ((e = cudaMemcpyAsync(P->mofs, mofs.data(), sizeof(int64_t) * mofs.size(),
                             cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(P->fft_radix, radix.data(), sizeof(int) * radix.size(),
                             cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(P->fft_nst, nst.data(), sizeof(int) * nst.size(),
                             cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(P->tw_ofs, tw_ofs.data(), sizeof(int64_t) * tw_ofs.size(),
                             cudaMemcpyHostToDevice, st)) != cudaSuccess) {
        glg_plan_destroy(P);
        return glg_cuda_status(e, "glg_plan_create: upload");
    }
    k_plan_rings<<<(np + 127) / 128, 128, 0, st>>>(nside, np, P->cth, P->sth, P->nph, P->half,
                                                  P->startN, P->startS);
    dim3 gc((lmax + 256) / 256 < 64 ? (lmax + 256) / 256 : 64, lmax + 1);
    k_plan_coef<<<gc, 256, 0, st>>>(lmax, P->mofs, P->coef);
    k_plan_lmm<<<(np + 127) / 128, 128, 0, st>>>(lmax, np, P->sth, P->lmm, P->lmm_scale);
    dim3 gt(8, nside);
    k_plan_tw<<<gt, 256, 0, st>>>(nside, P->tw_ofs, P->tw);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // host vectors go out of scope
    if (e != cudaSuccess) {
        glg_plan_destroy(P);
        return glg_cuda_status(e, "glg_plan_create: table kernels");
    }
    *out = P;
    return GLG_OK;
}

extern "C" size_t glg_plan_device_bytes(const glg_plan *P) { return P ? P->bytes : 0; }

extern "C" int glg_plan_has_plm_table(const glg_plan *P) { return P && P->plm ? 1 : 0; }

extern "C" int glg_plan_info(const glg_plan *P, int *nside, int *lmax, int *nrings, int64_t *npix,
                             int64_t *nalm) {
    GLG_REQUIRE(P != nullptr, "glg_plan_info: null plan");
    if (nside) *nside = P->nside;
    if (lmax) *lmax = P->lmax;
    if (nrings) *nrings = P->nrings;
    if (npix) *npix = P->npix;
    if (nalm) *nalm = P->nalm;
    return GLG_OK;
}
