// Plan creation: HEALPix ring geometry, FP64 Legendre recurrence tables and
// ring-FFT tables, built on the device once per (nside, lmax).
//
// Geometry follows the HEALPix RING scheme (Gorski et al. 2005), which the
// reference reaches through healpy/healpix (glass/healpix.py:38-78,
// :293-310).
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>
#include <string>
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

template <typename T>
static int dalloc(glg_plan *P, T **ptr, size_t count) {
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
                    P->goff,  P->seeds,     P->lstart};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    delete P;
}

// ------------------------------------------------------- fast-form tables

// FP64 recurrence per (m, ring pair) that records, for every group of 16 l
// values starting at l0 = m + 16 j, the seed pair (lambda_s0, lambda_s0+1)
// with s0 = max(l0, ls), ls the first l whose |lambda| reaches 2^-100.  The
// FP32 recurrence of the fast contraction restarts from these seeds, so its
// rounding error never accumulates over more than 16 steps.
__global__ void k_plan_seeds(int lmax, int npairs, const double *__restrict__ cth,
                             const int64_t *__restrict__ mofs, const double2 *__restrict__ coef,
                             const double *__restrict__ lmm, const int *__restrict__ lmm_scale,
                             const int64_t *__restrict__ goff, float2 *__restrict__ seeds,
                             int *__restrict__ lstart) {
    const int m = blockIdx.y;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const double x = cth[p];
    const double thr = 7.888609052210118e-31;  // 2^-100
    double l0 = 0.0, l1 = lmm[(int64_t)m * npairs + p];
    int sc = lmm_scale[(int64_t)m * npairs + p];
    int ls = -1;
    float sx = 0.f;
    int64_t pend = -1;  // group whose seed still needs lambda_{s0+1}
    const int64_t base = mofs[m];
    const int64_t g0 = goff[m];
    for (int l = m; l <= lmax; ++l) {
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
        const double tv = sc == 0 ? l1 : 0.0;
        if (ls < 0 && fabs(tv) >= thr) ls = l;
        const int j = (l - m) / GLG_GROUP;
        const int lg0 = m + j * GLG_GROUP;
        if (pend >= 0) {  // l == s0 + 1 of the pending seed
            seeds[pend * npairs + p] = make_float2(sx, (float)tv);
            pend = -1;
        }
        if (ls >= 0 && l == (lg0 > ls ? lg0 : ls)) {
            sx = (float)tv;
            pend = g0 + j;
        }
        const bool group_end = ((l - m) % GLG_GROUP == GLG_GROUP - 1) || l == lmax;
        if (group_end && ls < 0) seeds[(g0 + j) * npairs + p] = make_float2(0.f, 0.f);
    }
    if (pend >= 0) seeds[pend * npairs + p] = make_float2(sx, 0.f);
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

__global__ void k_plan_coef32(int64_t n, const double2 *__restrict__ src, float4 *__restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 a = split_f64(src[i].x), b = split_f64(src[i].y);
        dst[i] = make_float4(a.x, a.y, b.x, b.y);
    }
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
    int rc;
    if ((rc = dalloc(P, &P->cth32, np)) || (rc = dalloc(P, &P->tw32, ntw)) ||
        (rc = dalloc(P, &P->coef32, P->nalm)) || (rc = dalloc(P, &P->goff, lmax + 2)) ||
        (rc = dalloc(P, &P->seeds, (size_t)P->ngroups * np)) ||
        (rc = dalloc(P, &P->lstart, (size_t)(lmax + 1) * np)))
        return rc;
    cudaError_t e = cudaMemcpyAsync(P->goff, goff.data(), sizeof(int64_t) * goff.size(),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_plan_prepare_fast: upload");
    k_plan_cth32<<<(np + 255) / 256, 256, 0, st>>>(np, P->cth, P->cth32);
    k_plan_f32<<<1024, 256, 0, st>>>(ntw, P->tw, P->tw32);
    k_plan_coef32<<<1024, 256, 0, st>>>(P->nalm, P->coef, P->coef32);
    dim3 gs((np + 127) / 128, lmax + 1);
    k_plan_seeds<<<gs, 128, 0, st>>>(lmax, np, P->cth, P->mofs, P->coef, P->lmm, P->lmm_scale,
                                     P->goff, P->seeds, P->lstart);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_plan_prepare_fast");
    P->fast_ready = true;
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
