// Internal definitions shared by the glass_gb300 CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/glass_gb300.h"

// ------------------------------------------------------------------ errors

void glg_set_error(const std::string &msg);
int glg_cuda_status(cudaError_t err, const char *where);

#define GLG_CHECK_LAUNCH(where)                                   \
    do {                                                          \
        cudaError_t e_ = cudaGetLastError();                      \
        if (e_ != cudaSuccess) return glg_cuda_status(e_, where); \
    } while (0)

#define GLG_REQUIRE(cond, msg)          \
    do {                                \
        if (!(cond)) {                  \
            glg_set_error(msg);         \
            return GLG_ERR_INVALID;     \
        }                               \
    } while (0)

// ------------------------------------------------------------------ timing

// Scope around one kernel launch: counts the launch and, when timing is
// enabled (glg_timing_enable), brackets it with CUDA events on its stream.
struct glg_launch_scope {
    glg_launch_scope(const char *name, cudaStream_t st);
    ~glg_launch_scope();
    const char *name;
    cudaStream_t st;
    cudaEvent_t ev0, ev1;
    bool timed;
};

#define GLG_LAUNCH_SCOPE(name, st) glg_launch_scope glg_scope_(name, st)

// -------------------------------------------------------------------- plan

// Maximum number of radix passes of one ring FFT (n = 4 i <= 4 * 8192).
#define GLG_MAX_FFT_STAGES 20

// One launch of the FP32 ring FFTs: `count` ring pairs of one kind
// (0: mixed radix, 1: Bluestein) starting at bucket_pairs[first].
#define GLG_MAX_RING_BUCKETS 40
struct glg_ring_bucket {
    int kind, count, threads;
    int size, fold;  // transform length bucket (n rounded up, or M) and fold scratch
    int64_t first;
    size_t smem;
    float ms;  // autotuner's time of one launch at `threads` (0 before tuning)
};

struct glg_plan {
    int nside, lmax, mmax;
    int nrings, npairs;
    int64_t npix, nalm;
    int device;
    size_t bytes;

    // ring pairs p = 0 .. npairs-1: north ring p (0-based), south ring
    // nrings-1-p; the last pair is the equator (north == south).
    double *cth, *sth;       // [npairs]
    int *nph;                // [npairs]
    int *half;               // [npairs] 1: phi0 = pi / nph, 0: phi0 = 0
    int64_t *startN, *startS;  // [npairs] first pixel of each ring

    // Legendre recurrence lambda_l = A (x lambda_{l-1}) - B lambda_{l-2}
    int64_t *mofs;           // [mmax+2] HEALPix index of (l=m, m)
    double2 *coef;           // [nalm] (A, B) at mofs[m] + l - m (l >= m+2)
    double *lmm;             // [mmax+1][npairs] lambda_mm mantissa
    int *lmm_scale;          // [mmax+1][npairs] exponent scale (x 2^800)

    // ring FFTs for lengths n = 4 i, i = 1 .. nside
    int *fft_radix;          // [nside+1][GLG_MAX_FFT_STAGES]
    int *fft_nst;            // [nside+1]
    int64_t *tw_ofs;         // [nside+1] offset of the table of length i
    double2 *tw;             // tw[ofs_i + t] = exp(i pi t / (4 i)), t < 8 i

    // fast-form tables (built on first use by glg_plan_prepare_fast)
    bool fast_ready;
    float2 *cth32;           // [npairs] cos theta as FP32 (hi, lo)
    float2 *tw32;            // FP32 copy of tw
    float4 *coef32;          // [nalm] (alpha_hi, alpha_lo, d, 0) of the scaled FP32 recurrence
    int64_t *goff;           // [mmax+2] first 16-l group of m: sum_{m'<m} ceil((lmax-m'+1)/16)
    int64_t ngroups;         // total groups
    float2 *seeds;           // [ngroups][seed_stride] (lambda_s0, lambda_s0+1) per group
    int64_t seed_stride;     // npairs rounded up to whole 128-pair tiles
    int *lstart;             // [mmax+1][npairs] first l with |lambda| >= 2^-40
    int *tfirst;             // [mmax+1][ntiles] first group with a lambda >= 2^-40 in the tile
    // P_lm table (built instead of the seeds when it fits the table budget):
    // per (group, ring tile) one 8 KB tile [l quad][128 ring pairs][4] of
    // mu_l = lambda_l / d_l as FP32 (the FP64 recurrence rounded once), zero
    // beyond lmax and beyond the last ring pair.  nullptr: recurrence path.
    float4 *plm;
    size_t plm_bytes;
    // Spin tables of the fast spin-s synthesis (s = 1, 2; index s - 1), built
    // on first use by glg_plan_prepare_spin: the same tile layout holding
    // lambda^+_l / d_l and lambda^-_l / d_l, and per (m, ring tile) the first
    // group where either reaches 2^-40 on some ring of the tile.
    float4 *plm_spin[2][2];  // [s - 1][+ / -]
    int *tfirst_spin[2];
    size_t spin_bytes;

    // FP32 ring FFTs of the fast form.  Class 0: ring lengths whose prime
    // factors are all <= 13 (mixed-radix DIF, output order from pos16).
    // Class 1: lengths with a larger prime factor (Bluestein with a
    // power-of-two length M >= 2n - 1 and a precomputed chirp spectrum).
    // Ring pairs are launched in size buckets (one launch per bucket, every
    // map of the call in the same grid), each with its own shared memory.
    int nbuckets;
    glg_ring_bucket buckets[GLG_MAX_RING_BUCKETS];
    int *bucket_pairs;       // ring pairs of all buckets, bucket after bucket (ascending in each)
    int *bucket_pairs_host;  // host copy (new[]), to launch a bucket over a ring-pair range
    int64_t *pos_ofs;        // [nside+1] offset of the output permutation of n = 4 i
    uint16_t *pos16;         // DIF output position of every frequency, per length
    int64_t *blu_ofs;        // [nside+1] offset of the chirp spectrum of n = 4 i (-1: class 0)
    int *blu_M;              // [nside+1] Bluestein length M of n = 4 i (0: class 0)
    float2 *blu_H;           // chirp spectra, each in DIF output order of its M
    int64_t *chirp_ofs;      // [nside+1] offset of the chirp of n = 4 i (-1: class 0)
    float2 *chirp;           // exp(i pi k^2 / n), k < n, per Bluestein length
    int blu_Mmax;
    float2 *twM;             // [blu_Mmax / 2 + 1] exp(2 pi i t / blu_Mmax)
    float2 *twMp;            // the same, padded (twMp[glg_zi(t)]), when blu_Mmax > 16384 (class 3)
    // padded half twiddle tables e^{2 pi i t / L}, t <= L / 2, at twp[twp_ofs[log2 L] + glg_zi(t)]
    // for L = 2^3 .. the largest power-of-two transform of the plan (each 16-byte aligned,
    // copied whole into shared memory by the staged kernels)
    float2 *twp;
    int64_t twp_ofs[16];
    int64_t twp3_ofs[16];  // the same for lengths 3 * 2^k (Bluestein lengths 6144, 12288), by k
};

// Radix passes of an FP32 ring FFT of length n (DIF order: 16s, then one 8,
// 4 or 2, then the odd primes up to 13).  Returns the pass count, or -1 when
// n has a prime factor above 13 (those lengths go through Bluestein).
__host__ __device__ inline int glg_fft32_radices(int n, int *r) {
    int k = 0;
    while (n % 16 == 0) { r[k++] = 16; n /= 16; }
    if (n % 8 == 0) { r[k++] = 8; n /= 8; }
    else if (n % 4 == 0) { r[k++] = 4; n /= 4; }
    else if (n % 2 == 0) { r[k++] = 2; n /= 2; }
    for (int p = 3; p <= 13; p += 2)
        while (n % p == 0) { r[k++] = p; n /= p; }
    return n == 1 ? k : -1;
}

// Shared-memory index of complex element e of a ring FFT buffer: a spare
// slot per 16 and per 256 values makes the strides 1, 16 and 256 of the
// radix-16 passes and of the digit-reversed output gather odd in slots, so
// none of them repeats a bank within a warp.
__host__ __device__ inline int glg_zi(int e) { return e + (e >> 4) + (e >> 8); }

// Slots of a padded buffer of `cnt` complex values.
__host__ __device__ inline int glg_zsize(int cnt) { return glg_zi(cnt - 1) + 1; }

// Dynamic shared memory of one ring FFT block: the padded transform buffer
// of length n (kind 0) or M (kind 1), a second padded buffer for the south
// ring's fold (kind 0 with n <= mmax), 2 x threads partial sums and the half
// twiddle table (padded like the buffers).
size_t glg_ring32_smem(int kind, int n_or_M, int threads, bool fold);

// l values per group of the fast Legendre contraction (8 even + 8 odd)
#define GLG_GROUP 16

int glg_plan_prepare_fast(glg_plan *P, cudaStream_t st);
// The spin-s tables of the fast spin synthesis (after glg_plan_prepare_fast);
// GLG_ERR_UNSUPPORTED when they do not fit the table budget and free memory.
int glg_plan_prepare_spin(glg_plan *P, int spin, cudaStream_t st);

// Bytes of one group's P_lm tile (128 ring pairs x 16 l, FP32).
#define GLG_PLM_TILE_BYTES (128 * GLG_GROUP * 4)

// ---------------------------------------------------------- device helpers

__host__ __device__ inline int64_t glg_nalm(int lmax) {
    return (int64_t)(lmax + 1) * (lmax + 2) / 2;
}

// extended-range constants of the Legendre recurrence
#define GLG_TWO_P800 6.668014432879854e+240
#define GLG_TWO_M800 1.499696813895631e-241
#define GLG_TWO_P400 2.5822498780869086e+120
#define GLG_TWO_M400 3.872591914849318e-121

// Launch helpers implemented in the individual .cu files.
int glg_launch_leg_syn(const glg_plan *P, const double2 *alm, int nmaps, double2 *F,
                       cudaStream_t st);
int glg_launch_leg_syn_spin(const glg_plan *P, const double2 *elm, const double2 *blm, int spin,
                            double2 *F, cudaStream_t st);
// FP64 ring FFTs; gbuf: glg_ring64_gbuf_bytes(P) bytes of device memory for
// rings too long for shared memory (nside > 2048), else unused (may be null).
size_t glg_ring64_gbuf_bytes(const glg_plan *P);
int glg_launch_ring_syn(const glg_plan *P, const double2 *F, int nmaps, double *maps,
                        const glg_epilogue *epi, void *gbuf, cudaStream_t st);
int glg_launch_ring_ana(const glg_plan *P, const double *maps, int nmaps, double2 *G, void *gbuf,
                        cudaStream_t st);
int glg_launch_leg_ana(const glg_plan *P, const double2 *G, int nmaps, double2 *alm, int accumulate,
                       cudaStream_t st);
// Tail refinement list of the fast form (in the fast workspace): hdr[0]
// entries appended by the ring FFTs, hdr[1] entries already refined; items
// (map, ring, pixel within the ring).
// Device-resident epilogue of a graph-captured fast synthesis (the kernels
// read it at run time instead of taking it as a launch argument, so one
// captured graph serves every epilogue); filled on the host by
// glg_epilogue_dev_fill and copied to the device before each replay.
#define GLG_EPI_MAPS 40
struct glg_epi_dev {
    int kind[GLG_EPI_MAPS];
    float hvar[GLG_EPI_MAPS], lam[GLG_EPI_MAPS], thr[GLG_EPI_MAPS];  // var / 2, shift, tail threshold
    double hv64[GLG_EPI_MAPS], lam64[GLG_EPI_MAPS];                  // the same in FP64 (tail refinement)
};
struct glg_refine_list {
    int *hdr;
    int cap;
    int4 *items;
    float2 *gz;  // nside > 2048: the global transform buffers of Bluestein class 3
    int *err;    // the call's status word (a staged copy's bounded wait that ran out), or null
    const glg_epi_dev *edev = nullptr;  // device epilogue (graph-captured calls), or null
};
// Fill a device-epilogue image in host memory from a host epilogue.
void glg_epi_dev_fill(const glg_epilogue *epi, int nmaps, glg_epi_dev *out);
// Class-3 buffers: GLG_RING_GSLOTS slices of glg_zsize(Mmax) complex values.
#define GLG_RING_GSLOTS 304
// Bytes of the class-3 buffers for a plan of this nside (0 when nside <= 2048).
size_t glg_ring_gz_bytes(int nside);
int glg_launch_ring_syn_f32(const glg_plan *P, const float2 *F, float2 *Ft, int nmaps, float *maps,
                            const glg_epilogue *epi, const glg_refine_list *rl, cudaStream_t st);
// FP64 recomputation of the listed pixels (no launch when no map of the call
// qualifies); returns GLG_OK.
bool glg_refine_wanted(const glg_epilogue *epi, int nmaps);
int glg_launch_refine(const glg_plan *P, const float2 *Ft, int nmaps, float *maps, const glg_epilogue *epi,
                      const glg_refine_list &rl, cudaStream_t st);
// One size bucket of the FP32 ring FFTs from transposed sums Ft, with
// `threads` per block (0: the bucket's own), no epilogue (autotuning).
int glg_launch_ring_bucket_f32(const glg_plan *P, int bucket, int threads, const float2 *Ft, int nmaps,
                               float *maps, float2 *gz, cudaStream_t st);
size_t glg_leg_tc_pack_bytes(const glg_plan *P, int nmaps);
// Ring tiles (128 ring pairs each) of one tensor-core contraction launch, the
// unit counter it draws from (slot in the status block) and whether the B
// tiles are packed first (once per call).
struct glg_tile_run {
    int tile0, ntiles, slot;
    bool pack;
};
int glg_launch_leg_tc(const glg_plan *P, const float2 *alm, int nmaps, float *bpack, float2 *F,
                      int *err, const glg_tile_run &run, cudaStream_t st);
// The same with the B columns of maps nsplit .. nmaps-1 taken from alm2
// (map nsplit + k is alm2 row k) and the lambda tiles and first groups of a
// spin table instead of the plan's P_lm table (table/tfirst null: the plan's).
int glg_launch_leg_tc_ex(const glg_plan *P, const float2 *alm, const float2 *alm2, int nsplit, int nmaps,
                         float *bpack, float2 *F, int *err, const glg_tile_run &run, const float4 *table,
                         const int *tfirst, cudaStream_t st);
// Ring FFTs of the ring pairs [p0, p1) only (transpose included; F null:
// Ft already holds the sums [map][ring][m]).
int glg_launch_ring_syn_f32_range(const glg_plan *P, const float2 *F, float2 *Ft, int nmaps, float *maps,
                                  const glg_epilogue *epi, int p0, int p1, const glg_refine_list *rl,
                                  cudaStream_t st);

// Fast-form workspace: [status ints | B pack | F (float2 [map][m][ring])]
// The status block holds the error word and, from byte 64, the unit
// counters of the contraction launches of one call.
#define GLG_WS_STATUS_BYTES 256
#define GLG_WS_UNIT_COUNTERS 24
