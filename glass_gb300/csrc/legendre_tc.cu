// Fast form of the Legendre sums: a shells-batched contraction on the
// sm_103a tensor cores (tcgen05, split-precision TF32: 3xTF32).
//
// For one ring tile (128 ring pairs, one per TMEM lane) and one m:
//   D_E[p][n] = sum_{l-m even} lambda_lm(x_p) B[l][n],
//   D_O[p][n] = sum_{l-m odd}  lambda_lm(x_p) B[l][n],
// with n = 2 * map + (0: re, 1: im); north F = D_E + D_O, south F = D_E - D_O
// (lambda_lm(-x) = (-1)^(l+m) lambda_lm(x)).  This is the work healpy does
// inside alm2map (glass/healpix.py:71, called from glass/fields.py:429).
//
// lambda is generated on the fly in FP32 by producer warps, restarting every
// 16 l (one "group") from seeds computed once per plan by an FP64
// recurrence, split into TF32 hi + lo parts and written straight into tensor
// memory as the MMA's A operand (hi and lo = v - hi both rounded to nearest
// TF32).  Within a group the producers carry the
// scaled mu_l = lambda_l / d_l, d = 1 at the group's first two l and
// d_l = B_l d_{l-2} after, whose recurrence mu_l = alpha_l x mu_{l-1} -
// mu_{l-2} (alpha_l = A_l d_{l-1} / d_l) has no second product; the alm
// carry d_l instead (B[l][n] = a_lm d_l), so the sums are unchanged.  B (the alm, split the same way), the
// group's seeds and its recurrence coefficients are streamed into shared
// memory with 1-D bulk copies.  Each group issues, per parity,
//   D += A_hi B_lo + A_lo B_hi + A_hi B_hi   (M = 128, N = 2 * maps, K = 8),
// with both lo parts rounded to nearest TF32 (3 passes; a fourth, A_lo B_lo,
// of relative size 2^-22, changed the benchmark's worst lognormal shell by
// 6e-10 and cost 2.4 ms, 9 % of the contraction).
//
// Groups before the first one where some ring of the tile has |lambda| >=
// 2^-40 are zero on the whole tile and are skipped (the dense algorithmic
// count is still the one reported).
//
// Pipeline.  The groups of a (tile, m) unit are processed in chunks of
// CH = 3 groups, one per producer warp set, from the unit's highest l down
// (smallest terms first into the running sums); a chunk is the unit of every
// hand-off: its lambda goes to one of two TMEM chunk slots, its B tiles come
// in one bulk copy into one of NBC shared-memory chunk slots, its MMAs
// accumulate into one of two TMEM accumulator sets, and one commit per chunk
// both frees the lambda slot and hands the accumulator to the drain warps,
// which add it into FP32 sums in shared memory (round to nearest).  The
// tensor core's FP32 accumulation rounds toward zero, so accumulating only a
// chunk in TMEM bounds that drift, and within a chunk the small cross terms
// of its groups go first and the large A_hi B_hi terms last, so the
// truncation never falls on a small term added to a large sum.
//
// Warp roles (640 threads): warps 0-11 produce lambda (set k = warps
// 4k..4k+3 makes group k of every chunk), warps 12-15 drain the
// accumulators and store F, warps 16 and 19 issue the even- and odd-parity
// MMAs, warp 17 streams B and warp 18 streams seeds / coefficients through
// a ring of NSEED group slots.
// Every wait is bounded; on time-out the kernel records GLG_ERR_TIMEOUT in
// *err, retires its outstanding MMAs and copies, frees its tensor memory and
// returns.
#include <cuda_runtime.h>

#include <type_traits>

#include "glg_internal.cuh"
#include "tc_ptx.cuh"

using namespace glg_tc;

namespace {

constexpr int CH = 3;             // groups per chunk = producer warp sets
constexpr int NSEED = 16;         // slots of the seed / coefficient ring (groups)
constexpr int NU = 8;             // slots of the unit ring
constexpr int NCONSUMERS = 19;    // warps that read the unit ring (all but the seed streamer)
constexpr int TMEM_COLS = 512;
constexpr int THREADS = 20 * 32;
constexpr uint32_t WAIT_LIMIT = 1u << 22;
// The tensor core's FP32 accumulation rounds toward zero, so every chunk sum
// comes out smaller in magnitude than the exact one, on average by the same
// fraction: measured on GB300 as a regression slope of -7.0e-8 (+-0.2e-8)
// of these sums against FP64 ones, the same at nside 512 and 2048, for every
// map, with the recurrence or the P_lm table.  The packed alm are scaled up by
// that fraction (k_pack_b adds it to the lo part, whose TF32 precision is
// 2^-22 of the value: a scaling of 7e-8 is carried to ~3%), which removes the
// systematic part -- a bias that the lognormal transform amplifies at its
// largest pixels -- and leaves the random part of the rounding.  (Scaling the
// FP32 sums themselves cannot do it: 7e-8 is below one FP32 ulp, so
// v + 7e-8 v rounds to v plus one whole ulp.)
constexpr float ACC_BIAS = 7.0e-8f;
constexpr int W_DRAIN = 12, W_MMA = 16, W_LOAD = 17, W_SEED = 18, W_MMA2 = 19;
// Table path: the drain warps keep the running sums of their lane (2 N FP32
// values) in registers instead of shared memory, which leaves that room to
// P_lm tile slots.  The kernel is launched with LEG_REGS registers a thread;
// each warpgroup then sets its own share (setmaxnreg): the producers and the
// MMA / streaming warps give up registers, the drain warpgroup takes them.
// The shares add up to the launch's total: 3 x 128 x 72 + 128 x 216 +
// 128 x 48 = 61440 = 640 x 96 (a larger sum would wait forever).
constexpr int LEG_REGS = 96, REGS_PROD = 72, REGS_DRAIN = 216, REGS_MISC = 48;
static_assert(3 * 128 * REGS_PROD + 128 * REGS_DRAIN + 128 * REGS_MISC <= THREADS * LEG_REGS,
              "warpgroup register shares above the launch's registers");
static_assert(W_DRAIN == 12 && W_MMA == 16 && THREADS == 5 * 128, "warpgroups: 3 producer, drain, the rest");
template <uint32_t R>
__device__ __forceinline__ void regs_inc() {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(R));
}
template <uint32_t R>
__device__ __forceinline__ void regs_dec() {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(R));
}
static_assert(W_DRAIN == 4 * CH, "one producer warp set per group of a chunk");
static_assert((W_MMA2 + 1) * 32 == THREADS, "one warp per role after the producers and drains");
static_assert(W_MMA % 4 != W_MMA2 % 4, "the two MMA-issuing warps on different SM sub-partitions");

struct LegTcArgs {
    int npairs, nrings, lmax, nmaps, ntiles;
    int tile0, nrun;  // this launch's ring tiles: tile0 .. tile0 + nrun - 1
    int64_t nunits;   // nrun x (lmax + 1): unit u is tile tile0 + u % nrun of m unit_m(u / nrun)
    const float2 *cth32;
    const float4 *coef32;
    const int64_t *mofs;
    const int64_t *goff;
    const float2 *seeds;
    int64_t seed_stride;
    const int *lstart;
    const int *tfirst;  // [m][tile] first group holding a lambda >= 2^-40
    const float4 *plm;  // P_lm tiles (table path)
    const unsigned char *bpack;
    float2 *F;  // [map][m][ring]
    int *err;
    unsigned long long *ucount;  // next unit to hand out (zeroed before the launch)
    uint32_t wait_limit;         // polls of one pipeline wait before it gives up
    int stall;                   // test hook: the B streamer issues no copies
};

// Test hook (glg_test_stall_contraction): with `stall` set, the B streamer
// never fills its slots, so the MMA warps' waits for B run out after
// `wait_limit` polls and the kernel takes its time-out path.
uint32_t g_test_wait_limit = 0;
int g_test_stall = 0;

__device__ __forceinline__ uint32_t tf32_rna(float x) {
    // round the magnitude to 10 fraction bits, ties away from zero (the
    // rounding of cvt.rna.tf32.f32), as an integer add and mask
    return (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u;
}

// One step mu_l = alpha (x mu_{l-1}) - mu_{l-2} in FP32 with the products
// and the coefficient carried as (hi, lo) pairs (error-free transformations
// with fma): only the FP32 state itself is rounded, which keeps the 16-step
// runs between FP64 seeds near 1e-7.  c = (alpha_hi, alpha_lo, d, 0).  The
// __f*_rn forms keep the compiler from fusing the rounded products away.
__device__ __forceinline__ float rec_step(const float4 c, const float2 x, float lm1, float lm2) {
    const float yh = __fmul_rn(x.x, lm1);
    float ye = fmaf(x.x, lm1, -yh);
    ye = fmaf(x.y, lm1, ye);
    const float ph = __fmul_rn(c.x, yh);
    float pe = fmaf(c.x, yh, -ph);
    pe = fmaf(c.x, ye, pe);
    pe = fmaf(c.y, yh, pe);
    return __fadd_rn(__fsub_rn(ph, lm2), pe);
}

// Chunk k of a (tile, m) unit, groups [c0, c1): chunks are taken from the
// top of the unit down (k = 0 ends at the unit's last group), so the running
// sums receive the small high-l terms first and the large ones last -- the
// rounding of each drained addition is relative to a running sum that is
// still small for most of the unit.  The partial chunk, if any, is the last.
__device__ __forceinline__ void chunk_range(int k, int gf, int G, int &c0, int &c1) {
    c1 = G - CH * k;
    c0 = c1 - CH > gf ? c1 - CH : gf;
}

// m of the mi-th group of units: ascending m, so the longest units (most l
// groups) go first and the shortest last, which keeps the persistent grid's
// tail short (0.25 ms less over the 8 launches of a host-output call than
// alternating long and short units).
__device__ __forceinline__ int unit_m(int64_t mi) {
    return (int)mi;
}

// B chunk slots in shared memory: as many as fit beside the accumulators and
// the seed ring (up to 6), so the alm of a chunk are requested several chunks
// before the MMAs that read them.
// Recurrence path: as many B chunk slots as fit beside the accumulators and
// the seed ring (up to 6).  Table path: 2 B chunk slots for wide N (their
// tiles mostly come from L2, where the ring tiles of one m share them) and
// the room left to P_lm tile slots, up to 12 (8 KB each): the tiles come
// from HBM, and the copies in flight per SM bound the bandwidth.
template <int N, bool T>
constexpr int nbc_slots() {
    if constexpr (T) return N <= 32 ? 4 : 2;
    constexpr int room = (226 * 1024 - 512 * (2 * N + 4) - NSEED * 1280 - 1024) / (CH * 128 * N);
    return room > 6 ? 6 : room;
}
template <int N>
constexpr int plm_slots() {  // the running sums are in the drain warps' registers
    constexpr int room = (226 * 1024 - nbc_slots<N, true>() * CH * 128 * N - 2048) / GLG_PLM_TILE_BYTES;
    return room > 24 ? 24 : room;
}

struct SeedSlot {
    float2 seed[128];        // seeds of the group's 128 ring pairs
    float4 coef[GLG_GROUP];  // (alpha_hi, alpha_lo, d, 0) of l = l0 .. l0+15
};
struct PlmSlot {
    float4 v[4][128];  // P_lm tile: [l quad][ring pair], 4 l per float4
};

// T: lambda from the plan's P_lm table (tiles streamed into a ring of
// shared-memory slots), else from the FP32 recurrence and its seeds.
template <int N, bool T>
struct Smem {
    static constexpr uint32_t BBYTES = 128 * N;  // one group: 4 tiles of N x 8 tf32
    static constexpr int NBC = nbc_slots<N, T>();
    static constexpr int NS = T ? plm_slots<N>() : NSEED;  // group slots of the lambda source
    static_assert(!T || NS >= 2 * CH, "P_lm slots for two chunks");
    static_assert(NBC >= 2, "at least two B chunk slots");
    struct BSlot {
        unsigned char b[CH * BBYTES];
    } bs[NBC];
    std::conditional_t<T, PlmSlot, SeedSlot> sd[NS];
    static constexpr int ACC_LD = 2 * N + 4;  // floats per lane row (odd count of float4)
    float acc[T ? 1 : 128][T ? 4 : ACC_LD];  // FP32 sums of drained chunks, [lane][column] (recurrence path)
    uint64_t full_a[2], cdone[2], empty_d[2];
    uint64_t full_b[NBC], bempty[NBC];
    uint64_t sfull[NS], sempty[NS];
    uint64_t ufull[NU], uempty[NU];
    int64_t unit[NU];  // units handed out to this CTA, in order
    uint64_t drain;
    uint32_t tmem_base;
    int abort;
};

template <int N, bool T>
__device__ __forceinline__ void leg_tc_body(const LegTcArgs &a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    using SM = Smem<N, T>;
    SM &S = *reinterpret_cast<SM *>(smem_raw);
    constexpr int NBC = SM::NBC;
    constexpr int NS = SM::NS;
    constexpr uint32_t BBYTES = SM::BBYTES;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr uint32_t IDESC = idesc_tf32(128, N);
    constexpr uint32_t SEED_TX = 128 * 8 + GLG_GROUP * 16;
    constexpr int A_COL0 = 4 * N;     // D sets at [0, 2N) and [2N, 4N)
    constexpr int A_SLOT = CH * 32;   // columns of one lambda chunk slot
    static_assert(A_COL0 + 2 * A_SLOT <= TMEM_COLS, "tensor memory budget");

    if (threadIdx.x == 0) {
        for (int k = 0; k < 2; ++k) {
            mbar_init(&S.full_a[k], 4 * CH);  // every producer warp, once per chunk
            mbar_init(&S.cdone[k], 2);        // the chunk's commits (E and O warps)
            mbar_init(&S.empty_d[k], 4);      // the drain warps
        }
        for (int k = 0; k < NBC; ++k) {
            mbar_init(&S.full_b[k], 1);
            mbar_init(&S.bempty[k], 2);
        }
        for (int q = 0; q < NS; ++q) {
            mbar_init(&S.sfull[q], 1);
            mbar_init(&S.sempty[q], 4);
        }
        for (int q = 0; q < NU; ++q) {
            mbar_init(&S.ufull[q], 1);
            mbar_init(&S.uempty[q], NCONSUMERS);
        }
        mbar_init(&S.drain, 2);
        S.abort = 0;
        fence_barrier_init();
    }
    if constexpr (!T)
        for (int i = threadIdx.x; i < 128 * SM::ACC_LD; i += THREADS) (&S.acc[0][0])[i] = 0.f;
    if (warp == 0) {
        tmem_alloc(&S.tmem_base, TMEM_COLS);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tb = S.tmem_base;
    volatile int *abort_flag = &S.abort;
    auto fail = [&]() {
        *abort_flag = 1;
        atomicExch(a.err, GLG_ERR_TIMEOUT);
    };
    auto wait = [&](uint64_t *bar, uint32_t parity) -> bool {
        for (uint32_t i = 0; i < a.wait_limit; ++i) {
            if (mbar_try_wait(bar, parity)) return true;
            if (*abort_flag) return false;
        }
        fail();
        return false;
    };
    // Units are handed out dynamically from a global counter (by the seed
    // streamer, which runs ahead), so that all CTAs work on neighbouring units
    // at any time: the ring tiles of one m then read the same B tiles within
    // a short window and find them in L2.  next_unit() returns the i-th unit
    // of this CTA (>= nunits: no more) and frees its ring slot; called by all
    // lanes of a warp (whole_warp) or by lane 0 alone.
    auto next_unit = [&](uint32_t i, int64_t &u, bool whole_warp) -> bool {
        const uint32_t q = i % NU;
        if (!wait(&S.ufull[q], (i / NU) & 1u)) return false;
        u = *reinterpret_cast<volatile int64_t *>(&S.unit[q]);
        if (whole_warp) __syncwarp();
        if (lane == 0) mbar_arrive(&S.uempty[q]);
        return true;
    };
    const int lmax = a.lmax;
    const uint32_t lane_base = (uint32_t)((warp & 3) << 5) << 16;
    const int r = ((warp & 3) << 5) + lane;  // TMEM lane = ring pair in tile

    // Chunk cc (counted over the CTA's units) uses lambda slot and
    // accumulator set cc & 1 (phase cc >> 1 of their barriers) and B slot
    // cc % NBC (phase cc / NBC); group gg (counted likewise) uses seed slot
    // gg % NSEED (phase gg / NSEED).
    if (warp < W_DRAIN) {
        // ------------------------------------------------ lambda producers
        if constexpr (T) regs_dec<REGS_PROD>();
        const int set = warp >> 2;
        uint32_t cc = 0, gc = 0;
        bool ok = true;
        for (uint32_t ui = 0; ok; ++ui) {
            int64_t u;
            if (!next_unit(ui, u, true)) { ok = false; break; }
            if (u >= a.nunits) break;
            const int tile = a.tile0 + (int)(u % a.nrun);
            const int m = unit_m(u / a.nrun);
            const int G = (lmax - m + GLG_GROUP) / GLG_GROUP;
            const int p = tile * 128 + r;
            const bool live = p < a.npairs;
            const int pp = live ? p : a.npairs - 1;
            const float2 x = a.cth32[pp];
            const int ls = live ? a.lstart[(int64_t)m * a.npairs + pp] : lmax + 1;
            const int gf = a.tfirst[(int64_t)m * a.ntiles + tile];
            for (int kc = 0, nch = (G - gf + CH - 1) / CH; kc < nch; ++kc, ++cc) {
                int g0, g1;
                chunk_range(kc, gf, G, g0, g1);
                const uint32_t slot = cc & 1u;
                // lambda slot free: chunk cc - 2 has retired
                if (cc >= 2 && !wait(&S.cdone[slot], ((cc >> 1) - 1) & 1u)) { ok = false; break; }
                const int g = g0 + set;
                if (g < g1) {
                    const uint32_t gg = gc + (uint32_t)(CH * kc + set);  // groups in hand-out order
                    const int q = (int)(gg % NS);
                    if (!wait(&S.sfull[q], (gg / NS) & 1u)) { ok = false; break; }
                    fence_after_sync();
                    uint32_t ehi[8], elo[8], ohi[8], olo[8];
                    if constexpr (T) {
                        // the lane's 16 lambda of the group from the staged P_lm tile
#pragma unroll
                        for (int qq = 0; qq < 4; ++qq) {
                            const float4 t4 = S.sd[q].v[qq][r];
                            const float vv[4] = {t4.x, t4.y, t4.z, t4.w};
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const int j = 4 * qq + i;
                                const uint32_t hi = tf32_rna(vv[i]);
                                const uint32_t lo = tf32_rna(vv[i] - __uint_as_float(hi));
                                if (j & 1) {
                                    ohi[j >> 1] = hi;
                                    olo[j >> 1] = lo;
                                } else {
                                    ehi[j >> 1] = hi;
                                    elo[j >> 1] = lo;
                                }
                            }
                        }
                    } else {
                    const SeedSlot &sd = S.sd[q];
                    const int l0 = m + g * GLG_GROUP;
                    const int s0 = l0 > ls ? l0 : ls;
                    const float2 seed = sd.seed[r];
                    float lm2 = 0.f, lm1 = 0.f;
                    // every lane starts at l0 and the group ends inside lmax: no per-step tests
                    const bool regular = __all_sync(0xffffffffu, s0 == l0) && l0 + GLG_GROUP - 1 <= lmax;
                    if (regular) {
#pragma unroll
                        for (int j = 0; j < GLG_GROUP; ++j) {
                            const float v = j == 0 ? seed.x : j == 1 ? seed.y : rec_step(sd.coef[j], x, lm1, lm2);
                            lm2 = lm1;
                            lm1 = v;
                            const uint32_t hi = tf32_rna(v);
                            const uint32_t lo = tf32_rna(v - __uint_as_float(hi));
                            if (j & 1) {
                                ohi[j >> 1] = hi;
                                olo[j >> 1] = lo;
                            } else {
                                ehi[j >> 1] = hi;
                                elo[j >> 1] = lo;
                            }
                        }
                    } else {
                        // rings of the tile start at different l: branch-free
                        // steps, the recurrence of zeros staying zero until the
                        // lane's seeds at js = s0 - l0 are selected in
                        const int js = s0 - l0, jend = lmax - l0;
#pragma unroll
                        for (int j = 0; j < GLG_GROUP; ++j) {
                            float v = rec_step(sd.coef[j], x, lm1, lm2);
                            v = j == js ? seed.x : v;
                            v = j == js + 1 ? seed.y : v;
                            v = j > jend ? 0.f : v;
                            lm2 = lm1;
                            lm1 = v;
                            const uint32_t hi = tf32_rna(v);
                            const uint32_t lo = tf32_rna(v - __uint_as_float(hi));
                            if (j & 1) {
                                ohi[j >> 1] = hi;
                                olo[j >> 1] = lo;
                            } else {
                                ehi[j >> 1] = hi;
                                elo[j >> 1] = lo;
                            }
                        }
                    }
                    }
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&S.sempty[q]);  // seed slot read
                    const uint32_t col = tb + lane_base + A_COL0 + slot * A_SLOT + 32 * set;
                    tmem_st8(col + 0, ehi);
                    tmem_st8(col + 8, elo);
                    tmem_st8(col + 16, ohi);
                    tmem_st8(col + 24, olo);
                    tmem_wait_st();
                }
                fence_before_sync();
                __syncwarp();
                if (lane == 0) mbar_arrive(&S.full_a[slot]);  // every set arrives, active or not
            }
            gc += (uint32_t)(G - gf);
        }
        if (!ok) fail();
    } else if (warp < W_MMA) {
        // --------------------------------- drain: chunk sums -> F
        if constexpr (T) {
            regs_inc<REGS_DRAIN>();
            // running sums of this lane (ring pair): E in columns 0..N-1, O
            // in N..2N-1, added chunk by chunk in the order of the
            // shared-memory path (same FP32 results)
            float acc[2 * N];
#pragma unroll
            for (int c = 0; c < 2 * N; ++c) acc[c] = 0.f;
            uint32_t cc = 0;
            bool ok = true;
            for (uint32_t ui = 0; ok; ++ui) {
                int64_t u;
                if (!next_unit(ui, u, true)) { ok = false; break; }
                if (u >= a.nunits) break;
                const int tile = a.tile0 + (int)(u % a.nrun);
                const int m = unit_m(u / a.nrun);
                const int G = (lmax - m + GLG_GROUP) / GLG_GROUP;
                const int gf = a.tfirst[(int64_t)m * a.ntiles + tile];
                for (int kc = 0, nch = (G - gf + CH - 1) / CH; kc < nch; ++kc, ++cc) {
                    const uint32_t d = cc & 1u;
                    if (!wait(&S.cdone[d], (cc >> 1) & 1u)) { ok = false; break; }
                    fence_after_sync();
                    static_assert((2 * N) % 32 == 0, "accumulator columns in pairs of 16");
                    const uint32_t dcol = tb + lane_base + 2 * N * d;
#pragma unroll
                    for (int c0 = 0; c0 < 2 * N; c0 += 32) {
                        uint32_t v[32];
                        tmem_ld16(dcol + c0, *reinterpret_cast<uint32_t(*)[16]>(&v[0]));
                        tmem_ld16(dcol + c0 + 16, *reinterpret_cast<uint32_t(*)[16]>(&v[16]));
                        tmem_wait_ld();
#pragma unroll
                        for (int j = 0; j < 32; ++j) acc[c0 + j] += __uint_as_float(v[j]);
                    }
                    fence_before_sync();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&S.empty_d[d]);
                }
                if (!ok) break;
                // unit complete: north = E + O, south = E - O
                const int p = tile * 128 + r;
                if (p < a.npairs) {
                    const int rs = a.nrings - 1 - p;
#pragma unroll
                    for (int map = 0; map < N / 2; ++map) {
                        if (map < a.nmaps) {
                            const float er = acc[2 * map], ei = acc[2 * map + 1];
                            const float orr = acc[N + 2 * map], oi = acc[N + 2 * map + 1];
                            float2 *Fm = a.F + ((int64_t)map * (lmax + 1) + m) * a.nrings;
                            Fm[p] = make_float2(er + orr, ei + oi);
                            if (rs != p) Fm[rs] = make_float2(er - orr, ei - oi);
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < 2 * N; ++c) acc[c] = 0.f;
            }
            if (!ok) fail();
        } else {
        uint32_t cc = 0;
        bool ok = true;
        for (uint32_t ui = 0; ok; ++ui) {
            int64_t u;
            if (!next_unit(ui, u, true)) { ok = false; break; }
            if (u >= a.nunits) break;
            const int tile = a.tile0 + (int)(u % a.nrun);
            const int m = unit_m(u / a.nrun);
            const int G = (lmax - m + GLG_GROUP) / GLG_GROUP;
            const int gf = a.tfirst[(int64_t)m * a.ntiles + tile];
            for (int kc = 0, nch = (G - gf + CH - 1) / CH; kc < nch; ++kc, ++cc) {
                int g0, g1;
                chunk_range(kc, gf, G, g0, g1);
                const uint32_t d = cc & 1u;
                if (!wait(&S.cdone[d], (cc >> 1) & 1u)) { ok = false; break; }
                fence_after_sync();
                static_assert((2 * N) % 32 == 0, "accumulator columns in pairs of 16");
                float4 *row = reinterpret_cast<float4 *>(&S.acc[r][0]);
                const uint32_t dcol = tb + lane_base + 2 * N * d;
                // rounds of 32 columns: the running sums' shared-memory loads
                // are issued before the tensor-memory loads, so both
                // latencies overlap before the adds
#pragma unroll 1
                for (int c0 = 0; c0 < 2 * N; c0 += 32) {
                    float4 t[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) t[j] = row[c0 / 4 + j];
                    uint32_t v[32];
                    tmem_ld16(dcol + c0, *reinterpret_cast<uint32_t(*)[16]>(&v[0]));
                    tmem_ld16(dcol + c0 + 16, *reinterpret_cast<uint32_t(*)[16]>(&v[16]));
                    tmem_wait_ld();
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        t[j].x += __uint_as_float(v[4 * j]);
                        t[j].y += __uint_as_float(v[4 * j + 1]);
                        t[j].z += __uint_as_float(v[4 * j + 2]);
                        t[j].w += __uint_as_float(v[4 * j + 3]);
                        row[c0 / 4 + j] = t[j];
                    }
                }
                fence_before_sync();
                __syncwarp();
                if (lane == 0) mbar_arrive(&S.empty_d[d]);
            }
            if (!ok) break;
            // unit complete: north = E + O, south = E - O
            const int p = tile * 128 + r;
            if (p < a.npairs) {
                const int rs = a.nrings - 1 - p;
                for (int map = 0; map < a.nmaps; ++map) {
                    const float er = S.acc[r][2 * map], ei = S.acc[r][2 * map + 1];
                    const float orr = S.acc[r][N + 2 * map], oi = S.acc[r][N + 2 * map + 1];
                    float2 *Fm = a.F + ((int64_t)map * (lmax + 1) + m) * a.nrings;
                    Fm[p] = make_float2(er + orr, ei + oi);
                    if (rs != p) Fm[rs] = make_float2(er - orr, ei - oi);
                }
            }
            for (int c0 = 0; c0 < 2 * N; c0 += 4)
                *reinterpret_cast<float4 *>(&S.acc[r][c0]) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        if (!ok) fail();
        }
    } else {
    if constexpr (T) regs_dec<REGS_MISC>();  // warps 16-19: one warpgroup
    if (warp == W_MMA || warp == W_MMA2) {
        // ---------------------------------------------------------- MMA issue
        // Warp W_MMA issues the even-parity (E) accumulator's MMAs, warp
        // W_MMA2 the odd (O) one's, from different SM sub-partitions: each
        // competes with that sub-partition's producer and drain warps for
        // issue slots, so two issuers halve the time spent waiting for them.
        const uint32_t par = warp == W_MMA ? 0u : 1u;
        uint32_t cc = 0;
        bool ok = true, issued = false;
        for (uint32_t ui = 0; ok && lane == 0; ++ui) {
            int64_t u;
            if (!next_unit(ui, u, false)) { ok = false; break; }
            if (u >= a.nunits) break;
            {
                const int tile = a.tile0 + (int)(u % a.nrun);
                const int m = unit_m(u / a.nrun);
                const int G = (lmax - m + GLG_GROUP) / GLG_GROUP;
                const int gf = a.tfirst[(int64_t)m * a.ntiles + tile];
                for (int kc = 0, nch = (G - gf + CH - 1) / CH; kc < nch; ++kc, ++cc) {
                int g0, g1;
                chunk_range(kc, gf, G, g0, g1);
                    const uint32_t k = cc & 1u, bsl = cc % NBC;
                    if (cc >= 2 && !wait(&S.empty_d[k], ((cc >> 1) - 1) & 1u)) { ok = false; break; }
                    if (!wait(&S.full_b[bsl], (cc / NBC) & 1u) || !wait(&S.full_a[k], (cc >> 1) & 1u)) {
                        ok = false;
                        break;
                    }
                    fence_after_sync();
                    const int ng = g1 - g0;
                    const uint32_t dD = tb + 2 * N * k + N * par;              // this parity's accumulator
                    const uint32_t a0 = tb + A_COL0 + k * A_SLOT + 16 * par;   // its (A_hi, A_lo) columns
                    // descriptor of the slot's first tile; the 14-bit start
                    // address field (bytes / 16) takes the tile offsets
                    constexpr uint64_t TT = (32 * N) >> 4, GT = BBYTES >> 4;  // tile, group strides
                    // this parity's (B_hi, B_lo) tiles: E at tiles 0, 1; O at 2, 3
                    const uint64_t d0 = sdesc_noswz(smem_u32(S.bs[bsl].b), 128, 256) + 2 * TT * par;
                    // small cross terms of every group first, then the large
                    // terms; fully unrolled so that nothing but the MMAs
                    // themselves sits between consecutive issues
#pragma unroll
                    for (int q = 0; q < CH; ++q) {
                        if (q < ng) {
                            mma_tf32_ts(dD, a0 + 32 * q + 0, d0 + q * GT + TT, IDESC, q > 0 ? 1u : 0u);
                            mma_tf32_ts(dD, a0 + 32 * q + 8, d0 + q * GT, IDESC, 1u);
                        }
                    }
#pragma unroll
                    for (int q = 0; q < CH; ++q) {
                        if (q < ng) mma_tf32_ts(dD, a0 + 32 * q + 0, d0 + q * GT, IDESC, 1u);
                    }
                    issued = true;
                    mma_commit(&S.cdone[k]);   // lambda slot free, accumulator ready
                    mma_commit(&S.bempty[bsl]);
                }
            }
        }
        if (lane == 0) {
            if (!ok) fail();
            if (issued) {  // every MMA of this CTA retired before TMEM is freed
                mma_commit(&S.drain);
                for (uint32_t i = 0; i < WAIT_LIMIT && !mbar_try_wait(&S.drain, 0); ++i) {
                }
            }
        }
        __syncwarp();
    } else if (warp == W_LOAD) {
        // ------------------------------------------------------- B streaming
        uint32_t cc = 0;
        bool ok = true;
        int64_t last_use[NBC];
        for (int k = 0; k < NBC; ++k) last_use[k] = -1;
        for (uint32_t ui = 0; ok && lane == 0; ++ui) {
            int64_t u;
            if (!next_unit(ui, u, false)) { ok = false; break; }
            if (u >= a.nunits) break;
            {
                const int tile = a.tile0 + (int)(u % a.nrun);
                const int m = unit_m(u / a.nrun);
                const int G = (lmax - m + GLG_GROUP) / GLG_GROUP;
                const int gf = a.tfirst[(int64_t)m * a.ntiles + tile];
                const int64_t gb = a.goff[m];
                for (int kc = 0, nch = (G - gf + CH - 1) / CH; kc < nch; ++kc, ++cc) {
                int g0, g1;
                chunk_range(kc, gf, G, g0, g1);
                    const uint32_t bsl = cc % NBC, use = cc / NBC;
                    if (use > 0 && !wait(&S.bempty[bsl], (use - 1) & 1u)) { ok = false; break; }
                    const int ng = g1 - g0;
                    if (a.stall) continue;  // test hook: the slot is never filled
                    mbar_arrive_expect_tx(&S.full_b[bsl], ng * BBYTES);
                    bulk_g2s(S.bs[bsl].b, a.bpack + (size_t)(gb + g0) * BBYTES, ng * BBYTES, &S.full_b[bsl]);
                    last_use[bsl] = use;
                }
            }
        }
        if (lane == 0) {
            if (!ok) fail();
            // outstanding copies land before the CTA exits
            for (int k = 0; k < NBC; ++k)
                if (last_use[k] >= 0)
                    for (uint32_t i = 0; i < WAIT_LIMIT && !mbar_try_wait(&S.full_b[k], (uint32_t)(last_use[k] & 1)); ++i) {
                    }
        }
        __syncwarp();
    } else if (warp == W_SEED) {
        // ------------------- unit hand-out, seed / coefficient streaming
        if (lane == 0) {
            uint32_t gc = 0;
            bool ok = true;
            int64_t last_use[NS];
            for (int q = 0; q < NS; ++q) last_use[q] = -1;
            for (uint32_t ui = 0; ok; ++ui) {
                const uint32_t uq = ui % NU;
                if (ui >= NU && !wait(&S.uempty[uq], ((ui / NU) - 1) & 1u)) { ok = false; break; }
                const int64_t u = (int64_t)atomicAdd(a.ucount, 1ull);
                S.unit[uq] = u;
                mbar_arrive(&S.ufull[uq]);  // release: the slot's unit is visible to its readers
                if (u >= a.nunits) break;
                const int tile = a.tile0 + (int)(u % a.nrun);
                const int m = unit_m(u / a.nrun);
                const int G = (lmax - m + GLG_GROUP) / GLG_GROUP;
                const int64_t gb = a.goff[m];
                const int64_t cb = a.mofs[m];
                const int gf = a.tfirst[(int64_t)m * a.ntiles + tile];
                for (int gi = 0; gi < G - gf; ++gi) {  // groups in the order the producers take them
                    int c0, c1;
                    chunk_range(gi / CH, gf, G, c0, c1);
                    const int g = c0 + gi % CH;
                    const uint32_t gg = gc + (uint32_t)gi;
                    const int q = (int)(gg % NS);
                    const uint32_t use = gg / NS;
                    if (use > 0 && !wait(&S.sempty[q], (use - 1) & 1u)) { ok = false; break; }
                    if constexpr (T) {
                        mbar_arrive_expect_tx(&S.sfull[q], GLG_PLM_TILE_BYTES);
                        bulk_g2s(&S.sd[q], a.plm + ((gb + g) * a.ntiles + tile) * (GLG_PLM_TILE_BYTES / 16),
                                 GLG_PLM_TILE_BYTES, &S.sfull[q]);
                    } else {
                        SeedSlot &sd = S.sd[q];
                        mbar_arrive_expect_tx(&S.sfull[q], SEED_TX);
                        bulk_g2s(sd.seed, a.seeds + (gb + g) * a.seed_stride + (int64_t)tile * 128, 128 * 8,
                                 &S.sfull[q]);
                        bulk_g2s(sd.coef, a.coef32 + cb + (int64_t)g * GLG_GROUP, GLG_GROUP * 16, &S.sfull[q]);
                    }
                    last_use[q] = use;
                }
                gc += (uint32_t)(G - gf);
            }
            if (!ok) fail();
            for (int q = 0; q < NS; ++q)
                if (last_use[q] >= 0)
                    for (uint32_t i = 0; i < WAIT_LIMIT && !mbar_try_wait(&S.sfull[q], (uint32_t)(last_use[q] & 1)); ++i) {
                    }
        }
        __syncwarp();
    }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        tmem_dealloc(tb, TMEM_COLS);
    }
}

// The recurrence path (running sums in shared memory) and the table path
// (running sums in the drain warps' registers, warpgroup register shares).
template <int N>
__global__ void __launch_bounds__(THREADS, 1) k_leg_tc(const LegTcArgs a) {
    leg_tc_body<N, false>(a);
}
template <int N>
__global__ void __maxnreg__(LEG_REGS) k_leg_tc_plm(const LegTcArgs a) {
    leg_tc_body<N, true>(a);
}

// ------------------------------------------------------------------ packing

// Bpack[goff[m] + g] = 4 tiles (E_hi, E_lo, O_hi, O_lo) of N x 8 tf32 values,
// element (n, k) of a tile at float index (n/8)*64 + (k/4)*32 + (n%8)*4 + k%4,
// holding the re (n even) or im (n odd) part of a_lm d_l (1 + ACC_BIAS) of
// map n/2 at l = m + 16 g + 2 k + parity (d_l the group scale of the
// recurrence; the product's rounding error is carried into the lo part).  One thread per (group, parity, map, k/4): it
// loads the 4 alm of its k quad and writes re and im of the hi and lo tiles
// as 16-byte stores; consecutive threads take consecutive maps and quads, so
// a warp writes 1 KB of a tile contiguously.
template <int N>
__global__ void __launch_bounds__(256) k_pack_b(int mmax, int lmax, int nmaps, int64_t nalm, int64_t ngroups,
                                                const int64_t *__restrict__ mofs,
                                                const int64_t *__restrict__ goff, const float4 *__restrict__ coef32,
                                                const float2 *__restrict__ alm, const float2 *__restrict__ alm2,
                                                int nsplit, float *__restrict__ bpack) {
    const int64_t idx = blockIdx.x * 256LL + threadIdx.x;
    // 2N is a multiple of 32: a warp's items share one group gg, and the
    // warp finds its m (the last m with goff[m] <= gg) by a 32-way search,
    // each lane testing one of 32 candidates per round
    const int64_t gg = idx / (2 * N);
    if (gg >= ngroups) return;  // whole warps
    const int item = (int)(idx - gg * 2 * N);
    const int lane = (int)(threadIdx.x & 31);
    int lo = 0, hi = mmax + 1;  // goff[lo] <= gg < goff[hi] (goff[mmax + 1] = ngroups)
    while (hi - lo > 1) {
        const int step = (hi - lo + 31) / 32;
        const int c = lo + lane * step;
        const bool ok = c < hi && goff[c] <= gg;
        const unsigned bal = __ballot_sync(0xffffffffu, ok);
        const int last = 31 - __clz(bal);  // lane 0 tests lo itself: at least one lane holds
        lo = lo + last * step;
        hi = lo + step < hi ? lo + step : hi;
    }
    const int m = lo;
    const int g = (int)(gg - goff[m]);
    const int mi = item & 3, j = (item >> 2) & 1, rest = item >> 3;
    const int ng = rest % (N / 8), par = rest / (N / 8);
    const int map = ng * 4 + mi;
    float4 rh, rl, ih, il;
    float *r4 = &rh.x, *i4 = &ih.x, *rl4 = &rl.x, *il4 = &il.x;
    const float2 *src = map < nsplit ? alm + (int64_t)map * nalm : alm2 + (int64_t)(map - nsplit) * nalm;
    const int64_t base = mofs[m];
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        const int l = m + g * GLG_GROUP + par + 8 * j + 2 * kk;
        float2 z = make_float2(0.f, 0.f);
        float d = 0.f;
        if (l <= lmax && map < nmaps) {
            z = src[base + (l - m)];
            d = coef32[mofs[m] + (l - m)].z;
        }
        if (m == 0) z.y = 0.f;  // imaginary part of a_l0 is ignored
        const float pr = __fmul_rn(z.x, d), pi = __fmul_rn(z.y, d);
        const float er = fmaf(z.x, d, -pr), ei = fmaf(z.y, d, -pi);  // exact product errors
        const uint32_t zr = tf32_rna(pr), zi = tf32_rna(pi);
        r4[kk] = __uint_as_float(zr);
        i4[kk] = __uint_as_float(zi);
        // lo = the remainder of the hi part, the product's rounding error and
        // the accumulator-bias scaling pr * ACC_BIAS
        rl4[kk] = __uint_as_float(tf32_rna(fmaf(pr, ACC_BIAS, __fadd_rn(__fsub_rn(pr, __uint_as_float(zr)), er))));
        il4[kk] = __uint_as_float(tf32_rna(fmaf(pi, ACC_BIAS, __fadd_rn(__fsub_rn(pi, __uint_as_float(zi)), ei))));
    }
    float *dst = bpack + gg * (int64_t)(32 * N) + ng * 64 + j * 32 + mi * 8;
    float *th = dst + (2 * par) * (8 * N), *tl = dst + (2 * par + 1) * (8 * N);
    reinterpret_cast<float4 *>(th)[0] = rh;
    reinterpret_cast<float4 *>(th)[1] = ih;
    reinterpret_cast<float4 *>(tl)[0] = rl;
    reinterpret_cast<float4 *>(tl)[1] = il;
}

template <int N>
int launch_tc(const glg_plan *P, const float2 *alm, const float2 *alm2, int nsplit, int nmaps, float *bpack,
              float2 *F, int *err, const glg_tile_run &run, const float4 *table, const int *tfirst,
              cudaStream_t st) {
    if (run.pack) {
        const int64_t items = P->ngroups * 2 * N;
        GLG_LAUNCH_SCOPE("k_pack_b", st);
        k_pack_b<N><<<(unsigned)((items + 255) / 256), 256, 0, st>>>(P->mmax, P->lmax, nmaps, P->nalm, P->ngroups,
                                                                     P->mofs, P->goff, P->coef32, alm, alm2,
                                                                     nsplit, bpack);
        GLG_CHECK_LAUNCH("k_pack_b");
    }
    LegTcArgs a;
    a.npairs = P->npairs;
    a.nrings = P->nrings;
    a.lmax = P->lmax;
    a.nmaps = nmaps;
    a.ntiles = (P->npairs + 127) / 128;
    a.tile0 = run.tile0;
    a.nrun = run.ntiles;
    if (a.tile0 < 0 || a.nrun <= 0 || a.tile0 + a.nrun > a.ntiles || run.slot < 0 ||
        run.slot >= GLG_WS_UNIT_COUNTERS) {
        glg_set_error("fast Legendre contraction: tile range or counter slot out of range");
        return GLG_ERR_INVALID;
    }
    a.nunits = (int64_t)a.nrun * (P->mmax + 1);
    a.cth32 = P->cth32;
    a.coef32 = P->coef32;
    a.mofs = P->mofs;
    a.goff = P->goff;
    a.seeds = P->seeds;
    a.seed_stride = P->seed_stride;
    a.lstart = P->lstart;
    a.tfirst = tfirst ? tfirst : P->tfirst;
    a.bpack = reinterpret_cast<const unsigned char *>(bpack);
    a.F = F;
    a.err = err;
    // one zeroed counter per launch of a call (the status block is cleared once per call)
    a.ucount = reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(err) + 64) + run.slot;
    a.wait_limit = g_test_wait_limit ? g_test_wait_limit : WAIT_LIMIT;
    a.stall = g_test_stall;
    a.plm = table ? table : P->plm;
    int nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t grid = a.nunits < nsm ? a.nunits : nsm;
    // more than half of the SM's shared memory: one CTA per SM, so no two
    // CTAs contend for the 512 tensor-memory columns
    auto go = [&](auto kern, size_t bytes) {
        size_t smem = bytes + 128;
        if (smem < 120 * 1024) smem = 120 * 1024;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        GLG_LAUNCH_SCOPE("k_leg_tc", st);
        kern<<<(unsigned)grid, THREADS, smem, st>>>(a);
    };
    if (a.plm) {
        // the warpgroup register shares assume the launch's LEG_REGS registers a thread
        static int regs = -1;
        if (regs < 0) {
            cudaFuncAttributes fa;
            regs = cudaFuncGetAttributes(&fa, k_leg_tc_plm<N>) == cudaSuccess ? fa.numRegs : 0;
        }
        if (regs != LEG_REGS) {
            glg_set_error("fast Legendre contraction: the table kernel was not built with its register count");
            return GLG_ERR_UNSUPPORTED;
        }
        go(k_leg_tc_plm<N>, sizeof(Smem<N, true>));
    } else {
        go(k_leg_tc<N>, sizeof(Smem<N, false>));
    }
    GLG_CHECK_LAUNCH("k_leg_tc");
    return GLG_OK;
}

}  // namespace

extern "C" int glg_test_stall_contraction(int on, unsigned int wait_limit) {
    g_test_stall = on ? 1 : 0;
    g_test_wait_limit = on ? (wait_limit ? wait_limit : 1u) : 0u;
    return GLG_OK;
}

size_t glg_leg_tc_pack_bytes(const glg_plan *P, int nmaps) {
    const int N = ((2 * nmaps + 15) / 16) * 16;
    return (size_t)P->ngroups * 128 * N;
}

int glg_launch_leg_tc(const glg_plan *P, const float2 *alm, int nmaps, float *bpack, float2 *F,
                      int *err, const glg_tile_run &run, cudaStream_t st) {
    return glg_launch_leg_tc_ex(P, alm, nullptr, nmaps, nmaps, bpack, F, err, run, nullptr, nullptr, st);
}

int glg_launch_leg_tc_ex(const glg_plan *P, const float2 *alm, const float2 *alm2, int nsplit, int nmaps,
                         float *bpack, float2 *F, int *err, const glg_tile_run &run, const float4 *table,
                         const int *tfirst, cudaStream_t st) {
    const int N = ((2 * nmaps + 15) / 16) * 16;
    if ((table == nullptr) != (tfirst == nullptr)) {
        glg_set_error("fast Legendre contraction: a spin table needs its first-group table");
        return GLG_ERR_INVALID;
    }
#define GLG_TC(n) launch_tc<n>(P, alm, alm2, nsplit, nmaps, bpack, F, err, run, table, tfirst, st)
    switch (N) {
        case 16: return GLG_TC(16);
        case 32: return GLG_TC(32);
        case 48: return GLG_TC(48);
        case 64: return GLG_TC(64);
        case 80: return GLG_TC(80);
        default:
            glg_set_error("fast Legendre contraction: at most 40 maps per launch");
            return GLG_ERR_UNSUPPORTED;
    }
}
#undef GLG_TC
