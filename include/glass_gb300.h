/*
 * glass_gb300 -- C ABI of the GB300 (sm_103a) field-generation path.
 *
 * Every entry point takes DEVICE pointers (CUDA global memory), plain sizes
 * and a cudaStream_t passed as void*, launches asynchronously on that
 * stream, and returns an int status (GLG_OK = 0, negative on error; the
 * message is in glg_last_error()).  Nothing here traps or aborts.  Complex
 * arrays are interleaved (re, im) pairs of the element type named by the
 * `dtype` argument: GLG_F64 = complex128 / float64, GLG_F32 = complex64 /
 * float32.
 *
 * Each function names the reference interface it replaces (GLASS, file:line
 * within the glass-dev/glass project).  The Python package glass_gb300 binds
 * these through ctypes (glass_gb300/_lib.py); a binding on the GLASS side
 * would be a ctypes module of the same kind.
 */
#ifndef GLASS_GB300_H
#define GLASS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GLG_OK 0
#define GLG_ERR_INVALID (-1)      /* bad argument        -> ValueError  */
#define GLG_ERR_NOT_POSDEF (-2)   /* iternorm s^2 < 0    -> ValueError  */
#define GLG_ERR_CUDA (-3)         /* CUDA runtime error  -> RuntimeError */
#define GLG_ERR_NOMEM (-4)        /* allocation failed   -> MemoryError */
#define GLG_ERR_UNSUPPORTED (-5)  /* size beyond a kernel limit          */
#define GLG_ERR_TIMEOUT (-6)      /* a bounded device wait gave up       */

/* element types */
#define GLG_F64 0
#define GLG_F32 1

/* precision forms of the spherical-harmonic transforms */
#define GLG_FORM_PLAIN 0   /* FP64 everywhere (drop-in form)                 */
#define GLG_FORM_FAST 1    /* FP32 maps; split-precision Legendre contraction */

/* fused map epilogues (glass/grf/_transformations.py) */
#define GLG_EPI_NONE 0       /* Normal.__call__, :26-28                   */
#define GLG_EPI_LOGNORMAL 1  /* Lognormal.__call__, :83-89: l*expm1(x - v/2) */

typedef struct glg_plan glg_plan;

/* Library version string and last error message of the calling thread. */
const char *glg_version(void);
const char *glg_last_error(void);

/*
 * Plan: HEALPix ring geometry, Legendre recurrence tables (FP64) and ring-FFT
 * twiddle tables for one (nside, lmax), resident on the current device.
 * Replaces the implicit per-call set-up inside healpy.alm2map / map2alm
 * (called at glass/healpix.py:71, :107, :270).  nside must be a power of two.
 * Creating a plan allocates device memory (cudaMalloc) and is the only
 * allocating call of this library besides glg_plan_destroy.
 */
int glg_plan_create(int nside, int lmax, void *stream, glg_plan **plan);
void glg_plan_destroy(glg_plan *plan);
size_t glg_plan_device_bytes(const glg_plan *plan);
/*
 * The fast form's Legendre values P_lm: when the first fast transform of a
 * plan builds its tables, it keeps every lambda_lm(x_ring) resident in
 * device memory as FP32 (the FP64 recurrence rounded once; 4 bytes per
 * (l, m, ring pair), 138 GB at nside 2048 / lmax 4096) if that fits
 * `bytes` (default 160 GiB) and the free device memory with 4 GiB to spare;
 * otherwise the contraction recomputes lambda in FP32 from FP64 seeds every
 * 16 l (less accurate: about 3e-7 instead of 1.4e-7 relative RMS of the
 * Legendre sums).  No counterpart in the reference (healpy recomputes the
 * Legendre functions in every transform).  glg_plan_has_plm_table: 1 once
 * the plan's fast tables hold the P_lm table, else 0.
 */
int glg_set_plm_table_budget(size_t bytes);
int glg_plan_has_plm_table(const glg_plan *plan);
int glg_plan_info(const glg_plan *plan, int *nside, int *lmax, int *nrings, int64_t *npix,
                  int64_t *nalm);

/*
 * Iterative Cholesky scaling vectors, glass/fields.py:101-188 (iternorm).
 * cov: float64 [nrows][nl][k+1], row i = the covariance row of field i for
 * every mode l, as produced by cls2cov (glass/fields.py:191-236).
 * w: float64 [nrows][nl][k+1] = [a_0..a_{k-1}, s].  status: one uint64 of
 * device memory; it is set to UINT64_MAX before the launch and, when a row's
 * variance becomes negative, to the first such row -- the caller then raises
 * "covariance matrix is not positive definite" (glass/fields.py:180-181).
 * Asynchronous; allocates nothing.  Bit-identical to the fixed-order
 * restatement in oracle/orc_sht.c.  Limit: k <= 120 (the two k x k FP64
 * matrices of one mode l live in one block's shared memory).
 */
int glg_iternorm(const double *cov, int64_t nrows, int64_t nl, int k, double *w,
                 uint64_t *status, void *stream);

/*
 * Covariance rows of every field at once, glass/fields.py:191-236 (cls2cov),
 * and the variances of glass/fields.py:890 (transformcl.cltovar of each
 * auto-spectrum).  flat: the nf(nf+1)/2 spectra in GLASS order, float64,
 * concatenated; offs: int64 [nspec+1] offsets into flat.  cov: float64
 * [nf][nl][nc+1] (= C^{j,j-i}_l / 2, zero-padded); var: float64 [nf].
 * status: one uint64 of device memory, UINT64_MAX, or the first field whose
 * auto-spectrum has a negative value ("negative values in cl").
 */
int glg_cls2cov(const double *flat, const int64_t *offs, int nf, int nl, int nc, double *cov,
                double *var, uint64_t *status, void *stream);

/*
 * Host-only: concatenate n host buffers (src[i], bytes[i] bytes each) into
 * dst, in order, split over up to nthreads host threads (the copy of the
 * spectra into one page-locked block before their upload, in place of the
 * single-threaded numpy concatenation).  No device call.
 */
int glg_gather_host(const void *const *src, const int64_t *bytes, int n, void *dst, int nthreads);

/*
 * Standard complex normals of the counter-based stream that replaces the
 * reference's numpy draw standard_normal((z_size, 2)) @ [1, 1j]
 * (glass/fields.py:407; generator seam glass/rng.py:21-55).  Element e of
 * stream `sid` under `seed` is one Philox4x32-10 block (counter = e, sid;
 * key = seed) mapped by Box-Muller; writes n complex values for elements
 * offset..offset+n-1.
 */
int glg_philox_normals(uint64_t seed, uint64_t sid, int64_t offset, int64_t n, int dtype,
                       void *out, void *stream);

/*
 * Correlated alm of shells t0..t0+nshell-1 (glass/fields.py:401-425):
 *   alm_t = sum_{d=0..min(t,k)} multalm(z_{t-d}, w_t[:, k-d])
 * (glass/harmonics.py:17-47), reordered from GLASS to HEALPix order
 * (glass/fields.py:943-962) with the m = 0 realification of
 * glass/fields.py:425.  w: [nshell][L][k+1] (iternorm output of those
 * shells, L = lmax+1).  z: complex [nz][nalm] in GLASS order holding
 * shells z_first..t0+nshell-1 (z_first = max(0, t0-k)), or NULL to draw them
 * from the Philox stream (key seed, stream sid_base + shell index, element =
 * GLASS index).  alm: complex [nshell][nalm], HEALPix order.  dtype applies
 * to w (float64 or float32, the iternorm rows rounded to float32 by the
 * caller), z and alm.
 */
int glg_alm_correlate(const void *w, int nshell, int lmax, int k, int64_t t0, const void *z,
                      int64_t z_first, uint64_t seed, uint64_t sid_base, int dtype, void *alm,
                      void *stream);

/* multalm, glass/harmonics.py:17-47: alm (GLASS order) * repeat(bl, l+1). */
int glg_multalm(const void *alm, const double *bl, int lmax, int dtype, void *out, void *stream);

/* almxfl, glass/healpix.py:111-140: HEALPix-order alm * fl[l] (0 beyond nfl). */
int glg_almxfl(const void *alm, const double *fl, int nfl, int lmax, int nmaps, int dtype,
               void *out, void *stream);

/*
 * Autotuner of the fast form (no counterpart in the reference, whose
 * transforms are healpy's): times every ring-FFT size bucket of the plan at
 * 128, 256, 512 and (power-of-two transforms) 1024 threads per block on the
 * given workspace (sized by
 * glg_alm2map_workspace for nmaps, GLG_FORM_FAST) and float32 output maps
 * [nmaps][npix] (overwritten), and keeps the fastest in the plan.  Builds the
 * fast-form tables on first use; synchronises the stream.
 */
int glg_autotune_fast(glg_plan *plan, int nmaps, void *maps, void *ws, size_t ws_bytes, void *stream);

/* Ring-FFT launch buckets of a plan: (kind, size, ring pairs, threads) per
 * bucket into out[4 * max_buckets], kind 0 mixed radix, 1 Bluestein, 2
 * power-of-two equatorial length; returns the number written. */
int glg_plan_buckets(const glg_plan *plan, int *out, int max_buckets);
/* The autotuner's time (ms) of one launch of each bucket at its chosen block
 * size (0 before glg_autotune_fast ran); returns the number written. */
int glg_plan_bucket_times(const glg_plan *plan, float *ms, int max_buckets);

/*
 * One step of the multi-plane convergence recurrence, replacing
 * glass/lensing.py:577-581 (MultiPlaneConvergence.add_plane):
 *   kappa3 <- kappa3 * (1 - t);  kappa3 += t * kappa2;  kappa3 += f * delta2
 * in place, in that order, each step rounded to the maps' type (float64 or
 * float32, dtype) with FP64 products.  delta2 may be NULL (a zero plane).
 * t and f are computed on the host from the cosmology as the reference does.
 */
int glg_convergence_step(void *kappa3, const void *kappa2, const void *delta2, int dtype, int64_t n,
                         double t, double f, void *stream);

/*
 * HEALPix RING-scheme pixel indices (healpy.ang2pix, used at
 * glass/galaxies.py:329 through glass/healpix.py): lonlat != 0 takes
 * longitude / latitude in degrees, else colatitude theta / longitude phi in
 * radians.  Device arrays: float64 inputs [n], int64 output [n].
 */
int glg_ang2pix(int nside, const double *theta_or_lon, const double *phi_or_lat, int64_t n, int lonlat,
                int64_t *ipix, void *stream);

/*
 * Lensed galaxy ellipticities, replacing glass/galaxies.py:271-347
 * (galaxy_shear): kappa, gamma1, gamma2 gathered at the RING pixel of each
 * (lon, lat) in degrees; reduced != 0: g = gamma / (1 - kappa), result
 * (eps + g) / (1 + conj(g) eps); else eps + gamma.  lon, lat: float64 [n];
 * eps, out: complex128 [n]; maps: float64 or float32 [12 nside^2] (dtype).
 */
int glg_galaxy_shear(const double *lon, const double *lat, const void *eps, int64_t n, const void *kappa,
                     const void *gamma1, const void *gamma2, int dtype, int nside, int reduced,
                     void *out, void *stream);

/*
 * Positions of counted galaxies inside their pixels, replacing the
 * healpy.randang sampling of glass/points.py:351-440 (positions_from_delta):
 * galaxy g (first <= g < first + n) belongs to the RING pixel p with
 * offsets[p] <= g < offsets[p+1] (offsets: int64 exclusive prefix sums of
 * the counts, [12 nside^2]); its position is uniform on the pixel's area,
 * from the Philox stream (key seed, stream sid < 2^32, counter g).  lon in
 * [0, 360) and lat in degrees, float64 [n].  misses: one uint64 of device
 * memory counting galaxies whose 64 draws all fell outside the pixel (left
 * at the pixel centre; none expected).
 */
int glg_positions(int nside, const int64_t *offsets, int64_t first, int64_t n, uint64_t seed, uint64_t sid,
                  double *lon, double *lat, unsigned long long *misses, void *stream);

/*
 * Per-pixel Poisson galaxy counts, replacing glass/points.py:252-348
 * (_compute_expected_count, _apply_visibility, _sample_number_galaxies):
 *   n_e = ((bias * delta_e - offset) + 1) * scale  [* vis_e],  clipped at 0,
 *   counts_e ~ Poisson(n_e)
 * with scale = ARCMIN2_SPHERE / npix * ngal and offset the monopole that
 * remove_monopole subtracts (0 otherwise).  delta: float64 or float32
 * [npix] (dtype); vis: float64 [npix] or NULL; counts: int64 [npix].  The
 * draw uses the Philox stream (key seed, stream sid < 2^32, element = pixel)
 * and is reproducible bit for bit from the same delta values, whatever their
 * producer (plain or fast form).
 */
int glg_poisson_counts(const void *delta, int dtype, int64_t npix, double bias, double offset,
                       double scale, const double *vis, uint64_t seed, uint64_t sid,
                       int64_t *counts, void *stream);

/* Fused epilogue applied while maps are stored. */
typedef struct glg_epilogue {
    int kind;             /* GLG_EPI_* for every map, unless `kinds` is set  */
    const int *kinds;     /* host array [nmaps] of GLG_EPI_*, or NULL        */
    const double *var;    /* host array [nmaps]: Gaussian variance sigma^2   */
    const double *lamda;  /* host array [nmaps]: lognormal shift lambda      */
} glg_epilogue;

/*
 * Spin-0 synthesis, glass/healpix.py:38-78 (healpy.alm2map with pol=False,
 * pixwin=False; as called at glass/fields.py:429).  alm: complex [nmaps][nalm]
 * (HEALPix order, mmax = lmax of the plan); maps: [nmaps][npix] RING order.
 * form GLG_FORM_PLAIN: FP64 throughout (alm complex128, maps float64).
 * form GLG_FORM_FAST: alm complex64, maps float32; the Legendre sums run on
 *   the tensor cores as split-precision 3xTF32 with FP32 accumulation,
 *   lambda_lm from an FP32 recurrence restarted every 16 l from FP64 seeds
 *   (built once per plan on first use; that first call synchronises the
 *   stream); at most 40 maps per call; nside <= 2048.
 * workspace: device scratch of glg_alm2map_workspace() bytes.  For the fast
 * form its first int receives GLG_ERR_TIMEOUT if a bounded device wait gave
 * up; glg_workspace_status() reads it.
 */
size_t glg_alm2map_workspace(const glg_plan *plan, int nmaps, int form);
int glg_alm2map(const glg_plan *plan, const void *alm, int nmaps, int form, void *maps,
                const glg_epilogue *epi, void *workspace, size_t workspace_bytes, void *stream);

/* Device address of page-locked host memory (allocated by cudaHostAlloc or
 * registered with cudaHostRegister, mapped into the device), so that maps
 * can be written straight into host buffers across the CPU-GPU link:
 * GLG_ERR_INVALID for any other pointer.  No counterpart in the reference. */
int glg_host_device_pointer(const void *host, void **dev);

/*
 * Fast-form spin-0 synthesis into HOST maps: float32 [nmaps][npix] at
 * maps_host, alm complex64 [nmaps][nalm] on the device, at most 40 maps.
 * Same result as glg_alm2map(GLG_FORM_FAST) into device maps, then copied.
 * The transform runs in ring-tile runs from the equator to the poles; each
 * run's pixel bands are copied to the host (one 2-D copy per band on a copy
 * stream of the call) while the next run computes, so most of the copy hides
 * behind the computation.  maps_host should be page-locked (cudaHostAlloc or
 * cudaHostRegister) for the copies to overlap; pageable memory works, but
 * the call then returns only after its copies end.  The caller's stream
 * waits for the last copy.  The call creates and destroys its copy stream:
 * do not capture it into a CUDA graph (glg_alm2map into device maps can
 * be).  workspace: glg_alm2map_host_workspace() bytes
 * (the fast-form workspace plus device staging maps); its status word is
 * read by glg_workspace_status() as for glg_alm2map.  Host-side entry of
 * glass/fields.py:839-894 (generate) when numpy maps are wanted.
 */
size_t glg_alm2map_host_workspace(const glg_plan *plan, int nmaps);
int glg_alm2map_host(const glg_plan *plan, const void *alm, int nmaps, void *maps_host,
                     const glg_epilogue *epi, void *workspace, size_t workspace_bytes, void *stream);

/* The runs glg_alm2map_host makes at this nside (host arithmetic only, no
 * device): per run 8 int64 into out[8 * max_runs]: ring tiles t0, t1
 * (128 ring pairs each), ring pairs p0, p1, then the pixel bands [n0, n1)
 * (north rings) and [s0, s1) (south rings; [0, 0) when empty).  Returns the
 * run count, or GLG_ERR_INVALID (nside outside [1, 8192], max_runs below the
 * count).  No counterpart in the reference. */
int glg_host_output_runs(int nside, int64_t *out, int max_runs);

/*
 * Graph-capturable fast synthesis: glg_alm2map's fast form with the epilogue
 * read from device memory at run time (epi_dev: glg_epilogue_dev_bytes()
 * bytes, filled on the host by glg_epilogue_dev_fill and copied to the
 * device before each launch or graph replay), so one captured CUDA graph
 * serves every epilogue.  The plan's fast tables must exist (one fast
 * glg_alm2map first).  nmaps <= 40; float32 maps.  Used by the serving loop
 * (glass/fields.py:839-894 per request) and SynthGraph; no counterpart in
 * the reference.  Check glg_workspace_status afterwards.
 */
size_t glg_epilogue_dev_bytes(void);
int glg_epilogue_dev_fill(const glg_epilogue *epi, int nmaps, void *host_out);
int glg_alm2map_fast_devepi(const glg_plan *plan, const void *alm, int nmaps, void *maps, const void *epi_dev,
                            void *workspace, size_t workspace_bytes, void *stream);

/* Status word of a fast-form workspace (synchronises `stream`): GLG_OK or
 * GLG_ERR_TIMEOUT.  No counterpart in the reference (no device waits there). */
int glg_workspace_status(const void *workspace, void *stream);

/*
 * Spin-s synthesis (s = 1, 2), glass/healpix.py:81-108 (healpy.alm2map_spin,
 * as called at glass/lensing.py:343, :366).  elm, blm: complex128 [nalm]
 * (blm may be NULL = zero B-modes); q, u: float64 [npix].
 * Convention: Q + iU = -sum (E + iB) sY_lm.
 */
size_t glg_alm2map_spin_workspace(const glg_plan *plan);
int glg_alm2map_spin(const glg_plan *plan, const void *elm, const void *blm, int spin, void *q,
                     void *u, void *workspace, size_t workspace_bytes, void *stream);

/*
 * Fast form of the spin-s synthesis (s = 1, 2) of the same convention, for
 * nfields fields at once (glass/healpix.py:81-108 as called at
 * glass/lensing.py:343, :366): two split-precision TF32 contractions on the
 * tensor cores (lambda^+ and lambda^-, from FP32 tables of the FP64
 * recurrence kept with the plan; GLG_ERR_UNSUPPORTED when they do not fit the
 * P_lm table budget or the free device memory) and FP32 ring FFTs.
 * elm: complex64 [nfields][nalm]; blm: complex64 [nfields][nalm] or NULL
 * (zero B-modes); qu: float32 [2][nfields][npix] (the Q maps, then the U
 * maps).  nfields <= 20.  Check glg_workspace_status afterwards.
 */
size_t glg_alm2map_spin_fast_workspace(const glg_plan *plan, int nfields, int with_b);
int glg_alm2map_spin_fast(const glg_plan *plan, const void *elm, const void *blm, int nfields, int spin,
                          void *qu, void *workspace, size_t workspace_bytes, void *stream);

/*
 * Spin-0 analysis, glass/healpix.py:232-276 (healpy.map2alm with pol=False,
 * as called at glass/lensing.py:306), uniform pixel weights 4 pi / npix and
 * `niter` Jacobi refinements (healpy's default iter = 3).  maps: float64
 * [nmaps][npix]; alm: complex128 [nmaps][nalm].
 */
size_t glg_map2alm_workspace(const glg_plan *plan, int nmaps);
int glg_map2alm(const glg_plan *plan, const void *maps, int nmaps, int niter, void *alm,
                void *workspace, size_t workspace_bytes, void *stream);

/*
 * HEALPix pixel window functions, replacing healpy.pixwin as called at
 * glass/healpix.py:351 (and used by glass/lensing.py:360-362 for discretized
 * shear).  healpy reads them from data files; here they are computed on the
 * device from their definition: pw0_l^2 = mean over pixels of the pair
 * average <<P_l(cos gamma)>> over two uniform points of the pixel (the
 * pixel-averaged harmonics' power), pw2_l^2 the same with the spin-2 kernel
 * d^l_22 (pw2_l = 0 for l < 2).  One pass accumulates the pixels' pair
 * moments <<sin^2(gamma/2)^k>> (8 x 8 Gauss-Legendre nodes on each half of
 * every pixel's diamond in the equal-area HEALPix projection, one pixel per
 * congruence class); every l follows from the hypergeometric series of the
 * kernels in sin^2(gamma/2).  pw0, pw2: float64 [lmax+1] (pw2 may be NULL).
 * Limits: 1 <= nside <= 8192, lmax <= 4 nside.  Parity with healpy's
 * tables is not established (they are not available offline).
 */
size_t glg_pixwin_workspace(int nside);
int glg_pixwin(int nside, int lmax, double *pw0, double *pw2, void *ws, size_t ws_bytes, void *stream);

/*
 * Spin-0 synthesis that allocates nothing.  No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc where they need a map --
 * loops whose device memory is fixed at start-up (an allocation there can
 * fail or stall the loop), or programs whose device memory belongs to an
 * allocator (a framework's caching pool, a per-process memory budget) that
 * must not be bypassed.  It needs no plan and no
 * workspace: alm complex128 [nmaps][nalm] (HEALPix order, lmax), maps float64
 * [nmaps][npix]; FP64 throughout, same result as glg_alm2map's plain form.
 * Its scratch is one fixed array of GLG_NOALLOC_SCRATCH_BYTES in the
 * library's device memory, held by every GPU that loads the library until
 * the process exits.  Limits: nside <= 256, lmax + 1 <= 65535, nmaps <= 65535
 * and nmaps * (4 nside - 1) * (lmax + 1) * 16 <= GLG_NOALLOC_SCRATCH_BYTES,
 * else GLG_ERR_UNSUPPORTED.  All calls share that array: calls that overlap
 * on the GPU race, so serialise them.  The first call on each device looks up
 * the array's address; make it before any stream capture begins.  The
 * address is kept per device index: the entry point assumes the CUDA
 * runtime's primary context of each device.
 */
#define GLG_NOALLOC_SCRATCH_BYTES (16u << 20)
int glg_alm2map_noalloc(int nside, int lmax, const void *alm, int nmaps, void *maps, void *stream);

/*
 * Failure injection for tests (no counterpart in the reference).
 * glg_test_fail_plan_alloc(n): the n-th device allocation of plan creation
 * from now (1 = the next) fails as if cudaMalloc had run out of memory, so
 * the caller sees GLG_ERR_NOMEM (0 clears it).
 * glg_test_stall_contraction(on, polls): while on, the fast contraction's B
 * streamer issues no copies, so its MMA warps' waits run out after `polls`
 * polls; the kernel then records GLG_ERR_TIMEOUT in the workspace status
 * word, retires what it started, frees its tensor memory and returns (no
 * fault, no trap; the context stays usable).  Off restores the normal wait
 * limit.  Process-wide settings, for tests only.
 */
int glg_test_fail_plan_alloc(int nth);
int glg_test_stall_contraction(int on, unsigned int polls);

/*
 * Launch accounting (no counterpart in the reference, which has no GPU
 * code): every kernel launch of this library is counted; with timing
 * enabled each launch is bracketed by CUDA events on its own stream and
 * glg_timing_query sums the durations per kernel name (it waits for them).
 */
int glg_timing_enable(int on);
int glg_timing_reset(void);
int64_t glg_launch_count(void);
int glg_timing_query(const char *kernel, double *total_ms, int64_t *launches);

/*
 * Peak-rate kernels (measurement utilities, no counterpart in the
 * reference): glg_peak_tf32 runs `ctas` CTAs (one per SM), each issuing
 * `iters` tcgen05.mma kind::tf32 of M = 128, N = 256, K = 8 (2 * 128 * 256 * 8
 * flop each) and sets *err to 1 if a completion wait ran out; glg_peak_fma
 * runs `blocks` x 256 threads of 8 independent FMA chains of `iters` steps
 * (16 * iters flop per thread) in FP64 (dtype GLG_F64) or FP32 (GLG_F32),
 * `sink` a device buffer of `blocks` elements of that type.  Time them with
 * CUDA events on `stream`.
 */
int glg_peak_tf32(int ctas, int iters, unsigned int *err, void *stream);
int glg_peak_fma(int dtype, int blocks, int iters, void *sink, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GLASS_GB300_H */
