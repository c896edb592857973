/*
 * CPU oracle for the GLASS field-generation path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker, never the product: only tests/, the smoke test
 * and bench.py's cpu_baseline / reference arm load it.  It restates, in plain
 * FP64 C, the pieces of the reference path whose algorithms live in
 * dependencies that are not vendored with GLASS:
 *
 *   - the HEALPix RING geometry (Gorski et al. 2005, ApJ 622, 759),
 *     used by healpy.alm2map / map2alm, called at glass/healpix.py:71, :270;
 *   - the normalised associated-Legendre recurrence and the ring Legendre
 *     sums of the spin-0 and spin-s spherical-harmonic transforms
 *     (healpy.alm2map / alm2map_spin / map2alm, glass/healpix.py:38-108,
 *     :232-276), with an extended exponent range so that lmax up to 8192
 *     works;
 *   - the iterative Cholesky of glass/fields.py:101-188 (iternorm), in a
 *     fixed summation order with explicit fma() so the GPU kernel can be
 *     checked bit for bit;
 *   - the Philox4x32-10 counter-based generator (Salmon et al., SC'11) and
 *     the Box-Muller map that the GPU path uses in place of numpy's PCG64
 *     (the RNG seam is glass/rng.py:21-55);
 *   - the per-pixel Poisson galaxy counts of glass/points.py:252-348, with
 *     the GPU kernel's exact operation order so counts agree bit for bit.
 *
 * Conventions (HEALPix, with the Condon-Shortley phase):
 *   Y_lm(theta, phi) = lambda_lm(cos theta) exp(i m phi),
 *   map = sum_l a_l0 lambda_l0 + 2 Re sum_{m>0} a_lm lambda_lm e^{i m phi}.
 * Spin-s maps (s = 1, 2): Q + iU = -sum_lm (E_lm + i B_lm) sY_lm, with
 * sY_lm = sqrt((l-s)!/(l+s)!) eth^s Y_lm.
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* values are mant * 2^(EXP_STEP * scale); scale < 0 means "negligible" */
#define EXP_STEP 800
static const double TWO_P800 = 6.668014432879854e+240;  /* 2^800 */
static const double TWO_M800 = 1.499696813895631e-241;  /* 2^-800 */
static const double TWO_P400 = 2.5822498780869086e+120; /* 2^400 */
static const double TWO_M400 = 3.872591914849318e-121;  /* 2^-400 */

/* ---------------------------------------------------------------- geometry */

/* Ring i (1-based, 1..4*nside-1) of a HEALPix RING map. */
void orc_ring_info(int nside, int i, double *z, double *sth, int *nph,
                   double *phi0, int64_t *start)
{
    const double ns = nside;
    const int64_t npix = 12LL * nside * nside;
    const int64_t ncap = 2LL * nside * (nside - 1);
    int north = i <= 2 * nside;
    int ir = north ? i : 4 * nside - i; /* ring index counted from the nearer pole */
    double zz, st;
    if (ir < nside) {
        double t = (double)ir * ir / (3.0 * ns * ns); /* 1 - |z| */
        zz = 1.0 - t;
        st = sqrt(t * (2.0 - t));
        *nph = 4 * ir;
        *phi0 = M_PI / (4.0 * ir);
        *start = north ? 2LL * ir * (ir - 1) : npix - 2LL * ir * (ir + 1);
    } else {
        zz = (2.0 * ns - ir) * 2.0 / (3.0 * ns);
        st = sqrt((1.0 - zz) * (1.0 + zz));
        *nph = 4 * nside;
        *phi0 = ((ir - nside) % 2 == 0) ? M_PI / (4.0 * ns) : 0.0;
        *start = ncap + (int64_t)(i - nside) * 4 * nside;
    }
    *z = north ? zz : -zz;
    *sth = st;
}

/* ------------------------------------------------------------ recurrences */

/* Coefficients of lambda_l = A_l (x lambda_{l-1}) - B_l lambda_{l-2}, for one m,
 * l = m+2 .. lmax; index l-m. */
static void leg_coefs(int m, int lmax, double *A, double *B)
{
    for (int l = m + 2; l <= lmax; ++l) {
        double l2 = (double)l * l, m2 = (double)m * m;
        double lm1 = l - 1.0;
        A[l - m] = sqrt((4.0 * l2 - 1.0) / (l2 - m2));
        B[l - m] = sqrt((4.0 * l2 - 1.0) * (lm1 * lm1 - m2) /
                        ((l2 - m2) * (4.0 * lm1 * lm1 - 1.0)));
    }
}

/* lambda_mm for all m at one ring (sin theta = sth), as (mant, scale). */
static void lmm_table(int mmax, double sth, double *mant, int *scale)
{
    double v = 1.0 / sqrt(4.0 * M_PI);
    int sc = 0;
    mant[0] = v;
    scale[0] = 0;
    for (int m = 1; m <= mmax; ++m) {
        v *= -sth * sqrt((2.0 * m + 1.0) / (2.0 * m));
        if (fabs(v) < TWO_M400) {
            v *= TWO_P800;
            sc -= 1;
        }
        mant[m] = v;
        scale[m] = sc;
    }
}

/* Fill lam[l-m] (l = m..lmax) with lambda_lm(x), zero where negligible. */
static void leg_column(int m, int lmax, double x, double mant0, int scale0,
                       const double *A, const double *B, double *lam)
{
    double l0 = mant0, l1;
    int sc = scale0;
    lam[0] = sc == 0 ? l0 : 0.0;
    if (m == lmax) return;
    l1 = sqrt(2.0 * m + 3.0) * x * l0;
    lam[1] = sc == 0 ? l1 : 0.0;
    for (int l = m + 2; l <= lmax; ++l) {
        double l2 = A[l - m] * (x * l1) - B[l - m] * l0;
        l0 = l1;
        l1 = l2;
        if (sc < 0 && fabs(l1) > TWO_P400) {
            l0 *= TWO_M800;
            l1 *= TWO_M800;
            sc += 1;
        }
        lam[l - m] = sc == 0 ? l1 : 0.0;
    }
}

static int64_t alm_index(int l, int m, int lmax) /* HEALPix m-major order */
{
    return (int64_t)m * (2 * lmax + 1 - m) / 2 + l;
}

/*
 * Spin-0 synthesis Legendre sums over every ring of an nside map, the form
 * used for timing: ring pairs (north ring i and its mirror share
 * lambda_lm(-x) = (-1)^(l+m) lambda_lm(x)), OpenMP over m, one coefficient
 * table per m.  alm: complex128 [nmaps][nalm] (HEALPix order, mmax = lmax);
 * out F: complex128 [nmaps][4 nside - 1][lmax+1].
 */
void orc_alm2ring_all(const double *alm, int nmaps, int lmax, int nside, double *F)
{
    const int mmax = lmax;
    const int nring = 4 * nside - 1, npair = 2 * nside;
    const int64_t nalm = (int64_t)(lmax + 1) * (lmax + 2) / 2;
    double *x = malloc(sizeof(double) * npair);
    double *mant = malloc(sizeof(double) * (size_t)npair * (mmax + 1));
    int *scl = malloc(sizeof(int) * (size_t)npair * (mmax + 1));
#pragma omp parallel for schedule(dynamic)
    for (int p = 0; p < npair; ++p) {
        double sth, phi0;
        int nph;
        int64_t start;
        orc_ring_info(nside, p + 1, &x[p], &sth, &nph, &phi0, &start);
        lmm_table(mmax, sth, mant + (size_t)p * (mmax + 1), scl + (size_t)p * (mmax + 1));
    }
#pragma omp parallel
    {
        double *A = malloc(sizeof(double) * (lmax + 2));
        double *B = malloc(sizeof(double) * (lmax + 2));
        double *lam = malloc(sizeof(double) * (lmax + 2));
        double *acc = malloc(sizeof(double) * 4 * nmaps);
#pragma omp for schedule(dynamic)
        for (int m = 0; m <= mmax; ++m) {
            leg_coefs(m, lmax, A, B);
            const int64_t base = alm_index(m, m, lmax);
            for (int p = 0; p < npair; ++p) {
                leg_column(m, lmax, x[p], mant[(size_t)p * (mmax + 1) + m],
                           scl[(size_t)p * (mmax + 1) + m], A, B, lam);
                for (int k = 0; k < nmaps; ++k) {
                    const double *a = alm + 2 * ((int64_t)k * nalm + base);
                    double er = 0, ei = 0, or_ = 0, oi = 0;
                    for (int l = m; l <= lmax; l += 2) {
                        er += a[2 * (l - m)] * lam[l - m];
                        ei += a[2 * (l - m) + 1] * lam[l - m];
                    }
                    for (int l = m + 1; l <= lmax; l += 2) {
                        or_ += a[2 * (l - m)] * lam[l - m];
                        oi += a[2 * (l - m) + 1] * lam[l - m];
                    }
                    double *fn = F + 2 * (((int64_t)k * nring + p) * (mmax + 1) + m);
                    fn[0] = er + or_;
                    fn[1] = ei + oi;
                    if (p != nring - 1 - p) {
                        double *fs = F + 2 * (((int64_t)k * nring + (nring - 1 - p)) * (mmax + 1) + m);
                        fs[0] = er - or_;
                        fs[1] = ei - oi;
                    }
                }
            }
        }
        free(A); free(B); free(lam); free(acc);
    }
    free(x); free(mant); free(scl);
}

/*
 * Spin-0 synthesis Legendre sums.  alm: complex128 [nmaps][nalm] (HEALPix
 * order, mmax == lmax); rings: list of 1-based ring indices; out F:
 * complex128 [nmaps][nring][mmax+1], F_m(ring) = sum_l a_lm lambda_lm(z).
 */
void orc_alm2ring(const double *alm, int nmaps, int lmax, int nside,
                  const int *rings, int nring, double *F)
{
    const int mmax = lmax;
    const int64_t nalm = (int64_t)(lmax + 1) * (lmax + 2) / 2;
#pragma omp parallel
    {
        double *A = malloc(sizeof(double) * (lmax + 2));
        double *B = malloc(sizeof(double) * (lmax + 2));
        double *lam = malloc(sizeof(double) * (lmax + 2));
        double *mant = malloc(sizeof(double) * (mmax + 1));
        int *scl = malloc(sizeof(int) * (mmax + 1));
#pragma omp for schedule(dynamic)
        for (int r = 0; r < nring; ++r) {
            double z, sth, phi0;
            int nph;
            int64_t start;
            orc_ring_info(nside, rings[r], &z, &sth, &nph, &phi0, &start);
            lmm_table(mmax, sth, mant, scl);
            for (int m = 0; m <= mmax; ++m) {
                leg_coefs(m, lmax, A, B);
                leg_column(m, lmax, z, mant[m], scl[m], A, B, lam);
                for (int k = 0; k < nmaps; ++k) {
                    const double *a = alm + 2 * ((int64_t)k * nalm);
                    double re = 0.0, im = 0.0;
                    for (int l = m; l <= lmax; ++l) {
                        int64_t ix = alm_index(l, m, lmax);
                        re += a[2 * ix] * lam[l - m];
                        im += a[2 * ix + 1] * lam[l - m];
                    }
                    double *f = F + 2 * (((int64_t)k * nring + r) * (mmax + 1) + m);
                    f[0] = re;
                    f[1] = im;
                }
            }
        }
        free(A); free(B); free(lam); free(mant); free(scl);
    }
}

/*
 * Spin-0 analysis Legendre sums: alm[l,m] = sum_rings lambda_lm(z_r) G_m(r).
 * G: complex128 [nmaps][nring][mmax+1] (already weighted ring Fourier
 * coefficients); out alm complex128 [nmaps][nalm] (HEALPix order).
 */
void orc_ring2alm(const double *G, int nmaps, int lmax, int nside,
                  const int *rings, int nring, double *alm)
{
    const int mmax = lmax;
    const int64_t nalm = (int64_t)(lmax + 1) * (lmax + 2) / 2;
    memset(alm, 0, sizeof(double) * 2 * nalm * nmaps);
    double *sth = malloc(sizeof(double) * nring);
    double *z = malloc(sizeof(double) * nring);
    for (int r = 0; r < nring; ++r) {
        double phi0;
        int nph;
        int64_t start;
        orc_ring_info(nside, rings[r], &z[r], &sth[r], &nph, &phi0, &start);
    }
#pragma omp parallel
    {
        double *A = malloc(sizeof(double) * (lmax + 2));
        double *B = malloc(sizeof(double) * (lmax + 2));
        double *lam = malloc(sizeof(double) * (lmax + 2));
#pragma omp for schedule(dynamic)
        for (int m = 0; m <= mmax; ++m) {
            leg_coefs(m, lmax, A, B);
            for (int r = 0; r < nring; ++r) {
                /* lambda_mm at this ring directly (product form, scaled) */
                double v = 1.0 / sqrt(4.0 * M_PI);
                int sc = 0;
                for (int k = 1; k <= m; ++k) {
                    v *= -sth[r] * sqrt((2.0 * k + 1.0) / (2.0 * k));
                    if (fabs(v) < TWO_M400) { v *= TWO_P800; sc -= 1; }
                }
                leg_column(m, lmax, z[r], v, sc, A, B, lam);
                for (int k = 0; k < nmaps; ++k) {
                    const double *g = G + 2 * (((int64_t)k * nring + r) * (mmax + 1) + m);
                    double *a = alm + 2 * ((int64_t)k * nalm);
                    for (int l = m; l <= lmax; ++l) {
                        int64_t ix = alm_index(l, m, lmax);
                        a[2 * ix] += lam[l - m] * g[0];
                        a[2 * ix + 1] += lam[l - m] * g[1];
                    }
                }
            }
        }
        free(A); free(B); free(lam);
    }
    free(sth); free(z);
}

/*
 * Spin-s (s = 1, 2) synthesis Legendre sums for E/B input.  Produces, per
 * ring and m, the Fourier coefficients Q_m and U_m such that
 *   Q(phi) = Re sum_m c_m Q_m e^{i m phi},  U(phi) = Re sum_m c_m U_m e^{i m phi}
 * with c_0 = 1, c_m = 2.  Uses lambda^+ = (sY + (-1)^s (-s)Y)/2 and
 * lambda^- = (sY - (-1)^s (-s)Y)/2 (theta parts), obtained from lambda_lm,
 * lambda_{l-1,m} and the eth / eth-bar operators:
 *   s = 1: N lambda^+ = -dlambda/dtheta, N lambda^- = m lambda / sin(theta),
 *          N = sqrt(l(l+1));
 *   s = 2: N lambda^+ = -2 cot(theta) dlambda/dtheta + (2 m^2/sin^2 - l(l+1)) lambda,
 *          N lambda^- = (2m / sin theta)(cot(theta) lambda - dlambda/dtheta),
 *          N = sqrt((l-1) l (l+1) (l+2)),
 * with sin(theta) dlambda_lm/dtheta = l x lambda_lm
 *          - sqrt((2l+1)/(2l-1) (l^2-m^2)) lambda_{l-1,m}.
 * Then Q_m = -sum_l lambda^+ E_lm - i sum_l lambda^- B_lm,
 *      U_m =  i sum_l lambda^- E_lm - sum_l lambda^+ B_lm.
 * blm may be NULL (zero B).  Output QU: complex128 [2][nring][mmax+1].
 */
void orc_alm2ring_spin(const double *elm, const double *blm, int spin, int lmax,
                       int nside, const int *rings, int nring, double *QU)
{
    const int mmax = lmax;
#pragma omp parallel
    {
        double *A = malloc(sizeof(double) * (lmax + 2));
        double *B = malloc(sizeof(double) * (lmax + 2));
        double *lam = malloc(sizeof(double) * (lmax + 2));
        double *mant = malloc(sizeof(double) * (mmax + 1));
        int *scl = malloc(sizeof(int) * (mmax + 1));
#pragma omp for schedule(dynamic)
        for (int r = 0; r < nring; ++r) {
            double x, sth, phi0;
            int nph;
            int64_t start;
            orc_ring_info(nside, rings[r], &x, &sth, &nph, &phi0, &start);
            lmm_table(mmax, sth, mant, scl);
            double cot = x / sth;
            for (int m = 0; m <= mmax; ++m) {
                leg_coefs(m, lmax, A, B);
                leg_column(m, lmax, x, mant[m], scl[m], A, B, lam);
                double pEr = 0, pEi = 0, mEr = 0, mEi = 0;
                double pBr = 0, pBi = 0, mBr = 0, mBi = 0;
                for (int l = (m > spin ? m : spin); l <= lmax; ++l) {
                    double lam_l = lam[l - m];
                    double lam_lm1 = (l - 1 >= m) ? lam[l - 1 - m] : 0.0;
                    double fl = l, fm = m;
                    double d = (fl * x * lam_l -
                                sqrt((2 * fl + 1) / (2 * fl - 1) * (fl * fl - fm * fm)) * lam_lm1) / sth;
                    double lp, lmn;
                    if (spin == 1) {
                        double nrm = 1.0 / sqrt(fl * (fl + 1));
                        lp = -d * nrm;
                        lmn = fm * lam_l / sth * nrm;
                    } else {
                        double nrm = 1.0 / sqrt((fl - 1) * fl * (fl + 1) * (fl + 2));
                        lp = (-2.0 * cot * d + (2.0 * fm * fm / (sth * sth) - fl * (fl + 1)) * lam_l) * nrm;
                        lmn = (2.0 * fm / sth) * (cot * lam_l - d) * nrm;
                    }
                    int64_t ix = alm_index(l, m, lmax);
                    pEr += lp * elm[2 * ix]; pEi += lp * elm[2 * ix + 1];
                    mEr += lmn * elm[2 * ix]; mEi += lmn * elm[2 * ix + 1];
                    if (blm) {
                        pBr += lp * blm[2 * ix]; pBi += lp * blm[2 * ix + 1];
                        mBr += lmn * blm[2 * ix]; mBi += lmn * blm[2 * ix + 1];
                    }
                }
                double *q = QU + 2 * (((int64_t)0 * nring + r) * (mmax + 1) + m);
                double *u = QU + 2 * (((int64_t)1 * nring + r) * (mmax + 1) + m);
                /* Q_m = -(pE) - i (mB) ; U_m = i (mE) - (pB) */
                q[0] = -pEr + mBi;
                q[1] = -pEi - mBr;
                u[0] = -mEi - pBr;
                u[1] = mEr - pBi;
            }
        }
        free(A); free(B); free(lam); free(mant); free(scl);
    }
}

/* ---------------------------------------------------------------- iternorm */

/*
 * Restatement of glass/fields.py:101-188 (iternorm) for a stack of nl
 * independent covariance problems (one per angular mode l), processed for
 * nrows rows (fields) in sequence.  cov: [nrows][nl][k+1] (row i gives, for
 * each l, [C_ii, C_i,i-1, ..., C_i,i-k]); w: same shape, w = [a..., s].
 * Fixed summation order, explicit fma: the GPU kernel follows the same
 * order and is compared bit for bit.  Returns -1 on success, else the first
 * row whose variance went negative ("covariance matrix is not positive
 * definite", glass/fields.py:180-181).
 *
 * State per l: m (k x k), a (k), s.  Row update (glass/fields.py:143-169):
 *   atm = a^T m ; new last row = [-atm, u] / s' (u = s>0, s' = s>0 ? s : 1);
 *   m <- last k rows/cols of [[m, 0], [row]] ;
 *   a = m c with c = reversed(cov[1:]) ; s = sqrt(cov[0] - a.a).
 */
long orc_iternorm(const double *cov, long nrows, long nl, int k, double *w)
{
    /* After the update of row i only the trailing z = min(i, k) rows and
     * columns of m (and entries of a) can be non-zero; every sum starts at
     * the first index of that block.  The terms skipped are exact zeros, so
     * the result is the same as summing over all k indices. */
    long bad = -1;
    const int kp = k + 1;
    for (long l = 0; l < nl; ++l) {
        double *m = calloc((size_t)(k > 0 ? k * k : 1), sizeof(double));
        double *mn = calloc((size_t)(k > 0 ? k * k : 1), sizeof(double));
        double *a = calloc((size_t)(k > 0 ? k : 1), sizeof(double));
        double *atm = calloc((size_t)(k > 0 ? k : 1), sizeof(double));
        double s = 1.0;
        for (long i = 0; i < nrows; ++i) {
            const double *row = cov + ((size_t)i * nl + l) * kp;
            const int z = i < k ? (int)i : k, zp = i - 1 < k ? (int)(i - 1) : k;
            const int lo = k - z, lop = k - (zp > 0 ? zp : 0);
            if (i > 0 && k > 0) {
                /* atm_j = sum_p a_p m[p][j] (p ascending) */
                for (int j = 0; j < k; ++j) {
                    double acc = 0.0;
                    if (j >= lop)
                        for (int p = lop; p < k; ++p) acc = fma(a[p], m[p * k + j], acc);
                    atm[j] = acc;
                }
                double u = s > 0 ? 1.0 : 0.0;
                double sd = s > 0 ? s : 1.0;
                /* new matrix (k+1)x(k+1) = [[m,0],[-atm,u]]/..., keep last k rows/cols:
                 * rows 1..k-1 of old m shifted up, columns 1..k of extended. */
                for (int r = 0; r < k - 1; ++r)
                    for (int c = 0; c < k; ++c)
                        mn[r * k + c] = (c + 1 < k) ? m[(r + 1) * k + (c + 1)] : 0.0;
                for (int c = 0; c < k; ++c) {
                    double v = (c + 1 < k) ? -atm[c + 1] : u;
                    mn[(k - 1) * k + c] = v / sd;
                }
                double *t = m; m = mn; mn = t;
            }
            /* a = m c, c_j = row[k - j] (reversed, oldest first) */
            double aa = 0.0;
            for (int r = 0; r < k; ++r) {
                double acc = 0.0;
                if (r >= lo)
                    for (int c = lo; c < k; ++c) acc = fma(m[r * k + c], row[k - c], acc);
                a[r] = acc;
            }
            for (int r = lo; r < k; ++r) aa = fma(a[r], a[r], aa);
            double sv = row[0] - aa;
            if (sv < 0) {
                if (bad < 0 || i < bad) bad = i;
                sv = 0.0;
            }
            s = sqrt(sv);
            double *wo = w + ((size_t)i * nl + l) * kp;
            for (int r = 0; r < k; ++r) wo[r] = a[r];
            wo[k] = s;
        }
        free(m); free(mn); free(a); free(atm);
    }
    return bad;
}

/*
 * The same iternorm with every sum over all k indices (no block restriction):
 * the straightforward form, against which the block-restricted sums of
 * orc_iternorm (and of the GPU kernel) are checked bit for bit.
 */
long orc_iternorm_dense(const double *cov, long nrows, long nl, int k, double *w)
{
    long bad = -1;
    const int kp = k + 1;
    for (long l = 0; l < nl; ++l) {
        double *m = calloc((size_t)(k > 0 ? k * k : 1), sizeof(double));
        double *mn = calloc((size_t)(k > 0 ? k * k : 1), sizeof(double));
        double *a = calloc((size_t)(k > 0 ? k : 1), sizeof(double));
        double *atm = calloc((size_t)(k > 0 ? k : 1), sizeof(double));
        double s = 1.0;
        for (long i = 0; i < nrows; ++i) {
            const double *row = cov + ((size_t)i * nl + l) * kp;
            if (i > 0 && k > 0) {
                for (int j = 0; j < k; ++j) {
                    double acc = 0.0;
                    for (int p = 0; p < k; ++p) acc = fma(a[p], m[p * k + j], acc);
                    atm[j] = acc;
                }
                double u = s > 0 ? 1.0 : 0.0;
                double sd = s > 0 ? s : 1.0;
                for (int r = 0; r < k - 1; ++r)
                    for (int c = 0; c < k; ++c)
                        mn[r * k + c] = (c + 1 < k) ? m[(r + 1) * k + (c + 1)] : 0.0;
                for (int c = 0; c < k; ++c) {
                    double v = (c + 1 < k) ? -atm[c + 1] : u;
                    mn[(k - 1) * k + c] = v / sd;
                }
                double *t = m; m = mn; mn = t;
            }
            double aa = 0.0;
            for (int r = 0; r < k; ++r) {
                double acc = 0.0;
                for (int c = 0; c < k; ++c) acc = fma(m[r * k + c], row[k - c], acc);
                a[r] = acc;
            }
            for (int r = 0; r < k; ++r) aa = fma(a[r], a[r], aa);
            double sv = row[0] - aa;
            if (sv < 0) {
                if (bad < 0 || i < bad) bad = i;
                sv = 0.0;
            }
            s = sqrt(sv);
            double *wo = w + ((size_t)i * nl + l) * kp;
            for (int r = 0; r < k; ++r) wo[r] = a[r];
            wo[k] = s;
        }
        free(m); free(mn); free(a); free(atm);
    }
    return bad;
}

/* ------------------------------------------------------------------ philox */

static inline uint32_t mulhilo32(uint32_t a, uint32_t b, uint32_t *hi)
{
    uint64_t p = (uint64_t)a * b;
    *hi = (uint32_t)(p >> 32);
    return (uint32_t)p;
}

/* Philox4x32-10 block: counter c[4], key k[2] -> out[4]. */
void orc_philox4x32_10(const uint32_t c_in[4], const uint32_t k_in[2], uint32_t out[4])
{
    uint32_t c0 = c_in[0], c1 = c_in[1], c2 = c_in[2], c3 = c_in[3];
    uint32_t k0 = k_in[0], k1 = k_in[1];
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, hi1;
        uint32_t lo0 = mulhilo32(0xD2511F53u, c0, &hi0);
        uint32_t lo1 = mulhilo32(0xCD9E8D57u, c2, &hi1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/*
 * Standard complex normals of the GPU stream: element e of stream `sid`
 * under key `seed` is one Philox block with counter (e_lo, e_hi, sid_lo,
 * sid_hi) and key (seed_lo, seed_hi); 53-bit uniforms
 * u1 = ((x0>>5)*2^26 + (x1>>6) + 0.5) 2^-53 in (0,1), u2 likewise from x2, x3;
 * z = sqrt(-2 ln u1) (cos 2 pi u2 + i sin 2 pi u2).
 * raw (optional): uint32 [n][4] Philox outputs for bit-exact checks.
 */
void orc_philox_normals(uint64_t seed, uint64_t sid, int64_t offset, int64_t n,
                        double *z, uint32_t *raw)
{
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int64_t i = 0; i < n; ++i) {
        uint64_t e = (uint64_t)(offset + i);
        uint32_t c[4] = {(uint32_t)e, (uint32_t)(e >> 32), (uint32_t)sid, (uint32_t)(sid >> 32)};
        uint32_t x[4];
        orc_philox4x32_10(c, key, x);
        if (raw) memcpy(raw + 4 * i, x, sizeof(x));
        double u1 = ((double)(x[0] >> 5) * 67108864.0 + (double)(x[1] >> 6) + 0.5) * 1.1102230246251565e-16;
        double u2 = ((double)(x[2] >> 5) * 67108864.0 + (double)(x[3] >> 6) + 0.5) * 1.1102230246251565e-16;
        double r = sqrt(-2.0 * log(u1));
        z[2 * i] = r * cos(2.0 * M_PI * u2);
        z[2 * i + 1] = r * sin(2.0 * M_PI * u2);
    }
}

/* ---------------------------------------------------------- poisson */

/*
 * Per-pixel Poisson counts of glass/points.py:252-348 (expected count
 * n = ((b delta - offset) + 1) scale [* vis], clipped at 0, one Poisson draw
 * per pixel), restating the GPU kernel's exact operation sequence so the
 * counts agree bit for bit.  e^{-x} is a Cody-Waite reduction plus a degree-13
 * Taylor polynomial (no libm), every step a single rounded FP64 operation
 * (this file is built with -ffp-contract=off).  Poisson(n) is a sum of
 * pieces of mean <= 256 (Poisson additivity), each drawn by sequential
 * inversion from one 53-bit uniform (p_k = (p_{k-1} lam) (1/k), 1/k the
 * correctly rounded reciprocal); piece c of pixel e uses words
 * 2(c&1), 2(c&1)+1 of the Philox block with counter (e_lo, e_hi, sid, c>>1).
 */
double orc_exp_neg(double x)
{
    const double inv_ln2 = 0x1.71547652b82fep+0;
    const double ln2_hi = 0x1.62e42fee00000p-1, ln2_lo = 0x1.a39ef35793c76p-33;
    static const double c[14] = {
        0x1.0000000000000p+0, 0x1.0000000000000p+0, 0x1.0000000000000p-1, 0x1.5555555555555p-3,
        0x1.5555555555555p-5, 0x1.1111111111111p-7, 0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13,
        0x1.a01a01a01a01ap-16, 0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
        0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33};
    double kd = floor(x * inv_ln2 + 0.5);
    double r = (x - kd * ln2_hi) - kd * ln2_lo;
    double y = -r;
    double p = c[13];
    for (int i = 12; i >= 0; --i) p = p * y + c[i];
    return ldexp(p, -(int)kd);
}

static int64_t orc_poisson_piece(double lam, double u)
{
    double p = orc_exp_neg(lam), F = p;
    int64_t k = 0;
    while (u > F && p > 0.0 && k < (1 << 20)) {
        k += 1;
        p = (p * lam) * (1.0 / (double)k);
        F = F + p;
    }
    return k;
}

static double orc_u53(uint32_t a, uint32_t b)
{
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6) + 0.5) * 1.1102230246251565e-16;
}

void orc_poisson_counts(const double *delta, int64_t npix, double bias, double offset, double scale,
                        const double *vis, uint64_t seed, uint32_t sid, int64_t *counts)
{
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t e = 0; e < npix; ++e) {
        double n = ((bias * delta[e]) - offset) + 1.0;
        n = n * scale;
        if (vis) n = n * vis[e];
        double rest = n > 0.0 ? n : 0.0;
        int64_t total = 0;
        uint32_t x[4] = {0, 0, 0, 0};
        for (uint32_t c = 0; rest > 0.0; ++c) {
            double lam = rest > 256.0 ? 256.0 : rest;
            rest = rest - lam;
            if ((c & 1u) == 0u) {
                uint32_t ctr[4] = {(uint32_t)e, (uint32_t)((uint64_t)e >> 32), sid, c >> 1};
                orc_philox4x32_10(ctr, key, x);
            }
            double u = (c & 1u) ? orc_u53(x[2], x[3]) : orc_u53(x[0], x[1]);
            total += orc_poisson_piece(lam, u);
        }
        counts[e] = total;
    }
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
