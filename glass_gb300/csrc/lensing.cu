// Map-level kernels: the multi-plane convergence update
// (glass/lensing.py:511-586, MultiPlaneConvergence.add_plane), the galaxy
// shear gather (glass/galaxies.py:271-347, galaxy_shear) with the HEALPix
// RING-scheme ang2pix it needs (glass/healpix.py ang2pix, healpy's published
// pixelisation, Gorski et al. 2005, ApJ 622, 759), and the positions of
// counted galaxies inside their pixels (glass/points.py:351-440, the
// healpy.randang sampling of positions_from_delta).
//
// Every floating-point step is an explicitly rounded operation in the order
// numpy evaluates the reference's expressions, so FP64 results are those of
// the reference on the same inputs.
#include <cuda_runtime.h>
#include <math.h>

#include "glg_internal.cuh"
#include "philox.cuh"

namespace {

// kappa3 <- kappa3 * (1 - t); kappa3 += t * kappa2; kappa3 += f * delta2
// (glass/lensing.py:579-581).  Each in-place step rounds to the map's type;
// the products are taken in FP64 (numpy promotes the 0-d float64 scalars).
template <typename T>
__global__ void k_convergence_step(T *__restrict__ k3, const T *__restrict__ k2, const T *__restrict__ d2,
                                   int64_t n, double omt, double t, double f) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        T a = (T)__dmul_rn((double)k3[i], omt);
        a = (T)__dadd_rn((double)a, __dmul_rn(t, (double)k2[i]));
        const double dd = d2 ? (double)d2[i] : 0.0;
        a = (T)__dadd_rn((double)a, __dmul_rn(f, dd));
        k3[i] = a;
    }
}

// RING-scheme pixel of a position given as z = cos(theta), sin(theta) and
// phi (Gorski et al. 2005, eqs. for the polar caps and the equatorial belt);
// near the poles the cap formula uses sin(theta) for accuracy, like the
// HEALPix library.
__device__ __forceinline__ int64_t ang2pix_zphi(int64_t nside, double z, double sth, double phi) {
    const double za = fabs(z);
    const double twopi = 6.283185307179586476925286766559;
    double ph = fmod(phi, twopi);
    if (ph < 0.0) ph += twopi;
    const double tt = ph * 0.63661977236758134308;  // 2 / pi: tt in [0, 4)
    const int64_t ncap = 2 * nside * (nside - 1), npix = 12 * nside * nside;
    if (za <= 2.0 / 3.0) {
        const double t1 = nside * (0.5 + tt), t2 = nside * (z * 0.75);
        const int64_t jp = (int64_t)(t1 - t2), jm = (int64_t)(t1 + t2);
        const int64_t ir = nside + 1 + jp - jm;  // 1 .. 2 nside + 1
        const int64_t kshift = 1 - (ir & 1);
        int64_t ip = (jp + jm - nside + kshift + 1) / 2;
        ip %= 4 * nside;
        if (ip < 0) ip += 4 * nside;
        return ncap + (ir - 1) * 4 * nside + ip;
    }
    const double tp = tt - (double)(int64_t)tt;
    const double tmp = za < 0.99 ? nside * sqrt(3.0 * (1.0 - za)) : nside * sth / sqrt((1.0 + za) / 3.0);
    const int64_t jp = (int64_t)(tp * tmp), jm = (int64_t)((1.0 - tp) * tmp);
    const int64_t ir = jp + jm + 1;  // ring number counted from the closer pole
    int64_t ip = (int64_t)(tt * ir);
    ip %= 4 * ir;
    if (ip < 0) ip += 4 * ir;
    return z > 0 ? 2 * ir * (ir - 1) + ip : npix - 2 * ir * (ir + 1) + ip;
}

__device__ __forceinline__ int64_t ang2pix_ring(int64_t nside, double theta, double phi) {
    return ang2pix_zphi(nside, cos(theta), sin(theta), phi);
}

__device__ __forceinline__ void lonlat_to_thetaphi(double lon, double lat, double &theta, double &phi) {
    const double d2r = 0.017453292519943295769236907684886;  // pi / 180
    theta = __dsub_rn(1.5707963267948966192313216916398, __dmul_rn(lat, d2r));
    phi = __dmul_rn(lon, d2r);
}

__global__ void k_ang2pix(int64_t nside, const double *__restrict__ lon, const double *__restrict__ lat,
                          int64_t n, int lonlat, int64_t *__restrict__ ipix) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double theta = lon[i], phi = lat[i];  // (theta, phi) unless lonlat
        if (lonlat) lonlat_to_thetaphi(lon[i], lat[i], theta, phi);
        ipix[i] = ang2pix_ring(nside, theta, phi);
    }
}

// numpy's complex128 division (Smith's method with a reciprocal scale).
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    const double br = fabs(b.x), bi = fabs(b.y);
    if (br >= bi) {
        if (br == 0.0 && bi == 0.0) return make_double2(a.x / br, a.y / br);
        const double rat = b.y / b.x;
        const double scl = 1.0 / __dadd_rn(b.x, __dmul_rn(b.y, rat));
        return make_double2(__dmul_rn(__dadd_rn(a.x, __dmul_rn(a.y, rat)), scl),
                            __dmul_rn(__dsub_rn(a.y, __dmul_rn(a.x, rat)), scl));
    }
    const double rat = b.x / b.y;
    const double scl = 1.0 / __dadd_rn(b.y, __dmul_rn(b.x, rat));
    return make_double2(__dmul_rn(__dadd_rn(__dmul_rn(a.x, rat), a.y), scl),
                        __dmul_rn(__dsub_rn(__dmul_rn(a.y, rat), a.x), scl));
}

// Lensed ellipticity of galaxy i (glass/galaxies.py:325-345): gather kappa,
// gamma at the galaxy's pixel, g = gamma / (1 - kappa), eps' = (eps + g) /
// (1 + conj(g) eps); or eps + gamma without reduced shear.
template <typename T>
__global__ void k_galaxy_shear(int64_t nside, const double *__restrict__ lon, const double *__restrict__ lat,
                               const double2 *__restrict__ eps, int64_t n, const T *__restrict__ kappa,
                               const T *__restrict__ g1, const T *__restrict__ g2, int reduced,
                               double2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double theta, phi;
        lonlat_to_thetaphi(lon[i], lat[i], theta, phi);
        const int64_t p = ang2pix_ring(nside, theta, phi);
        const double k = (double)kappa[p];
        double2 g = make_double2((double)g1[p], (double)g2[p]);
        const double2 e = eps[i];
        if (reduced) {
            g = cdiv(g, make_double2(__dsub_rn(1.0, k), 0.0));
            // 1 + conj(g) * eps
            const double pr = __dsub_rn(__dmul_rn(g.x, e.x), __dmul_rn(-g.y, e.y));
            const double pi = __dadd_rn(__dmul_rn(g.x, e.y), __dmul_rn(-g.y, e.x));
            g = cdiv(make_double2(__dadd_rn(e.x, g.x), __dadd_rn(e.y, g.y)), make_double2(__dadd_rn(1.0, pr), pi));
        } else {
            g = make_double2(__dadd_rn(g.x, e.x), __dadd_rn(g.y, e.y));
        }
        out[i] = g;
    }
}

// z of ring r (1 .. 4 nside - 1) of the RING scheme.
__device__ __forceinline__ double ring_z(int64_t nside, int64_t r) {
    const double ns = (double)nside;
    if (r < nside) return 1.0 - (double)(r * r) / (3.0 * ns * ns);
    if (r <= 3 * nside) return (4.0 / 3.0) - 2.0 * (double)r / (3.0 * ns);
    const int64_t q = 4 * nside - r;
    return (double)(q * q) / (3.0 * ns * ns) - 1.0;
}

__device__ __forceinline__ int64_t isqrt64(int64_t v) {
    int64_t q = (int64_t)sqrt((double)v);
    while (q * q > v) --q;
    while ((q + 1) * (q + 1) <= v) ++q;
    return q;
}

// Ring r, position j and ring length nph of RING pixel p.
__device__ __forceinline__ void pix_ring(int64_t nside, int64_t p, int64_t &r, int64_t &j, int64_t &nph) {
    const int64_t ncap = 2 * nside * (nside - 1), npix = 12 * nside * nside;
    if (p < ncap) {
        r = (1 + isqrt64(1 + 2 * p)) / 2;
        j = p - 2 * r * (r - 1);
        nph = 4 * r;
    } else if (p < npix - ncap) {
        const int64_t q = p - ncap;
        r = q / (4 * nside) + nside;
        j = q % (4 * nside);
        nph = 4 * nside;
    } else {
        const int64_t q = npix - 1 - p;
        const int64_t rs = (1 + isqrt64(1 + 2 * q)) / 2;
        r = 4 * nside - rs;
        nph = 4 * rs;
        j = nph - 1 - (q - 2 * rs * (rs - 1));
    }
}

// Galaxy g of the count map: its pixel is the p with off[p] <= g < off[p+1]
// (off = exclusive prefix sums of the counts); its position is uniform on
// the pixel's area: (z, phi) uniform in the box that holds the pixel (z
// between the centres of rings r+1 and r-1, phi within half a pixel width of
// the centre; uniform in z and phi is uniform on the sphere, and the pixel
// fills half of the box), drawn from the Philox stream (counter g, sid,
// attempt) until ang2pix puts it in p.  Output longitude in [0, 360) and
// latitude in degrees, as healpy.randang(..., lonlat=True) returns them.
__global__ void k_positions(int64_t nside, const int64_t *__restrict__ off, int64_t npix, int64_t n0, int64_t n,
                            uint64_t seed, uint32_t sid, double *__restrict__ lon, double *__restrict__ lat,
                            unsigned long long *__restrict__ misses) {
    const double twopi = 6.283185307179586476925286766559;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = n0 + i;
        int64_t lo = 0, hi = npix;  // last p with off[p] <= g
        while (hi - lo > 1) {
            const int64_t mid = (lo + hi) >> 1;
            if (off[mid] <= g) lo = mid;
            else hi = mid;
        }
        const int64_t p = lo;
        int64_t r, j, nph;
        pix_ring(nside, p, r, j, nph);
        const double zhi = r == 1 ? 1.0 : ring_z(nside, r - 1);
        const double zlo = r == 4 * nside - 1 ? -1.0 : ring_z(nside, r + 1);
        const bool shifted = r < nside || r > 3 * nside || ((r - nside) & 1) == 0;
        const double dphi = twopi / (double)nph;
        const double phic = ((double)j + (shifted ? 0.5 : 0.0)) * dphi;
        double z = ring_z(nside, r), phi = phic;
        bool ok = false;
        for (uint32_t t = 0; t < 64 && !ok; ++t) {
            const glg_rng::U4 x = glg_rng::philox4x32_10((uint32_t)g, (uint32_t)(g >> 32), sid, t, (uint32_t)seed,
                                                         (uint32_t)(seed >> 32));
            const double u1 = glg_rng::u53(x.x, x.y), u2 = glg_rng::u53(x.z, x.w);
            const double zz = zlo + u1 * (zhi - zlo);
            const double pp = phic + (u2 - 0.5) * dphi;
            if (ang2pix_zphi(nside, zz, sqrt((1.0 - zz) * (1.0 + zz)), pp) == p) {
                z = zz;
                phi = pp;
                ok = true;
            }
        }
        if (!ok) atomicAdd(misses, 1ull);
        double ph = fmod(phi, twopi);
        if (ph < 0.0) ph += twopi;
        lon[i] = ph * 57.295779513082320876798154814105;
        lat[i] = asin(z) * 57.295779513082320876798154814105;
    }
}

unsigned grid_of(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (unsigned)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
}

}  // namespace

extern "C" int glg_convergence_step(void *kappa3, const void *kappa2, const void *delta2, int dtype, int64_t n,
                                    double t, double f, void *stream) {
    GLG_REQUIRE(dtype == GLG_F64 || dtype == GLG_F32, "glg_convergence_step: bad dtype");
    GLG_REQUIRE(n >= 0, "glg_convergence_step: negative size");
    if (n == 0) return GLG_OK;
    GLG_REQUIRE(kappa3 && kappa2, "glg_convergence_step: null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    const double omt = 1.0 - t;
    GLG_LAUNCH_SCOPE("k_convergence_step", st);
    if (dtype == GLG_F64)
        k_convergence_step<double><<<grid_of(n), 256, 0, st>>>((double *)kappa3, (const double *)kappa2,
                                                               (const double *)delta2, n, omt, t, f);
    else
        k_convergence_step<float><<<grid_of(n), 256, 0, st>>>((float *)kappa3, (const float *)kappa2,
                                                              (const float *)delta2, n, omt, t, f);
    GLG_CHECK_LAUNCH("k_convergence_step");
    return GLG_OK;
}

extern "C" int glg_ang2pix(int nside, const double *theta_or_lon, const double *phi_or_lat, int64_t n, int lonlat,
                           int64_t *ipix, void *stream) {
    GLG_REQUIRE(nside >= 1 && nside <= (1 << 29), "glg_ang2pix: bad nside");
    GLG_REQUIRE(n >= 0, "glg_ang2pix: negative size");
    if (n == 0) return GLG_OK;
    GLG_REQUIRE(theta_or_lon && phi_or_lat && ipix, "glg_ang2pix: null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    GLG_LAUNCH_SCOPE("k_ang2pix", st);
    k_ang2pix<<<grid_of(n), 256, 0, st>>>(nside, theta_or_lon, phi_or_lat, n, lonlat, ipix);
    GLG_CHECK_LAUNCH("k_ang2pix");
    return GLG_OK;
}

extern "C" int glg_galaxy_shear(const double *lon, const double *lat, const void *eps, int64_t n, const void *kappa,
                                const void *gamma1, const void *gamma2, int dtype, int nside, int reduced,
                                void *out, void *stream) {
    GLG_REQUIRE(dtype == GLG_F64 || dtype == GLG_F32, "glg_galaxy_shear: bad dtype");
    GLG_REQUIRE(nside >= 1 && n >= 0, "glg_galaxy_shear: bad size");
    if (n == 0) return GLG_OK;
    GLG_REQUIRE(lon && lat && eps && kappa && gamma1 && gamma2 && out, "glg_galaxy_shear: null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    GLG_LAUNCH_SCOPE("k_galaxy_shear", st);
    if (dtype == GLG_F64)
        k_galaxy_shear<double><<<grid_of(n), 256, 0, st>>>(nside, lon, lat, (const double2 *)eps, n,
                                                           (const double *)kappa, (const double *)gamma1,
                                                           (const double *)gamma2, reduced, (double2 *)out);
    else
        k_galaxy_shear<float><<<grid_of(n), 256, 0, st>>>(nside, lon, lat, (const double2 *)eps, n,
                                                          (const float *)kappa, (const float *)gamma1,
                                                          (const float *)gamma2, reduced, (double2 *)out);
    GLG_CHECK_LAUNCH("k_galaxy_shear");
    return GLG_OK;
}

extern "C" int glg_positions(int nside, const int64_t *offsets, int64_t first, int64_t n, uint64_t seed,
                             uint64_t sid, double *lon, double *lat, unsigned long long *misses, void *stream) {
    GLG_REQUIRE(nside >= 1 && nside <= (1 << 20), "glg_positions: bad nside");
    GLG_REQUIRE(first >= 0 && n >= 0, "glg_positions: negative size");
    GLG_REQUIRE(sid <= 0xFFFFFFFFull, "glg_positions: stream id must fit in 32 bits");
    if (n == 0) return GLG_OK;
    GLG_REQUIRE(offsets && lon && lat && misses, "glg_positions: null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    GLG_LAUNCH_SCOPE("k_positions", st);
    k_positions<<<grid_of(n), 256, 0, st>>>(nside, offsets, 12LL * nside * nside, first, n, seed, (uint32_t)sid,
                                            lon, lat, misses);
    GLG_CHECK_LAUNCH("k_positions");
    return GLG_OK;
}
