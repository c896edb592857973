// Fast form of the spin-s synthesis (alm2map_spin, glass/healpix.py:81-108,
// as called by from_convergence for the deflection and the shear,
// glass/lensing.py:337-368): split-precision TF32 contractions on the tensor
// cores, FP32 ring FFTs.
//
// Q_m = -sum_l lambda^+_l E_l - i sum_l lambda^-_l B_l,
// U_m =  i sum_l lambda^-_l E_l - sum_l lambda^+_l B_l.
// The two sums over lambda^+ and lambda^- are two launches of the fast
// contraction (k_leg_tc) with the plan's spin tables in place of the P_lm
// table and the E (then B) alm of every field as the B-operand columns.  Each
// launch leaves per ring pair the north sum (even + odd l - m) and the south
// sum (even - odd); the mirror relations lambda^+(pi - t) = (-1)^(l+m+s)
// lambda^+(t), lambda^-(pi - t) = -(-1)^(l+m+s) lambda^-(t) make the south
// ring's sums (-1)^s and -(-1)^s times those.  k_spin_combine applies the
// signs, forms Q_m and U_m and writes them transposed for the ring FFTs.
#include <cuda_runtime.h>

#include "glg_internal.cuh"

namespace {

size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

// Fp, Fm: [nc][m][ring], nc = nf (E only) or 2 nf (E rows, then B rows).
// Ft: [2 nf][ring][m], Q of field f at row f and U at row nf + f.
// 32 x 32 (ring, m) tiles through shared memory, like the plain transpose.
__global__ void k_spin_combine(const float2 *__restrict__ Fp, const float2 *__restrict__ Fm,
                               float2 *__restrict__ Ft, int nm, int nr, int npairs, int nf, int hasb, float sg) {
    __shared__ float2 tq[32][33], tu[32][33];
    const int f = blockIdx.z;
    const int r0 = blockIdx.x * 32, m0 = blockIdx.y * 32;
    const int64_t plane = (int64_t)nm * nr;
    const float2 *pE = Fp + f * plane, *mE = Fm + f * plane;
    const float2 *pB = Fp + (nf + f) * plane, *mB = Fm + (nf + f) * plane;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int y = threadIdx.y + 8 * i, m = m0 + y, r = r0 + threadIdx.x;
        float2 q = make_float2(0.f, 0.f), u = q;
        if (m < nm && r < nr) {
            const int64_t ix = (int64_t)m * nr + r;
            const bool south = r >= npairs;  // ring nr - 1 - p of pair p (the equator is north)
            const float sp = south ? sg : 1.f, sm = south ? -sg : 1.f;
            const float2 a = pE[ix], c = mE[ix];
            q = make_float2(-sp * a.x, -sp * a.y);  // -lambda^+ E
            u = make_float2(-sm * c.y, sm * c.x);   // i lambda^- E
            if (hasb) {
                const float2 b = pB[ix], d = mB[ix];
                q.x += sm * d.y;  // -i lambda^- B
                q.y -= sm * d.x;
                u.x -= sp * b.x;  // -lambda^+ B
                u.y -= sp * b.y;
            }
        }
        tq[y][threadIdx.x] = q;
        tu[y][threadIdx.x] = u;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, m = m0 + threadIdx.x;
        if (m < nm && r < nr) {
            Ft[((int64_t)f * nr + r) * nm + m] = tq[threadIdx.x][y];
            Ft[((int64_t)(nf + f) * nr + r) * nm + m] = tu[threadIdx.x][y];
        }
    }
}

// Workspace: status block | B pack | F+ | F- | Ft | class-3 ring buffers
// (nside > 2048), each 256-byte aligned.
struct SpinWs {
    int *err;
    float *bpack;
    float2 *Fp, *Fm, *Ft, *gz;
    char *end;
};
SpinWs spin_ws(const glg_plan *P, int nf, bool hasb, void *ws) {
    SpinWs w;
    char *c = (char *)ws;
    const int nc = hasb ? 2 * nf : nf;
    const size_t plane = sizeof(float2) * (size_t)P->nrings * (P->mmax + 1);
    w.err = (int *)c;
    c += GLG_WS_STATUS_BYTES;
    w.bpack = (float *)c;
    c += up256(glg_leg_tc_pack_bytes(P, nc));
    w.Fp = (float2 *)c;
    c += up256(plane * nc);
    w.Fm = (float2 *)c;
    c += up256(plane * nc);
    w.Ft = (float2 *)c;
    c += up256(plane * 2 * nf);
    const size_t gzb = glg_ring_gz_bytes(P->nside);
    w.gz = gzb ? (float2 *)c : nullptr;
    c += up256(gzb);
    c += 256;  // slack: the staged ring FFTs copy whole 16-byte words around each row of Ft
    w.end = c;
    return w;
}

}  // namespace

extern "C" size_t glg_alm2map_spin_fast_workspace(const glg_plan *P, int nfields, int with_b) {
    if (!P || nfields <= 0 || nfields > 20) return 0;
    char base[1];
    return (size_t)(spin_ws(P, nfields, with_b != 0, base).end - base);
}

extern "C" int glg_alm2map_spin_fast(const glg_plan *P, const void *elm, const void *blm, int nfields, int spin,
                                     void *qu, void *ws, size_t ws_bytes, void *stream) {
    GLG_REQUIRE(P != nullptr, "glg_alm2map_spin_fast: null plan");
    GLG_REQUIRE(spin == 1 || spin == 2, "glg_alm2map_spin_fast: spin must be 1 or 2");
    GLG_REQUIRE(nfields >= 0 && nfields <= 20, "glg_alm2map_spin_fast: nfields must be in [0, 20]");
    if (nfields == 0) return GLG_OK;
    GLG_REQUIRE(elm && qu, "glg_alm2map_spin_fast: null pointer");
    const bool hasb = blm != nullptr;
    GLG_REQUIRE(ws && ws_bytes >= glg_alm2map_spin_fast_workspace(P, nfields, hasb),
                "glg_alm2map_spin_fast: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    glg_plan *Pm = const_cast<glg_plan *>(P);
    int rc = glg_plan_prepare_fast(Pm, st);
    if (!rc) rc = glg_plan_prepare_spin(Pm, spin, st);
    if (rc) return rc;
    const SpinWs w = spin_ws(P, nfields, hasb, ws);
    cudaError_t e = cudaMemsetAsync(w.err, 0, GLG_WS_STATUS_BYTES, st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_alm2map_spin_fast: status reset");
    const int nc = hasb ? 2 * nfields : nfields;
    const int k = spin - 1, ntiles = (P->npairs + 127) / 128;
    const float2 *E = (const float2 *)elm, *B = (const float2 *)blm;
    rc = glg_launch_leg_tc_ex(P, E, B, nfields, nc, w.bpack, w.Fp, w.err, glg_tile_run{0, ntiles, 0, true},
                              P->plm_spin[k][0], P->tfirst_spin[k], st);
    if (!rc)
        rc = glg_launch_leg_tc_ex(P, E, B, nfields, nc, w.bpack, w.Fm, w.err, glg_tile_run{0, ntiles, 1, false},
                                  P->plm_spin[k][1], P->tfirst_spin[k], st);
    if (rc) return rc;
    {
        const int nm = P->mmax + 1, nr = P->nrings;
        dim3 grid((nr + 31) / 32, (nm + 31) / 32, nfields);
        GLG_LAUNCH_SCOPE("k_spin_combine", st);
        k_spin_combine<<<grid, dim3(32, 8), 0, st>>>(w.Fp, w.Fm, w.Ft, nm, nr, P->npairs, nfields, hasb ? 1 : 0,
                                                     (spin & 1) ? -1.f : 1.f);
        GLG_CHECK_LAUNCH("k_spin_combine");
    }
    glg_refine_list rl{nullptr, 0, nullptr, w.gz, w.err};
    return glg_launch_ring_syn_f32_range(P, nullptr, w.Ft, 2 * nfields, (float *)qu, nullptr, 0, P->npairs, &rl,
                                         st);
}
