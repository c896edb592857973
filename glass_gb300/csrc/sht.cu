// C-ABI entry points of the spherical-harmonic transforms (plain FP64 form):
// alm2map, alm2map_spin and map2alm, built from the Legendre and ring-FFT
// launches.  Every call works in caller-provided device workspace.
#include <cuda_runtime.h>

#include "glg_internal.cuh"

namespace {

__global__ void k_residual(const double *__restrict__ f, double *__restrict__ r, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        r[i] = f[i] - r[i];
}

size_t ring_coef_bytes(const glg_plan *P, int nmaps) {
    return sizeof(double2) * (size_t)nmaps * P->nrings * (P->mmax + 1);
}
size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

// Plain-form workspaces end with the FP64 ring FFTs' global ring buffers
// (nside > 2048 only; none below).
void *ring_gbuf(const glg_plan *P, void *ws, size_t before) {
    return glg_ring64_gbuf_bytes(P) ? (char *)ws + up256(before) : nullptr;
}
size_t with_gbuf(const glg_plan *P, size_t before) {
    const size_t g = glg_ring64_gbuf_bytes(P);
    return g ? up256(before) + g : before;
}

}  // namespace

static size_t fast_pack_bytes(const glg_plan *P, int nmaps) {
    // group counts are fixed by (lmax); the tables need not exist yet
    int64_t ng = 0;
    for (int m = 0; m <= P->lmax; ++m) ng += (P->lmax - m + GLG_GROUP) / GLG_GROUP;
    const int N = ((2 * nmaps + 15) / 16) * 16;
    return (size_t)ng * 128 * N;
}

// Fast-form workspace: status block | B pack | F [map][m][ring] |
// F [map][ring][m] | tail-refinement header (256 B) and list.
namespace {
constexpr int kRefinePerMap = 65536;  // listed pixels per map of a call
struct FastWs {
    int *err;
    float *bpack;
    float2 *F, *Ft;
    glg_refine_list rl;
    char *end;
};
// Offsets from the workspace's start (256-byte aligned blocks: the lists'
// int4 items and the staged maps' float4 stores need 16-byte alignment).
FastWs fast_ws(const glg_plan *P, int nmaps, void *ws) {
    FastWs w;
    char *c = (char *)ws;
    const size_t fb = up256(sizeof(float2) * (size_t)nmaps * P->nrings * (P->mmax + 1));
    w.err = (int *)c;
    c += GLG_WS_STATUS_BYTES;
    w.bpack = (float *)c;
    c += up256(fast_pack_bytes(P, nmaps));
    w.F = (float2 *)c;
    c += fb;
    w.Ft = (float2 *)c;
    c += fb;
    w.rl.hdr = (int *)c;
    w.rl.cap = kRefinePerMap * nmaps;
    c += 256;
    w.rl.items = (int4 *)c;
    c += up256(sizeof(int4) * (size_t)w.rl.cap);
    const size_t gzb = glg_ring_gz_bytes(P->nside);
    w.rl.gz = gzb ? (float2 *)c : nullptr;
    w.rl.err = w.err;
    c += up256(gzb);
    w.end = c;
    return w;
}
size_t fast_ws_bytes(const glg_plan *P, int nmaps) {
    char base[1];
    return (size_t)(fast_ws(P, nmaps, base).end - base);
}
}  // namespace

extern "C" size_t glg_alm2map_workspace(const glg_plan *P, int nmaps, int form) {
    if (!P || nmaps <= 0) return 0;
    if (form == GLG_FORM_FAST) return fast_ws_bytes(P, nmaps);
    return with_gbuf(P, ring_coef_bytes(P, nmaps));
}

extern "C" int glg_alm2map(const glg_plan *P, const void *alm, int nmaps, int form, void *maps,
                           const glg_epilogue *epi, void *ws, size_t ws_bytes, void *stream) {
    GLG_REQUIRE(P != nullptr, "glg_alm2map: null plan");
    GLG_REQUIRE(nmaps >= 0, "glg_alm2map: negative nmaps");
    if (nmaps == 0) return GLG_OK;
    GLG_REQUIRE(alm && maps, "glg_alm2map: null pointer");
    GLG_REQUIRE(form == GLG_FORM_PLAIN || form == GLG_FORM_FAST, "glg_alm2map: unknown form");
    GLG_REQUIRE(ws && ws_bytes >= glg_alm2map_workspace(P, nmaps, form),
                "glg_alm2map: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    if (form == GLG_FORM_FAST) {
        GLG_REQUIRE(nmaps <= 40, "glg_alm2map: the fast form takes at most 40 maps per call");
        int rc = glg_plan_prepare_fast(const_cast<glg_plan *>(P), st);
        if (rc) return rc;
        const FastWs w = fast_ws(P, nmaps, ws);
        cudaError_t e = cudaMemsetAsync(w.err, 0, GLG_WS_STATUS_BYTES, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(w.rl.hdr, 0, 256, st);
        if (e != cudaSuccess) return glg_cuda_status(e, "glg_alm2map: status reset");
        const glg_tile_run all{0, (P->npairs + 127) / 128, 0, true};
        rc = glg_launch_leg_tc(P, (const float2 *)alm, nmaps, w.bpack, w.F, w.err, all, st);
        if (rc) return rc;
        rc = glg_launch_ring_syn_f32(P, w.F, w.Ft, nmaps, (float *)maps, epi, &w.rl, st);
        if (rc) return rc;
        return glg_launch_refine(P, w.Ft, nmaps, (float *)maps, epi, w.rl, st);
    }
    double2 *F = (double2 *)ws;
    int rc = glg_launch_leg_syn(P, (const double2 *)alm, nmaps, F, st);
    if (rc) return rc;
    return glg_launch_ring_syn(P, F, nmaps, (double *)maps, epi, ring_gbuf(P, ws, ring_coef_bytes(P, nmaps)), st);
}

// The fast synthesis with its epilogue in device memory (glg_epi_dev):
// every step is a stream operation whose arguments do not depend on the
// epilogue, so a capture of it replays with whatever epilogue was copied to
// `epi_dev` before the replay.
extern "C" int glg_alm2map_fast_devepi(const glg_plan *P, const void *alm, int nmaps, void *maps,
                                       const void *epi_dev, void *ws, size_t ws_bytes, void *stream) {
    GLG_REQUIRE(P != nullptr, "glg_alm2map_fast_devepi: null plan");
    GLG_REQUIRE(nmaps >= 0 && nmaps <= GLG_EPI_MAPS, "glg_alm2map_fast_devepi: nmaps must be in [0, 40]");
    if (nmaps == 0) return GLG_OK;
    GLG_REQUIRE(alm && maps && epi_dev, "glg_alm2map_fast_devepi: null pointer");
    GLG_REQUIRE(ws && ws_bytes >= glg_alm2map_workspace(P, nmaps, GLG_FORM_FAST),
                "glg_alm2map_fast_devepi: workspace too small");
    GLG_REQUIRE(P->fast_ready, "glg_alm2map_fast_devepi: the plan's fast tables are not built (run one fast "
                               "synthesis first)");
    cudaStream_t st = (cudaStream_t)stream;
    FastWs w = fast_ws(P, nmaps, ws);
    w.rl.edev = (const glg_epi_dev *)epi_dev;
    cudaError_t e = cudaMemsetAsync(w.err, 0, GLG_WS_STATUS_BYTES, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.rl.hdr, 0, 256, st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_alm2map_fast_devepi: status reset");
    const glg_tile_run all{0, (P->npairs + 127) / 128, 0, true};
    int rc = glg_launch_leg_tc(P, (const float2 *)alm, nmaps, w.bpack, w.F, w.err, all, st);
    if (rc) return rc;
    rc = glg_launch_ring_syn_f32(P, w.F, w.Ft, nmaps, (float *)maps, nullptr, &w.rl, st);
    if (rc) return rc;
    return glg_launch_refine(P, w.Ft, nmaps, (float *)maps, nullptr, w.rl, st);
}

extern "C" size_t glg_epilogue_dev_bytes(void) { return sizeof(glg_epi_dev); }

extern "C" int glg_epilogue_dev_fill(const glg_epilogue *epi, int nmaps, void *host_out) {
    GLG_REQUIRE(host_out != nullptr, "glg_epilogue_dev_fill: null output");
    GLG_REQUIRE(nmaps >= 0 && nmaps <= GLG_EPI_MAPS, "glg_epilogue_dev_fill: nmaps must be in [0, 40]");
    glg_epi_dev_fill(epi, nmaps, (glg_epi_dev *)host_out);
    return GLG_OK;
}

extern "C" size_t glg_alm2map_host_workspace(const glg_plan *P, int nmaps) {
    if (!P || nmaps <= 0) return 0;
    return glg_alm2map_workspace(P, nmaps, GLG_FORM_FAST) + sizeof(float) * (size_t)nmaps * P->npix;
}

namespace {

// HEALPix RING first pixel and length of the north and south rings of pair p
// (the formulas of the plan's ring table, on the host).
int64_t ring_startN(int nside, int p) {
    const int64_t ir = p + 1, ns = nside;
    return ir < ns ? 2 * ir * (ir - 1) : 2 * ns * (ns - 1) + (ir - ns) * 4 * ns;
}
int64_t ring_startS(int nside, int p) {
    const int64_t ir = p + 1, ns = nside;
    return ir < ns ? 12 * ns * ns - 2 * ir * (ir + 1) : 2 * ns * (ns - 1) + (3 * ns - ir) * 4 * ns;
}
int64_t ring_nph(int nside, int p) { return p + 1 < nside ? 4LL * (p + 1) : 4LL * nside; }

// Run k of the host-output synthesis: ring tiles t0 .. t1-1 (128 pairs each,
// counted from the equator end), ring pairs p0 .. p1-1, and its two pixel
// bands [band[b][0], band[b][1]) in every map: the north rings p0 .. p1-1,
// then the south rings of pairs p0 .. q1-1 (all but the equator, which is its
// own south ring; an empty band is [0, 0)).
constexpr int kHostRuns = 8;
struct HostRun {
    int t0, t1, p0, p1;
    int64_t band[2][2];
};
int host_run_count(int nside) {
    const int ntiles = (2 * nside + 127) / 128;
    return ntiles < kHostRuns ? ntiles : kHostRuns;
}
HostRun host_run(int nside, int k) {
    const int npairs = 2 * nside, ntiles = (npairs + 127) / 128, nrun = host_run_count(nside);
    HostRun r;
    r.t1 = ntiles - (int)((int64_t)ntiles * k / nrun);
    r.t0 = ntiles - (int)((int64_t)ntiles * (k + 1) / nrun);
    r.p0 = r.t0 * 128;
    r.p1 = r.t1 * 128 < npairs ? r.t1 * 128 : npairs;
    const int q1 = r.p1 < npairs ? r.p1 : npairs - 1;
    r.band[0][0] = ring_startN(nside, r.p0);
    r.band[0][1] = ring_startN(nside, r.p1 - 1) + ring_nph(nside, r.p1 - 1);
    r.band[1][0] = r.band[1][1] = 0;
    if (q1 > r.p0) {
        r.band[1][0] = ring_startS(nside, q1 - 1);
        r.band[1][1] = ring_startS(nside, r.p0) + ring_nph(nside, r.p0);
    }
    return r;
}

}  // namespace

extern "C" int glg_host_output_runs(int nside, int64_t *out, int max_runs) {
    GLG_REQUIRE(nside >= 1 && nside <= 8192, "glg_host_output_runs: nside must be in [1, 8192]");
    GLG_REQUIRE(out != nullptr, "glg_host_output_runs: null pointer");
    const int nrun = host_run_count(nside);
    GLG_REQUIRE(max_runs >= nrun, "glg_host_output_runs: max_runs below the run count");
    for (int k = 0; k < nrun; ++k) {
        const HostRun r = host_run(nside, k);
        const int64_t row[8] = {r.t0, r.t1, r.p0, r.p1, r.band[0][0], r.band[0][1], r.band[1][0], r.band[1][1]};
        for (int j = 0; j < 8; ++j) out[8 * k + j] = row[j];
    }
    return nrun;
}

extern "C" int glg_alm2map_host(const glg_plan *P, const void *alm, int nmaps, void *maps_host,
                                const glg_epilogue *epi, void *ws, size_t ws_bytes, void *stream) {
    GLG_REQUIRE(P != nullptr, "glg_alm2map_host: null plan");
    GLG_REQUIRE(nmaps >= 0 && nmaps <= 40, "glg_alm2map_host: nmaps must be in [0, 40]");
    if (nmaps == 0) return GLG_OK;
    GLG_REQUIRE(alm && maps_host, "glg_alm2map_host: null pointer");
    GLG_REQUIRE(ws && ws_bytes >= glg_alm2map_host_workspace(P, nmaps), "glg_alm2map_host: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    int rc = glg_plan_prepare_fast(const_cast<glg_plan *>(P), st);
    if (rc) return rc;
    const FastWs w = fast_ws(P, nmaps, ws);
    int *err = w.err;
    float *bpack = w.bpack;
    float2 *F = w.F, *Ft = w.Ft;
    float *stage = (float *)w.end;
    cudaError_t e = cudaMemsetAsync(err, 0, GLG_WS_STATUS_BYTES, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.rl.hdr, 0, 256, st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_alm2map_host: status reset");

    // Ring tiles in runs from the equator to the poles: each run's maps go to
    // the host on a copy stream while the next run computes, and the last
    // run (the polar caps) has the fewest pixels left to copy at the end.
    const int nrun = host_run_count(P->nside);
    cudaStream_t cs = nullptr;
    cudaEvent_t ev[kHostRuns + 1] = {};
    int made = 0;  // events created: one per run and one for the final join
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) cs = nullptr;
    while (e == cudaSuccess && made <= nrun) {
        e = cudaEventCreateWithFlags(&ev[made], cudaEventDisableTiming);
        if (e == cudaSuccess) ++made;
    }
    if (e != cudaSuccess) rc = glg_cuda_status(e, "glg_alm2map_host: copy stream");
    // every run's sums and ring FFTs first, then every run's copies (a copy
    // into pageable memory returns only when done: it must not hold back the
    // launches of later runs)
    int started = 0;
    for (int k = 0; !rc && k < nrun; ++k) {
        const HostRun r = host_run(P->nside, k);
        const glg_tile_run run{r.t0, r.t1 - r.t0, k, k == 0};
        rc = glg_launch_leg_tc(P, (const float2 *)alm, nmaps, bpack, F, err, run, st);
        if (!rc) rc = glg_launch_ring_syn_f32_range(P, F, Ft, nmaps, stage, epi, r.p0, r.p1, &w.rl, st);
        if (!rc) rc = glg_launch_refine(P, Ft, nmaps, stage, epi, w.rl, st);  // this run's listed pixels
        if (!rc && (e = cudaEventRecord(ev[k], st)) != cudaSuccess) rc = glg_cuda_status(e, "glg_alm2map_host: event");
        if (!rc) ++started;
    }
    const size_t pitch = sizeof(float) * (size_t)P->npix;
    for (int k = 0; k < started && !rc; ++k) {
        const HostRun r = host_run(P->nside, k);
        e = cudaStreamWaitEvent(cs, ev[k], 0);
        for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
            const int64_t a0 = r.band[b][0], a1 = r.band[b][1];
            if (a1 > a0)
                e = cudaMemcpy2DAsync((float *)maps_host + a0, pitch, stage + a0, pitch, sizeof(float) * (size_t)(a1 - a0),
                                      (size_t)nmaps, cudaMemcpyDeviceToHost, cs);
        }
        if (e != cudaSuccess) rc = glg_cuda_status(e, "glg_alm2map_host: map copy");
    }
    // the caller's stream resumes after the last copy (also after a failure:
    // nothing may still be reading the workspace when it is reused)
    if (cs && made > nrun) {
        if (cudaEventRecord(ev[nrun], cs) == cudaSuccess) cudaStreamWaitEvent(st, ev[nrun], 0);
        else cudaStreamSynchronize(cs);
    }
    for (int k = 0; k < made; ++k) cudaEventDestroy(ev[k]);  // released once complete
    if (cs) cudaStreamDestroy(cs);
    return rc;
}

extern "C" int glg_host_device_pointer(const void *host, void **dev) {
    GLG_REQUIRE(host && dev, "glg_host_device_pointer: null pointer");
    *dev = nullptr;
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, host);
    if (e != cudaSuccess || attr.type != cudaMemoryTypeHost || attr.devicePointer == nullptr) {
        cudaGetLastError();
        glg_set_error("glg_host_device_pointer: not page-locked host memory mapped into the device");
        return GLG_ERR_INVALID;
    }
    *dev = attr.devicePointer;
    return GLG_OK;
}

extern "C" int glg_workspace_status(const void *ws, void *stream) {
    GLG_REQUIRE(ws != nullptr, "glg_workspace_status: null workspace");
    int st_host = 0;
    cudaError_t e = cudaMemcpyAsync(&st_host, ws, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_workspace_status");
    if (st_host != 0) {
        glg_set_error("a bounded device wait of the fast Legendre contraction timed out");
        return st_host;
    }
    return GLG_OK;
}

extern "C" size_t glg_alm2map_spin_workspace(const glg_plan *P) {
    return P ? with_gbuf(P, ring_coef_bytes(P, 2)) : 0;
}

extern "C" int glg_alm2map_spin(const glg_plan *P, const void *elm, const void *blm, int spin,
                                void *q, void *u, void *ws, size_t ws_bytes, void *stream) {
    GLG_REQUIRE(P != nullptr, "glg_alm2map_spin: null plan");
    GLG_REQUIRE(elm && q && u, "glg_alm2map_spin: null pointer");
    GLG_REQUIRE(spin == 1 || spin == 2, "glg_alm2map_spin: spin must be 1 or 2");
    GLG_REQUIRE(ws && ws_bytes >= glg_alm2map_spin_workspace(P), "glg_alm2map_spin: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    double2 *F = (double2 *)ws;
    int rc = glg_launch_leg_syn_spin(P, (const double2 *)elm, (const double2 *)blm, spin, F, st);
    if (rc) return rc;
    void *gb = ring_gbuf(P, ws, ring_coef_bytes(P, 2));
    rc = glg_launch_ring_syn(P, F, 1, (double *)q, nullptr, gb, st);
    if (rc) return rc;
    return glg_launch_ring_syn(P, F + (size_t)P->nrings * (P->mmax + 1), 1, (double *)u, nullptr, gb, st);
}

extern "C" size_t glg_map2alm_workspace(const glg_plan *P, int nmaps) {
    if (!P || nmaps <= 0) return 0;
    return with_gbuf(P, ring_coef_bytes(P, nmaps) + sizeof(double) * (size_t)nmaps * P->npix);
}

extern "C" int glg_map2alm(const glg_plan *P, const void *maps, int nmaps, int niter, void *alm,
                           void *ws, size_t ws_bytes, void *stream) {
    GLG_REQUIRE(P != nullptr, "glg_map2alm: null plan");
    GLG_REQUIRE(nmaps >= 0 && niter >= 0, "glg_map2alm: negative size");
    if (nmaps == 0) return GLG_OK;
    GLG_REQUIRE(maps && alm, "glg_map2alm: null pointer");
    GLG_REQUIRE(ws && ws_bytes >= glg_map2alm_workspace(P, nmaps), "glg_map2alm: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    double2 *G = (double2 *)ws;
    double *tmp = (double *)((char *)ws + ring_coef_bytes(P, nmaps));
    const double *f = (const double *)maps;
    double2 *a = (double2 *)alm;
    void *gb = ring_gbuf(P, ws, ring_coef_bytes(P, nmaps) + sizeof(double) * (size_t)nmaps * P->npix);
    int rc = glg_launch_ring_ana(P, f, nmaps, G, gb, st);
    if (rc) return rc;
    if ((rc = glg_launch_leg_ana(P, G, nmaps, a, 0, st))) return rc;
    const int64_t n = (int64_t)nmaps * P->npix;
    for (int it = 0; it < niter; ++it) {
        if ((rc = glg_launch_leg_syn(P, a, nmaps, G, st))) return rc;
        if ((rc = glg_launch_ring_syn(P, G, nmaps, tmp, nullptr, gb, st))) return rc;
        {
            GLG_LAUNCH_SCOPE("k_residual", st);
            k_residual<<<1216, 256, 0, st>>>(f, tmp, n);
            GLG_CHECK_LAUNCH("k_residual");
        }
        if ((rc = glg_launch_ring_ana(P, tmp, nmaps, G, gb, st))) return rc;
        if ((rc = glg_launch_leg_ana(P, G, nmaps, a, 1, st))) return rc;
    }
    return GLG_OK;
}

// Autotuner of the fast form's ring FFTs: each size bucket is timed at
// 128, 256 and 512 threads per block (where its shared memory fits) on the
// caller's workspace and output, and the fastest is kept in the plan.
extern "C" int glg_autotune_fast(glg_plan *P, int nmaps, void *maps, void *ws, size_t ws_bytes, void *stream) {
    GLG_REQUIRE(P != nullptr, "glg_autotune_fast: null plan");
    GLG_REQUIRE(nmaps >= 1 && nmaps <= 40, "glg_autotune_fast: nmaps must be in [1, 40]");
    GLG_REQUIRE(maps && ws && ws_bytes >= glg_alm2map_workspace(P, nmaps, GLG_FORM_FAST),
                "glg_autotune_fast: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    int rc = glg_plan_prepare_fast(P, st);
    if (rc) return rc;
    const size_t fbytes = sizeof(float2) * (size_t)nmaps * P->nrings * (P->mmax + 1);
    float2 *Ft = fast_ws(P, nmaps, ws).Ft;
    float2 *gz = fast_ws(P, nmaps, ws).rl.gz;
    cudaError_t e = cudaMemsetAsync(Ft, 0, fbytes, st);
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_autotune_fast");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    for (int k = 0; k < P->nbuckets; ++k) {
        int best = P->buckets[k].threads;
        float best_ms = 1e30f;
        for (int threads : {128, 256, 512, 1024}) {
            // 1024 threads only for the power-of-two kernels (kinds 1, 2)
            if (threads > 512 && P->buckets[k].kind == 0) continue;
            if (glg_ring32_smem(P->buckets[k].kind, P->buckets[k].size, threads, P->buckets[k].fold != 0) >
                227 * 1024)
                continue;
            if ((rc = glg_launch_ring_bucket_f32(P, k, threads, Ft, nmaps, (float *)maps, gz, st))) break;
            cudaEventRecord(a, st);
            for (int r = 0; r < 2 && !rc; ++r)
                rc = glg_launch_ring_bucket_f32(P, k, threads, Ft, nmaps, (float *)maps, gz, st);
            cudaEventRecord(b, st);
            if (rc) break;
            e = cudaEventSynchronize(b);
            if (e != cudaSuccess) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            if (ms < best_ms) {
                best_ms = ms;
                best = threads;
            }
        }
        if (rc || e != cudaSuccess) break;
        P->buckets[k].threads = best;
        P->buckets[k].ms = best_ms / 2.0f;
        P->buckets[k].smem = glg_ring32_smem(P->buckets[k].kind, P->buckets[k].size, best, P->buckets[k].fold != 0);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc) return rc;
    if (e != cudaSuccess) return glg_cuda_status(e, "glg_autotune_fast");
    return GLG_OK;
}

extern "C" int glg_plan_bucket_times(const glg_plan *P, float *ms, int max_buckets) {
    GLG_REQUIRE(P != nullptr && ms != nullptr, "glg_plan_bucket_times: null pointer");
    int n = 0;
    for (; n < P->nbuckets && n < max_buckets; ++n) ms[n] = P->buckets[n].ms;
    return n;
}

extern "C" int glg_plan_buckets(const glg_plan *P, int *out, int max_buckets) {
    GLG_REQUIRE(P != nullptr && out != nullptr, "glg_plan_buckets: null pointer");
    int n = 0;
    for (; n < P->nbuckets && n < max_buckets; ++n) {
        out[4 * n + 0] = P->buckets[n].kind;
        out[4 * n + 1] = P->buckets[n].size;
        out[4 * n + 2] = P->buckets[n].count;
        out[4 * n + 3] = P->buckets[n].threads;
    }
    return n;
}
