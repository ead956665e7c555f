// ref_harness.cpp -- executes the reference's own dosecalc-beam kernel source
// on the CPU (test infrastructure; used only to pin the oracle and to write
// golden fixtures, never by the engine).
//
// The reference kernel files are compiled unmodified from the reference
// checkout (include path set by oracle/ref_harness/build.py):
//   CCCS/CudaUtilities/geometry.cu                rotations
//   CCCS/DoseCalcAlgo/cudaSiddon.cu                cudaSiddon (TERMA)
//   CCCS/dosecalc-beam/nvbbRayConvolve_device.cu   cudaRaytrace, RowConvolve,
//                                                  REV2XYZdose
// cuda_cpu_shim.h supplies the device environment.  The host orchestration
// (crop box, findREV, launch shapes, per-ray loop) cannot be compiled here --
// nvbbRayConvolve_host.cu launches with <<<>>> and binds CUDA arrays -- so it
// is restated below from CCCS/dosecalc-beam/nvbbRayConvolve_host.cu:159-293,
// 297-742, in the reference's FP32 arithmetic with its geometry functions.
#include "cuda_cpu_shim.h"

#include <cfloat>
#include <cstdio>
#include <limits>
#include <vector>

// __shared__ arrays declared `extern` inside the kernels
thread_local float shmBlock[2 * 1200];
thread_local float s_subterma[1024];

#include "DoseCalcIO/kernel.h"  // N_KERNEL_RADII
#include "CudaUtilities/geometry.cu"
#include "DoseCalcAlgo/cudaSiddon.cu"
#include "dosecalc-beam/nvbbRayConvolve_device.cu"

namespace ccsim {
thread_local uint3 tIdx, bIdx;
thread_local dim3 bDim, gDim;
thread_local int barrier_count = 0, phase_limit = 2147483647;
int tex_emulate = 1;
}  // namespace ccsim

namespace {

template <class F>
void launch(dim3 grid, dim3 block, int nthreads, F&& body) {
    const long long nb = (long long)grid.x * grid.y * grid.z;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (long long b = 0; b < nb; b++) {
        ccsim::gDim = grid;
        ccsim::bDim = block;
        ccsim::bIdx = make_uint3((unsigned)(b % grid.x), (unsigned)((b / grid.x) % grid.y), (unsigned)(b / ((long long)grid.x * grid.y)));
        for (unsigned tz = 0; tz < block.z; tz++)
            for (unsigned ty = 0; ty < block.y; ty++)
                for (unsigned tx = 0; tx < block.x; tx++) {
                    ccsim::tIdx = make_uint3(tx, ty, tz);
                    ccsim::barrier_count = 0;
                    body();
                }
    }
}

// A block whose threads exchange values through shared memory between
// __syncthreads calls (cudaSiddon with TERMA supersampling): the block is run
// `phases` times; in pass p every thread runs from the start up to its p-th
// barrier, the last pass runs to the end.  Exact for kernels whose code
// before a barrier only (re)writes the thread's own shared-memory slots and
// whose reader of the other slots runs before their owners in the last pass
// (cudaSiddon: thread x == 0 averages the block's sub-voxels).
template <class F>
void launch_phased(dim3 grid, dim3 block, int nthreads, int phases, F&& body) {
    const long long nb = (long long)grid.x * grid.y * grid.z;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (long long b = 0; b < nb; b++) {
        ccsim::gDim = grid;
        ccsim::bDim = block;
        ccsim::bIdx = make_uint3((unsigned)(b % grid.x), (unsigned)((b / grid.x) % grid.y), (unsigned)(b / ((long long)grid.x * grid.y)));
        for (int p = 1; p <= phases; p++) {
            ccsim::phase_limit = p < phases ? p : 2147483647;
            for (unsigned tz = 0; tz < block.z; tz++)
                for (unsigned ty = 0; ty < block.y; ty++)
                    for (unsigned tx = 0; tx < block.x; tx++) {
                        ccsim::tIdx = make_uint3(tx, ty, tz);
                        ccsim::barrier_count = 0;
                        try {
                            body();
                        } catch (const ccsim::PhaseStop&) {
                        }
                    }
        }
        ccsim::phase_limit = 2147483647;
    }
}

struct REV {
    uint3 size;
    float3 min_coords, max_coords;
};

}  // namespace

extern "C" {

typedef struct {
    int size[3];
    float voxel[3];
    float start[3];
    int bbox_start[3];
    int bbox_size[3];
    const float* density;
    int nE;
    const float* energy;
    const float* fluence;  // normalised to unit sum
    const float* mu;
    const float* mu_en;
    int ntheta, nphi, nradii;
    const float* radii;
    const float* cumkern;  // [ntheta][nradii]
    const float* theta_deg;
    const float* phi_deg;
    float rev_latspacing, rev_longspacing, penumbra;
    int tex_emulate;
    int nthreads;
    int ss_factor;  // TERMA supersampling (omni-header ss_factor); <= 1 off
} ref_setup;

typedef struct {
    float azimuth, zenith, coll;
    float iso[3];
    float sad;
    int fmap[2];
    float beamlet[2];
} ref_beam;

// info: bev_cropbox_size[3], status (0 ok, 1 crop box error, 2 ArraySizeError,
// 3 rev.x > 1024)
int ccref_beam_dose(const ref_setup* S, const ref_beam* B, const float* fluence_map, float* dose, float* terma_out,
                    int* info) {
    ccsim::tex_emulate = S->tex_emulate;
    const int nth = S->nthreads > 0 ? S->nthreads : 1;
    const float3 start = make_float3(S->start[0], S->start[1], S->start[2]);
    const float3 voxel = make_float3(S->voxel[0], S->voxel[1], S->voxel[2]);
    const uint3 size = make_uint3(S->size[0], S->size[1], S->size[2]);
    const uint3 bb0 = make_uint3(S->bbox_start[0], S->bbox_start[1], S->bbox_start[2]);
    const uint3 bbs = make_uint3(S->bbox_size[0], S->bbox_size[1], S->bbox_size[2]);
    const long long nb = (long long)bbs.x * bbs.y * bbs.z, nfull = (long long)size.x * size.y * size.z;
    for (int a = 0; a < 4; a++) info[a] = 0;

    // BEAM::reconfigure (beam.cpp:300-321), angle orientation
    float az = fmodf(B->azimuth, 2 * PI), zen = fmodf(B->zenith, 2 * PI);
    auto close = [](float a, float b) { return fabsf(b - a) <= 1e-6f; };
    if (!close(zen, 0.f) && (close(az, 0.f) || close(az, PI))) zen = 0.f;
    const float3 iso = make_float3(B->iso[0], B->iso[1], B->iso[2]);
    const float3 source = inverseRotateBeamAtOriginRHS(make_float3(0.f, -B->sad, 0.f), az, zen, 0.f) + iso;
    const float3 direction = normalize(iso - source);

    // textures and constants (initCudaConstandTex, host.cu:178-242)
    ccsim::Tex texDens{S->density, {S->size[0], S->size[1], S->size[2]}, 3, true, true};
    std::vector<float> spectrum(4 * S->nE);
    for (int e = 0; e < S->nE; e++) {
        spectrum[e] = S->fluence[e];
        spectrum[e + S->nE] = S->energy[e];
        spectrum[e + 2 * S->nE] = S->mu_en[e];
        spectrum[e + 3 * S->nE] = S->mu[e];
    }
    ccsim::Tex texSpec{spectrum.data(), {S->nE, 4, 1}, 2, false, false};
    ccsim::Tex texKern{S->cumkern, {S->nradii, S->ntheta, 1}, 2, true, false};
    for (int r = 0; r < S->nradii && r < N_KERNEL_RADII; r++) KERN_RADII[r] = S->radii[r];
    const float min_vox = fminf(S->rev_latspacing, S->rev_longspacing);
    const unsigned max_diag = (unsigned)ceilf(length(make_float3(bbs)) * voxel.x / min_vox);
    const unsigned mr = max_diag + (unsigned)(2 * (REV_PAD / min_vox + S->penumbra / min_vox)) + 100;
    const uint3 max_rev = make_uint3(mr, mr, mr);

    // TERMA (cudaSiddon, launch shape of host.cu:326-341, launch :392-413)
    std::vector<float> terma(nb, 0.f);
    std::vector<float> fmap(fluence_map, fluence_map + B->fmap[0] * B->fmap[1]);
    {
        dim3 blk(1, 32, 3);
        const unsigned ss = S->ss_factor > 1 ? (unsigned)S->ss_factor : 1u;
        if (ss > 1) {
            const unsigned nsub = ss * ss * ss;
            const unsigned tile = (unsigned)floorf(sqrtf(256.f / (float)nsub));
            blk = dim3(nsub, tile, tile);
            if (nsub * tile * tile > 1024 || tile == 0) return 4;  // beyond s_subterma / the 256-thread tile rule
        }
        dim3 grd(bbs.z, (unsigned)ceilf((float)bbs.x / blk.y), (unsigned)ceilf((float)bbs.y / blk.z));
        const float2 bsz = make_float2(B->beamlet[0], B->beamlet[1]);
        const uint2 fsz = make_uint2(B->fmap[0], B->fmap[1]);
        float* tp = terma.data();
        float* fp = fmap.data();
        auto body = [&] {
            cudaSiddon(tp, fp, start, make_float3(size), voxel, bb0, bbs, 1.0f, source, direction, iso, B->sad, bsz,
                       fsz, az, zen, B->coll, S->nE, (cudaTextureObject_t)(uintptr_t)&texDens,
                       (cudaTextureObject_t)(uintptr_t)&texSpec, -1);
        };
        if (ss > 1) launch_phased(grd, blk, nth, 3, body);  // two __syncthreads in cudaSiddon
        else launch(grd, blk, nth, body);
    }
    if (terma_out) std::copy(terma.begin(), terma.end(), terma_out);

    // crop box (host.cu:429-499)
    float3 b_min = make_float3(std::numeric_limits<float>::max()), b_max = make_float3(std::numeric_limits<float>::min());
    for (unsigned z = 0; z < bbs.z; z++)
        for (unsigned y = 0; y < bbs.y; y++)
            for (unsigned x = 0; x < bbs.x; x++) {
                if (terma[x + (long long)bbs.x * (y + (long long)bbs.y * z)] != 0) {
                    float3 bi = rotateBeamAtOriginRHS(make_float3(x, y, z), az, zen, B->coll);
                    b_min.x = fminf(b_min.x, bi.x); b_min.y = fminf(b_min.y, bi.y); b_min.z = fminf(b_min.z, bi.z);
                    b_max.x = fmaxf(b_max.x, bi.x); b_max.y = fmaxf(b_max.y, bi.y); b_max.z = fmaxf(b_max.z, bi.z);
                }
            }
    b_min.x -= S->penumbra / S->rev_latspacing; b_min.y -= S->penumbra / S->rev_longspacing; b_min.z -= S->penumbra / S->rev_latspacing;
    b_max.x += S->penumbra / S->rev_latspacing; b_max.y += S->penumbra / S->rev_longspacing; b_max.z += S->penumbra / S->rev_latspacing;
    const uint3 bev = make_uint3((unsigned)ceilf(fabsf(b_max.x - b_min.x)), (unsigned)ceilf(fabsf(b_max.y - b_min.y)),
                                 (unsigned)ceilf(fabsf(b_max.z - b_min.z)));
    info[0] = bev.x; info[1] = bev.y; info[2] = bev.z;
    if (bev.x <= 0 || bev.x >= 1000 || bev.y <= 0 || bev.y >= 1000 || bev.z <= 0 || bev.z >= 1000) { info[3] = 1; return 1; }
    const float3 tmn = inverseRotateBeamAtOriginRHS(b_min, az, zen, B->coll);
    const float3 lim_min = make_float3(start.x + (tmn.x + bb0.x) * voxel.x, start.y + (tmn.y + bb0.y) * voxel.y,
                                       start.z + (tmn.z + bb0.z) * voxel.z);
    ccsim::Tex texTerma{terma.data(), {(int)bbs.x, (int)bbs.y, (int)bbs.z}, 3, true, true};

    // findREV for every ray (host.cu:75-155, 536-587)
    const float3 rev_vox = make_float3(S->rev_latspacing, S->rev_longspacing, S->rev_latspacing);
    const int nrays = S->nphi * (S->ntheta / 2);
    std::vector<REV> rev(nrays);
    for (int r = 0; r < nrays; r++) {
        const float th = S->theta_deg[r] * PI / 180.f, ph = S->phi_deg[r] * PI / 180.f;
        float3 bd = make_float3(bev) * rev_vox;
        float3 rmn = make_float3(std::numeric_limits<float>::max()), rmx = make_float3(std::numeric_limits<float>::min());
        for (int xo = 0; xo < 2; xo++)
            for (int yo = 0; yo < 2; yo++)
                for (int zo = 0; zo < 2; zo++) {
                    float3 o = rotateKernelAtOriginRHS(make_float3(bd.x * xo, bd.y * yo, bd.z * zo), th, ph);
                    rmn = fminf(rmn, o);
                    rmx = fmaxf(rmx, o);
                }
        rmn -= REV_PAD;
        rmx += REV_PAD;
        uint3 rs = make_uint3((unsigned)ceil(fabsf(rmx.y - rmn.y) / S->rev_longspacing),
                              (unsigned)ceil(fabsf(rmx.z - rmn.z) / S->rev_latspacing),
                              (unsigned)ceil(fabsf(rmx.x - rmn.x) / S->rev_latspacing));
        if (rs.x > max_rev.x || rs.y > max_rev.y || rs.z > max_rev.z) { info[3] = 2; return 2; }
        if (rs.x > 1024) { info[3] = 3; return 3; }
        rev[r] = REV{rs, rmn, rmx};
    }

    // per ray: cudaRaytrace -> RowConvolve -> REV2XYZdose (host.cu:592-703)
    const long long revn = (long long)max_rev.x * max_rev.y * max_rev.z;
    std::vector<float> bevDens(revn), bevTerma(revn), doseArr(revn, 0.f);
    ccsim::Surf surfDose{doseArr.data(), {(int)max_rev.x, (int)max_rev.y, (int)max_rev.z}};
    ccsim::Tex texDose{doseArr.data(), {(int)max_rev.x, (int)max_rev.y, (int)max_rev.z}, 3, true, true};
    std::fill(dose, dose + nfull, 0.f);
    for (int r = 0; r < nrays; r++) {
        const int kern_wt_idx = r % (S->ntheta / 2);
        const float th = S->theta_deg[r] * PI / 180.f, ph = S->phi_deg[r] * PI / 180.f;
        std::fill(bevDens.begin(), bevDens.end(), 0.f);
        std::fill(bevTerma.begin(), bevTerma.end(), 0.f);
        const REV& R = rev[r];
        {
            dim3 blk(32, 3, 1);
            dim3 grd((unsigned)ceilf((float)R.size.x / blk.x), (unsigned)ceilf((float)R.size.y / blk.y), R.size.z);
            float *dp = bevDens.data(), *tp = bevTerma.data();
            launch(grd, blk, nth, [&] {
                cudaRaytrace(dp, tp, az, zen, B->coll, th, ph, R.min_coords, lim_min, R.size, bev, max_rev, start, voxel,
                             rev_vox, make_float3(bb0), make_float3(bb0 + bbs), (cudaTextureObject_t)(uintptr_t)&texDens,
                             (cudaTextureObject_t)(uintptr_t)&texTerma);
            });
        }
        {
            // one block per REV row; each block first stages its row in
            // shared memory and synchronises (device.cu:113-117).  Threads run
            // one after another here, so the row is staged before the
            // block's threads start; the kernel then stores the same values.
            const int overwrite = 2;
            dim3 blk(R.size.x + overwrite, 1, 1);
            dim3 grd(1, R.size.y + overwrite, R.size.z + overwrite);
            const long long nblk = (long long)grd.y * grd.z;
            float* dp = bevDens.data();
            float* tp = bevTerma.data();
            cudaSurfaceObject_t so = (cudaSurfaceObject_t)(uintptr_t)&surfDose;
            cudaTextureObject_t kt = (cudaTextureObject_t)(uintptr_t)&texKern;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nth)
            for (long long b = 0; b < nblk; b++) {
                ccsim::gDim = grd;
                ccsim::bDim = blk;
                ccsim::bIdx = make_uint3(0, (unsigned)(b % grd.y), (unsigned)(b / grd.y));
                const unsigned ty = ccsim::bIdx.y, tz = ccsim::bIdx.z;
                if (ty < R.size.y && tz < R.size.z)
                    for (unsigned tx = 0; tx < R.size.x; tx++) {
                        long long m = tx + (long long)max_rev.x * (ty + (long long)max_rev.y * tz);
                        shmBlock[tx] = dp[m];
                        shmBlock[tx + R.size.x] = tp[m];
                    }
                for (unsigned tx = 0; tx < blk.x; tx++) {
                    ccsim::tIdx = make_uint3(tx, 0, 0);
                    RowConvolve(dp, tp, so, (float)kern_wt_idx, R.size, max_rev, S->rev_longspacing, S->nradii, S->ntheta,
                                S->nphi, S->penumbra, kt);
                }
            }
        }
        {
            dim3 blk(TILE_DIM_X, TILE_DIM_Y, 1);
            dim3 grd((unsigned)ceilf((float)bbs.x / blk.x), (unsigned)ceilf((float)bbs.y / blk.y),
                     (unsigned)ceilf((float)bbs.z / blk.z));
            launch(grd, blk, nth, [&] {
                REV2XYZdose(dose, (cudaTextureObject_t)(uintptr_t)&texDose, az, zen, B->coll, th, ph, start, voxel,
                            rev_vox, size, bb0, bb0 + bbs, R.min_coords, R.size, lim_min);
            });
        }
    }
    return 0;
}

}  // extern "C"
