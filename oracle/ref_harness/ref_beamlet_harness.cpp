// ref_beamlet_harness.cpp -- executes the reference's own dosecalc-beamlet
// kernel source on the CPU (test infrastructure; used only to write golden
// beamlet columns, never by the engine).
//
// The reference kernel files are compiled unmodified from the reference
// checkout (include path set by oracle/ref_harness/build.py):
//   CCCS/CudaUtilities/geometry.cu                  rotations
//   CCCS/DoseCalcAlgo/cudaSiddon.cu                  cudaSiddon_device (TERMA)
//   CCCS/dosecalc-beamlet/nvbbRayConvolve_device.cu  cudaBeamletRaytrace,
//       PackRowConvolve, PackedREVtoBEVdose, UnpackBEVDosePillar
// The host orchestration (nvbbRayConvolve_host.cu launches with <<<>>> and
// binds CUDA arrays) is restated below from
// CCCS/dosecalc-beamlet/nvbbRayConvolve_host.cu:75-155 (findREV),
// :180-280 (calcBeamletAnchors), :318-357 (mean kernel radii), :444-1107
// (pillar grid, ArraySizeError re-batching against max_rev_size, per-ray
// launches) and :1172-1260 (per-pillar unpack), in the reference's FP32
// arithmetic with its geometry functions.
#include "cuda_cpu_shim.h"

#include <cfloat>
#include <cstdio>
#include <limits>
#include <stdexcept>
#include <vector>

thread_local float shmBlock[2 * 1200];
thread_local float s_subterma[1024];

#include "DoseCalcIO/kernel.h"  // N_KERNEL_RADII
#include "CudaUtilities/geometry.cu"
#include "DoseCalcAlgo/cudaSiddon.cu"
#include "dosecalc-beamlet/nvbbRayConvolve_device.cu"

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
        ccsim::bIdx = make_uint3((unsigned)(b % grid.x), (unsigned)((b / grid.x) % grid.y),
                                 (unsigned)(b / ((long long)grid.x * grid.y)));
        for (unsigned tz = 0; tz < block.z; tz++)
            for (unsigned ty = 0; ty < block.y; ty++)
                for (unsigned tx = 0; tx < block.x; tx++) {
                    ccsim::tIdx = make_uint3(tx, ty, tz);
                    ccsim::barrier_count = 0;
                    body();
                }
    }
}

inline float comp(const float3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// calcBeamletAnchors (host.cu:180-280): beamlet isocentre, divergence
// angles and the entry/exit points of the beamlet axis on the calc bbox
bool beamlet_anchors(float3& first, float3& last, float2& angles, float3& biso, float3 src, float3 iso, unsigned idx,
                     float2 bsize, uint2 fdims, float3 voxel, float3 dstart, uint3 bb0, uint3 bbs, float az, float zen,
                     float coll) {
    const unsigned bx = idx % fdims.x, by = idx / fdims.x;
    const float3 bdiff = make_float3(bsize.x * (-0.5f * fdims.x + bx + 0.5f), 0.f, bsize.y * (-0.5f * fdims.y + by + 0.5f));
    biso = iso + inverseRotateBeamAtOriginRHS(bdiff, az, zen, coll);
    angles = make_float2(acosf(length(iso - src) / length(biso - src)), atan2f(bdiff.z, bdiff.x));
    const float3 lo = dstart + voxel * make_float3(bb0);
    const float3 hi = lo + voxel * make_float3(bbs);
    const double buf = 0.05;
    float3 hit[6];
    const float3 d = biso - src;
    for (int a = 0; a < 3; a++) {
        const double den = comp(d, a);
        const double t1 = (comp(lo, a) - comp(src, a)) / (den + 1e-12);
        const double t2 = (comp(hi, a) - comp(src, a)) / (den + 1e-12);
        hit[2 * a] = src + t1 * d;
        hit[2 * a + 1] = src + t2 * d;
    }
    first = make_float3(std::numeric_limits<float>::max());
    last = make_float3(std::numeric_limits<float>::min());
    double dmin = std::numeric_limits<double>::max(), dmax = std::numeric_limits<double>::min();
    for (int a = 0; a < 3; a++)
        for (int s = 0; s < 2; s++) {
            const float3 p = hit[2 * a + s];
            const int u = (a + 1) % 3, v = (a + 2) % 3;
            if (comp(p, u) + buf >= comp(lo, u) && comp(p, u) - buf <= comp(hi, u) && comp(p, v) + buf >= comp(lo, v) &&
                comp(p, v) - buf <= comp(hi, v)) {
                if (length(p - src) < dmin) { first = p; dmin = length(first - src); }
                if (length(p - src) > dmax) { last = p; dmax = length(last - src); }
            }
        }
    return dmin < std::numeric_limits<float>::max() && dmax > std::numeric_limits<float>::min();
}

struct REV {
    uint3 size;
    float3 min_coords;
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
    const float* fluence;
    const float* mu;
    const float* mu_en;
    int ntheta, nphi, nradii;
    const float* radii;
    const float* cumkern;
    const float* theta_deg;
    const float* phi_deg;
    float rev_latspacing, rev_longspacing, penumbra;
    int tex_emulate;
    int nthreads;
} ref_setup;

typedef struct {
    float azimuth, zenith, coll;
    float iso[3];
    float sad;
    int fmap[2];
    float beamlet[2];
} ref_beam;

// Dense dose columns on the calc bbox (x fastest) of every active beamlet
// (fluence > 0, fluence-map order), as UnpackBEVDosePillar leaves them before
// sparsification (rev_jitter = 0).  columns: [max_cols][bbox voxels].  info: [0] active
// beamlets, [1..3] pillar dims, [4] batches, [7] status (0 ok, 1 no anchor,
// 2 too many beamlets, 3 rev.x > 1024, 4 more than 100 batches).
int ccref_beamlet_columns(const ref_setup* S, const ref_beam* B, const float* fluence_map, float kernel_extent,
                          const int* max_rev_size, float rev_jitter, int max_cols, float* columns, int* beamlet_index,
                          int* info) {
    ccsim::tex_emulate = S->tex_emulate;
    const int nth = S->nthreads > 0 ? S->nthreads : 1;
    for (int a = 0; a < 8; a++) info[a] = 0;
    const float3 start = make_float3(S->start[0], S->start[1], S->start[2]);
    const float3 voxel = make_float3(S->voxel[0], S->voxel[1], S->voxel[2]);
    const uint3 size = make_uint3(S->size[0], S->size[1], S->size[2]);
    const uint3 bb0 = make_uint3(S->bbox_start[0], S->bbox_start[1], S->bbox_start[2]);
    const uint3 bbs = make_uint3(S->bbox_size[0], S->bbox_size[1], S->bbox_size[2]);
    const long long nb = (long long)bbs.x * bbs.y * bbs.z;

    // BEAM::reconfigure (beam.cpp:300-321)
    float az = fmodf(B->azimuth, 2 * PI), zen = fmodf(B->zenith, 2 * PI);
    auto close = [](float a, float b) { return fabsf(b - a) <= 1e-6f; };
    if (!close(zen, 0.f) && (close(az, 0.f) || close(az, PI))) zen = 0.f;
    const float coll = B->coll;
    const float3 iso = make_float3(B->iso[0], B->iso[1], B->iso[2]);
    const float3 source = inverseRotateBeamAtOriginRHS(make_float3(0.f, -B->sad, 0.f), az, zen, 0.f) + iso;
    const float3 direction = normalize(iso - source);
    const float2 bsize = make_float2(B->beamlet[0], B->beamlet[1]);
    const uint2 fsz = make_uint2(B->fmap[0], B->fmap[1]);

    // textures and constants (initCudaConstandTex, host.cu:318-357): kernel
    // radii are the mean radii of the radial bins
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
    KERN_RADII[0] = 0.5f * S->radii[0];
    for (int r = 1; r < S->nradii && r < N_KERNEL_RADII; r++) KERN_RADII[r] = 0.5f * (S->radii[r] + S->radii[r - 1]);

    const float3 rev_vox = make_float3(S->rev_latspacing, S->rev_longspacing, S->rev_latspacing);
    std::vector<float> fmap(fluence_map, fluence_map + fsz.x * fsz.y);

    // active beamlets and their anchors (host.cu:573-649)
    std::vector<int> idx;
    for (int i = 0; i < (int)(fsz.x * fsz.y); i++)
        if (fmap[i] > 0) idx.push_back(i);
    const int n = (int)idx.size();
    info[0] = n;
    if (n == 0) return 0;
    if (n > max_cols) { info[7] = 2; return 2; }
    std::vector<float3> bstart(n), bend(n), biso(n), pstart(n);
    std::vector<float2> bang(n);
    std::vector<float> blen(n);
    float max_len = 0.f;
    float2 max_size = make_float2(0.f, 0.f);
    for (int i = 0; i < n; i++) {
        if (!beamlet_anchors(bstart[i], bend[i], bang[i], biso[i], source, iso, (unsigned)idx[i], bsize, fsz, voxel, start,
                             bb0, bbs, az, zen, coll)) {
            info[7] = 1;
            return 1;
        }
        blen[i] = length(bend[i] - bstart[i]);
        max_len = fmaxf(max_len, blen[i]);
        const float2 dv = bsize * length(bend[i] - source) / length(biso[i] - source);
        max_size.x = fmaxf(max_size.x, dv.x);
        max_size.y = fmaxf(max_size.y, dv.y);
    }
    const int wall = 2, pbuf = 2;
    const float psize_long = max_len + 2.f * kernel_extent + wall * rev_vox.y;
    const float2 psize_trans = max_size + 2.f * kernel_extent + wall * rev_vox.x;
    const float3 expand = rev_vox - make_float3(fmodf(psize_trans.x, rev_vox.x), fmodf(psize_long, rev_vox.y),
                                                fmodf(psize_trans.y, rev_vox.z));
    const float3 psize = make_float3(psize_trans.x, psize_long, psize_trans.y) + expand + 2.f * float(pbuf) * rev_vox;
    const int3 pdims = make_int3(psize / rev_vox);
    for (int i = 0; i < n; i++) {
        float3 g = make_float3(-0.5f * (psize.x + wall * rev_vox.x), -0.5f * (psize.y - blen[i] + wall * rev_vox.y),
                               -0.5f * (psize.z + wall * rev_vox.z));
        g = inverseRotateBeamAtOriginRHS(inverseRotateBeamletAtOriginRHS(g, bang[i].x, bang[i].y), az, zen, coll);
        pstart[i] = bstart[i] + g;
    }
    // batches: the fewest whose REV arrays all fit max_rev (the reference
    // restarts with one more batch on ArraySizeError, host.cu:805-819)
    const int nrays = S->nphi * (S->ntheta / 2);
    int nbat = 1;
    std::vector<int> bsizes;
    std::vector<std::vector<REV>> revs;
    for (;; nbat++) {
        if (nbat > 100) { info[7] = 4; return 4; }
        bsizes.assign(nbat, n / nbat);
        for (int r = n - (n / nbat) * nbat, k = 0; r > 0; r--) bsizes[(k++) % nbat] += 1;
        revs.assign(nbat, std::vector<REV>(nrays));
        bool ok = true;
        for (int k = 0; k < nbat && ok; k++) {
            const int npx = (int)ceil(sqrt(float(bsizes[k])));
            const int npy = (int)ceil(float(bsizes[k]) / npx);
            const int3 gd = make_int3(npx * pdims.x + wall, pdims.y + wall, npy * pdims.z + wall);
            const float3 gsize = make_float3(gd) * rev_vox;
            // findREV on the pillar grid box (host.cu:75-155)
            for (int r = 0; r < nrays && ok; r++) {
                const float th = S->theta_deg[r] * PI / 180.f, ph = S->phi_deg[r] * PI / 180.f;
                float3 mn3 = make_float3(std::numeric_limits<float>::max()),
                       mx3 = make_float3(std::numeric_limits<float>::min());
                for (int xo = 0; xo < 2; xo++)
                    for (int yo = 0; yo < 2; yo++)
                        for (int zo = 0; zo < 2; zo++) {
                            float3 o = rotateKernelAtOriginRHS(make_float3(gsize.x * xo, gsize.y * yo, gsize.z * zo), th, ph);
                            mn3 = fminf(mn3, o);
                            mx3 = fmaxf(mx3, o);
                        }
                const uint3 rs = make_uint3((unsigned)ceil(fabsf(mx3.y - mn3.y) / S->rev_longspacing),
                                            (unsigned)ceil(fabsf(mx3.z - mn3.z) / S->rev_latspacing),
                                            (unsigned)ceil(fabsf(mx3.x - mn3.x) / S->rev_latspacing));
                if (rs.x > (unsigned)max_rev_size[0] || rs.y > (unsigned)max_rev_size[1] || rs.z > (unsigned)max_rev_size[2])
                    ok = false;
                // rev_jitter (cm, test sensitivity probes only; 0 = reference)
                // moves the REV lattice origin of every direction
                revs[k][r] = REV{rs, mn3 + make_float3(rev_jitter, -rev_jitter, rev_jitter)};
            }
        }
        if (ok) break;
    }
    for (int k = 0; k < nbat; k++)
        for (int r = 0; r < nrays; r++)
            if (revs[k][r].size.x > 1024) { info[7] = 3; return 3; }
    info[1] = pdims.x; info[2] = pdims.y; info[3] = pdims.z;
    info[4] = nbat;

    int first = 0;
    for (int k = 0; k < nbat; k++) {
    const int m = bsizes[k];
    const int2 np = make_int2((int)ceil(sqrt(float(m))), (int)ceil(float(m) / (int)ceil(sqrt(float(m)))));
    const int3 gdims = make_int3(np.x * pdims.x + wall, pdims.y + wall, np.y * pdims.z + wall);
    uint3 mx = make_uint3(0, 0, 0);
    for (int r = 0; r < nrays; r++) {
        mx.x = std::max(mx.x, revs[k][r].size.x);
        mx.y = std::max(mx.y, revs[k][r].size.y);
        mx.z = std::max(mx.z, revs[k][r].size.z);
    }
    std::vector<REV>& rev = revs[k];
    // REV arrays large enough that the raytrace's out-of-range lanes and the
    // convolution's 2-sample overwrite margin stay inside them
    const uint3 max_rev = make_uint3(mx.x + 34, mx.y + 5, mx.z + 3);
    const long long revn = (long long)max_rev.x * max_rev.y * max_rev.z;
    std::vector<float> bevDens(revn, 0.f), bevTerma(revn, 0.f), doseArr(revn, 0.f);
    ccsim::Surf surfDose{doseArr.data(), {(int)max_rev.x, (int)max_rev.y, (int)max_rev.z}};
    ccsim::Tex texDose{doseArr.data(), {(int)max_rev.x, (int)max_rev.y, (int)max_rev.z}, 3, true, true};
    const long long pgn = (long long)gdims.x * gdims.y * gdims.z;
    std::vector<float> packed(pgn, 0.f);
    std::vector<float2> d_ang(bang.begin() + first, bang.begin() + first + m);
    std::vector<float3> d_pstart(pstart.begin() + first, pstart.begin() + first + m),
        d_biso(biso.begin() + first, biso.begin() + first + m);
    std::vector<int> d_idx(idx.begin() + first, idx.begin() + first + m);
    const dim3 tile(TILE_DIM_X, TILE_DIM_Y, 1);
    for (int r = 0; r < nrays; r++) {
        const int kw = r % (S->ntheta / 2);
        const float th = S->theta_deg[r] * PI / 180.f, ph = S->phi_deg[r] * PI / 180.f;
        const REV& R = rev[r];
        {
            dim3 blk(1, 32, 3);
            dim3 grd(R.size.z, (unsigned)ceilf((float)R.size.x / blk.y), (unsigned)ceilf((float)R.size.y / blk.z));
            float *dp = bevDens.data(), *tp = bevTerma.data();
            launch(grd, blk, nth, [&] {
                cudaBeamletRaytrace(dp, tp, source, bsize, az, zen, coll, make_float3(gdims), make_float3(pdims), m, wall,
                                    np, d_idx.data(), d_ang.data(), d_pstart.data(), d_biso.data(), th, ph,
                                    R.min_coords, R.size, max_rev, start, voxel, rev_vox, make_float3(bb0),
                                    (cudaTextureObject_t)(uintptr_t)&texDens, (cudaTextureObject_t)(uintptr_t)&texDens,
                                    fmap.data(), make_float3(size), bbs, 1.0f, direction, iso, B->sad, fsz, S->nE,
                                    (cudaTextureObject_t)(uintptr_t)&texSpec);
            });
        }
        {
            // one block per REV row, its row staged in shared memory before
            // the block's threads run (device.cu:270-279)
            const int ow = 2;
            dim3 blk(R.size.x + ow, 1, 1);
            dim3 grd(1, R.size.y + ow, R.size.z + ow);
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
                    PackRowConvolve(dp, tp, so, (float)kw, R.size, max_rev, S->rev_longspacing, S->nradii, S->ntheta,
                                    S->nphi, kt, false);
                }
            }
        }
        {
            dim3 grd((unsigned)ceilf((float)gdims.y / tile.x), (unsigned)ceilf((float)gdims.z / tile.y),
                     (unsigned)ceilf((float)gdims.x / tile.z));
            float* pp = packed.data();
            launch(grd, tile, nth, [&] {
                PackedREVtoBEVdose(pp, (cudaTextureObject_t)(uintptr_t)&texDose, th, ph, R.min_coords, rev_vox, gdims);
            });
        }
    }

    // per-pillar unpack onto the calc bbox (host.cu:1172-1260)
    ccsim::Tex texPacked{packed.data(), {gdims.y, gdims.z, gdims.x}, 3, true, true};
    dim3 grd((unsigned)ceilf((float)bbs.x / tile.x), (unsigned)ceilf((float)bbs.y / tile.y),
             (unsigned)ceilf((float)bbs.z / tile.z));
    for (int i = 0; i < m; i++) {
        float* col = columns + (long long)(first + i) * nb;
        std::fill(col, col + nb, 0.f);
        beamlet_index[first + i] = idx[first + i];
        launch(grd, tile, nth, [&] {
            UnpackBEVDosePillar(col, (cudaTextureObject_t)(uintptr_t)&texPacked, B->sad, source, az, zen, coll, start,
                                voxel, make_float3(bb0), bbs, rev_vox, i, i % np.x, i / np.x, pdims, wall, pbuf, pstart[first + i],
                                bang[first + i]);
        });
    }
    first += m;
    }
    return 0;
}

}  // extern "C"
