// ee_kernels.cu -- sm_103a kernels of the CCCS beam-dose engine.
//
// Stages per beam (forward):
//   k_terma     Siddon radiological path + polyenergetic TERMA, one thread per
//               calc-bbox voxel, fused with the crop-box min/max reduction.
//               Restates CCCS/DoseCalcAlgo/cudaSiddon.cu:20-308 and the host
//               extent scan CCCS/dosecalc-beam/nvbbRayConvolve_host.cu:429-499.
//   k_geometry  crop box -> BEV box, findREV for every cone, affine maps
//               (host.cu:460-499, :75-155).
//   k_cone_*    one warp per collapsed-cone line: trilinear gather of density
//               and TERMA along the rotated line into shared memory
//               (nvbbRayConvolve_device.cu:11-80), then the bidirectional line
//               convolution (device.cu:87-218): EE_KERNEL_EXP as two warp-shuffle
//               affine scans, EE_KERNEL_TABLE as the reference walk.
//   k_gather    patient voxel <- sum over cones of the trilinear REV dose
//               (device.cu:222-261), all cones of all beams of the batch in
//               registers, one write per voxel.
// Adjoint: k_gather_T (scatter), k_cone_T (reverse scans + TERMA scatter),
// k_terma_T (per-beamlet reduction).
#include "ee_internal.h"
#include <algorithm>
#include <cfloat>
#include <cstddef>
#include <mutex>

#include "ee_device.cuh"

namespace {

// TERMA without supersampling.  Threads take the box's voxels brick by brick
// (4x4x4, ee_brick_vol), 256 per block.  A voxel needs a ray trace when it
// has a beamlet (beamlet_of, cudaSiddon.cu:143-165) whose fluence is
// positive, or any beamlet when the unit TERMA is kept for the adjoint; the
// rest are written at once.  The box is the field's axis-aligned hull, so
// warps at the field's edge hold both kinds: the voxels to trace are first
// gathered into a shared list in box order, and the block's leading threads
// trace them, so the Siddon loops run with full warps (measured 10 % faster
// than tracing in place).  Each voxel's arithmetic is unchanged.  The crop
// box (host.cu:442-459) is reduced from the traced voxels with non-zero
// TERMA: min/max of BEV indices as ordered-int keys, one merge per warp.
// Five resident blocks per SM: 48 registers, no spills.
__global__ void __launch_bounds__(256, 5) k_terma(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                   EeBeamGeom* __restrict__ geoms, const float* __restrict__ fluence,
                                                   float* __restrict__ terma, float* __restrict__ unit,
                                                   int* __restrict__ bl_idx) {
    __shared__ int s_v[256], s_bl[256], s_wcnt[8];
    __shared__ float s_fl[256];
    const int b = blockIdx.z;
    const EeBeamSpec& S = specs[b];
    const long long bvol = ee_brick_vol(S.tn);
    const long long vb = (long long)blockIdx.x * 256;
    if (vb >= bvol) return;
    const int nbx = (S.tn[0] + 3) >> 2, nby = (S.tn[1] + 3) >> 2;
    // box indices of bricked box element v
    auto coords = [&](long long v, int& xr, int& yr, int& zr) {
        const long long brick = v >> 6;
        const int w = (int)(v & 63);
        const long long bxy = brick % ((long long)nbx * nby);
        xr = (int)(bxy % nbx) * 4 + (w & 3);
        yr = (int)(bxy / nbx) * 4 + ((w >> 2) & 3);
        zr = (int)(brick / ((long long)nbx * nby)) * 4 + (w >> 4);
    };
    const long long v = vb + threadIdx.x;
    bool need = false;
    int bl = -1;
    float fl = 0.f;
    if (v < bvol) {
        int xr, yr, zr;
        coords(v, xr, yr, zr);
        // padding of the last bricks: never sampled, kept zero
        const bool inbox = xr < S.tn[0] && yr < S.tn[1] && zr < S.tn[2];
        if (inbox) {
            const int x = S.t0[0] + xr, y = S.t0[1] + yr, z = S.t0[2] + zr;
            const f3 vox = mk(P.start[0] + x * P.voxel[0], P.start[1] + y * P.voxel[1], P.start[2] + z * P.voxel[2]);
            bl = beamlet_of(S, vox);
            if (bl == -2) bl = beamlet_of_fp64(P, S, x, y, z);
            if (bl >= 0) {
                fl = __ldg(fluence + S.fl_off + bl);
                need = fl > 0.f || unit;
            }
        }
        if (!need) {
            terma[S.t_off + v] = 0.f;
            if (unit) unit[S.t_off + v] = 0.f;
            if (bl_idx) bl_idx[S.t_off + v] = bl;
        }
    }
    // the list of voxels to trace, in box order
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(FULL, need);
    if (lane == 0) s_wcnt[warp] = __popc(m);
    __syncthreads();
    int off = 0, total = 0;
#pragma unroll
    for (int w = 0; w < 8; w++) {
        const int c = s_wcnt[w];
        off += w < warp ? c : 0;
        total += c;
    }
    if (need) {
        const int p = off + __popc(m & ((1u << lane) - 1u));
        s_v[p] = threadIdx.x;
        s_bl[p] = bl;
        s_fl[p] = fl;
    }
    __syncthreads();
    if (warp * 32 >= total) return;
    bool nz = false, cap = false;
    f3 bi = mk(0.f, 0.f, 0.f);
    if ((int)threadIdx.x < total) {
        const long long vt = vb + s_v[threadIdx.x];
        int xr, yr, zr;
        coords(vt, xr, yr, zr);
        const int x = S.t0[0] + xr, y = S.t0[1] + yr, z = S.t0[2] + zr;
        const f3 vox = mk(P.start[0] + x * P.voxel[0], P.start[1] + y * P.voxel[1], P.start[2] + z * P.voxel[2]);
        const f3 src = ld3(S.src);
        const float flt = s_fl[threadIdx.x];
        const float rpl = siddon_rpl(P, vox, src, cap);
        const float u = terma_per_fluence(P, rpl, vox, src, S.sad);
        const float t = flt > 0.f ? flt * u : 0.f;
        terma[S.t_off + vt] = t;
        if (unit) unit[S.t_off + vt] = u;
        if (bl_idx) bl_idx[S.t_off + vt] = s_bl[threadIdx.x];
        if (t != 0.f) {
            nz = true;
            // crop box works on calc-bbox-relative indices (host.cu:445-448)
            bi = mv(S.MB, mk((float)(x - P.bb0[0]), (float)(y - P.bb0[1]), (float)(z - P.bb0[2])));
        }
    }
    int kmin0 = nz ? f2key(bi.x) : INT_MAX, kmin1 = nz ? f2key(bi.y) : INT_MAX, kmin2 = nz ? f2key(bi.z) : INT_MAX;
    int kmax0 = nz ? f2key(bi.x) : INT_MIN, kmax1 = nz ? f2key(bi.y) : INT_MIN, kmax2 = nz ? f2key(bi.z) : INT_MIN;
    const unsigned cnt = __popc(__ballot_sync(FULL, nz));
    const bool anycap = __any_sync(FULL, cap);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        kmin0 = min(kmin0, __shfl_xor_sync(FULL, kmin0, o));
        kmin1 = min(kmin1, __shfl_xor_sync(FULL, kmin1, o));
        kmin2 = min(kmin2, __shfl_xor_sync(FULL, kmin2, o));
        kmax0 = max(kmax0, __shfl_xor_sync(FULL, kmax0, o));
        kmax1 = max(kmax1, __shfl_xor_sync(FULL, kmax1, o));
        kmax2 = max(kmax2, __shfl_xor_sync(FULL, kmax2, o));
    }
    if (lane == 0) {
        EeBeamGeom& G = geoms[b];
        if (cnt > 0) {
            atomicMin(&G.key_min[0], kmin0); atomicMin(&G.key_min[1], kmin1); atomicMin(&G.key_min[2], kmin2);
            atomicMax(&G.key_max[0], kmax0); atomicMax(&G.key_max[1], kmax1); atomicMax(&G.key_max[2], kmax2);
            atomicAdd(&G.nnz, cnt);
        }
        if (anycap) atomicExch(&G.status, 7 /* EE_ERR_SIDDON_ITER */);
    }
}

// TERMA with supersampling (ss > 1): one thread per TERMA-box voxel, walking
// the box brick by brick.
__global__ void __launch_bounds__(256, 1) k_terma_ss(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                    EeBeamGeom* __restrict__ geoms, const float* __restrict__ fluence,
                                                    float* __restrict__ terma, float* __restrict__ unit,
                                                    int* __restrict__ bl_idx) {
    const int b = blockIdx.z;
    const EeBeamSpec& S = specs[b];
    const long long bvol = ee_brick_vol(S.tn);
    long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool nz = false, cap = false;
    f3 bi = mk(0.f, 0.f, 0.f);
    // threads walk the box brick by brick (4x4x4, ee_brick_vol): each warp
    // traces half a brick of neighbouring rays and writes 128 contiguous bytes
    int xr = 0, yr = 0, zr = 0;
    bool inbox = false;
    if (v < bvol) {
        const long long brick = v >> 6;
        const int w = (int)(v & 63), nbx = (S.tn[0] + 3) >> 2, nby = (S.tn[1] + 3) >> 2;
        const long long bxy = brick % ((long long)nbx * nby);
        xr = (int)(bxy % nbx) * 4 + (w & 3);
        yr = (int)(bxy / nbx) * 4 + ((w >> 2) & 3);
        zr = (int)(brick / ((long long)nbx * nby)) * 4 + (w >> 4);
        inbox = xr < S.tn[0] && yr < S.tn[1] && zr < S.tn[2];
        if (!inbox) {  // padding of the last bricks: never sampled, kept zero
            terma[S.t_off + v] = 0.f;
            if (unit) unit[S.t_off + v] = 0.f;
            if (bl_idx) bl_idx[S.t_off + v] = -1;
        }
    }
    if (inbox) {
        // full-grid voxel index of this TERMA-box voxel
        int x = S.t0[0] + xr;
        int y = S.t0[1] + yr;
        int z = S.t0[2] + zr;
        f3 vox = mk(P.start[0] + x * P.voxel[0], P.start[1] + y * P.voxel[1], P.start[2] + z * P.voxel[2]);
        f3 src = ld3(S.src);
        float t = 0.f, u = 0.f;
        int bl = -1;
        {
            // supersampled TERMA (cudaSiddon.cu:248-258, 297-306): the mean
            // over ss^3 sub-voxel centres, each with its own beamlet lookup
            // and ray trace, summed x fastest (unit and bl_idx are not kept:
            // k_terma_T_ss recomputes the sub-voxel beamlets)
            const int ss = P.ss, nsub = ss * ss * ss;
            const float sv0 = P.voxel[0] / (float)ss, sv1 = P.voxel[1] / (float)ss, sv2 = P.voxel[2] / (float)ss;
            float acc = 0.f;
            for (int ii = 0; ii < nsub; ii++) {
                const int sx = ii % ss, sy = (ii / ss) % ss, sz = ii / (ss * ss);
                const f3 p = mk(P.start[0] + ((float)x - 0.5f) * P.voxel[0] + ((float)sx + 0.5f) * sv0,
                                P.start[1] + ((float)y - 0.5f) * P.voxel[1] + ((float)sy + 0.5f) * sv1,
                                P.start[2] + ((float)z - 0.5f) * P.voxel[2] + ((float)sz + 0.5f) * sv2);
                int bs = beamlet_of(S, p);
                if (bs == -2) bs = beamlet_point_fp64(S, (double)p.x, (double)p.y, (double)p.z);
                if (bs < 0) continue;
                const float fl = __ldg(fluence + S.fl_off + bs);
                if (!(fl > 0.f)) continue;
                const float rpl = siddon_rpl(P, p, src, cap);
                acc += fl * terma_per_fluence(P, rpl, p, src, S.sad);
            }
            t = acc / (float)nsub;
        }
        terma[S.t_off + v] = t;
        if (unit) unit[S.t_off + v] = u;
        if (bl_idx) bl_idx[S.t_off + v] = bl;
        if (t != 0.f) {
            nz = true;
            // crop box works on calc-bbox-relative indices (host.cu:445-448)
            bi = mv(S.MB, mk((float)(x - P.bb0[0]), (float)(y - P.bb0[1]), (float)(z - P.bb0[2])));
        }
    }
    // crop-box reduction (host.cu:442-459): min/max of BEV indices of voxels
    // with non-zero TERMA, as ordered-int keys.
    int kmin0 = nz ? f2key(bi.x) : INT_MAX, kmin1 = nz ? f2key(bi.y) : INT_MAX, kmin2 = nz ? f2key(bi.z) : INT_MAX;
    int kmax0 = nz ? f2key(bi.x) : INT_MIN, kmax1 = nz ? f2key(bi.y) : INT_MIN, kmax2 = nz ? f2key(bi.z) : INT_MIN;
    unsigned cnt = __popc(__ballot_sync(FULL, nz));
    bool anycap = __any_sync(FULL, cap);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        kmin0 = min(kmin0, __shfl_xor_sync(FULL, kmin0, o));
        kmin1 = min(kmin1, __shfl_xor_sync(FULL, kmin1, o));
        kmin2 = min(kmin2, __shfl_xor_sync(FULL, kmin2, o));
        kmax0 = max(kmax0, __shfl_xor_sync(FULL, kmax0, o));
        kmax1 = max(kmax1, __shfl_xor_sync(FULL, kmax1, o));
        kmax2 = max(kmax2, __shfl_xor_sync(FULL, kmax2, o));
    }
    // one lane per warp merges into the beam's keys: no block barrier, so a
    // warp whose rays are short does not wait for the block's longest trace
    if ((threadIdx.x & 31) == 0) {
        EeBeamGeom& G = geoms[b];
        if (cnt > 0) {
            atomicMin(&G.key_min[0], kmin0); atomicMin(&G.key_min[1], kmin1); atomicMin(&G.key_min[2], kmin2);
            atomicMax(&G.key_max[0], kmax0); atomicMax(&G.key_max[1], kmax1); atomicMax(&G.key_max[2], kmax2);
            atomicAdd(&G.nnz, cnt);
        }
        if (anycap) atomicExch(&G.status, 7 /* EE_ERR_SIDDON_ITER */);
    }
}

__global__ void k_geom_init(const EeBeamSpec* __restrict__ specs, EeBeamGeom* g, int n) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    for (int a = 0; a < 3; a++) { g[b].key_min[a] = f2key(FLT_MAX); g[b].key_max[a] = f2key(FLT_MIN); }
    g[b].nnz = 0;
    g[b].status = 0;
    // planned slot, or unbounded (the host sizes the arena after read-back)
    g[b].arena_off = specs[b].plan_off;
    g[b].arena_cap = specs[b].plan_cap;
}

// ------------------------------------------------------------- geometry --
// Crop box (host.cu:460-499) and findREV (host.cu:75-155) for every cone.
__global__ void k_geometry(EeParams P, const EeBeamSpec* __restrict__ specs, EeBeamGeom* __restrict__ geoms) {
    const int b = blockIdx.x;
    EeBeamGeom& G = geoms[b];
    const EeBeamSpec& S = specs[b];
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int ok = (G.status == 0);
        if (ok && G.nnz == 0) { G.status = 3; ok = 0; }
        if (ok) {
            float pl = P.penumbra / P.lat, plg = P.penumbra / P.lng;
            float mn[3], mx[3];
            for (int a = 0; a < 3; a++) { mn[a] = key2f(G.key_min[a]); mx[a] = key2f(G.key_max[a]); }
            mn[0] -= pl; mn[1] -= plg; mn[2] -= pl;
            mx[0] += pl; mx[1] += plg; mx[2] += pl;
            for (int a = 0; a < 3; a++) {
                float s = snap_ceilf(fabsf(mx[a] - mn[a]));
                if (!(s > 0.f) || s >= 1000.f) { ok = 0; }
                G.bev[a] = ok ? (int)s : 0;
                G.bmin[a] = mn[a];
            }
            if (!ok) G.status = 3;
            f3 tmn = mv(S.MBi, mk(mn[0], mn[1], mn[2]));
            G.lim_min[0] = P.start[0] + (tmn.x + P.bb0[0]) * P.voxel[0];
            G.lim_min[1] = P.start[1] + (tmn.y + P.bb0[1]) * P.voxel[1];
            G.lim_min[2] = P.start[2] + (tmn.z + P.bb0[2]) * P.voxel[2];
            for (int a = 0; a < 3; a++) G.lim_off[a] = (G.lim_min[a] - P.start[a]) / P.voxel[a];
            G.v_beam = (long long)G.bev[0] * G.bev[1] * G.bev[2];
        }
        s_ok = ok;
    }
    __syncthreads();
    if (!s_ok) return;
    const f3 bd = mk(G.bev[0] * P.lat, G.bev[1] * P.lng, G.bev[2] * P.lat);
    for (int r = threadIdx.x; r < P.nrays; r += blockDim.x) {
        const EeRayConst& RC = P.rays[r];
        EeRayGeom& R = G.ray[r];
        float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {FLT_MIN, FLT_MIN, FLT_MIN};
        for (int c = 0; c < 8; c++) {
            f3 o = mv(RC.MK, mk(bd.x * (c & 1), bd.y * ((c >> 1) & 1), bd.z * ((c >> 2) & 1)));
            mn[0] = fminf(mn[0], o.x); mn[1] = fminf(mn[1], o.y); mn[2] = fminf(mn[2], o.z);
            mx[0] = fmaxf(mx[0], o.x); mx[1] = fmaxf(mx[1], o.y); mx[2] = fmaxf(mx[2], o.z);
        }
        int sz[3] = {(int)snap_ceilf(fabsf(mx[1] - mn[1]) / P.lng), (int)snap_ceilf(fabsf(mx[2] - mn[2]) / P.lat),
                     (int)snap_ceilf(fabsf(mx[0] - mn[0]) / P.lat)};
        bool bad = false;
        for (int a = 0; a < 3; a++) {
            if (P.max_rev[a] > 0 && sz[a] > P.max_rev[a]) bad = true;
            R.rev[a] = sz[a];
        }
        if (sz[0] > EE_MAX_LINE || sz[0] <= 0 || sz[1] <= 0 || sz[2] <= 0) bad = true;
        if (bad) atomicExch(&G.status, 4);
        R.nlines = sz[1] * sz[2];
        f3 q0 = mk(mn[0] / P.lat, mn[1] / P.lng, mn[2] / P.lat);
        R.q0[0] = q0.x; R.q0[1] = q0.y; R.q0[2] = q0.z;
        // REV vector (tZ, tX, tY) + q0 -> BEV (inverseRotateKernel)
        f3 B0 = mv(RC.MKi, q0);
        f3 Bx = mk(RC.MKi[1], RC.MKi[4], RC.MKi[7]);  // column for tX (REV y)
        f3 By = mk(RC.MKi[2], RC.MKi[5], RC.MKi[8]);  // column for tY (REV z)
        f3 Bz = mk(RC.MKi[0], RC.MKi[3], RC.MKi[6]);  // column for tZ (REV x)
        f3 lo = mk(G.lim_off[0], G.lim_off[1], G.lim_off[2]);
        f3 G0 = lo + mv(S.MBi, B0), Gx = mv(S.MBi, Bx), Gy = mv(S.MBi, By), Gz = mv(S.MBi, Bz);
        R.B0[0] = B0.x; R.B0[1] = B0.y; R.B0[2] = B0.z;
        R.Bx[0] = Bx.x; R.Bx[1] = Bx.y; R.Bx[2] = Bx.z;
        R.By[0] = By.x; R.By[1] = By.y; R.By[2] = By.z;
        R.Bz[0] = Bz.x; R.Bz[1] = Bz.y; R.Bz[2] = Bz.z;
        R.G0[0] = G0.x; R.G0[1] = G0.y; R.G0[2] = G0.z;
        R.Gx[0] = Gx.x; R.Gx[1] = Gx.y; R.Gx[2] = Gx.z;
        R.Gy[0] = Gy.x; R.Gy[1] = Gy.y; R.Gy[2] = Gy.z;
        R.Gz[0] = Gz.x; R.Gz[1] = Gz.y; R.Gz[2] = Gz.z;
        for (int i = 0; i < 9; i++) R.M[i] = RC.MK[i];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                R.A[3 * i + j] = RC.MK[3 * i] * S.MB[j] + RC.MK[3 * i + 1] * S.MB[3 + j] + RC.MK[3 * i + 2] * S.MB[6 + j];
    }
    __syncthreads();
    if (threadIdx.x == 0 && G.status == 0) {
        // patient-index AABB of the crop box dilated by 2 BEV voxels
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int c = 0; c < 8; c++) {
            f3 bc = mk((c & 1) ? G.bev[0] + 2.f : -2.f, ((c >> 1) & 1) ? G.bev[1] + 2.f : -2.f,
                       ((c >> 2) & 1) ? G.bev[2] + 2.f : -2.f);
            f3 t = mv(S.MBi, bc) + mk(G.lim_off[0], G.lim_off[1], G.lim_off[2]);
            lo[0] = fminf(lo[0], t.x); lo[1] = fminf(lo[1], t.y); lo[2] = fminf(lo[2], t.z);
            hi[0] = fmaxf(hi[0], t.x); hi[1] = fmaxf(hi[1], t.y); hi[2] = fmaxf(hi[2], t.z);
        }
        int x0 = max(P.bb0[0], (int)floorf(lo[0]) - 1), x1 = min(P.bb0[0] + P.bbs[0] - 1, (int)ceilf(hi[0]) + 1);
        int y0 = max(P.bb0[1], (int)floorf(lo[1]) - 1), y1 = min(P.bb0[1] + P.bbs[1] - 1, (int)ceilf(hi[1]) + 1);
        int z0 = max(P.bb0[2], (int)floorf(lo[2]) - 1), z1 = min(P.bb0[2] + P.bbs[2] - 1, (int)ceilf(hi[2]) + 1);
        G.gx0 = x0; G.gy0 = y0; G.gz0 = z0;
        G.gnx = max(0, x1 - x0 + 1); G.gny = max(0, y1 - y0 + 1); G.gnz = max(0, z1 - z0 + 1);
        G.rows = (int)ee_gather_groups(G.gny, G.gnz);
        G.tiles = ((G.gnx + 7) / 8) * ((G.gny + 7) / 8) * ((G.gnz + 3) / 4);
        long long off = 0;
        int ml = 0, mls = 0;
        for (int r = 0; r < P.nrays; r++) {
            // bricked REV arrays (rev_brick); the lane kernels run one lane
            // slot per line of an 8 (tY) x 4 (tZ) tile
            G.ray[r].offset = off;
            off += ee_brick_vol(G.ray[r].rev);
            ml = max(ml, G.ray[r].rev[0]);
            mls = max(mls, ((G.ray[r].rev[1] + 7) >> 3) * 8 * (((G.ray[r].rev[2] + 3) >> 2) * 4));
        }
        G.rev_total = off;
        // the gather addresses a cone's REV array with a 32-bit offset
        if (off > 2147483647ll) G.status = 4;  // EE_ERR_REV_SIZE
        G.max_line = ml;
        G.max_lines = mls;
        if (G.arena_cap > 0 && off > G.arena_cap) G.status = 8;
    }
}


// ------------------------------------------------------- cone: gather ----
// Samples of REV line (tY, tZ) that can be valid: the line's intersection
// with the BEV crop box and the calc bbox (both convex, so one segment),
// widened by one sample for rounding.  Outside it every sample is a sentinel
// (-3 outside the BEV box, -2 outside the bbox, device.cu:51-70) and its dose
// is zero, so neither the gather nor the scans visit it.
__device__ __forceinline__ void line_segment(const EeParams& P, const EeBeamGeom& G, const EeRayGeom& R, int tY,
                                             int tZ, int L, int& i0, int& n) {
    const f3 bl = ld3(R.B0) + ld3(R.By) * (float)tY + ld3(R.Bz) * (float)tZ;
    const f3 gl = ld3(R.G0) + ld3(R.Gy) * (float)tY + ld3(R.Gz) * (float)tZ;
    const float c[6] = {bl.x, bl.y, bl.z, gl.x, gl.y, gl.z};
    const float m[6] = {R.Bx[0], R.Bx[1], R.Bx[2], R.Gx[0], R.Gx[1], R.Gx[2]};
    const float lo[6] = {0.f, 0.f, 0.f, (float)P.bb0[0], (float)P.bb0[1], (float)P.bb0[2]};
    const float hi[6] = {(float)G.bev[0], (float)G.bev[1], (float)G.bev[2], (float)(P.bb0[0] + P.bbs[0]),
                         (float)(P.bb0[1] + P.bbs[1]), (float)(P.bb0[2] + P.bbs[2])};
    float a = 0.f, b = (float)(L - 1);
#pragma unroll
    for (int k = 0; k < 6; k++) {
        if (fabsf(m[k]) < 1e-6f) {
            if (c[k] < lo[k] - 1e-3f || c[k] > hi[k] + 1e-3f) { n = 0; i0 = 0; return; }
        } else {
            float t0 = (lo[k] - c[k]) / m[k], t1 = (hi[k] - c[k]) / m[k];
            a = fmaxf(a, fminf(t0, t1));
            b = fminf(b, fmaxf(t0, t1));
        }
    }
    if (!(a <= b + 2.f)) { n = 0; i0 = 0; return; }
    i0 = max(0, (int)floorf(a) - 1);
    int i1 = min(L - 1, (int)ceilf(b) + 1);
    n = max(0, i1 - i0 + 1);
}

// Samples of a REV line that k_gather can read (and k_gather_T can add to):
// k_gather visits voxels within 2 BEV voxels of the crop box and reads the
// REV cells within one REV step (per axis) of each voxel's REV point, i.e.
// within sum_k |B[a][k]| BEV units per axis a.  So the line's intersection
// with the crop box dilated by 2 + sum_k |B[a][k]| (+0.05, +1 sample each
// side) holds every sample either kernel touches; samples outside it are
// never read and need no zero.  z1 < z0: none.
__device__ __forceinline__ void line_read_span(const EeBeamGeom& G, const EeRayGeom& R, int tY, int tZ, int L,
                                               int& z0, int& z1) {
    const f3 bl = ld3(R.B0) + ld3(R.By) * (float)tY + ld3(R.Bz) * (float)tZ;
    const float c[3] = {bl.x, bl.y, bl.z};
    float a = 0.f, b = (float)(L - 1);
    z0 = 0;
    z1 = -1;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float D = 2.05f + fabsf(R.Bx[k]) + fabsf(R.By[k]) + fabsf(R.Bz[k]);
        const float lo = -D, hi = (float)G.bev[k] + D, m = R.Bx[k];
        if (fabsf(m) < 1e-6f) {
            if (c[k] < lo || c[k] > hi) return;
        } else {
            const float t0 = (lo - c[k]) / m, t1 = (hi - c[k]) / m;
            a = fmaxf(a, fminf(t0, t1));
            b = fminf(b, fmaxf(t0, t1));
        }
    }
    if (!(a <= b + 2.f)) return;
    z0 = max(0, (int)floorf(a) - 1);
    z1 = min(L - 1, (int)ceilf(b) + 1);
}

// Zero the samples of a line's read span outside [i0, i0 + n) (the cone
// writes those): the REV dose arena needs no separate clear.
__device__ __forceinline__ void zero_outside_segment(float* out, const Brick& Bv, int z0, int z1, int i0, int n,
                                                     int first, int stride) {
    const int e0 = n > 0 ? min(z1 + 1, i0) : z1 + 1;  // [z0, e0) before the segment
    const int s1 = n > 0 ? max(z0, i0 + n) : z1 + 1;  // [s1, z1] after it
    for (int i = z0 + first; i < e0; i += stride) out[bk_x(i)] = 0.f;
    for (int i = s1 + first; i <= z1; i += stride) out[bk_x(i)] = 0.f;
}

// REV resample of samples i0..i0+n-1 of one line into shared memory
// (device.cu:47-79): density sentinel -3 outside the BEV crop box, -2 outside
// the calc bbox; TERMA is zero at sentinel samples (never written by the
// reference).
__device__ __forceinline__ void gather_line(const EeParams& P, const EeBeamSpec& S, const EeBeamGeom& G,
                                            const EeRayGeom& R, const float* __restrict__ terma_b, int tY, int tZ,
                                            int i0, int n, int lane, float* rho, float* T, int stride = 32) {
    const f3 bl = ld3(R.B0) + ld3(R.By) * (float)tY + ld3(R.Bz) * (float)tZ;
    const f3 gl = ld3(R.G0) + ld3(R.Gy) * (float)tY + ld3(R.Gz) * (float)tZ;
    const f3 bx = ld3(R.Bx), gx = ld3(R.Gx);
    const float bsx = (float)G.bev[0], bsy = (float)G.bev[1], bsz = (float)G.bev[2];
    const float b0x = (float)P.bb0[0], b0y = (float)P.bb0[1], b0z = (float)P.bb0[2];
    const float b1x = (float)(P.bb0[0] + P.bbs[0]), b1y = (float)(P.bb0[1] + P.bbs[1]), b1z = (float)(P.bb0[2] + P.bbs[2]);
    for (int k = lane; k < n; k += stride) {
        const float fi = (float)(i0 + k);
        f3 bev = bl + bx * fi;
        float r = -3.f, t = 0.f;
        if (!(bev.x < 0.f || bev.y < 0.f || bev.z < 0.f || bev.x >= bsx || bev.y >= bsy || bev.z >= bsz)) {
            f3 g = gl + gx * fi;
            if (g.x < b0x || g.x >= b1x || g.y < b0y || g.y >= b1y || g.z < b0z || g.z >= b1z) {
                r = -2.f;
            } else {
                r = tex3D<float>(P.dens_tex, g.x + 0.5f, g.y + 0.5f, g.z + 0.5f);
                if (terma_b)
                    t = tri_brick(terma_b, brick_of(S.tn), g.x - (float)S.t0[0], g.y - (float)S.t0[1],
                                   g.z - (float)S.t0[2]);
            }
        }
        rho[k] = r;
        if (T) T[k] = t;
    }
}

// --------------------------------------------------- cone: exp scans -----
// Collapsed-cone line convolution with K(r) = A/a (1-e^{-ar}) + B/b (1-e^{-br})
// on the reference discretisation (device.cu:140-211: no self term, radii
// measured from the receiving voxel's boundary to the source voxel's centre):
//   D_i = sum_c A_c/a_c [ Y_i + T_{i-1} (1 - h_{i-1}) ],
//   Y_{i+1} = h_i^2 Y_i + T_{i-1} h_i (1 - h_{i-1} h_i),  h_j = e^{-a p_j/2},
// p = delr*rho, with p = T = 0 at sentinel samples.  Work-efficient warp
// scan: each lane owns a contiguous chunk of the line, composes its chunk's
// affine maps Y -> F Y + U sequentially, one 5-step shuffle scan over the 32
// chunk maps gives every lane its starting Y, and a second sequential pass
// replays the chunk.  Odd chunk lengths keep the lanes' shared-memory
// strides bank-conflict free.  FWD walks ascending i (contributions from
// k < i); the reverse pass adds its part to D and applies 1/nphi.

// inclusive warp scan of affine maps (F, U): lane j gets maps 0..j composed
__device__ __forceinline__ void warp_affine_scan(int lane, float& F1, float& U1, float& F2, float& U2) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        float fF1 = __shfl_up_sync(FULL, F1, off), fU1 = __shfl_up_sync(FULL, U1, off);
        float fF2 = __shfl_up_sync(FULL, F2, off), fU2 = __shfl_up_sync(FULL, U2, off);
        if (lane >= off) {
            U1 = fmaf(F1, fU1, U1); F1 *= fF1;
            U2 = fmaf(F2, fU2, U2); F2 *= fF2;
        }
    }
}

template <bool FWD>
__device__ __forceinline__ void line_scan(const float* rho, const float* T, int n, int lane, float delr,
                                          const float* prm, float* D, float inv_nphi) {
    const float c1 = prm[0] / prm[1], c2 = prm[2] / prm[3];
    const float e1 = -0.5f * prm[1] * delr, e2 = -0.5f * prm[3] * delr;  // h = exp(e * rho)
    const int cs = ((n + 31) >> 5) | 1;
    const int w0 = min(n, lane * cs), w1 = min(n, w0 + cs);
    // previous sample (walk order) of the chunk's first step
    float tm0 = 0.f, hm10 = 1.f, hm20 = 1.f;
    if (w0 > 0 && w0 < w1) {
        const int im = FWD ? w0 - 1 : n - w0;
        const float rm = rho[im];
        if (rm >= 0.f) { tm0 = T[im]; hm10 = __expf(e1 * rm); hm20 = __expf(e2 * rm); }
    }
    // pass 1: compose this chunk's steps
    float F1 = 1.f, U1 = 0.f, F2 = 1.f, U2 = 0.f;
    float tm = tm0, hm1 = hm10, hm2 = hm20;
    for (int w = w0; w < w1; w++) {
        const int i = FWD ? w : n - 1 - w;
        const float r = rho[i];
        float t = 0.f, h1 = 1.f, h2 = 1.f;
        if (r >= 0.f) { t = T[i]; h1 = __expf(e1 * r); h2 = __expf(e2 * r); }
        const float f1 = h1 * h1, f2 = h2 * h2;
        U1 = fmaf(f1, U1, tm * h1 * (1.f - hm1 * h1)); F1 *= f1;
        U2 = fmaf(f2, U2, tm * h2 * (1.f - hm2 * h2)); F2 *= f2;
        tm = t; hm1 = h1; hm2 = h2;
    }
    warp_affine_scan(lane, F1, U1, F2, U2);
    // Y at the start of the chunk: the line starts from Y = 0
    float Y1 = __shfl_up_sync(FULL, U1, 1), Y2 = __shfl_up_sync(FULL, U2, 1);
    if (lane == 0) { Y1 = 0.f; Y2 = 0.f; }
    // pass 2: replay
    tm = tm0; hm1 = hm10; hm2 = hm20;
    for (int w = w0; w < w1; w++) {
        const int i = FWD ? w : n - 1 - w;
        const float r = rho[i];
        float t = 0.f, h1 = 1.f, h2 = 1.f;
        if (r >= 0.f) { t = T[i]; h1 = __expf(e1 * r); h2 = __expf(e2 * r); }
        const float d = c1 * (Y1 + tm * (1.f - hm1)) + c2 * (Y2 + tm * (1.f - hm2));
        if (FWD) D[i] = d;
        else D[i] = r >= 0.f ? (D[i] + d) * inv_nphi : 0.f;
        Y1 = fmaf(h1 * h1, Y1, tm * h1 * (1.f - hm1 * h1));
        Y2 = fmaf(h2 * h2, Y2, tm * h2 * (1.f - hm2 * h2));
        tm = t; hm1 = h1; hm2 = h2;
    }
}

// Transpose of line_scan<FWD> for the TERMA adjoint.  With g_i the incoming
// REV-dose gradient (already / nphi, zero at sentinels) and im the forward
// walk's previous sample of i,
//   Z_i = c g_i + h_i^2 Z_{i+1}         (walking opposite to FWD),
//   Tbar_im += c g_i (1 - h_im) + Z_{i+1} h_i (1 - h_im h_i),
// with the same chunked scan.  im is the next sample of this walk, so its
// h is computed once and carried.
template <bool FWD>
__device__ __forceinline__ void line_scan_T(const float* rho, const float* g, int n, int lane, float delr,
                                            const float* prm, float* Tb) {
    const float c1 = prm[0] / prm[1], c2 = prm[2] / prm[3];
    const float e1 = -0.5f * prm[1] * delr, e2 = -0.5f * prm[3] * delr;
    const int cs = ((n + 31) >> 5) | 1;
    const int v0 = min(n, lane * cs), v1 = min(n, v0 + cs);
    // pass 1: compose Z -> h^2 Z + c g over the chunk
    float F1 = 1.f, U1 = 0.f, F2 = 1.f, U2 = 0.f;
    for (int v = v0; v < v1; v++) {
        const int i = FWD ? n - 1 - v : v;
        const float r = rho[i];
        float gi = 0.f, h1 = 1.f, h2 = 1.f;
        if (r >= 0.f) { gi = g[i]; h1 = __expf(e1 * r); h2 = __expf(e2 * r); }
        const float f1 = h1 * h1, f2 = h2 * h2;
        U1 = fmaf(f1, U1, c1 * gi); F1 *= f1;
        U2 = fmaf(f2, U2, c2 * gi); F2 *= f2;
    }
    warp_affine_scan(lane, F1, U1, F2, U2);
    float Z1 = __shfl_up_sync(FULL, U1, 1), Z2 = __shfl_up_sync(FULL, U2, 1);
    if (lane == 0) { Z1 = 0.f; Z2 = 0.f; }
    // pass 2: replay, emitting the TERMA-gradient contributions
    float h1 = 1.f, h2 = 1.f, gi = 0.f;
    bool vi = false;
    if (v0 < v1) {
        const int i = FWD ? n - 1 - v0 : v0;
        const float r = rho[i];
        if (r >= 0.f) { vi = true; gi = g[i]; h1 = __expf(e1 * r); h2 = __expf(e2 * r); }
    }
    for (int v = v0; v < v1; v++) {
        const int i = FWD ? n - 1 - v : v;
        const int im = FWD ? i - 1 : i + 1;
        float hm1 = 1.f, hm2 = 1.f, gm = 0.f;
        bool vm = false;
        if (im >= 0 && im < n) {
            const float rm = rho[im];
            if (rm >= 0.f) { vm = true; gm = g[im]; hm1 = __expf(e1 * rm); hm2 = __expf(e2 * rm); }
        }
        if (vm) {
            const float c = c1 * gi * (1.f - hm1) + Z1 * h1 * (1.f - hm1 * h1) + c2 * gi * (1.f - hm2) +
                            Z2 * h2 * (1.f - hm2 * h2);
            Tb[im] += c;  // each im has exactly one i per pass
        }
        (void)vi;
        Z1 = fmaf(h1 * h1, Z1, c1 * gi);
        Z2 = fmaf(h2 * h2, Z2, c2 * gi);
        // the next step's sample is im
        h1 = hm1; h2 = hm2; gi = gm; vi = vm;
    }
}

// --------------------------------------------------- cone: table walk ----
// RowConvolve walk (device.cu:126-211) over shared memory with exact FP32
// linear interpolation of the cumulative kernel between radial boundaries.
// coef == nullptr: returns sum_k w_k T_k; otherwise adds w_k * gscale into
// coef[k] with shared-memory atomics (adjoint).
__device__ __forceinline__ float table_walk(const float* rho, const float* T, int L, int i, int step, const float* K,
                                            const float* RAD, int nr, float delr, float* coef, float gscale) {
    float sum = 0.f, r_eff = 0.f, cumval = 0.f, last_cumval = 0.f, last_rad = 0.f, next_rad = RAD[0];
    int rad_start = 0, k1 = i;
    do {
        k1 += step;
        if (k1 < 0 || k1 >= L) break;
        float de = delr * rho[k1];
        r_eff += 0.5f * de;
        if (r_eff > RAD[nr - 1]) break;
        while (next_rad < r_eff) {
            if (rad_start == nr - 1) break;
            last_rad = next_rad;
            next_rad = RAD[++rad_start];
        }
        float interp = (r_eff - last_rad) / (next_rad - last_rad);
        if (rad_start == 0) cumval = interp * K[0];
        else cumval = K[rad_start - 1] + interp * (K[rad_start] - K[rad_start - 1]);
        float w = cumval - last_cumval;
        if (coef) atomicAdd(coef + k1, w * gscale);
        else sum += w * T[k1];
        last_cumval = cumval;
        r_eff += 0.5f * de;
    } while (rad_start < nr - 1);
    return sum;
}

// ------------------------------------------------------- cone kernels ----
constexpr int CONE_WARPS = 4;

__global__ void __launch_bounds__(CONE_WARPS * 32) k_cone(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                          const EeBeamGeom* __restrict__ geoms,
                                                          const float* __restrict__ terma, float* __restrict__ rev,
                                                          int maxL) {
    extern __shared__ float sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ray = blockIdx.y, b = blockIdx.z;
    const EeBeamGeom& G = geoms[b];
    float* tabK = sm + (size_t)CONE_WARPS * 3 * maxL;  // [2][nradii] kernel rows + radii
    float* tabR = tabK + 2 * EE_MAX_RADII;
    if (P.mode != EE_KERNEL_EXP) {
        const EeRayConst& RC = P.rays[ray];
        for (int k = threadIdx.x; k < P.nradii; k += blockDim.x) {
            tabK[k] = P.cumkern[RC.row_fwd * P.nradii + k];
            tabK[EE_MAX_RADII + k] = P.cumkern[RC.row_rev * P.nradii + k];
            tabR[k] = P.radii[k];
        }
        __syncthreads();
    }
    if (G.status != 0) return;
    const EeRayGeom& R = G.ray[ray];
    const int line = blockIdx.x * CONE_WARPS + warp;
    if (line >= R.nlines) return;
    const int L = R.rev[0];
    const int tY = line % R.rev[1], tZ = line / R.rev[1];
    float* rho = sm + (size_t)warp * 3 * maxL;
    float* T = rho + maxL;
    float* D = T + maxL;
    // bricked REV arena (rev_brick): sample i at out + bk_x(i)
    const Brick Bv = rev_brick(R.rev[0], R.rev[1], R.rev[2]);
    float* out = rev + G.arena_off + R.offset + rev_line(Bv, tY, tZ);
    int i0, n, z0, z1;
    line_segment(P, G, R, tY, tZ, L, i0, n);
    line_read_span(G, R, tY, tZ, L, z0, z1);
    zero_outside_segment(out, Bv, z0, z1, i0, n, lane, 32);
    if (n > 0) {
        gather_line(P, specs[b], G, R, terma + specs[b].t_off, tY, tZ, i0, n, lane, rho, T);
        __syncwarp();
        const float inv_nphi = 1.f / (float)P.nphi;
        const EeRayConst& RC = P.rays[ray];
        if (P.mode == EE_KERNEL_EXP) {
            line_scan<true>(rho, T, n, lane, P.lng, P.expp + 4 * RC.row_fwd, D, inv_nphi);
            __syncwarp();
            line_scan<false>(rho, T, n, lane, P.lng, P.expp + 4 * RC.row_rev, D, inv_nphi);
        } else {
            for (int k = lane; k < n; k += 32) {
                float v = 0.f;
                if (rho[k] >= 0.f) {
                    v = table_walk(rho, T, n, k, -1, tabK, tabR, P.nradii, P.lng, nullptr, 0.f);
                    v += table_walk(rho, T, n, k, +1, tabK + EE_MAX_RADII, tabR, P.nradii, P.lng, nullptr, 0.f);
                    v = __fdiv_rn(v, (float)P.nphi);
                }
                D[k] = v;
            }
        }
        __syncwarp();
    }
    for (int k = lane; k < n; k += 32) out[bk_x(i0 + k)] = D[k];
}

// ------------------------------------- cone: exact table scan, O(n nr) ----
// The reference's RowConvolve walk (device.cu:126-211) with the cumulative
// kernel interpolated linearly between its nr = 24 radial boundaries (the
// reference's N_KERNEL_RADII), evaluated exactly in O(n * nr) per line
// instead of O(n^2).
//
// One walk direction at a time, in walk order w = 0..n-1 (FWD: line order,
// the sources of receiver w are k < w; reverse: the mirrored order).  With
// d_w = delr * rho_w (0 at sentinels), P_w = sum_{m<w} d_m and
// M_w = P_w + d_w / 2, the walk from receiver w gives source k the
// radiological distance c_k = P_w - M_k (half the source voxel plus every
// voxel in between, device.cu:144-164).  It includes every source with
// c_k <= R_{nr-2} plus the first one beyond that, if its c_k <= R_{nr-1} (the
// loop's two exits, device.cu:146-147,171).  With s the last included source
// and V_k = T_k - T_{k-1}, summation by parts of sum T_k (K(c_k) - K(c_{k+1}))
// gives
//   D_w = T_s K(c_s) + sum_{k=s+1}^{w-1} V_k K(c_k).
// K is linear on segment j, (Rm_j, R_j] with Rm_j = R_{j-1} (Rm_0 = 0):
// K(c) = Km_j + beta_j (c - Rm_j), Km_j = K_{j-1} (Km_0 = 0).  The sources of
// segment j form the index window [x_j, x_{j-1}) with x_j = the first k whose
// M_k >= P_w - R_j (x_{-1} = w), so with the prefix sums SV_k = T_{k-1} and
// SVM_k = sum_{m<k} V_m M_m a window costs two lookups, and regrouping the
// windows at their shared ends leaves one per boundary:
//   D_w = T_s K(c_s) + beta_0 (P_w SV_w - SVM_w)
//       + sum_{j=0}^{nr-3} gamma_{j+1} ((P_w - R_j) SV_{x_j} - SVM_{x_j})
//       - coef_{nr-2} SV_{x_{nr-2}} + beta_{nr-2} SVM_{x_{nr-2}},
// gamma_j = beta_j - beta_{j-1}, coef_j = Km_j + beta_j (P_w - Rm_j), every
// x_j clipped below at s + 1 (source s enters through its own term).  Each
// lane walks a contiguous chunk of receivers; the x_j only move forward as w
// grows, so after a binary search for the chunk's first receiver each is
// advanced, not searched.  Plain FP32: the regrouped terms are bounded by
// |gamma| * P * T, measured at <= 2e-5 of the line's maximum against the
// FP64 walk on 1000-sample lines.
//
// Transpose (TERMA gradient from the REV-dose gradient g): with the last
// receiver b_k whose walk reaches source k (P_i - M_{k+1} <= R_{nr-2} and
// P_i - M_k <= R_{nr-1}, or i = k + 1), and
//   Phi_b(m) = sum_{i <= b} g_i K(P_i - m)   (K = 0 for P_i <= m),
// source k receives Tbar_k = Phi_{b_k}(M_k) - Phi_{b_k}(M_{k+1}).  Phi_b(m)
// regroups the same way over the receiver windows y_j = the first i with
// P_i > m + R_j, with prefix sums Sg_i = sum_{m<i} g_m and
// SgP_i = sum_{m<i} g_m P_m; source k evaluates W_k = Phi_{b_k}(M_k) and
// U_k = Phi_{b_{k-1}}(M_k) in one pass over its pointers, and
// Tbar_k = W_k - U_{k+1}.
constexpr int TAB_NR = 24;            // radial boundaries of the fast path
constexpr int TAB_NB = TAB_NR - 1;    // receiver windows of the forward walk

// Per-block kernel-row tables: R, Rm (shared by both rows), then for the
// forward row and for the reverse row Km, beta, gamma and the suffix sums
// SG_j = sum_{m=j}^{nr-2} gamma_{m+1} and SGR_j = sum_{m=j}^{nr-2}
// gamma_{m+1} R_m (EE_MAX_RADII each).  Window ends that cannot move on a
// line (radius at least the line's radiological length) all sit at the same
// position, so their terms are summed in closed form from SG and SGR.
struct TabRow {
    const float *R, *Rm, *Km, *B, *G, *SG, *SGR;
};
constexpr int TAB_SMEM = 12 * EE_MAX_RADII;

// Fills the tables; the caller synchronises the block before using them.
__device__ __forceinline__ void tab_tables(const EeParams& P, const EeRayConst& RC, float* t) {
    for (int k = threadIdx.x; k < TAB_NR * 2; k += blockDim.x) {
        const int row = k < TAB_NR ? RC.row_fwd : RC.row_rev, j = k % TAB_NR;
        const float* Kr = P.cumkern + (size_t)row * P.nradii;
        const float R = P.radii[j], Rm = j ? P.radii[j - 1] : 0.f;
        const float K = Kr[j], Km = j ? Kr[j - 1] : 0.f;
        const float b = (K - Km) / (R - Rm);
        float bm = 0.f;
        if (j) bm = (Km - (j > 1 ? Kr[j - 2] : 0.f)) / (Rm - (j > 1 ? P.radii[j - 2] : 0.f));
        float* o = t + (k < TAB_NR ? 2 : 7) * EE_MAX_RADII;
        o[j] = Km;
        o[EE_MAX_RADII + j] = b;
        o[2 * EE_MAX_RADII + j] = b - bm;
        if (k < TAB_NR) {
            t[j] = R;
            t[EE_MAX_RADII + j] = Rm;
        }
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        float* o = t + (threadIdx.x == 0 ? 2 : 7) * EE_MAX_RADII;
        float sg = 0.f, sgr = 0.f;
        o[3 * EE_MAX_RADII + TAB_NR - 1] = 0.f;
        o[4 * EE_MAX_RADII + TAB_NR - 1] = 0.f;
        for (int j = TAB_NR - 2; j >= 0; j--) {
            sg += o[2 * EE_MAX_RADII + j + 1];
            sgr = fmaf(o[2 * EE_MAX_RADII + j + 1], t[j], sgr);
            o[3 * EE_MAX_RADII + j] = sg;
            o[4 * EE_MAX_RADII + j] = sgr;
        }
    }
}

__device__ __forceinline__ TabRow tab_row(const float* t, bool fwd) {
    const float* o = t + (fwd ? 2 : 7) * EE_MAX_RADII;
    return TabRow{t, t + EE_MAX_RADII, o, o + EE_MAX_RADII, o + 2 * EE_MAX_RADII, o + 3 * EE_MAX_RADII,
                  o + 4 * EE_MAX_RADII};
}

// exclusive prefix sum over the W-lane group of `lane` (W = 32: the warp; W =
// 16: each half separately); all 32 lanes take part
template <int W = 32>
__device__ __forceinline__ float warp_excl_scan(float x, int lane) {
    float s = x;
#pragma unroll
    for (int off = 1; off < W; off <<= 1) {
        const float y = __shfl_up_sync(FULL, s, off, W);
        if (lane >= off) s += y;
    }
    return s - x;
}

template <bool FWD>
__device__ __forceinline__ int wmap(int w, int n) { return FWD ? w : n - 1 - w; }

// lane chunks of a line over the W lanes that share it: the shortest length
// that covers it, so that as many lanes as possible work (measured faster
// than odd lengths, which spread the lanes' strided shared-memory accesses
// over all the banks but leave up to a third of the lanes idle)
template <int W = 32>
__device__ __forceinline__ void tab_chunk(int n, int lane, int& w0, int& w1) {
    const int cs = max(1, (n + W - 1) / W);
    w0 = min(n, lane * cs);
    w1 = min(n, w0 + cs);
}

// M_w, P_w, SV_w = T_{w-1} and SVM_w in walk order (separate arrays: lanes
// reading scattered samples then spread over all the banks); T is 0 at
// sentinels.
template <bool FWD, int W = 32>
__device__ __forceinline__ void tab_build(const float* rho, const float* T, int n, int lane, float delr, float* Mv,
                                          float* Pv, float* SVv, float* SVMv) {
    int w0, w1;
    tab_chunk<W>(n, lane, w0, w1);
    const float tp0 = (w0 > 0 && w0 < w1) ? T[wmap<FWD>(w0 - 1, n)] : 0.f;
    float sd = 0.f, svm = 0.f, tp = tp0;
    for (int w = w0; w < w1; w++) {  // chunk sums, P local to the chunk
        const int i = wmap<FWD>(w, n);
        const float r = rho[i], t = T[i];
        const float d = r >= 0.f ? delr * r : 0.f;
        svm = fmaf(t - tp, fmaf(0.5f, d, sd), svm);
        sd += d;
        tp = t;
    }
    const float Pst = warp_excl_scan<W>(sd, lane);
    float S = warp_excl_scan<W>(fmaf(Pst, tp - tp0, svm), lane);
    float Pw = Pst;
    tp = tp0;
    for (int w = w0; w < w1; w++) {
        const int i = wmap<FWD>(w, n);
        const float r = rho[i], t = T[i];
        const float d = r >= 0.f ? delr * r : 0.f;
        const float M = fmaf(0.5f, d, Pw);
        Mv[w] = M;
        Pv[w] = Pw;
        SVv[w] = tp;
        SVMv[w] = S;
        S = fmaf(t - tp, M, S);
        Pw += d;
        tp = t;
    }
}

// Receivers of one walk direction.  FWD writes D[i]; the reverse direction
// adds its part, divides by nphi and zeroes sentinel samples.  X: this lane's
// window ends, X[32 j] = x_j (shared memory, so the loops over the window
// ends stay loops).
template <bool FWD, int W = 32>
__device__ __forceinline__ void tab_receivers(const float* Mv, const float* Pv, const float* SVv, const float* SVMv,
                                              const float* rho, int n, int lane, const TabRow& K, int* X, float* D,
                                              float nphi) {
    int w0, w1;
    tab_chunk<W>(n, lane, w0, w1);
    if (w0 >= w1) return;
    const float Rl = K.R[TAB_NR - 1];
    // window ends with R_j >= M_{n-1} - M_0 stay at 0 for every receiver
    const float span = Mv[n - 1] - Mv[0];
    int ja = 0;
    while (ja < TAB_NB && K.R[ja] < span) ++ja;
    const int jm = min(ja, TAB_NB - 1);  // moving middle window ends: j < jm
    // closed form of the fixed middle ends j in [jm, nr-3]
    const float sgf = K.SG[jm] - K.SG[TAB_NB - 1], sgrf = K.SGR[jm] - K.SGR[TAB_NB - 1];
    {   // the chunk's first receiver: binary searches (x_j <= x_{j-1})
        const float Pw = Pv[w0];
        int hi = w0;
        for (int j = 0; j < ja; j++) {
            const float t = Pw - K.R[j];
            int lo = 0, h = hi;
            while (lo < h) {
                const int mid = (lo + h) >> 1;
                if (Mv[mid] >= t) h = mid;
                else lo = mid + 1;
            }
            X[32 * j] = lo;
            hi = lo;
        }
        for (int j = ja; j < TAB_NB; j++) X[32 * j] = 0;
    }
    for (int w = w0; w < w1; w++) {
        const float Pw = Pv[w];
        // the last window end (radius R_{nr-2}) decides the last included source s
        int xs = X[32 * (TAB_NB - 1)];
        if (TAB_NB - 1 < ja) {
            const float t = Pw - K.R[TAB_NB - 1];
            while (xs < w && Mv[xs] < t) ++xs;
            X[32 * (TAB_NB - 1)] = xs;
        }
        const bool back = xs >= 1 && Pw - Mv[xs - 1] <= Rl;
        const int s = back ? xs - 1 : xs;
        const int clip = s + 1;  // window ends are clipped below at s + 1
        float tot = 0.f;
        int seg = 0;
#pragma unroll 1
        for (int j = 0; j < jm; j++) {
            const float t = Pw - K.R[j];
            int xx = X[32 * j];
            while (xx < w && Mv[xx] < t) ++xx;
            X[32 * j] = xx;
            if (s < w) {
                seg += xx > s ? 1 : 0;
                const int lo = max(xx, clip);
                tot = fmaf(K.G[j + 1], fmaf(t, SVv[lo], -SVMv[lo]), tot);
            }
        }
        if (s < w) {
            const float svc = SVv[clip], svmc = SVMv[clip];
            tot += fmaf(svc, fmaf(Pw, sgf, -sgrf), -svmc * sgf);  // fixed middle ends
            tot = fmaf(K.B[0], fmaf(Pw, SVv[w], -SVMv[w]), tot);   // top end w
            {   // the lowest window's lower end
                seg += xs > s ? 1 : 0;
                const int lo = max(xs, clip);
                const float coef = fmaf(K.B[TAB_NB - 1], Pw - K.Rm[TAB_NB - 1], K.Km[TAB_NB - 1]);
                tot = fmaf(K.B[TAB_NB - 1], SVMv[lo], fmaf(-coef, SVv[lo], tot));
            }
            const int sg = back ? TAB_NR - 1 : seg;  // segment of c_s
            tot = fmaf(svc, fmaf(K.B[sg], (Pw - Mv[s]) - K.Rm[sg], K.Km[sg]), tot);
        }
        const int i = wmap<FWD>(w, n);
        if (FWD) D[i] = tot;
        else D[i] = rho[i] >= 0.f ? __fdiv_rn(D[i] + tot, nphi) : 0.f;
    }
}

// P_w, Sg_w, SgP_w (w = 0..n, P_n = +inf: pointer stop) and M_w in walk order.
template <bool FWD, int W = 32>
__device__ __forceinline__ void tab_build_T(const float* rho, const float* g, int n, int lane, float delr, float* Pv,
                                            float* Sgv, float* SgPv, float* Mv) {
    int w0, w1;
    tab_chunk<W>(n, lane, w0, w1);
    float sd = 0.f, sg = 0.f, sgp = 0.f;
    for (int w = w0; w < w1; w++) {
        const int i = wmap<FWD>(w, n);
        const float r = rho[i], gi = g[i];
        sgp = fmaf(gi, sd, sgp);
        sg += gi;
        sd += r >= 0.f ? delr * r : 0.f;
    }
    float Pw = warp_excl_scan<W>(sd, lane);
    float Sg = warp_excl_scan<W>(sg, lane);
    float SgP = warp_excl_scan<W>(fmaf(Pw, sg, sgp), lane);
    for (int w = w0; w < w1; w++) {
        const int i = wmap<FWD>(w, n);
        const float r = rho[i], gi = g[i];
        const float d = r >= 0.f ? delr * r : 0.f;
        Pv[w] = Pw;
        Sgv[w] = Sg;
        SgPv[w] = SgP;
        Mv[w] = fmaf(0.5f, d, Pw);
        SgP = fmaf(gi, Pw, SgP);
        Sg += gi;
        Pw += d;
    }
    if (w1 == n && w0 < w1) {
        Pv[n] = __int_as_float(0x7f800000);
        Sgv[n] = Sg;
        SgPv[n] = SgP;
    }
}

// Sources of one walk direction: W[k] = Phi_{b_k}(M_k), U[k] = Phi_{b_{k-1}}(M_k),
// with the window ends y_j (Y[32 j], shared memory) clipped above at cap + 1
// for each cap.
template <bool FWD, int W = 32>
__device__ __forceinline__ void tab_sources(const float* Pv, const float* Sgv, const float* SgPv, const float* Mv,
                                            int n, int lane, const TabRow& K, int* Y, float* Wk, float* Uk) {
    int w0, w1;
    tab_chunk<W>(n, lane, w0, w1);
    if (w0 >= w1) return;
    const float Rl = K.R[TAB_NR - 1], Rl2 = K.R[TAB_NR - 2];
    // window ends with R_j >= P_{n-1} - M_0 stay at n for every source
    const float span = Pv[n - 1] - Mv[0];
    int ja = 0;
    while (ja < TAB_NR && K.R[ja] < span) ++ja;
    const int jm = min(ja, TAB_NR - 1);  // moving middle window ends: j < jm
    auto lim_of = [&](int k) {
        float l = Mv[k] + Rl;
        if (k + 1 < n) l = fminf(l, Mv[k + 1] + Rl2);
        return l;
    };
    // the first receiver i in [lo, n] with P_i > v (P_n = +inf)
    auto ub = [&](float v, int lo) {
        int h = n;
        while (lo < h) {
            const int mid = (lo + h) >> 1;
            if (Pv[mid] > v) h = mid;
            else lo = mid + 1;
        }
        return lo;
    };
    {   // the chunk's first source: binary searches (y_j >= y_{j-1})
        const float m = Mv[w0];
        int lo = min(w0 + 1, n);
        for (int j = 0; j < ja; j++) {
            lo = ub(m + K.R[j], lo);
            Y[32 * j] = lo;
        }
        for (int j = ja; j < TAB_NR; j++) Y[32 * j] = n;
    }
    int ylim = ub(lim_of(w0), min(w0 + 1, n));
    int capU = w0 >= 1 ? min(max(ub(lim_of(w0 - 1), w0) - 1, w0), n - 1) : w0;  // b_{w0-1}
    for (int k = w0; k < w1; k++) {
        const float m = Mv[k];
        {
            const float l = lim_of(k);
            while (Pv[ylim] <= l) ++ylim;
        }
        const int capW = min(max(ylim - 1, k + 1), n - 1);  // b_k
        float W = 0.f, U = 0.f;
        if (k + 1 < n) {
            const float sW = Sgv[capW + 1], sWp = SgPv[capW + 1], sU = Sgv[capU + 1], sUp = SgPv[capU + 1];
            // bottom end k + 1: beta_0 (m Sg - SgP)
            W = K.B[0] * fmaf(m, Sgv[k + 1], -SgPv[k + 1]);
            U = W;
#pragma unroll 1
            for (int j = 0; j < jm; j++) {
                const float t = m + K.R[j];
                int yy = Y[32 * j];
                while (Pv[yy] <= t) ++yy;
                Y[32 * j] = yy;
                const float a = Sgv[yy], ap = SgPv[yy];
                const bool inW = yy <= capW + 1, inU = yy <= capU + 1;
                W = fmaf(K.G[j + 1], fmaf(t, inW ? a : sW, -(inW ? ap : sWp)), W);
                U = fmaf(K.G[j + 1], fmaf(t, inU ? a : sU, -(inU ? ap : sUp)), U);
            }
            // fixed middle ends j in [jm, nr-2] sit at n: past both caps
            const float sg = K.SG[jm], sgr = K.SGR[jm];
            W += fmaf(sW, fmaf(m, sg, sgr), -sWp * sg);
            U += fmaf(sU, fmaf(m, sg, sgr), -sUp * sg);
            {   // top end (radius R_{nr-1}): coef'_{nr-1} Sg + beta_{nr-1} SgP
                const int j = TAB_NR - 1;
                int yy = Y[32 * j];
                if (j < ja) {
                    while (Pv[yy] <= m + K.R[j]) ++yy;
                    Y[32 * j] = yy;
                }
                const float coef = K.Km[j] - K.B[j] * (m + K.Rm[j]);
                const bool inW = yy <= capW + 1, inU = yy <= capU + 1;
                W = fmaf(coef, inW ? Sgv[yy] : sW, fmaf(K.B[j], inW ? SgPv[yy] : sWp, W));
                U = fmaf(coef, inU ? Sgv[yy] : sU, fmaf(K.B[j], inU ? SgPv[yy] : sUp, U));
            }
        }
        Wk[k] = W;
        Uk[k] = U;
        capU = capW;
    }
}

// Exact-table cone kernel (mode EE_KERNEL_TABLE, nr = 24): REV resample of a
// line into shared memory, then the two walk directions.
constexpr int TAB_WARPS = 4;

__host__ __device__ constexpr int tab_lp(int maxL) { return ((maxL + 3) & ~3) + 4; }
__host__ __device__ constexpr int tab_fwd_stride(int maxL) { return 7 * tab_lp(maxL) + 32 * TAB_NB; }
__host__ __device__ constexpr int tab_adj_stride(int maxL) { return 9 * tab_lp(maxL) + 32 * TAB_NR; }

// One line of k_cone_tab on the W lanes of its group (`lane` counts within
// the group; W = 32: the whole warp, W = 16: half of it), with the group's
// arrays at `arr`.  line < 0 or n <= 0: nothing to write, but the group still
// takes part in the scans, which all 32 lanes execute.
template <int W>
__device__ __forceinline__ void tab_fwd_line(const EeParams& P, const EeBeamSpec& S, const EeBeamGeom& G,
                                             const EeRayGeom& R, const float* __restrict__ terma_b,
                                             float* __restrict__ rev_beam, int line, int i0, int n, int lane,
                                             float* arr, int Lp, const float* tab, int* X) {
    float* Mv = arr;
    float* Pv = Mv + Lp;
    float* SVv = Pv + Lp;
    float* SVMv = SVv + Lp;
    float* rho = SVMv + Lp;
    float* T = rho + Lp;
    float* D = T + Lp;
    float* out = nullptr;
    int nn = 0;
    if (line >= 0) {
        const int L = R.rev[0];
        const int tY = line % R.rev[1], tZ = line / R.rev[1];
        const Brick Bv = rev_brick(R.rev[0], R.rev[1], R.rev[2]);
        out = rev_beam + R.offset + rev_line(Bv, tY, tZ);
        int z0, z1;
        line_read_span(G, R, tY, tZ, L, z0, z1);
        zero_outside_segment(out, Bv, z0, z1, i0, n, lane, W);
        if (n > 0) {
            gather_line(P, S, G, R, terma_b, tY, tZ, i0, n, lane, rho, T, W);
            nn = n;
        }
    }
    __syncwarp();
    const float nphi = (float)P.nphi;
    tab_build<true, W>(rho, T, nn, lane, P.lng, Mv, Pv, SVv, SVMv);
    __syncwarp();
    tab_receivers<true, W>(Mv, Pv, SVv, SVMv, rho, nn, lane, tab_row(tab, true), X, D, nphi);
    __syncwarp();
    tab_build<false, W>(rho, T, nn, lane, P.lng, Mv, Pv, SVv, SVMv);
    __syncwarp();
    tab_receivers<false, W>(Mv, Pv, SVv, SVMv, rho, nn, lane, tab_row(tab, false), X, D, nphi);
    __syncwarp();
    for (int k = lane; k < nn; k += W) out[bk_x(i0 + k)] = D[k];
}

// A warp takes two neighbouring lines.  When both fit half of its arrays
// (n below Lp / 2 - 1), each half-warp runs one of them, 16 lanes per line;
// else the whole warp runs one after the other.  A lane's first receiver costs a
// binary search per window end, so a lane that runs one chunk of a line
// instead of two shorter chunks of two lines saves one set of searches, and
// short lines keep more lanes busy.
__global__ void __launch_bounds__(TAB_WARPS * 32) k_cone_tab(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                             const EeBeamGeom* __restrict__ geoms,
                                                             const float* __restrict__ terma, float* __restrict__ rev,
                                                             int maxL) {
    extern __shared__ float4 sm4[];
    float* sm = reinterpret_cast<float*>(sm4);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ray = blockIdx.y, b = blockIdx.z;
    const int Lp = tab_lp(maxL);
    float* tab = sm + (size_t)TAB_WARPS * tab_fwd_stride(maxL);
    const EeRayConst& RC = P.rays[ray];
    tab_tables(P, RC, tab);
    __syncthreads();
    const EeBeamGeom& G = geoms[b];
    if (G.status != 0) return;
    const EeRayGeom& R = G.ray[ray];
    const int la = 2 * (blockIdx.x * TAB_WARPS + warp);
    if (la >= R.nlines) return;
    const int lb = la + 1 < R.nlines ? la + 1 : -1;
    const int L = R.rev[0];
    int i0a, na, i0b = 0, nb = 0;
    line_segment(P, G, R, la % R.rev[1], la / R.rev[1], L, i0a, na);
    if (lb >= 0) line_segment(P, G, R, lb % R.rev[1], lb / R.rev[1], L, i0b, nb);
    float* arr = sm + (size_t)warp * tab_fwd_stride(maxL);
    int* X = reinterpret_cast<int*>(arr + 7 * Lp) + lane;
    const EeBeamSpec& S = specs[b];
    const float* terma_b = terma + S.t_off;
    float* rev_beam = rev + G.arena_off;
    // the second half-warp's arrays start one cell past the middle: an odd
    // offset puts the two halves' strided accesses on different banks
    const int half = Lp >> 1;
    if (max(na, nb) < half - 1) {
        const int sub = lane >> 4;
        tab_fwd_line<16>(P, S, G, R, terma_b, rev_beam, sub ? lb : la, sub ? i0b : i0a, sub ? nb : na, lane & 15,
                         arr + sub * (half + 1), Lp, tab, X);
    } else {
        tab_fwd_line<32>(P, S, G, R, terma_b, rev_beam, la, i0a, na, lane, arr, Lp, tab, X);
        if (lb >= 0) {
            __syncwarp();
            tab_fwd_line<32>(P, S, G, R, terma_b, rev_beam, lb, i0b, nb, lane, arr, Lp, tab, X);
        }
    }
}

// One line of k_cone_T_tab on the W lanes of its group (as tab_fwd_line).
template <int W>
__device__ __forceinline__ void tab_adj_line(const EeParams& P, const EeBeamSpec& S, const EeBeamGeom& G,
                                             const EeRayGeom& R, const float* __restrict__ grad_beam,
                                             float* __restrict__ terma_grad, int line, int i0, int n, int lane,
                                             float* arr, int Lp, const float* tab, int* Y) {
    float* Pv = arr;
    float* Sgv = Pv + Lp;
    float* SgPv = Sgv + Lp;
    float* Mv = SgPv + Lp;
    float* rho = Mv + Lp;
    float* g = rho + Lp;
    float* Tb = g + Lp;
    float* Wk = Tb + Lp;
    float* Uk = Wk + Lp;
    int nn = 0, tY = 0, tZ = 0;
    if (line >= 0 && n > 0) {
        tY = line % R.rev[1];
        tZ = line / R.rev[1];
        gather_line(P, S, G, R, nullptr, tY, tZ, i0, n, lane, rho, nullptr, W);
        nn = n;
    }
    __syncwarp();
    if (nn > 0) {
        const Brick Bv = rev_brick(R.rev[0], R.rev[1], R.rev[2]);
        const float* gin = grad_beam + R.offset + rev_line(Bv, tY, tZ);
        const float inv_nphi = 1.f / (float)P.nphi;
        for (int k = lane; k < nn; k += W) {
            g[k] = rho[k] >= 0.f ? gin[bk_x(i0 + k)] * inv_nphi : 0.f;
            Tb[k] = 0.f;
        }
    }
    __syncwarp();
#pragma unroll 1
    for (int dir = 0; dir < 2; dir++) {
        if (dir == 0) tab_build_T<true, W>(rho, g, nn, lane, P.lng, Pv, Sgv, SgPv, Mv);
        else tab_build_T<false, W>(rho, g, nn, lane, P.lng, Pv, Sgv, SgPv, Mv);
        __syncwarp();
        if (dir == 0) tab_sources<true, W>(Pv, Sgv, SgPv, Mv, nn, lane, tab_row(tab, true), Y, Wk, Uk);
        else tab_sources<false, W>(Pv, Sgv, SgPv, Mv, nn, lane, tab_row(tab, false), Y, Wk, Uk);
        __syncwarp();
        for (int w = lane; w < nn; w += W) {
            const float v = Wk[w] - (w + 1 < nn ? Uk[w + 1] : 0.f);
            Tb[dir == 0 ? w : nn - 1 - w] += v;
        }
        __syncwarp();
    }
    if (nn > 0) {
        // transpose of the REV TERMA resample
        const f3 gl = ld3(R.G0) + ld3(R.Gy) * (float)tY + ld3(R.Gz) * (float)tZ;
        const f3 gx = ld3(R.Gx);
        float* tg = terma_grad + S.t_off;
        for (int k = lane; k < nn; k += W) {
            const float v = Tb[k];
            if (rho[k] < 0.f || v == 0.f) continue;
            const f3 gp = gl + gx * (float)(i0 + k);
            tri_brick_scatter(tg, brick_of(S.tn), gp.x - (float)S.t0[0], gp.y - (float)S.t0[1],
                              gp.z - (float)S.t0[2], v);
        }
    }
}

// Its adjoint followed by the transpose of the REV TERMA resample; two lines
// per warp as k_cone_tab.
__global__ void __launch_bounds__(TAB_WARPS * 32) k_cone_T_tab(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                               const EeBeamGeom* __restrict__ geoms,
                                                               const float* __restrict__ rev_grad,
                                                               float* __restrict__ terma_grad, int maxL) {
    extern __shared__ float4 sm4[];
    float* sm = reinterpret_cast<float*>(sm4);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ray = blockIdx.y, b = blockIdx.z;
    const int Lp = tab_lp(maxL);
    float* tab = sm + (size_t)TAB_WARPS * tab_adj_stride(maxL);
    const EeRayConst& RC = P.rays[ray];
    tab_tables(P, RC, tab);
    __syncthreads();
    const EeBeamGeom& G = geoms[b];
    if (G.status != 0) return;
    const EeRayGeom& R = G.ray[ray];
    const int la = 2 * (blockIdx.x * TAB_WARPS + warp);
    if (la >= R.nlines) return;
    const int lb = la + 1 < R.nlines ? la + 1 : -1;
    const int L = R.rev[0];
    int i0a, na, i0b = 0, nb = 0;
    line_segment(P, G, R, la % R.rev[1], la / R.rev[1], L, i0a, na);
    if (lb >= 0) line_segment(P, G, R, lb % R.rev[1], lb / R.rev[1], L, i0b, nb);
    float* arr = sm + (size_t)warp * tab_adj_stride(maxL);
    int* Y = reinterpret_cast<int*>(arr + 9 * Lp) + lane;
    const EeBeamSpec& S = specs[b];
    const float* grad_beam = rev_grad + G.arena_off;
    const int half = Lp >> 1;  // second half-warp's arrays at an odd offset, as k_cone_tab
    if (max(na, nb) < half - 1) {
        const int sub = lane >> 4;
        tab_adj_line<16>(P, S, G, R, grad_beam, terma_grad, sub ? lb : la, sub ? i0b : i0a, sub ? nb : na,
                         lane & 15, arr + sub * (half + 1), Lp, tab, Y);
    } else {
        tab_adj_line<32>(P, S, G, R, grad_beam, terma_grad, la, i0a, na, lane, arr, Lp, tab, Y);
        if (lb >= 0) {
            __syncwarp();
            tab_adj_line<32>(P, S, G, R, grad_beam, terma_grad, lb, i0b, nb, lane, arr, Lp, tab, Y);
        }
    }
}

// ------------------------------------------- cone: one lane per line ----
// EE_KERNEL_EXP fast path.  Each thread owns one REV line (adjacent threads
// own adjacent lines, so their segments and gathers stay close): it computes
// its segment analytically and runs the recurrence sequentially, without
// shuffles or shared memory.  Forward pass (ascending i) stores D_fwd in the
// pre-zeroed REV arena; reverse pass (descending i) gathers the samples again,
// adds its part and applies 1/nphi.  Same operator as line_scan.
struct LineFrame {
    f3 bl, gl, bx, gx;
};

__device__ __forceinline__ LineFrame line_frame(const EeRayGeom& R, int tY, int tZ) {
    LineFrame F;
    F.bl = ld3(R.B0) + ld3(R.By) * (float)tY + ld3(R.Bz) * (float)tZ;
    F.gl = ld3(R.G0) + ld3(R.Gy) * (float)tY + ld3(R.Gz) * (float)tZ;
    F.bx = ld3(R.Bx);
    F.gx = ld3(R.Gx);
    return F;
}

// One REV sample (device.cu:47-79): returns rho (sentinel < 0 outside) and,
// when terma_b != nullptr, the TERMA sample.
__device__ __forceinline__ float sample_rho(const EeParams& P, const EeBeamSpec& S, const EeBeamGeom& G,
                                            const LineFrame& F, int i, const float* __restrict__ terma_b, float& t) {
    const float fi = (float)i;
    f3 bev = F.bl + F.bx * fi;
    t = 0.f;
    if (bev.x < 0.f || bev.y < 0.f || bev.z < 0.f || bev.x >= (float)G.bev[0] || bev.y >= (float)G.bev[1] ||
        bev.z >= (float)G.bev[2])
        return -3.f;
    f3 g = F.gl + F.gx * fi;
    if (g.x < (float)P.bb0[0] || g.x >= (float)(P.bb0[0] + P.bbs[0]) || g.y < (float)P.bb0[1] ||
        g.y >= (float)(P.bb0[1] + P.bbs[1]) || g.z < (float)P.bb0[2] || g.z >= (float)(P.bb0[2] + P.bbs[2]))
        return -2.f;
    if (terma_b)
        t = tri_brick(terma_b, brick_of(S.tn), g.x - (float)S.t0[0], g.y - (float)S.t0[1],
                       g.z - (float)S.t0[2]);
    return tex3D<float>(P.dens_tex, g.x + 0.5f, g.y + 0.5f, g.z + 0.5f);
}

// Sample indices [s0, s1] of a REV line whose TERMA trilinear corners can lie
// inside the beam's field frustum.  A voxel has a beamlet only where its
// iso-plane projection falls inside the fluence-map rectangle (beamlet_of,
// cudaSiddon.cu:143-165): with diff = p - src, proj = dir.diff and
// u = MB_row.(diff - proj dir), the fluence coordinate is inside iff
// u + k proj >= 0 and k proj - u > 0, k = half the map's width / isodist,
// per BEV axis x and z.  Outside, TERMA is exactly zero (k_terma writes 0
// where there is no beamlet) and the TERMA adjoint drops the voxel, so the
// cone kernels skip the TERMA reads and the TERMA-gradient scatter of the
// samples outside [s0, s1].  The four sides are linear in the sample index;
// a sample is outside when one side's form is below minus its change over
// two voxels per axis (the trilinear corners, and supersampled centres half
// a voxel beyond them).
__device__ __forceinline__ void field_span(const EeParams& P, const EeBeamSpec& S, const LineFrame& F, int i0, int n,
                                           int& s0, int& s1) {
    const f3 vox = mk(P.voxel[0], P.voxel[1], P.voxel[2]);
    const f3 d0 = mk(P.start[0] + vox.x * F.gl.x - S.src[0], P.start[1] + vox.y * F.gl.y - S.src[1],
                     P.start[2] + vox.z * F.gl.z - S.src[2]);  // diff at sample 0
    const f3 d1 = mk(vox.x * F.gx.x, vox.y * F.gx.y, vox.z * F.gx.z);  // diff step per sample
    const f3 dir = ld3(S.dir);
    // the forms hold in front of the source (proj > 0); beamlet_of mirrors
    // points behind it, so a segment that does not stay well in front of
    // the source (proj linear in i: its ends decide) is not restricted
    const float pa = dot(dir, d0) + dot(dir, d1) * (float)i0, pb = dot(dir, d0) + dot(dir, d1) * (float)(i0 + n - 1);
    if (!(fminf(pa, pb) > 1e-2f * S.isodist)) {
        s0 = -0x3fffffff;
        s1 = 0x3fffffff;
        return;
    }
    float lo = -1e9f, hi = 1e9f;
#pragma unroll
    for (int a = 0; a < 2; a++) {
        const f3 m = ld3(S.MB + (a ? 6 : 0));
        const f3 g = m - dir * dot(m, dir);  // u = g . diff
        const float k = 0.5f * (float)S.fmap[a] * S.beamlet[a] / S.isodist;
#pragma unroll
        for (int sg = -1; sg <= 1; sg += 2) {
            const f3 gl = g * (float)sg + dir * k;  // the side's form: gl . diff >= 0 inside
            const float M = 2.f * (fabsf(gl.x) * vox.x + fabsf(gl.y) * vox.y + fabsf(gl.z) * vox.z) + 1e-3f;
            const float al = dot(gl, d1), be = dot(gl, d0) + M;  // maybe inside where al i + be >= 0
            if (fabsf(al) < 1e-20f) {
                if (be < 0.f) { lo = 1e9f; hi = -1e9f; }
            } else {
                const float t = fminf(fmaxf(-be / al, -1e9f), 1e9f);
                if (al > 0.f) lo = fmaxf(lo, t);
                else hi = fminf(hi, t);
            }
        }
    }
    s0 = (int)floorf(lo) - 1;
    s1 = (int)ceilf(hi) + 1;
}

// Lane slot -> REV line for the one-lane-per-line kernels: the lanes of a
// warp own an 8 (tY) x 4 (tZ) tile of lines, so at every sample index the
// warp's reads and writes of the bricked REV arrays fall in two 64-byte brick
// slabs.  False for slots of a tile that lie outside the cone's array.
__device__ __forceinline__ bool lane_line(const EeRayGeom& R, int slot, int& tY, int& tZ) {
    const int wt = slot >> 5, l = slot & 31;
    const int nty = (R.rev[1] + 7) >> 3;
    tY = (wt % nty) * 8 + (l & 7);
    tZ = (wt / nty) * 4 + (l >> 3);
    return tY < R.rev[1] && tZ < R.rev[2];
}

template <int LANE_BLOCK>
__global__ void __launch_bounds__(LANE_BLOCK) k_cone_lane(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                          const EeBeamGeom* __restrict__ geoms,
                                                          const float* __restrict__ terma, float* __restrict__ rev,
                                                          float2* __restrict__ samples) {
    const int ray = blockIdx.y, b = blockIdx.z;
    const EeBeamGeom& G = geoms[b];
    if (G.status != 0) return;
    const EeRayGeom& R = G.ray[ray];
    int tY, tZ;
    if (!lane_line(R, blockIdx.x * LANE_BLOCK + threadIdx.x, tY, tZ)) return;
    const int L = R.rev[0];
    // bricked REV arena (rev_brick): this line's sample i sits at out + bk_x(i)
    const Brick Bv = rev_brick(R.rev[0], R.rev[1], R.rev[2]);
    float* out = rev + G.arena_off + R.offset + rev_line(Bv, tY, tZ);
    int i0, n, z0, z1;
    line_segment(P, G, R, tY, tZ, L, i0, n);
    line_read_span(G, R, tY, tZ, L, z0, z1);
    zero_outside_segment(out, Bv, z0, z1, i0, n, 0, 1);
    if (n <= 0) return;
    const EeBeamSpec& S = specs[b];
    const float* tb = terma + S.t_off;
    const LineFrame F = line_frame(R, tY, tZ);
    int f0, f1;  // samples that can see TERMA
    field_span(P, S, F, i0, n, f0, f1);
    // (rho, T) of each sample, kept from the forward pass for the reverse
    // one, in this cone's slot of the scratch bricked like the REV arena.
    // Both passes walk whole quads of samples (4q .. 4q+3): a lane reads and
    // writes a quad's dose and (rho, T) with 16-byte accesses, and the warp's
    // 8 x 4 lines cover two whole bricks.  Samples of an end quad outside the
    // segment get dose 0 (they are inside the read span or never read) and
    // scratch (-1, 0).
    float2* smp = samples + G.arena_off + R.offset + rev_line(Bv, tY, tZ);
    const EeRayConst& RC = P.rays[ray];
    const float delr = P.lng;
    const int iend = i0 + n;
    {   // forward direction: contributions from k < i, kernel row P
        const float* prm = P.expp + 4 * RC.row_fwd;
        const float c1 = prm[0] / prm[1], c2 = prm[2] / prm[3];
        const float e1 = -0.5f * prm[1] * delr, e2 = -0.5f * prm[3] * delr;
        float Y1 = 0.f, Y2 = 0.f, tm = 0.f, hm1 = 1.f, hm2 = 1.f;
        for (int ib = i0 & ~3; ib < iend; ib += 4) {
            // the quad's samples gathered before the recurrence consumes
            // them, so each lane keeps several independent loads in flight
            float rr[4], tt[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int i = ib + j;
                rr[j] = -1.f;
                tt[j] = 0.f;
                if (i >= i0 && i < iend) rr[j] = sample_rho(P, S, G, F, i, (i >= f0 && i <= f1) ? tb : nullptr, tt[j]);
            }
            float dq[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int i = ib + j;
                dq[j] = 0.f;
                if (i < i0 || i >= iend) continue;
                const float r = rr[j];
                const bool v = r >= 0.f;
                const float h1 = v ? __expf(e1 * r) : 1.f, h2 = v ? __expf(e2 * r) : 1.f;
                const float t = v ? tt[j] : 0.f;
                rr[j] = r;
                tt[j] = t;
                dq[j] = v ? c1 * (Y1 + tm * (1.f - hm1)) + c2 * (Y2 + tm * (1.f - hm2)) : 0.f;
                Y1 = fmaf(h1 * h1, Y1, tm * h1 * (1.f - hm1 * h1));
                Y2 = fmaf(h2 * h2, Y2, tm * h2 * (1.f - hm2 * h2));
                tm = t; hm1 = h1; hm2 = h2;
            }
            float4* sq = reinterpret_cast<float4*>(smp + bk_x(ib));
            sq[0] = make_float4(rr[0], tt[0], rr[1], tt[1]);
            sq[1] = make_float4(rr[2], tt[2], rr[3], tt[3]);
            *reinterpret_cast<float4*>(out + bk_x(ib)) = make_float4(dq[0], dq[1], dq[2], dq[3]);
        }
    }
    {   // reverse direction: contributions from k > i, kernel row ntheta-1-P
        const float* prm = P.expp + 4 * RC.row_rev;
        const float c1 = prm[0] / prm[1], c2 = prm[2] / prm[3];
        const float e1 = -0.5f * prm[1] * delr, e2 = -0.5f * prm[3] * delr;
        const float inv_nphi = 1.f / (float)P.nphi;
        float Y1 = 0.f, Y2 = 0.f, tm = 0.f, hm1 = 1.f, hm2 = 1.f;
        for (int ib = (iend - 1) & ~3; ib >= (i0 & ~3); ib -= 4) {
            const float4* sq = reinterpret_cast<const float4*>(smp + bk_x(ib));
            const float4 s01 = sq[0], s23 = sq[1];
            const float4 o4 = *reinterpret_cast<const float4*>(out + bk_x(ib));
            const float rs[4] = {s01.x, s01.z, s23.x, s23.z}, ts[4] = {s01.y, s01.w, s23.y, s23.w};
            const float ov[4] = {o4.x, o4.y, o4.z, o4.w};
            float dq[4];
#pragma unroll
            for (int j = 3; j >= 0; j--) {
                const int i = ib + j;
                dq[j] = 0.f;
                if (i < i0 || i >= iend) continue;
                const float r = rs[j];
                const bool v = r >= 0.f;
                const float t = v ? ts[j] : 0.f;
                const float h1 = v ? __expf(e1 * r) : 1.f, h2 = v ? __expf(e2 * r) : 1.f;
                const float d = c1 * (Y1 + tm * (1.f - hm1)) + c2 * (Y2 + tm * (1.f - hm2));
                dq[j] = v ? (ov[j] + d) * inv_nphi : 0.f;
                Y1 = fmaf(h1 * h1, Y1, tm * h1 * (1.f - hm1 * h1));
                Y2 = fmaf(h2 * h2, Y2, tm * h2 * (1.f - hm2 * h2));
                tm = t; hm1 = h1; hm2 = h2;
            }
            *reinterpret_cast<float4*>(out + bk_x(ib)) = make_float4(dq[0], dq[1], dq[2], dq[3]);
        }
    }
}

// Zero the segment (line_segment) of every line of a chunk's REV gradient
// arena before k_gather_T adds into it: the samples the adjoint cone reads.
// k_gather_T also adds into the rest of the line's read span; those cells are
// never read, so they need no zero.  A lane zeroes the quads of samples that
// hold its segment with 16-byte stores (the end quads' other samples are
// never read either); a warp's store covers two whole bricks.
template <int LANE_BLOCK>
__global__ void __launch_bounds__(LANE_BLOCK) k_rev_zero(EeParams P, const EeBeamGeom* __restrict__ geoms,
                                                         float* __restrict__ rev_grad) {
    const int ray = blockIdx.y, b = blockIdx.z;
    const EeBeamGeom& G = geoms[b];
    if (G.status != 0) return;
    const EeRayGeom& R = G.ray[ray];
    int tY, tZ;
    if (!lane_line(R, blockIdx.x * LANE_BLOCK + threadIdx.x, tY, tZ)) return;
    int i0, n;
    line_segment(P, G, R, tY, tZ, R.rev[0], i0, n);
    const Brick Bv = rev_brick(R.rev[0], R.rev[1], R.rev[2]);
    float* row = rev_grad + G.arena_off + R.offset + rev_line(Bv, tY, tZ);
    for (int ib = i0 & ~3; ib < i0 + n; ib += 4)
        *reinterpret_cast<float4*>(row + bk_x(ib)) = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Adjoint of k_cone_lane followed by the transpose of the REV TERMA resample.
// Pass A (descending i) runs the transpose of the forward recurrence and
// stores its contribution to Tbar[i-1] in `scratch` (the REV-arena layout);
// pass B (ascending i) runs the transpose of the reverse recurrence, adds its
// contribution to Tbar[i] and scatters Tbar[i] into the TERMA-box gradient.
template <int LANE_BLOCK>
__global__ void __launch_bounds__(LANE_BLOCK) k_cone_T_lane(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                            const EeBeamGeom* __restrict__ geoms,
                                                            const float* __restrict__ rev_grad,
                                                            float2* __restrict__ scratch, float* __restrict__ terma_grad) {
    const int ray = blockIdx.y, b = blockIdx.z;
    const EeBeamGeom& G = geoms[b];
    if (G.status != 0) return;
    const EeRayGeom& R = G.ray[ray];
    int tY, tZ;
    if (!lane_line(R, blockIdx.x * LANE_BLOCK + threadIdx.x, tY, tZ)) return;
    const int L = R.rev[0];
    int i0, n;
    line_segment(P, G, R, tY, tZ, L, i0, n);
    if (n <= 0) return;
    const EeBeamSpec& S = specs[b];
    const LineFrame F = line_frame(R, tY, tZ);
    int f0, f1;  // samples whose TERMA corners can lie in the field (field_span)
    field_span(P, S, F, i0, n, f0, f1);
    // REV gradient and scratch bricked like the REV arena (rev_brick): sample
    // i at gin + bk_x(i) and sA + bk_x(i).  Both passes walk whole quads of
    // samples with 16-byte loads and stores, as k_cone_lane does.
    const Brick Bv = rev_brick(R.rev[0], R.rev[1], R.rev[2]);
    const float* gin = rev_grad + G.arena_off + R.offset + rev_line(Bv, tY, tZ);
    float2* sA = scratch + G.arena_off + R.offset + rev_line(Bv, tY, tZ);  // (pass-A part of Tbar[i], rho[i])
    const EeRayConst& RC = P.rays[ray];
    const float delr = P.lng, inv_nphi = 1.f / (float)P.nphi;
    const int i1 = i0 + n - 1;
    float dummy;
    {   // pass A: transpose of the forward recurrence, walking down; step i
        // writes the entry of sample i - 1, so a quad's top entry comes from
        // the quad above (carry) and the top sample's entry is (0, rho[i1])
        const float* prm = P.expp + 4 * RC.row_fwd;
        const float c1 = prm[0] / prm[1], c2 = prm[2] / prm[3];
        const float e1 = -0.5f * prm[1] * delr, e2 = -0.5f * prm[3] * delr;
        float r = sample_rho(P, S, G, F, i1, nullptr, dummy);
        bool v = r >= 0.f;
        float h1 = v ? __expf(e1 * r) : 1.f, h2 = v ? __expf(e2 * r) : 1.f;
        float Z1 = 0.f, Z2 = 0.f;
        float2 carry = make_float2(0.f, r);
        for (int qb = i1 & ~3; qb >= (i0 & ~3); qb -= 4) {
            const float4 g4 = *reinterpret_cast<const float4*>(gin + bk_x(qb));
            const float gl[4] = {g4.x, g4.y, g4.z, g4.w};
            float rl[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int i = qb + j;
                rl[j] = -1.f;
                if (i > i0 && i <= i1) rl[j] = sample_rho(P, S, G, F, i - 1, nullptr, dummy);
            }
            float2 o[4];
            const int cs = min(3, i1 - qb);  // slot of the carried entry
#pragma unroll
            for (int j = 0; j < 4; j++) o[j] = j == cs ? carry : make_float2(0.f, -1.f);
#pragma unroll
            for (int j = 3; j >= 0; j--) {
                const int i = qb + j;
                if (i > i1 || i <= i0) continue;
                const float gi = v ? gl[j] * inv_nphi : 0.f;
                const float rm = rl[j];
                const bool vm = rm >= 0.f;
                const float hm1 = vm ? __expf(e1 * rm) : 1.f, hm2 = vm ? __expf(e2 * rm) : 1.f;
                const float2 e = make_float2(vm ? c1 * gi * (1.f - hm1) + Z1 * h1 * (1.f - hm1 * h1) +
                                                      c2 * gi * (1.f - hm2) + Z2 * h2 * (1.f - hm2 * h2)
                                                : 0.f,
                                             rm);
                if (j > 0) o[j - 1] = e;
                else carry = e;
                Z1 = fmaf(h1 * h1, Z1, c1 * gi);
                Z2 = fmaf(h2 * h2, Z2, c2 * gi);
                v = vm; h1 = hm1; h2 = hm2;
            }
            float4* sq = reinterpret_cast<float4*>(sA + bk_x(qb));
            sq[0] = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
            sq[1] = make_float4(o[2].x, o[2].y, o[3].x, o[3].y);
        }
    }
    {   // pass B: transpose of the reverse recurrence, walking up; scatter
        const float* prm = P.expp + 4 * RC.row_rev;
        const float c1 = prm[0] / prm[1], c2 = prm[2] / prm[3];
        const float e1 = -0.5f * prm[1] * delr, e2 = -0.5f * prm[3] * delr;
        float* tg = terma_grad + S.t_off;
        const float r = sA[bk_x(i0)].y;
        bool v = r >= 0.f;
        float h1 = v ? __expf(e1 * r) : 1.f, h2 = v ? __expf(e2 * r) : 1.f;
        float Z1 = 0.f, Z2 = 0.f, cprev = 0.f;
        for (int qb = i0 & ~3; qb <= i1; qb += 4) {
            const float4* sq = reinterpret_cast<const float4*>(sA + bk_x(qb));
            const float4 s01 = sq[0], s23 = sq[1];
            // the first entry of the next quad, for the step at qb + 3
            const float4 nx = qb + 4 <= i1 ? *reinterpret_cast<const float4*>(sA + bk_x(qb + 4))
                                            : make_float4(0.f, -1.f, 0.f, -1.f);
            const float4 g4 = *reinterpret_cast<const float4*>(gin + bk_x(qb));
            const float2 al[5] = {make_float2(s01.x, s01.y), make_float2(s01.z, s01.w), make_float2(s23.x, s23.y),
                                  make_float2(s23.z, s23.w), make_float2(nx.x, nx.y)};
            const float gl[4] = {g4.x, g4.y, g4.z, g4.w};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int i = qb + j;
                if (i < i0 || i > i1) continue;
                const float gi = v ? gl[j] * inv_nphi : 0.f;
                const float tot = al[j].x + cprev;
                if (v && tot != 0.f && i >= f0 && i <= f1) {
                    f3 gp = F.gl + F.gx * (float)i;
                    tri_brick_scatter(tg, brick_of(S.tn), gp.x - (float)S.t0[0], gp.y - (float)S.t0[1],
                                       gp.z - (float)S.t0[2], tot);
                }
                if (i < i1) {
                    const float rm = al[j + 1].y;
                    const bool vm = rm >= 0.f;
                    const float hm1 = vm ? __expf(e1 * rm) : 1.f, hm2 = vm ? __expf(e2 * rm) : 1.f;
                    cprev = vm ? c1 * gi * (1.f - hm1) + Z1 * h1 * (1.f - hm1 * h1) + c2 * gi * (1.f - hm2) +
                                     Z2 * h2 * (1.f - hm2 * h2)
                               : 0.f;
                    Z1 = fmaf(h1 * h1, Z1, c1 * gi);
                    Z2 = fmaf(h2 * h2, Z2, c2 * gi);
                    v = vm; h1 = hm1; h2 = hm2;
                }
            }
        }
    }
}

// Adjoint of k_cone followed by the transpose of the REV TERMA resample:
// terma_grad (bbox grid) += R_T^T C^T rev_grad.
__global__ void __launch_bounds__(CONE_WARPS * 32) k_cone_T(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                            const EeBeamGeom* __restrict__ geoms,
                                                            const float* __restrict__ rev_grad,
                                                            float* __restrict__ terma_grad, int maxL) {
    extern __shared__ float sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ray = blockIdx.y, b = blockIdx.z;
    const EeBeamGeom& G = geoms[b];
    float* tabK = sm + (size_t)CONE_WARPS * 3 * maxL;
    float* tabR = tabK + 2 * EE_MAX_RADII;
    if (P.mode != EE_KERNEL_EXP) {
        const EeRayConst& RC = P.rays[ray];
        for (int k = threadIdx.x; k < P.nradii; k += blockDim.x) {
            tabK[k] = P.cumkern[RC.row_fwd * P.nradii + k];
            tabK[EE_MAX_RADII + k] = P.cumkern[RC.row_rev * P.nradii + k];
            tabR[k] = P.radii[k];
        }
        __syncthreads();
    }
    if (G.status != 0) return;
    const EeRayGeom& R = G.ray[ray];
    const int line = blockIdx.x * CONE_WARPS + warp;
    if (line >= R.nlines) return;
    const int L = R.rev[0];
    const int tY = line % R.rev[1], tZ = line / R.rev[1];
    float* rho = sm + (size_t)warp * 3 * maxL;
    float* g = rho + maxL;
    float* Tb = g + maxL;
    const EeBeamSpec& S = specs[b];
    int i0, n;
    line_segment(P, G, R, tY, tZ, L, i0, n);
    if (n == 0) return;
    gather_line(P, S, G, R, nullptr, tY, tZ, i0, n, lane, rho, nullptr);
    const Brick Bv = rev_brick(R.rev[0], R.rev[1], R.rev[2]);  // bricked REV gradient
    const float* gin = rev_grad + G.arena_off + R.offset + rev_line(Bv, tY, tZ);
    const float inv_nphi = 1.f / (float)P.nphi;
    __syncwarp();
    for (int k = lane; k < n; k += 32) {
        g[k] = rho[k] >= 0.f ? gin[bk_x(i0 + k)] * inv_nphi : 0.f;
        Tb[k] = 0.f;
    }
    __syncwarp();
    const EeRayConst& RC = P.rays[ray];
    if (P.mode == EE_KERNEL_EXP) {
        line_scan_T<true>(rho, g, n, lane, P.lng, P.expp + 4 * RC.row_fwd, Tb);
        __syncwarp();
        line_scan_T<false>(rho, g, n, lane, P.lng, P.expp + 4 * RC.row_rev, Tb);
    } else {
        for (int k = lane; k < n; k += 32) {
            if (rho[k] >= 0.f && g[k] != 0.f) {
                table_walk(rho, nullptr, n, k, -1, tabK, tabR, P.nradii, P.lng, Tb, g[k]);
                table_walk(rho, nullptr, n, k, +1, tabK + EE_MAX_RADII, tabR, P.nradii, P.lng, Tb, g[k]);
            }
        }
    }
    __syncwarp();
    // transpose of the REV TERMA resample
    const f3 gl = ld3(R.G0) + ld3(R.Gy) * (float)tY + ld3(R.Gz) * (float)tZ;
    const f3 gx = ld3(R.Gx);
    float* tg = terma_grad + S.t_off;
    for (int k = lane; k < n; k += 32) {
        float v = Tb[k];
        if (rho[k] < 0.f || v == 0.f) continue;
        f3 gp = gl + gx * (float)(i0 + k);
        tri_brick_scatter(tg, brick_of(S.tn), gp.x - (float)S.t0[0], gp.y - (float)S.t0[1],
                           gp.z - (float)S.t0[2], v);
    }
}

// ------------------------------------------------------------- gather ----
// Voxel range [x0, x1] of patient row (y, z) whose BEV index lies within the
// crop box dilated by 2 voxels (the BEV index is affine in x), widened by one
// voxel for rounding and clipped to the calc bbox.
__device__ __forceinline__ bool row_span(const EeParams& P, const EeBeamSpec& S, const EeBeamGeom& G, int y, int z,
                                         int& x0, int& x1) {
    float xa = (float)P.bb0[0], xb = (float)(P.bb0[0] + P.bbs[0] - 1);
    const float dy = (float)y - G.lim_off[1], dz = (float)z - G.lim_off[2];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float m = S.MB[3 * a];
        float c = S.MB[3 * a + 1] * dy + S.MB[3 * a + 2] * dz - m * G.lim_off[0];
        float lo = -2.f, hi = (float)G.bev[a] + 2.f;
        if (fabsf(m) < 1e-6f) {
            if (c < lo - 1e-3f || c > hi + 1e-3f) return false;
        } else {
            float t0 = (lo - c) / m, t1 = (hi - c) / m;
            xa = fmaxf(xa, fminf(t0, t1));
            xb = fminf(xb, fmaxf(t0, t1));
        }
    }
    if (!(xa <= xb + 2.f)) return false;
    x0 = max(P.bb0[0], (int)floorf(xa) - 1);
    x1 = min(P.bb0[0] + P.bbs[0] - 1, (int)ceilf(xb) + 1);
    return x0 <= x1;
}

constexpr int ROW_WARPS = 8;

// REV2XYZdose (device.cu:222-261) for all cones at once.  A warp takes a
// group of PY x PZ patient rows (EE_GATHER_*) of one beam's AABB and sweeps
// the union of their spans in PX x PY x PZ patches: a compact patch of voxels
// maps to a compact patch of REV cells, so a corner load of the warp touches
// fewer cache lines than a run of 32 voxels along x would.  A voxel sums the
// trilinear REV dose of every cone.  mode 0/1: atomic accumulation into dose;
// mode 2: dose[b] written directly.  Six resident blocks per SM: 40
// registers without spills, measured faster than 48.
__global__ void __launch_bounds__(ROW_WARPS * 32, 6) k_gather(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                           const EeBeamGeom* __restrict__ geoms,
                                                           const float* __restrict__ rev, float* __restrict__ dose,
                                                           int mode, long long nfull) {
    const int b = blockIdx.z;
    const EeBeamGeom& G = geoms[b];
    if (G.status != 0) return;
    // the beam's cone maps, staged once per block: rows of [A | -q0] (REV
    // from crop-box-relative patient index), (rev sizes, arena offset) and
    // the REV array's brick strides
    __shared__ float4 s_ray[EE_MAX_RAYS][5];
    for (int k = threadIdx.x; k < P.nrays * 5; k += blockDim.x) {
        const int r = k / 5, c = k - 5 * r;
        const EeRayGeom& R = G.ray[r];
        float4 v;
        if (c < 3) {
            v = make_float4(R.A[3 * c], R.A[3 * c + 1], R.A[3 * c + 2], -R.q0[c]);
        } else if (c == 4) {
            const Brick Bq = rev_brick(R.rev[0], R.rev[1], R.rev[2]);
            v = make_float4(__int_as_float(Bq.sy), __int_as_float(Bq.sz), 0.f, 0.f);
        } else {
            v = make_float4(__int_as_float(R.rev[0]), __int_as_float(R.rev[1]), __int_as_float(R.rev[2]),
                            __int_as_float((int)R.offset));
        }
        s_ray[r][c] = v;
    }
    __syncthreads();
    const int grp = blockIdx.x * ROW_WARPS + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (grp >= G.rows) return;
    constexpr int PX = EE_GATHER_PX, PY = EE_GATHER_PY;
    const int ngy = (G.gny + PY - 1) / PY;
    const int lx = lane % PX, yy = (grp % ngy) * PY + (lane / PX) % PY;
    const int zz = (grp / ngy) * EE_GATHER_PZ + lane / (PX * PY);
    const int y = G.gy0 + yy, z = G.gz0 + zz;
    const EeBeamSpec& S = specs[b];
    int x0 = 0, x1 = -1;
    if (yy >= G.gny || zz >= G.gnz || !row_span(P, S, G, y, z, x0, x1)) {
        x0 = 0;
        x1 = -1;
    }
    const int wx0 = __reduce_min_sync(FULL, x0 <= x1 ? x0 : INT_MAX);
    const int wx1 = __reduce_max_sync(FULL, x0 <= x1 ? x1 : INT_MIN);
    if (wx0 > wx1) return;
    float* out = dose + S.out_off + (mode == 2 ? (long long)b * nfull : 0ll);
    const long long rbase = (long long)P.size[0] * (y + (long long)P.size[1] * z);
    const float* base = rev + G.arena_off;
    const float dy = (float)y - G.lim_off[1], dz = (float)z - G.lim_off[2];
    for (int xs = wx0; xs <= wx1; xs += PX) {
        const int x = xs + lx;
        if (x < x0 || x > x1) continue;
        const float dx = (float)x - G.lim_off[0];
        // voxels more than 2 BEV voxels outside the crop box see no REV dose
        const f3 bi = mv(S.MB, mk(dx, dy, dz));
        float acc = 0.f;
        if (!(bi.x < -2.f || bi.y < -2.f || bi.z < -2.f || bi.x > G.bev[0] + 2.f || bi.y > G.bev[1] + 2.f ||
              bi.z > G.bev[2] + 2.f)) {
            for (int r = 0; r < P.nrays; r++) {
                const float4 a0 = s_ray[r][0], a1 = s_ray[r][1], a2 = s_ray[r][2], rv = s_ray[r][3];
                const float qx = fmaf(a0.x, dx, fmaf(a0.y, dy, fmaf(a0.z, dz, a0.w)));
                const float qy = fmaf(a1.x, dx, fmaf(a1.y, dy, fmaf(a1.z, dz, a1.w)));
                const float qz = fmaf(a2.x, dx, fmaf(a2.y, dy, fmaf(a2.z, dz, a2.w)));
                const int n0 = __float_as_int(rv.x), n1 = __float_as_int(rv.y), n2 = __float_as_int(rv.z);
                // q.y along the line (rev[0]), q.z -> rev[1], q.x -> rev[2]
                if (qy >= (float)n0 || qz >= (float)n1 || qx >= (float)n2 || qx < 0.f || qy < 0.f || qz < 0.f)
                    continue;
                // bricked REV arrays over (i, tY, tZ): x = i (q.y), y = tY (q.z), z = tZ (q.x)
                const float4 st = s_ray[r][4];
                Brick Bq;
                Bq.n0 = n0; Bq.n1 = n1; Bq.n2 = n2;
                Bq.sy = __float_as_int(st.x); Bq.sz = __float_as_int(st.y);
                acc += tri_brick_in(base + __float_as_int(rv.w), Bq, qy, qz, qx);
            }
        }
        if (mode == 2) out[rbase + x] = acc;
        else if (acc != 0.f) atomicAdd(out + rbase + x, acc);
    }
}

// Transpose of k_gather's per-voxel sum: rev_grad += S^T dose_grad, one block per
// 8x8x4 tile of patient voxels.  For each cone the tile's trilinear
// footprint in the REV grid (an AABB computed from the tile's corners under
// the affine patient -> REV map) is accumulated in shared memory first, then
// flushed with one global reduction per non-zero quad of REV samples.  The
// footprints of all cones are computed up front; consecutive cones alternate
// between two shared buffers.  The flush clears the quads it sends, so every
// buffer is all zero again when its next cone scatters into it, and one
// barrier per cone (between its scatter and its flush) suffices.
//
// The shared boxes accumulate in 32-bit fixed point: integer adds are native
// shared-memory atomics, while a float add to shared memory is a
// compare-and-swap loop (measured on the whole kernel: 1.41x as long with
// float adds; the integer form within 2 % of non-atomic adds, which give wrong
// sums and served only as a bound).  Each tile scales its
// gradients by a power of two s with max|g| * s in [2^21, 2^22), so one
// contribution w * g * s (w <= 1) is below 2^22 in magnitude and rounds to
// an integer exactly through the FP32 sum with 1.5 * 2^23; a box cell takes
// at most one contribution per tile voxel, so its sum stays below
// 256 * 2^22 = 2^30.  The rounding error per contribution is at most
// 2^-22 max|g| of the tile, about FP32 rounding at the tile's largest
// gradient; the flush converts each sum back with the exact factor 1 / s.
constexpr int GT_TX = 8, GT_TY = 8, GT_TZ = 4;
// floats per footprint buffer: an 8x8x4 tile spans at most |(7,7,3)| + 2 = 13
// REV cells per axis when the REV spacing equals the voxel size (16 along i
// after the quad alignment; 16 x 13 x 13 = 2704 < 4096).  A box clipped at
// the array's end takes one cell more on that axis, which can pass 4096 only
// for a tile at the array's corner under the widest rotation; such boxes and
// larger footprints (finer REV spacing) take the direct-scatter path
constexpr int GT_BUF = 4096;
constexpr int GT_SMEM = 2 * GT_BUF;

__global__ void __launch_bounds__(GT_TX * GT_TY * GT_TZ) k_gather_T(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                                   const EeBeamGeom* __restrict__ geoms,
                                                                   const float* __restrict__ dose_grad,
                                                                   float* __restrict__ rev_grad) {
    extern __shared__ int acc_all[];  // two fixed-point footprint boxes
    // per cone: {l0 | n0 << 16, l1 | n1 << 16, l2 | n2 << 16, s0} (box origin
    // and extent along i, tY and tZ, the box's row stride along i; all below
    // 2^16) and {v0, v1, v2} (rev - l: the box cells inside the REV array),
    // read with two vector loads before the scatter, and {sy, sz, offset lo,
    // offset hi} (the REV gradient's brick strides and the cone's arena
    // offset), read with one before the flush
    __shared__ int4 s_p[EE_MAX_RAYS][3];
    __shared__ float4 s_A[EE_MAX_RAYS][3];
    const int b = blockIdx.z;
    const EeBeamGeom& G = geoms[b];
    if (G.status != 0 || (int)blockIdx.x >= G.tiles) return;
    const EeBeamSpec& S = specs[b];
    const int ntx = (G.gnx + GT_TX - 1) / GT_TX, nty = (G.gny + GT_TY - 1) / GT_TY;
    const int tile = blockIdx.x;
    const int ox = G.gx0 + (tile % ntx) * GT_TX, oy = G.gy0 + ((tile / ntx) % nty) * GT_TY,
              oz = G.gz0 + (tile / (ntx * nty)) * GT_TZ;
    const int t = threadIdx.x;
    const int x = ox + t % GT_TX, y = oy + (t / GT_TX) % GT_TY, z = oz + t / (GT_TX * GT_TY);
    float gd = 0.f;
    const float dx = (float)x - G.lim_off[0], dy = (float)y - G.lim_off[1], dz = (float)z - G.lim_off[2];
    if (x < G.gx0 + G.gnx && y < G.gy0 + G.gny && z < G.gz0 + G.gnz) {
        gd = __ldg(dose_grad + S.out_off + x + (long long)P.size[0] * (y + (long long)P.size[1] * z));
        const f3 bi = mv(S.MB, mk(dx, dy, dz));
        if (bi.x < -2.f || bi.y < -2.f || bi.z < -2.f || bi.x > G.bev[0] + 2.f || bi.y > G.bev[1] + 2.f ||
            bi.z > G.bev[2] + 2.f)
            gd = 0.f;
    }
    __shared__ int s_gmax;  // bits of the tile's largest |gradient| (ordered as ints)
    if (t == 0) s_gmax = 0;
    if (!__syncthreads_or(gd != 0.f)) return;
    {
        const int m = __reduce_max_sync(0xffffffffu, __float_as_int(fabsf(gd)));
        if ((t & 31) == 0 && m != 0) atomicMax(&s_gmax, m);
    }
    // tile origin relative to the crop box, in patient index units
    const float o0 = (float)ox - G.lim_off[0], o1 = (float)oy - G.lim_off[1], o2 = (float)oz - G.lim_off[2];
    // REV footprint of the tile for every cone: q(v) = A (v - lim_off) - q0,
    // one (cone, REV axis) per thread; bounds widened by 1e-3 so that the
    // per-voxel q (formed in another order) never falls outside
    for (int k = t; k < 3 * P.nrays; k += blockDim.x) {
        const int r = k / 3, a = k - 3 * r;
        const EeRayGeom& R = G.ray[r];
        const float ext[3] = {(float)(GT_TX - 1), (float)(GT_TY - 1), (float)(GT_TZ - 1)};
        const float* Ar = R.A + 3 * a;
        float lo = Ar[0] * o0 + Ar[1] * o1 + Ar[2] * o2 - R.q0[a], hi = lo;
#pragma unroll
        for (int e = 0; e < 3; e++) {
            const float d = Ar[e] * ext[e];
            lo += fminf(d, 0.f);
            hi += fmaxf(d, 0.f);
        }
        // REV axes: q.y -> rev[0] (along the line), q.z -> rev[1], q.x -> rev[2]
        const int dim = a == 1 ? R.rev[0] : (a == 2 ? R.rev[1] : R.rev[2]);
        int l = max(0, (int)floorf(lo - 1e-3f));
        int h = min(dim - 1, (int)floorf(hi + 1e-3f) + 1);
        // A voxel's corners are floor(q) - l and the cell above, and floor(q)
        // <= floor(hi + 1e-3), so unclipped they stay inside [0, h - l].  Where
        // the box is clipped at the array's last cell it gets one more, so the
        // upper corner of a voxel in the last cell lands in the box; the flush
        // drops it (the forward reads 0 past the array).
        if (h == dim - 1 && h >= l) h++;
        int w = h - l + 1;
        int* sp = reinterpret_cast<int*>(s_p[r]);
        sp[8 + (a == 1 ? 0 : (a == 2 ? 1 : 2))] = dim - (a == 1 ? (l & ~3) : l);
        if (a == 1) {
            int s0 = 0;
            if (w > 0) {
                // i range on whole quads: a box row of 4 samples is one
                // 16-byte brick row of the REV gradient (flushed as one
                // vector reduction); the cells past rev[0] are brick padding
                w = ((h | 3) + 1) - (l & ~3);
                l &= ~3;
                // row stride 4 (mod 8) floats: the rows of adjacent voxels
                // spread over the shared banks; the extra quad of a row is
                // never scattered to, stays zero and is not sent
                s0 = (w & 7) == 0 ? w + 4 : w;
            }
            sp[3] = s0;
        }
        sp[a == 1 ? 0 : (a == 2 ? 1 : 2)] = l | (max(w, 0) << 16);
        if (a == 0) {
            const Brick Bv = rev_brick(R.rev[0], R.rev[1], R.rev[2]);
            sp[4] = Bv.sy;
            sp[5] = Bv.sz;
            sp[6] = (int)(unsigned)(R.offset & 0xffffffffll);
            sp[7] = (int)(R.offset >> 32);
        }
        // this cone's map for the voxels: the row [A | -q0] of REV axis a
        // (the forward gather forms q in the same order)
        s_A[r][a] = make_float4(Ar[0], Ar[1], Ar[2], -R.q0[a]);
    }
    int4* const all4 = reinterpret_cast<int4*>(acc_all);
    for (int k = t; k < GT_SMEM / 4; k += blockDim.x) all4[k] = make_int4(0, 0, 0, 0);
    __syncthreads();
    float* base = rev_grad + G.arena_off;
    // fixed-point scale s = 2^(148 - e) for the biased exponent e of max|g|
    // (max|g| < 2^(e - 126)), clamped to normal floats; a NaN or infinite
    // gradient makes 1 / s a NaN, so it reaches the cells the tile touches
    const int ge = (s_gmax >> 23) & 0xff;
    const int se = min(max(275 - ge, 1), 253);
    const float fx_scale = __int_as_float(se << 23);
    const float fx_inv = ge == 0xff ? __int_as_float(0x7fc00000) : __int_as_float((254 - se) << 23);
    const float gds = gd * fx_scale;
    int parity = 0;  // buffer of the next shared-memory cone
    for (int r = 0; r < P.nrays; r++) {
        const int4 p0 = s_p[r][0];
        const int l0 = p0.x & 0xffff, n0 = p0.x >> 16, l1 = p0.y & 0xffff, n1 = p0.y >> 16, l2 = p0.z & 0xffff,
                  n2 = p0.z >> 16;
        const bool empty = n0 <= 0 || n1 <= 0 || n2 <= 0;
        // box cell (k0, k1, k2) over (i, tY, tZ) at k0 + s0 * (k1 + n1p * k2)
        const int s0 = empty ? 0 : p0.w;  // row stride of the box (>= n0, a multiple of 4)
        // rows per slab: odd, so that the slab stride s0 * n1p is 4 x odd
        // (mod 32) and the slabs of adjacent voxels spread over the banks
        // too; the padding rows (k1 >= n1) are never scattered to
        const int n1p = n1 | 1;
        const int nbox = empty ? 0 : n1p * s0 * n2;
        if (nbox > 0 && nbox <= GT_BUF) {
            // buffers alternate over the shared-memory cones: the last flush
            // of this buffer (two such cones back) was cleared by every
            // thread before the barrier of the previous cone
            int* acc = acc_all + parity * GT_BUF;
            parity ^= 1;
            if (gd != 0.f) {
                const float4 a0 = s_A[r][0], a1 = s_A[r][1], a2 = s_A[r][2];
                const f3 q = mk(fmaf(a0.x, dx, fmaf(a0.y, dy, fmaf(a0.z, dz, a0.w))),
                                fmaf(a1.x, dx, fmaf(a1.y, dy, fmaf(a1.z, dz, a1.w))),
                                fmaf(a2.x, dx, fmaf(a2.y, dy, fmaf(a2.z, dz, a2.w))));
                // the forward gather skips a cone where q is outside [0, rev)
                if (!(q.x < 0.f || q.y < 0.f || q.z < 0.f)) {
                    const int4 pv = s_p[r][2];  // rev - l per axis
                    const float f0 = floorf(q.y), f1 = floorf(q.z), f2 = floorf(q.x);
                    const int j0 = (int)f0 - l0, j1 = (int)f1 - l1, j2 = (int)f2 - l2;
                    if (j0 < pv.x && j1 < pv.y && j2 < pv.z) {
                        const float a0 = q.y - f0, a1 = q.z - f1, a2 = q.x - f2;
                        // all eight corners lie in the box (its set-up above);
                        // those past the array's end are dropped by the flush
                        const float w0[2] = {1.f - a0, a0}, w1[2] = {1.f - a1, a1}, w2[2] = {1.f - a2, a2};
                        int* const c = acc + j0 + s0 * (j1 + n1p * j2);
                        const int ss = s0 * n1p;
#pragma unroll
                        for (int d2 = 0; d2 < 2; d2++) {
                            const float t2 = w2[d2] * gds;
#pragma unroll
                            for (int d1 = 0; d1 < 2; d1++) {
                                const float t1 = w1[d1] * t2;
                                // w * g * s rounded to an integer: the sum with
                                // 1.5 * 2^23 has unit spacing, its low bits are
                                // the integer (|w g s| < 2^22)
#pragma unroll
                                for (int d0 = 0; d0 < 2; d0++)
                                    atomicAdd(c + d0 + d1 * s0 + d2 * ss,
                                              __float_as_int(fmaf(w0[d0], t1, 12582912.f)) - 0x4B400000);
                            }
                        }
                    }
                }
            }
            __syncthreads();
            const int4 p1 = s_p[r][1];
            float* rb = base + (long long)(((unsigned long long)(unsigned)p1.w << 32) | (unsigned)p1.z);
            Brick Bv;  // strides only (bk_y, bk_z)
            Bv.sy = p1.x;
            Bv.sz = p1.y;
            // one box quad (4 samples) per iteration, quad index = kq + nq0 *
            // (k1 + n1p * k2); (k + 0.5) / n is at least 1/(2n) away from an
            // integer, far above the FP32 error of (k + 0.5) * rcp(n) for
            // these sizes, so the floored quotients are exact.  A non-zero quad is one 16-byte vector
            // reduction into the bricked REV gradient (brick rows are 16-byte
            // aligned: arena and cone offsets are multiples of 64 floats),
            // and is cleared for the buffer's next cone.
            int4* acc4 = reinterpret_cast<int4*>(acc);  // s0 is a multiple of 4
            const int nquad = nbox >> 2;
            const int nq0 = s0 >> 2;
            const float invq = __frcp_rn((float)nq0), inv1 = __frcp_rn((float)n1p);
            for (int k = t; k < nquad; k += blockDim.x) {
                const int4 v = acc4[k];
                if (v.x != 0 || v.y != 0 || v.z != 0 || v.w != 0) {
                    acc4[k] = make_int4(0, 0, 0, 0);
                    const int q1 = __float2int_rd(((float)k + 0.5f) * invq);
                    const int kq = k - q1 * nq0;
                    const int k2 = __float2int_rd(((float)q1 + 0.5f) * inv1);
                    const int k1 = q1 - k2 * n1p;
                    // rows and slabs past the array's end and quads that
                    // start past it hold the forward's border corners (0):
                    // cleared, not sent; a quad that starts inside the array
                    // ends in its last brick, whose padding nothing reads
                    const int4 pv = s_p[r][2];
                    if (4 * kq < pv.x && k1 < pv.y && k2 < pv.z)
                        red_v4(rb + bk_x(l0 + 4 * kq) + bk_y(Bv, l1 + k1) + bk_z(Bv, l2 + k2), (float)v.x * fx_inv,
                               (float)v.y * fx_inv, (float)v.z * fx_inv, (float)v.w * fx_inv);
                }
            }
        } else if (nbox > GT_BUF && gd != 0.f) {
            // footprint too large for a shared buffer (a REV spacing finer
            // than the voxels): scatter directly
            const EeRayGeom& R = G.ray[r];
            const float4 a0 = s_A[r][0], a1 = s_A[r][1], a2 = s_A[r][2];
            const f3 q = mk(fmaf(a0.x, dx, fmaf(a0.y, dy, fmaf(a0.z, dz, a0.w))),
                            fmaf(a1.x, dx, fmaf(a1.y, dy, fmaf(a1.z, dz, a1.w))),
                            fmaf(a2.x, dx, fmaf(a2.y, dy, fmaf(a2.z, dz, a2.w))));
            if (!(q.y >= (float)R.rev[0] || q.z >= (float)R.rev[1] || q.x >= (float)R.rev[2] || q.x < 0.f ||
                  q.y < 0.f || q.z < 0.f))
                tri_brick_scatter(base + R.offset, rev_brick(R.rev[0], R.rev[1], R.rev[2]), q.y, q.z, q.x, gd);
        }
    }
}

// TERMA adjoint with supersampling (ss > 1): the transpose of k_terma_ss,
// whose voxel TERMA is the mean over ss^3 sub-voxel centres of fluence x
// unit TERMA, each centre with its own beamlet lookup and ray trace
// (cudaSiddon.cu:248-258, 297-306).  The forward keeps neither the beamlets
// nor the unit TERMA of the centres, so each voxel with a non-zero TERMA
// gradient recomputes them (the same centres, lookups and traces) and adds
// gradient x unit / ss^3 to its centres' beamlets; consecutive centres that
// share a beamlet add once.  The fluence enters linearly, as in the ss = 1
// adjoint (a centre whose beamlet has zero fluence still has its slope).
__global__ void __launch_bounds__(256) k_terma_T_ss(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                    const float* __restrict__ terma_grad, float* __restrict__ fgrad) {
    const int b = blockIdx.z;
    const EeBeamSpec& S = specs[b];
    const long long bvol = ee_brick_vol(S.tn);
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= bvol) return;
    const long long brick = v >> 6;
    const int w = (int)(v & 63), nbx = (S.tn[0] + 3) >> 2, nby = (S.tn[1] + 3) >> 2;
    const long long bxy = brick % ((long long)nbx * nby);
    const int xr = (int)(bxy % nbx) * 4 + (w & 3);
    const int yr = (int)(bxy / nbx) * 4 + ((w >> 2) & 3);
    const int zr = (int)(brick / ((long long)nbx * nby)) * 4 + (w >> 4);
    if (xr >= S.tn[0] || yr >= S.tn[1] || zr >= S.tn[2]) return;
    const float g = terma_grad[S.t_off + v];
    if (g == 0.f) return;
    const int x = S.t0[0] + xr, y = S.t0[1] + yr, z = S.t0[2] + zr;
    const f3 src = ld3(S.src);
    const int ss = P.ss, nsub = ss * ss * ss;
    const float gs = g / (float)nsub;
    const float sv0 = P.voxel[0] / (float)ss, sv1 = P.voxel[1] / (float)ss, sv2 = P.voxel[2] / (float)ss;
    bool cap = false;
    int cur = -1;
    float acc = 0.f;
    for (int ii = 0; ii < nsub; ii++) {
        const int sx = ii % ss, sy = (ii / ss) % ss, sz = ii / (ss * ss);
        const f3 p = mk(P.start[0] + ((float)x - 0.5f) * P.voxel[0] + ((float)sx + 0.5f) * sv0,
                        P.start[1] + ((float)y - 0.5f) * P.voxel[1] + ((float)sy + 0.5f) * sv1,
                        P.start[2] + ((float)z - 0.5f) * P.voxel[2] + ((float)sz + 0.5f) * sv2);
        int bs = beamlet_of(S, p);
        if (bs == -2) bs = beamlet_point_fp64(S, (double)p.x, (double)p.y, (double)p.z);
        if (bs < 0) continue;
        const float rpl = siddon_rpl(P, p, src, cap);
        const float u = terma_per_fluence(P, rpl, p, src, S.sad);
        if (bs != cur) {
            if (cur >= 0 && acc != 0.f) atomicAdd(fgrad + S.fl_off + cur, acc);
            cur = bs;
            acc = 0.f;
        }
        acc = fmaf(gs, u, acc);
    }
    if (cur >= 0 && acc != 0.f) atomicAdd(fgrad + S.fl_off + cur, acc);
}

// TERMA adjoint: fluence_grad[beamlet(v)] += G_v * terma_grad[v].  A block
// takes TT_VPT * 256 consecutive bricked voxels (a run of bricks along x) and
// sums them per beamlet in a shared histogram of the beam's fluence map, then
// adds the non-zero bins to the fluence gradient: one global atomic per
// beamlet the run touches.  Maps above TT_HIST beamlets aggregate per warp
// (lanes of equal beamlet index summed before one atomic) instead.
constexpr int TT_HIST = 4096, TT_VPT = 4;

__global__ void __launch_bounds__(256) k_terma_T(EeParams P, const EeBeamSpec* __restrict__ specs,
                                                 const float* __restrict__ unit, const int* __restrict__ bl_idx,
                                                 const float* __restrict__ terma_grad, float* __restrict__ fluence_grad) {
    __shared__ float hist[TT_HIST];
    const int b = blockIdx.z;
    const EeBeamSpec& S = specs[b];
    const long long tvol = ee_brick_vol(S.tn);  // padding: bl_idx -1
    const long long v0 = (long long)blockIdx.x * (256 * TT_VPT);
    if (v0 >= tvol) return;
    const int t = threadIdx.x, nfl = S.fmap[0] * S.fmap[1];
    float* fg = fluence_grad + S.fl_off;
    if (nfl > TT_HIST) {
        for (int j = 0; j < TT_VPT; j++) {
            const long long v = v0 + j * 256 + t;
            int bl = -1;
            float val = 0.f;
            if (v < tvol) {
                const long long o = S.t_off + v;
                bl = bl_idx[o];
                if (bl >= 0) val = unit[o] * terma_grad[o];
            }
            const unsigned peers = __match_any_sync(FULL, bl);
            const int leader = __ffs(peers) - 1;
            float sum = 0.f;
            for (unsigned m = peers; m; m &= m - 1) sum += __shfl_sync(peers, val, __ffs(m) - 1);
            if ((t & 31) == leader && bl >= 0 && sum != 0.f) atomicAdd(fg + bl, sum);
        }
        return;
    }
    for (int k = t; k < nfl; k += 256) hist[k] = 0.f;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < TT_VPT; j++) {
        const long long v = v0 + j * 256 + t;
        if (v < tvol) {
            const long long o = S.t_off + v;
            const int bl = bl_idx[o];
            if (bl >= 0) {
                const float val = unit[o] * terma_grad[o];
                if (val != 0.f) atomicAdd(hist + bl, val);
            }
        }
    }
    __syncthreads();
    for (int k = t; k < nfl; k += 256) {
        const float h = hist[k];
        if (h != 0.f) atomicAdd(fg + k, h);
    }
}

}  // namespace

// ----------------------------------------------------------- launchers ---
static inline unsigned grid1(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

cudaError_t ee_launch_geom_init(const EeBeamSpec* specs, EeBeamGeom* g, int nbeams, cudaStream_t s) {
    k_geom_init<<<grid1(nbeams, 128), 128, 0, s>>>(specs, g, nbeams);
    return cudaGetLastError();
}

cudaError_t ee_copy_status(const EeBeamGeom* geoms, int* status_host, int nbeams, cudaStream_t s) {
    return cudaMemcpy2DAsync(status_host, sizeof(int), (const char*)geoms + offsetof(EeBeamGeom, status),
                             sizeof(EeBeamGeom), sizeof(int), nbeams, cudaMemcpyDeviceToHost, s);
}

cudaError_t ee_launch_terma(const EeParams& P, const EeBeamSpec* specs, EeBeamGeom* geoms, const float* fluence,
                            float* terma, float* unit, int* beamlet_idx, int nbeams, long long max_tvol,
                            cudaStream_t s) {
    dim3 grid(grid1(max_tvol, 256), 1, nbeams);
    if (P.ss > 1) k_terma_ss<<<grid, 256, 0, s>>>(P, specs, geoms, fluence, terma, unit, beamlet_idx);
    else k_terma<<<grid, 256, 0, s>>>(P, specs, geoms, fluence, terma, unit, beamlet_idx);
    return cudaGetLastError();
}

cudaError_t ee_launch_geometry(const EeParams& P, const EeBeamSpec* specs, EeBeamGeom* geoms, int nbeams,
                               cudaStream_t s) {
    k_geometry<<<nbeams, 64, 0, s>>>(P, specs, geoms);
    return cudaGetLastError();
}

static size_t cone_smem(int maxL) { return sizeof(float) * ((size_t)CONE_WARPS * 3 * maxL + 2 * EE_MAX_RADII + EE_MAX_RADII); }

// Raise a kernel's dynamic shared-memory limit on the current device.  The
// attribute belongs to the (device, kernel) pair, so the cache of what was
// set is keyed by both; the lock covers concurrent server threads.  The
// first eager launch on a device sets it, before any graph capture.
static cudaError_t smem_attr(const void* fn, size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    struct Done {
        int dev;
        const void* fn;
        size_t sz;
    };
    static std::mutex mu;
    static Done done[64];
    static int ndone = 0;
    std::lock_guard<std::mutex> lock(mu);
    for (int k = 0; k < ndone; k++)
        if (done[k].dev == dev && done[k].fn == fn && done[k].sz >= smem) return cudaSuccess;
    size_t got = std::max(smem, (size_t)200 * 1024);  // once, to the largest size any line needs
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)got);
    if (e != cudaSuccess) {
        got = smem;
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)got);
    }
    if (e != cudaSuccess) return e;
    for (int k = 0; k < ndone; k++)
        if (done[k].dev == dev && done[k].fn == fn) { done[k].sz = got; return cudaSuccess; }
    if (ndone < 64) done[ndone++] = Done{dev, fn, got};
    return cudaSuccess;
}

cudaError_t ee_launch_cone(const EeParams& P, const EeBeamSpec* specs, const EeBeamGeom* geoms, const float* terma,
                           float* rev, float2* samples, int nbeams, int max_lines, int max_line, cudaStream_t s,
                           int lane_block) {
    if (P.mode == 1 && samples) {  // exp kernel: one lane per line; the caller zeroed `rev`
        dim3 grid(grid1(max_lines, lane_block), P.nrays, nbeams);
        if (lane_block == 64) k_cone_lane<64><<<grid, 64, 0, s>>>(P, specs, geoms, terma, rev, samples);
        else if (lane_block == 256) k_cone_lane<256><<<grid, 256, 0, s>>>(P, specs, geoms, terma, rev, samples);
        else k_cone_lane<128><<<dim3(grid1(max_lines, 128), P.nrays, nbeams), 128, 0, s>>>(P, specs, geoms, terma, rev, samples);
        return cudaGetLastError();
    }
    if (P.mode == EE_KERNEL_TABLE && P.nradii == TAB_NR) {  // exact O(n nr) table scan
        const size_t smem = sizeof(float) * ((size_t)TAB_WARPS * tab_fwd_stride(max_line) + TAB_SMEM);
        cudaError_t e = smem_attr((const void*)k_cone_tab, smem);
        if (e != cudaSuccess) return e;
        dim3 grid(grid1(max_lines, 2 * TAB_WARPS), P.nrays, nbeams);
        k_cone_tab<<<grid, TAB_WARPS * 32, smem, s>>>(P, specs, geoms, terma, rev, max_line);
        return cudaGetLastError();
    }
    size_t smem = cone_smem(max_line);
    cudaError_t e = smem_attr((const void*)k_cone, smem);
    if (e != cudaSuccess) return e;
    dim3 grid(grid1(max_lines, CONE_WARPS), P.nrays, nbeams);
    k_cone<<<grid, CONE_WARPS * 32, smem, s>>>(P, specs, geoms, terma, rev, max_line);
    return cudaGetLastError();
}

cudaError_t ee_launch_rev_zero(const EeParams& P, const EeBeamGeom* geoms, float* rev_grad, int nbeams, int max_lines,
                               cudaStream_t s) {
    k_rev_zero<128><<<dim3(grid1(max_lines, 128), P.nrays, nbeams), 128, 0, s>>>(P, geoms, rev_grad);
    return cudaGetLastError();
}

cudaError_t ee_launch_gather(const EeParams& P, const EeBeamSpec* specs, const EeBeamGeom* geoms, const float* rev,
                             float* dose, int nbeams, int dose_mode, int max_rows, cudaStream_t s) {
    long long nfull = (long long)P.size[0] * P.size[1] * P.size[2];
    dim3 grid(grid1(max_rows, ROW_WARPS), 1, nbeams);
    k_gather<<<grid, ROW_WARPS * 32, 0, s>>>(P, specs, geoms, rev, dose, dose_mode, nfull);
    return cudaGetLastError();
}

cudaError_t ee_launch_gather_T(const EeParams& P, const EeBeamSpec* specs, const EeBeamGeom* geoms,
                               const float* dose_grad, float* rev_grad, int nbeams, int max_tiles, cudaStream_t s) {
    const size_t smem = sizeof(float) * GT_SMEM;
    cudaError_t e = smem_attr((const void*)k_gather_T, smem);
    if (e != cudaSuccess) return e;
    dim3 grid(max(1, max_tiles), 1, nbeams);
    k_gather_T<<<grid, GT_TX * GT_TY * GT_TZ, smem, s>>>(P, specs, geoms, dose_grad, rev_grad);
    return cudaGetLastError();
}

cudaError_t ee_launch_cone_T(const EeParams& P, const EeBeamSpec* specs, const EeBeamGeom* geoms, const float* rev_grad,
                             float2* scratch, float* terma_grad, int nbeams, int max_lines, int max_line,
                             cudaStream_t s, int lane_block) {
    if (P.mode == 1 && scratch) {
        dim3 grid(grid1(max_lines, lane_block), P.nrays, nbeams);
        if (lane_block == 64) k_cone_T_lane<64><<<grid, 64, 0, s>>>(P, specs, geoms, rev_grad, scratch, terma_grad);
        else if (lane_block == 256) k_cone_T_lane<256><<<grid, 256, 0, s>>>(P, specs, geoms, rev_grad, scratch, terma_grad);
        else
            k_cone_T_lane<128><<<dim3(grid1(max_lines, 128), P.nrays, nbeams), 128, 0, s>>>(P, specs, geoms, rev_grad,
                                                                                          scratch, terma_grad);
        return cudaGetLastError();
    }
    if (P.mode == EE_KERNEL_TABLE && P.nradii == TAB_NR) {
        const size_t smem = sizeof(float) * ((size_t)TAB_WARPS * tab_adj_stride(max_line) + TAB_SMEM);
        cudaError_t e = smem_attr((const void*)k_cone_T_tab, smem);
        if (e != cudaSuccess) return e;
        dim3 grid(grid1(max_lines, 2 * TAB_WARPS), P.nrays, nbeams);
        k_cone_T_tab<<<grid, TAB_WARPS * 32, smem, s>>>(P, specs, geoms, rev_grad, terma_grad, max_line);
        return cudaGetLastError();
    }
    size_t smem = cone_smem(max_line);
    cudaError_t e = smem_attr((const void*)k_cone_T, smem);
    if (e != cudaSuccess) return e;
    dim3 grid(grid1(max_lines, CONE_WARPS), P.nrays, nbeams);
    k_cone_T<<<grid, CONE_WARPS * 32, smem, s>>>(P, specs, geoms, rev_grad, terma_grad, max_line);
    return cudaGetLastError();
}

cudaError_t ee_launch_terma_T(const EeParams& P, const EeBeamSpec* specs, const EeBeamGeom* geoms,
                              const float* unit_terma, const int* beamlet_idx, const float* terma_grad,
                              float* fluence_grad, int nbeams, long long max_tvol, cudaStream_t s) {
    (void)geoms;
    if (P.ss > 1) {  // supersampled TERMA: recompute the sub-voxel beamlets
        k_terma_T_ss<<<dim3(grid1(max_tvol, 256), 1, nbeams), 256, 0, s>>>(P, specs, terma_grad, fluence_grad);
        return cudaGetLastError();
    }
    dim3 grid(grid1(max_tvol, 256 * TT_VPT), 1, nbeams);
    k_terma_T<<<grid, 256, 0, s>>>(P, specs, unit_terma, beamlet_idx, terma_grad, fluence_grad);
    return cudaGetLastError();
}

// ------------------------------------------------- EndtoEnd loss terms ----
// Dose terms of the EndtoEnd loss (README.md:20):
//   L_d = sum_i w0_i (d_i - t0_i)^2 + sum_i w_i max(d_i - t_i, 0)^2
// and its gradient dL/dd.  acc[0] += PTV term, acc[1] += OAR term.
__global__ void __launch_bounds__(256) k_loss_grad(const float* __restrict__ dose, const float* __restrict__ ptv_w,
                                                   const float* __restrict__ ptv_t, const float* __restrict__ oar_w,
                                                   const float* __restrict__ oar_t, float* __restrict__ grad,
                                                   double* __restrict__ acc, long long n) {
    double lp = 0.0, lo = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float d = dose[i];
        float g = 0.f;
        if (ptv_w) {
            float w = ptv_w[i], e = d - ptv_t[i];
            lp += (double)w * e * e;
            g += 2.f * w * e;
        }
        if (oar_w) {
            float w = oar_w[i], e = fmaxf(d - oar_t[i], 0.f);
            lo += (double)w * e * e;
            g += 2.f * w * e;
        }
        grad[i] = g;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lp += __shfl_xor_sync(FULL, lp, o);
        lo += __shfl_xor_sync(FULL, lo, o);
    }
    __shared__ double sp[8], so[8];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { sp[w] = lp; so[w] = lo; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) { a += sp[k]; b += so[k]; }
        atomicAdd(acc, a);
        atomicAdd(acc + 1, b);
    }
}

// Fluence-map convolution with a normalised 2-D Gaussian (the EndtoEnd
// fluence-spread step, README.md:15-18), zero padding.  The kernel is
// symmetric, so the same launch is its own transpose.  One thread per output
// pixel of beam blockIdx.z.
__global__ void __launch_bounds__(256) k_spread(const EeBeamSpec* __restrict__ specs, const float* __restrict__ in,
                                                float* __restrict__ out, const float* __restrict__ w1d, int R) {
    const EeBeamSpec& S = specs[blockIdx.z];
    const int fx = S.fmap[0], fy = S.fmap[1];
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fx * fy) return;
    int x = p % fx, y = p / fx;
    const float* src = in + S.fl_off;
    float acc = 0.f;
    for (int dy = -R; dy <= R; dy++) {
        int yy = y + dy;
        if (yy < 0 || yy >= fy) continue;
        float wy = w1d[dy + R];
        for (int dx = -R; dx <= R; dx++) {
            int xx = x + dx;
            if (xx < 0 || xx >= fx) continue;
            acc += wy * w1d[dx + R] * src[xx + fx * yy];
        }
    }
    out[S.fl_off + p] = acc;
}

// eta * ||D x||_1 with D the forward differences along both fluence-map axes
// (BOO/BOO_QL/CreateDxDyFMO.m:1-36); adds eta * D^T sign(D x)
// into grad and the term into acc[2].
__global__ void __launch_bounds__(256) k_smooth(const EeBeamSpec* __restrict__ specs, const float* __restrict__ x,
                                                float* __restrict__ grad, float eta, double* __restrict__ acc) {
    const EeBeamSpec& S = specs[blockIdx.z];
    const int fx = S.fmap[0], fy = S.fmap[1];
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (p < fx * fy) {
        int i = p % fx, j = p / fx;
        const float* m = x + S.fl_off;
        float v = m[p], g = 0.f;
        if (i + 1 < fx) { float d = m[p + 1] - v; l += fabsf(d); g -= (d > 0.f) - (d < 0.f); }
        if (i > 0) { float d = v - m[p - 1]; g += (d > 0.f) - (d < 0.f); }
        if (j + 1 < fy) { float d = m[p + fx] - v; l += fabsf(d); g -= (d > 0.f) - (d < 0.f); }
        if (j > 0) { float d = v - m[p - fx]; g += (d > 0.f) - (d < 0.f); }
        grad[S.fl_off + p] += eta * g;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(FULL, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(acc + 2, (double)eta * l);
}

cudaError_t ee_launch_loss_grad(const float* dose, const float* ptv_w, const float* ptv_t, const float* oar_w,
                                const float* oar_t, float* grad, double* acc, long long n, cudaStream_t s) {
    k_loss_grad<<<std::min<long long>(grid1(n, 256), 152 * 8), 256, 0, s>>>(dose, ptv_w, ptv_t, oar_w, oar_t, grad, acc, n);
    return cudaGetLastError();
}

cudaError_t ee_launch_spread(const EeBeamSpec* specs, const float* in, float* out, const float* w1d, int R, int nbeams,
                             int max_pix, cudaStream_t s) {
    dim3 grid(grid1(max_pix, 256), 1, nbeams);
    k_spread<<<grid, 256, 0, s>>>(specs, in, out, w1d, R);
    return cudaGetLastError();
}

cudaError_t ee_launch_smooth(const EeBeamSpec* specs, const float* x, float* grad, float eta, double* acc, int nbeams,
                             int max_pix, cudaStream_t s) {
    dim3 grid(grid1(max_pix, 256), 1, nbeams);
    k_smooth<<<grid, 256, 0, s>>>(specs, x, grad, eta, acc);
    return cudaGetLastError();
}
