// ee_beamlet.cu -- beamlet dose columns (the dosecalc-beamlet path) on sm_103a.
//
// Semantics follow CCCS/dosecalc-beamlet/nvbbRayConvolve_host.cu and
// nvbbRayConvolve_device.cu: every active beamlet (fluence > 0) owns a pillar
// -- a box along its own divergent axis spanning the calc bbox plus the
// kernel extent, walled off from its neighbours -- the pillars are packed in
// one grid, and for each of the nphi*ntheta/2 convolution directions the
// grid is resampled into the rotated REV frame, convolved along REV lines with
// the cumulative-kernel walk (walls stop the walk), and gathered back.  Each
// pillar is then unpacked onto the calc bbox and thresholded into one sparse
// column.
//
// GB300 organisation:
//   k_bl_samples one thread per REV sample: pillar lookup and the beamlet
//                test (exact only inside a box around the footprint);
//                samples inside their beamlet are queued (the reference runs
//                a Siddon trace for every sample).
//   k_bl_terma   Siddon TERMA of the queued samples, lane-dense, flagging
//                their lines.
//   k_bl_walk    one warp per flagged REV line: densities sampled into
//                shared memory, each lane summing its outputs over the line's
//                TERMA samples as the walk would; other lines stay 0.
//   k_bl_gather  packed-grid voxel += trilinear REV dose of one direction.
//   k_bl_rows .. k_bl_emit
//                unpack: per pillar only the calc-bbox rows its oriented box
//                crosses, with the exact x-interval of each row; column max,
//                threshold count, prefix sums and a sorted CSR write, all on
//                the device (the reference copies a dense bbox per beamlet to
//                the host and sparsifies there, sparse_io.cpp:22-59).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>

#include "../../include/ee_cccs.h"
#include "ee_device.cuh"
#include "ee_internal.h"

int ee_internal_fail(int code, const char* msg);

namespace {

constexpr int BL_WALL = 2;  // pillar wall thickness, REV voxels (io_data_structs.h:147)
constexpr int BL_BUF = 2;   // unusable buffer inside the walls (io_data_structs.h:148)
constexpr int BL_WARPS = 4;

// ------------------------------------------------------------- tables ---
struct BlPillar {
    float M[9];        // pillar-index vector -> RCS offset (inverse beamlet, then inverse beam rotation)
    float Mi[9];       // RCS offset -> pillar-index vector
    float ps[3];       // pillar start, RCS cm
    int fidx;          // fluence-map index of the beamlet
    int ix, iz;        // pillar position in the packed grid
    int b0[3], bn[3];  // calc-bbox-index AABB of the pillar's usable region (unpack)
    long long row0;    // first unpack row of this pillar
    // the beamlet's footprint (the rays from the source through the corners
    // of its fluence-map cell) in pillar-index coordinates: corner ray c is
    // x = ex[c] + sx[c] * y, z = ez[c] + sz[c] * y
    float ex[4], sx[4], ez[4], sz[4];
};

struct BlGrid {
    int n;             // pillars in this batch
    int npx, npz;      // pillars along the packed grid's x and z
    int pd[3];         // pillar dims (REV voxels)
    int gd[3];         // packed grid dims
    float vs[3];       // REV voxel size (lat, long, lat)
    float kr[EE_MAX_RADII];  // kernel radii: the radial bins' mean radii (host.cu:352-357)
    float kern_extent;
};

// --------------------------------------------- host geometry (FP32) ------
// The reference computes the pillar layout on the host in FP32
// (nvbbRayConvolve_host.cu:180-280, 600-690, 75-155); the pillar and REV
// sizes truncate ratios that are integers in exact arithmetic, so the same
// FP32 operations are kept here to land on the same sizes.
struct v3 {
    float x, y, z;
};
v3 operator+(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
v3 operator-(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
v3 operator*(v3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
v3 operator*(v3 a, v3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
float len(v3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
float comp(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// Rodrigues rotation of p about the unit axis r by t, in the operation order
// of geometry.cu's rotateAroundAxisAtOriginRHS
v3 rot_axis(v3 p, v3 r, float t) {
    float s = sinf(t), c = cosf(t);
    float d = -r.x * p.x - r.y * p.y - r.z * p.z;
    return {(-r.x * d) * (1 - c) + p.x * c + (-r.z * p.y + r.y * p.z) * s,
            (-r.y * d) * (1 - c) + p.y * c + (+r.z * p.x - r.x * p.z) * s,
            (-r.z * d) * (1 - c) + p.z * c + (-r.y * p.x + r.x * p.y) * s};
}
v3 inv_rot_beam(v3 v, float az, float zen, float coll) {
    v3 t = rot_axis(v, {0.f, 1.f, 0.f}, -(zen + coll));
    return rot_axis(t, {sinf(-zen), 0.f, cosf(-zen)}, az);
}
v3 rot_beam(v3 v, float az, float zen, float coll) {
    v3 t = rot_axis(v, {sinf(-zen), 0.f, cosf(-zen)}, -az);
    return rot_axis(t, {0.f, 1.f, 0.f}, zen + coll);
}
// beamlet frame about the divergence angles (geometry.cu:99-115)
v3 inv_rot_beamlet(v3 v, float th, float ph) { return rot_axis(v, {sinf(-ph), 0.f, cosf(-ph)}, -th); }
v3 rot_beamlet(v3 v, float th, float ph) { return inv_rot_beamlet(v, -th, ph); }
v3 rot_kern(v3 v, float th, float ph) {
    v3 u = rot_axis(v, {cosf(ph), 0.f, -sinf(ph)}, -th);
    return rot_axis(u, {0.f, 1.f, 0.f}, -ph);
}

template <class F>
void matrix(F f, float* M) {
    v3 c[3] = {f({1.f, 0.f, 0.f}), f({0.f, 1.f, 0.f}), f({0.f, 0.f, 1.f})};
    for (int j = 0; j < 3; j++) {
        M[0 * 3 + j] = c[j].x;
        M[1 * 3 + j] = c[j].y;
        M[2 * 3 + j] = c[j].z;
    }
}

struct Beamlet {
    int fidx;
    v3 first, last, biso;
    float th, ph;  // divergence angles
    float length;
};

// calcBeamletAnchors (host.cu:180-280): the beamlet's isocentre, divergence
// angles, and the nearest / farthest crossings of its axis with the calc
// bbox faces (0.05 cm tolerance).  false: the axis misses the bbox.
bool anchors(Beamlet& B, v3 src, v3 iso, int idx, float bsx, float bsy, int fx, int fy, v3 voxel, v3 dstart, v3 bb0,
             v3 bbs, float az, float zen, float coll) {
    const unsigned bx = (unsigned)idx % (unsigned)fx, by = (unsigned)idx / (unsigned)fx;
    const v3 bdiff = {bsx * (-0.5f * fx + bx + 0.5f), 0.f, bsy * (-0.5f * fy + by + 0.5f)};
    B.biso = iso + inv_rot_beam(bdiff, az, zen, coll);
    B.th = acosf(len(iso - src) / len(B.biso - src));
    B.ph = atan2f(bdiff.z, bdiff.x);
    const v3 lo = dstart + voxel * bb0;
    const v3 hi = lo + voxel * bbs;
    const double buf = 0.05;
    const v3 d = B.biso - src;
    v3 hit[6];
    for (int a = 0; a < 3; a++) {
        const double den = comp(d, a);
        const double t1 = (comp(lo, a) - comp(src, a)) / (den + 1e-12);
        const double t2 = (comp(hi, a) - comp(src, a)) / (den + 1e-12);
        hit[2 * a] = src + d * (float)t1;
        hit[2 * a + 1] = src + d * (float)t2;
    }
    B.first = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(), std::numeric_limits<float>::max()};
    B.last = {std::numeric_limits<float>::min(), std::numeric_limits<float>::min(), std::numeric_limits<float>::min()};
    double dmin = std::numeric_limits<double>::max(), dmax = std::numeric_limits<double>::min();
    for (int a = 0; a < 3; a++)
        for (int s = 0; s < 2; s++) {
            const v3 p = hit[2 * a + s];
            const int u = (a + 1) % 3, v = (a + 2) % 3;
            if (comp(p, u) + buf >= comp(lo, u) && comp(p, u) - buf <= comp(hi, u) && comp(p, v) + buf >= comp(lo, v) &&
                comp(p, v) - buf <= comp(hi, v)) {
                if (len(p - src) < dmin) { B.first = p; dmin = len(B.first - src); }
                if (len(p - src) > dmax) { B.last = p; dmax = len(B.last - src); }
            }
        }
    B.length = len(B.last - B.first);
    return dmin < std::numeric_limits<float>::max() && dmax > std::numeric_limits<float>::min();
}

}  // namespace

namespace {

// ------------------------------------------------------------ kernels ----
// One convolution direction of a batch.
struct BlRayDev {
    int rev[3];        // REV size: along the line, lateral, lateral
    float rs[3];       // REV box origin (cm, REV frame)
    float rcp[3];      // 1 / REV voxel size
    float MK[9], MKi[9];
    int row_f, row_r;  // kernel rows of the two walk directions
};

// Linear filtering of one kernel row at texel coordinate x (unnormalised,
// clamp addressing) with the filter weight rounded to 8 fractional bits as
// the texture unit does.
__device__ __forceinline__ float kern_tex(const float* K, int nr, float x) {
    float xb = x - 0.5f;
    float fx = floorf(xb);
    int i = (int)fx;
    float a = xb - fx;
    a = floorf(a * 256.f + 0.5f) * (1.f / 256.f);
    int i0 = min(max(i, 0), nr - 1), i1 = min(max(i + 1, 0), nr - 1);
    return (1.f - a) * K[i0] + a * K[i1];
}

// fmodf(x, y) for 0 <= x < 2^24 and an integer-valued y, given q =
// floor(x / y) (possibly off by one from rounding): x - q*y is exact here
// (q*y is an integer and the difference is a multiple of ulp(x) below y), and
// one correction step lands it in [0, y) -- the value fmodf returns.
__device__ __forceinline__ float fmod_int(float x, float y, float q) {
    float r = fmaf(-q, y, x);
    if (r < 0.f) r += y;
    else if (r >= y) r -= y;
    return r;
}

// One REV sample of the packed pillar grid (cudaBeamletRaytrace,
// device.cu:20-246 with ss_factor 1): the sample's pillar and its pillar
// index coordinate; false for walls, empty pillars and points outside the
// grid (the reference's INVALID density, -1e-12).
__device__ __forceinline__ bool bl_locate(const BlGrid& G, const BlRayDev& R, int tX, int tY, int tZ, int& pidx,
                                          f3& ip) {
    const f3 rv = mk(fmaf(R.rs[0], R.rcp[0], (float)tZ), fmaf(R.rs[1], R.rcp[1], (float)tX),
                     fmaf(R.rs[2], R.rcp[2], (float)tY));
    f3 pb = mv(R.MKi, rv);
    pb = mk(pb.x + 0.5f, pb.y + 0.5f, pb.z + 0.5f);
    if (pb.x < 0.f || pb.y < 0.f || pb.z < 0.f || pb.x >= (float)G.gd[0] || pb.y >= (float)G.gd[1] ||
        pb.z >= (float)G.gd[2])
        return false;
    const float qx = floorf(__fdiv_rn(pb.x, (float)G.pd[0])), qz = floorf(__fdiv_rn(pb.z, (float)G.pd[2]));
    pidx = (int)qx + (int)qz * G.npx;
    if (pidx >= G.n) return false;
    // pb.y < pd.y + wall: fmodf(pb.y, pd.y) is pb.y or pb.y - pd.y (exact)
    const float py = pb.y >= (float)G.pd[1] ? pb.y - (float)G.pd[1] : pb.y;
    ip = mk(fmod_int(pb.x, (float)G.pd[0], qx), py, fmod_int(pb.z, (float)G.pd[2], qz));
    if (ip.x < (float)BL_WALL || ip.y < (float)BL_WALL || ip.z < (float)BL_WALL) return false;
    ip = mk(ip.x - 0.5f, ip.y - 0.5f, ip.z - 0.5f);
    return true;
}

// TERMA point of a sample: pillar index rotated, then scaled, + start
__device__ __forceinline__ f3 bl_terma_point(const BlGrid& G, const BlPillar& Q, f3 ip) {
    const f3 tr = mv(Q.M, ip);
    return mk(fmaf(tr.x, G.vs[0], Q.ps[0]), fmaf(tr.y, G.vs[1], Q.ps[1]), fmaf(tr.z, G.vs[2], Q.ps[2]));
}

constexpr int BL_SAMPLE_BLOCK = 256;

// Can pillar-index point ip lie in the pillar's beamlet?  The footprint's
// cross-section at pillar depth y is inside the box spanned by its four
// corner rays there (a rotation keeps rays straight); 0.05 index units of
// margin keep every point the exact test could accept.
__device__ __forceinline__ bool bl_near_footprint(const BlPillar& Q, f3 ip) {
    float x0 = 1e30f, x1 = -1e30f, z0 = 1e30f, z1 = -1e30f;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const float x = fmaf(Q.sx[c], ip.y, Q.ex[c]), z = fmaf(Q.sz[c], ip.y, Q.ez[c]);
        x0 = fminf(x0, x); x1 = fmaxf(x1, x);
        z0 = fminf(z0, z); z1 = fmaxf(z1, z);
    }
    return ip.x >= x0 - 0.05f && ip.x <= x1 + 0.05f && ip.z >= z0 - 0.05f && ip.z <= z1 + 0.05f;
}

// Pass 1 of a direction, one thread per REV sample (line-contiguous layout):
// the sample's pillar and the beamlet test of its TERMA point -- the exact
// test of the reference only near the footprint.  Samples inside their
// pillar's beamlet are queued for the Siddon pass; nothing else is written
// (density is sampled later, on the lines that carry TERMA).
__global__ void __launch_bounds__(BL_SAMPLE_BLOCK)
    k_bl_samples(EeParams P, const EeBeamSpec* __restrict__ spec, BlGrid G, const BlPillar* __restrict__ pil,
                 BlRayDev R, int* __restrict__ queue, int* __restrict__ qcount) {
    // REV arrays stay below 2^31 samples (checked on the host): 32-bit index
    // arithmetic
    const unsigned n = (unsigned)R.rev[0] * (unsigned)R.rev[1] * (unsigned)R.rev[2];
    const unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    bool in_beamlet = false;
    if (v < n) {
        const unsigned line = v / (unsigned)R.rev[0];
        const int tX = (int)(v - line * (unsigned)R.rev[0]);
        const unsigned zq = line / (unsigned)R.rev[1];
        const int tY = (int)(line - zq * (unsigned)R.rev[1]), tZ = (int)zq;
        int pidx;
        f3 ip;
        if (bl_locate(G, R, tX, tY, tZ, pidx, ip)) {
            const BlPillar& Q = pil[pidx];
            if (bl_near_footprint(Q, ip)) {
                const f3 gt = bl_terma_point(G, Q, ip);
                int bl = beamlet_of(*spec, gt);
                if (bl == -2) bl = beamlet_point_fp64(*spec, (double)gt.x, (double)gt.y, (double)gt.z);
                in_beamlet = bl == Q.fidx;
            }
        }
    }
    // warp-aggregated enqueue
    const unsigned m = __ballot_sync(FULL, in_beamlet);
    if (m) {
        const int lane = threadIdx.x & 31;
        int base = 0;
        if (lane == __ffs(m) - 1) base = atomicAdd(qcount, __popc(m));
        base = __shfl_sync(FULL, base, __ffs(m) - 1);
        if (in_beamlet) queue[base + __popc(m & ((1u << lane) - 1u))] = (int)v;
    }
}

// Density of a sample (pillar index scaled, rotated, + start; the reference's
// INVALID -1e-12 for walls / outside).
__device__ __forceinline__ float bl_density(const EeParams& P, const BlGrid& G, const BlPillar* __restrict__ pil,
                                            const BlRayDev& R, int tX, int tY, int tZ) {
    int pidx;
    f3 ip;
    if (!bl_locate(G, R, tX, tY, tZ, pidx, ip)) return -1e-12f;
    const BlPillar& Q = pil[pidx];
    const f3 gd = mv(Q.M, mk(ip.x * G.vs[0], ip.y * G.vs[1], ip.z * G.vs[2]));
    const f3 g = mk(gd.x + Q.ps[0], gd.y + Q.ps[1], gd.z + Q.ps[2]);
    return tex3D<float>(P.dens_tex, __fdiv_rn(g.x - P.start[0], P.voxel[0]) + 0.5f,
                        __fdiv_rn(g.y - P.start[1], P.voxel[1]) + 0.5f, __fdiv_rn(g.z - P.start[2], P.voxel[2]) + 0.5f);
}

// Pass 2: Siddon radiological path + polyenergetic TERMA of every queued
// sample (one thread each, so the ray traces run lane-dense), and the flag
// of the sample's line.
__global__ void __launch_bounds__(256)
    k_bl_terma(EeParams P, const EeBeamSpec* __restrict__ spec, BlGrid G, const BlPillar* __restrict__ pil,
               BlRayDev R, const float* __restrict__ fluence, const int* __restrict__ queue,
               const int* __restrict__ qcount, float* __restrict__ t_out, unsigned char* __restrict__ line_flag,
               int* __restrict__ status) {
    const int nq = *qcount;
    const EeBeamSpec& S = *spec;
    const f3 src = ld3(S.src);
    bool cap = false;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        const unsigned v = (unsigned)queue[q];
        const unsigned line = v / (unsigned)R.rev[0];
        const int tX = (int)(v - line * (unsigned)R.rev[0]);
        const unsigned zq = line / (unsigned)R.rev[1];
        const int tY = (int)(line - zq * (unsigned)R.rev[1]), tZ = (int)zq;
        int pidx;
        f3 ip;
        if (!bl_locate(G, R, tX, tY, tZ, pidx, ip)) continue;
        const BlPillar& Q = pil[pidx];
        const f3 gt = bl_terma_point(G, Q, ip);
        const float f = __ldg(fluence + Q.fidx);
        if (!(f > 0.f)) continue;
        const float rpl = siddon_rpl(P, gt, src, cap);
        t_out[v] = f * terma_per_fluence(P, rpl, gt, src, S.sad);
        line_flag[line] = 1;
    }
    if (cap) atomicOr(status, 1);
}

// Cumulative kernel at radiological distance r as PackRowConvolve reads it:
// first mean radius >= r, texture-filtered between the two table entries
// (device.cu:326-339).
__device__ __forceinline__ float bl_ck(const float* K, const float* KR, int nr, float r) {
    int lo = 0, hi = nr - 1;  // first index with KR[idx] >= r (r <= KR[nr-1])
    while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (KR[m] < r) lo = m + 1;
        else hi = m;
    }
    if (lo <= 0) return kern_tex(K, nr, 0.5f) * (r * (1.f / KR[0]));
    const float interp = (r - KR[lo - 1]) * (1.f / (KR[lo] - KR[lo - 1]));
    return kern_tex(K, nr, (float)lo - 0.5f + interp);
}

constexpr int BL_MAX_SRC = 1024;

// Pass 3, one warp per flagged line (lines without TERMA keep the zeros the
// dose array was cleared to).  The reference's walk from output i visits
// every sample up to the next wall, adding T_k * (CK(s_k) - CK(s_k')) where
// s_k is the radiological distance between the centres of i and k (half of
// i's own step for k = i) and s_k' that of the previous sample; only samples
// with TERMA contribute.  Here each lane sums those terms directly over the
// line's TERMA samples in i's wall-bounded segment, with the distances from
// a prefix sum of the radiological steps, under the walk's stopping rules
// (the last radius for s_k, the one before it for s_k').
__global__ void __launch_bounds__(BL_WARPS * 32)
    k_bl_walk(EeParams P, BlGrid G, const BlPillar* __restrict__ pil, BlRayDev R, const float* __restrict__ t_in,
              const unsigned char* __restrict__ line_flag, float* __restrict__ rev_dose) {
    extern __shared__ float sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int L = R.rev[0];
    const int nr = P.nradii;
    float* Kf = sm;
    float* Kr = Kf + EE_MAX_RADII;
    float* KR = Kr + EE_MAX_RADII;
    for (int k = threadIdx.x; k < nr; k += blockDim.x) {
        Kf[k] = P.cumkern[R.row_f * nr + k];
        Kr[k] = P.cumkern[R.row_r * nr + k];
        KR[k] = G.kr[k];
    }
    __syncthreads();
    const long long line = (long long)blockIdx.x * BL_WARPS + warp;
    if (line >= (long long)R.rev[1] * R.rev[2] || !line_flag[line]) return;
    // per warp: d[L] (radiological step, -1 for walls), pre[L+1] (prefix of
    // steps), seg[L] (wall count before the sample), src[BL_MAX_SRC]
    float* d = sm + 3 * EE_MAX_RADII + (size_t)warp * (3 * L + 2 + BL_MAX_SRC);
    float* pre = d + L;
    int* seg = (int*)(pre + L + 1);
    int* src = seg + L;
    const int tY = (int)(line % R.rev[1]), tZ = (int)(line / R.rev[1]);
    const float* tl = t_in + (size_t)line * L;
    const float delr = P.lng;
    // prefix sums (steps of walls count 0) and the TERMA-sample list, in
    // ascending order, 32 samples at a time
    float carry = 0.f;
    int wcarry = 0, ns = 0;
    for (int i0 = 0; i0 < L; i0 += 32) {
        const int i = i0 + lane;
        const float rho = i < L ? bl_density(P, G, pil, R, i, tY, tZ) : 0.f;
        const bool wall = i < L && rho < 0.f;
        const float step = (i < L && !wall) ? delr * rho : 0.f;
        float x = step;
        int w = wall ? 1 : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(FULL, x, o);
            const int wy = __shfl_up_sync(FULL, w, o);
            if (lane >= o) { x += y; w += wy; }
        }
        if (i < L) {
            d[i] = wall ? -1.f : step;
            pre[i + 1] = carry + x;
            seg[i] = wcarry + w - (wall ? 1 : 0);
        }
        const bool is_src = i < L && !wall && tl[i] != 0.f;
        const unsigned m = __ballot_sync(FULL, is_src);
        if (is_src) {
            const int p = ns + __popc(m & ((1u << lane) - 1u));
            if (p < BL_MAX_SRC) src[p] = i;
        }
        ns += __popc(m);
        carry = __shfl_sync(FULL, carry + x, 31);
        wcarry = __shfl_sync(FULL, wcarry + w, 31);
    }
    if (lane == 0) pre[0] = 0.f;
    ns = min(ns, BL_MAX_SRC);
    __syncwarp();
    const float rmax = KR[nr - 1], rstop = KR[nr - 2];
    const float nphi = (float)P.nphi;
    float* out = rev_dose + (size_t)line * L;
    for (int i = lane; i < L; i += 32) {
        const float di = d[i];
        if (di < 0.f) continue;  // wall: stays 0
        const float h = 0.5f * di;
        const int si = seg[i];
        float sum = 0.f;
        // backward walk (kernel row P): sources k <= i
        for (int q = 0; q < ns; q++) {
            const int k = src[q];
            if (k > i) break;
            if (seg[k] != si) continue;
            const float tk = tl[k];
            if (k == i) {
                if (h <= rmax) sum += bl_ck(Kf, KR, nr, h) * tk;
                continue;
            }
            const float sk = h + (pre[i] - pre[k + 1]) + 0.5f * d[k];
            const float sp = (k + 1 == i) ? h : h + (pre[i] - pre[k + 2]) + 0.5f * d[k + 1];
            if (sk > rmax || sp > rstop) continue;
            sum += (bl_ck(Kf, KR, nr, sk) - bl_ck(Kf, KR, nr, sp)) * tk;
        }
        // forward walk (kernel row ntheta-1-P): sources k >= i
        for (int q = ns - 1; q >= 0; q--) {
            const int k = src[q];
            if (k < i) break;
            if (seg[k] != si) continue;
            const float tk = tl[k];
            if (k == i) {
                if (h <= rmax) sum += bl_ck(Kr, KR, nr, h) * tk;
                continue;
            }
            const float sk = h + (pre[k] - pre[i + 1]) + 0.5f * d[k];
            const float sp = (k - 1 == i) ? h : h + (pre[k - 1] - pre[i + 1]) + 0.5f * d[k - 1];
            if (sk > rmax || sp > rstop) continue;
            sum += (bl_ck(Kr, KR, nr, sk) - bl_ck(Kr, KR, nr, sp)) * tk;
        }
        out[i] = sum / nphi;
    }
}

// tex3D<float> of a linear-memory volume as the texture unit filters it:
// border addressing, linear filtering with each weight rounded to 8
// fractional bits.  (x, y, z) are texel-space coordinates after the -0.5
// texel-centre shift.  The reference's REV-dose and packed-dose fetches go
// through textures (device.cu:423, 511); exact FP32 weights would move
// beamlet columns by ~0.25% of their maximum.
__device__ __forceinline__ float tri_border_q(const float* __restrict__ v, int nx, int ny, int nz, float x, float y,
                                              float z) {
    if (!(x > -1.f && x < (float)nx && y > -1.f && y < (float)ny && z > -1.f && z < (float)nz)) return 0.f;
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const int i = (int)fx, j = (int)fy, k = (int)fz;
    const float ax = floorf((x - fx) * 256.f + 0.5f) * (1.f / 256.f);
    const float ay = floorf((y - fy) * 256.f + 0.5f) * (1.f / 256.f);
    const float az = floorf((z - fz) * 256.f + 0.5f) * (1.f / 256.f);
    const long long sxy = (long long)nx * ny;
    float acc = 0.f;
#pragma unroll
    for (int dk = 0; dk < 2; dk++) {
        const int kk = k + dk;
        if (kk < 0 || kk >= nz) continue;
        const float wz = dk ? az : 1.f - az;
#pragma unroll
        for (int dj = 0; dj < 2; dj++) {
            const int jj = j + dj;
            if (jj < 0 || jj >= ny) continue;
            const float wy = dj ? ay : 1.f - ay;
            const float* row = v + (long long)nx * jj + sxy * kk;
#pragma unroll
            for (int di = 0; di < 2; di++) {
                const int ii = i + di;
                if (ii < 0 || ii >= nx) continue;
                const float w = (di ? ax : 1.f - ax) * wy * wz;
                if (w != 0.f) acc += w * __ldg(row + ii);
            }
        }
    }
    return acc;
}

// PackedREVtoBEVdose (device.cu:407-431): packed voxel (pX, pY, pZ) += the
// positive trilinear REV dose at its rotated position.  Packed layout: pY
// fastest, then pZ, then pX.
__global__ void __launch_bounds__(256) k_bl_gather(BlGrid G, BlRayDev R, const float* __restrict__ rev_dose,
                                                   float* __restrict__ packed) {
    const unsigned n = (unsigned)G.gd[0] * (unsigned)G.gd[1] * (unsigned)G.gd[2];
    const unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const unsigned r2 = v / (unsigned)G.gd[1];
    const int pY = (int)(v - r2 * (unsigned)G.gd[1]);
    const unsigned r3 = r2 / (unsigned)G.gd[2];
    const int pZ = (int)(r2 - r3 * (unsigned)G.gd[2]), pX = (int)r3;
    const f3 rot = mv(R.MK, mk((float)pX, (float)pY, (float)pZ));
    const float qx = fmaf(-R.rs[0], R.rcp[0], rot.x), qy = fmaf(-R.rs[1], R.rcp[1], rot.y),
                qz = fmaf(-R.rs[2], R.rcp[2], rot.z);
    const float d = tri_border_q(rev_dose, R.rev[0], R.rev[1], R.rev[2], qy, qz, qx);
    if (d > 0.f) packed[v] += d;
}

// ---- unpack (UnpackBEVDosePillar, device.cu:438-521) + sparsification ----
// Pillar-index coordinate of calc-bbox voxel (x, y, z) and the usable-region
// test of the reference.
__device__ __forceinline__ bool bl_unpack_coord(const EeParams& P, const BlGrid& G, const BlPillar& Q, int x, int y,
                                                int z, f3& u) {
    const float gx = ((float)x + (float)P.bb0[0]) * P.voxel[0] + P.start[0];
    const float gy = ((float)y + (float)P.bb0[1]) * P.voxel[1] + P.start[1];
    const float gz = ((float)z + (float)P.bb0[2]) * P.voxel[2] + P.start[2];
    const f3 r = mv(Q.Mi, mk(gx - Q.ps[0], gy - Q.ps[1], gz - Q.ps[2]));
    u = mk(r.x / G.vs[0] + 0.5f, r.y / G.vs[1] + 0.5f, r.z / G.vs[2] + 0.5f);
    const float lo = (float)(BL_WALL + BL_BUF);
    return !(u.x < lo || u.y < lo || u.z < lo || u.x >= (float)(G.pd[0] - BL_BUF) ||
             u.y >= (float)(G.pd[1] - BL_BUF) || u.z >= (float)(G.pd[2] - BL_BUF));
}

__device__ __forceinline__ float bl_unpack_value(const BlGrid& G, const BlPillar& Q, const float* __restrict__ packed,
                                                 f3 u) {
    const float ux = u.x + (float)(Q.ix * G.pd[0]), uz = u.z + (float)(Q.iz * G.pd[2]);
    const float d = tri_border_q(packed, G.gd[1], G.gd[2], G.gd[0], u.y - 0.5f, uz - 0.5f, ux - 0.5f);
    return d > 0.f ? d : 0.f;
}

// Rows (y, z) of each pillar's calc-bbox AABB: conservative x-interval of the
// row inside the pillar's usable region (the region is convex and the
// pillar coordinate is affine along the row).
__global__ void __launch_bounds__(256) k_bl_rows(EeParams P, BlGrid G, const BlPillar* __restrict__ pil,
                                                 int* __restrict__ len, int* __restrict__ xs) {
    const BlPillar& Q = pil[blockIdx.y];
    const int nrows = Q.bn[1] * Q.bn[2];
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
        const int y = Q.b0[1] + r % Q.bn[1], z = Q.b0[2] + r / Q.bn[1];
        f3 u0, u1;
        bl_unpack_coord(P, G, Q, 0, y, z, u0);
        bl_unpack_coord(P, G, Q, 1, y, z, u1);
        const float du[3] = {u1.x - u0.x, u1.y - u0.y, u1.z - u0.z};
        const float uo[3] = {u0.x, u0.y, u0.z};
        float xlo = -1e30f, xhi = 1e30f;
        bool empty = false;
        for (int a = 0; a < 3; a++) {
            const float lo = (float)(BL_WALL + BL_BUF), hi = (float)(G.pd[a] - BL_BUF);
            if (fabsf(du[a]) < 1e-12f) {
                if (uo[a] < lo - 1e-3f || uo[a] > hi + 1e-3f) empty = true;
                continue;
            }
            float t0 = (lo - uo[a]) / du[a], t1 = (hi - uo[a]) / du[a];
            xlo = fmaxf(xlo, fminf(t0, t1));
            xhi = fminf(xhi, fmaxf(t0, t1));
        }
        int a = 0, b = -1;
        if (!empty && xlo <= xhi + 2.f) {
            a = max(Q.b0[0], (int)floorf(xlo) - 1);
            b = min(Q.b0[0] + Q.bn[0] - 1, (int)ceilf(xhi) + 1);
        }
        len[Q.row0 + r] = max(0, b - a + 1);
        xs[Q.row0 + r] = a;
    }
}

// Pillar of a flat unpack row (rows of a pillar are contiguous).
__device__ __forceinline__ int bl_pillar_of(const BlPillar* __restrict__ pil, int n, long long row) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int m = (lo + hi + 1) >> 1;
        if (pil[m].row0 <= row) lo = m;
        else hi = m - 1;
    }
    return lo;
}

// Unpacked values of every candidate voxel (warp per row) and each column's
// maximum (as the ordered bits of a non-negative float).
__global__ void __launch_bounds__(256) k_bl_values(EeParams P, BlGrid G, const BlPillar* __restrict__ pil,
                                                   const float* __restrict__ packed, long long nrows,
                                                   const int* __restrict__ len, const int* __restrict__ xs,
                                                   const long long* __restrict__ seg, float* __restrict__ vals,
                                                   int* __restrict__ colmax) {
    const int lane = threadIdx.x & 31;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long row = w0; row < nrows; row += nw) {
        const int n = len[row];
        if (n == 0) continue;
        const int j = bl_pillar_of(pil, G.n, row);
        const BlPillar& Q = pil[j];
        const long long r = row - Q.row0;
        const int y = Q.b0[1] + (int)(r % Q.bn[1]), z = Q.b0[2] + (int)(r / Q.bn[1]);
        float m = 0.f;
        for (int k = lane; k < n; k += 32) {
            f3 u;
            float v = 0.f;
            if (bl_unpack_coord(P, G, Q, xs[row] + k, y, z, u)) v = bl_unpack_value(G, Q, packed, u);
            vals[seg[row] + k] = v;
            m = fmaxf(m, v);
        }
        for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL, m, o));
        if (lane == 0 && m > 0.f) atomicMax(colmax + j, __float_as_int(m));
    }
}

// Voxels kept by the reference's threshold (value > thresh * column max).
__global__ void __launch_bounds__(256) k_bl_count(BlGrid G, const BlPillar* __restrict__ pil, long long nrows,
                                                  const int* __restrict__ len, const long long* __restrict__ seg,
                                                  const float* __restrict__ vals, const int* __restrict__ colmax,
                                                  float thresh, int* __restrict__ cnt) {
    const int lane = threadIdx.x & 31;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long row = w0; row < nrows; row += nw) {
        const int n = len[row];
        int c = 0;
        if (n > 0) {
            const float cut = thresh * __int_as_float(colmax[bl_pillar_of(pil, G.n, row)]);
            for (int k = lane; k < n; k += 32) c += vals[seg[row] + k] > cut;
            for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(FULL, c, o);
        }
        if (lane == 0) cnt[row] = c;
    }
}

// Sorted CSR write: rows are in (z, y) order within a pillar and x ascends
// along a row, so the full-grid voxel index ascends within each column.
__global__ void __launch_bounds__(256) k_bl_emit(EeParams P, BlGrid G, const BlPillar* __restrict__ pil,
                                                 long long nrows, const int* __restrict__ len,
                                                 const int* __restrict__ xs, const long long* __restrict__ seg,
                                                 const float* __restrict__ vals, const int* __restrict__ colmax,
                                                 float thresh, const long long* __restrict__ off, long long base,
                                                 int* __restrict__ out_rows, float* __restrict__ out_vals) {
    const int lane = threadIdx.x & 31;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long row = w0; row < nrows; row += nw) {
        const int n = len[row];
        if (n == 0) continue;
        const int j = bl_pillar_of(pil, G.n, row);
        const BlPillar& Q = pil[j];
        const long long r = row - Q.row0;
        const int y = Q.b0[1] + (int)(r % Q.bn[1]), z = Q.b0[2] + (int)(r / Q.bn[1]);
        const float cut = thresh * __int_as_float(colmax[j]);
        long long pos = base + off[row];
        for (int k0 = 0; k0 < n; k0 += 32) {
            const int k = k0 + lane;
            const float v = k < n ? vals[seg[row] + k] : 0.f;
            const bool keep = k < n && v > cut;
            const unsigned m = __ballot_sync(FULL, keep);
            if (keep) {
                const long long p = pos + __popc(m & ((1u << lane) - 1u));
                const int x = xs[row] + k;
                out_rows[p] = ((z + P.bb0[2]) * P.size[1] + (y + P.bb0[1])) * P.size[0] + (x + P.bb0[0]);
                out_vals[p] = v;
            }
            pos += __popc(m);
        }
    }
}

// ---- exclusive prefix sum (int -> long long), 1024 elements per block ----
__global__ void __launch_bounds__(1024) k_scan_block(const int* __restrict__ in, const long long* __restrict__ in64,
                                                     long long n, long long* __restrict__ out,
                                                     long long* __restrict__ block_sums) {
    __shared__ long long wsum[32];
    const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long v = i < n ? (in ? (long long)in[i] : in64[i]) : 0;
    long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        long long s = wsum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            long long y = __shfl_up_sync(FULL, s, o);
            if (lane >= o) s += y;
        }
        wsum[lane] = s;
    }
    __syncthreads();
    const long long excl = x - v + (warp ? wsum[warp - 1] : 0);
    if (i < n) out[i] = excl;
    if (threadIdx.x == 1023) block_sums[blockIdx.x] = wsum[31];
}

__global__ void __launch_bounds__(1024) k_scan_add(long long* __restrict__ out, long long n,
                                                   const long long* __restrict__ block_off) {
    const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += block_off[blockIdx.x];
}

// col_ptr[c] = CSR offset of pillar c's first row; col_ptr[n] = batch total.
__global__ void k_bl_colptr(const BlPillar* __restrict__ pil, int n, const long long* __restrict__ off,
                            const int* __restrict__ cnt, long long nrows, long long base, long long* __restrict__ colptr) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) colptr[j] = base + (pil[j].row0 < nrows ? off[pil[j].row0] : (nrows ? off[nrows - 1] + cnt[nrows - 1] : 0));
    if (j == n) colptr[n] = base + (nrows ? off[nrows - 1] + cnt[nrows - 1] : 0);
}

}  // namespace

// ================================================================ host ====
namespace {

template <class T>
struct Dev {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        size_t want = std::max<size_t>(count, 1);
        cudaError_t e = cudaMalloc((void**)&p, want * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
    // grow keeping the first `keep` elements (stream-ordered copy)
    cudaError_t grow_keep(size_t count, size_t keep, cudaStream_t s) {
        if (count <= n && p) return cudaSuccess;
        T* q = nullptr;
        size_t want = std::max<size_t>(std::max(count, n + n / 2), 1);
        cudaError_t e = cudaMalloc((void**)&q, want * sizeof(T));
        if (e != cudaSuccess) return e;
        if (p && keep) e = cudaMemcpyAsync(q, p, keep * sizeof(T), cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (p) cudaFree(p);
        p = q;
        n = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct BlWork {
    Dev<EeBeamSpec> spec;
    Dev<float> fluence, revd, terma, packed, vals, out_vals;
    Dev<unsigned char> line_flag;
    Dev<int> queue, qcount;
    Dev<BlPillar> pil;
    Dev<int> len, xs, cnt, colmax, status, out_rows, out_bidx;
    Dev<long long> seg, off, out_colptr;
    Dev<long long> scan_tmp[6];
    long long nnz = 0;
    int ncols = 0;
    void release() {
        spec.release(); fluence.release(); revd.release(); terma.release(); line_flag.release();
        queue.release(); qcount.release(); packed.release(); vals.release(); out_vals.release();
        pil.release(); len.release(); xs.release(); cnt.release(); colmax.release(); status.release();
        out_rows.release(); out_bidx.release(); seg.release(); off.release(); out_colptr.release();
        for (auto& t : scan_tmp) t.release();
    }
};

#define BL_CUDA(call)                                                                                    \
    do {                                                                                                 \
        cudaError_t _e = (call);                                                                         \
        if (_e != cudaSuccess) return fail_cuda(#call, _e);                                              \
    } while (0)

int fail_cuda(const char* what, cudaError_t e) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s failed: %s", what, cudaGetErrorString(e));
    return ee_internal_fail(EE_ERR_CUDA, buf);
}

// exclusive prefix sum of n ints (or long longs) into out; recursion over the
// per-block totals
cudaError_t scan_excl(BlWork& W, const int* in, const long long* in64, long long n, long long* out, int depth,
                      cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const long long nb = (n + 1023) / 1024;
    cudaError_t e = W.scan_tmp[2 * depth].ensure(nb);
    if (e != cudaSuccess) return e;
    k_scan_block<<<(unsigned)nb, 1024, 0, s>>>(in, in64, n, out, W.scan_tmp[2 * depth].p);
    if (nb == 1) return cudaGetLastError();
    if (2 * depth + 1 >= 6) return cudaErrorInvalidValue;
    if ((e = W.scan_tmp[2 * depth + 1].ensure(nb)) != cudaSuccess) return e;
    if ((e = scan_excl(W, nullptr, W.scan_tmp[2 * depth].p, nb, W.scan_tmp[2 * depth + 1].p, depth + 1, s)) != cudaSuccess)
        return e;
    k_scan_add<<<(unsigned)nb, 1024, 0, s>>>(out, n, W.scan_tmp[2 * depth + 1].p);
    return cudaGetLastError();
}

// last exclusive prefix + last element = total
cudaError_t scan_total(const long long* out, const int* in, long long n, cudaStream_t s, long long* total) {
    *total = 0;
    if (n <= 0) return cudaSuccess;
    long long a = 0;
    int b = 0;
    cudaError_t e = cudaMemcpyAsync(&a, out + n - 1, sizeof(a), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&b, in + n - 1, sizeof(b), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    *total = a + b;
    return e;
}

// allocate_batch_sizes (host.cu:64-76): even split, remainder to the first
std::vector<int> batch_sizes(int n, int nb) {
    std::vector<int> v(nb, n / nb);
    for (int r = n - (n / nb) * nb, k = 0; r > 0; r--) v[(k++) % nb] += 1;
    return v;
}

struct RevBox {
    int size[3];
    v3 mn;
};

// findREV (host.cu:88-155) on the packed grid box [0, gsize]: REV sizes in
// the reference's (line, lateral, lateral) order; false if over max_rev
bool find_rev(v3 gsize, float th, float ph, float lat, float lng, const int max_rev[3], RevBox& R) {
    v3 mn = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(), std::numeric_limits<float>::max()};
    v3 mx = {std::numeric_limits<float>::min(), std::numeric_limits<float>::min(), std::numeric_limits<float>::min()};
    for (int xo = 0; xo < 2; xo++)
        for (int yo = 0; yo < 2; yo++)
            for (int zo = 0; zo < 2; zo++) {
                v3 o = rot_kern({gsize.x * xo, gsize.y * yo, gsize.z * zo}, th, ph);
                mn = {std::min(mn.x, o.x), std::min(mn.y, o.y), std::min(mn.z, o.z)};
                mx = {std::max(mx.x, o.x), std::max(mx.y, o.y), std::max(mx.z, o.z)};
            }
    R.size[0] = (int)(unsigned)std::ceil(std::fabs(mx.y - mn.y) / lng);
    R.size[1] = (int)(unsigned)std::ceil(std::fabs(mx.z - mn.z) / lat);
    R.size[2] = (int)(unsigned)std::ceil(std::fabs(mx.x - mn.x) / lat);
    R.mn = mn;
    return R.size[0] <= max_rev[0] && R.size[1] <= max_rev[1] && R.size[2] <= max_rev[2];
}

}  // namespace

void ee_beamlet_free(void* ws) {
    if (!ws) return;
    BlWork* W = (BlWork*)ws;
    W->release();
    delete W;
}

// Beamlet columns of one beam (dosecalc-beamlet radconvolveTexture,
// nvbbRayConvolve_host.cu:444-1330, one beam).  Outputs stay in the
// workspace; `out` receives device pointers.
int ee_beamlet_run(const EeParams& P, const EeRayConst* rays, cudaStream_t s, void** ws, const EeBeamletOptions& opt,
                   const ee_beam& beam, const EeBeamSpec& S, const float* fluence_host, float thresh, ee_csr* out) {
    if (!*ws) *ws = new BlWork();
    BlWork& W = *(BlWork*)*ws;
    std::memset(out, 0, sizeof(*out));
    W.nnz = 0;
    W.ncols = 0;
    const int fx = beam.fmap_size[0], fy = beam.fmap_size[1];
    // BEAM::reconfigure in FP32 (beam.cpp:300-321)
    const float PI_F = 3.14159265358979323846f;
    float az = fmodf(beam.azimuth, 2 * PI_F), zen = fmodf(beam.zenith, 2 * PI_F);
    auto close = [](float a, float b) { return fabsf(b - a) <= 1e-6f; };
    if (!close(zen, 0.f) && (close(az, 0.f) || close(az, PI_F))) zen = 0.f;
    const float coll = beam.coll;
    const v3 iso = {beam.isocenter[0], beam.isocenter[1], beam.isocenter[2]};
    const v3 src = inv_rot_beam({0.f, -beam.sad, 0.f}, az, zen, 0.f) + iso;
    const v3 voxel = {P.voxel[0], P.voxel[1], P.voxel[2]}, start = {P.start[0], P.start[1], P.start[2]};
    const v3 bb0 = {(float)P.bb0[0], (float)P.bb0[1], (float)P.bb0[2]}, bbs = {(float)P.bbs[0], (float)P.bbs[1], (float)P.bbs[2]};
    const v3 vs = {P.lat, P.lng, P.lat};

    // active beamlets and anchors (host.cu:573-649)
    std::vector<Beamlet> bl;
    for (int i = 0; i < fx * fy; i++)
        if (fluence_host[i] > 0.f) {
            Beamlet B{};
            B.fidx = i;
            if (!anchors(B, src, iso, i, beam.beamlet_size[0], beam.beamlet_size[1], fx, fy, voxel, start, bb0, bbs, az,
                         zen, coll)) {
                char m[160];
                snprintf(m, sizeof(m), "failed to determine beamlet anchor coordinates for beamlet #%d", i);
                return ee_internal_fail(EE_ERR_INVALID_ARG, m);
            }
            bl.push_back(B);
        }
    const int n = (int)bl.size();
    W.ncols = n;
    BL_CUDA(W.out_colptr.ensure((size_t)n + 1));
    BL_CUDA(cudaMemsetAsync(W.out_colptr.p, 0, sizeof(long long) * ((size_t)n + 1), s));
    BL_CUDA(W.out_bidx.ensure(std::max(n, 1)));
    out->nbeamlets = n;
    out->beamlet_index = W.out_bidx.p;
    out->col_ptr = W.out_colptr.p;
    if (n == 0) return EE_OK;
    {
        std::vector<int> h(n);
        for (int i = 0; i < n; i++) h[i] = bl[i].fidx;
        BL_CUDA(cudaMemcpyAsync(W.out_bidx.p, h.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
        BL_CUDA(cudaStreamSynchronize(s));
    }
    float max_len = 0.f, msx = 0.f, msy = 0.f;
    for (auto& B : bl) {
        max_len = std::max(max_len, B.length);
        const float r = len(B.last - src), q = len(B.biso - src);
        msx = std::max(msx, beam.beamlet_size[0] * r / q);
        msy = std::max(msy, beam.beamlet_size[1] * r / q);
    }
    // pillar size: beamlet + 2 kernel extents + a wall, rounded up to whole
    // REV voxels, + the buffers (host.cu:651-662)
    const float ke = opt.kernel_extent;
    const float psl = max_len + 2.f * ke + BL_WALL * vs.y;
    const float ptx = msx + 2.f * ke + BL_WALL * vs.x, pty = msy + 2.f * ke + BL_WALL * vs.x;
    const v3 expand = vs - v3{fmodf(ptx, vs.x), fmodf(psl, vs.y), fmodf(pty, vs.z)};
    const v3 psize = v3{ptx, psl, pty} + expand + vs * (2.f * (float)BL_BUF);
    const int pd[3] = {(int)(psize.x / vs.x), (int)(psize.y / vs.y), (int)(psize.z / vs.z)};
    std::vector<v3> pstart(n);
    std::vector<float> Ms(9 * n), Mis(9 * n);
    for (int i = 0; i < n; i++) {
        const Beamlet& B = bl[i];
        v3 g = {-0.5f * (psize.x + BL_WALL * vs.x), -0.5f * (psize.y - B.length + BL_WALL * vs.y),
                -0.5f * (psize.z + BL_WALL * vs.z)};
        g = inv_rot_beam(inv_rot_beamlet(g, B.th, B.ph), az, zen, coll);
        pstart[i] = B.first + g;
        matrix([&](v3 v) { return inv_rot_beam(inv_rot_beamlet(v, B.th, B.ph), az, zen, coll); }, &Ms[9 * i]);
        matrix([&](v3 v) { return rot_beamlet(rot_beam(v, az, zen, coll), B.th, B.ph); }, &Mis[9 * i]);
    }

    // batching: the fewest batches whose REV arrays all fit max_rev
    // (ArraySizeError re-batching, host.cu:805-819)
    const int nrays = P.nrays;
    int nb = 1;
    std::vector<std::vector<RevBox>> revs;
    for (;; nb++) {
        if (nb > 100) return ee_internal_fail(EE_ERR_REV_SIZE, "beamlet batches exceed the REV size limit");
        std::vector<int> bs = batch_sizes(n, nb);
        revs.assign(nb, std::vector<RevBox>(nrays));
        bool ok = true;
        for (int k = 0; k < nb && ok; k++) {
            const int npx = (int)ceil(sqrt(float(bs[k])));
            const int npz = (int)ceil(float(bs[k]) / npx);
            const v3 gsize = v3{(float)(npx * pd[0] + BL_WALL), (float)(pd[1] + BL_WALL), (float)(npz * pd[2] + BL_WALL)} * vs;
            for (int r = 0; r < nrays && ok; r++) ok = find_rev(gsize, rays[r].th, rays[r].ph, P.lat, P.lng, opt.max_rev, revs[k][r]);
        }
        if (ok) break;
    }
    std::vector<int> bsz = batch_sizes(n, nb);
    for (int k = 0; k < nb; k++)
        for (int r = 0; r < nrays; r++)
            if (revs[k][r].size[0] > EE_MAX_LINE)
                return ee_internal_fail(EE_ERR_REV_SIZE, "size of rev (x-dim) exceeds maximum #threads allowed");

    BL_CUDA(W.spec.ensure(1));
    BL_CUDA(cudaMemcpyAsync(W.spec.p, &S, sizeof(S), cudaMemcpyHostToDevice, s));
    BL_CUDA(W.fluence.ensure((size_t)fx * fy));
    BL_CUDA(cudaMemcpyAsync(W.fluence.p, fluence_host, sizeof(float) * fx * fy, cudaMemcpyHostToDevice, s));
    BL_CUDA(W.status.ensure(1));
    BL_CUDA(cudaMemsetAsync(W.status.p, 0, sizeof(int), s));

    int first = 0;
    for (int k = 0; k < nb; k++) {
        const int m = bsz[k];
        BlGrid G{};
        G.n = m;
        G.npx = (int)ceil(sqrt(float(m)));
        G.npz = (int)ceil(float(m) / G.npx);
        for (int a = 0; a < 3; a++) G.pd[a] = pd[a];
        G.gd[0] = G.npx * pd[0] + BL_WALL;
        G.gd[1] = pd[1] + BL_WALL;
        G.gd[2] = G.npz * pd[2] + BL_WALL;
        G.vs[0] = vs.x; G.vs[1] = vs.y; G.vs[2] = vs.z;
        G.kr[0] = 0.5f * P.radii[0];
        for (int r = 1; r < P.nradii; r++) G.kr[r] = 0.5f * (P.radii[r] + P.radii[r - 1]);
        G.kern_extent = ke;
        // pillar table with the calc-bbox AABB of each usable region
        std::vector<BlPillar> pil(m);
        long long rows = 0;
        for (int i = 0; i < m; i++) {
            BlPillar& Q = pil[i];
            const int gi = first + i;
            std::memcpy(Q.M, &Ms[9 * gi], sizeof(Q.M));
            std::memcpy(Q.Mi, &Mis[9 * gi], sizeof(Q.Mi));
            Q.ps[0] = pstart[gi].x; Q.ps[1] = pstart[gi].y; Q.ps[2] = pstart[gi].z;
            Q.fidx = bl[gi].fidx;
            {
                // corner rays of the beamlet's fluence-map cell in pillar
                // index coordinates, ip = Mi ((p - ps) / vs)
                const int bx = Q.fidx % fx, by = Q.fidx / fx;
                const v3 ps = pstart[gi];
                auto to_pil = [&](v3 p) {
                    const v3 q = (p - ps) * v3{1.f / vs.x, 1.f / vs.y, 1.f / vs.z};
                    const float* Mi = Q.Mi;
                    return v3{Mi[0] * q.x + Mi[1] * q.y + Mi[2] * q.z, Mi[3] * q.x + Mi[4] * q.y + Mi[5] * q.z,
                              Mi[6] * q.x + Mi[7] * q.y + Mi[8] * q.z};
                };
                const v3 a = to_pil(src);
                for (int c = 0; c < 4; c++) {
                    const float cx = beam.beamlet_size[0] * (-0.5f * fx + bx + (c & 1));
                    const float cz = beam.beamlet_size[1] * (-0.5f * fy + by + (c >> 1));
                    const v3 corner = iso + inv_rot_beam({cx, 0.f, cz}, az, zen, coll);
                    const v3 e = to_pil(corner) - a;
                    const float sy = std::fabs(e.y) > 1e-12f ? e.y : 1e-12f;
                    Q.sx[c] = e.x / sy;
                    Q.sz[c] = e.z / sy;
                    Q.ex[c] = a.x - Q.sx[c] * a.y;
                    Q.ez[c] = a.z - Q.sz[c] * a.y;
                }
            }
            Q.ix = i % G.npx;
            Q.iz = i / G.npx;
            double lo[3] = {1e30, 1e30, 1e30}, hi[3] = {-1e30, -1e30, -1e30};
            for (int c = 0; c < 8; c++) {
                double u[3];
                for (int a = 0; a < 3; a++)
                    u[a] = (((c >> a) & 1) ? (double)(pd[a] - BL_BUF) : (double)(BL_WALL + BL_BUF)) - 0.5;
                for (int a = 0; a < 3; a++) {
                    double g = Q.ps[a];
                    for (int b2 = 0; b2 < 3; b2++) g += (double)Q.M[3 * a + b2] * u[b2] * (double)(b2 == 1 ? vs.y : vs.x);
                    double t = (g - (double)P.start[a]) / (double)P.voxel[a] - (double)P.bb0[a];
                    lo[a] = std::min(lo[a], t);
                    hi[a] = std::max(hi[a], t);
                }
            }
            for (int a = 0; a < 3; a++) {
                int l = std::max(0, (int)std::floor(lo[a]) - 1), h = std::min(P.bbs[a] - 1, (int)std::ceil(hi[a]) + 1);
                Q.b0[a] = l;
                Q.bn[a] = std::max(0, h - l + 1);
            }
            Q.row0 = rows;
            rows += (long long)Q.bn[1] * Q.bn[2] * (Q.bn[0] > 0 ? 1 : 0);
            if (Q.bn[0] == 0) Q.bn[1] = Q.bn[2] = 0;
        }
        BL_CUDA(W.pil.ensure(m));
        BL_CUDA(cudaMemcpyAsync(W.pil.p, pil.data(), sizeof(BlPillar) * m, cudaMemcpyHostToDevice, s));
        const long long npk = (long long)G.gd[0] * G.gd[1] * G.gd[2];
        BL_CUDA(W.packed.ensure(npk));
        BL_CUDA(cudaMemsetAsync(W.packed.p, 0, sizeof(float) * npk, s));
        long long rmax = 1;
        for (int r = 0; r < nrays; r++)
            rmax = std::max(rmax, (long long)revs[k][r].size[0] * revs[k][r].size[1] * revs[k][r].size[2]);
        if (rmax >= (1ll << 31) || npk >= (1ll << 31))
            return ee_internal_fail(EE_ERR_REV_SIZE, "beamlet REV / packed grid exceeds 2^31 samples");
        BL_CUDA(W.revd.ensure(rmax));
        BL_CUDA(W.terma.ensure(rmax));
        BL_CUDA(W.queue.ensure(rmax));
        BL_CUDA(W.qcount.ensure(1));
        {
            long long lmax = 1;
            for (int r = 0; r < nrays; r++) lmax = std::max(lmax, (long long)revs[k][r].size[1] * revs[k][r].size[2]);
            BL_CUDA(W.line_flag.ensure(lmax));
        }
        // per direction: REV lines, then the gather into the packed grid
        for (int r = 0; r < nrays; r++) {
            const RevBox& RB = revs[k][r];
            BlRayDev R{};
            for (int a = 0; a < 3; a++) R.rev[a] = RB.size[a];
            R.rs[0] = RB.mn.x; R.rs[1] = RB.mn.y; R.rs[2] = RB.mn.z;
            R.rcp[0] = 1.f / vs.x; R.rcp[1] = 1.f / vs.y; R.rcp[2] = 1.f / vs.z;
            std::memcpy(R.MK, rays[r].MK, sizeof(R.MK));
            std::memcpy(R.MKi, rays[r].MKi, sizeof(R.MKi));
            const int kw = r % (P.ntheta / 2);
            R.row_f = kw;
            R.row_r = P.ntheta - kw - 1;
            const long long lines = (long long)R.rev[1] * R.rev[2];
            if (lines == 0 || R.rev[0] == 0) continue;
            const long long nsamp = (long long)R.rev[0] * lines;
            BL_CUDA(cudaMemsetAsync(W.revd.p, 0, sizeof(float) * nsamp, s));
            BL_CUDA(cudaMemsetAsync(W.terma.p, 0, sizeof(float) * nsamp, s));
            BL_CUDA(cudaMemsetAsync(W.line_flag.p, 0, (size_t)lines, s));
            BL_CUDA(cudaMemsetAsync(W.qcount.p, 0, sizeof(int), s));
            k_bl_samples<<<(unsigned)((nsamp + BL_SAMPLE_BLOCK - 1) / BL_SAMPLE_BLOCK), BL_SAMPLE_BLOCK, 0, s>>>(
                P, W.spec.p, G, W.pil.p, R, W.queue.p, W.qcount.p);
            BL_CUDA(cudaGetLastError());
            k_bl_terma<<<152 * 8, 256, 0, s>>>(P, W.spec.p, G, W.pil.p, R, W.fluence.p, W.queue.p, W.qcount.p,
                                               W.terma.p, W.line_flag.p, W.status.p);
            BL_CUDA(cudaGetLastError());
            const size_t smem = sizeof(float) * (3 * EE_MAX_RADII + (size_t)BL_WARPS * (3 * R.rev[0] + 2 + BL_MAX_SRC));
            if (smem > 48 * 1024)
                BL_CUDA(cudaFuncSetAttribute(k_bl_walk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_bl_walk<<<(unsigned)((lines + BL_WARPS - 1) / BL_WARPS), BL_WARPS * 32, smem, s>>>(
                P, G, W.pil.p, R, W.terma.p, W.line_flag.p, W.revd.p);
            BL_CUDA(cudaGetLastError());
            k_bl_gather<<<(unsigned)((npk + 255) / 256), 256, 0, s>>>(G, R, W.revd.p, W.packed.p);
            BL_CUDA(cudaGetLastError());
        }
        // unpack + threshold + CSR
        BL_CUDA(W.len.ensure(std::max(rows, 1ll)));
        BL_CUDA(W.xs.ensure(std::max(rows, 1ll)));
        BL_CUDA(W.cnt.ensure(std::max(rows, 1ll)));
        BL_CUDA(W.seg.ensure(std::max(rows, 1ll)));
        BL_CUDA(W.off.ensure(std::max(rows, 1ll)));
        BL_CUDA(W.colmax.ensure(m));
        BL_CUDA(cudaMemsetAsync(W.colmax.p, 0, sizeof(int) * m, s));
        long long nvals = 0, nnz_b = 0;
        if (rows > 0) {
            k_bl_rows<<<dim3(64, m), 256, 0, s>>>(P, G, W.pil.p, W.len.p, W.xs.p);
            BL_CUDA(cudaGetLastError());
            BL_CUDA(scan_excl(W, W.len.p, nullptr, rows, W.seg.p, 0, s));
            BL_CUDA(scan_total(W.seg.p, W.len.p, rows, s, &nvals));
            BL_CUDA(W.vals.ensure(std::max(nvals, 1ll)));
            const unsigned wblocks = (unsigned)std::min<long long>((rows + 7) / 8, 152ll * 64);
            k_bl_values<<<wblocks, 256, 0, s>>>(P, G, W.pil.p, W.packed.p, rows, W.len.p, W.xs.p, W.seg.p, W.vals.p,
                                                W.colmax.p);
            BL_CUDA(cudaGetLastError());
            k_bl_count<<<wblocks, 256, 0, s>>>(G, W.pil.p, rows, W.len.p, W.seg.p, W.vals.p, W.colmax.p, thresh, W.cnt.p);
            BL_CUDA(cudaGetLastError());
            BL_CUDA(scan_excl(W, W.cnt.p, nullptr, rows, W.off.p, 0, s));
            BL_CUDA(scan_total(W.off.p, W.cnt.p, rows, s, &nnz_b));
            BL_CUDA(W.out_rows.grow_keep((size_t)(W.nnz + nnz_b), (size_t)W.nnz, s));
            BL_CUDA(W.out_vals.grow_keep((size_t)(W.nnz + nnz_b), (size_t)W.nnz, s));
            k_bl_emit<<<wblocks, 256, 0, s>>>(P, G, W.pil.p, rows, W.len.p, W.xs.p, W.seg.p, W.vals.p, W.colmax.p,
                                              thresh, W.off.p, W.nnz, W.out_rows.p, W.out_vals.p);
            BL_CUDA(cudaGetLastError());
        }
        k_bl_colptr<<<(m + 1 + 127) / 128, 128, 0, s>>>(W.pil.p, m, W.off.p, W.cnt.p, rows, W.nnz,
                                                       W.out_colptr.p + first);
        BL_CUDA(cudaGetLastError());
        W.nnz += nnz_b;
        first += m;
    }
    int st = 0;
    BL_CUDA(cudaMemcpyAsync(&st, W.status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    BL_CUDA(cudaStreamSynchronize(s));
    if (st & 1) return ee_internal_fail(EE_ERR_SIDDON_ITER, "Siddon ray trace hit its iteration cap");
    out->nnz = W.nnz;
    out->row_index = W.out_rows.p;
    out->value = W.out_vals.p;
    out->col_ptr = W.out_colptr.p;
    return EE_OK;
}
