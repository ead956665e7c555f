// ee_device.cuh -- device helpers shared by the beam-dose kernels
// (ee_kernels.cu) and the beamlet-column kernels (ee_beamlet.cu): vector
// arithmetic, the border-mode trilinear gather, the Siddon radiological path,
// the beamlet lookup and the polyenergetic TERMA of one point.
#pragma once
#include "ee_internal.h"
#include <cfloat>

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ int f2key(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : (i ^ 0x7fffffff);
}
__device__ __forceinline__ float key2f(int k) { return __int_as_float(k >= 0 ? k : (k ^ 0x7fffffff)); }

// ceil() with extents within 1e-3 of an integer snapped to it, so that
// axis-aligned beams (exactly integer crop-box / REV extents) do not flip by
// one voxel with the last bit of the FP32 rotation (the reference's plain
// ceilf at host.cu:469-473, :111-114 is rounding-dependent there).
__device__ __forceinline__ float snap_ceilf(float v) {
    float r = rintf(v);
    return fabsf(v - r) <= 1e-3f ? r : ceilf(v);
}

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ f3 mv(const float* M, f3 v) {
    return {M[0] * v.x + M[1] * v.y + M[2] * v.z, M[3] * v.x + M[4] * v.y + M[5] * v.z,
            M[6] * v.x + M[7] * v.y + M[8] * v.z};
}

// tex3D<float> with linear filtering, unnormalised coordinates and border
// addressing, written as an explicit FP32 trilinear gather.  (x,y,z) are
// texel-space coordinates after the -0.5 texel-centre shift.
__device__ __forceinline__ float tri_border(const float* __restrict__ v, int nx, int ny, int nz, float x, float y,
                                            float z) {
    // all eight texels outside (or a NaN coordinate): the border value 0
    if (!(x > -1.f && x < (float)nx && y > -1.f && y < (float)ny && z > -1.f && z < (float)nz)) return 0.f;
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    int i = (int)fx, j = (int)fy, k = (int)fz;
    float ax = x - fx, ay = y - fy, az = z - fz;
    long long sxy = (long long)nx * ny;
    if (i >= 0 && j >= 0 && k >= 0 && i + 1 < nx && j + 1 < ny && k + 1 < nz) {
        const float* p = v + i + (long long)nx * j + sxy * k;
        float c000 = __ldg(p), c100 = __ldg(p + 1), c010 = __ldg(p + nx), c110 = __ldg(p + nx + 1);
        float c001 = __ldg(p + sxy), c101 = __ldg(p + sxy + 1), c011 = __ldg(p + sxy + nx), c111 = __ldg(p + sxy + nx + 1);
        float c00 = c000 + ax * (c100 - c000), c10 = c010 + ax * (c110 - c010);
        float c01 = c001 + ax * (c101 - c001), c11 = c011 + ax * (c111 - c011);
        float c0 = c00 + ay * (c10 - c00), c1 = c01 + ay * (c11 - c01);
        return c0 + az * (c1 - c0);
    }
    float acc = 0.f;
#pragma unroll
    for (int dk = 0; dk < 2; dk++) {
        int kk = k + dk;
        if (kk < 0 || kk >= nz) continue;
        float wz = dk ? az : 1.f - az;
#pragma unroll
        for (int dj = 0; dj < 2; dj++) {
            int jj = j + dj;
            if (jj < 0 || jj >= ny) continue;
            float wy = dj ? ay : 1.f - ay;
#pragma unroll
            for (int di = 0; di < 2; di++) {
                int ii = i + di;
                if (ii < 0 || ii >= nx) continue;
                float wx = di ? ax : 1.f - ax;
                acc += wx * wy * wz * __ldg(v + ii + (long long)nx * jj + sxy * kk);
            }
        }
    }
    return acc;
}

// Vector reduction of four floats into a 16-byte aligned quad of global
// memory (red.global.add.v4.f32, sm_90+): no value comes back, unlike an
// atomicAdd whose result the caller ignores.
__device__ __forceinline__ void red_v4(float* q, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(q), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}

// Add (a, b) to p[0], p[1] with vector reductions: both land in one 16-byte
// aligned quad unless p sits in its last slot.  The other slots of the quad
// receive +0, so the buffer must hold 3 floats of padding past its last
// element and its base must be 16-byte aligned (cudaMalloc'd).
__device__ __forceinline__ void red_pair(float* p, float a, float b) {
    const uintptr_t u = (uintptr_t)p;
    float* q = (float*)(u & ~(uintptr_t)15);
    const int o = (int)((u >> 2) & 3);
    if (o == 0) red_v4(q, a, b, 0.f, 0.f);
    else if (o == 1) red_v4(q, 0.f, a, b, 0.f);
    else if (o == 2) red_v4(q, 0.f, 0.f, a, b);
    else {
        atomicAdd(p, a);
        atomicAdd(p + 1, b);
    }
}

// ------------------------------------------------ bricked TERMA boxes ----
// Address parts of box element (x, y, z) in the 4x4x4-brick layout
// (ee_brick_vol): the element sits at bk_x(x) + bk_y(y) + bk_z(z).  32-bit:
// ee_set_volume keeps the bricked calc bbox, which bounds every box, below 2^31.
struct Brick {
    int n0, n1, n2;
    int sy, sz;  // 64*nbx, 64*nbx*nby
};
__device__ __forceinline__ Brick brick_of(const int tn[3]) {
    Brick B;
    B.n0 = tn[0]; B.n1 = tn[1]; B.n2 = tn[2];
    B.sy = 64 * ((tn[0] + 3) >> 2);
    B.sz = B.sy * ((tn[1] + 3) >> 2);
    return B;
}
__device__ __forceinline__ int bk_x(int x) { return ((x >> 2) << 6) + (x & 3); }
__device__ __forceinline__ int bk_y(const Brick& B, int y) { return (y >> 2) * B.sy + ((y & 3) << 2); }
__device__ __forceinline__ int bk_z(const Brick& B, int z) { return (z >> 2) * B.sz + ((z & 3) << 4); }

// A cone's REV arrays (dose, dose gradient, cone scratch) are bricked over
// (i, tY, tZ), the sample index along the line fastest: dimensions (rev[0],
// rev[1], rev[2]); ee_brick_vol(rev) cells.  Four consecutive samples of a
// line are one 16-byte brick row, and the 8 x 4 lines of a warp cover two
// whole bricks per quad of samples.
__device__ __forceinline__ Brick rev_brick(int n0, int n1, int n2) {  // n0 = rev[0] (along the line)
    Brick B;
    B.n0 = n0; B.n1 = n1; B.n2 = n2;
    B.sy = 64 * ((n0 + 3) >> 2);
    B.sz = B.sy * ((n1 + 3) >> 2);
    return B;
}
// Offset of line (tY, tZ) in a bricked REV array: its sample i sits at
// rev_line(B, tY, tZ) + bk_x(i).
__device__ __forceinline__ int rev_line(const Brick& B, int tY, int tZ) { return bk_y(B, tY) + bk_z(B, tZ); }

// tri_border on a bricked box: the same weights, products and order, so the
// value is bit-identical to tri_border on the x-fastest box.
__device__ __forceinline__ float tri_brick(const float* __restrict__ v, const Brick& B, float x, float y, float z) {
    if (!(x > -1.f && x < (float)B.n0 && y > -1.f && y < (float)B.n1 && z > -1.f && z < (float)B.n2)) return 0.f;
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    int i = (int)fx, j = (int)fy, k = (int)fz;
    float ax = x - fx, ay = y - fy, az = z - fz;
    if (i >= 0 && j >= 0 && k >= 0 && i + 1 < B.n0 && j + 1 < B.n1 && k + 1 < B.n2) {
        const int x0 = bk_x(i), x1 = bk_x(i + 1), y0 = bk_y(B, j), y1 = bk_y(B, j + 1);
        const int z0 = bk_z(B, k), z1 = bk_z(B, k + 1);
        const float* p0 = v + z0;
        const float* p1 = v + z1;
        float c000 = __ldg(p0 + y0 + x0), c100 = __ldg(p0 + y0 + x1), c010 = __ldg(p0 + y1 + x0),
              c110 = __ldg(p0 + y1 + x1);
        float c001 = __ldg(p1 + y0 + x0), c101 = __ldg(p1 + y0 + x1), c011 = __ldg(p1 + y1 + x0),
              c111 = __ldg(p1 + y1 + x1);
        float c00 = c000 + ax * (c100 - c000), c10 = c010 + ax * (c110 - c010);
        float c01 = c001 + ax * (c101 - c001), c11 = c011 + ax * (c111 - c011);
        float c0 = c00 + ay * (c10 - c00), c1 = c01 + ay * (c11 - c01);
        return c0 + az * (c1 - c0);
    }
    float acc = 0.f;
#pragma unroll
    for (int dk = 0; dk < 2; dk++) {
        int kk = k + dk;
        if (kk < 0 || kk >= B.n2) continue;
        float wz = dk ? az : 1.f - az;
#pragma unroll
        for (int dj = 0; dj < 2; dj++) {
            int jj = j + dj;
            if (jj < 0 || jj >= B.n1) continue;
            float wy = dj ? ay : 1.f - ay;
#pragma unroll
            for (int di = 0; di < 2; di++) {
                int ii = i + di;
                if (ii < 0 || ii >= B.n0) continue;
                float wx = di ? ax : 1.f - ax;
                acc += wx * wy * wz * __ldg(v + bk_x(ii) + bk_y(B, jj) + bk_z(B, kk));
            }
        }
    }
    return acc;
}

// tri_brick for a point the caller has placed in [0, n0) x [0, n1) x [0, n2)
// (B's sizes and brick strides): no entry or lower-bound tests, and the
// corners addressed from the first one by per-axis steps (+1, +4, +16 inside
// a brick; +61, +sy - 12, +sz - 48 across a brick face).  The same loads,
// weights and order as tri_brick.
__device__ __forceinline__ float tri_brick_in(const float* __restrict__ v, const Brick& B, float x, float y, float z) {
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const int i = (int)fx, j = (int)fy, k = (int)fz;
    if (i + 1 < B.n0 && j + 1 < B.n1 && k + 1 < B.n2) {
        const float ax = x - fx, ay = y - fy, az = z - fz;
        const float* p = v + bk_x(i) + bk_y(B, j) + bk_z(B, k);
        const int dx = (i & 3) == 3 ? 61 : 1, dy = (j & 3) == 3 ? B.sy - 12 : 4, dz = (k & 3) == 3 ? B.sz - 48 : 16;
        float c000 = __ldg(p), c100 = __ldg(p + dx), c010 = __ldg(p + dy), c110 = __ldg(p + dy + dx);
        float c001 = __ldg(p + dz), c101 = __ldg(p + dz + dx), c011 = __ldg(p + dz + dy),
              c111 = __ldg(p + dz + dy + dx);
        float c00 = c000 + ax * (c100 - c000), c10 = c010 + ax * (c110 - c010);
        float c01 = c001 + ax * (c101 - c001), c11 = c011 + ax * (c111 - c011);
        float c0 = c00 + ay * (c10 - c00), c1 = c01 + ay * (c11 - c01);
        return c0 + az * (c1 - c0);
    }
    return tri_brick(v, B, x, y, z);  // the last cell of an axis: border corners
}

// Transpose of tri_brick (same weights as tri_border_scatter).  Each (y, z)
// corner row takes one vector reduction on the 16-byte brick row of corner
// i, holding both x corners unless the pair straddles a brick edge (i % 4 ==
// 3), and a second one on slot 0 of the next brick row only then (or when
// corner i is outside the box).  The other slots of a quad receive +0.  No
// branch on the slot, so the lanes of a warp issue the same two reductions.
__device__ __forceinline__ void tri_brick_scatter(float* v, const Brick& B, float x, float y, float z, float g) {
    if (!(x > -1.f && x < (float)B.n0 && y > -1.f && y < (float)B.n1 && z > -1.f && z < (float)B.n2)) return;
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    int i = (int)fx, j = (int)fy, k = (int)fz;
    float ax = x - fx, ay = y - fy, az = z - fz;
    const bool in0 = i >= 0, in1 = i + 1 < B.n0;
    const int o = i & 3;                        // slot of corner i in its brick row
    const bool both = in0 && in1 && o != 3;     // corner i + 1 in the same row
    const int xa = in0 ? (i >> 2) << 6 : 0;     // brick row of corner i
    const int xb = in1 ? ((i + 1) >> 2) << 6 : 0;  // brick row of corner i + 1 (slot 0 unless both)
    // the x weights in the four slots of corner i's brick row, the same for
    // the four corner rows: each row's reduction is w times this pattern
    const float a0 = 1.f - ax;
    const float p0 = o == 0 ? a0 : 0.f, p1 = o == 1 ? a0 : (o == 0 && both ? ax : 0.f);
    const float p2 = o == 2 ? a0 : (o == 1 && both ? ax : 0.f), p3 = o == 3 ? a0 : (o == 2 && both ? ax : 0.f);
#pragma unroll
    for (int dk = 0; dk < 2; dk++) {
        int kk = k + dk;
        if (kk < 0 || kk >= B.n2) continue;
        float wz = dk ? az : 1.f - az;
#pragma unroll
        for (int dj = 0; dj < 2; dj++) {
            int jj = j + dj;
            if (jj < 0 || jj >= B.n1) continue;
            float w = (dj ? ay : 1.f - ay) * wz * g;
            float* row = v + bk_y(B, jj) + bk_z(B, kk);
            if (in0) red_v4(row + xa, w * p0, w * p1, w * p2, w * p3);
            if (in1 && !both) red_v4(row + xb, w * ax, 0.f, 0.f, 0.f);
        }
    }
}

// Transpose of tri_border: atomically scatter g with the trilinear weights,
// x-adjacent corner pairs as one vector reduction (see red_pair).
__device__ __forceinline__ void tri_border_scatter(float* v, int nx, int ny, int nz, float x, float y, float z, float g) {
    if (!(x > -1.f && x < (float)nx && y > -1.f && y < (float)ny && z > -1.f && z < (float)nz)) return;
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    int i = (int)fx, j = (int)fy, k = (int)fz;
    float ax = x - fx, ay = y - fy, az = z - fz;
    long long sxy = (long long)nx * ny;
    const bool in0 = i >= 0, in1 = i + 1 < nx;
#pragma unroll
    for (int dk = 0; dk < 2; dk++) {
        int kk = k + dk;
        if (kk < 0 || kk >= nz) continue;
        float wz = dk ? az : 1.f - az;
#pragma unroll
        for (int dj = 0; dj < 2; dj++) {
            int jj = j + dj;
            if (jj < 0 || jj >= ny) continue;
            float w = (dj ? ay : 1.f - ay) * wz * g;
            float* row = v + (long long)nx * jj + sxy * kk;
            if (in0 && in1) red_pair(row + i, (1.f - ax) * w, ax * w);
            else if (in0) atomicAdd(row + i, (1.f - ax) * w);
            else if (in1) atomicAdd(row + i + 1, ax * w);
        }
    }
}

// ---------------------------------------------------------------- TERMA --
// Radiological path of the ray source -> voxel centre (cudaSiddon.cu:20-115):
// plane crossings advanced from a common a_min, midpoint density samples of
// the border-mode trilinear density at (pos-start)/voxel, segments shorter
// than 1e-3 cm skipped, 5000-iteration cap.
__device__ float siddon_rpl(const EeParams& P, f3 vox, f3 src, bool& iter_cap) {
    const f3 start = mk(P.start[0], P.start[1], P.start[2]);
    const f3 voxel = mk(P.voxel[0], P.voxel[1], P.voxel[2]);
    const f3 end = mk(start.x + P.size[0] * voxel.x, start.y + P.size[1] * voxel.y, start.z + P.size[2] * voxel.z);
    f3 diff = vox - src, sd = start - src, ed = end - src;
    float afx = (sd.x - 0.5f * voxel.x) / diff.x, afy = (sd.y - 0.5f * voxel.y) / diff.y,
          afz = (sd.z - 0.5f * voxel.z) / diff.z;
    float alx = (ed.x + 0.5f * voxel.x) / diff.x, aly = (ed.y + 0.5f * voxel.y) / diff.y,
          alz = (ed.z + 0.5f * voxel.z) / diff.z;
    float a_min = fmaxf(0.f, fmaxf(fmaxf(fminf(afx, alx), fminf(afy, aly)), fminf(afz, alz)));
    float a_max = fminf(1.f, fminf(fminf(fmaxf(afx, alx), fmaxf(afy, aly)), fmaxf(afz, alz)));
    float rpl = 0.f;
    if (!(a_min >= a_max)) {
        float d12 = sqrtf(dot(diff, diff));
        float stx = fabsf(voxel.x / diff.x), sty = fabsf(voxel.y / diff.y), stz = fabsf(voxel.z / diff.z);
        float alpha = a_min, ax = a_min, ay = a_min, az = a_min, next = 0.f;
        const float ivx = 1.f / voxel.x, ivy = 1.f / voxel.y, ivz = 1.f / voxel.z;
        int iter = 0;
        while (alpha < a_max && ++iter < 5000) {
            bool vx = (ax >= 0.f && ax < 1.f), vy = (ay >= 0.f && ay < 1.f), vz = (az >= 0.f && az < 1.f);
            if (!(vx || vy || vz)) break;
            if (vx && (!vy || ax <= ay) && (!vz || ax <= az)) { next = ax; ax += stx; }
            if (vy && (!vx || ay <= ax) && (!vz || ay <= az)) { next = ay; ay += sty; }
            if (vz && (!vx || az <= ax) && (!vy || az <= ay)) { next = az; az += stz; }
            float isect = fabsf(d12 * (next - alpha));
            if (isect >= 0.001f) {
                float mid = (next + alpha) * 0.5f;
                float fx = (src.x + mid * diff.x - start.x) * ivx;
                float fy = (src.y + mid * diff.y - start.y) * ivy;
                float fz = (src.z + mid * diff.z - start.z) * ivz;
                rpl += isect * tex3D<float>(P.dens_tex, fx, fy, fz);
            }
            alpha = next;
        }
        if (iter >= 5000) iter_cap = true;
    }
    return rpl;
}

// The beamlet decision of beamlet_of in FP64 (same formula), for voxels
// whose FP32 fluence-map coordinate is within 1e-4 of a beamlet boundary
// (50x the FP32 error of that coordinate):
// there the FP32 rounding of the projection decides which beamlet (of two
// with different fluence) the voxel takes, and the result would not be
// reproducible.  About two voxels per beam take this path.
__device__ __noinline__ int beamlet_point_fp64(const EeBeamSpec& S, double vx, double vy, double vz) {
    const double dx = vx - S.srcd[0], dy = vy - S.srcd[1], dz = vz - S.srcd[2];
    const double pl = dx * S.dird[0] + dy * S.dird[1] + dz * S.dird[2];
    const double rx = dx - pl * S.dird[0], ry = dy - pl * S.dird[1], rz = dz - pl * S.dird[2];
    const double rl = sqrt(rx * rx + ry * ry + rz * rz);
    if (!(rl > 0.0)) return -1;
    const double prl = fabs(pl);
    const double trad = rl * fabs(S.isodistd / prl);
    const double sc = trad / rl;
    const double px = rx * sc, py = ry * sc, pz = rz * sc;
    const double bx = S.MBd[0] * px + S.MBd[1] * py + S.MBd[2] * pz;
    const double bz = S.MBd[6] * px + S.MBd[7] * py + S.MBd[8] * pz;
    const double fx = bx / (double)S.beamlet[0] + S.fmap[0] * 0.5;
    const double fz = bz / (double)S.beamlet[1] + S.fmap[1] * 0.5;
    if (!(fx >= 0.0 && fx < (double)S.fmap[0] && fz >= 0.0 && fz < (double)S.fmap[1])) return -1;
    const int idx = (int)floor(fx) + S.fmap[0] * (int)floor(fz);
    if (idx < 0 || idx >= S.fmap[0] * S.fmap[1]) return -1;
    return idx;
}

__device__ __forceinline__ int beamlet_of_fp64(const EeParams& P, const EeBeamSpec& S, int x, int y, int z) {
    return beamlet_point_fp64(S, (double)P.start[0] + (double)x * (double)P.voxel[0],
                              (double)P.start[1] + (double)y * (double)P.voxel[1],
                              (double)P.start[2] + (double)z * (double)P.voxel[2]);
}

// Beamlet under this voxel (cudaSiddon.cu:143-165), -1 if none.
__device__ __forceinline__ int beamlet_of(const EeBeamSpec& S, f3 vox) {
    f3 src = ld3(S.src), nd = ld3(S.dir);
    f3 diff = vox - src;
    float pl = dot(diff, nd);
    f3 proj = nd * pl;
    f3 rej = diff - proj;
    float rl = sqrtf(dot(rej, rej));
    if (!(rl > 0.f)) return -1;  // normalize(0) is NaN in the reference: no fluence
    float trad = rl * fabsf(S.isodist / sqrtf(dot(proj, proj)));
    f3 pf = rej * (trad / rl);
    f3 pb = mv(S.MB, pf);
    float fx = pb.x / S.beamlet[0] + S.fmap[0] * 0.5f;
    float fz = pb.z / S.beamlet[1] + S.fmap[1] * 0.5f;
    // near a beamlet boundary (integer coordinate): signal the FP64 path
    if (fabsf(fx - rintf(fx)) < 1e-4f || fabsf(fz - rintf(fz)) < 1e-4f) return -2;
    if (!(fx >= 0.f && fx < (float)S.fmap[0] && fz >= 0.f && fz < (float)S.fmap[1])) return -1;
    int idx = (int)floorf(fx) + S.fmap[0] * (int)floorf(fz);
    if (idx < 0 || idx >= S.fmap[0] * S.fmap[1]) return -1;
    return idx;
}

__device__ __forceinline__ float terma_per_fluence(const EeParams& P, float rpl, f3 vox, f3 src, float sad) {
    float tsum = 0.f;
    for (int e = 0; e < P.nE; e++) {
        float mu = P.sp_mu[e];
        tsum += P.sp_fluence[e] * P.sp_energy[e] * mu * expf(-mu * rpl);
    }
    f3 d = vox - src;
    return tsum * (sad * sad) / dot(d, d);
}

}  // namespace
