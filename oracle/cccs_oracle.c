/*
 * cccs_oracle.c -- CPU restatement of the reference collapsed-cone (CCCS)
 * full-beam dose chain, used ONLY as test infrastructure: the parity checker
 * for the CUDA engine and the timed CPU baseline.  The product never links,
 * loads or calls this file.
 *
 * Compiled twice by oracle/build.py:
 *   ORC_REAL=double -> liboracle64.so  (FP64 oracle: error figures, parity)
 *   ORC_REAL=float  -> liboracle32.so  (FP32 OpenMP CPU baseline)
 *
 * Every stage restates a reference function (paths relative to the
 * reference checkout, CCCS/ prefix):
 *   geometry            CudaUtilities/geometry.cu:46-145
 *   beam source/dir     DoseCalcIO/beam.cpp:92-97,300-321
 *   Siddon raytrace     DoseCalcAlgo/cudaSiddon.cu:20-115
 *   polyenergetic TERMA DoseCalcAlgo/cudaSiddon.cu:117-208 (s=1 path :264-267)
 *   crop box            dosecalc-beam/nvbbRayConvolve_host.cu:429-499
 *   findREV             dosecalc-beam/nvbbRayConvolve_host.cu:75-155
 *   REV resample        dosecalc-beam/nvbbRayConvolve_device.cu:11-80
 *   line convolution    dosecalc-beam/nvbbRayConvolve_device.cu:87-218
 *   REV -> patient      dosecalc-beam/nvbbRayConvolve_device.cu:222-261
 * CUDA texture fetches (unnormalised coordinates, linear filter, border or
 * clamp addressing, CCCS/CudaUtilities/make_tex_surf.cuh:102-124) are
 * emulated in software; with tex_emulate=1 the filter weights are rounded to
 * the 8 fractional bits that the CUDA Programming Guide documents for the
 * texture unit's linear filter.
 *
 * kernel_mode selects the line-convolution kernel:
 *   0  cumulative-kernel table with linear interpolation between radial
 *      boundaries (what the reference does with tex2D)                    -- walk
 *   1  exact double-exponential cumulative kernel K(r)=A/a(1-e^-ar)+B/b(1-e^-br)
 *      evaluated on the same walk (same truncation)                        -- walk
 *   2  the same discrete operator as mode 1 computed with the O(L) affine
 *      recurrence (no radial truncation)                                    -- scan
 *
 * The adjoint (orc_beam_dose_adjoint) is the exact transpose of the linear
 * map fluence -> dose with the crop box held at the one the given fluence
 * produces.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORC_REAL
#define ORC_REAL double
#endif
typedef ORC_REAL real;

#define ORC_MAX_RAYS 256
#define ORC_MAX_RADII 64
#define ORC_PI 3.14159265358979323846

enum { ORC_OK = 0, ORC_ERR_ARG = 1, ORC_ERR_CROPBOX = 2, ORC_ERR_REVSIZE = 3, ORC_ERR_ITER = 4 };

typedef struct {
    int    size[3];
    double voxel[3];
    double start[3];
    int    bbox_start[3];
    int    bbox_size[3];
    const float *density;
    int    nE;
    const double *energy, *fluence, *mu, *mu_en;
    int    ntheta, nphi, nradii;
    const double *radii;
    const double *cumkern;     /* [ntheta][nradii] */
    const double *exp_params;  /* [ntheta][4] */
    const double *theta_deg;   /* [nrays] */
    const double *phi_deg;     /* [nrays] */
    int    kernel_mode;
    double rev_latspacing, rev_longspacing, penumbra;
    int    max_rev_size[3];
    int    tex_emulate;
    int    nthreads;
    int    ss_factor;   /* TERMA supersampling per axis (omni-header ss_factor); <= 1: off */
} orc_setup;

typedef struct {
    double azimuth, zenith, coll;
    double iso[3];
    double sad;
    int    fmap[2];
    double beamlet[2];
} orc_beam;

typedef struct {
    double source[3];
    double direction[3];
    double azimuth, zenith;
    double b_min[3];
    double b_max[3];
    int    bev_size[3];
    double lim_min[3];
    int    nrays;
    int    rev_size[ORC_MAX_RAYS][3];
    double rev_min[ORC_MAX_RAYS][3];
    long   v_beam;
    long   n_terma_nonzero;
    int    status;
} orc_beam_info;

typedef struct { real x, y, z; } r3;
static inline r3 mk3(real x, real y, real z) { r3 v = {x, y, z}; return v; }
static inline r3 add3(r3 a, r3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline r3 sub3(r3 a, r3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline r3 scl3(r3 a, real s) { return mk3(a.x * s, a.y * s, a.z * s); }
static inline real dot3(r3 a, r3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline real len3(r3 a) { return (real)sqrt((double)dot3(a, a)); }
static inline r3 nrm3(r3 a) { real il = (real)(1.0 / sqrt((double)dot3(a, a))); return scl3(a, il); }

/* ---------------- geometry: CudaUtilities/geometry.cu:46-145 ---------------- */
/* Rodrigues rotation of p about unit axis r by angle t (geometry.cu:46-58). */
static r3 rot_axis(r3 p, r3 r, real t) {
    real s = (real)sin((double)t), c = (real)cos((double)t);
    real d = -r.x * p.x - r.y * p.y - r.z * p.z;
    return mk3((-r.x * d) * (1 - c) + p.x * c + (-r.z * p.y + r.y * p.z) * s,
               (-r.y * d) * (1 - c) + p.y * c + (r.z * p.x - r.x * p.z) * s,
               (-r.z * d) * (1 - c) + p.z * c + (-r.y * p.x + r.x * p.y) * s);
}
/* RCS -> BEV (geometry.cu:69-75) */
static r3 rot_beam(r3 v, real az, real zen, real coll) {
    r3 ax = mk3((real)sin(-(double)zen), 0, (real)cos(-(double)zen));
    r3 t = rot_axis(v, ax, -az);
    return rot_axis(t, mk3(0, 1, 0), zen + coll);
}
/* BEV -> RCS (geometry.cu:85-92) */
static r3 inv_rot_beam(r3 v, real az, real zen, real coll) {
    r3 t = rot_axis(v, mk3(0, 1, 0), -(zen + coll));
    r3 ax = mk3((real)sin(-(double)zen), 0, (real)cos(-(double)zen));
    return rot_axis(t, ax, az);
}
/* BEV -> REV (geometry.cu:126-131) */
static r3 rot_kern(r3 v, real th, real ph) {
    r3 ax = mk3((real)cos((double)ph), 0, -(real)sin((double)ph));
    r3 u = rot_axis(v, ax, -th);
    return rot_axis(u, mk3(0, 1, 0), -ph);
}
/* REV -> BEV (geometry.cu:140-145) */
static r3 inv_rot_kern(r3 v, real th, real ph) {
    r3 u = rot_axis(v, mk3(0, 1, 0), ph);
    r3 ax = mk3((real)cos((double)ph), 0, -(real)sin((double)ph));
    return rot_axis(u, ax, th);
}

/* exported for host-side geometry tests */
void orc_rotate(int which, const double *in, double az_or_th, double zen_or_ph, double coll, double *out) {
    r3 v = mk3((real)in[0], (real)in[1], (real)in[2]), o;
    switch (which) {
        case 0: o = rot_beam(v, (real)az_or_th, (real)zen_or_ph, (real)coll); break;
        case 1: o = inv_rot_beam(v, (real)az_or_th, (real)zen_or_ph, (real)coll); break;
        case 2: o = rot_kern(v, (real)az_or_th, (real)zen_or_ph); break;
        default: o = inv_rot_kern(v, (real)az_or_th, (real)zen_or_ph); break;
    }
    out[0] = o.x; out[1] = o.y; out[2] = o.z;
}

static int closeto(double a, double b) { return fabs(b - a) <= 1e-6; }

/* BEAM::reconfigure, ANGLE branch (beam.cpp:300-321) with
 * calc_source_from_angles (beam.cpp:92-97). */
static void beam_reconfigure(const orc_beam *b, r3 *src, r3 *dir, real *az, real *zen) {
    double a = fmod(b->azimuth, 2 * ORC_PI), z = fmod(b->zenith, 2 * ORC_PI);
    if (!closeto(z, 0.0) && (closeto(a, 0.0) || closeto(a, ORC_PI))) z = 0.0;
    r3 iso = mk3((real)b->iso[0], (real)b->iso[1], (real)b->iso[2]);
    *src = add3(inv_rot_beam(mk3(0, (real)-b->sad, 0), (real)a, (real)z, 0), iso);
    *dir = nrm3(sub3(iso, *src));
    *az = (real)a; *zen = (real)z;
}

/* ---------------- texture emulation ---------------- */
/* emulate: 0 exact weights, 1 rounded to 8 fractional bits, 2 truncated to
 * 8 fractional bits (the two readings of the texture unit's 9-bit fixed
 * point weight with 8 fractional bits) */
static inline real quant_w(real a, int emulate) {
    if (!emulate) return a;
    if (emulate == 2) return (real)(floor((double)a * 256.0) / 256.0);
    return (real)(floor((double)a * 256.0 + 0.5) / 256.0);
}
/* tex3D<float>, unnormalised coordinates, linear filter, border address
 * mode (zero outside), applied to a float volume. */
static real tex3d_border_f(const float *vol, const int n[3], real x, real y, real z, int emu) {
    real xb = x - (real)0.5, yb = y - (real)0.5, zb = z - (real)0.5;
    real fx = (real)floor((double)xb), fy = (real)floor((double)yb), fz = (real)floor((double)zb);
    int i = (int)fx, j = (int)fy, k = (int)fz;
    real ax = quant_w(xb - fx, emu), ay = quant_w(yb - fy, emu), az = quant_w(zb - fz, emu);
    real acc = 0;
    for (int dk = 0; dk < 2; dk++) {
        int kk = k + dk; if (kk < 0 || kk >= n[2]) continue;
        real wz = dk ? az : 1 - az;
        for (int dj = 0; dj < 2; dj++) {
            int jj = j + dj; if (jj < 0 || jj >= n[1]) continue;
            real wy = dj ? ay : 1 - ay;
            for (int di = 0; di < 2; di++) {
                int ii = i + di; if (ii < 0 || ii >= n[0]) continue;
                real wx = di ? ax : 1 - ax;
                acc += wx * wy * wz * (real)vol[ii + (long)n[0] * (jj + (long)n[1] * kk)];
            }
        }
    }
    return acc;
}
static real tex3d_border_r(const real *vol, const int n[3], real x, real y, real z, int emu) {
    real xb = x - (real)0.5, yb = y - (real)0.5, zb = z - (real)0.5;
    real fx = (real)floor((double)xb), fy = (real)floor((double)yb), fz = (real)floor((double)zb);
    int i = (int)fx, j = (int)fy, k = (int)fz;
    real ax = quant_w(xb - fx, emu), ay = quant_w(yb - fy, emu), az = quant_w(zb - fz, emu);
    real acc = 0;
    for (int dk = 0; dk < 2; dk++) {
        int kk = k + dk; if (kk < 0 || kk >= n[2]) continue;
        real wz = dk ? az : 1 - az;
        for (int dj = 0; dj < 2; dj++) {
            int jj = j + dj; if (jj < 0 || jj >= n[1]) continue;
            real wy = dj ? ay : 1 - ay;
            for (int di = 0; di < 2; di++) {
                int ii = i + di; if (ii < 0 || ii >= n[0]) continue;
                real wx = di ? ax : 1 - ax;
                acc += wx * wy * wz * vol[ii + (long)n[0] * (jj + (long)n[1] * kk)];
            }
        }
    }
    return acc;
}
/* Transpose of tex3d_border_r: scatter g with the same weights. */
static void tex3d_border_scatter(real *vol, const int n[3], real x, real y, real z, int emu, real g) {
    real xb = x - (real)0.5, yb = y - (real)0.5, zb = z - (real)0.5;
    real fx = (real)floor((double)xb), fy = (real)floor((double)yb), fz = (real)floor((double)zb);
    int i = (int)fx, j = (int)fy, k = (int)fz;
    real ax = quant_w(xb - fx, emu), ay = quant_w(yb - fy, emu), az = quant_w(zb - fz, emu);
    for (int dk = 0; dk < 2; dk++) {
        int kk = k + dk; if (kk < 0 || kk >= n[2]) continue;
        real wz = dk ? az : 1 - az;
        for (int dj = 0; dj < 2; dj++) {
            int jj = j + dj; if (jj < 0 || jj >= n[1]) continue;
            real wy = dj ? ay : 1 - ay;
            for (int di = 0; di < 2; di++) {
                int ii = i + di; if (ii < 0 || ii >= n[0]) continue;
                real wx = di ? ax : 1 - ax;
                real *p = &vol[ii + (long)n[0] * (jj + (long)n[1] * kk)];
                real v = wx * wy * wz * g;
#ifdef _OPENMP
#pragma omp atomic
#endif
                *p += v;
            }
        }
    }
}

/* ---------------- Siddon + TERMA: DoseCalcAlgo/cudaSiddon.cu ---------------- */
/* cudaRaytrace_device (cudaSiddon.cu:20-115).  Density is sampled through a
 * border-mode linear texture at (pos-start)/voxel, i.e. without the +0.5
 * texel-centre offset used elsewhere (cudaSiddon.cu:104-108). */
static real siddon_rpl(const orc_setup *S, r3 vox, r3 start, r3 end, r3 voxel, r3 src, int *iter_err) {
    r3 diff = sub3(vox, src), sd = sub3(start, src), ed = sub3(end, src);
    real afx = (sd.x - (real)0.5 * voxel.x) / diff.x, afy = (sd.y - (real)0.5 * voxel.y) / diff.y,
         afz = (sd.z - (real)0.5 * voxel.z) / diff.z;
    real alx = (ed.x + (real)0.5 * voxel.x) / diff.x, aly = (ed.y + (real)0.5 * voxel.y) / diff.y,
         alz = (ed.z + (real)0.5 * voxel.z) / diff.z;
    real aminx = fmin(afx, alx), amaxx = fmax(afx, alx);
    real aminy = fmin(afy, aly), amaxy = fmax(afy, aly);
    real aminz = fmin(afz, alz), amaxz = fmax(afz, alz);
    real a_min = fmax(0, fmax(fmax(aminx, aminy), aminz));
    real a_max = fmin(1, fmin(fmin(amaxx, amaxy), amaxz));
    real rpl = 0;
    if (!(a_min >= a_max)) {
        real d12 = len3(diff);
        real stx = (real)fabs((double)(voxel.x / diff.x));
        real sty = (real)fabs((double)(voxel.y / diff.y));
        real stz = (real)fabs((double)(voxel.z / diff.z));
        real alpha = a_min, ax = a_min, ay = a_min, az = a_min, next = 0;
        int iter = 0;
        while (alpha < a_max && ++iter < 5000) {
            int vx = (ax >= 0 && ax < 1), vy = (ay >= 0 && ay < 1), vz = (az >= 0 && az < 1);
            if (!(vx || vy || vz)) break;
            if (vx && (!vy || ax <= ay) && (!vz || ax <= az)) { next = ax; ax += stx; }
            if (vy && (!vx || ay <= ax) && (!vz || ay <= az)) { next = ay; ay += sty; }
            if (vz && (!vx || az <= ax) && (!vy || az <= ay)) { next = az; az += stz; }
            real isect = (real)fabs((double)(d12 * (next - alpha)));
            if (isect >= (real)0.001) {
                real mid = (next + alpha) * (real)0.5;
                real fxx = (src.x + mid * diff.x - start.x) / voxel.x;
                real fyy = (src.y + mid * diff.y - start.y) / voxel.y;
                real fzz = (src.z + mid * diff.z - start.z) / voxel.z;
                rpl += isect * tex3d_border_f(S->density, S->size, fxx, fyy, fzz, S->tex_emulate);
            }
            alpha = next;
        }
        if (iter >= 5000) *iter_err = 1;
    }
    return rpl;
}

/* Geometric part of cudaSiddon_device (cudaSiddon.cu:143-165): the beamlet
 * index this voxel projects onto, or -1. */
static int siddon_beamlet(const orc_beam *b, r3 vox, r3 src, r3 dir, real az, real zen) {
    r3 diff = sub3(vox, src);
    r3 nd = nrm3(dir);
    r3 proj = scl3(nd, dot3(diff, nd));
    r3 rej = sub3(diff, proj);
    r3 iso = mk3((real)b->iso[0], (real)b->iso[1], (real)b->iso[2]);
    real rl = len3(rej);
    if (!(rl > 0)) return -1; /* normalize(0) is NaN in the reference: no fluence */
    real trad = rl * (real)fabs((double)(len3(sub3(iso, src)) / len3(proj)));
    r3 pf = scl3(scl3(rej, 1 / rl), trad);
    pf = rot_beam(pf, az, zen, (real)b->coll);
    real fx = pf.x / (real)b->beamlet[0] + (real)b->fmap[0] * (real)0.5;
    real fz = pf.z / (real)b->beamlet[1] + (real)b->fmap[1] * (real)0.5;
    if (fx < 0 || fx >= (real)b->fmap[0] || fz < 0 || fz >= (real)b->fmap[1]) return -1;
    long idx = (long)floor((double)fx) + (long)b->fmap[0] * (long)floor((double)fz);
    if (idx < 0 || idx >= (long)b->fmap[0] * b->fmap[1]) return -1;
    return (int)idx;
}

/* TERMA per unit fluence (cudaSiddon.cu:182-203, beamhard_correct = 1 as
 * forced at dosecalc-beam/nvbbRayConvolve_host.cu:204). */
static real terma_unit(const orc_setup *S, real rpl, r3 vox, r3 src, real sad) {
    real tsum = 0;
    for (int e = 0; e < S->nE; e++) {
        real mu = (real)S->mu[e];
        tsum += (real)S->fluence[e] * (real)S->energy[e] * mu * (real)exp(-(double)(mu * rpl));
    }
    real l = len3(sub3(vox, src));
    real invsq = (sad * sad) / (l * l);
    return tsum * invsq;
}

typedef struct {
    r3 start, end, voxel;
} frame_t;
static frame_t make_frame(const orc_setup *S) {
    frame_t f;
    f.start = mk3((real)S->start[0], (real)S->start[1], (real)S->start[2]);
    f.voxel = mk3((real)S->voxel[0], (real)S->voxel[1], (real)S->voxel[2]);
    f.end = mk3(f.start.x + (real)S->size[0] * f.voxel.x, f.start.y + (real)S->size[1] * f.voxel.y,
                f.start.z + (real)S->size[2] * f.voxel.z);
    return f;
}

/* cudaSiddon over the calc bbox (cudaSiddon.cu:210-308).
 * unit != NULL additionally receives the TERMA per unit fluence and
 * beamlet != NULL the beamlet index of every bbox voxel (adjoint; only
 * without supersampling).  With ss_factor > 1 each voxel's TERMA is the mean
 * over ss^3 sub-voxel centres start + (i - 1/2) voxel + (s + 1/2) voxel/ss,
 * each traced and looked up in the fluence map on its own, summed in the
 * sub-voxel order x fastest (cudaSiddon.cu:248-258, 297-306). */
static int compute_terma(const orc_setup *S, const orc_beam *b, const float *fluence, real *terma,
                         real *unit, int *beamlet, r3 src, r3 dir, real az, real zen) {
    frame_t F = make_frame(S);
    const int bx = S->bbox_size[0], by = S->bbox_size[1], bz = S->bbox_size[2];
    long nv = (long)bx * by * bz;
    int iter_err = 0;
    const int ss = S->ss_factor > 1 ? S->ss_factor : 1;
    if (ss > 1 && (unit || beamlet)) return ORC_ERR_ARG;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(S->nthreads) reduction(|| : iter_err)
#endif
    for (long v = 0; v < nv; v++) {
        int x = (int)(v % bx), y = (int)((v / bx) % by), z = (int)(v / ((long)bx * by));
        r3 vox = mk3(F.start.x + (real)(S->bbox_start[0] + x) * F.voxel.x,
                     F.start.y + (real)(S->bbox_start[1] + y) * F.voxel.y,
                     F.start.z + (real)(S->bbox_start[2] + z) * F.voxel.z);
        real t = 0, u = 0;
        if (ss > 1) {
            const int nsub = ss * ss * ss;
            const r3 sv = mk3(F.voxel.x / (real)ss, F.voxel.y / (real)ss, F.voxel.z / (real)ss);
            real acc = 0;
            for (int ii = 0; ii < nsub; ii++) {
                const int sx = ii % ss, sy = (ii / ss) % ss, sz = ii / (ss * ss);
                r3 p = mk3(F.start.x + ((real)(S->bbox_start[0] + x) - (real)0.5) * F.voxel.x + ((real)sx + (real)0.5) * sv.x,
                           F.start.y + ((real)(S->bbox_start[1] + y) - (real)0.5) * F.voxel.y + ((real)sy + (real)0.5) * sv.y,
                           F.start.z + ((real)(S->bbox_start[2] + z) - (real)0.5) * F.voxel.z + ((real)sz + (real)0.5) * sv.z);
                int bs = siddon_beamlet(b, p, src, dir, az, zen);
                if (bs < 0) continue;
                real fl = (real)fluence[bs];
                if (!(fl > 0)) continue;
                int ie = 0;
                real rpl = siddon_rpl(S, p, F.start, F.end, F.voxel, src, &ie);
                iter_err = iter_err || ie;
                acc += fl * terma_unit(S, rpl, p, src, (real)b->sad);
            }
            terma[v] = acc / (real)nsub;
            continue;
        }
        int bl = siddon_beamlet(b, vox, src, dir, az, zen);
        if (beamlet) beamlet[v] = bl;
        if (bl >= 0) {
            real fl = (real)fluence[bl];
            if (fl > 0 || unit) {
                int ie = 0;
                real rpl = siddon_rpl(S, vox, F.start, F.end, F.voxel, src, &ie);
                iter_err = iter_err || ie;
                u = terma_unit(S, rpl, vox, src, (real)b->sad);
                if (fl > 0) t = fl * u;
            }
        }
        terma[v] = t;
        if (unit) unit[v] = u;
    }
    return iter_err ? ORC_ERR_ITER : ORC_OK;
}

/* ---------------- crop box + findREV ---------------- */
static void ray_angles(const orc_setup *S, int ray, real *th, real *ph) {
    *th = (real)(S->theta_deg[ray] * ORC_PI / 180.0);
    *ph = (real)(S->phi_deg[ray] * ORC_PI / 180.0);
}

/* ceil() of a non-negative extent with values within 1e-3 of an integer
 * snapped to that integer.  The reference takes a plain ceilf of FP32 rotated
 * extents (host.cu:469-473, :111-114); for axis-aligned beams the exact
 * extent is an integer and its ceil then depends on the last bit of the
 * rotation, moving the crop-box face by one voxel (a dose discontinuity of a
 * few % of Dmax at that face).  Snapping makes the result independent of
 * the arithmetic precision; the engine does the same. */
static double snap_ceil(double v) {
    double r = floor(v + 0.5);
    if (fabs(v - r) <= 1e-3) return r;
    return ceil(v);
}

/* nvbbRayConvolve_host.cu:429-499 and findREV :75-155 (REV_PAD = 0). */
static int compute_geometry(const orc_setup *S, const orc_beam *b, const real *terma, real az, real zen,
                            orc_beam_info *info) {
    const int bx = S->bbox_size[0], by = S->bbox_size[1], bz = S->bbox_size[2];
    /* b_max starts at the smallest positive float, as in the reference
     * (std::numeric_limits<float>::min(), nvbbRayConvolve_host.cu:436). */
    double mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {FLT_MIN, FLT_MIN, FLT_MIN};
    long nnz = 0;
    for (int z = 0; z < bz; z++)
        for (int y = 0; y < by; y++)
            for (int x = 0; x < bx; x++) {
                long v = x + (long)bx * (y + (long)by * z);
                if (terma[v] != 0) {
                    r3 bi = rot_beam(mk3((real)x, (real)y, (real)z), az, zen, (real)b->coll);
                    nnz++;
                    mn[0] = fmin(mn[0], bi.x); mn[1] = fmin(mn[1], bi.y); mn[2] = fmin(mn[2], bi.z);
                    mx[0] = fmax(mx[0], bi.x); mx[1] = fmax(mx[1], bi.y); mx[2] = fmax(mx[2], bi.z);
                }
            }
    info->n_terma_nonzero = nnz;
    double pl = S->penumbra / S->rev_latspacing, plong = S->penumbra / S->rev_longspacing;
    mn[0] -= pl; mn[1] -= plong; mn[2] -= pl;
    mx[0] += pl; mx[1] += plong; mx[2] += pl;
    for (int a = 0; a < 3; a++) {
        info->b_min[a] = mn[a];
        info->b_max[a] = mx[a];
        double s = snap_ceil(fabs(mx[a] - mn[a]));
        if (!(s > 0) || s >= 1000.0) { info->status = ORC_ERR_CROPBOX; return ORC_ERR_CROPBOX; }
        info->bev_size[a] = (int)s;
    }
    info->v_beam = (long)info->bev_size[0] * info->bev_size[1] * info->bev_size[2];
    r3 tmn = inv_rot_beam(mk3((real)mn[0], (real)mn[1], (real)mn[2]), az, zen, (real)b->coll);
    info->lim_min[0] = S->start[0] + ((double)tmn.x + S->bbox_start[0]) * S->voxel[0];
    info->lim_min[1] = S->start[1] + ((double)tmn.y + S->bbox_start[1]) * S->voxel[1];
    info->lim_min[2] = S->start[2] + ((double)tmn.z + S->bbox_start[2]) * S->voxel[2];

    int nrays = S->nphi * (S->ntheta / 2);
    if (nrays > ORC_MAX_RAYS) return ORC_ERR_ARG;
    info->nrays = nrays;
    double lat = S->rev_latspacing, lng = S->rev_longspacing;
    r3 bd = mk3((real)(info->bev_size[0] * lat), (real)(info->bev_size[1] * lng), (real)(info->bev_size[2] * lat));
    for (int ray = 0; ray < nrays; ray++) {
        real th, ph;
        ray_angles(S, ray, &th, &ph);
        double rmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rmx[3] = {FLT_MIN, FLT_MIN, FLT_MIN};
        for (int xo = 0; xo < 2; xo++)
            for (int yo = 0; yo < 2; yo++)
                for (int zo = 0; zo < 2; zo++) {
                    r3 o = rot_kern(mk3(bd.x * xo, bd.y * yo, bd.z * zo), th, ph);
                    rmn[0] = fmin(rmn[0], o.x); rmn[1] = fmin(rmn[1], o.y); rmn[2] = fmin(rmn[2], o.z);
                    rmx[0] = fmax(rmx[0], o.x); rmx[1] = fmax(rmx[1], o.y); rmx[2] = fmax(rmx[2], o.z);
                }
        int sz[3] = {(int)snap_ceil(fabs(rmx[1] - rmn[1]) / lng), (int)snap_ceil(fabs(rmx[2] - rmn[2]) / lat),
                     (int)snap_ceil(fabs(rmx[0] - rmn[0]) / lat)};
        for (int a = 0; a < 3; a++) {
            if (S->max_rev_size[a] > 0 && sz[a] > S->max_rev_size[a]) { info->status = ORC_ERR_REVSIZE; return ORC_ERR_REVSIZE; }
            info->rev_size[ray][a] = sz[a];
            info->rev_min[ray][a] = rmn[a];
        }
    }
    info->status = ORC_OK;
    return ORC_OK;
}

/* ---------------- REV resample: nvbbRayConvolve_device.cu:11-80 ---------------- */
typedef struct {
    r3 revq0;      /* rev_min / rev_voxelsize */
    real th, ph, az, zen, coll;
    r3 bev_size;   /* float */
    r3 lim_off;    /* (lim_min - start) / voxel */
    r3 bb0, bb1;   /* calc bbox [start, end) in voxel indices */
} rayframe_t;

static rayframe_t make_rayframe(const orc_setup *S, const orc_beam *b, const orc_beam_info *info, int ray, real az, real zen) {
    rayframe_t R;
    ray_angles(S, ray, &R.th, &R.ph);
    R.az = az; R.zen = zen; R.coll = (real)b->coll;
    R.revq0 = mk3((real)(info->rev_min[ray][0] / S->rev_latspacing), (real)(info->rev_min[ray][1] / S->rev_longspacing),
                  (real)(info->rev_min[ray][2] / S->rev_latspacing));
    R.bev_size = mk3((real)info->bev_size[0], (real)info->bev_size[1], (real)info->bev_size[2]);
    R.lim_off = mk3((real)((info->lim_min[0] - S->start[0]) / S->voxel[0]), (real)((info->lim_min[1] - S->start[1]) / S->voxel[1]),
                    (real)((info->lim_min[2] - S->start[2]) / S->voxel[2]));
    R.bb0 = mk3((real)S->bbox_start[0], (real)S->bbox_start[1], (real)S->bbox_start[2]);
    R.bb1 = mk3((real)(S->bbox_start[0] + S->bbox_size[0]), (real)(S->bbox_start[1] + S->bbox_size[1]),
                (real)(S->bbox_start[2] + S->bbox_size[2]));
    return R;
}

/* REV sample (tX,tY,tZ) -> patient voxel index coordinate; returns 0 if
 * valid, -3 outside the BEV crop box, -2 outside the calc bbox. */
static int rev_to_patient(const rayframe_t *R, int tX, int tY, int tZ, r3 *g) {
    r3 q = add3(R->revq0, mk3((real)tZ, (real)tX, (real)tY));
    r3 bi = inv_rot_kern(q, R->th, R->ph);
    if (bi.x < 0 || bi.y < 0 || bi.z < 0 || bi.x >= R->bev_size.x || bi.y >= R->bev_size.y || bi.z >= R->bev_size.z) return -3;
    *g = add3(R->lim_off, inv_rot_beam(bi, R->az, R->zen, R->coll));
    if (g->x < R->bb0.x || g->x >= R->bb1.x || g->y < R->bb0.y || g->y >= R->bb1.y || g->z < R->bb0.z || g->z >= R->bb1.z) return -2;
    return 0;
}

/* ---------------- line convolution: nvbbRayConvolve_device.cu:87-218 ---------------- */
static inline real cumkern_table(const orc_setup *S, int row, int rad_start, real interp) {
    /* tex2D(kernTex, rad_start - 0.5 + interp, row + 0.5), clamp, linear
     * filter (device.cu:161,163,202,204). rad_start == 0 uses interp*K[0]. */
    const double *K = S->cumkern + (long)row * S->nradii;
    if (rad_start == 0) return interp * (real)K[0];
    real xb = (real)rad_start - 1 + interp; /* texel-space coordinate */
    real fx = (real)floor((double)xb);
    int i = (int)fx;
    real a = quant_w(xb - fx, S->tex_emulate);
    int i0 = i < 0 ? 0 : (i >= S->nradii ? S->nradii - 1 : i);
    int i1 = i + 1 < 0 ? 0 : (i + 1 >= S->nradii ? S->nradii - 1 : i + 1);
    return (1 - a) * (real)K[i0] + a * (real)K[i1];
}
static inline real cumkern_exp(const orc_setup *S, int row, real r) {
    const double *p = S->exp_params + 4 * (long)row;
    real A = (real)p[0], a = (real)p[1], B = (real)p[2], bb = (real)p[3];
    return A / a * (1 - (real)exp(-(double)(a * r))) + B / bb * (1 - (real)exp(-(double)(bb * r)));
}

/* One directional walk from sample i (step -1: forward kernel row P,
 * step +1: reverse row ntheta-1-P).  When coef != NULL, coef[k] receives
 * the weight of T[k] in the walk's sum (for the adjoint); otherwise returns
 * sum_k w_k T[k]. */
static real walk(const orc_setup *S, const real *dens, const real *terma, int L, int i, int step, int row, real delr, real *coef) {
    const int nr = S->nradii;
    const double *RAD = S->radii;
    real sum = 0, r_eff = 0, delr_eff = 0, cumval = 0, last_cumval = 0, last_rad = 0, next_rad = (real)RAD[0];
    int rad_start = 0, k1 = i;
    do {
        k1 += step;
        if (k1 < 0 || k1 >= L) break;
        delr_eff = delr * dens[k1];
        r_eff += (real)0.5 * delr_eff;
        if (r_eff > (real)RAD[nr - 1]) break;
        while (next_rad < r_eff) {
            if (rad_start == nr - 1) break;
            last_rad = next_rad;
            next_rad = (real)RAD[++rad_start];
        }
        real interp = (r_eff - last_rad) / (next_rad - last_rad);
        if (S->kernel_mode == 0) cumval = cumkern_table(S, row, rad_start, interp);
        else cumval = cumkern_exp(S, row, r_eff);
        real w = cumval - last_cumval;
        if (coef) coef[k1] += w; else sum += w * terma[k1];
        last_cumval = cumval;
        r_eff += (real)0.5 * delr_eff;
    } while (rad_start < nr - 1);
    return sum;
}

/* O(L) affine recurrence for the double-exponential kernel.  For one
 * component (A, a) and the forward direction (contributions from k < i):
 *   D_i = A/a [ Y_i + T_{i-1} (1 - e^{-a p_{i-1}/2}) ]
 *   Y_{i+1} = e^{-a p_i} Y_i + T_{i-1} e^{-a p_i/2} (1 - e^{-a (p_{i-1}+p_i)/2})
 * with p = delr * rho; identical to the walk with K exact and no truncation.
 * Samples with rho < 0 (sentinels) carry p = 0 and T = 0. */
static void scan_dir(const real *p, const real *T, int L, const double *prm, int step, real *out) {
    for (int c = 0; c < 2; c++) {
        real A = (real)prm[2 * c], a = (real)prm[2 * c + 1];
        real Y = 0;
        int i0 = step > 0 ? 0 : L - 1;
        /* prev = index i-1 in walk order */
        for (int n = 0; n < L; n++) {
            int i = i0 + step * n;
            int im1 = i - step, im2 = i - 2 * step;
            real d = 0;
            if (n >= 1) d = T[im1] * (1 - (real)exp(-(double)(a * p[im1] * (real)0.5)));
            out[i] += A / a * (Y + d);
            /* advance Y_i -> Y_{i+1} */
            real Yn = (real)exp(-(double)(a * p[i])) * Y;
            if (n >= 1)
                Yn += T[im1] * (real)exp(-(double)(a * p[i] * (real)0.5)) * (1 - (real)exp(-(double)(a * (p[im1] + p[i]) * (real)0.5)));
            (void)im2;
            Y = Yn;
        }
    }
}
/* Transpose of scan_dir: gT[k] += sum_i W_ik g[i]. */
static void scan_dir_T(const real *p, const real *g, int L, const double *prm, int step, real *gT) {
    /* Forward: out_i = A/a (Y_i + T_{i-1} c_{i-1}),  Y_{i+1} = f_i Y_i + T_{i-1} h_i.
     * Adjoint runs the walk order backwards: Ybar accumulates dOut/dY. */
    for (int c = 0; c < 2; c++) {
        real A = (real)prm[2 * c], a = (real)prm[2 * c + 1];
        real Yb = 0; /* adjoint of Y_{n+1} */
        int i0 = step > 0 ? 0 : L - 1;
        for (int n = L - 1; n >= 0; n--) {
            int i = i0 + step * n;
            int im1 = i - step;
            /* Y_{n+1} = f_i Y_n + T_{im1} h_i */
            if (n >= 1) {
                real h = (real)exp(-(double)(a * p[i] * (real)0.5)) * (1 - (real)exp(-(double)(a * (p[im1] + p[i]) * (real)0.5)));
                gT[im1] += Yb * h;
            }
            real Ybn = Yb * (real)exp(-(double)(a * p[i]));
            /* out_n = A/a (Y_n + T_{im1} c) */
            real go = g[i] * A / a;
            Ybn += go;
            if (n >= 1) gT[im1] += go * (1 - (real)exp(-(double)(a * p[im1] * (real)0.5)));
            Yb = Ybn;
        }
    }
}

/* RowConvolve for one REV row (device.cu:87-218).  dens/terma are the
 * resampled row; out receives the row's dose already divided by nphi. */
static void row_convolve(const orc_setup *S, const real *dens, const real *terma, int L, int P, real *out, real *work) {
    const real delr = (real)S->rev_longspacing;
    const int rowf = P, rowr = S->ntheta - 1 - P;
    if (S->kernel_mode == 2) {
        real *p = work, *T = work + L;
        for (int i = 0; i < L; i++) {
            int ok = dens[i] >= 0;
            p[i] = ok ? delr * dens[i] : 0;
            T[i] = ok ? terma[i] : 0;
            out[i] = 0;
        }
        scan_dir(p, T, L, S->exp_params + 4 * rowf, +1, out);
        scan_dir(p, T, L, S->exp_params + 4 * rowr, -1, out);
        for (int i = 0; i < L; i++) out[i] = dens[i] < 0 ? 0 : out[i] / (real)S->nphi;
        return;
    }
    for (int i = 0; i < L; i++) {
        if (dens[i] < 0) { out[i] = 0; continue; }
        real s = walk(S, dens, terma, L, i, -1, rowf, delr, NULL);
        s += walk(S, dens, terma, L, i, +1, rowr, delr, NULL);
        out[i] = s / (real)S->nphi;
    }
}
/* Transpose of row_convolve: gT receives sum_i W_ik g_i (terma adjoint). */
static void row_convolve_T(const orc_setup *S, const real *dens, const real *g, int L, int P, real *gT, real *work) {
    const real delr = (real)S->rev_longspacing;
    const int rowf = P, rowr = S->ntheta - 1 - P;
    for (int i = 0; i < L; i++) gT[i] = 0;
    if (S->kernel_mode == 2) {
        real *p = work, *gg = work + L;
        for (int i = 0; i < L; i++) {
            p[i] = dens[i] >= 0 ? delr * dens[i] : 0;
            gg[i] = dens[i] >= 0 ? g[i] / (real)S->nphi : 0;
        }
        scan_dir_T(p, gg, L, S->exp_params + 4 * rowf, +1, gT);
        scan_dir_T(p, gg, L, S->exp_params + 4 * rowr, -1, gT);
        for (int i = 0; i < L; i++) if (dens[i] < 0) gT[i] = 0;
        return;
    }
    real *coef = work;
    for (int i = 0; i < L; i++) {
        if (dens[i] < 0 || g[i] == 0) continue;
        for (int k = 0; k < L; k++) coef[k] = 0;
        walk(S, dens, NULL, L, i, -1, rowf, delr, coef);
        walk(S, dens, NULL, L, i, +1, rowr, delr, coef);
        real gi = g[i] / (real)S->nphi;
        for (int k = 0; k < L; k++) gT[k] += coef[k] * gi;
    }
    /* terma at sentinel samples is never written (stays 0) */
    for (int i = 0; i < L; i++) if (dens[i] < 0) gT[i] = 0;
}

/* ---------------- REV -> patient: nvbbRayConvolve_device.cu:222-261 ---------------- */
/* Patient voxel (full-grid index t) -> REV coordinate (r.y along the row). */
static inline r3 patient_to_rev(const orc_setup *S, const rayframe_t *R, const orc_beam_info *info, int tx, int ty, int tz) {
    r3 g = mk3((real)tx * (real)S->voxel[0] + (real)S->start[0], (real)ty * (real)S->voxel[1] + (real)S->start[1],
               (real)tz * (real)S->voxel[2] + (real)S->start[2]);
    r3 d = mk3((g.x - (real)info->lim_min[0]) / (real)S->voxel[0], (g.y - (real)info->lim_min[1]) / (real)S->voxel[1],
               (g.z - (real)info->lim_min[2]) / (real)S->voxel[2]);
    r3 bi = rot_beam(d, R->az, R->zen, R->coll);
    return sub3(rot_kern(bi, R->th, R->ph), R->revq0);
}

/* ---------------- full beam ---------------- */
typedef struct {
    real *dens, *terma, *dose; /* REV arrays [rev.z][rev.y][rev.x] */
} revbuf_t;

static long rev_count(const orc_beam_info *info, int ray) {
    return (long)info->rev_size[ray][0] * info->rev_size[ray][1] * info->rev_size[ray][2];
}

/* Fill REV density/terma for one ray (cudaRaytrace). */
static void rev_resample(const orc_setup *S, const rayframe_t *R, const orc_beam_info *info, int ray, const real *terma, real *rdens, real *rterm) {
    const int rx = info->rev_size[ray][0], ry = info->rev_size[ray][1], rz = info->rev_size[ray][2];
    const int *bs = S->bbox_size;
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static) num_threads(S->nthreads)
#endif
    for (int tZ = 0; tZ < rz; tZ++)
        for (int tY = 0; tY < ry; tY++)
            for (int tX = 0; tX < rx; tX++) {
                long o = tX + (long)rx * (tY + (long)ry * tZ);
                r3 g;
                int st = rev_to_patient(R, tX, tY, tZ, &g);
                if (st < 0) { rdens[o] = (real)st; rterm[o] = 0; continue; }
                rdens[o] = tex3d_border_f(S->density, S->size, g.x + (real)0.5, g.y + (real)0.5, g.z + (real)0.5, S->tex_emulate);
                rterm[o] = tex3d_border_r(terma, bs, g.x - R->bb0.x + (real)0.5, g.y - R->bb0.y + (real)0.5, g.z - R->bb0.z + (real)0.5,
                                          S->tex_emulate);
            }
}

static void rev_convolve(const orc_setup *S, const orc_beam_info *info, int ray, const real *rdens, const real *rterm, real *rdose) {
    const int rx = info->rev_size[ray][0], ry = info->rev_size[ray][1], rz = info->rev_size[ray][2];
    const int P = ray % (S->ntheta / 2);
#ifdef _OPENMP
#pragma omp parallel num_threads(S->nthreads)
#endif
    {
        real *work = (real *)malloc(sizeof(real) * 2 * (size_t)(rx + 1));
#ifdef _OPENMP
#pragma omp for collapse(2) schedule(dynamic, 4)
#endif
        for (int tZ = 0; tZ < rz; tZ++)
            for (int tY = 0; tY < ry; tY++) {
                long o = (long)rx * (tY + (long)ry * tZ);
                row_convolve(S, rdens + o, rterm + o, rx, P, rdose + o, work);
            }
        free(work);
    }
}

static void rev_gather(const orc_setup *S, const rayframe_t *R, const orc_beam_info *info, int ray, const real *rdose, real *dose) {
    const int rn[3] = {info->rev_size[ray][0], info->rev_size[ray][1], info->rev_size[ray][2]};
    const int *b0 = S->bbox_start, *bs = S->bbox_size;
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static) num_threads(S->nthreads)
#endif
    for (int z = 0; z < bs[2]; z++)
        for (int y = 0; y < bs[1]; y++)
            for (int x = 0; x < bs[0]; x++) {
                int tx = b0[0] + x, ty = b0[1] + y, tz = b0[2] + z;
                r3 r = patient_to_rev(S, R, info, tx, ty, tz);
                if (r.y >= (real)rn[0] || r.z >= (real)rn[1] || r.x >= (real)rn[2] || r.x < 0 || r.y < 0 || r.z < 0) continue;
                long t = tx + (long)S->size[0] * (ty + (long)S->size[1] * tz);
                dose[t] += tex3d_border_r(rdose, rn, r.y + (real)0.5, r.z + (real)0.5, r.x + (real)0.5, S->tex_emulate);
            }
}
static void rev_gather_T(const orc_setup *S, const rayframe_t *R, const orc_beam_info *info, int ray, const real *gdose, real *grev) {
    const int rn[3] = {info->rev_size[ray][0], info->rev_size[ray][1], info->rev_size[ray][2]};
    const int *b0 = S->bbox_start, *bs = S->bbox_size;
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static) num_threads(S->nthreads)
#endif
    for (int z = 0; z < bs[2]; z++)
        for (int y = 0; y < bs[1]; y++)
            for (int x = 0; x < bs[0]; x++) {
                int tx = b0[0] + x, ty = b0[1] + y, tz = b0[2] + z;
                r3 r = patient_to_rev(S, R, info, tx, ty, tz);
                if (r.y >= (real)rn[0] || r.z >= (real)rn[1] || r.x >= (real)rn[2] || r.x < 0 || r.y < 0 || r.z < 0) continue;
                long t = tx + (long)S->size[0] * (ty + (long)S->size[1] * tz);
                real g = gdose[t];
                if (g != 0) tex3d_border_scatter(grev, rn, r.y + (real)0.5, r.z + (real)0.5, r.x + (real)0.5, S->tex_emulate, g);
            }
}

static int check_setup(const orc_setup *S) {
    if (!S || !S->density || S->nE <= 0 || S->ntheta <= 0 || S->nphi <= 0 || (S->ntheta & 1)) return ORC_ERR_ARG;
    if (S->nradii <= 0 || S->nradii > ORC_MAX_RADII || !S->radii) return ORC_ERR_ARG;
    if (S->kernel_mode == 0 && !S->cumkern) return ORC_ERR_ARG;
    if (S->kernel_mode != 0 && !S->exp_params) return ORC_ERR_ARG;
    for (int a = 0; a < 3; a++)
        if (S->size[a] <= 0 || S->bbox_size[a] <= 0 || S->bbox_start[a] < 0 || S->bbox_start[a] + S->bbox_size[a] > S->size[a]) return ORC_ERR_ARG;
    return ORC_OK;
}

/* Per-beam TERMA only (bbox-sized output) plus the beam geometry. */
int orc_beam_terma(const orc_setup *S, const orc_beam *b, const float *fluence, real *terma_out, orc_beam_info *info) {
    int st = check_setup(S);
    if (st) return st;
    r3 src, dir; real az, zen;
    beam_reconfigure(b, &src, &dir, &az, &zen);
    memset(info, 0, sizeof(*info));
    info->source[0] = src.x; info->source[1] = src.y; info->source[2] = src.z;
    info->direction[0] = dir.x; info->direction[1] = dir.y; info->direction[2] = dir.z;
    info->azimuth = az; info->zenith = zen;
    st = compute_terma(S, b, fluence, terma_out, NULL, NULL, src, dir, az, zen);
    if (st) return st;
    return compute_geometry(S, b, terma_out, az, zen, info);
}

/* One beam's dose on the full grid (dose_out is overwritten; voxels outside
 * the calc bbox are zero).  terma_out (bbox sized) is optional. */
int orc_beam_dose(const orc_setup *S, const orc_beam *b, const float *fluence, real *dose_out, real *terma_out, orc_beam_info *info) {
    int st = check_setup(S);
    if (st) return st;
    long nb = (long)S->bbox_size[0] * S->bbox_size[1] * S->bbox_size[2];
    long nfull = (long)S->size[0] * S->size[1] * S->size[2];
    real *terma = terma_out ? terma_out : (real *)malloc(sizeof(real) * nb);
    st = orc_beam_terma(S, b, fluence, terma, info);
    for (long i = 0; i < nfull; i++) dose_out[i] = 0;
    if (st) { if (!terma_out) free(terma); return st; }
    long maxrev = 0;
    for (int ray = 0; ray < info->nrays; ray++) if (rev_count(info, ray) > maxrev) maxrev = rev_count(info, ray);
    real *rd = (real *)malloc(sizeof(real) * maxrev), *rt = (real *)malloc(sizeof(real) * maxrev), *ro = (real *)malloc(sizeof(real) * maxrev);
    for (int ray = 0; ray < info->nrays; ray++) {
        rayframe_t R = make_rayframe(S, b, info, ray, (real)info->azimuth, (real)info->zenith);
        rev_resample(S, &R, info, ray, terma, rd, rt);
        rev_convolve(S, info, ray, rd, rt, ro);
        rev_gather(S, &R, info, ray, ro, dose_out);
    }
    free(rd); free(rt); free(ro);
    if (!terma_out) free(terma);
    return ORC_OK;
}

/* Exact transpose of fluence -> dose for the crop box set by `fluence`:
 * fluence_grad[b] = sum_v G_v [beamlet(v)=b] (R^T C^T S^T dose_grad)_v,
 * G_v = TERMA of voxel v per unit fluence (computed for every in-field
 * voxel, whatever its beamlet's current fluence). */
int orc_beam_dose_adjoint(const orc_setup *S, const orc_beam *b, const float *fluence, const real *dose_grad, real *fluence_grad, orc_beam_info *info) {
    int st = check_setup(S);
    if (st) return st;
    long nb = (long)S->bbox_size[0] * S->bbox_size[1] * S->bbox_size[2];
    real *terma = (real *)malloc(sizeof(real) * nb), *unit = (real *)malloc(sizeof(real) * nb), *gterma = (real *)calloc(nb, sizeof(real));
    int *bl = (int *)malloc(sizeof(int) * nb);
    r3 src, dir; real az, zen;
    beam_reconfigure(b, &src, &dir, &az, &zen);
    memset(info, 0, sizeof(*info));
    info->azimuth = az; info->zenith = zen;
    info->source[0] = src.x; info->source[1] = src.y; info->source[2] = src.z;
    info->direction[0] = dir.x; info->direction[1] = dir.y; info->direction[2] = dir.z;
    st = compute_terma(S, b, fluence, terma, unit, bl, src, dir, az, zen);
    if (!st) st = compute_geometry(S, b, terma, az, zen, info);
    int nfm = b->fmap[0] * b->fmap[1];
    for (int i = 0; i < nfm; i++) fluence_grad[i] = 0;
    if (st) { free(terma); free(unit); free(gterma); free(bl); return st; }
    long maxrev = 0;
    for (int ray = 0; ray < info->nrays; ray++) if (rev_count(info, ray) > maxrev) maxrev = rev_count(info, ray);
    real *rd = (real *)malloc(sizeof(real) * maxrev), *rt = (real *)malloc(sizeof(real) * maxrev);
    real *gr = (real *)malloc(sizeof(real) * maxrev), *gt = (real *)malloc(sizeof(real) * maxrev);
    for (int ray = 0; ray < info->nrays; ray++) {
        rayframe_t R = make_rayframe(S, b, info, ray, az, zen);
        const int rx = info->rev_size[ray][0], ry = info->rev_size[ray][1], rz = info->rev_size[ray][2];
        long nr = rev_count(info, ray);
        rev_resample(S, &R, info, ray, terma, rd, rt);
        for (long i = 0; i < nr; i++) gr[i] = 0;
        rev_gather_T(S, &R, info, ray, dose_grad, gr);
        const int P = ray % (S->ntheta / 2);
#ifdef _OPENMP
#pragma omp parallel num_threads(S->nthreads)
#endif
        {
            real *work = (real *)malloc(sizeof(real) * 2 * (size_t)(rx + 1));
#ifdef _OPENMP
#pragma omp for collapse(2) schedule(dynamic, 4)
#endif
            for (int tZ = 0; tZ < rz; tZ++)
                for (int tY = 0; tY < ry; tY++) {
                    long o = (long)rx * (tY + (long)ry * tZ);
                    row_convolve_T(S, rd + o, gr + o, rx, P, gt + o, work);
                }
            free(work);
        }
        /* transpose of the REV terma resample */
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static) num_threads(S->nthreads)
#endif
        for (int tZ = 0; tZ < rz; tZ++)
            for (int tY = 0; tY < ry; tY++)
                for (int tX = 0; tX < rx; tX++) {
                    long o = tX + (long)rx * (tY + (long)ry * tZ);
                    if (gt[o] == 0) continue;
                    r3 g;
                    if (rev_to_patient(&R, tX, tY, tZ, &g) < 0) continue;
                    tex3d_border_scatter(gterma, S->bbox_size, g.x - R.bb0.x + (real)0.5, g.y - R.bb0.y + (real)0.5, g.z - R.bb0.z + (real)0.5,
                                         S->tex_emulate, gt[o]);
                }
    }
    for (long v = 0; v < nb; v++)
        if (bl[v] >= 0) fluence_grad[bl[v]] += unit[v] * gterma[v];
    free(rd); free(rt); free(gr); free(gt);
    free(terma); free(unit); free(gterma); free(bl);
    return ORC_OK;
}

/* 1-D operator access for unit tests: one REV row through row_convolve. */
void orc_row_convolve(const orc_setup *S, const real *dens, const real *terma, int L, int P, real *out) {
    real *work = (real *)malloc(sizeof(real) * 2 * (size_t)(L + 1));
    row_convolve(S, dens, terma, L, P, out, work);
    free(work);
}
void orc_row_convolve_T(const orc_setup *S, const real *dens, const real *g, int L, int P, real *gT) {
    real *work = (real *)malloc(sizeof(real) * (2 * (size_t)L + 2));
    row_convolve_T(S, dens, g, L, P, gT, work);
    free(work);
}
/* ---------------- preprocessing: CCCS/dosecalc-preprocess ---------------- */
/* cudaMakeIsotropicWithLUT / cudaMakeIsotropic + deviceHU2dens
 * (dosecalc-preprocess/kernels.cuh:12-102, cudaMemFunctions.cu:82-176): the
 * CT (HU, x fastest, frame ct_size / ct_voxel) resampled at iso voxel
 * centres (X,Y,Z)*iso_voxel / ct_voxel through a border-0 linear texture,
 * then converted by the sorted LUT (clamped below, linear extrapolation from
 * the last two points above) or, when nlut == 0, by max((HU+1024)/1024,
 * 0.05).  out_size = ceil(ct_voxel*ct_size/iso_voxel) per axis. */
void orc_iso_size(const int ct_size[3], const double ct_voxel[3], double iso_voxel, int out_size[3]) {
    for (int a = 0; a < 3; a++) out_size[a] = (int)ceilf((float)ct_voxel[a] * ((float)ct_size[a] / (float)iso_voxel));
}

int orc_ct_to_density(const float *hu, const int ct_size[3], const double ct_voxel[3], double iso_voxel,
                      const double *lut_hu, const double *lut_dens, int nlut, int tex_emulate, real *out) {
    int os[3];
    orc_iso_size(ct_size, ct_voxel, iso_voxel, os);
    for (int i = 1; i < nlut; i++)
        if (!(lut_hu[i] > lut_hu[i - 1])) return ORC_ERR_ARG;
    const long n = (long)os[0] * os[1] * os[2];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long v = 0; v < n; v++) {
        const int X = (int)(v % os[0]), Y = (int)((v / os[0]) % os[1]), Z = (int)(v / ((long)os[0] * os[1]));
        const real px = (real)X * (real)iso_voxel / (real)ct_voxel[0];
        const real py = (real)Y * (real)iso_voxel / (real)ct_voxel[1];
        const real pz = (real)Z * (real)iso_voxel / (real)ct_voxel[2];
        /* tex3d_border_f takes texture coordinates (before the -0.5 shift) */
        real val = tex3d_border_f(hu, ct_size, px + (real)0.5, py + (real)0.5, pz + (real)0.5, tex_emulate);
        if (nlut > 0) {
            if (val <= lut_hu[0]) val = lut_dens[0];
            else if (val >= lut_hu[nlut - 1])
                val = lut_dens[nlut - 2] + (val - lut_hu[nlut - 2]) * (lut_dens[nlut - 1] - lut_dens[nlut - 2]) /
                                               (lut_hu[nlut - 1] - lut_hu[nlut - 2]);
            else {
                int lo = 0;
                while (lut_hu[lo] < val && lo < nlut - 1) lo++;
                lo--;
                val = lut_dens[lo] + (val - lut_hu[lo]) * (lut_dens[lo + 1] - lut_dens[lo]) / (lut_hu[lo + 1] - lut_hu[lo]);
            }
        } else {
            val = (val + (real)1024) / (real)1024;
            if (val < (real)0.05) val = (real)0.05;
        }
        out[v] = val;
    }
    return ORC_OK;
}

/* cudaRaycast (kernels.cuh:138-224): a fluence pixel is 1 when any of its
 * sub-rays (3x3 at half-beamlet offsets with supersampling, else the centre
 * ray) from the source to three times the bixel centre on the isocentre
 * plane accumulates a positive radiological path through the mask (the
 * Siddon trace of cudaSiddon.cu:20-115 on the mask frame in S). */
int orc_fluence_projection(const orc_setup *S, const orc_beam *b, int supersample, float *fmap) {
    r3 src, dir;
    real az, zen;
    beam_reconfigure(b, &src, &dir, &az, &zen);
    const r3 start = mk3((real)S->start[0], (real)S->start[1], (real)S->start[2]);
    const r3 voxel = mk3((real)S->voxel[0], (real)S->voxel[1], (real)S->voxel[2]);
    const r3 end = mk3(start.x + (real)S->size[0] * voxel.x, start.y + (real)S->size[1] * voxel.y,
                       start.z + (real)S->size[2] * voxel.z);
    const r3 iso = mk3((real)b->iso[0], (real)b->iso[1], (real)b->iso[2]);
    const int fx = b->fmap[0], fy = b->fmap[1], nsub = supersample ? 9 : 1;
    int err = 0;
    for (int Z = 0; Z < fy; Z++)
        for (int X = 0; X < fx; X++) {
            float hit = 0.f;
            for (int k = 0; k < nsub && hit == 0.f; k++) {
                const int sx = supersample ? k % 3 - 1 : 0, sz = supersample ? k / 3 - 1 : 0;
                r3 f = mk3((real)b->beamlet[0] * ((real)X + (real)0.5 * sx - (real)fx * (real)0.5 + (real)0.5), 0,
                           (real)b->beamlet[1] * ((real)Z + (real)0.5 * sz - (real)fy * (real)0.5 + (real)0.5));
                r3 c = add3(inv_rot_beam(f, az, zen, (real)b->coll), iso);
                c = add3(c, mk3((real)1e-9, (real)1e-9, (real)1e-9));
                const r3 sink = add3(src, scl3(sub3(c, src), 3));
                if (siddon_rpl(S, sink, start, end, voxel, src, &err) > 0) hit = 1.f;
            }
            fmap[X + fx * Z] = hit;
        }
    return err ? ORC_ERR_ITER : ORC_OK;
}

/* fmap_post_apertureready (dosecalc-preprocess/fmapProcessing.cpp:33-48):
 * per fluence-map row, the zero pixels between its first and last non-zero
 * pixels are set to fill. */
void orc_aperture_ready(float *fmap, int fx, int fy, float fill) {
    for (int y = 0; y < fy; y++) {
        int a = -1, z = -1;
        for (int x = 0; x < fx; x++)
            if (fmap[fx * y + x] != 0.f) {
                if (a < 0) a = x;
                z = x;
            }
        for (int x = a + 1; a >= 0 && x < z; x++)
            if (fmap[fx * y + x] == 0.f) fmap[fx * y + x] = fill;
    }
}

int orc_sizeof_real(void) { return (int)sizeof(real); }
int orc_sizeof_info(void) { return (int)sizeof(orc_beam_info); }
int orc_sizeof_setup(void) { return (int)sizeof(orc_setup); }
