// Internal structures shared by the CCCS host code (ee_api.cpp) and the
// sm_103a kernels (ee_kernels.cu).  POD only, identical on host and device.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/ee_cccs.h"

#define EE_MAX_RAYS 64
#define EE_MAX_E 32
#define EE_MAX_RADII 32
#define EE_MAX_THETA 48
#define EE_MAX_LINE 1024  // longest convolution line (reference limit, host.cu:567)

// Per-context constants, passed by value to every kernel.
struct EeParams {
    int size[3];
    float voxel[3];
    float start[3];
    int bb0[3];
    int bbs[3];
    const float* density;  // full grid
    cudaTextureObject_t dens_tex;  // same volume as a 3-D texture: linear filter, border 0,
                                   // unnormalised coordinates (the reference's texDens,
                                   // nvbbRayConvolve_host.cu:229-242)
    int nE;
    float sp_fluence[EE_MAX_E];
    float sp_energy[EE_MAX_E];
    float sp_mu[EE_MAX_E];
    int ntheta, nphi, nradii, nrays;
    float radii[EE_MAX_RADII];
    float lat, lng, penumbra;
    int max_rev[3];
    int mode;                   // ee_kernel_mode
    int ss;                     // TERMA supersampling per axis (1: off)
    const float* cumkern;       // [ntheta][nradii]
    const float* expp;          // [ntheta][4]
    const struct EeRayConst* rays;  // [nrays]
};

// Per-cone constants (angles and rotations), built on the host.
struct EeRayConst {
    float th, ph;
    int row_fwd, row_rev;  // kernel rows for the two walk directions
    float MK[9];           // BEV -> REV   (rotateKernelAtOriginRHS), row-major
    float MKi[9];          // REV -> BEV   (inverseRotateKernelAtOriginRHS)
};

// TERMA boxes, and their unit-TERMA, beamlet-index and gradient companions,
// are stored in 4x4x4 bricks so that the eight corners of a trilinear cell,
// and the cells of neighbouring REV lines, share cache lines whatever the
// cone's direction.  Box element (x, y, z) sits at bx(x) + by(y) + bz(z):
//   bx(x) = (x>>2)*64 + (x&3),  by(y) = (y>>2)*64*nbx + (y&3)*4,
//   bz(z) = (z>>2)*64*nbx*nby + (z&3)*16,   nb* = ceil(n*/4);
// bricks, and so the rows of 4 x-neighbours, start on 256-byte boundaries.
inline __host__ __device__ long long ee_brick_vol(const int tn[3]) {
    return 64ll * ((tn[0] + 3) >> 2) * ((tn[1] + 3) >> 2) * ((tn[2] + 3) >> 2);
}

// The forward gather's warp patch: EE_GATHER_PX x EE_GATHER_PY x EE_GATHER_PZ
// patient voxels (32 lanes); a warp owns a group of PY x PZ patient rows.
constexpr int EE_GATHER_PX = 8, EE_GATHER_PY = 2, EE_GATHER_PZ = 2;
inline __host__ __device__ long long ee_gather_groups(long long ny, long long nz) {
    return ((ny + EE_GATHER_PY - 1) / EE_GATHER_PY) * ((nz + EE_GATHER_PZ - 1) / EE_GATHER_PZ);
}

// Per-beam constants built on the host.
struct EeBeamSpec {
    float src[3];
    float dir[3];          // unit
    float iso[3];
    float az, zen, coll, sad;
    float isodist;         // |iso - src|
    float MB[9];           // RCS -> BEV (rotateBeamAtOriginRHS)
    float MBi[9];          // BEV -> RCS
    int fmap[2];
    float beamlet[2];
    long long fl_off;      // offset of this beam's fluence map
    // TERMA box: axis-aligned patient-index box holding the field frustum
    // (clipped to the calc bbox); TERMA is identically zero outside it.
    int t0[3];             // origin (full-grid voxel index)
    int tn[3];             // size
    long long t_off;       // element offset in the TERMA arena (a multiple of 64: bricks, below)
    // FP64 copies for re-deciding the beamlet of voxels whose FP32 fluence-map
    // coordinate lands within 1e-4 of a beamlet boundary
    double srcd[3];
    double dird[3];
    double MBd[9];
    double isodistd;
    // REV arena slot planned from geometric upper bounds (ee_plan);
    // plan_cap == 0: the arena is sized after the geometry read-back
    long long plan_off;
    long long plan_cap;
    // element offset of this beam's dose (and dose-gradient) volume: grouped
    // outputs of the request server; 0 otherwise
    long long out_off;
};

// Per-cone geometry of one beam, computed on the device.
struct EeRayGeom {
    int rev[3];            // (along-line, lateral-1, lateral-2) sizes
    int nlines;            // rev[1]*rev[2]
    long long offset;      // element offset in the beam's REV arena
    float q0[3];           // rev_min / spacing (reference vector order)
    float G0[3], Gx[3], Gy[3], Gz[3];  // REV (tX,tY,tZ) -> patient voxel index
    float B0[3], Bx[3], By[3], Bz[3];  // REV (tX,tY,tZ) -> BEV crop-box index
    float M[9];            // BEV -> REV (copy of MK for the gather)
    float A[9];            // patient index step -> REV step (MK MB), row-major
};

// Per-beam geometry computed on the device (crop box + REV frames).
struct EeBeamGeom {
    int key_min[3];        // ordered-int keys for atomic min/max
    int key_max[3];
    unsigned int nnz;
    int status;
    float bmin[3];
    int bev[3];
    float lim_off[3];      // (lim_min - start)/voxel
    float lim_min[3];
    long long v_beam;
    long long rev_total;
    int max_line;
    int max_lines;
    // patient rows (y,z) whose voxels can see this beam's REV dose: the AABB
    // of the crop box dilated by 2 voxels, clipped to the calc bbox
    int gy0, gz0, gny, gnz;
    int rows;              // row groups of the forward gather (ee_gather_groups)
    int gx0, gnx;          // x range of the same AABB
    int tiles;             // 8x8x4 patient tiles covering the AABB (adjoint gather)
    long long arena_off;   // element offset of this beam's REV arena
    long long arena_cap;   // elements available to this beam
    EeRayGeom ray[EE_MAX_RAYS];
};

// Launch wrappers implemented in ee_kernels.cu.  All enqueue on `s`.
cudaError_t ee_launch_geom_init(const EeBeamSpec* specs, EeBeamGeom* g, int nbeams, cudaStream_t s);
// unit/beamlet_idx (both optional) receive TERMA per unit fluence of every
// in-field voxel and its beamlet index (adjoint).
cudaError_t ee_launch_terma(const EeParams& P, const EeBeamSpec* specs, EeBeamGeom* geoms, const float* fluence,
                            float* terma, float* unit, int* beamlet_idx, int nbeams, long long max_tvol,
                            cudaStream_t s);
cudaError_t ee_launch_geometry(const EeParams& P, const EeBeamSpec* specs, EeBeamGeom* geoms, int nbeams,
                               cudaStream_t s);
// exp mode writes only each line's valid segment: `rev` must be zeroed;
// `samples` (REV-arena sized float2, exp mode) keeps (rho, T) per sample
// between the two passes; nullptr selects the warp kernel
cudaError_t ee_launch_cone(const EeParams& P, const EeBeamSpec* specs, const EeBeamGeom* geoms, const float* terma,
                           float* rev, float2* samples, int nbeams, int max_lines, int max_line, cudaStream_t s,
                           int lane_block = 128);
// dose_mode 0/1 accumulate atomically into dose (the caller zeroes it for
// mode 0); mode 2 writes dose[b] rows (the caller zeroes the volumes).
cudaError_t ee_launch_gather(const EeParams& P, const EeBeamSpec* specs, const EeBeamGeom* geoms, const float* rev,
                             float* dose, int nbeams, int dose_mode, int max_rows, cudaStream_t s);
// adjoint
cudaError_t ee_launch_gather_T(const EeParams& P, const EeBeamSpec* specs, const EeBeamGeom* geoms,
                               const float* dose_grad, float* rev_grad, int nbeams, int max_tiles, cudaStream_t s);
// scratch: REV-arena sized float2 (exp mode's lane kernel keeps one pass's
// contributions and the samples' density there); nullptr selects the warp
// kernel
cudaError_t ee_launch_cone_T(const EeParams& P, const EeBeamSpec* specs, const EeBeamGeom* geoms, const float* rev_grad,
                             float2* scratch, float* terma_grad, int nbeams, int max_lines, int max_line,
                             cudaStream_t s, int lane_block = 128);
// zeros on every line's segment of a chunk's REV gradient arena (before
// ee_launch_gather_T; the forward cone kernels zero their own arena)
cudaError_t ee_launch_rev_zero(const EeParams& P, const EeBeamGeom* geoms, float* rev_grad, int nbeams, int max_lines,
                               cudaStream_t s);
// test option: EE_DEBUG_POISON=1 fills scratch with NaN where the engine
// relies on its kernels, not on a clear, to write every sample it reads
bool ee_debug_poison();
// per-beam status words of a geometry array (strided copy), for plans
cudaError_t ee_copy_status(const EeBeamGeom* geoms, int* status_host, int nbeams, cudaStream_t s);
cudaError_t ee_launch_terma_T(const EeParams& P, const EeBeamSpec* specs, const EeBeamGeom* geoms,
                              const float* unit_terma, const int* beamlet_idx, const float* terma_grad,
                              float* fluence_grad, int nbeams, long long max_tvol, cudaStream_t s);
// EndtoEnd loss pieces
cudaError_t ee_launch_loss_grad(const float* dose, const float* ptv_w, const float* ptv_t, const float* oar_w,
                                const float* oar_t, float* grad, double* acc, long long n, cudaStream_t s);
cudaError_t ee_launch_spread(const EeBeamSpec* specs, const float* in, float* out, const float* w1d, int R, int nbeams,
                             int max_pix, cudaStream_t s);
cudaError_t ee_launch_smooth(const EeBeamSpec* specs, const float* x, float* grad, float eta, double* acc, int nbeams,
                             int max_pix, cudaStream_t s);

// Beamlet-column path (ee_beamlet.cu).
struct EeBeamletOptions {
    float kernel_extent;  // dose kernel truncation, cm (argparser.h:27: 2 cm)
    int max_rev[3];       // REV size limit that triggers re-batching (argparser.h:29: 500^3)
};
int ee_beamlet_run(const EeParams& P, const EeRayConst* rays, cudaStream_t s, void** ws, const EeBeamletOptions& opt,
                   const ee_beam& beam, const EeBeamSpec& S, const float* fluence_host, float thresh, ee_csr* out);
void ee_beamlet_free(void* ws);
