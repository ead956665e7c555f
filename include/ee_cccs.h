/*
 * ee_cccs.h -- C ABI of the GB300 collapsed-cone convolution/superposition
 * (CCCS) beam-dose engine.
 *
 * Plain C types only: pointers, sizes, POD structs.  Every entry point
 * returns an ee_status (0 = success); ee_last_error() gives the message of
 * the calling thread's last failure.  Nothing here calls exit().
 *
 * Units: centimetres for lengths, radians for beam angles (VarianIEC:
 * azimuth = gantry, zenith = couch, coll = collimator), degrees for the
 * convolution-cone angles, g/cc for density.  Volumes are x-fastest
 * [size[2]][size[1]][size[0]] float32 arrays; `start` is the centre of voxel
 * (0,0,0).
 *
 * Reference interfaces replaced (paths within the reference checkout):
 *   ee_create/ee_set_volume/ee_set_spectrum/ee_set_kernel_table/
 *   ee_set_kernel_exp   <- initCudaConstandTex
 *                          CCCS/dosecalc-beam/nvbbRayConvolve_host.cu:159
 *   ee_beam_dose        <- radconvolveTexture + cuda_sum_device_float_dose
 *                          CCCS/dosecalc-beam/nvbbRayConvolve_host.cu:297,775
 *   ee_destroy          <- freeCudaTexture
 *                          CCCS/dosecalc-beam/nvbbRayConvolve_host.cu:746
 *   ee_beam_dose_adjoint, ee_loss_and_grad, ee_dose_and_adjoint_device
 *                       <- the EndtoEnd forward-dose and fluence-gradient
 *                          calls (README.md:15-22; that source is not in the
 *                          reference snapshot, so only the README defines them)
 */
#ifndef EE_CCCS_H
#define EE_CCCS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EE_ABI_VERSION 1

typedef enum {
    EE_OK = 0,
    EE_ERR_INVALID_ARG = 1,   /* bad pointer / size / order of calls            */
    EE_ERR_CUDA = 2,          /* a CUDA runtime call failed (message has it)    */
    EE_ERR_CROPBOX = 3,       /* empty or oversized beam crop box
                                 (reference: runtime_error, host.cu:494-498)    */
    EE_ERR_REV_SIZE = 4,      /* REV array larger than allowed
                                 (reference: ArraySizeError, host.cu:148-154,
                                  runtime_error for rev.x > 1024, host.cu:567)  */
    EE_ERR_NOMEM = 5,         /* device allocation failed / admission refused  */
    EE_ERR_NOT_READY = 6,     /* volume, spectrum or kernel not set             */
    EE_ERR_SIDDON_ITER = 7,   /* ray trace hit its iteration cap
                                 (reference: assert, cudaSiddon.cu:112)         */
    EE_ERR_CAPACITY = 8,      /* caller-provided scratch too small              */
    EE_ERR_IO = 9             /* input file missing or malformed                */
} ee_status;

/* line-convolution kernel representation */
typedef enum {
    EE_KERNEL_TABLE = 0,  /* cumulative kernel table, linear interpolation in
                             radius: the reference's discretisation           */
    EE_KERNEL_EXP = 1,    /* double exponential A e^{-ar} + B e^{-br} per
                             zenith bin: O(L) recurrence (fast path)          */
    EE_KERNEL_TABLE_WALK = 2 /* the table discretisation evaluated by the
                             reference's step-by-step walk, O(L^2) per line
                             (EE_KERNEL_TABLE evaluates the same sums in
                             O(L * nradii) when nradii is 24)                 */
} ee_kernel_mode;

/* dose output modes for ee_beam_dose* */
typedef enum {
    EE_DOSE_SUM = 0,        /* dose = sum over the given beams (overwrite)   */
    EE_DOSE_ACCUMULATE = 1, /* dose += sum over the given beams              */
    EE_DOSE_PER_BEAM = 2    /* dose[b] = beam b's dose, nbeams full volumes  */
} ee_dose_mode;

typedef struct ee_context ee_context;

/* Frame of reference and calculation bounding box (CONSTANTS fields size,
 * voxel, start, calc_bbox_start, calc_bbox_size;
 * CCCS/include/server/brain_defs.h:38-57). */
typedef struct {
    int   size[3];
    float voxel[3];
    float start[3];
    int   bbox_start[3];
    int   bbox_size[3];
} ee_frame;

/* Convolution parameters (CONSTANTS nphi, ntheta, nradii, rev_latspacing,
 * rev_longspacing, penumbra, max_rev_size; brain_defs.h:14-52). */
typedef struct {
    int   ntheta;
    int   nphi;
    int   nradii;
    float rev_latspacing;
    float rev_longspacing;
    float penumbra;
    int   max_rev_size[3];  /* 0 = derive as the reference does (host.cu:248-258) */
} ee_conv_params;

/* One beam (BEAM, CCCS/DoseCalcIO/beam.h:35-50, angle orientation). */
typedef struct {
    float azimuth;
    float zenith;
    float coll;
    float isocenter[3];
    float sad;
    int   fmap_size[2];
    float beamlet_size[2];
} ee_beam;

/* Per-beam geometry of the last dose call (crop box and REV extents). */
typedef struct {
    float     source[3];
    float     direction[3];
    float     b_min[3];       /* crop box origin, BEV voxel units           */
    int       bev_size[3];    /* crop box size (host.cu:469-473)            */
    float     lim_min[3];     /* crop box origin in RCS cm (host.cu:478)    */
    long long v_beam;         /* bev_size product                           */
    long long rev_samples;    /* sum over cones of REV array sizes          */
    long long terma_nonzero;
    int       max_line;       /* longest convolution line (max rev.x)       */
    int       status;
} ee_beam_info;

/* ---- context ---- */
int         ee_create(int device, ee_context **ctx);
int         ee_destroy(ee_context *ctx);
const char *ee_last_error(void);
int         ee_abi_version(void);

/* ---- set-up (initCudaConstandTex) ---- */
int ee_set_volume(ee_context *ctx, const ee_frame *frame, const float *density_host);
int ee_set_spectrum(ee_context *ctx, int nE, const float *energy, const float *fluence,
                    const float *mu, const float *mu_en);
/* cumkern: [ntheta][nradii] cumulative kernel; theta_deg/phi_deg: per ray
 * (nphi*ntheta/2) cone angles (convolution_{theta,phi}_angles.raw). */
int ee_set_kernel_table(ee_context *ctx, const ee_conv_params *conv, const float *radii,
                        const float *cumkern, const float *theta_deg, const float *phi_deg);
/* params: [ntheta][4] = (A, a, B, b); selects EE_KERNEL_EXP. */
int ee_set_kernel_exp(ee_context *ctx, const float *params);
int ee_set_kernel_mode(ee_context *ctx, int mode);
/* TERMA supersampling (the omni-header ss_factor; cudaSiddon.cu:248-306):
 * each calc-bbox voxel's TERMA is the mean over ss^3 sub-voxel centres, each
 * with its own beamlet lookup and ray trace.  1 (the default) = off; up to 8.
 * Adjoint and loss calls recompute each sub-voxel centre's beamlet and unit
 * TERMA in the TERMA adjoint (a supersampled voxel draws on several
 * beamlets). */
int ee_set_terma_supersampling(ee_context *ctx, int ss_factor);

/* ---- forward dose (radconvolveTexture) ----
 * fluence: concatenation of the beams' fmap_size[0]*fmap_size[1] maps.
 * Host-pointer form: copies in, computes, copies dose out (synchronous). */
int ee_beam_dose(ee_context *ctx, const ee_beam *beams, int nbeams, const float *fluence_host,
                 float *dose_host, int dose_mode);
/* Device-pointer form: d_fluence and d_dose are device buffers; runs on the
 * context stream; returns after enqueueing unless the batch needs a
 * geometry read-back (the plain path does one per batch). */
int ee_beam_dose_device(ee_context *ctx, const ee_beam *beams, int nbeams, const float *d_fluence,
                        float *d_dose, int dose_mode);

/* ---- adjoint: fluence gradient of <dose_grad, dose(fluence)> ----
 * Exact transpose of the forward chain with each beam's crop box held at
 * the one its current fluence produces. */
int ee_beam_dose_adjoint(ee_context *ctx, const ee_beam *beams, int nbeams, const float *fluence_host,
                         const float *dose_grad_host, float *fluence_grad_host);
int ee_beam_dose_adjoint_device(ee_context *ctx, const ee_beam *beams, int nbeams, const float *d_fluence,
                                const float *d_dose_grad, float *d_fluence_grad);

/* Device scratch budget for one chunk of beams (TERMA and REV arenas);
 * larger batches are processed in chunks that fit.  Default 8 GiB. */
int ee_set_scratch_limit(ee_context *ctx, long long bytes);

/* ---- EndtoEnd loss and fluence gradient ----
 * L = sum_i w0_i (d_i - t0_i)^2 + sum_i w_i max(d_i - t_i, 0)^2 + eta sum_k ||D x_k||_1
 * (README.md:20), d = sum_k A_k (G * x_k): A_k the CCCS chain of beam k, G a
 * normalised Gaussian fluence-spread kernel of `spread_sigma` pixels (0 = none,
 * README.md:15-18), D the forward differences along both fluence-map axes
 * (BOO/BOO_QL/CreateDxDyFMO.m).  Weight/target pointers are device arrays of
 * the volume's size; either pair may be NULL. */
typedef struct {
    const float *ptv_weight;
    const float *ptv_target;
    const float *oar_weight;
    const float *oar_target;
    float eta;
    float spread_sigma;
} ee_loss;

/* d_x: the beams' fluence maps (optimisation variable, concatenated);
 * outputs the summed dose, dL/dx and loss_out = {PTV term, OAR term,
 * smoothness term}.  TERMA, crop boxes and REV frames are computed once and
 * shared by the forward and adjoint passes. */
int ee_loss_and_grad(ee_context *ctx, const ee_beam *beams, int nbeams, const float *d_x, const ee_loss *loss,
                     float *d_dose, float *d_xgrad, double loss_out[3]);
/* Forward dose and the adjoint of a caller-given dose gradient in one call
 * (shared TERMA/geometry).  Either output may be NULL. */
int ee_dose_and_adjoint_device(ee_context *ctx, const ee_beam *beams, int nbeams, const float *d_fluence,
                               float *d_dose, int dose_mode, const float *d_dose_grad, float *d_fluence_grad);
/* Host-pointer form of ee_dose_and_adjoint_device (copies in and out, synchronous). */
int ee_dose_and_adjoint(ee_context *ctx, const ee_beam *beams, int nbeams, const float *fluence_host,
                        float *dose_host, int dose_mode, const float *dose_grad_host, float *fluence_grad_host);

/* ---- allocation-free single-beam dose ----
 * No counterpart in the reference: an extra entry point for callers that
 * must not allocate device memory per call (a pre-carved memory pool owned
 * by another allocator, a per-process memory budget, a real-time loop).
 * Same result as ee_beam_dose_device for one beam (dose = that beam's dose on
 * the full grid, overwritten), with all intermediates in a 64 MiB static
 * device array held by every GPU that loads the library; beams whose TERMA
 * box + REV arena exceed it fail with EE_ERR_CAPACITY.  Calls no cudaMalloc /
 * cudaFree.  The context must be set up (ee_set_*, which allocate) first.
 * Calls share the array, so calls that overlap on the GPU race; the first
 * call on a device looks the array's address up and should come before any
 * stream capture.  Every call reads the beam's crop box back to the host and
 * waits for `stream` before it returns.  The call reads the context's
 * density texture and kernel tables on `stream`, so synchronise `stream`
 * before an ee_set_* or ee_destroy of that context.  `stream` is a
 * cudaStream_t (NULL = legacy default). */
int ee_beam_dose_noalloc(ee_context *ctx, const ee_beam *beam, const float *d_fluence, float *d_dose, void *stream);

/* ---- planned batches (CUDA graph) ----
 * ee_plan_create fixes a batch of beams and the device buffers it reads and
 * writes (fluence in, dose out, and optionally dose gradient in / fluence
 * gradient out), sizes every intermediate from geometric upper bounds, runs
 * the batch once to validate them, autotunes the cone kernels' block shape
 * on it and captures the whole forward(+adjoint) chain into one CUDA graph.
 * ee_plan_launch replays that graph on the context stream with no host
 * synchronisation (new fluence / gradient values are read from the same
 * buffers); ee_plan_status then reports per-beam failures. */
typedef struct ee_plan ee_plan;
int ee_plan_create(ee_context *ctx, const ee_beam *beams, int nbeams, const float *d_fluence, float *d_dose,
                   const float *d_dose_grad, float *d_fluence_grad, ee_plan **plan);
int ee_plan_launch(ee_plan *plan);
int ee_plan_status(ee_plan *plan, int *nfailed);
int ee_plan_info(ee_plan *plan, int *lane_block, long long *device_bytes, int *nchunks);
int ee_plan_destroy(ee_plan *plan);

/* ---- beamlet dose columns (dosecalc-beamlet) ----
 * Replaces dosecalc-beamlet's radconvolveTexture (CCCS/dosecalc-beamlet/
 * nvbbRayConvolve_host.cu:444) + the sparsify workers (CCCS/DoseCalcIO/
 * sparse_io.cpp:22-59) for one beam: one column per active beamlet (fluence
 * > 0, fluence-map order), the beamlet's dose on the calc bbox computed in its
 * own pillar (kernel truncated at the kernel extent), entries kept where
 * value > thresh * column max.  Column c holds row_index/value[col_ptr[c] ..
 * col_ptr[c+1]), row_index = full-grid voxel index (x fastest), ascending.
 * The kernel table and cone angles of ee_set_kernel_table are used with the
 * reference's beamlet conventions (mean radii); ee_set_kernel_exp is not. */
typedef struct {
    int              nbeamlets;
    long long        nnz;
    const int       *beamlet_index;  /* [nbeamlets] fluence-map linear index    */
    const long long *col_ptr;        /* [nbeamlets+1]                           */
    const int       *row_index;      /* [nnz]                                   */
    const float     *value;          /* [nnz]                                   */
} ee_csr;
/* kernel_extent_cm (default 2, argparser.h:27) and the REV size limit that
 * splits the beamlets of a beam into batches (default 500^3, argparser.h:29;
 * NULL keeps it). */
int ee_set_beamlet_options(ee_context *ctx, float kernel_extent_cm, const int max_rev_size[3]);
/* Device pointers owned by the context, valid until its next beamlet call. */
int ee_beamlet_columns_device(ee_context *ctx, const ee_beam *beam, const float *fluence_host, float thresh,
                              ee_csr *out);
/* Copies `bytes` of device memory (e.g. the arrays of an ee_csr) to the
 * host, ordered after the context's queued work. */
int ee_copy_to_host(ee_context *ctx, void *dst, const void *src, long long bytes);
/* Host copy.  beamlet_index / col_ptr need fmap_size[0]*fmap_size[1] (+1)
 * entries; row_index / value `capacity` entries.  *nnz and *nbeamlets are
 * always set; EE_ERR_CAPACITY when nnz > capacity (nothing else copied). */
int ee_beamlet_columns(ee_context *ctx, const ee_beam *beam, const float *fluence, float thresh, long long capacity,
                       int *beamlet_index, long long *col_ptr, int *row_index, float *value, long long *nnz,
                       int *nbeamlets);

/* ---- ROI reduction of sparse columns (dosecalc-beamlet, header `reduce`) ----
 * Replaces _reduce_by_roi (CCCS/DoseCalcIO/sparse_io.cpp:62-158), host code
 * as in the reference.  A column's rows are kept only where the voxel lies in
 * an ROI; the ROIs form row blocks in list order, and a kept row's key is the
 * block's first row (the sum of the previous ROIs' masked voxel counts) plus
 * the voxel's position among its ROI's masked voxels, counted over the ROI's
 * crop box with x slowest and z fastest (the reference's loop order).  A
 * voxel in several ROIs gives one row in each block; rows with value 0 are
 * dropped.  Keys are 64-bit, as the reference's lindex dataset. */
typedef struct {
    int crop_start[3];          /* voxel index of the crop box in the volume */
    int crop_size[3];
    const unsigned char *mask;  /* crop_size[0]*crop_size[1]*crop_size[2], x fastest; non-zero = in the ROI */
} ee_roi_mask;
typedef struct ee_roi_list ee_roi_list;
/* size: the full volume (x, y, z); the masks are copied into position tables. */
int ee_roi_list_create(const int size[3], const ee_roi_mask *rois, int nrois, ee_roi_list **out);
/* capacities[r] = masked voxel count of ROI r (the reference's row_block_capacities). */
int ee_roi_list_capacities(const ee_roi_list *list, long long *capacities);
/* One column: row_index (full-volume voxel keys, as ee_csr) and values of n
 * entries in; out_keys / out_values receive the reduced rows (capacity
 * entries), *out_n their count, row_block_sizes[r] the rows kept per ROI.
 * EE_ERR_CAPACITY when *out_n > capacity (rows beyond capacity not copied). */
int ee_roi_reduce(const ee_roi_list *list, const int *row_index, const float *values, long long n,
                  unsigned long long *out_keys, float *out_values, long long capacity, long long *out_n,
                  long long *row_block_sizes);
int ee_roi_list_destroy(ee_roi_list *list);

/* ---- request server (continuous batching) ----
 * No counterpart in the reference (dosecalc-beam is a one-shot batch job):
 * a serving loop for many small dose / dose+gradient requests on one GPU.
 * `slots` worker threads, each with its own stream and a cache of
 * device-resident volume contexts (density texture, kernels, scratch),
 * least recently used first out when the HBM budget (bytes; <= 0: 80% of the
 * free memory) would be exceeded.  A free slot takes the oldest queued
 * request plus every other queued request for the same volume and kind (up
 * to max_batch_beams beams) and computes them in one pass of the chain, each
 * request's beams summed into its own dose volume.  Results equal those of
 * ee_dose_and_adjoint on the same request alone.  Host buffers of a request
 * are copied at submit (inputs) and written before its wait returns
 * (outputs). */
typedef struct ee_server ee_server;
enum { EE_REQ_DOSE = 0, EE_REQ_DOSE_AND_GRAD = 1 };
typedef struct {
    int            volume_id;          /* from ee_server_add_volume                 */
    int            kind;               /* EE_REQ_*                                  */
    const ee_beam *beams;
    int            nbeams;
    const float   *fluence;            /* host, concatenated fluence maps           */
    const float   *dose_grad;          /* host, full grid (EE_REQ_DOSE_AND_GRAD)    */
    float         *dose_out;           /* host, full grid, summed over the beams    */
    float         *fluence_grad_out;   /* host, like fluence (EE_REQ_DOSE_AND_GRAD) */
} ee_request;
int ee_server_create(int device, int slots, long long hbm_budget_bytes, int max_batch_beams, ee_server **server);
/* Physics shared by every volume (ee_set_spectrum + ee_set_kernel_table +
 * ee_set_kernel_exp when exp_params is non-null); before the first submit. */
int ee_server_set_physics(ee_server *server, int nE, const float *energy, const float *fluence, const float *mu,
                          const float *mu_en, const ee_conv_params *conv, const float *radii, const float *cumkern,
                          const float *theta_deg, const float *phi_deg, const float *exp_params);
int ee_server_add_volume(ee_server *server, const ee_frame *frame, const float *density, int *volume_id);
int ee_server_submit(ee_server *server, const ee_request *request, long long *ticket);
/* Wait for a ticket (timeout_s < 0: forever).  *status = -1 while still
 * pending (the ticket stays valid), else the request's final status, which is
 * also the return value. */
int ee_server_wait(ee_server *server, long long ticket, double timeout_s, int *status);
/* Latency percentiles (submit -> outputs written) and throughput since the
 * last reset. */
int ee_server_stats(ee_server *server, double *p50_ms, double *p99_ms, long long *completed, double *beams_per_s);
int ee_server_reset_stats(ee_server *server);
int ee_server_destroy(ee_server *server);

/* ---- fluence and beam-angle optimisation (EndtoEnd) ----
 * The EndtoEnd programs optimize_stationary_smoothness and
 * optimize_annealing_constrain (README.md:75-95; their source is not in the
 * reference snapshot, so these follow the README's description).
 *
 * ee_optimize_fluence: `iterations` projected gradient steps
 * x <- max(x - step_size * dL/dx, 0) on the device fluence d_x (in/out) with
 * the angles fixed.  dose_loss[iterations] (PTV + OAR terms, before each step)
 * and smoothness_loss[iterations][nbeams] (eta * ||D x_k||_1 after each step)
 * may be NULL. */
int ee_optimize_fluence(ee_context *ctx, const ee_beam *beams, int nbeams, float *d_x, const ee_loss *loss,
                        int iterations, float step_size, float *dose_loss, float *smoothness_loss);
typedef struct {
    int                iterations;
    float              step_size;      /* fluence gradient step                          */
    float              sigma_deg;      /* N(0, sigma) perturbation of gantry and couch    */
    float              temperature;    /* Metropolis temperature (loss units), 0 = greedy */
    float              cooling;        /* temperature factor per iteration                */
    int                fluence_steps;  /* gradient steps per iteration                    */
    unsigned long long seed;
} ee_anneal_params;
/* Output arrays, each may be NULL: [iterations][nbeams][2] for zenith,
 * azimuth and perturbation_loss (the two possibilities: keep, take),
 * [iterations][nbeams] for possibility (probability of taking) and taken,
 * [iterations] dose_loss, [iterations][nbeams] smoothness_loss. */
typedef struct {
    float         *zenith;
    float         *azimuth;
    float         *perturbation_loss;
    float         *possibility;
    unsigned char *taken;
    float         *dose_loss;
    float         *smoothness_loss;
} ee_anneal_record;
/* Simulated annealing of the beam angles + gradient descent of the fluence.
 * Per iteration every beam gets a proposal (its gantry and couch moved by
 * N(0, sigma)); all proposals' doses come from one batched call, and the
 * proposals are accepted beam by beam with probability min(1,
 * exp(-(L_take - L_keep) / T)) against the running total dose; then
 * `fluence_steps` gradient steps.  beams (angles) and d_x are updated. */
int ee_optimize_annealing(ee_context *ctx, ee_beam *beams, int nbeams, float *d_x, const ee_loss *loss,
                          const ee_anneal_params *params, ee_anneal_record *record);
/* Batched evaluation of whole-set proposals: proposals[nprop][nbeams]
 * (same fluence-map sizes in every proposal) share the fluence d_x; losses[q]
 * = PTV + OAR terms of proposal q's summed dose.  One grouped pipeline call. */
int ee_evaluate_proposals(ee_context *ctx, const ee_beam *proposals, int nprop, int nbeams, const float *d_x,
                          const ee_loss *loss, double *losses);

/* ---- preprocessing (dosecalc-preprocess) ----
 * ee_ct_to_density: the CT volume (HU, x fastest, frame `ct`: size, voxel in
 * cm) resampled onto an isotropic grid of iso_voxel_cm through linear
 * filtering, converted with the HU -> mass-density table (lut_hu ascending,
 * nlut in [2, 64]; outside it: clamped below, extrapolated from the last two
 * points above) or, with nlut == 0, by max((HU + 1024) / 1024, 0.05)
 * (replaces read_dicom / cudaCreateTexIso, dosecalc-preprocess/
 * cudaMemFunctions.cu:32-176).  out_size = ceil(voxel * size / iso_voxel);
 * density == NULL only returns out_size.  The density keeps the CT's start.
 * ee_fluence_projection: the binary conformal fluence map of every beam
 * through the PTV mask (findFluenceProjection, cudaMemFunctions.cu:308-388):
 * a pixel opens when any of its sub-rays (3x3 with supersample, else the
 * centre) crosses the mask; aperture_ready fills each row's holes
 * (fmap_post_apertureready).  fluence: the concatenated maps. */
int ee_ct_to_density(int device, const ee_frame *ct, const float *hu, float iso_voxel_cm, const float *lut_hu,
                     const float *lut_density, int nlut, float *density, int out_size[3]);
int ee_fluence_projection(int device, const ee_frame *mask_frame, const float *mask, const ee_beam *beams, int nbeams,
                          int supersample, int aperture_ready, float *fluence);

/* ---- kernel tables from measured point kernels (dosecalc-preprocess) ----
 * Replace read_spectrum_file (CCCS/DoseCalcIO/spectra.cpp:7-62), read_kernel
 * (CCCS/DoseCalcIO/kernel.cpp:27-122), make_poly_kernel (kernel.cpp:123-258)
 * and make_cumulative_kernel (kernel.cpp:260-431); the outputs are what the
 * reference stores in cumulative_kernel.h5 (total_weights, weights) and
 * convolution_{theta,phi}_angles.raw, bit for bit.
 * ee_read_spectrum_file: records "energy fluence mu mu_en kernel_file" until
 * the first that does not parse; fluence divided by its FP32 sum; kernel file
 * names NUL-terminated at kernel_names + i * name_stride (may be NULL).  *n
 * is the record count (EE_ERR_CAPACITY when above capacity).
 * ee_read_mono_kernel: a dsa kernel file, 48 polar x 24 radial cells of seven
 * (value, uncertainty) pairs; weights = the five category values as
 * [5][48][24] (primary, first scatter, second scatter, multiple scatter,
 * bremsstrahlung + annihilation).
 * ee_read_kernel_radii: radii.dat, the 24 radial boundaries [cm].
 * ee_cumulative_kernel (GPU): mono = [nkernels][5][48][24]; poly kernel
 * weighted by fluence*energy*mu per category, total = sum of categories,
 * 48/ntheta polar bins summed per cone, running sum over radius.
 * cum_total [ntheta][24] is what ee_set_kernel_table takes; cum_weights
 * [5][ntheta][24], poly_total [48][24], poly_weights [5][48][24] and the
 * nphi*ntheta/2 cone angles may be NULL.  ntheta even and a divisor of 48.
 * ee_fit_exp_kernel (host): per cone the least-squares (A, a, B, b), A, B >= 0,
 * of A/a (1 - e^{-a r}) + B/b (1 - e^{-b r}) to the cumulative table at the
 * radii: the ee_set_kernel_exp parameters for these kernels.  max_rel_err[t]
 * (may be NULL) = max |fit - table| / max |table| of cone t. */
#define EE_DSA_NRADII 24
#define EE_DSA_NANGLES 48
#define EE_DSA_NCATEGORIES 5
int ee_read_spectrum_file(const char *path, int capacity, float *energy, float *fluence, float *mu, float *mu_en,
                          char *kernel_names, int name_stride, int *n);
int ee_read_mono_kernel(const char *path, float *weights);
int ee_read_kernel_radii(const char *path, float *radii);
int ee_cumulative_kernel(int device, int nkernels, const float *energy, const float *fluence, const float *mu,
                         const float *mono, int ntheta, int nphi, float *cum_total, float *cum_weights,
                         float *poly_total, float *poly_weights, float *conv_theta_deg, float *conv_phi_deg);
int ee_fit_exp_kernel(int ntheta, int nradii, const float *radii, const float *cum_total, float *params,
                      float *max_rel_err);

/* ---- diagnostics ---- */
/* Stage ids for ee_read_profile. */
#define EE_STAGE_TERMA 0     /* k_terma (+crop-box reduction)           */
#define EE_STAGE_GEOMETRY 1  /* k_geom_init + k_geometry                */
#define EE_STAGE_CONE 2      /* k_cone: REV resample + line convolution */
#define EE_STAGE_GATHER 3    /* k_gather: REV -> patient accumulation   */
#define EE_STAGE_GATHER_T 4  /* adjoint of k_gather                     */
#define EE_STAGE_CONE_T 5    /* adjoint of k_cone + TERMA resample      */
#define EE_STAGE_TERMA_T 6   /* adjoint of TERMA (per-beamlet reduce)   */
#define EE_NSTAGES 7
/* Per-stage device-time accounting with CUDA events on the context stream
 * (off by default).  ee_read_profile returns the accumulated milliseconds
 * and kernel-launch counts of the first n stages and resets them. */
int ee_set_profiling(ee_context *ctx, int enable);
int ee_read_profile(ee_context *ctx, double *ms, long long *launches, int n);
int ee_get_beam_info(ee_context *ctx, int beam_index, ee_beam_info *info);
int ee_synchronize(ee_context *ctx);
/* CUDA stream (cudaStream_t) that the context enqueues on. */
void *ee_get_stream(ee_context *ctx);
/* Host-side beam geometry (BEAM::reconfigure, beam.cpp:300-321):
 * source and unit direction for the given angles. */
int ee_beam_source(const ee_beam *beam, float source[3], float direction[3]);

#ifdef __cplusplus
}
#endif
#endif /* EE_CCCS_H */
