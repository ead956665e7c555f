// ee_api.cpp -- host side of the CCCS engine: context, device-resident
// caches, beam geometry, the per-batch pipeline and the C ABI of ee_cccs.h.
//
// Pipeline of one batch of beams (the reference runs the same stages one
// beam and one cone at a time, CCCS/dosecalc-beam/nvbbRayConvolve_host.cu:376-725):
//   H2D beam specs -> k_geom_init -> k_terma (+crop-box reduction)
//   -> k_geometry -> [one read-back of the per-beam geometry: REV arena
//   offsets] -> k_cone (all cones of all beams) -> k_gather (all cones of all
//   beams accumulated per voxel).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ee_cccs.h"
#include "ee_internal.h"

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define EE_CUDA(call)                                                                              \
    do {                                                                                           \
        cudaError_t _e = (call);                                                                   \
        if (_e != cudaSuccess)                                                                     \
            return fail(EE_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, \
                        __LINE__);                                                                 \
    } while (0)

// ----------------------------------------------------------- geometry ---
// Double-precision restatement of CCCS/CudaUtilities/geometry.cu:46-145.
struct d3 {
    double x, y, z;
};
d3 rot_axis(d3 p, d3 r, double t) {
    double s = std::sin(t), c = std::cos(t);
    double d = -r.x * p.x - r.y * p.y - r.z * p.z;
    return {(-r.x * d) * (1 - c) + p.x * c + (-r.z * p.y + r.y * p.z) * s,
            (-r.y * d) * (1 - c) + p.y * c + (r.z * p.x - r.x * p.z) * s,
            (-r.z * d) * (1 - c) + p.z * c + (-r.y * p.x + r.x * p.y) * s};
}
d3 rot_beam(d3 v, double az, double zen, double coll) {
    d3 t = rot_axis(v, {std::sin(-zen), 0, std::cos(-zen)}, -az);
    return rot_axis(t, {0, 1, 0}, zen + coll);
}
d3 inv_rot_beam(d3 v, double az, double zen, double coll) {
    d3 t = rot_axis(v, {0, 1, 0}, -(zen + coll));
    return rot_axis(t, {std::sin(-zen), 0, std::cos(-zen)}, az);
}
d3 rot_kern(d3 v, double th, double ph) {
    d3 u = rot_axis(v, {std::cos(ph), 0, -std::sin(ph)}, -th);
    return rot_axis(u, {0, 1, 0}, -ph);
}
d3 inv_rot_kern(d3 v, double th, double ph) {
    d3 u = rot_axis(v, {0, 1, 0}, ph);
    return rot_axis(u, {std::cos(ph), 0, -std::sin(ph)}, th);
}
template <class F>
void matrix_of_d(F f, double* M) {
    d3 c[3] = {f({1, 0, 0}), f({0, 1, 0}), f({0, 0, 1})};
    for (int j = 0; j < 3; j++) {
        M[0 * 3 + j] = c[j].x;
        M[1 * 3 + j] = c[j].y;
        M[2 * 3 + j] = c[j].z;
    }
}
template <class F>
void matrix_of(F f, float* M) {
    d3 c[3] = {f({1, 0, 0}), f({0, 1, 0}), f({0, 0, 1})};
    for (int j = 0; j < 3; j++) {
        M[0 * 3 + j] = (float)c[j].x;
        M[1 * 3 + j] = (float)c[j].y;
        M[2 * 3 + j] = (float)c[j].z;
    }
}

const double kPi = 3.14159265358979323846;

// BEAM::reconfigure, angle orientation (CCCS/DoseCalcIO/beam.cpp:300-321).
void reconfigure(const ee_beam& b, double& az, double& zen, d3& src, d3& dir) {
    az = std::fmod((double)b.azimuth, 2 * kPi);
    zen = std::fmod((double)b.zenith, 2 * kPi);
    auto close = [](double a, double c) { return std::fabs(c - a) <= 1e-6; };
    if (!close(zen, 0.0) && (close(az, 0.0) || close(az, kPi))) zen = 0.0;
    d3 s = inv_rot_beam({0, -(double)b.sad, 0}, az, zen, 0);
    src = {s.x + b.isocenter[0], s.y + b.isocenter[1], s.z + b.isocenter[2]};
    d3 d = {b.isocenter[0] - src.x, b.isocenter[1] - src.y, b.isocenter[2] - src.z};
    double l = std::sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
    dir = {d.x / l, d.y / l, d.z / l};
}

template <class T>
struct DevBuf {
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
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

template <class T>
struct PinBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        size_t want = std::max<size_t>(count, 1);
        cudaError_t e = cudaMallocHost((void**)&p, want * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
};

}  // namespace

struct ee_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    bool have_volume = false, have_spectrum = false, have_table = false, have_exp = false;
    EeParams P{};
    ee_frame frame{};
    ee_conv_params conv{};
    std::vector<EeRayConst> rays;
    DevBuf<float> density, cumkern, expp;
    cudaArray_t dens_array = nullptr;
    cudaTextureObject_t dens_tex = 0;
    DevBuf<EeRayConst> d_rays;
    // per-call scratch
    DevBuf<EeBeamSpec> d_specs;
    DevBuf<EeBeamGeom> d_geoms;
    DevBuf<float> terma, unit, rev, rev_grad, terma_grad;
    DevBuf<float2> samples;  // per-REV-sample (rho, T) / (contribution, rho) of the exp-mode cone kernels
    DevBuf<int> bl_idx;
    DevBuf<float> io_fluence, io_dose, io_grad;
    DevBuf<float> xf, xg, spread_w;
    DevBuf<double> acc;
    PinBuf<EeBeamSpec> h_specs;
    PinBuf<EeBeamGeom> h_geoms;
    std::vector<EeBeamGeom> last_geoms;
    std::vector<EeBeamSpec> last_specs;
    long long max_batch_bytes = 8ll << 30;  // scratch budget for one chunk of beams
    // profiling
    bool profiling = false;
    struct Pending {
        int stage;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> event_pool;
    double stage_ms[EE_NSTAGES] = {0};
    long long stage_launches[EE_NSTAGES] = {0};
    // beamlet-column path: options and its own device workspace
    EeBeamletOptions bl_opt{2.0f, {500, 500, 500}};
    void* beamlet_ws = nullptr;
};

namespace {

int check_ready(ee_context* c) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    if (!c->have_volume) return fail(EE_ERR_NOT_READY, "ee_set_volume has not been called");
    if (!c->have_spectrum) return fail(EE_ERR_NOT_READY, "ee_set_spectrum has not been called");
    if (!c->have_table) return fail(EE_ERR_NOT_READY, "ee_set_kernel_table has not been called");
    if (c->P.mode == EE_KERNEL_EXP && !c->have_exp) return fail(EE_ERR_NOT_READY, "exp kernel mode without ee_set_kernel_exp");
    return EE_OK;
}

int check_beams(const ee_beam* beams, int nbeams) {
    if (!beams || nbeams <= 0) return fail(EE_ERR_INVALID_ARG, "no beams");
    for (int b = 0; b < nbeams; b++) {
        const ee_beam& B = beams[b];
        if (B.fmap_size[0] <= 0 || B.fmap_size[1] <= 0 || !(B.beamlet_size[0] > 0) || !(B.beamlet_size[1] > 0) ||
            !(B.sad > 0))
            return fail(EE_ERR_INVALID_ARG, "beam %d: invalid fluence map / beamlet size / SAD", b);
    }
    return EE_OK;
}

// Axis-aligned patient-index box holding the beam's field frustum between the
// calc bbox's nearest and farthest axial distances from the source (the
// convex hull of 8 vertices), widened by one voxel and clipped to the bbox.
// TERMA is zero outside it: a voxel gets TERMA only when its projection onto
// the isocentre plane lands inside the fluence map (cudaSiddon.cu:143-165).
void terma_box(const EeParams& P, const EeBeamSpec& S, int t0[3], int tn[3]) {
    const d3 src = {S.src[0], S.src[1], S.src[2]}, dir = {S.dir[0], S.dir[1], S.dir[2]};
    double dmin = 1e300, dmax = -1e300;
    for (int c = 0; c < 8; c++) {
        double p[3];
        for (int a = 0; a < 3; a++) {
            int idx = ((c >> a) & 1) ? P.bb0[a] + P.bbs[a] - 1 : P.bb0[a];
            p[a] = P.start[a] + (double)idx * P.voxel[a];
        }
        double d = (p[0] - src.x) * dir.x + (p[1] - src.y) * dir.y + (p[2] - src.z) * dir.z;
        dmin = std::min(dmin, d);
        dmax = std::max(dmax, d);
    }
    for (int a = 0; a < 3; a++) { t0[a] = P.bb0[a]; tn[a] = 0; }
    if (dmax <= 0) return;  // the bbox lies behind the source
    if (dmin <= 1e-3 * S.isodist) {
        // the source sits inside (or close to) the calc bbox: the beamlet
        // lookup takes |depth| (cudaSiddon.cu:148-152), so voxels behind the
        // source see a mirrored field; TERMA over the whole bbox, as the
        // reference computes it
        for (int a = 0; a < 3; a++) tn[a] = P.bbs[a];
        return;
    }
    const double hu = 0.5 * S.fmap[0] * S.beamlet[0], hw = 0.5 * S.fmap[1] * S.beamlet[1];
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int c = 0; c < 8; c++) {
        double u = (c & 1) ? hu : -hu, w = (c & 2) ? hw : -hw, d = (c & 4) ? dmax : dmin;
        // point on the isocentre plane, BEV lateral offsets (u, 0, w)
        double q[3];
        for (int a = 0; a < 3; a++) q[a] = S.src[a] + S.dir[a] * S.isodist + S.MBi[3 * a] * u + S.MBi[3 * a + 2] * w;
        double sc = d / S.isodist;
        for (int a = 0; a < 3; a++) {
            double pos = S.src[a] + (q[a] - S.src[a]) * sc;
            double idx = (pos - P.start[a]) / P.voxel[a];
            lo[a] = std::min(lo[a], idx);
            hi[a] = std::max(hi[a], idx);
        }
    }
    for (int a = 0; a < 3; a++) {
        long long l = (long long)std::floor(lo[a]) - 1, h = (long long)std::ceil(hi[a]) + 1;
        l = std::max<long long>(l, P.bb0[a]);
        h = std::min<long long>(h, P.bb0[a] + P.bbs[a] - 1);
        if (h < l) { for (int k = 0; k < 3; k++) tn[k] = 0; return; }
        t0[a] = (int)l;
        tn[a] = (int)(h - l + 1);
    }
}

void build_specs(const EeParams& P, const ee_beam* beams, int nbeams, EeBeamSpec* out) {
    long long off = 0, toff = 0;
    for (int b = 0; b < nbeams; b++) {
        const ee_beam& B = beams[b];
        double az, zen;
        d3 src, dir;
        reconfigure(B, az, zen, src, dir);
        EeBeamSpec& S = out[b];
        std::memset(&S, 0, sizeof(S));
        S.src[0] = (float)src.x; S.src[1] = (float)src.y; S.src[2] = (float)src.z;
        S.dir[0] = (float)dir.x; S.dir[1] = (float)dir.y; S.dir[2] = (float)dir.z;
        for (int a = 0; a < 3; a++) S.iso[a] = B.isocenter[a];
        S.az = (float)az; S.zen = (float)zen; S.coll = B.coll; S.sad = B.sad;
        d3 id = {B.isocenter[0] - src.x, B.isocenter[1] - src.y, B.isocenter[2] - src.z};
        S.isodist = (float)std::sqrt(id.x * id.x + id.y * id.y + id.z * id.z);
        double coll = B.coll;
        matrix_of([&](d3 v) { return rot_beam(v, az, zen, coll); }, S.MB);
        matrix_of([&](d3 v) { return inv_rot_beam(v, az, zen, coll); }, S.MBi);
        matrix_of_d([&](d3 v) { return rot_beam(v, az, zen, coll); }, S.MBd);
        S.srcd[0] = src.x; S.srcd[1] = src.y; S.srcd[2] = src.z;
        S.dird[0] = dir.x; S.dird[1] = dir.y; S.dird[2] = dir.z;
        S.isodistd = std::sqrt(id.x * id.x + id.y * id.y + id.z * id.z);
        S.fmap[0] = B.fmap_size[0]; S.fmap[1] = B.fmap_size[1];
        S.beamlet[0] = B.beamlet_size[0]; S.beamlet[1] = B.beamlet_size[1];
        S.fl_off = off;
        off += (long long)B.fmap_size[0] * B.fmap_size[1];
        terma_box(P, S, S.t0, S.tn);
        S.t_off = toff;
        toff += ee_brick_vol(S.tn);
    }
}

// elements of the beam's bricked TERMA box (4x4x4 bricks, padded)
long long tvol_of(const EeBeamSpec& S) { return ee_brick_vol(S.tn); }

const char* status_text(int st) {
    switch (st) {
        case EE_ERR_CROPBOX: return "bev_cropbox_size error (no TERMA in the calc bbox, or crop box >= 1000 voxels)";
        case EE_ERR_REV_SIZE: return "convolution array size exceeds the REV limit";
        case EE_ERR_SIDDON_ITER: return "Siddon ray trace hit its iteration cap";
        case EE_ERR_CAPACITY: return "REV arena too small";
        default: return "geometry error";
    }
}

cudaEvent_t take_event(ee_context* c) {
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Resolve recorded event pairs into per-stage milliseconds.
void drain_profile(ee_context* c) {
    for (auto& p : c->pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess)
            c->stage_ms[p.stage] += ms;
        c->event_pool.push_back(p.a);
        c->event_pool.push_back(p.b);
    }
    c->pending.clear();
}

// Launch `fn` bracketed by profiling events when enabled; counts launches.
template <class F>
cudaError_t staged(ee_context* c, int stage, int nlaunch, F fn) {
    c->stage_launches[stage] += nlaunch;
    if (!c->profiling) return fn();
    cudaEvent_t a = take_event(c), b = take_event(c);
    cudaEventRecord(a, c->stream);
    cudaError_t e = fn();
    cudaEventRecord(b, c->stream);
    c->pending.push_back({stage, a, b});
    return e;
}

long long nfull_of(const ee_context* c) { return (long long)c->P.size[0] * c->P.size[1] * c->P.size[2]; }

// Beams per chunk so that TERMA (+unit/index for the adjoint) fits the budget.
// Split the beams into chunks whose REV arena fits the scratch budget
// (estimate: nrays x 4 x the TERMA box per beam, x2 with the adjoint's REV
// gradient).  TERMA boxes of all beams stay resident for the whole call so
// the adjoint reuses the forward's TERMA, crop boxes and REV frames.
std::vector<int> plan_chunks(const ee_context* c, const EeBeamSpec* specs, int nbeams, bool adjoint) {
    std::vector<int> starts;
    long long acc = 0;
    // REV arena + (rho, T) sample scratch (+ REV gradient for the adjoint)
    const long long per_vox = 4ll * (long long)c->P.nrays * 4 * (adjoint ? 4 : 3);
    for (int b = 0; b < nbeams; b++) {
        long long need = std::max(1ll, tvol_of(specs[b])) * per_vox;
        if (starts.empty() || (acc + need > c->max_batch_bytes && acc > 0)) {
            starts.push_back(b);
            acc = 0;
        }
        acc += need;
    }
    starts.push_back(nbeams);
    return starts;
}

struct ChunkDims {
    long long rev_total = 0, max_tvol = 1;
    int max_line = 1, max_lines = 1, max_rows = 1, max_tiles = 1;
};

// Device buffer growth: a freed buffer may still be read by queued kernels,
// so drain the stream first when a buffer has to grow.
bool ee_debug_poison() {
    static const bool on = [] {
        const char* v = std::getenv("EE_DEBUG_POISON");
        return v && *v && *v != '0';
    }();
    return on;
}

template <class T>
cudaError_t grow(ee_context* c, DevBuf<T>& b, size_t n) {
    if (n <= b.n && b.p) return cudaSuccess;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return e;
    return b.ensure(n);
}

struct PipeArgs {
    const ee_beam* beams = nullptr;
    int nbeams = 0;
    const float* d_fluence = nullptr;  // fluence the dose engine sees
    float* d_dose = nullptr;           // forward output (nullptr: no forward dose)
    int dose_mode = EE_DOSE_SUM;
    const float* d_dose_grad = nullptr;  // adjoint input given by the caller
    const ee_loss* loss = nullptr;       // or: gradient of the EndtoEnd dose terms
    float* d_fgrad = nullptr;            // adjoint output (nullptr: no adjoint)
    double* loss_acc = nullptr;          // device accumulator [3] for loss terms
    const int* group = nullptr;          // host: output volume index of each beam (grouped sums)
    int ngroups = 1;
};

// One call of the CCCS chain over a list of beams:
//   geometry pass per chunk (TERMA + crop box + REV frames, one read-back)
//   with the forward dose (REV cones + gather) when requested, then the loss
//   gradient, then the adjoint per chunk reusing the resident TERMA/geometry.
int pipeline(ee_context* c, const PipeArgs& A) {
    int st = check_ready(c);
    if (st) return st;
    if ((st = check_beams(A.beams, A.nbeams))) return st;
    if (!A.d_fluence) return fail(EE_ERR_INVALID_ARG, "null fluence pointer");
    if (A.dose_mode < 0 || A.dose_mode > 2) return fail(EE_ERR_INVALID_ARG, "bad dose mode %d", A.dose_mode);
    const bool fwd = A.d_dose != nullptr;
    const bool adj = A.d_fgrad != nullptr;
    if (adj && !A.d_dose_grad && !A.loss) return fail(EE_ERR_INVALID_ARG, "adjoint needs a dose gradient or a loss");
    if (A.loss && (!fwd || A.dose_mode != EE_DOSE_SUM)) return fail(EE_ERR_INVALID_ARG, "loss needs the summed dose");
    EE_CUDA(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const int n = A.nbeams;
    const long long nfull = nfull_of(c);
    EE_CUDA(c->h_specs.ensure(n));
    EE_CUDA(c->h_geoms.ensure(n));
    build_specs(c->P, A.beams, n, c->h_specs.p);
    if (A.group)
        for (int b = 0; b < n; b++) c->h_specs.p[b].out_off = (long long)A.group[b] * nfull;
    long long tvol_total = 0;
    for (int b = 0; b < n; b++) tvol_total += tvol_of(c->h_specs.p[b]);
    EE_CUDA(grow(c, c->d_specs, n));
    EE_CUDA(grow(c, c->d_geoms, n));
    EE_CUDA(grow(c, c->terma, tvol_total));
    if (adj) {
        EE_CUDA(grow(c, c->unit, tvol_total));
        EE_CUDA(grow(c, c->bl_idx, tvol_total));
        EE_CUDA(grow(c, c->terma_grad, tvol_total + 4));  // +4: vector-reduction padding
    }
    EE_CUDA(cudaMemcpyAsync(c->d_specs.p, c->h_specs.p, sizeof(EeBeamSpec) * n, cudaMemcpyHostToDevice, s));
    std::vector<int> starts = plan_chunks(c, c->h_specs.p, n, adj);
    const int nchunks = (int)starts.size() - 1;
    std::vector<ChunkDims> dims(nchunks);
    c->last_geoms.clear();
    c->last_specs.assign(c->h_specs.p, c->h_specs.p + n);
    if (fwd && A.dose_mode == EE_DOSE_SUM)
        EE_CUDA(cudaMemsetAsync(A.d_dose, 0, sizeof(float) * nfull * (A.group ? A.ngroups : 1), s));
    if (fwd && A.dose_mode == EE_DOSE_PER_BEAM) EE_CUDA(cudaMemsetAsync(A.d_dose, 0, sizeof(float) * nfull * n, s));

    // ---- geometry + forward, chunk by chunk
    for (int k = 0; k < nchunks; k++) {
        const int b0 = starts[k], nb = starts[k + 1] - b0;
        EeBeamSpec* dsp = c->d_specs.p + b0;
        EeBeamGeom* dge = c->d_geoms.p + b0;
        ChunkDims& D = dims[k];
        for (int b = b0; b < b0 + nb; b++) D.max_tvol = std::max(D.max_tvol, tvol_of(c->h_specs.p[b]));
        EE_CUDA(staged(c, EE_STAGE_GEOMETRY, 1, [&] { return ee_launch_geom_init(dsp, dge, nb, s); }));
        EE_CUDA(staged(c, EE_STAGE_TERMA, 1, [&] {
            return ee_launch_terma(c->P, dsp, dge, A.d_fluence, c->terma.p, adj ? c->unit.p : nullptr,
                                   adj ? c->bl_idx.p : nullptr, nb, D.max_tvol, s);
        }));
        EE_CUDA(staged(c, EE_STAGE_GEOMETRY, 1, [&] { return ee_launch_geometry(c->P, dsp, dge, nb, s); }));
        EeBeamGeom* hg = c->h_geoms.p + b0;
        EE_CUDA(cudaMemcpyAsync(hg, dge, sizeof(EeBeamGeom) * nb, cudaMemcpyDeviceToHost, s));
        EE_CUDA(cudaStreamSynchronize(s));
        for (int b = 0; b < nb; b++) {
            EeBeamGeom& G = hg[b];
            if (G.status != 0) return fail(G.status, "beam %d: %s", b0 + b, status_text(G.status));
            G.arena_off = D.rev_total;
            G.arena_cap = G.rev_total;
            D.rev_total += G.rev_total;
            D.max_line = std::max(D.max_line, G.max_line);
            D.max_lines = std::max(D.max_lines, G.max_lines);
            D.max_rows = std::max(D.max_rows, G.rows);
            D.max_tiles = std::max(D.max_tiles, G.tiles);
        }
        EE_CUDA(cudaMemcpyAsync(dge, hg, sizeof(EeBeamGeom) * nb, cudaMemcpyHostToDevice, s));
        c->last_geoms.insert(c->last_geoms.end(), hg, hg + nb);
        if (!fwd) continue;
        EE_CUDA(grow(c, c->rev, D.rev_total));
        // no clear: the cone kernels write every sample k_gather reads
        if (ee_debug_poison()) EE_CUDA(cudaMemsetAsync(c->rev.p, 0xFF, sizeof(float) * D.rev_total, s));
        if (c->P.mode == EE_KERNEL_EXP) EE_CUDA(grow(c, c->samples, D.rev_total));
        EE_CUDA(staged(c, EE_STAGE_CONE, 1, [&] {
            return ee_launch_cone(c->P, dsp, dge, c->terma.p, c->rev.p,
                                  c->P.mode == EE_KERNEL_EXP ? c->samples.p : nullptr, nb, D.max_lines, D.max_line, s);
        }));
        float* out = A.dose_mode == EE_DOSE_PER_BEAM ? A.d_dose + (long long)b0 * nfull : A.d_dose;
        const int m = A.dose_mode == EE_DOSE_PER_BEAM ? 2 : 1;
        EE_CUDA(staged(c, EE_STAGE_GATHER, 1, [&] {
            return ee_launch_gather(c->P, dsp, dge, c->rev.p, out, nb, m, D.max_rows, s);
        }));
    }
    if (!adj) return EE_OK;

    // ---- dose gradient of the loss
    const float* dgrad = A.d_dose_grad;
    if (A.loss) {
        EE_CUDA(grow(c, c->io_grad, nfull));
        EE_CUDA(ee_launch_loss_grad(A.d_dose, A.loss->ptv_weight, A.loss->ptv_target, A.loss->oar_weight,
                                    A.loss->oar_target, c->io_grad.p, A.loss_acc, nfull, s));
        dgrad = c->io_grad.p;
    }

    // ---- adjoint, chunk by chunk (same plan, geometry resident)
    long long nfl_all = 0;
    for (int b = 0; b < n; b++) nfl_all += (long long)A.beams[b].fmap_size[0] * A.beams[b].fmap_size[1];
    EE_CUDA(cudaMemsetAsync(A.d_fgrad, 0, sizeof(float) * nfl_all, s));
    EE_CUDA(cudaMemsetAsync(c->terma_grad.p, 0, sizeof(float) * tvol_total, s));
    for (int k = 0; k < nchunks; k++) {
        const int b0 = starts[k], nb = starts[k + 1] - b0;
        const EeBeamSpec* dsp = c->d_specs.p + b0;
        const EeBeamGeom* dge = c->d_geoms.p + b0;
        const ChunkDims& D = dims[k];
        EE_CUDA(grow(c, c->rev_grad, D.rev_total + 4));  // +4: vector-reduction padding
        if (c->P.mode == EE_KERNEL_EXP) EE_CUDA(grow(c, c->samples, D.rev_total));  // adjoint cone scratch
        if (ee_debug_poison()) EE_CUDA(cudaMemsetAsync(c->rev_grad.p, 0xFF, sizeof(float) * D.rev_total, s));
        EE_CUDA(ee_launch_rev_zero(c->P, dge, c->rev_grad.p, nb, D.max_lines, s));
        EE_CUDA(staged(c, EE_STAGE_GATHER_T, 1, [&] {
            return ee_launch_gather_T(c->P, dsp, dge, dgrad, c->rev_grad.p, nb, D.max_tiles, s);
        }));
        EE_CUDA(staged(c, EE_STAGE_CONE_T, 1, [&] {
            return ee_launch_cone_T(c->P, dsp, dge, c->rev_grad.p, c->P.mode == EE_KERNEL_EXP ? c->samples.p : nullptr,
                                    c->terma_grad.p, nb, D.max_lines, D.max_line, s);
        }));
        EE_CUDA(staged(c, EE_STAGE_TERMA_T, 1, [&] {
            return ee_launch_terma_T(c->P, dsp, dge, c->unit.p, c->bl_idx.p, c->terma_grad.p, A.d_fgrad, nb,
                                     D.max_tvol, s);
        }));
    }
    return EE_OK;
}

int dose_device(ee_context* c, const ee_beam* beams, int nbeams, const float* d_fluence, float* d_dose, int mode) {
    if (!d_dose) return fail(EE_ERR_INVALID_ARG, "null dose pointer");
    PipeArgs A;
    A.beams = beams; A.nbeams = nbeams; A.d_fluence = d_fluence; A.d_dose = d_dose; A.dose_mode = mode;
    return pipeline(c, A);
}

int adjoint_device(ee_context* c, const ee_beam* beams, int nbeams, const float* d_fluence, const float* d_grad,
                   float* d_fgrad) {
    if (!d_grad || !d_fgrad) return fail(EE_ERR_INVALID_ARG, "null pointer");
    PipeArgs A;
    A.beams = beams; A.nbeams = nbeams; A.d_fluence = d_fluence; A.d_dose_grad = d_grad; A.d_fgrad = d_fgrad;
    return pipeline(c, A);
}

// max_rev_size as initCudaConstandTex derives it when the caller gives none
// (host.cu:248-258, REV_PAD = 0).
void derive_max_rev(ee_context* c) {
    EeParams& P = c->P;
    for (int a = 0; a < 3; a++) P.max_rev[a] = c->conv.max_rev_size[a];
    if (!c->have_volume || c->conv.max_rev_size[0] > 0 || !(c->conv.rev_latspacing > 0)) return;
    double mvs = std::min(c->conv.rev_latspacing, c->conv.rev_longspacing);
    double bl = std::sqrt((double)P.bbs[0] * P.bbs[0] + (double)P.bbs[1] * P.bbs[1] + (double)P.bbs[2] * P.bbs[2]);
    unsigned diag = (unsigned)std::ceil((float)bl * P.voxel[0] / (float)mvs);
    unsigned m = diag + (unsigned)(2 * (c->conv.penumbra / mvs)) + 100;
    for (int a = 0; a < 3; a++) P.max_rev[a] = (int)m;
}

long long total_fluence(const ee_beam* beams, int nbeams) {
    long long n = 0;
    for (int b = 0; b < nbeams; b++) n += (long long)beams[b].fmap_size[0] * beams[b].fmap_size[1];
    return n;
}

// ====================================================== planned batches ==
// An ee_plan fixes one batch of beams and sizes every device buffer from
// geometric upper bounds, so the whole chain (TERMA, crop boxes, REV frames,
// cones, gather and optionally the adjoint) runs without a host read-back and
// is captured once into a CUDA graph; replaying the graph re-evaluates the
// batch for new fluence / dose-gradient values in the same device buffers.
//
// Bounds: a beam's TERMA-non-zero voxels lie in its field frustum, so their
// BEV indices lie in the BEV AABB of the frustum's 8 vertices; the crop box
// (that AABB, its maximum floored at 0 as the reference's FLT_MIN start does,
// widened by the penumbra) bounds every REV array (findREV is monotone in the
// box size) and the patient rows/tiles the gather kernels visit.
struct PlanBound {
    long long rev = 0;
    int max_line = 1, max_lines = 1, rows = 1, tiles = 1;
};

PlanBound plan_bound(const ee_context* c, const EeBeamSpec& S) {
    const EeParams& P = c->P;
    PlanBound B;
    // frustum vertices in patient index space (as terma_box)
    const double dir[3] = {S.dird[0], S.dird[1], S.dird[2]};
    double dmin = 1e300, dmax = -1e300;
    for (int k = 0; k < 8; k++) {
        double d = 0;
        for (int a = 0; a < 3; a++) {
            int idx = ((k >> a) & 1) ? P.bb0[a] + P.bbs[a] - 1 : P.bb0[a];
            d += (P.start[a] + (double)idx * P.voxel[a] - S.srcd[a]) * dir[a];
        }
        dmin = std::min(dmin, d);
        dmax = std::max(dmax, d);
    }
    dmin = std::max(dmin, 1e-6);
    const double hu = 0.5 * S.fmap[0] * S.beamlet[0], hw = 0.5 * S.fmap[1] * S.beamlet[1];
    double blo[3] = {1e300, 1e300, 1e300}, bhi[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < 8; k++) {
        double u = (k & 1) ? hu : -hu, w = (k & 2) ? hw : -hw, d = (k & 4) ? dmax : dmin;
        double rel[3];
        for (int a = 0; a < 3; a++) {
            double q = S.srcd[a] + dir[a] * S.isodistd + S.MBi[3 * a] * u + S.MBi[3 * a + 2] * w;
            double pos = S.srcd[a] + (q - S.srcd[a]) * (d / S.isodistd);
            rel[a] = (pos - P.start[a]) / P.voxel[a] - P.bb0[a];
        }
        for (int a = 0; a < 3; a++) {
            double b = S.MBd[3 * a] * rel[0] + S.MBd[3 * a + 1] * rel[1] + S.MBd[3 * a + 2] * rel[2];
            blo[a] = std::min(blo[a], b);
            bhi[a] = std::max(bhi[a], b);
        }
    }
    const double pen[3] = {P.penumbra / P.lat, P.penumbra / P.lng, P.penumbra / P.lat};
    double bmn[3], bev[3];
    for (int a = 0; a < 3; a++) {
        bmn[a] = blo[a] - pen[a] - 1.0;
        double bmx = std::max(bhi[a], 0.0) + pen[a] + 1.0;
        bev[a] = std::ceil(bmx - bmn[a]) + 1.0;
    }
    const double bd[3] = {bev[0] * P.lat, bev[1] * P.lng, bev[2] * P.lat};
    for (int r = 0; r < P.nrays; r++) {
        const float* M = c->rays[r].MK;
        double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
        for (int k = 0; k < 8; k++) {
            double v[3] = {bd[0] * (k & 1), bd[1] * ((k >> 1) & 1), bd[2] * ((k >> 2) & 1)};
            for (int a = 0; a < 3; a++) {
                double o = M[3 * a] * v[0] + M[3 * a + 1] * v[1] + M[3 * a + 2] * v[2];
                mn[a] = std::min(mn[a], o);
                mx[a] = std::max(mx[a], o);
            }
        }
        long long s0 = (long long)std::ceil((mx[1] - mn[1]) / P.lng) + 2;
        long long s1 = (long long)std::ceil((mx[2] - mn[2]) / P.lat) + 2;
        long long s2 = (long long)std::ceil((mx[0] - mn[0]) / P.lat) + 2;
        // bricked REV arrays and 8 x 4 lane tiles, as k_geometry sizes them
        B.rev += 64 * ((s0 + 3) / 4) * ((s1 + 3) / 4) * ((s2 + 3) / 4);
        B.max_line = (int)std::max<long long>(B.max_line, std::min<long long>(s0, EE_MAX_LINE));
        const long long slots = std::max(((s1 + 7) / 8) * 8 * (((s2 + 3) / 4) * 4),
                                         ((s2 + 7) / 8) * 8 * (((s1 + 3) / 4) * 4));  // either lateral order
        B.max_lines = (int)std::max<long long>(B.max_lines, slots);
    }
    // patient AABB of the dilated bound box: t = MBi (b + bmn) + bb0
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < 8; k++) {
        double b[3] = {((k & 1) ? bev[0] + 2.0 : -2.0) + bmn[0], (((k >> 1) & 1) ? bev[1] + 2.0 : -2.0) + bmn[1],
                       (((k >> 2) & 1) ? bev[2] + 2.0 : -2.0) + bmn[2]};
        for (int a = 0; a < 3; a++) {
            double t = S.MBi[3 * a] * b[0] + S.MBi[3 * a + 1] * b[1] + S.MBi[3 * a + 2] * b[2] + P.bb0[a];
            lo[a] = std::min(lo[a], t);
            hi[a] = std::max(hi[a], t);
        }
    }
    long long n[3];
    for (int a = 0; a < 3; a++) {
        long long l = std::max<long long>(P.bb0[a], (long long)std::floor(lo[a]) - 2);
        long long h = std::min<long long>(P.bb0[a] + P.bbs[a] - 1, (long long)std::ceil(hi[a]) + 2);
        n[a] = std::max<long long>(1, h - l + 1);
    }
    B.rows = (int)ee_gather_groups(n[1], n[2]);
    B.tiles = (int)(((n[0] + 7) / 8) * ((n[1] + 7) / 8) * ((n[2] + 3) / 4));
    return B;
}

}  // namespace

struct ee_plan {
    ee_context* c = nullptr;
    int nbeams = 0;
    bool adjoint = false;
    std::vector<ee_beam> beams;
    std::vector<EeBeamSpec> specs;
    std::vector<int> starts;
    std::vector<ChunkDims> dims;
    long long tvol_total = 0, rev_max = 0, nfl = 0;
    DevBuf<EeBeamSpec> d_specs;
    DevBuf<EeBeamGeom> d_geoms;
    DevBuf<float> terma, unit, terma_grad, rev, rev_grad;
    DevBuf<int> bl_idx;
    DevBuf<float2> samples;
    const float* d_fluence = nullptr;
    float* d_dose = nullptr;
    const float* d_grad = nullptr;
    float* d_fgrad = nullptr;
    int lane_block = 128;
    std::vector<int> status;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // releases everything, also when ee_plan_create fails half-way
    ~ee_plan() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        d_specs.release(); d_geoms.release(); terma.release(); unit.release(); terma_grad.release();
        rev.release(); rev_grad.release(); bl_idx.release(); samples.release();
    }
};

namespace {

// Every memset and launch of one plan evaluation, on stream s.
cudaError_t plan_enqueue(ee_plan* pl, cudaStream_t s) {
    ee_context* c = pl->c;
    const EeParams& P = c->P;
    const long long nfull = nfull_of(c);
    cudaError_t e;
#define PL(x)                              \
    do {                                   \
        if ((e = (x)) != cudaSuccess) return e; \
    } while (0)
    PL(cudaMemsetAsync(pl->d_dose, 0, sizeof(float) * nfull, s));
    const int nchunks = (int)pl->starts.size() - 1;
    for (int k = 0; k < nchunks; k++) {
        const int b0 = pl->starts[k], nb = pl->starts[k + 1] - b0;
        const EeBeamSpec* dsp = pl->d_specs.p + b0;
        EeBeamGeom* dge = pl->d_geoms.p + b0;
        const ChunkDims& D = pl->dims[k];
        PL(ee_launch_geom_init(dsp, dge, nb, s));
        PL(ee_launch_terma(P, dsp, dge, pl->d_fluence, pl->terma.p, pl->adjoint ? pl->unit.p : nullptr,
                           pl->adjoint ? pl->bl_idx.p : nullptr, nb, D.max_tvol, s));
        PL(ee_launch_geometry(P, dsp, dge, nb, s));
        if (ee_debug_poison()) PL(cudaMemsetAsync(pl->rev.p, 0xFF, sizeof(float) * D.rev_total, s));
        PL(ee_launch_cone(P, dsp, dge, pl->terma.p, pl->rev.p, P.mode == EE_KERNEL_EXP ? pl->samples.p : nullptr, nb,
                          D.max_lines, D.max_line, s, pl->lane_block));
        PL(ee_launch_gather(P, dsp, dge, pl->rev.p, pl->d_dose, nb, 1, D.max_rows, s));
    }
    if (!pl->adjoint) return cudaSuccess;
    PL(cudaMemsetAsync(pl->d_fgrad, 0, sizeof(float) * pl->nfl, s));
    PL(cudaMemsetAsync(pl->terma_grad.p, 0, sizeof(float) * pl->tvol_total, s));
    for (int k = 0; k < nchunks; k++) {
        const int b0 = pl->starts[k], nb = pl->starts[k + 1] - b0;
        const EeBeamSpec* dsp = pl->d_specs.p + b0;
        const EeBeamGeom* dge = pl->d_geoms.p + b0;
        const ChunkDims& D = pl->dims[k];
        if (ee_debug_poison()) PL(cudaMemsetAsync(pl->rev_grad.p, 0xFF, sizeof(float) * D.rev_total, s));
        PL(ee_launch_rev_zero(P, dge, pl->rev_grad.p, nb, D.max_lines, s));
        PL(ee_launch_gather_T(P, dsp, dge, pl->d_grad, pl->rev_grad.p, nb, D.max_tiles, s));
        PL(ee_launch_cone_T(P, dsp, dge, pl->rev_grad.p, P.mode == EE_KERNEL_EXP ? pl->samples.p : nullptr,
                            pl->terma_grad.p, nb, D.max_lines, D.max_line, s, pl->lane_block));
        PL(ee_launch_terma_T(P, dsp, dge, pl->unit.p, pl->bl_idx.p, pl->terma_grad.p, pl->d_fgrad, nb, D.max_tvol, s));
    }
#undef PL
    return cudaSuccess;
}

}  // namespace



// ======================================================================= ABI
extern "C" {

const char* ee_last_error(void) { return g_err.c_str(); }
int ee_abi_version(void) { return EE_ABI_VERSION; }

int ee_create(int device, ee_context** out) {
    if (!out) return fail(EE_ERR_INVALID_ARG, "null output pointer");
    *out = nullptr;
    int n = 0;
    EE_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(EE_ERR_INVALID_ARG, "device %d out of range (%d devices)", device, n);
    EE_CUDA(cudaSetDevice(device));
    ee_context* c = new ee_context();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return fail(EE_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    c->P.mode = EE_KERNEL_TABLE;
    c->P.ss = 1;
    *out = c;
    return EE_OK;
}

int ee_destroy(ee_context* c) {
    if (!c) return EE_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->dens_tex) cudaDestroyTextureObject(c->dens_tex);
    if (c->dens_array) cudaFreeArray(c->dens_array);
    c->density.release(); c->cumkern.release(); c->expp.release(); c->d_rays.release();
    c->d_specs.release(); c->d_geoms.release(); c->terma.release(); c->unit.release(); c->rev.release();
    c->rev_grad.release(); c->terma_grad.release(); c->bl_idx.release(); c->samples.release();
    c->io_fluence.release(); c->io_dose.release(); c->io_grad.release();
    c->xf.release(); c->xg.release(); c->spread_w.release(); c->acc.release();
    c->h_specs.release(); c->h_geoms.release();
    ee_beamlet_free(c->beamlet_ws);
    c->beamlet_ws = nullptr;
    drain_profile(c);
    for (auto e : c->event_pool) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return EE_OK;
}

int ee_set_volume(ee_context* c, const ee_frame* f, const float* density) {
    if (!c || !f || !density) return fail(EE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(c->mu);
    ee_frame fr = *f;
    for (int a = 0; a < 3; a++) {
        if (fr.size[a] <= 0 || !(fr.voxel[a] > 0)) return fail(EE_ERR_INVALID_ARG, "bad volume size/voxel");
        // enforce a valid bbox as load_omni_header does (calc_header.cpp:127-133)
        if (fr.bbox_start[a] < 0 || fr.bbox_start[a] >= fr.size[a]) fr.bbox_start[a] = 0;
        if (fr.bbox_size[a] <= 0 || fr.bbox_size[a] + fr.bbox_start[a] > fr.size[a]) fr.bbox_size[a] = fr.size[a] - fr.bbox_start[a];
    }
    // every TERMA box lies in the calc bbox; the kernels address a bricked
    // box with 32-bit offsets
    if (ee_brick_vol(fr.bbox_size) > 2147483647ll)
        return fail(EE_ERR_INVALID_ARG, "calc bbox of %d x %d x %d voxels: bricked TERMA boxes above 2^31 elements",
                    fr.bbox_size[0], fr.bbox_size[1], fr.bbox_size[2]);
    EE_CUDA(cudaSetDevice(c->device));
    size_t n = (size_t)fr.size[0] * fr.size[1] * fr.size[2];
    EE_CUDA(c->density.ensure(n));
    EE_CUDA(cudaMemcpyAsync(c->density.p, density, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    EE_CUDA(cudaStreamSynchronize(c->stream));
    // the density also as a 3-D texture: the SM texture units do the
    // trilinear interpolation of every Siddon and REV-resample fetch
    // (linear filter, border 0, unnormalised coordinates; the reference's
    // texDens, nvbbRayConvolve_host.cu:229-242)
    if (c->dens_tex) { cudaDestroyTextureObject(c->dens_tex); c->dens_tex = 0; }
    if (c->dens_array) { cudaFreeArray(c->dens_array); c->dens_array = nullptr; }
    {
        cudaChannelFormatDesc fd = cudaCreateChannelDesc<float>();
        cudaExtent ext = make_cudaExtent(fr.size[0], fr.size[1], fr.size[2]);
        EE_CUDA(cudaMalloc3DArray(&c->dens_array, &fd, ext));
        cudaMemcpy3DParms cp = {};
        cp.srcPtr = make_cudaPitchedPtr((void*)c->density.p, fr.size[0] * sizeof(float), fr.size[0], fr.size[1]);
        cp.dstArray = c->dens_array;
        cp.extent = ext;
        cp.kind = cudaMemcpyDeviceToDevice;
        EE_CUDA(cudaMemcpy3DAsync(&cp, c->stream));
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = c->dens_array;
        cudaTextureDesc td = {};
        for (int a = 0; a < 3; a++) td.addressMode[a] = cudaAddressModeBorder;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        EE_CUDA(cudaCreateTextureObject(&c->dens_tex, &rd, &td, nullptr));
        EE_CUDA(cudaStreamSynchronize(c->stream));
    }
    c->frame = fr;
    for (int a = 0; a < 3; a++) {
        c->P.size[a] = fr.size[a]; c->P.voxel[a] = fr.voxel[a]; c->P.start[a] = fr.start[a];
        c->P.bb0[a] = fr.bbox_start[a]; c->P.bbs[a] = fr.bbox_size[a];
    }
    c->P.density = c->density.p;
    c->P.dens_tex = c->dens_tex;
    c->have_volume = true;
    derive_max_rev(c);
    return EE_OK;
}

int ee_set_spectrum(ee_context* c, int nE, const float* energy, const float* fluence, const float* mu, const float* mu_en) {
    if (!c || !energy || !fluence || !mu) return fail(EE_ERR_INVALID_ARG, "null argument");
    if (nE <= 0 || nE > EE_MAX_E) return fail(EE_ERR_INVALID_ARG, "nE must be in [1, %d]", EE_MAX_E);
    (void)mu_en;  // beam-hardening correction is fixed to 1 (host.cu:204)
    std::lock_guard<std::mutex> lk(c->mu);
    double sum = 0;
    for (int e = 0; e < nE; e++) sum += fluence[e];
    if (!(sum > 0)) return fail(EE_ERR_INVALID_ARG, "spectrum fluence sums to zero");
    c->P.nE = nE;
    for (int e = 0; e < nE; e++) {
        // fluence normalised to unit sum as read_spectrum_file does (spectra.cpp:56-58)
        c->P.sp_fluence[e] = (float)(fluence[e] / sum);
        c->P.sp_energy[e] = energy[e];
        c->P.sp_mu[e] = mu[e];
    }
    c->have_spectrum = true;
    return EE_OK;
}

int ee_set_kernel_table(ee_context* c, const ee_conv_params* cv, const float* radii, const float* cumkern,
                        const float* theta_deg, const float* phi_deg) {
    if (!c || !cv || !radii || !cumkern || !theta_deg || !phi_deg) return fail(EE_ERR_INVALID_ARG, "null argument");
    if (cv->ntheta <= 0 || cv->ntheta > EE_MAX_THETA || (cv->ntheta & 1))
        return fail(EE_ERR_INVALID_ARG, "ntheta must be even and <= %d", EE_MAX_THETA);
    int nrays = cv->nphi * (cv->ntheta / 2);
    if (cv->nphi <= 0 || nrays > EE_MAX_RAYS) return fail(EE_ERR_INVALID_ARG, "nphi*ntheta/2 must be in [1, %d]", EE_MAX_RAYS);
    if (cv->nradii <= 0 || cv->nradii > EE_MAX_RADII) return fail(EE_ERR_INVALID_ARG, "nradii must be in [1, %d]", EE_MAX_RADII);
    if (!(cv->rev_latspacing > 0) || !(cv->rev_longspacing > 0) || !(cv->penumbra >= 0))
        return fail(EE_ERR_INVALID_ARG, "bad convolution spacing/penumbra");
    std::lock_guard<std::mutex> lk(c->mu);
    EE_CUDA(cudaSetDevice(c->device));
    c->conv = *cv;
    EeParams& P = c->P;
    P.ntheta = cv->ntheta; P.nphi = cv->nphi; P.nradii = cv->nradii; P.nrays = nrays;
    for (int r = 0; r < cv->nradii; r++) P.radii[r] = radii[r];
    P.lat = cv->rev_latspacing; P.lng = cv->rev_longspacing; P.penumbra = cv->penumbra;
    for (int a = 0; a < 3; a++) P.max_rev[a] = cv->max_rev_size[a];
    derive_max_rev(c);
    size_t nk = (size_t)cv->ntheta * cv->nradii;
    EE_CUDA(c->cumkern.ensure(nk));
    EE_CUDA(cudaMemcpy(c->cumkern.p, cumkern, nk * sizeof(float), cudaMemcpyHostToDevice));
    P.cumkern = c->cumkern.p;
    c->rays.resize(nrays);
    for (int r = 0; r < nrays; r++) {
        EeRayConst& R = c->rays[r];
        double th = (double)theta_deg[r] * kPi / 180.0, ph = (double)phi_deg[r] * kPi / 180.0;
        R.th = (float)th; R.ph = (float)ph;
        R.row_fwd = r % (cv->ntheta / 2);
        R.row_rev = cv->ntheta - 1 - R.row_fwd;
        matrix_of([&](d3 v) { return rot_kern(v, th, ph); }, R.MK);
        matrix_of([&](d3 v) { return inv_rot_kern(v, th, ph); }, R.MKi);
    }
    EE_CUDA(c->d_rays.ensure(nrays));
    EE_CUDA(cudaMemcpy(c->d_rays.p, c->rays.data(), sizeof(EeRayConst) * nrays, cudaMemcpyHostToDevice));
    P.rays = c->d_rays.p;
    c->have_table = true;
    return EE_OK;
}

int ee_set_kernel_exp(ee_context* c, const float* params) {
    if (!c || !params) return fail(EE_ERR_INVALID_ARG, "null argument");
    if (!c->have_table) return fail(EE_ERR_NOT_READY, "call ee_set_kernel_table first (cone angles, radii)");
    std::lock_guard<std::mutex> lk(c->mu);
    for (int t = 0; t < c->P.ntheta; t++)
        if (!(params[4 * t + 1] > 0) || !(params[4 * t + 3] > 0))
            return fail(EE_ERR_INVALID_ARG, "exp kernel attenuation coefficients must be > 0");
    EE_CUDA(cudaSetDevice(c->device));
    EE_CUDA(c->expp.ensure((size_t)4 * c->P.ntheta));
    EE_CUDA(cudaMemcpy(c->expp.p, params, sizeof(float) * 4 * c->P.ntheta, cudaMemcpyHostToDevice));
    c->P.expp = c->expp.p;
    c->have_exp = true;
    c->P.mode = EE_KERNEL_EXP;
    return EE_OK;
}

int ee_set_kernel_mode(ee_context* c, int mode) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    if (mode != EE_KERNEL_TABLE && mode != EE_KERNEL_EXP && mode != EE_KERNEL_TABLE_WALK)
        return fail(EE_ERR_INVALID_ARG, "bad kernel mode %d", mode);
    if (mode == EE_KERNEL_EXP && !c->have_exp) return fail(EE_ERR_NOT_READY, "ee_set_kernel_exp has not been called");
    c->P.mode = mode;
    return EE_OK;
}

int ee_set_terma_supersampling(ee_context* c, int ss_factor) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    if (ss_factor < 1 || ss_factor > 8) return fail(EE_ERR_INVALID_ARG, "ss_factor %d outside [1, 8]", ss_factor);
    std::lock_guard<std::mutex> lk(c->mu);
    c->P.ss = ss_factor;
    return EE_OK;
}

int ee_beam_dose_device(ee_context* c, const ee_beam* beams, int nbeams, const float* d_fluence, float* d_dose,
                        int dose_mode) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    std::lock_guard<std::mutex> lk(c->mu);
    return dose_device(c, beams, nbeams, d_fluence, d_dose, dose_mode);
}

int ee_beam_dose(ee_context* c, const ee_beam* beams, int nbeams, const float* fluence, float* dose, int dose_mode) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    int st = check_ready(c);
    if (st) return st;
    if ((st = check_beams(beams, nbeams))) return st;
    if (!fluence || !dose) return fail(EE_ERR_INVALID_ARG, "null fluence/dose pointer");
    std::lock_guard<std::mutex> lk(c->mu);
    EE_CUDA(cudaSetDevice(c->device));
    long long nfl = total_fluence(beams, nbeams);
    long long nout = nfull_of(c) * (dose_mode == EE_DOSE_PER_BEAM ? nbeams : 1);
    EE_CUDA(c->io_fluence.ensure(nfl));
    EE_CUDA(c->io_dose.ensure(nout));
    EE_CUDA(cudaMemcpyAsync(c->io_fluence.p, fluence, sizeof(float) * nfl, cudaMemcpyHostToDevice, c->stream));
    if (dose_mode == EE_DOSE_ACCUMULATE)
        EE_CUDA(cudaMemcpyAsync(c->io_dose.p, dose, sizeof(float) * nout, cudaMemcpyHostToDevice, c->stream));
    st = dose_device(c, beams, nbeams, c->io_fluence.p, c->io_dose.p, dose_mode);
    if (st) return st;
    EE_CUDA(cudaMemcpyAsync(dose, c->io_dose.p, sizeof(float) * nout, cudaMemcpyDeviceToHost, c->stream));
    EE_CUDA(cudaStreamSynchronize(c->stream));
    return EE_OK;
}

int ee_beam_dose_adjoint_device(ee_context* c, const ee_beam* beams, int nbeams, const float* d_fluence,
                                const float* d_grad, float* d_fgrad) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    std::lock_guard<std::mutex> lk(c->mu);
    return adjoint_device(c, beams, nbeams, d_fluence, d_grad, d_fgrad);
}

int ee_beam_dose_adjoint(ee_context* c, const ee_beam* beams, int nbeams, const float* fluence, const float* grad,
                         float* fgrad) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    int st = check_ready(c);
    if (st) return st;
    if ((st = check_beams(beams, nbeams))) return st;
    if (!fluence || !grad || !fgrad) return fail(EE_ERR_INVALID_ARG, "null pointer");
    std::lock_guard<std::mutex> lk(c->mu);
    EE_CUDA(cudaSetDevice(c->device));
    long long nfl = total_fluence(beams, nbeams);
    long long nfull = nfull_of(c);
    EE_CUDA(c->io_fluence.ensure(nfl));
    EE_CUDA(c->io_grad.ensure(nfull + nfl));
    EE_CUDA(cudaMemcpyAsync(c->io_fluence.p, fluence, sizeof(float) * nfl, cudaMemcpyHostToDevice, c->stream));
    EE_CUDA(cudaMemcpyAsync(c->io_grad.p, grad, sizeof(float) * nfull, cudaMemcpyHostToDevice, c->stream));
    st = adjoint_device(c, beams, nbeams, c->io_fluence.p, c->io_grad.p, c->io_grad.p + nfull);
    if (st) return st;
    EE_CUDA(cudaMemcpyAsync(fgrad, c->io_grad.p + nfull, sizeof(float) * nfl, cudaMemcpyDeviceToHost, c->stream));
    EE_CUDA(cudaStreamSynchronize(c->stream));
    return EE_OK;
}

int ee_dose_and_adjoint_device(ee_context* c, const ee_beam* beams, int nbeams, const float* d_fluence, float* d_dose,
                               int dose_mode, const float* d_grad, float* d_fgrad) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    std::lock_guard<std::mutex> lk(c->mu);
    if ((d_fgrad == nullptr) != (d_grad == nullptr)) return fail(EE_ERR_INVALID_ARG, "adjoint needs both gradient pointers");
    PipeArgs A;
    A.beams = beams; A.nbeams = nbeams; A.d_fluence = d_fluence; A.d_dose = d_dose; A.dose_mode = dose_mode;
    A.d_dose_grad = d_grad; A.d_fgrad = d_fgrad;
    return pipeline(c, A);
}

int ee_dose_and_adjoint(ee_context* c, const ee_beam* beams, int nbeams, const float* fluence, float* dose, int dose_mode,
                        const float* grad, float* fgrad) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    int st = check_ready(c);
    if (st) return st;
    if ((st = check_beams(beams, nbeams))) return st;
    if (!fluence || (!dose && !fgrad) || ((fgrad == nullptr) != (grad == nullptr)))
        return fail(EE_ERR_INVALID_ARG, "null pointer");
    if (dose_mode < 0 || dose_mode > 2) return fail(EE_ERR_INVALID_ARG, "bad dose mode %d", dose_mode);
    std::lock_guard<std::mutex> lk(c->mu);
    EE_CUDA(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const long long nfl = total_fluence(beams, nbeams), nfull = nfull_of(c);
    const long long nout = dose ? nfull * (dose_mode == EE_DOSE_PER_BEAM ? nbeams : 1) : 0;
    EE_CUDA(grow(c, c->io_fluence, 2 * nfl));
    EE_CUDA(grow(c, c->io_dose, std::max(1ll, nout) + (grad ? nfull : 0)));
    EE_CUDA(cudaMemcpyAsync(c->io_fluence.p, fluence, sizeof(float) * nfl, cudaMemcpyHostToDevice, s));
    float* d_dose = dose ? c->io_dose.p : nullptr;
    float* d_grad = grad ? c->io_dose.p + std::max(1ll, nout) : nullptr;
    if (dose && dose_mode == EE_DOSE_ACCUMULATE)
        EE_CUDA(cudaMemcpyAsync(d_dose, dose, sizeof(float) * nout, cudaMemcpyHostToDevice, s));
    if (grad) EE_CUDA(cudaMemcpyAsync(d_grad, grad, sizeof(float) * nfull, cudaMemcpyHostToDevice, s));
    PipeArgs A;
    A.beams = beams; A.nbeams = nbeams; A.d_fluence = c->io_fluence.p; A.d_dose = d_dose; A.dose_mode = dose_mode;
    A.d_dose_grad = d_grad; A.d_fgrad = fgrad ? c->io_fluence.p + nfl : nullptr;
    st = pipeline(c, A);
    if (st) return st;
    if (dose) EE_CUDA(cudaMemcpyAsync(dose, d_dose, sizeof(float) * nout, cudaMemcpyDeviceToHost, s));
    if (fgrad) EE_CUDA(cudaMemcpyAsync(fgrad, c->io_fluence.p + nfl, sizeof(float) * nfl, cudaMemcpyDeviceToHost, s));
    EE_CUDA(cudaStreamSynchronize(s));
    return EE_OK;
}

int ee_loss_and_grad(ee_context* c, const ee_beam* beams, int nbeams, const float* d_x, const ee_loss* loss,
                     float* d_dose, float* d_xgrad, double loss_out[3]) {
    if (!c || !loss || !d_x || !d_dose || !d_xgrad) return fail(EE_ERR_INVALID_ARG, "null argument");
    if (!(loss->eta >= 0) || !(loss->spread_sigma >= 0)) return fail(EE_ERR_INVALID_ARG, "bad eta / spread sigma");
    if ((loss->ptv_weight == nullptr) != (loss->ptv_target == nullptr) ||
        (loss->oar_weight == nullptr) != (loss->oar_target == nullptr))
        return fail(EE_ERR_INVALID_ARG, "weight and target arrays come in pairs");
    int st = check_ready(c);
    if (st) return st;
    if ((st = check_beams(beams, nbeams))) return st;
    std::lock_guard<std::mutex> lk(c->mu);
    EE_CUDA(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    long long nfl = total_fluence(beams, nbeams);
    int max_pix = 1;
    for (int b = 0; b < nbeams; b++) max_pix = std::max(max_pix, beams[b].fmap_size[0] * beams[b].fmap_size[1]);
    EE_CUDA(grow(c, c->acc, 3));
    EE_CUDA(cudaMemsetAsync(c->acc.p, 0, 3 * sizeof(double), s));
    // fluence seen by the dose engine: G * x
    const float* f = d_x;
    int R = 0;
    if (loss->spread_sigma > 0) {
        R = (int)std::ceil(3.0 * loss->spread_sigma);
        std::vector<float> w(2 * R + 1);
        double sum = 0;
        for (int k = -R; k <= R; k++) sum += (w[k + R] = (float)std::exp(-0.5 * k * k / (loss->spread_sigma * loss->spread_sigma)));
        for (auto& v : w) v = (float)(v / sum);
        EE_CUDA(grow(c, c->spread_w, w.size()));
        EE_CUDA(cudaMemcpyAsync(c->spread_w.p, w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice, s));
        EE_CUDA(c->h_specs.ensure(nbeams));
        build_specs(c->P, beams, nbeams, c->h_specs.p);
        EE_CUDA(grow(c, c->d_specs, nbeams));
        EE_CUDA(cudaMemcpyAsync(c->d_specs.p, c->h_specs.p, sizeof(EeBeamSpec) * nbeams, cudaMemcpyHostToDevice, s));
        EE_CUDA(grow(c, c->xf, nfl));
        EE_CUDA(ee_launch_spread(c->d_specs.p, d_x, c->xf.p, c->spread_w.p, R, nbeams, max_pix, s));
        f = c->xf.p;
    }
    PipeArgs A;
    A.beams = beams; A.nbeams = nbeams; A.d_fluence = f; A.d_dose = d_dose; A.dose_mode = EE_DOSE_SUM;
    A.loss = loss; A.loss_acc = c->acc.p;
    float* fg = d_xgrad;
    if (R > 0) {
        EE_CUDA(grow(c, c->xg, nfl));
        fg = c->xg.p;
    }
    A.d_fgrad = fg;
    st = pipeline(c, A);
    if (st) return st;
    if (R > 0) EE_CUDA(ee_launch_spread(c->d_specs.p, c->xg.p, d_xgrad, c->spread_w.p, R, nbeams, max_pix, s));
    if (loss->eta > 0) EE_CUDA(ee_launch_smooth(c->d_specs.p, d_x, d_xgrad, loss->eta, c->acc.p, nbeams, max_pix, s));
    double h[3];
    EE_CUDA(cudaMemcpyAsync(h, c->acc.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    EE_CUDA(cudaStreamSynchronize(s));
    if (loss_out) for (int k = 0; k < 3; k++) loss_out[k] = h[k];
    return EE_OK;
}

int ee_plan_create(ee_context* c, const ee_beam* beams, int nbeams, const float* d_fluence, float* d_dose,
                   const float* d_dose_grad, float* d_fluence_grad, ee_plan** out) {
    if (!c || !out) return fail(EE_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    int st = check_ready(c);
    if (st) return st;
    if ((st = check_beams(beams, nbeams))) return st;
    if (!d_fluence || !d_dose) return fail(EE_ERR_INVALID_ARG, "null fluence/dose pointer");
    if ((d_dose_grad == nullptr) != (d_fluence_grad == nullptr))
        return fail(EE_ERR_INVALID_ARG, "adjoint needs both gradient pointers");
    std::lock_guard<std::mutex> lk(c->mu);
    EE_CUDA(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    std::unique_ptr<ee_plan> pl(new ee_plan());
    pl->c = c;
    pl->nbeams = nbeams;
    pl->adjoint = d_fluence_grad != nullptr;
    pl->beams.assign(beams, beams + nbeams);
    pl->specs.resize(nbeams);
    pl->d_fluence = d_fluence; pl->d_dose = d_dose; pl->d_grad = d_dose_grad; pl->d_fgrad = d_fluence_grad;
    build_specs(c->P, beams, nbeams, pl->specs.data());
    const bool expm = c->P.mode == EE_KERNEL_EXP;
    const long long per_float = 4ll * (1 + (expm ? 2 : 0) + (pl->adjoint ? 1 : 0));
    long long acc = 0;
    for (int b = 0; b < nbeams; b++) {
        EeBeamSpec& S = pl->specs[b];
        PlanBound B = plan_bound(c, S);
        long long need = B.rev * per_float;
        if (pl->starts.empty() || (acc + need > c->max_batch_bytes && acc > 0)) {
            pl->starts.push_back(b);
            pl->dims.push_back(ChunkDims());
            acc = 0;
        }
        ChunkDims& D = pl->dims.back();
        S.plan_off = D.rev_total;
        S.plan_cap = B.rev;
        S.t_off = pl->tvol_total;
        D.rev_total += B.rev;
        D.max_tvol = std::max(D.max_tvol, tvol_of(S));
        D.max_line = std::max(D.max_line, B.max_line);
        D.max_lines = std::max(D.max_lines, B.max_lines);
        D.max_rows = std::max(D.max_rows, B.rows);
        D.max_tiles = std::max(D.max_tiles, B.tiles);
        pl->tvol_total += tvol_of(S);
        pl->rev_max = std::max(pl->rev_max, D.rev_total);
        acc += need;
    }
    pl->starts.push_back(nbeams);
    pl->nfl = total_fluence(beams, nbeams);
    EE_CUDA(pl->d_specs.ensure(nbeams));
    EE_CUDA(pl->d_geoms.ensure(nbeams));
    EE_CUDA(pl->terma.ensure(pl->tvol_total));
    EE_CUDA(pl->rev.ensure(pl->rev_max));
    if (expm) EE_CUDA(pl->samples.ensure(pl->rev_max));
    if (pl->adjoint) {
        EE_CUDA(pl->unit.ensure(pl->tvol_total));
        EE_CUDA(pl->bl_idx.ensure(pl->tvol_total));
        EE_CUDA(pl->terma_grad.ensure(pl->tvol_total + 4));
        EE_CUDA(pl->rev_grad.ensure(pl->rev_max + 4));
    }
    EE_CUDA(cudaMemcpyAsync(pl->d_specs.p, pl->specs.data(), sizeof(EeBeamSpec) * nbeams, cudaMemcpyHostToDevice, s));
    pl->status.resize(nbeams);
    // eager run: validates the bounds and sets kernel attributes before capture
    EE_CUDA(plan_enqueue(pl.get(), s));
    EE_CUDA(ee_copy_status(pl->d_geoms.p, pl->status.data(), nbeams, s));
    EE_CUDA(cudaStreamSynchronize(s));
    for (int b = 0; b < nbeams; b++)
        if (pl->status[b] != 0) return fail(pl->status[b], "beam %d: %s", b, status_text(pl->status[b]));
    // autotune the lane kernels' block size on this batch
    if (expm) {
        cudaEvent_t e0 = take_event(c), e1 = take_event(c);
        float best = 1e30f;
        int best_lb = 128;
        for (int lb : {64, 128, 256}) {
            pl->lane_block = lb;
            cudaEventRecord(e0, s);
            EE_CUDA(plan_enqueue(pl.get(), s));
            cudaEventRecord(e1, s);
            EE_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) { best = ms; best_lb = lb; }
        }
        pl->lane_block = best_lb;
        c->event_pool.push_back(e0);
        c->event_pool.push_back(e1);
    }
    EE_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    cudaError_t ce = plan_enqueue(pl.get(), s);
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(s, &g);
    if (ce != cudaSuccess) { if (g) cudaGraphDestroy(g); return fail(EE_ERR_CUDA, "plan capture: %s", cudaGetErrorString(ce)); }
    if (ee != cudaSuccess) return fail(EE_ERR_CUDA, "plan capture: %s", cudaGetErrorString(ee));
    pl->graph = g;
    EE_CUDA(cudaGraphInstantiate(&pl->exec, g, 0));
    *out = pl.release();
    return EE_OK;
}

int ee_plan_launch(ee_plan* pl) {
    if (!pl) return fail(EE_ERR_INVALID_ARG, "null plan");
    EE_CUDA(cudaSetDevice(pl->c->device));
    EE_CUDA(cudaGraphLaunch(pl->exec, pl->c->stream));
    return EE_OK;
}

int ee_plan_status(ee_plan* pl, int* nfailed) {
    if (!pl) return fail(EE_ERR_INVALID_ARG, "null plan");
    EE_CUDA(cudaSetDevice(pl->c->device));
    EE_CUDA(ee_copy_status(pl->d_geoms.p, pl->status.data(), pl->nbeams, pl->c->stream));
    EE_CUDA(cudaStreamSynchronize(pl->c->stream));
    int n = 0, first = -1;
    for (int b = 0; b < pl->nbeams; b++)
        if (pl->status[b] != 0) { n++; if (first < 0) first = b; }
    if (nfailed) *nfailed = n;
    if (n) return fail(pl->status[first], "beam %d: %s", first, status_text(pl->status[first]));
    return EE_OK;
}

int ee_plan_info(ee_plan* pl, int* lane_block, long long* device_bytes, int* nchunks) {
    if (!pl) return fail(EE_ERR_INVALID_ARG, "null plan");
    if (lane_block) *lane_block = pl->lane_block;
    if (nchunks) *nchunks = (int)pl->starts.size() - 1;
    if (device_bytes) {
        long long b = 4ll * (pl->tvol_total + pl->rev_max) + 8ll * pl->samples.n;
        if (pl->adjoint) b += 4ll * (3 * pl->tvol_total + pl->rev_max);
        *device_bytes = b;
    }
    return EE_OK;
}

int ee_plan_destroy(ee_plan* pl) {
    if (!pl) return EE_OK;
    cudaSetDevice(pl->c->device);
    cudaStreamSynchronize(pl->c->stream);
    delete pl;
    return EE_OK;
}

int ee_get_beam_info(ee_context* c, int i, ee_beam_info* info) {
    if (!c || !info) return fail(EE_ERR_INVALID_ARG, "null argument");
    if (i < 0 || i >= (int)c->last_geoms.size()) return fail(EE_ERR_INVALID_ARG, "beam index %d out of range", i);
    const EeBeamGeom& G = c->last_geoms[i];
    const EeBeamSpec& S = c->last_specs[i];
    std::memset(info, 0, sizeof(*info));
    for (int a = 0; a < 3; a++) {
        info->source[a] = S.src[a];
        info->direction[a] = S.dir[a];
        info->b_min[a] = G.bmin[a];
        info->bev_size[a] = G.bev[a];
        info->lim_min[a] = G.lim_min[a];
    }
    info->v_beam = G.v_beam;
    info->rev_samples = G.rev_total;
    info->terma_nonzero = G.nnz;
    info->max_line = G.max_line;
    info->status = G.status;
    return EE_OK;
}

int ee_synchronize(ee_context* c) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    EE_CUDA(cudaStreamSynchronize(c->stream));
    return EE_OK;
}

void* ee_get_stream(ee_context* c) { return c ? (void*)c->stream : nullptr; }

int ee_set_scratch_limit(ee_context* c, long long bytes) {
    if (!c || bytes <= 0) return fail(EE_ERR_INVALID_ARG, "bad scratch limit");
    std::lock_guard<std::mutex> lk(c->mu);
    c->max_batch_bytes = bytes;
    return EE_OK;
}

int ee_set_profiling(ee_context* c, int enable) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    std::lock_guard<std::mutex> lk(c->mu);
    drain_profile(c);
    c->profiling = enable != 0;
    return EE_OK;
}

int ee_read_profile(ee_context* c, double* ms, long long* launches, int n) {
    if (!c) return fail(EE_ERR_INVALID_ARG, "null context");
    std::lock_guard<std::mutex> lk(c->mu);
    drain_profile(c);
    for (int i = 0; i < n && i < EE_NSTAGES; i++) {
        if (ms) ms[i] = c->stage_ms[i];
        if (launches) launches[i] = c->stage_launches[i];
    }
    for (int i = 0; i < EE_NSTAGES; i++) {
        c->stage_ms[i] = 0;
        c->stage_launches[i] = 0;
    }
    return EE_OK;
}

int ee_beam_source(const ee_beam* b, float source[3], float direction[3]) {
    if (!b || !source || !direction) return fail(EE_ERR_INVALID_ARG, "null argument");
    double az, zen;
    d3 s, d;
    reconfigure(*b, az, zen, s, d);
    source[0] = (float)s.x; source[1] = (float)s.y; source[2] = (float)s.z;
    direction[0] = (float)d.x; direction[1] = (float)d.y; direction[2] = (float)d.z;
    return EE_OK;
}

// ---- beamlet dose columns (dosecalc-beamlet) ----
int ee_set_beamlet_options(ee_context* c, float kernel_extent_cm, const int max_rev_size[3]) {
    if (!c || !(kernel_extent_cm >= 0.f)) return fail(EE_ERR_INVALID_ARG, "bad beamlet options");
    std::lock_guard<std::mutex> lk(c->mu);
    c->bl_opt.kernel_extent = kernel_extent_cm;
    if (max_rev_size)
        for (int a = 0; a < 3; a++) {
            if (max_rev_size[a] <= 0) return fail(EE_ERR_INVALID_ARG, "bad max_rev_size");
            c->bl_opt.max_rev[a] = max_rev_size[a];
        }
    return EE_OK;
}

int ee_beamlet_columns_device(ee_context* c, const ee_beam* beam, const float* fluence, float thresh, ee_csr* out) {
    int st = check_ready(c);
    if (st) return st;
    if (!out || !fluence) return fail(EE_ERR_INVALID_ARG, "null argument");
    if ((st = check_beams(beam, 1))) return st;
    if (!(thresh >= 0.f)) return fail(EE_ERR_INVALID_ARG, "threshold must be >= 0");
    std::lock_guard<std::mutex> lk(c->mu);
    cudaSetDevice(c->device);
    EeBeamSpec S;
    build_specs(c->P, beam, 1, &S);
    return ee_beamlet_run(c->P, c->rays.data(), c->stream, &c->beamlet_ws, c->bl_opt, *beam, S, fluence, thresh, out);
}

int ee_copy_to_host(ee_context* c, void* dst, const void* src, long long bytes) {
    if (!c || (bytes > 0 && (!dst || !src)) || bytes < 0) return fail(EE_ERR_INVALID_ARG, "bad copy arguments");
    if (bytes == 0) return EE_OK;
    std::lock_guard<std::mutex> lk(c->mu);
    EE_CUDA(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost, c->stream));
    EE_CUDA(cudaStreamSynchronize(c->stream));
    return EE_OK;
}

int ee_beamlet_columns(ee_context* c, const ee_beam* beam, const float* fluence, float thresh, long long capacity,
                       int* beamlet_index, long long* col_ptr, int* row_index, float* value, long long* nnz,
                       int* nbeamlets) {
    if (!beamlet_index || !col_ptr || !nnz || !nbeamlets) return fail(EE_ERR_INVALID_ARG, "null argument");
    ee_csr d;
    int st = ee_beamlet_columns_device(c, beam, fluence, thresh, &d);
    if (st) return st;
    *nnz = d.nnz;
    *nbeamlets = d.nbeamlets;
    std::lock_guard<std::mutex> lk(c->mu);
    EE_CUDA(cudaMemcpy(beamlet_index, d.beamlet_index, sizeof(int) * d.nbeamlets, cudaMemcpyDeviceToHost));
    EE_CUDA(cudaMemcpy(col_ptr, d.col_ptr, sizeof(long long) * ((size_t)d.nbeamlets + 1), cudaMemcpyDeviceToHost));
    if (d.nnz > capacity) return fail(EE_ERR_CAPACITY, "CSR needs %lld entries, capacity %lld", d.nnz, capacity);
    if (d.nnz > 0) {
        if (!row_index || !value) return fail(EE_ERR_INVALID_ARG, "null CSR output");
        EE_CUDA(cudaMemcpy(row_index, d.row_index, sizeof(int) * d.nnz, cudaMemcpyDeviceToHost));
        EE_CUDA(cudaMemcpy(value, d.value, sizeof(float) * d.nnz, cudaMemcpyDeviceToHost));
    }
    return EE_OK;
}

}  // extern "C"

// ------------------------------------------------ internal accessors ----
// Used by ee_noalloc.cu: a copy of the context's kernel parameters (device
// pointers to its resident density and kernel tables) and the host-side
// beam set-up, so that file's entry point needs no context scratch.
int ee_internal_snapshot(ee_context* c, EeParams* P, int* device) {
    int st = check_ready(c);
    if (st) return st;
    std::lock_guard<std::mutex> lk(c->mu);
    *P = c->P;
    *device = c->device;
    return EE_OK;
}

void ee_internal_build_spec(const EeParams& P, const ee_beam& beam, EeBeamSpec* out) { build_specs(P, &beam, 1, out); }

const char* ee_internal_status_text(int st) { return status_text(st); }

int ee_internal_fail(int code, const char* msg) { return fail(code, "%s", msg); }

// Grouped forward (+adjoint) used by the request server: beam b's dose is
// summed into volume group[b] of d_dose (ngroups volumes) and its adjoint
// reads volume group[b] of d_dose_grad.
int ee_internal_pipeline_grouped(ee_context* c, const ee_beam* beams, int nbeams, const float* d_fluence, float* d_dose,
                                 const int* group, int ngroups, const float* d_dose_grad, float* d_fgrad) {
    std::lock_guard<std::mutex> lk(c->mu);
    PipeArgs A;
    A.beams = beams; A.nbeams = nbeams; A.d_fluence = d_fluence; A.d_dose = d_dose; A.dose_mode = EE_DOSE_SUM;
    A.d_dose_grad = d_dose_grad; A.d_fgrad = d_fgrad; A.group = group; A.ngroups = ngroups;
    return pipeline(c, A);
}

// Device bytes the context's resident data and scratch occupy.
long long ee_internal_context_bytes(ee_context* c) {
    std::lock_guard<std::mutex> lk(c->mu);
    long long b = 0;
    b += 4ll * (c->density.n + c->cumkern.n + c->expp.n + c->terma.n + c->unit.n + c->rev.n + c->rev_grad.n +
                c->terma_grad.n + c->io_fluence.n + c->io_dose.n + c->io_grad.n + c->xf.n + c->xg.n + c->spread_w.n +
                c->bl_idx.n);
    b += 8ll * (c->samples.n + c->acc.n);
    b += (long long)sizeof(EeBeamSpec) * c->d_specs.n + (long long)sizeof(EeBeamGeom) * c->d_geoms.n;
    if (c->dens_array) b += 4ll * c->density.n;
    return b;
}
