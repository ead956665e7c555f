// ee_noalloc.cu -- ee_beam_dose_noalloc: the single-beam forward dose with
// every intermediate (beam spec, crop-box/REV geometry, TERMA box, REV dose
// arena) placed in one file-scope device array instead of cudaMalloc'd
// buffers.
//
// It exists for callers that must not allocate device memory per call: a
// service whose GPU memory is carved up in advance (a caching allocator such
// as PyTorch's owns the pool, or a hard per-process budget is enforced), a
// real-time loop where cudaMalloc/cudaFree would stall or synchronise the
// device, or a plug-in host that forbids new allocations after start-up.
// Such a caller sets the context up once (ee_create/ee_set_* allocate the
// resident density and kernel tables) and then calls this entry point as
// often as it likes: it calls no cudaMalloc, cudaFree or other allocating
// routine.
//
// Limits and sharing rules:
//  * The array holds EE_NOALLOC_SCRATCH_BYTES (64 MiB) on every GPU that loads
//    the library, for the life of the process.  A beam whose TERMA box plus
//    REV arena does not fit is rejected with EE_ERR_CAPACITY (the message
//    gives the sizes); the beam-dose sizes of a 64^3 phantom at 2.5 mm fit.
//  * Every call shares the one array and it keeps the last call's contents;
//    everything that must start at zero is cleared by the call itself.
//    Calls whose work overlaps on the GPU (different streams, or different
//    host threads on one stream without ordering) race on the array.
//  * The first call on a device looks the array's device address up with
//    cudaGetSymbolAddress (that device current); make that first call before
//    any stream capture.
//  * Every call reads the beam's crop box back to the host and waits for the
//    caller's stream before it returns.  The kernels run on that stream and
//    read the context's density texture and kernel tables, which ee_set_* and
//    ee_destroy release after synchronising only the context's own stream:
//    the caller synchronises its stream before either.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/ee_cccs.h"
#include "ee_internal.h"

int ee_internal_snapshot(ee_context* c, EeParams* P, int* device);
void ee_internal_build_spec(const EeParams& P, const ee_beam& beam, EeBeamSpec* out);
const char* ee_internal_status_text(int st);
int ee_internal_fail(int code, const char* msg);

#define EE_NOALLOC_SCRATCH_BYTES (64ull << 20)
#define EE_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char ee_noalloc_scratch[EE_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_addr_mu;
void* g_addr[EE_NOALLOC_MAX_DEVICES] = {nullptr};

// Device address of the scratch array on `device` (which is current).
int scratch_address(int device, unsigned char** out) {
    if (device < 0 || device >= EE_NOALLOC_MAX_DEVICES) return ee_internal_fail(EE_ERR_INVALID_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, ee_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            char m[256];
            snprintf(m, sizeof(m), "cudaGetSymbolAddress(ee_noalloc_scratch) failed: %s", cudaGetErrorString(e));
            return ee_internal_fail(EE_ERR_CUDA, m);
        }
        g_addr[device] = p;
    }
    *out = (unsigned char*)g_addr[device];
    return EE_OK;
}

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

int cuda_fail(cudaError_t e, const char* what) {
    char m[256];
    snprintf(m, sizeof(m), "%s failed: %s", what, cudaGetErrorString(e));
    return ee_internal_fail(EE_ERR_CUDA, m);
}

}  // namespace

extern "C" int ee_beam_dose_noalloc(ee_context* ctx, const ee_beam* beam, const float* d_fluence, float* d_dose,
                                    void* stream) {
    if (!ctx || !beam || !d_fluence || !d_dose) return ee_internal_fail(EE_ERR_INVALID_ARG, "null argument");
    if (beam->fmap_size[0] <= 0 || beam->fmap_size[1] <= 0 || !(beam->beamlet_size[0] > 0) ||
        !(beam->beamlet_size[1] > 0) || !(beam->sad > 0))
        return ee_internal_fail(EE_ERR_INVALID_ARG, "invalid fluence map / beamlet size / SAD");
    EeParams P;
    int device = 0;
    int st = ee_internal_snapshot(ctx, &P, &device);
    if (st) return st;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    unsigned char* base = nullptr;
    if ((st = scratch_address(device, &base))) return st;
    cudaStream_t s = (cudaStream_t)stream;

    // scratch layout: [spec][geometry][TERMA box floats][REV arena floats]
    EeBeamSpec S;
    ee_internal_build_spec(P, *beam, &S);
    S.fl_off = 0;
    S.t_off = 0;
    const size_t off_geom = align256(sizeof(EeBeamSpec));
    const size_t off_terma = off_geom + align256(sizeof(EeBeamGeom));
    const long long tvol = ee_brick_vol(S.tn);  // bricked TERMA box
    const size_t cap_floats = (EE_NOALLOC_SCRATCH_BYTES - off_terma) / sizeof(float);
    if ((size_t)tvol > cap_floats) {
        char m[256];
        snprintf(m, sizeof(m), "TERMA box of %lld voxels exceeds the %llu-byte no-alloc scratch", tvol,
                 (unsigned long long)EE_NOALLOC_SCRATCH_BYTES);
        return ee_internal_fail(EE_ERR_CAPACITY, m);
    }
    EeBeamSpec* d_spec = (EeBeamSpec*)base;
    EeBeamGeom* d_geom = (EeBeamGeom*)(base + off_geom);
    float* d_terma = (float*)(base + off_terma);
    if ((e = cudaMemcpyAsync(d_spec, &S, sizeof(S), cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "spec upload");
    if ((e = ee_launch_geom_init(d_spec, d_geom, 1, s)) != cudaSuccess) return cuda_fail(e, "k_geom_init");
    if ((e = ee_launch_terma(P, d_spec, d_geom, d_fluence, d_terma, nullptr, nullptr, 1, tvol > 0 ? tvol : 1, s)) !=
        cudaSuccess)
        return cuda_fail(e, "k_terma");
    if ((e = ee_launch_geometry(P, d_spec, d_geom, 1, s)) != cudaSuccess) return cuda_fail(e, "k_geometry");
    EeBeamGeom G;  // host copy of the geometry (about 11 KB on the stack)
    if ((e = cudaMemcpyAsync(&G, d_geom, sizeof(G), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_fail(e, "geometry read-back");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    if (G.status != 0) return ee_internal_fail(G.status, ee_internal_status_text(G.status));
    if ((size_t)(tvol + G.rev_total) > cap_floats) {
        char m[256];
        snprintf(m, sizeof(m), "TERMA box (%lld) + REV arena (%lld floats) exceed the %llu-byte no-alloc scratch", tvol,
                 G.rev_total, (unsigned long long)EE_NOALLOC_SCRATCH_BYTES);
        return ee_internal_fail(EE_ERR_CAPACITY, m);
    }
    G.arena_off = 0;
    G.arena_cap = G.rev_total;
    if ((e = cudaMemcpyAsync(d_geom, &G, sizeof(G), cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "geometry upload");
    float* d_rev = d_terma + tvol;
    const long long nfull = (long long)P.size[0] * P.size[1] * P.size[2];
    if ((e = cudaMemsetAsync(d_dose, 0, sizeof(float) * nfull, s)) != cudaSuccess) return cuda_fail(e, "dose clear");
    if ((e = cudaMemsetAsync(d_rev, 0, sizeof(float) * G.rev_total, s)) != cudaSuccess) return cuda_fail(e, "REV clear");
    // no (rho, T) sample scratch here: the warp-per-line cone kernel keeps a
    // line's samples in shared memory instead
    float2* d_smp = nullptr;
    if ((e = ee_launch_cone(P, d_spec, d_geom, d_terma, d_rev, d_smp, 1, G.max_lines, G.max_line, s)) != cudaSuccess)
        return cuda_fail(e, "k_cone");
    if ((e = ee_launch_gather(P, d_spec, d_geom, d_rev, d_dose, 1, 1, G.rows > 0 ? G.rows : 1, s)) != cudaSuccess)
        return cuda_fail(e, "k_gather");
    // G may go out of scope now: a cudaMemcpyAsync from pageable host memory
    // has consumed its source when it returns
    return EE_OK;
}
