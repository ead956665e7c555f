// ee_preprocess.cu -- the GPU steps of dosecalc-preprocess that feed the
// dose engine: CT (HU) -> isotropic density, and the conformal fluence maps
// projected from the PTV mask.
//
//   k_iso_density  one thread per output voxel: the CT sampled through a
//                  border-0 linear 3-D texture at the isotropic voxel centre,
//                  then the HU -> density table (or the linear HU rule)
//                  (dosecalc-preprocess/kernels.cuh:12-102).
//   k_fluence_proj one thread per (beam, fluence pixel): up to nine sub-rays
//                  traced through the PTV mask texture with the Siddon walk
//                  (kernels.cuh:138-224); all beams of a call in one launch.
//   k_aperture     one thread per fluence-map row: zero pixels between the
//                  row's first and last open pixel are opened
//                  (fmapProcessing.cpp:33-48).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/ee_cccs.h"
#include "ee_device.cuh"
#include "ee_internal.h"

int ee_internal_fail(int code, const char* msg);
void ee_internal_build_spec(const EeParams& P, const ee_beam& beam, EeBeamSpec* out);

namespace {

constexpr int PP_MAX_LUT = 64;

__global__ void __launch_bounds__(256) k_iso_density(cudaTextureObject_t tex, float3 ct_voxel, float iso_voxel,
                                                     uint3 os, const float* __restrict__ lut_hu,
                                                     const float* __restrict__ lut_d, int nlut,
                                                     float* __restrict__ out) {
    __shared__ float sh[PP_MAX_LUT], sd[PP_MAX_LUT];
    for (int k = threadIdx.x; k < nlut; k += blockDim.x) {
        sh[k] = lut_hu[k];
        sd[k] = lut_d[k];
    }
    __syncthreads();
    const unsigned long long v = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long n = (unsigned long long)os.x * os.y * os.z;
    if (v >= n) return;
    const unsigned X = (unsigned)(v % os.x), Y = (unsigned)((v / os.x) % os.y),
                   Z = (unsigned)(v / ((unsigned long long)os.x * os.y));
    // position in CT texels: (X, Y, Z) * iso_voxel / ct_voxel, + 0.5 centre shift
    const float px = ((float)X * iso_voxel) / ct_voxel.x, py = ((float)Y * iso_voxel) / ct_voxel.y,
                pz = ((float)Z * iso_voxel) / ct_voxel.z;
    float val = tex3D<float>(tex, px + 0.5f, py + 0.5f, pz + 0.5f);
    if (nlut > 0) {
        if (val <= sh[0]) val = sd[0];
        else if (val >= sh[nlut - 1])
            val = sd[nlut - 2] + (val - sh[nlut - 2]) * (sd[nlut - 1] - sd[nlut - 2]) / (sh[nlut - 1] - sh[nlut - 2]);
        else {
            int lo = 0;
            while (sh[lo] < val && lo < nlut - 1) lo++;
            lo--;
            val = sd[lo] + (val - sh[lo]) * (sd[lo + 1] - sd[lo]) / (sh[lo + 1] - sh[lo]);
        }
    } else {
        val = (val + 1024.0f) / 1024.0f;
        if (val < 0.05f) val = 0.05f;
    }
    out[v] = val;
}

__global__ void __launch_bounds__(256) k_fluence_proj(EeParams M, const EeBeamSpec* __restrict__ specs,
                                                      int supersample, float* __restrict__ out, int* __restrict__ status) {
    const EeBeamSpec& S = specs[blockIdx.y];
    const int fx = S.fmap[0], fy = S.fmap[1];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fx * fy) return;
    const int X = p % fx, Z = p / fx;
    const f3 src = ld3(S.src), iso = ld3(S.iso);
    const int nsub = supersample ? 9 : 1;
    bool hit = false, cap = false;
    for (int k = 0; k < nsub && !hit; k++) {
        const int sx = supersample ? k % 3 - 1 : 0, sz = supersample ? k / 3 - 1 : 0;
        const f3 fcs = mk(S.beamlet[0] * ((float)X + 0.5f * (float)sx - (float)fx * 0.5f + 0.5f), 0.f,
                          S.beamlet[1] * ((float)Z + 0.5f * (float)sz - (float)fy * 0.5f + 0.5f));
        f3 c = mv(S.MBi, fcs) + iso;
        c = mk(c.x + 1e-9f, c.y + 1e-9f, c.z + 1e-9f);
        const f3 sink = src + (c - src) * 3.f;
        hit = siddon_rpl(M, sink, src, cap) > 0.f;
    }
    out[S.fl_off + p] = hit ? 1.f : 0.f;
    if (cap) atomicOr(status, 1);
}

__global__ void k_aperture(const EeBeamSpec* __restrict__ specs, float* __restrict__ fl, float fill) {
    const EeBeamSpec& S = specs[blockIdx.y];
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= S.fmap[1]) return;
    float* row = fl + S.fl_off + (long long)S.fmap[0] * y;
    int a = -1, z = -1;
    for (int x = 0; x < S.fmap[0]; x++)
        if (row[x] != 0.f) {
            if (a < 0) a = x;
            z = x;
        }
    for (int x = a + 1; a >= 0 && x < z; x++)
        if (row[x] == 0.f) row[x] = fill;
}

// 3-D float texture (linear filter, border 0, unnormalised) of a host volume
struct Tex3 {
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    cudaError_t make(const float* host, int nx, int ny, int nz) {
        cudaChannelFormatDesc cd = cudaCreateChannelDesc<float>();
        cudaExtent ext = make_cudaExtent(nx, ny, nz);
        cudaError_t e = cudaMalloc3DArray(&arr, &cd, ext);
        if (e != cudaSuccess) return e;
        cudaMemcpy3DParms cp = {};
        cp.srcPtr = make_cudaPitchedPtr((void*)host, sizeof(float) * nx, nx, ny);
        cp.dstArray = arr;
        cp.extent = ext;
        cp.kind = cudaMemcpyHostToDevice;
        if ((e = cudaMemcpy3D(&cp)) != cudaSuccess) return e;
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        cudaTextureDesc td = {};
        td.normalizedCoords = 0;
        td.filterMode = cudaFilterModeLinear;
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
        td.readMode = cudaReadModeElementType;
        return cudaCreateTextureObject(&tex, &rd, &td, nullptr);
    }
    ~Tex3() {
        if (tex) cudaDestroyTextureObject(tex);
        if (arr) cudaFreeArray(arr);
    }
};

template <class T>
struct DBuf {
    T* p = nullptr;
    cudaError_t alloc(size_t n) { return cudaMalloc((void**)&p, std::max<size_t>(n, 1) * sizeof(T)); }
    ~DBuf() {
        if (p) cudaFree(p);
    }
};

#define PP_CUDA(call)                                                        \
    do {                                                                     \
        cudaError_t _e = (call);                                             \
        if (_e != cudaSuccess) return ee_internal_fail(EE_ERR_CUDA, #call); \
    } while (0)

int set_device(int device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "device out of range");
    PP_CUDA(cudaSetDevice(device));
    return EE_OK;
}

}  // namespace

extern "C" {

int ee_ct_to_density(int device, const ee_frame* ct, const float* hu, float iso_voxel_cm, const float* lut_hu,
                     const float* lut_density, int nlut, float* density, int out_size[3]) {
    if (!ct || !out_size || !(iso_voxel_cm > 0.f) || nlut < 0 || nlut > PP_MAX_LUT || nlut == 1 ||
        (nlut > 0 && (!lut_hu || !lut_density)))
        return ee_internal_fail(EE_ERR_INVALID_ARG, "bad CT conversion arguments");
    for (int a = 0; a < 3; a++)
        if (ct->size[a] <= 0 || !(ct->voxel[a] > 0.f)) return ee_internal_fail(EE_ERR_INVALID_ARG, "bad CT frame");
    for (int i = 1; i < nlut; i++)
        if (!(lut_hu[i] > lut_hu[i - 1])) return ee_internal_fail(EE_ERR_INVALID_ARG, "LUT HU values must ascend");
    // float2uint_ceil(voxsize * (size / iso_voxel)) (cudaMemFunctions.cu:128)
    for (int a = 0; a < 3; a++) out_size[a] = (int)ceilf(ct->voxel[a] * ((float)ct->size[a] / iso_voxel_cm));
    if (!density) return EE_OK;  // size query
    if (!hu) return ee_internal_fail(EE_ERR_INVALID_ARG, "null CT");
    int st = set_device(device);
    if (st) return st;
    Tex3 T;
    PP_CUDA(T.make(hu, ct->size[0], ct->size[1], ct->size[2]));
    const unsigned long long n = (unsigned long long)out_size[0] * out_size[1] * out_size[2];
    DBuf<float> d_out, d_lh, d_ld;
    PP_CUDA(d_out.alloc(n));
    PP_CUDA(d_lh.alloc(nlut));
    PP_CUDA(d_ld.alloc(nlut));
    if (nlut > 0) {
        PP_CUDA(cudaMemcpy(d_lh.p, lut_hu, sizeof(float) * nlut, cudaMemcpyHostToDevice));
        PP_CUDA(cudaMemcpy(d_ld.p, lut_density, sizeof(float) * nlut, cudaMemcpyHostToDevice));
    }
    k_iso_density<<<(unsigned)((n + 255) / 256), 256>>>(T.tex, make_float3(ct->voxel[0], ct->voxel[1], ct->voxel[2]),
                                                         iso_voxel_cm,
                                                         make_uint3(out_size[0], out_size[1], out_size[2]), d_lh.p,
                                                         d_ld.p, nlut, d_out.p);
    PP_CUDA(cudaGetLastError());
    PP_CUDA(cudaMemcpy(density, d_out.p, sizeof(float) * n, cudaMemcpyDeviceToHost));
    return EE_OK;
}

int ee_fluence_projection(int device, const ee_frame* mask_frame, const float* mask, const ee_beam* beams, int nbeams,
                          int supersample, int aperture_ready, float* fluence) {
    if (!mask_frame || !mask || !beams || nbeams <= 0 || nbeams > 65535 || !fluence)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "bad projection arguments");
    for (int a = 0; a < 3; a++)
        if (mask_frame->size[a] <= 0 || !(mask_frame->voxel[a] > 0.f))
            return ee_internal_fail(EE_ERR_INVALID_ARG, "bad mask frame");
    int st = set_device(device);
    if (st) return st;
    Tex3 T;
    PP_CUDA(T.make(mask, mask_frame->size[0], mask_frame->size[1], mask_frame->size[2]));
    EeParams M;
    std::memset(&M, 0, sizeof(M));
    for (int a = 0; a < 3; a++) {
        M.size[a] = mask_frame->size[a];
        M.voxel[a] = mask_frame->voxel[a];
        M.start[a] = mask_frame->start[a];
        M.bb0[a] = 0;
        M.bbs[a] = mask_frame->size[a];
    }
    M.dens_tex = T.tex;
    std::vector<EeBeamSpec> h(nbeams);
    long long off = 0;
    int max_pix = 1, max_rows = 1;
    for (int b = 0; b < nbeams; b++) {
        if (beams[b].fmap_size[0] <= 0 || beams[b].fmap_size[1] <= 0 || !(beams[b].beamlet_size[0] > 0.f) ||
            !(beams[b].beamlet_size[1] > 0.f) || !(beams[b].sad > 0.f))
            return ee_internal_fail(EE_ERR_INVALID_ARG, "bad beam");
        ee_internal_build_spec(M, beams[b], &h[b]);
        h[b].fl_off = off;
        off += (long long)beams[b].fmap_size[0] * beams[b].fmap_size[1];
        max_pix = std::max(max_pix, beams[b].fmap_size[0] * beams[b].fmap_size[1]);
        max_rows = std::max(max_rows, beams[b].fmap_size[1]);
    }
    DBuf<EeBeamSpec> d_specs;
    DBuf<float> d_fl;
    DBuf<int> d_st;
    PP_CUDA(d_specs.alloc(nbeams));
    PP_CUDA(d_fl.alloc(off));
    PP_CUDA(d_st.alloc(1));
    PP_CUDA(cudaMemset(d_st.p, 0, sizeof(int)));
    PP_CUDA(cudaMemcpy(d_specs.p, h.data(), sizeof(EeBeamSpec) * nbeams, cudaMemcpyHostToDevice));
    k_fluence_proj<<<dim3((max_pix + 255) / 256, nbeams), 256>>>(M, d_specs.p, supersample ? 1 : 0, d_fl.p, d_st.p);
    PP_CUDA(cudaGetLastError());
    if (aperture_ready) {
        k_aperture<<<dim3((max_rows + 127) / 128, nbeams), 128>>>(d_specs.p, d_fl.p, 1.f);
        PP_CUDA(cudaGetLastError());
    }
    int hst = 0;
    PP_CUDA(cudaMemcpy(&hst, d_st.p, sizeof(int), cudaMemcpyDeviceToHost));
    PP_CUDA(cudaMemcpy(fluence, d_fl.p, sizeof(float) * off, cudaMemcpyDeviceToHost));
    if (hst) return ee_internal_fail(EE_ERR_SIDDON_ITER, "Siddon ray trace hit its iteration cap");
    return EE_OK;
}

}  // extern "C"
