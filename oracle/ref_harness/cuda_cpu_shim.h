// cuda_cpu_shim.h -- just enough of the CUDA device environment to compile
// the reference's kernel source files unmodified with a host C++ compiler
// and execute them on the CPU (test infrastructure: the reference harness).
//
// Execution qualifiers become no-ops, `__shared__` arrays become per-thread
// host arrays, thread/block indices are thread-local variables set by the
// emulated launch in ref_harness.cpp, texture fetches are software filters
// with the unnormalised-coordinate / texel-centre conventions of the CUDA
// Programming Guide (weights optionally rounded to 8 fractional bits), and
// the __*_rn arithmetic intrinsics map to IEEE host arithmetic.
#pragma once
#define _GNU_SOURCE 1
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#undef __global__
#undef __device__
#undef __host__
#undef __constant__
#undef __shared__
#undef __forceinline__
#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__ thread_local
#define __forceinline__ inline

namespace ccsim {
extern thread_local uint3 tIdx, bIdx;
extern thread_local dim3 bDim, gDim;
extern int tex_emulate;  // 1: filter weights rounded to 8 fractional bits

struct Tex {
    const float* data;
    int n[3];
    int dims;
    bool linear;  // else point sampling
    bool border;  // else clamp
};
struct Surf {
    float* data;
    int n[3];
};

inline float fetch(const Tex& t, int i, int j, int k) {
    if (t.border) {
        if (i < 0 || i >= t.n[0] || j < 0 || j >= t.n[1] || k < 0 || k >= t.n[2]) return 0.f;
    } else {
        i = std::min(std::max(i, 0), t.n[0] - 1);
        j = std::min(std::max(j, 0), t.n[1] - 1);
        k = std::min(std::max(k, 0), t.n[2] - 1);
    }
    return t.data[i + (long long)t.n[0] * (j + (long long)t.n[1] * k)];
}
inline float qw(float a) { return tex_emulate ? std::floor(a * 256.f + 0.5f) / 256.f : a; }

inline float sample(const Tex& t, float x, float y, float z) {
    if (!t.linear) return fetch(t, (int)std::floor(x), (int)std::floor(y), (int)std::floor(z));
    float xb = x - 0.5f, yb = y - 0.5f, zb = z - 0.5f;
    float fx = std::floor(xb), fy = std::floor(yb), fz = std::floor(zb);
    int i = (int)fx, j = (int)fy, k = (int)fz;
    float a = qw(xb - fx), b = qw(yb - fy), c = qw(zb - fz);
    if (t.dims < 3) { c = 0.f; k = 0; }
    if (t.dims < 2) { b = 0.f; j = 0; }
    float v = 0.f;
    for (int dk = 0; dk < (t.dims > 2 ? 2 : 1); dk++)
        for (int dj = 0; dj < (t.dims > 1 ? 2 : 1); dj++)
            for (int di = 0; di < 2; di++) {
                float w = (di ? a : 1.f - a) * (t.dims > 1 ? (dj ? b : 1.f - b) : 1.f) *
                          (t.dims > 2 ? (dk ? c : 1.f - c) : 1.f);
                if (w != 0.f) v += w * fetch(t, i + di, j + dj, k + dk);
            }
    return v;
}
}  // namespace ccsim

#define threadIdx ccsim::tIdx
#define blockIdx ccsim::bIdx
#define blockDim ccsim::bDim
#define gridDim ccsim::gDim

// __syncthreads for the phase-replay launch (ref_harness.cpp launch_phased):
// a thread stops when it reaches the barrier of the current phase; with the
// default limit every barrier is passed (threads run one after another).
namespace ccsim {
extern thread_local int barrier_count, phase_limit;
struct PhaseStop {};
}  // namespace ccsim
inline void __syncthreads() {
    if (++ccsim::barrier_count >= ccsim::phase_limit) throw ccsim::PhaseStop{};
}

template <class T>
inline T tex3D(cudaTextureObject_t t, float x, float y, float z) {
    return (T)ccsim::sample(*(const ccsim::Tex*)(uintptr_t)t, x, y, z);
}
template <class T>
inline T tex2D(cudaTextureObject_t t, float x, float y) {
    return (T)ccsim::sample(*(const ccsim::Tex*)(uintptr_t)t, x, y, 0.5f);
}
template <class T>
inline void surf3Dwrite(T v, cudaSurfaceObject_t s, int xbytes, int y, int z,
                        cudaSurfaceBoundaryMode = cudaBoundaryModeTrap) {
    ccsim::Surf& S = *(ccsim::Surf*)(uintptr_t)s;
    int x = xbytes / (int)sizeof(T);
    if (x < 0 || y < 0 || z < 0 || x >= S.n[0] || y >= S.n[1] || z >= S.n[2]) return;  // would trap on the GPU
    S.data[x + (long long)S.n[0] * (y + (long long)S.n[1] * z)] = (float)v;
}

inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
inline float __frcp_rn(float a) { return 1.0f / a; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fdiv_rn(float a, float b) { return a / b; }
inline float fdividef(float a, float b) { return a / b; }
inline float __int2float_rn(int a) { return (float)a; }
inline int __float2int_rd(float a) { return (int)std::floor(a); }
inline float __powf(float a, float b) { return std::pow(a, b); }
inline void __sincosf(float a, float* s, float* c) { *s = std::sin(a); *c = std::cos(a); }
inline float __cosf(float a) { return std::cos(a); }
inline float __sinf(float a) { return std::sin(a); }
