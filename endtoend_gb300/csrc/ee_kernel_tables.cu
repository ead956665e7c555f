// ee_kernel_tables.cu -- the dose-deposition kernel tables the engine runs
// on, built from the measured monoenergetic point kernels (the `dsa`
// files) and a beam spectrum, as dosecalc-preprocess does.
//
//   readers         spectrum file (CCCS/DoseCalcIO/spectra.cpp:7-62), mono
//                   kernel file (kernel.cpp:27-122), radii.dat (kernel.cpp:61-66)
//   k_kernel_tables one block: the fluence*energy*mu weighted poly kernel of
//                   each category (kernel.cpp:123-207), its total, the
//                   aggregation of 48 polar bins into ntheta cones and the
//                   radial running sum (kernel.cpp:364-396), and the cone
//                   angles (kernel.cpp:398-408).  Every value is
//                   formed with the reference's FP32 operations in its order
//                   (explicit round-to-nearest intrinsics, no contraction),
//                   so the tables are bit-identical to the reference's.
//   ee_fit_exp_kernel  host least-squares fit of the per-cone double
//                   exponential A/a(1-e^{-ar}) + B/b(1-e^{-br}) to a cumulative
//                   table: the parameters of the EE_KERNEL_EXP fast path.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ee_cccs.h"
#include "ee_internal.h"

int ee_internal_fail(int code, const char* msg);

namespace {

constexpr int KT_NRADII = EE_DSA_NRADII;
constexpr int KT_NANGLES = EE_DSA_NANGLES;
constexpr int KT_NCAT = EE_DSA_NCATEGORIES;
constexpr int KT_MAXE = 64;
constexpr int KT_CELLS = KT_NCAT * KT_NANGLES * KT_NRADII;

#define KT_CUDA(call)                                                        \
    do {                                                                     \
        cudaError_t _e = (call);                                             \
        if (_e != cudaSuccess) return ee_internal_fail(EE_ERR_CUDA, #call); \
    } while (0)

template <class T>
struct KBuf {
    T* p = nullptr;
    cudaError_t alloc(size_t n) { return cudaMalloc((void**)&p, std::max<size_t>(n, 1) * sizeof(T)); }
    ~KBuf() {
        if (p) cudaFree(p);
    }
};

bool read_tokens(const char* path, std::vector<std::string>& toks) {
    FILE* f = std::fopen(path, "r");
    if (!f) return false;
    std::string cur;
    int ch;
    while ((ch = std::fgetc(f)) != EOF) {
        if (ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r' || ch == '\f' || ch == '\v') {
            if (!cur.empty()) toks.push_back(cur), cur.clear();
        } else {
            cur.push_back((char)ch);
        }
    }
    if (!cur.empty()) toks.push_back(cur);
    std::fclose(f);
    return true;
}

// one whole token as a correctly rounded float (the value fscanf("%f") reads)
bool parse_f32(const std::string& t, float& v) {
    char* end = nullptr;
    errno = 0;
    v = std::strtof(t.c_str(), &end);
    return end != t.c_str() && *end == '\0' && std::isfinite(v);
}

// Block-wide build.  mono: [nE][5][48][24]; w[e] = (phi_e E_e) mu_e and
// wsum = their running sum, formed on the device in the reference's order.
__global__ void __launch_bounds__(256) k_kernel_tables(int nE, const float* __restrict__ phi, const float* __restrict__ E,
                                                       const float* __restrict__ mu, const float* __restrict__ mono,
                                                       int ntheta, int nphi, float* __restrict__ poly_cat,
                                                       float* __restrict__ poly_tot, float* __restrict__ cum_cat,
                                                       float* __restrict__ cum_tot, float* __restrict__ conv_theta,
                                                       float* __restrict__ conv_phi) {
    __shared__ float w[KT_MAXE];
    __shared__ float wsum;
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int e = 0; e < nE; e++) {
            w[e] = __fmul_rn(__fmul_rn(phi[e], E[e]), mu[e]);
            s = __fadd_rn(s, w[e]);
        }
        wsum = s;
    }
    // cone angles (kernel.cpp:274-276, 398-408): boundaries (180/ntheta)(t+1)
    // in FP32, theta = the bin centre, phi = (p + 0.5) 360 / nphi in double
    const int half = ntheta / 2;
    for (int a = threadIdx.x; a < nphi * half; a += blockDim.x) {
        const int p = a / half, t = a % half;
        const float step = __fdiv_rn(180.f, (float)ntheta);
        const float hi = __fmul_rn(step, (float)(t + 1)), lo = t > 0 ? __fmul_rn(step, (float)t) : 0.f;
        conv_theta[a] = __fmul_rn(0.5f, __fadd_rn(hi, lo));
        conv_phi[a] = (float)__ddiv_rn(__dmul_rn(__dadd_rn((double)p, 0.5), 360.0), (double)nphi);
    }
    __syncthreads();
    const int plane = KT_NANGLES * KT_NRADII;
    // poly kernel per category: sum_e w_e k_e, then / sum_e w_e
    for (int c = threadIdx.x; c < KT_CELLS; c += blockDim.x) {
        float acc = 0.f;
        for (int e = 0; e < nE; e++) acc = __fadd_rn(acc, __fmul_rn(w[e], mono[(size_t)e * KT_CELLS + c]));
        poly_cat[c] = __fdiv_rn(acc, wsum);
    }
    __syncthreads();
    // total = the five categories added in category order
    for (int c = threadIdx.x; c < plane; c += blockDim.x) {
        float t = 0.f;
        for (int k = 0; k < KT_NCAT; k++) t = __fadd_rn(t, poly_cat[k * plane + c]);
        poly_tot[c] = t;
    }
    __syncthreads();
    // ntheta cones of 48/ntheta polar bins each, then the running sum over
    // radius; one thread per (series, cone, ...) row: series 0..4 are the
    // categories, series 5 the total
    const int g = KT_NANGLES / ntheta;
    for (int row = threadIdx.x; row < (KT_NCAT + 1) * ntheta; row += blockDim.x) {
        const int series = row / ntheta, t = row % ntheta;
        const float* src = series < KT_NCAT ? poly_cat + series * plane : poly_tot;
        float* dst = series < KT_NCAT ? cum_cat + (series * ntheta + t) * KT_NRADII : cum_tot + t * KT_NRADII;
        float prev = 0.f;
        for (int r = 0; r < KT_NRADII; r++) {
            float v = 0.f;
            for (int k = 0; k < g; k++) v = __fadd_rn(v, src[(t * g + k) * KT_NRADII + r]);
            if (r > 0) v = __fadd_rn(v, prev);
            dst[r] = v;
            prev = v;
        }
    }
}

// ---------------------------------------------------------------- fit ----
// K(r) ~ A g(a, r) + B g(b, r), g(x, r) = (1 - e^{-x r}) / x.  For fixed
// decay rates the model is linear in (A, B): a 2x2 least-squares solve with
// non-negative amplitudes.  The rates come from a log-spaced grid search and
// a shrinking pattern search in (log a, log b).
struct ExpFit {
    double A, a, B, b, sse;
};

double gfun(double x, double r) { return -std::expm1(-x * r) / x; }

ExpFit solve_amplitudes(const double* r, const double* K, int n, double a, double b) {
    double gaa = 0, gbb = 0, gab = 0, ka = 0, kb = 0, kk = 0;
    for (int i = 0; i < n; i++) {
        const double ga = gfun(a, r[i]), gb = gfun(b, r[i]);
        gaa += ga * ga; gbb += gb * gb; gab += ga * gb;
        ka += ga * K[i]; kb += gb * K[i]; kk += K[i] * K[i];
    }
    ExpFit best{0, a, 0, b, kk};
    auto consider = [&](double A, double B) {
        if (A < 0 || B < 0) return;
        const double sse = kk - 2 * (A * ka + B * kb) + A * A * gaa + 2 * A * B * gab + B * B * gbb;
        if (sse < best.sse) best = ExpFit{A, a, B, b, sse};
    };
    const double det = gaa * gbb - gab * gab;
    if (det > 1e-300 * std::max(1.0, gaa * gbb)) consider((ka * gbb - kb * gab) / det, (kb * gaa - ka * gab) / det);
    if (gaa > 0) consider(ka / gaa, 0);
    if (gbb > 0) consider(0, kb / gbb);
    return best;
}

ExpFit fit_row(const double* r, const double* K, int n) {
    ExpFit best{0, 1, 0, 0.1, HUGE_VAL};
    const int NG = 48;
    const double la0 = std::log(1e-3), la1 = std::log(1e3);
    for (int i = 0; i < NG; i++)
        for (int j = 0; j < i; j++) {  // b < a
            const double a = std::exp(la0 + (la1 - la0) * i / (NG - 1));
            const double b = std::exp(la0 + (la1 - la0) * j / (NG - 1));
            ExpFit f = solve_amplitudes(r, K, n, a, b);
            if (f.sse < best.sse) best = f;
        }
    double step = (la1 - la0) / (NG - 1);
    for (int it = 0; it < 200 && step > 1e-7; it++) {
        bool moved = false;
        const double da[8] = {1, -1, 0, 0, 1, -1, 1, -1}, db[8] = {0, 0, 1, -1, 1, -1, -1, 1};
        for (int k = 0; k < 8; k++) {
            const double a = best.a * std::exp(da[k] * step), b = best.b * std::exp(db[k] * step);
            if (!(b < a) || a > 1e4 || b < 1e-5) continue;
            ExpFit f = solve_amplitudes(r, K, n, a, b);
            if (f.sse < best.sse) best = f, moved = true;
        }
        if (!moved) step *= 0.5;
    }
    return best;
}

}  // namespace

extern "C" {

int ee_read_spectrum_file(const char* path, int capacity, float* energy, float* fluence, float* mu, float* mu_en,
                          char* kernel_names, int name_stride, int* n) {
    if (!path || !n || capacity < 0 || (capacity > 0 && (!energy || !fluence || !mu || !mu_en)) ||
        (kernel_names && name_stride < 2))
        return ee_internal_fail(EE_ERR_INVALID_ARG, "bad spectrum reader arguments");
    std::vector<std::string> tok;
    if (!read_tokens(path, tok)) return ee_internal_fail(EE_ERR_IO, "cannot open spectrum file");
    // records of five fields until the first that does not parse
    std::vector<float> v[4];
    std::vector<std::string> names;
    for (size_t k = 0; k + 5 <= tok.size(); k += 5) {
        float x[4];
        bool ok = true;
        for (int j = 0; j < 4 && ok; j++) ok = parse_f32(tok[k + j], x[j]);
        if (!ok) break;
        for (int j = 0; j < 4; j++) v[j].push_back(x[j]);
        names.push_back(tok[k + 4]);
    }
    const int cnt = (int)names.size();
    *n = cnt;
    if (cnt == 0) return ee_internal_fail(EE_ERR_IO, "spectrum file holds no records");
    if (cnt > capacity) return ee_internal_fail(EE_ERR_CAPACITY, "more spectrum records than capacity");
    float s = 0.f;
    for (int i = 0; i < cnt; i++) s += v[1][i];
    if (!(s > 0.f)) return ee_internal_fail(EE_ERR_IO, "spectrum fluence does not sum to a positive value");
    for (int i = 0; i < cnt; i++) {
        energy[i] = v[0][i];
        fluence[i] = v[1][i] / s;
        mu[i] = v[2][i];
        mu_en[i] = v[3][i];
        if (kernel_names) {
            if ((int)names[i].size() >= name_stride)
                return ee_internal_fail(EE_ERR_CAPACITY, "kernel file name longer than name_stride");
            std::memset(kernel_names + (size_t)i * name_stride, 0, name_stride);
            std::memcpy(kernel_names + (size_t)i * name_stride, names[i].data(), names[i].size());
        }
    }
    return EE_OK;
}

int ee_read_mono_kernel(const char* path, float* weights) {
    if (!path || !weights) return ee_internal_fail(EE_ERR_INVALID_ARG, "bad kernel reader arguments");
    std::vector<std::string> tok;
    if (!read_tokens(path, tok)) return ee_internal_fail(EE_ERR_IO, "cannot open kernel file");
    const size_t need = (size_t)KT_NANGLES * KT_NRADII * 14;
    if (tok.size() < need) return ee_internal_fail(EE_ERR_IO, "kernel file too short (48 x 24 x 7 pairs)");
    size_t k = 0;
    for (int j = 0; j < KT_NANGLES; j++)
        for (int i = 0; i < KT_NRADII; i++)
            for (int c = 0; c < 7; c++, k += 2) {
                float val, unc;
                if (!parse_f32(tok[k], val) || !parse_f32(tok[k + 1], unc))
                    return ee_internal_fail(EE_ERR_IO, "kernel file holds a non-numeric value");
                if (c < KT_NCAT) weights[(c * KT_NANGLES + j) * KT_NRADII + i] = val;
            }
    return EE_OK;
}

int ee_read_kernel_radii(const char* path, float* radii) {
    if (!path || !radii) return ee_internal_fail(EE_ERR_INVALID_ARG, "bad radii reader arguments");
    std::vector<std::string> tok;
    if (!read_tokens(path, tok)) return ee_internal_fail(EE_ERR_IO, "cannot open radii file");
    if (tok.size() < (size_t)KT_NRADII) return ee_internal_fail(EE_ERR_IO, "radii file holds fewer than 24 values");
    for (int i = 0; i < KT_NRADII; i++) {
        if (!parse_f32(tok[i], radii[i])) return ee_internal_fail(EE_ERR_IO, "radii file holds a non-numeric value");
        if (i > 0 && !(radii[i] > radii[i - 1])) return ee_internal_fail(EE_ERR_IO, "radii must ascend");
    }
    return EE_OK;
}

int ee_cumulative_kernel(int device, int nkernels, const float* energy, const float* fluence, const float* mu,
                         const float* mono, int ntheta, int nphi, float* cum_total, float* cum_weights,
                         float* poly_total, float* poly_weights, float* conv_theta_deg, float* conv_phi_deg) {
    if (nkernels <= 0 || nkernels > KT_MAXE || !energy || !fluence || !mu || !mono || !cum_total)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "bad kernel-table arguments");
    if (ntheta < 2 || ntheta % 2 || KT_NANGLES % ntheta || nphi < 1 || nphi * (ntheta / 2) > EE_MAX_RAYS)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "ntheta must be even and divide 48; nphi*ntheta/2 rays");
    {
        int nd = 0;
        if (cudaGetDeviceCount(&nd) != cudaSuccess || device < 0 || device >= nd)
            return ee_internal_fail(EE_ERR_INVALID_ARG, "device out of range");
    }
    KT_CUDA(cudaSetDevice(device));
    const size_t plane = (size_t)KT_NANGLES * KT_NRADII;
    KBuf<float> d_in, d_out;
    KT_CUDA(d_in.alloc(3 * KT_MAXE + (size_t)nkernels * KT_CELLS));
    const int nang = nphi * (ntheta / 2);
    const size_t n_out =
        KT_CELLS + plane + (size_t)KT_NCAT * ntheta * KT_NRADII + (size_t)ntheta * KT_NRADII + 2 * (size_t)nang;
    KT_CUDA(d_out.alloc(n_out));
    float* phi = d_in.p;
    float* E = phi + KT_MAXE;
    float* m = E + KT_MAXE;
    float* k = m + KT_MAXE;
    KT_CUDA(cudaMemcpy(phi, fluence, nkernels * sizeof(float), cudaMemcpyHostToDevice));
    KT_CUDA(cudaMemcpy(E, energy, nkernels * sizeof(float), cudaMemcpyHostToDevice));
    KT_CUDA(cudaMemcpy(m, mu, nkernels * sizeof(float), cudaMemcpyHostToDevice));
    KT_CUDA(cudaMemcpy(k, mono, (size_t)nkernels * KT_CELLS * sizeof(float), cudaMemcpyHostToDevice));
    float* pc = d_out.p;
    float* pt = pc + KT_CELLS;
    float* cc = pt + plane;
    float* ct = cc + (size_t)KT_NCAT * ntheta * KT_NRADII;
    float* th = ct + (size_t)ntheta * KT_NRADII;
    float* ph = th + nang;
    k_kernel_tables<<<1, 256>>>(nkernels, phi, E, m, k, ntheta, nphi, pc, pt, cc, ct, th, ph);
    KT_CUDA(cudaGetLastError());
    KT_CUDA(cudaMemcpy(cum_total, ct, (size_t)ntheta * KT_NRADII * sizeof(float), cudaMemcpyDeviceToHost));
    if (cum_weights)
        KT_CUDA(cudaMemcpy(cum_weights, cc, (size_t)KT_NCAT * ntheta * KT_NRADII * sizeof(float),
                           cudaMemcpyDeviceToHost));
    if (poly_total) KT_CUDA(cudaMemcpy(poly_total, pt, plane * sizeof(float), cudaMemcpyDeviceToHost));
    if (poly_weights) KT_CUDA(cudaMemcpy(poly_weights, pc, KT_CELLS * sizeof(float), cudaMemcpyDeviceToHost));
    if (conv_theta_deg) KT_CUDA(cudaMemcpy(conv_theta_deg, th, nang * sizeof(float), cudaMemcpyDeviceToHost));
    if (conv_phi_deg) KT_CUDA(cudaMemcpy(conv_phi_deg, ph, nang * sizeof(float), cudaMemcpyDeviceToHost));
    return EE_OK;
}

int ee_fit_exp_kernel(int ntheta, int nradii, const float* radii, const float* cum_total, float* params,
                      float* max_rel_err) {
    if (ntheta <= 0 || nradii < 2 || nradii > 256 || !radii || !cum_total || !params)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "bad fit arguments");
    double r[256], K[256];
    for (int i = 0; i < nradii; i++) {
        r[i] = radii[i];
        if (!(r[i] > 0) || (i > 0 && !(r[i] > r[i - 1]))) return ee_internal_fail(EE_ERR_INVALID_ARG, "radii must ascend");
    }
    for (int t = 0; t < ntheta; t++) {
        for (int i = 0; i < nradii; i++) {
            K[i] = cum_total[t * nradii + i];
            if (!std::isfinite(K[i])) return ee_internal_fail(EE_ERR_INVALID_ARG, "non-finite kernel value");
        }
        const ExpFit f = fit_row(r, K, nradii);
        params[4 * t + 0] = (float)f.A;
        params[4 * t + 1] = (float)f.a;
        params[4 * t + 2] = (float)f.B;
        params[4 * t + 3] = (float)f.b;
        if (max_rel_err) {
            double e = 0, kmax = 0;
            for (int i = 0; i < nradii; i++) {
                const double v = f.A * gfun(f.a, r[i]) + f.B * gfun(f.b, r[i]);
                e = std::max(e, std::fabs(v - K[i]));
                kmax = std::max(kmax, std::fabs(K[i]));
            }
            max_rel_err[t] = (float)(kmax > 0 ? e / kmax : 0.0);
        }
    }
    return EE_OK;
}

}  // extern "C"
