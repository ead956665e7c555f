// ee_anneal.cu -- beam-angle and fluence optimisation around the CCCS chain:
// the EndtoEnd programs optimize_stationary_smoothness (fluence gradient
// descent with the angles fixed) and optimize_annealing_constrain (simulated
// annealing of the angles + gradient descent of the fluence), whose source is
// not in the reference snapshot; their inputs, outputs and loss are defined
// by README.md:15-22, 75-95.  Also the batched evaluation of whole-angle-set
// proposals.
//
// GB300 organisation: proposal doses are computed in one batched call (every
// beam's proposal as its own per-beam dose volume, or every proposal's beams
// summed into its own volume through the grouped pipeline); the acceptance
// test of a proposal is one fused reduction over the volume
// (total - old_k + new_k evaluated on the fly, FP64 accumulation).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/ee_cccs.h"
#include "ee_internal.h"

int ee_internal_fail(int code, const char* msg);
int ee_internal_snapshot(ee_context* c, EeParams* P, int* device);
void ee_internal_build_spec(const EeParams& P, const ee_beam& beam, EeBeamSpec* out);
int ee_internal_pipeline_grouped(ee_context* c, const ee_beam* beams, int nbeams, const float* d_fluence, float* d_dose,
                                 const int* group, int ngroups, const float* d_dose_grad, float* d_fgrad);

namespace {

constexpr unsigned FULL = 0xffffffffu;

// Dose terms of the loss for d = base + (add - sub) (add/sub optional):
// acc[0] += sum w0 (d - t0)^2, acc[1] += sum w max(d - t, 0)^2.
__global__ void __launch_bounds__(256) k_loss_eval(const float* __restrict__ base, const float* __restrict__ sub,
                                                   const float* __restrict__ add, const float* __restrict__ ptv_w,
                                                   const float* __restrict__ ptv_t, const float* __restrict__ oar_w,
                                                   const float* __restrict__ oar_t, long long n,
                                                   double* __restrict__ acc) {
    double lp = 0.0, lo = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float d = base[i];
        if (add) d += add[i] - sub[i];
        if (ptv_w) {
            const float e = d - ptv_t[i];
            lp += (double)ptv_w[i] * e * e;
        }
        if (oar_w) {
            const float e = fmaxf(d - oar_t[i], 0.f);
            lo += (double)oar_w[i] * e * e;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        lp += __shfl_xor_sync(FULL, lp, o);
        lo += __shfl_xor_sync(FULL, lo, o);
    }
    __shared__ double sp[8], so[8];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { sp[w] = lp; so[w] = lo; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) { a += sp[k]; b += so[k]; }
        atomicAdd(acc, a);
        atomicAdd(acc + 1, b);
    }
}

// d += a - b (accepting a proposal into the total dose)
__global__ void k_swap_in(float* __restrict__ d, const float* __restrict__ a, const float* __restrict__ b, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] += a[i] - b[i];
}

// total = sum over n per-beam volumes
__global__ void k_sum_volumes(float* __restrict__ total, const float* __restrict__ vols, int n, long long nv) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (long long)gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int b = 0; b < n; b++) acc += vols[(size_t)b * nv + i];
        total[i] = acc;
    }
}

// projected gradient step: x = max(x - step * g, 0)
__global__ void k_step(float* __restrict__ x, const float* __restrict__ g, float step, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = fmaxf(x[i] - step * g[i], 0.f);
}

// per-beam ||D x_k||_1 (forward differences along both map axes)
__global__ void __launch_bounds__(256) k_smooth_beam(const EeBeamSpec* __restrict__ specs, const float* __restrict__ x,
                                                     double* __restrict__ acc) {
    const EeBeamSpec& S = specs[blockIdx.z];
    const int fx = S.fmap[0], fy = S.fmap[1];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (p < fx * fy) {
        const int i = p % fx, j = p / fx;
        const float* m = x + S.fl_off;
        if (i + 1 < fx) l += fabsf(m[p + 1] - m[p]);
        if (j + 1 < fy) l += fabsf(m[p + fx] - m[p]);
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(FULL, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(acc + blockIdx.z, l);
}

template <class T>
struct Buf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t c) {
        if (c <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc((void**)&p, std::max<size_t>(c, 1) * sizeof(T));
        if (e == cudaSuccess) n = std::max<size_t>(c, 1);
        return e;
    }
    ~Buf() {
        if (p) cudaFree(p);
    }
};

#define AN_CUDA(call)                                                        \
    do {                                                                     \
        cudaError_t _e = (call);                                             \
        if (_e != cudaSuccess) return ee_internal_fail(EE_ERR_CUDA, #call); \
    } while (0)

unsigned grid_of(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152 * 8); }

long long nvox(const EeParams& P) { return (long long)P.size[0] * P.size[1] * P.size[2]; }

long long total_pixels(const ee_beam* beams, int n) {
    long long t = 0;
    for (int b = 0; b < n; b++) t += (long long)beams[b].fmap_size[0] * beams[b].fmap_size[1];
    return t;
}

// Dose terms of base (+ add - sub) on the context stream.
int loss_terms(const ee_loss& L, const float* base, const float* sub, const float* add, long long n, double* d_acc,
               cudaStream_t s, double out[2]) {
    AN_CUDA(cudaMemsetAsync(d_acc, 0, 2 * sizeof(double), s));
    k_loss_eval<<<grid_of(n), 256, 0, s>>>(base, sub, add, L.ptv_weight, L.ptv_target, L.oar_weight, L.oar_target, n,
                                           d_acc);
    AN_CUDA(cudaGetLastError());
    AN_CUDA(cudaMemcpyAsync(out, d_acc, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    AN_CUDA(cudaStreamSynchronize(s));
    return EE_OK;
}

// Fluence the dose engine sees: G * x (a copy of x without spread).
int spread_fluence(const EeParams& P, const ee_beam* beams, int n, const float* d_x, float sigma, Buf<EeBeamSpec>& specs,
                   Buf<float>& w, float* d_out, cudaStream_t s) {
    std::vector<EeBeamSpec> h(n);
    for (int b = 0; b < n; b++) {
        ee_internal_build_spec(P, beams[b], &h[b]);
        h[b].fl_off = 0;
    }
    long long off = 0;
    int max_pix = 1;
    for (int b = 0; b < n; b++) {
        h[b].fl_off = off;
        off += (long long)beams[b].fmap_size[0] * beams[b].fmap_size[1];
        max_pix = std::max(max_pix, beams[b].fmap_size[0] * beams[b].fmap_size[1]);
    }
    if (!(sigma > 0.f)) {
        AN_CUDA(cudaMemcpyAsync(d_out, d_x, sizeof(float) * off, cudaMemcpyDeviceToDevice, s));
        return EE_OK;
    }
    const int R = (int)std::ceil(3.0 * sigma);
    std::vector<float> hw(2 * R + 1);
    double sum = 0;
    for (int k = -R; k <= R; k++) sum += (hw[k + R] = (float)std::exp(-0.5 * k * k / ((double)sigma * sigma)));
    for (auto& v : hw) v = (float)(v / sum);
    AN_CUDA(w.ensure(hw.size()));
    AN_CUDA(cudaMemcpyAsync(w.p, hw.data(), sizeof(float) * hw.size(), cudaMemcpyHostToDevice, s));
    AN_CUDA(specs.ensure(n));
    AN_CUDA(cudaMemcpyAsync(specs.p, h.data(), sizeof(EeBeamSpec) * n, cudaMemcpyHostToDevice, s));
    AN_CUDA(ee_launch_spread(specs.p, d_x, d_out, w.p, R, n, max_pix, s));
    return EE_OK;
}

// per-beam ||D x_k||_1 into host out[n]
int smoothness(const EeParams& P, const ee_beam* beams, int n, const float* d_x, Buf<EeBeamSpec>& specs,
               Buf<double>& acc, cudaStream_t s, std::vector<double>& out) {
    std::vector<EeBeamSpec> h(n);
    long long off = 0;
    int max_pix = 1;
    for (int b = 0; b < n; b++) {
        ee_internal_build_spec(P, beams[b], &h[b]);
        h[b].fl_off = off;
        off += (long long)beams[b].fmap_size[0] * beams[b].fmap_size[1];
        max_pix = std::max(max_pix, beams[b].fmap_size[0] * beams[b].fmap_size[1]);
    }
    AN_CUDA(specs.ensure(n));
    AN_CUDA(cudaMemcpyAsync(specs.p, h.data(), sizeof(EeBeamSpec) * n, cudaMemcpyHostToDevice, s));
    AN_CUDA(acc.ensure(n));
    AN_CUDA(cudaMemsetAsync(acc.p, 0, sizeof(double) * n, s));
    k_smooth_beam<<<dim3((max_pix + 255) / 256, 1, n), 256, 0, s>>>(specs.p, d_x, acc.p);
    AN_CUDA(cudaGetLastError());
    out.resize(n);
    AN_CUDA(cudaMemcpyAsync(out.data(), acc.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    AN_CUDA(cudaStreamSynchronize(s));
    return EE_OK;
}

int check_loss(const ee_loss* L) {
    if (!L) return ee_internal_fail(EE_ERR_INVALID_ARG, "null loss");
    if (!(L->eta >= 0) || !(L->spread_sigma >= 0)) return ee_internal_fail(EE_ERR_INVALID_ARG, "bad eta / spread sigma");
    if ((L->ptv_weight == nullptr) != (L->ptv_target == nullptr) ||
        (L->oar_weight == nullptr) != (L->oar_target == nullptr))
        return ee_internal_fail(EE_ERR_INVALID_ARG, "weight and target arrays come in pairs");
    return EE_OK;
}

const double kPi = 3.14159265358979323846;

}  // namespace

extern "C" {

int ee_optimize_fluence(ee_context* c, const ee_beam* beams, int nbeams, float* d_x, const ee_loss* loss, int iterations,
                        float step_size, float* dose_loss, float* smoothness_loss) {
    int st = check_loss(loss);
    if (st) return st;
    if (!c || !beams || nbeams <= 0 || !d_x || iterations < 0 || !(step_size >= 0.f))
        return ee_internal_fail(EE_ERR_INVALID_ARG, "bad arguments");
    EeParams P;
    int dev;
    if ((st = ee_internal_snapshot(c, &P, &dev))) return st;
    cudaSetDevice(dev);
    cudaStream_t s = (cudaStream_t)ee_get_stream(c);
    const long long nv = nvox(P), npx = total_pixels(beams, nbeams);
    Buf<float> dose, g;
    Buf<EeBeamSpec> specs;
    Buf<double> acc;
    AN_CUDA(dose.ensure(nv));
    AN_CUDA(g.ensure(npx));
    std::vector<double> sm;
    for (int it = 0; it < iterations; it++) {
        double terms[3];
        if ((st = ee_loss_and_grad(c, beams, nbeams, d_x, loss, dose.p, g.p, terms))) return st;
        if (dose_loss) dose_loss[it] = (float)(terms[0] + terms[1]);
        k_step<<<grid_of(npx), 256, 0, s>>>(d_x, g.p, step_size, npx);
        AN_CUDA(cudaGetLastError());
        if (smoothness_loss) {
            if ((st = smoothness(P, beams, nbeams, d_x, specs, acc, s, sm))) return st;
            for (int b = 0; b < nbeams; b++) smoothness_loss[(size_t)it * nbeams + b] = (float)(loss->eta * sm[b]);
        }
    }
    AN_CUDA(cudaStreamSynchronize(s));
    return EE_OK;
}

int ee_optimize_annealing(ee_context* c, ee_beam* beams, int nbeams, float* d_x, const ee_loss* loss,
                          const ee_anneal_params* prm, ee_anneal_record* rec) {
    int st = check_loss(loss);
    if (st) return st;
    if (!c || !beams || nbeams <= 0 || !d_x || !prm || prm->iterations < 0 || !(prm->step_size >= 0.f) ||
        !(prm->sigma_deg >= 0.f) || !(prm->temperature >= 0.f) || !(prm->cooling > 0.f) || prm->fluence_steps < 0)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "bad arguments");
    EeParams P;
    int dev;
    if ((st = ee_internal_snapshot(c, &P, &dev))) return st;
    cudaSetDevice(dev);
    cudaStream_t s = (cudaStream_t)ee_get_stream(c);
    const long long nv = nvox(P), npx = total_pixels(beams, nbeams);
    const int n = nbeams;
    Buf<float> f, cur, prop, total, g;
    Buf<EeBeamSpec> specs;
    Buf<float> w;
    Buf<double> acc;
    AN_CUDA(f.ensure(npx));
    AN_CUDA(cur.ensure((size_t)nv * n));
    AN_CUDA(prop.ensure((size_t)nv * n));
    AN_CUDA(total.ensure(nv));
    AN_CUDA(g.ensure(npx));
    AN_CUDA(acc.ensure(n > 2 ? n : 2));
    std::mt19937_64 rng(prm->seed);
    std::normal_distribution<double> gauss(0.0, prm->sigma_deg * kPi / 180.0);
    std::uniform_real_distribution<double> unif(0.0, 1.0);
    std::vector<ee_beam> trial(beams, beams + n);
    std::vector<double> sm;
    double T = prm->temperature;
    for (int it = 0; it < prm->iterations; it++) {
        // every beam's dose at the current angles, and at its proposal
        if ((st = spread_fluence(P, beams, n, d_x, loss->spread_sigma, specs, w, f.p, s))) return st;
        if ((st = ee_beam_dose_device(c, beams, n, f.p, cur.p, EE_DOSE_PER_BEAM))) return st;
        for (int b = 0; b < n; b++) {
            trial[b] = beams[b];
            trial[b].azimuth = (float)(beams[b].azimuth + gauss(rng));
            trial[b].zenith = (float)(beams[b].zenith + gauss(rng));
        }
        if ((st = ee_beam_dose_device(c, trial.data(), n, f.p, prop.p, EE_DOSE_PER_BEAM))) return st;
        k_sum_volumes<<<grid_of(nv), 256, 0, s>>>(total.p, cur.p, n, nv);
        AN_CUDA(cudaGetLastError());
        double base[2];
        if ((st = loss_terms(*loss, total.p, nullptr, nullptr, nv, acc.p, s, base))) return st;
        double L0 = base[0] + base[1];
        // sequential acceptance against the running total
        for (int b = 0; b < n; b++) {
            double t2[2];
            const float* old_b = cur.p + (size_t)b * nv;
            const float* new_b = prop.p + (size_t)b * nv;
            if ((st = loss_terms(*loss, total.p, old_b, new_b, nv, acc.p, s, t2))) return st;
            const double L1 = t2[0] + t2[1];
            double p = L1 <= L0 ? 1.0 : (T > 0 ? std::exp(-(L1 - L0) / T) : 0.0);
            const bool take = unif(rng) < p;
            const size_t r2 = ((size_t)it * n + b) * 2, r1 = (size_t)it * n + b;
            if (rec) {
                if (rec->zenith) { rec->zenith[r2] = beams[b].zenith; rec->zenith[r2 + 1] = trial[b].zenith; }
                if (rec->azimuth) { rec->azimuth[r2] = beams[b].azimuth; rec->azimuth[r2 + 1] = trial[b].azimuth; }
                if (rec->perturbation_loss) {
                    rec->perturbation_loss[r2] = (float)L0;
                    rec->perturbation_loss[r2 + 1] = (float)L1;
                }
                if (rec->possibility) rec->possibility[r1] = (float)p;
                if (rec->taken) rec->taken[r1] = take ? 1 : 0;
            }
            if (take) {
                k_swap_in<<<grid_of(nv), 256, 0, s>>>(total.p, new_b, old_b, nv);
                AN_CUDA(cudaGetLastError());
                beams[b].azimuth = trial[b].azimuth;
                beams[b].zenith = trial[b].zenith;
                L0 = L1;
            }
        }
        // fluence gradient descent at the accepted angles
        double terms[3] = {0, 0, 0};
        for (int k = 0; k < prm->fluence_steps; k++) {
            if ((st = ee_loss_and_grad(c, beams, n, d_x, loss, total.p, g.p, terms))) return st;
            k_step<<<grid_of(npx), 256, 0, s>>>(d_x, g.p, prm->step_size, npx);
            AN_CUDA(cudaGetLastError());
        }
        // dose terms of the iteration: at the accepted angles, before the
        // last fluence step when there is one
        if (rec && rec->dose_loss) rec->dose_loss[it] = (float)(prm->fluence_steps > 0 ? terms[0] + terms[1] : L0);
        if (rec && rec->smoothness_loss) {
            if ((st = smoothness(P, beams, n, d_x, specs, acc, s, sm))) return st;
            for (int b = 0; b < n; b++) rec->smoothness_loss[(size_t)it * n + b] = (float)(loss->eta * sm[b]);
        }
        T *= prm->cooling;
    }
    AN_CUDA(cudaStreamSynchronize(s));
    return EE_OK;
}

int ee_evaluate_proposals(ee_context* c, const ee_beam* proposals, int nprop, int nbeams, const float* d_x,
                          const ee_loss* loss, double* losses) {
    int st = check_loss(loss);
    if (st) return st;
    if (!c || !proposals || nprop <= 0 || nbeams <= 0 || !d_x || !losses)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "bad arguments");
    EeParams P;
    int dev;
    if ((st = ee_internal_snapshot(c, &P, &dev))) return st;
    cudaSetDevice(dev);
    cudaStream_t s = (cudaStream_t)ee_get_stream(c);
    const long long nv = nvox(P), npx = total_pixels(proposals, nbeams);
    for (int q = 1; q < nprop; q++)
        for (int b = 0; b < nbeams; b++)
            if (proposals[(size_t)q * nbeams + b].fmap_size[0] != proposals[b].fmap_size[0] ||
                proposals[(size_t)q * nbeams + b].fmap_size[1] != proposals[b].fmap_size[1])
                return ee_internal_fail(EE_ERR_INVALID_ARG, "proposals must share the fluence-map sizes");
    // every proposal sees the same fluence: G * x, repeated per proposal
    Buf<float> f, fall, dose;
    Buf<EeBeamSpec> specs;
    Buf<float> w;
    Buf<double> acc;
    AN_CUDA(f.ensure(npx));
    AN_CUDA(fall.ensure((size_t)npx * nprop));
    AN_CUDA(dose.ensure((size_t)nv * nprop));
    AN_CUDA(acc.ensure(2));
    if ((st = spread_fluence(P, proposals, nbeams, d_x, loss->spread_sigma, specs, w, f.p, s))) return st;
    for (int q = 0; q < nprop; q++)
        AN_CUDA(cudaMemcpyAsync(fall.p + (size_t)q * npx, f.p, sizeof(float) * npx, cudaMemcpyDeviceToDevice, s));
    std::vector<int> group((size_t)nprop * nbeams);
    for (int q = 0; q < nprop; q++)
        for (int b = 0; b < nbeams; b++) group[(size_t)q * nbeams + b] = q;
    if ((st = ee_internal_pipeline_grouped(c, proposals, nprop * nbeams, fall.p, dose.p, group.data(), nprop, nullptr,
                                           nullptr)))
        return st;
    for (int q = 0; q < nprop; q++) {
        double t[2];
        if ((st = loss_terms(*loss, dose.p + (size_t)q * nv, nullptr, nullptr, nv, acc.p, s, t))) return st;
        losses[q] = t[0] + t[1];
    }
    return EE_OK;
}

}  // extern "C"
