// ee_server.cpp -- continuous-batching request server for dose and
// dose+gradient requests on one GPU.
//
// * Slots: `slots` worker threads, each with its own CUDA stream (its own
//   contexts), so requests handled by different slots overlap on the device.
// * Device-resident caches: a slot keeps one engine context per volume it
//   has served (density, its 3-D texture, kernel tables, scratch), evicting
//   least-recently-used idle contexts when the HBM budget would be exceeded.
// * Continuous batching: a free slot takes the oldest queued request and
//   every other queued request for the same volume and kind (up to
//   `max_batch_beams` beams) and runs them as ONE pipeline call, each
//   request's beams summed into its own output volume; requests that arrive
//   while slots are busy are admitted as slots and memory free up.
// * Admission by free HBM: a batch whose estimated footprint does not fit
//   the budget (after evicting idle contexts) waits; a request that can never
//   fit is failed with EE_ERR_NOMEM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ee_cccs.h"
#include "ee_internal.h"

int ee_internal_pipeline_grouped(ee_context* c, const ee_beam* beams, int nbeams, const float* d_fluence, float* d_dose,
                                 const int* group, int ngroups, const float* d_dose_grad, float* d_fgrad);
long long ee_internal_context_bytes(ee_context* c);
int ee_internal_fail(int code, const char* msg);

namespace {

using Clock = std::chrono::steady_clock;

struct Volume {
    ee_frame frame;
    std::vector<float> density;
    long long nvox() const { return (long long)frame.size[0] * frame.size[1] * frame.size[2]; }
};

struct Request {
    long long ticket = 0;
    int volume = 0;
    int kind = EE_REQ_DOSE;
    std::vector<ee_beam> beams;
    std::vector<float> fluence;
    std::vector<float> dose_grad;
    float* dose_out = nullptr;
    float* fgrad_out = nullptr;
    int status = -1;  // -1 pending
    std::string error;
    Clock::time_point t_submit, t_done;
};

struct SlotCtx {
    ee_context* ctx = nullptr;
    Clock::time_point last_use;
    long long bytes = 0;  // device bytes after its last batch
    bool busy = false;    // pinned by a batch being admitted or computed
};

struct Slot {
    std::thread th;
    std::map<int, SlotCtx> ctxs;
    float* pin = nullptr;
    size_t pin_n = 0;
    float* dbuf = nullptr;
    size_t dbuf_n = 0;
    long long dbuf_bytes = 0;  // device staging held (read under the server lock)
};

}  // namespace

struct ee_server {
    int device = 0;
    long long budget = 0;
    int max_batch_beams = 256;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    std::deque<std::shared_ptr<Request>> queue;
    std::map<long long, std::shared_ptr<Request>> all;
    std::deque<Volume> volumes;  // stable references while volumes are added
    std::vector<std::unique_ptr<Slot>> slots;
    long long next_ticket = 1;
    // physics (host copies, applied to every new context)
    bool have_physics = false;
    std::vector<float> E, fl, mu_, mu_en, radii, cumkern, th, ph, expp;
    ee_conv_params conv{};
    // stats
    std::vector<double> lat_ms;
    long long beams_done = 0;
    Clock::time_point t0 = Clock::now(), t_last = Clock::now();
    long long reserved = 0;     // admitted, not yet finished batches
    long long slot_scratch = 0; // per-context scratch limit
};

namespace {

int set_physics(ee_server* S, ee_context* c) {
    int st = ee_set_spectrum(c, (int)S->E.size(), S->E.data(), S->fl.data(), S->mu_.data(), S->mu_en.data());
    if (!st) st = ee_set_kernel_table(c, &S->conv, S->radii.data(), S->cumkern.data(), S->th.data(), S->ph.data());
    if (!st && !S->expp.empty()) st = ee_set_kernel_exp(c, S->expp.data());
    return st;
}

// device bytes held by every slot's contexts plus admitted batches (S->mu held)
long long bytes_in_use(ee_server* S) {
    long long b = S->reserved;
    for (auto& sl : S->slots) {
        b += sl->dbuf_bytes;
        for (auto& kv : sl->ctxs) b += kv.second.bytes;
    }
    return b;
}

// upper bound of what a batch adds: staging (fluence, dose and gradient
// volumes, in and out) and the growth of the volume's context up to
// resident data (density + texture + TERMA boxes) plus its scratch limit
long long batch_need(ee_server* S, const Volume& V, long long ctx_now, long long staging_now, long long nfl,
                     int ngroups, int nbeams, bool grad) {
    const long long nv = V.nvox();
    const long long bbox = (long long)V.frame.bbox_size[0] * V.frame.bbox_size[1] * V.frame.bbox_size[2];
    const long long staging = std::max(0ll, 4ll * (2 * nfl + nv * ngroups * (grad ? 2 : 1)) - staging_now);
    const long long ctx_after = 12ll * nv + 12ll * bbox * nbeams + S->slot_scratch;
    return staging + std::max(0ll, ctx_after - ctx_now);
}

void finish(ee_server* S, const std::vector<std::shared_ptr<Request>>& batch, int st, const char* err) {
    std::lock_guard<std::mutex> lk(S->mu);
    auto now = Clock::now();
    for (auto& r : batch) {
        r->status = st;
        if (err) r->error = err;
        r->t_done = now;
        if (st == EE_OK) {
            S->lat_ms.push_back(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
            S->beams_done += (long long)r->beams.size();
            S->t_last = now;
        }
    }
    S->cv_done.notify_all();
}

void release(ee_server* S, long long need) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->reserved -= need;
}

// end of a batch on a context: its admitted bytes become its measured size
void settle(ee_server* S, SlotCtx& sc, long long need) {
    const long long b = ee_internal_context_bytes(sc.ctx);
    std::lock_guard<std::mutex> lk(S->mu);
    S->reserved -= need;
    sc.bytes = b;
    sc.last_use = Clock::now();
    sc.busy = false;
}

void run_batch(ee_server* S, Slot& slot, std::vector<std::shared_ptr<Request>>& batch) {
    const int vol_id = batch[0]->volume;
    const bool grad = batch[0]->kind == EE_REQ_DOSE_AND_GRAD;
    const Volume& V = S->volumes[vol_id];
    const long long nv = V.nvox();
    const int ng = (int)batch.size();
    int nb = 0;
    long long nfl = 0;
    for (auto& r : batch) {
        nb += (int)r->beams.size();
        nfl += (long long)r->fluence.size();
    }
    // admission: the batch's footprint within the HBM budget, evicting the
    // least recently used idle contexts (of any slot) first; this slot's
    // context of the volume is pinned meanwhile
    long long need = 0;
    std::map<int, SlotCtx>::iterator it;
    bool have_ctx = false;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        auto deadline = Clock::now() + std::chrono::seconds(120);
        for (;;) {
            it = slot.ctxs.find(vol_id);
            have_ctx = it != slot.ctxs.end();
            if (have_ctx) it->second.busy = true;
            need = batch_need(S, V, have_ctx ? it->second.bytes : 0, slot.dbuf_bytes, nfl, ng, nb, grad);
            if (bytes_in_use(S) + need <= S->budget) break;
            Slot* vs = nullptr;
            int victim = -1;
            Clock::time_point oldest = Clock::time_point::max();
            for (auto& sl : S->slots)
                for (auto& kv : sl->ctxs)
                    if (!kv.second.busy && kv.second.last_use < oldest) {
                        oldest = kv.second.last_use;
                        victim = kv.first;
                        vs = sl.get();
                    }
            if (vs) {
                ee_destroy(vs->ctxs[victim].ctx);
                vs->ctxs.erase(victim);
                continue;
            }
            if (S->reserved == 0 || Clock::now() > deadline) {
                if (have_ctx) it->second.busy = false;
                lk.unlock();
                finish(S, batch, EE_ERR_NOMEM, "request does not fit the server's HBM budget");
                return;
            }
            S->cv_done.wait_for(lk, std::chrono::milliseconds(5));  // other slots release memory
        }
        S->reserved += need;
    }
    if (!have_ctx) {
        ee_context* c = nullptr;
        int st = ee_create(S->device, &c);
        if (!st) st = ee_set_volume(c, &V.frame, V.density.data());
        if (!st) st = set_physics(S, c);
        if (!st) st = ee_set_scratch_limit(c, S->slot_scratch);
        if (st) {
            std::string e = ee_last_error();
            if (c) ee_destroy(c);
            release(S, need);
            finish(S, batch, st, e.c_str());
            return;
        }
        std::lock_guard<std::mutex> lk(S->mu);
        it = slot.ctxs.emplace(vol_id, SlotCtx{c, Clock::now(), 0, true}).first;
    }
    SlotCtx& sc = it->second;
    ee_context* c = sc.ctx;
    cudaStream_t s = (cudaStream_t)ee_get_stream(c);
    // staging: [fluence | dose grads] in, [dose | fluence grads] out
    const size_t n_in = (size_t)nfl + (grad ? (size_t)nv * ng : 0);
    const size_t n_out = (size_t)nv * ng + (grad ? (size_t)nfl : 0);
    const size_t n_pin = std::max(n_in, n_out);
    auto fail_batch = [&](int st, const char* msg) {
        settle(S, sc, need);
        finish(S, batch, st, msg);
    };
    if (slot.pin_n < n_pin) {
        if (slot.pin) cudaFreeHost(slot.pin);
        slot.pin = nullptr;
        slot.pin_n = 0;
        if (cudaMallocHost((void**)&slot.pin, n_pin * sizeof(float)) != cudaSuccess) return fail_batch(EE_ERR_NOMEM, "pinned staging");
        slot.pin_n = n_pin;
    }
    const size_t n_dev = n_in + n_out;
    if (slot.dbuf_n < n_dev) {
        cudaSetDevice(S->device);
        cudaStreamSynchronize(s);
        if (slot.dbuf) cudaFree(slot.dbuf);
        slot.dbuf = nullptr;
        slot.dbuf_n = 0;
        if (cudaMalloc((void**)&slot.dbuf, n_dev * sizeof(float)) != cudaSuccess) return fail_batch(EE_ERR_NOMEM, "device staging");
        slot.dbuf_n = n_dev;
        std::lock_guard<std::mutex> lk(S->mu);
        slot.dbuf_bytes = (long long)(n_dev * sizeof(float));
    }
    std::vector<ee_beam> beams;
    std::vector<int> group;
    beams.reserve(nb);
    group.reserve(nb);
    size_t o = 0;
    for (int g = 0; g < ng; g++) {
        for (auto& b : batch[g]->beams) {
            beams.push_back(b);
            group.push_back(g);
        }
        std::memcpy(slot.pin + o, batch[g]->fluence.data(), batch[g]->fluence.size() * sizeof(float));
        o += batch[g]->fluence.size();
    }
    if (grad)
        for (int g = 0; g < ng; g++) {
            std::memcpy(slot.pin + o, batch[g]->dose_grad.data(), (size_t)nv * sizeof(float));
            o += (size_t)nv;
        }
    float* d_in = slot.dbuf;
    float* d_out = slot.dbuf + n_in;
    cudaSetDevice(S->device);
    if (cudaMemcpyAsync(d_in, slot.pin, n_in * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return fail_batch(EE_ERR_CUDA, "H2D");
    float* d_dose = d_out;
    float* d_fg = grad ? d_out + (size_t)nv * ng : nullptr;
    const float* d_dg = grad ? d_in + nfl : nullptr;
    int st = ee_internal_pipeline_grouped(c, beams.data(), nb, d_in, d_dose, group.data(), ng, d_dg, d_fg);
    if (st) {
        std::string e = ee_last_error();
        return fail_batch(st, e.c_str());
    }
    if (cudaMemcpyAsync(slot.pin, d_out, n_out * sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return fail_batch(EE_ERR_CUDA, "D2H");
    o = 0;
    for (int g = 0; g < ng; g++) {
        std::memcpy(batch[g]->dose_out, slot.pin + o, (size_t)nv * sizeof(float));
        o += (size_t)nv;
    }
    if (grad)
        for (int g = 0; g < ng; g++) {
            std::memcpy(batch[g]->fgrad_out, slot.pin + o, batch[g]->fluence.size() * sizeof(float));
            o += batch[g]->fluence.size();
        }
    settle(S, sc, need);
    finish(S, batch, EE_OK, nullptr);
}

void worker(ee_server* S, Slot* slot) {
    cudaSetDevice(S->device);
    for (;;) {
        std::vector<std::shared_ptr<Request>> batch;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop || !S->queue.empty(); });
            if (S->stop && S->queue.empty()) break;
            // the oldest request, plus the queued requests right behind it
            // for the same volume and kind, up to max_batch_beams beams:
            // merging stops at the first request it cannot take, so no
            // request overtakes an older one of another volume or kind
            auto first = S->queue.front();
            int nbeams = 0;
            while (!S->queue.empty()) {
                auto& r = S->queue.front();
                if (!(r->volume == first->volume && r->kind == first->kind &&
                      (batch.empty() || nbeams + (int)r->beams.size() <= S->max_batch_beams)))
                    break;
                nbeams += (int)r->beams.size();
                batch.push_back(r);
                S->queue.pop_front();
            }
        }
        run_batch(S, *slot, batch);
    }
    for (auto& kv : slot->ctxs) ee_destroy(kv.second.ctx);
    slot->ctxs.clear();
    if (slot->pin) cudaFreeHost(slot->pin);
    if (slot->dbuf) cudaFree(slot->dbuf);
}

}  // namespace

extern "C" {

int ee_server_create(int device, int slots, long long hbm_budget_bytes, int max_batch_beams, ee_server** out) {
    if (!out || slots <= 0 || slots > 64 || max_batch_beams <= 0) return ee_internal_fail(EE_ERR_INVALID_ARG, "bad server arguments");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "device out of range");
    ee_server* S = new ee_server();
    S->device = device;
    size_t fr = 0, tot = 0;
    cudaSetDevice(device);
    cudaMemGetInfo(&fr, &tot);
    S->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : (long long)(0.8 * (double)fr);
    S->max_batch_beams = max_batch_beams;
    S->slot_scratch = std::max(256ll << 20, std::min(8ll << 30, S->budget / (2ll * slots)));
    for (int k = 0; k < slots; k++) S->slots.emplace_back(new Slot());
    *out = S;
    return EE_OK;
}

int ee_server_set_physics(ee_server* S, int nE, const float* energy, const float* fluence, const float* mu,
                          const float* mu_en, const ee_conv_params* conv, const float* radii, const float* cumkern,
                          const float* theta_deg, const float* phi_deg, const float* exp_params) {
    if (!S || !energy || !fluence || !mu || !mu_en || !conv || !radii || !cumkern || !theta_deg || !phi_deg)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    if (!S->slots.empty() && S->slots[0]->th.joinable()) return ee_internal_fail(EE_ERR_INVALID_ARG, "server already started");
    S->E.assign(energy, energy + nE);
    S->fl.assign(fluence, fluence + nE);
    S->mu_.assign(mu, mu + nE);
    S->mu_en.assign(mu_en, mu_en + nE);
    S->conv = *conv;
    S->radii.assign(radii, radii + conv->nradii);
    S->cumkern.assign(cumkern, cumkern + (size_t)conv->ntheta * conv->nradii);
    const int nrays = conv->nphi * (conv->ntheta / 2);
    S->th.assign(theta_deg, theta_deg + nrays);
    S->ph.assign(phi_deg, phi_deg + nrays);
    if (exp_params) S->expp.assign(exp_params, exp_params + 4 * conv->ntheta);
    else S->expp.clear();
    S->have_physics = true;
    return EE_OK;
}

int ee_server_add_volume(ee_server* S, const ee_frame* frame, const float* density, int* volume_id) {
    if (!S || !frame || !density || !volume_id) return ee_internal_fail(EE_ERR_INVALID_ARG, "null argument");
    Volume V;
    V.frame = *frame;
    long long n = V.nvox();
    if (n <= 0) return ee_internal_fail(EE_ERR_INVALID_ARG, "empty volume");
    V.density.assign(density, density + n);
    std::lock_guard<std::mutex> lk(S->mu);
    S->volumes.push_back(std::move(V));
    *volume_id = (int)S->volumes.size() - 1;
    return EE_OK;
}

int ee_server_submit(ee_server* S, const ee_request* q, long long* ticket) {
    if (!S || !q || !ticket || !q->beams || q->nbeams <= 0 || !q->fluence || !q->dose_out)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "bad request");
    if (q->kind == EE_REQ_DOSE_AND_GRAD && (!q->dose_grad || !q->fluence_grad_out))
        return ee_internal_fail(EE_ERR_INVALID_ARG, "gradient request needs dose_grad and fluence_grad_out");
    auto r = std::make_shared<Request>();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (!S->have_physics) return ee_internal_fail(EE_ERR_NOT_READY, "ee_server_set_physics has not been called");
        if (q->volume_id < 0 || q->volume_id >= (int)S->volumes.size())
            return ee_internal_fail(EE_ERR_INVALID_ARG, "unknown volume id");
    }
    long long nfl = 0;
    for (int b = 0; b < q->nbeams; b++) {
        if (q->beams[b].fmap_size[0] <= 0 || q->beams[b].fmap_size[1] <= 0)
            return ee_internal_fail(EE_ERR_INVALID_ARG, "bad fluence map size");
        nfl += (long long)q->beams[b].fmap_size[0] * q->beams[b].fmap_size[1];
    }
    r->volume = q->volume_id;
    r->kind = q->kind;
    r->beams.assign(q->beams, q->beams + q->nbeams);
    r->fluence.assign(q->fluence, q->fluence + nfl);
    r->dose_out = q->dose_out;
    if (q->kind == EE_REQ_DOSE_AND_GRAD) {
        const long long nv = S->volumes[q->volume_id].nvox();
        r->dose_grad.assign(q->dose_grad, q->dose_grad + nv);
        r->fgrad_out = q->fluence_grad_out;
    }
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        r->ticket = S->next_ticket++;
        S->all[r->ticket] = r;
        S->queue.push_back(r);
        for (auto& sl : S->slots)
            if (!sl->th.joinable()) sl->th = std::thread(worker, S, sl.get());
    }
    S->cv_work.notify_one();
    *ticket = r->ticket;
    return EE_OK;
}

int ee_server_wait(ee_server* S, long long ticket, double timeout_s, int* status) {
    if (!S) return ee_internal_fail(EE_ERR_INVALID_ARG, "null server");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) return ee_internal_fail(EE_ERR_INVALID_ARG, "unknown ticket");
    auto r = it->second;
    auto pred = [&] { return r->status >= 0; };
    if (timeout_s < 0) S->cv_done.wait(lk, pred);
    else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
        if (status) *status = -1;
        return EE_OK;  // still pending
    }
    if (status) *status = r->status;
    S->all.erase(ticket);
    if (r->status != EE_OK) {
        std::string e = r->error;
        lk.unlock();
        return ee_internal_fail(r->status, e.c_str());
    }
    return EE_OK;
}

int ee_server_stats(ee_server* S, double* p50_ms, double* p99_ms, long long* completed, double* beams_per_s) {
    if (!S) return ee_internal_fail(EE_ERR_INVALID_ARG, "null server");
    std::lock_guard<std::mutex> lk(S->mu);
    std::vector<double> v = S->lat_ms;
    auto pct = [&](double q) {
        if (v.empty()) return 0.0;
        size_t k = (size_t)std::min<double>((double)v.size() - 1, std::floor(q * (double)(v.size() - 1) + 0.5));
        std::nth_element(v.begin(), v.begin() + k, v.end());
        return v[k];
    };
    if (p50_ms) *p50_ms = pct(0.50);
    if (p99_ms) *p99_ms = pct(0.99);
    if (completed) *completed = (long long)S->lat_ms.size();
    if (beams_per_s) {
        double t = std::chrono::duration<double>(S->t_last - S->t0).count();
        *beams_per_s = t > 0 ? (double)S->beams_done / t : 0.0;
    }
    return EE_OK;
}

int ee_server_reset_stats(ee_server* S) {
    if (!S) return ee_internal_fail(EE_ERR_INVALID_ARG, "null server");
    std::lock_guard<std::mutex> lk(S->mu);
    S->lat_ms.clear();
    S->beams_done = 0;
    S->t0 = S->t_last = Clock::now();
    return EE_OK;
}

int ee_server_destroy(ee_server* S) {
    if (!S) return EE_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    for (auto& sl : S->slots)
        if (sl->th.joinable()) sl->th.join();
    delete S;
    return EE_OK;
}

}  // extern "C"
