// hv_server.cpp -- continuous batching of mesh requests (hv_server_* in hvgpu.h).
//
// One worker thread and one hv_ctx (CUDA stream) per slot.  Admission is FIFO:
// the head request starts as soon as a slot is idle and its HBM estimate fits
// next to the estimates of the running requests (a request larger than the
// whole budget is refused at submission).  The running requests' kernels and
// copies overlap on the device through their separate streams; every result
// is a pure function of its request (canonical vertex order, fixed-order
// reductions), so it does not depend on what else is running.
#include <chrono>
#include <condition_variable>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "hvgpu.h"

namespace {

using clk = std::chrono::steady_clock;

struct Job {
    hv_request req;
    std::vector<double> pts, lo, hi, base, normal;
    std::vector<int> periodic;
    std::vector<int16_t> bc;
    std::vector<int8_t> shift;
    double est = 0;
    int state = 0;  // 0 queued, 1 running, 2 done
    int rc = HV_OK;
    std::string err;
    clk::time_point t_submit, t_start, t_end;
    std::vector<int64_t> sig, offs, nbr, sig_offs;
    std::vector<double> r, vol, area;
    int64_t nverts = 0, nnbr = 0;
    hv_stats stats;
};

// Device bytes of one request: vertex records, tables, lists (same model as
// the build's capacity estimate, src vertices-per-generator counts).
double estimate_bytes(int d, int64_t n, int K, bool polygon) {
    static const double vpp[7] = {0, 0, 2.2, 7.0, 30.0, 150.0, 1400.0};
    const double V = 1.3 * (vpp[d] * (double)n + (double)(1 << d) + 1024);
    // VI_POLYGON from d = 3 on: the mesh-wide face lattice's sort buffers (24
    // bytes per entry, at most C(d+1, (d+1)/2) entries per vertex), two levels
    // of its per-vertex face tables and the faces' lists
    static const double lat[7] = {0, 0, 0, 24.0 * 4 + 8.0 * 6 + 100, 24.0 * 10 + 8.0 * 10 + 150,
                                  24.0 * 20 + 8.0 * 20 + 200, 24.0 * 35 + 8.0 * 35 + 300};
    if (polygon) return V * lat[d] + estimate_bytes(d, n, K, false);
    const int DP = d <= 4 ? 4 : 8;
    const double per_vertex = 4.0 * (d + 1) + 8.0 * d + 4.0 * DP + 4 + 4 + 16 + 8.0 * (d + 1) + 8.0 * (d + 1) * 2 +
                              4.0 * (d + 1) + 8.0 * d;
    const double per_point = 8.0 * d * 2 + 4.0 * DP + 4.0 * K + 64;
    return V * per_vertex + (double)n * per_point + (64 << 20);
}

}  // namespace

struct hv_server {
    hv_server_config cfg;
    std::vector<hv_ctx*> ctxs;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<int64_t> pending;
    std::map<int64_t, std::unique_ptr<Job>> jobs;
    double budget = 0, inflight = 0;
    int running = 0;
    bool stopping = false;
    int64_t next_ticket = 1;
};

namespace {

void run_job(hv_ctx* ctx, Job& J) {
    const hv_request& q = J.req;
    hv_mesh* m = nullptr;
    int rc;
    if (!J.periodic.empty())
        rc = hv_mesh_build_periodic(ctx, q.d, q.n, J.pts.data(), J.lo.data(), J.hi.data(), J.periodic.data(),
                                    &q.params, &m);
    else if (q.nplanes > 0)
        rc = hv_mesh_build_planes(ctx, q.d, q.n, J.pts.data(), q.nplanes, J.base.data(), J.normal.data(),
                                  J.bc.empty() ? nullptr : J.bc.data(), &q.params, &m);
    else
        rc = hv_mesh_build(ctx, q.d, q.n, J.pts.data(), J.lo.data(), J.hi.data(), &q.params, &m);
    if (rc == HV_OK) {
        int64_t nv = 0, nn = 0;
        rc = hv_mesh_counts(m, &nv, &nn);
        int64_t tot = 0;
        int maxlen = 0;
        if (rc == HV_OK) rc = hv_mesh_signature_total(m, &tot, &maxlen);
        if (rc == HV_OK) {
            J.nverts = nv; J.nnbr = nn;
            J.r.resize((size_t)nv * q.d);
            J.offs.resize((size_t)q.n + 1);
            J.nbr.resize((size_t)std::max<int64_t>(nn, 1));
            if (maxlen > q.d + 1) {  // co-spherical generators: the signatures as a CSR
                J.sig.resize((size_t)std::max<int64_t>(tot, 1));
                J.sig_offs.resize((size_t)nv + 1);
                rc = hv_mesh_vertices_csr(m, J.sig_offs.data(), J.sig.data(), J.r.data());
            } else {
                J.sig.resize((size_t)nv * (q.d + 1));
                rc = hv_mesh_vertices(m, J.sig.data(), J.r.data());
            }
        }
        if (rc == HV_OK) rc = hv_mesh_neighbors(m, J.offs.data(), J.nbr.data());
        if (rc == HV_OK && !J.periodic.empty()) {
            J.shift.resize((size_t)std::max<int64_t>(J.nnbr, 1) * q.d);
            rc = hv_mesh_periodic_shifts(m, J.shift.data());
        }
        if (rc == HV_OK && q.integrator != HV_INTEGRATOR_NONE) {
            J.vol.resize((size_t)std::max<int64_t>(q.n, 1));
            J.area.resize((size_t)std::max<int64_t>(J.nnbr, 1));
            if (q.integrator == HV_INTEGRATOR_POLYGON) rc = hv_integrate_polygon(m, J.vol.data(), J.area.data());
            else rc = hv_integrate_heuristic_mc(m, q.ndir > 0 ? q.ndir : 1000, q.mc_seed, J.vol.data(), J.area.data());
        }
        if (rc == HV_OK) hv_mesh_stats(m, &J.stats);
    }
    if (rc != HV_OK) J.err = hv_last_error(ctx);
    if (m) hv_mesh_free(m);
    J.rc = rc;
}

void worker(hv_server* S, int slot) {
    hv_ctx* ctx = S->ctxs[slot];
    for (;;) {
        int64_t ticket = 0;
        Job* J = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] {
                if (S->stopping) return true;
                if (S->pending.empty()) return false;
                Job* h = S->jobs[S->pending.front()].get();
                return S->running == 0 || S->inflight + h->est <= S->budget;
            });
            if (S->stopping && S->pending.empty()) return;
            if (S->pending.empty()) continue;
            ticket = S->pending.front();
            J = S->jobs[ticket].get();
            if (!(S->running == 0 || S->inflight + J->est <= S->budget)) continue;
            S->pending.pop_front();
            S->inflight += J->est;
            S->running++;
            J->state = 1;
            J->t_start = clk::now();
        }
        run_job(ctx, *J);
        {
            std::lock_guard<std::mutex> lk(S->mu);
            J->t_end = clk::now();
            J->state = 2;
            S->inflight -= J->est;
            S->running--;
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
}

double ms(clk::time_point a, clk::time_point b) { return std::chrono::duration<double, std::milli>(b - a).count(); }

}  // namespace

extern "C" {

int hv_server_start(const hv_server_config* cfg, hv_server** out) {
    if (!cfg || !out || cfg->slots <= 0 || cfg->slots > 64) return HV_E_INVALID_ARG;
    std::unique_ptr<hv_server> S(new hv_server());
    S->cfg = *cfg;
    for (int k = 0; k < cfg->slots; ++k) {
        hv_ctx* c = nullptr;
        int rc = hv_ctx_create(cfg->device, &c);
        if (rc != HV_OK) {
            for (hv_ctx* x : S->ctxs) hv_ctx_destroy(x);
            return rc;
        }
        S->ctxs.push_back(c);
    }
    S->budget = cfg->hbm_budget_bytes;
    if (S->budget <= 0) {
        size_t fr = 0, tot = 0;
        cudaSetDevice(cfg->device);
        cudaMemGetInfo(&fr, &tot);
        S->budget = 0.8 * (double)fr;
    }
    hv_server* raw = S.get();
    for (int k = 0; k < cfg->slots; ++k) S->workers.emplace_back(worker, raw, k);
    *out = S.release();
    return HV_OK;
}

int hv_server_submit(hv_server* S, const hv_request* q, int64_t* ticket) {
    if (!S || !q || !ticket || q->d < 2 || q->d > 6 || q->n < 0 || (q->n > 0 && !q->pts))
        return HV_E_INVALID_ARG;
    const bool planes = q->nplanes > 0;
    if (planes && (q->nplanes > 64 || !q->base || !q->normal || q->periodic)) return HV_E_INVALID_ARG;
    if (!planes && (!q->lo || !q->hi)) return HV_E_INVALID_ARG;
    std::unique_ptr<Job> J(new Job());
    J->req = *q;
    J->pts.assign(q->pts, q->pts + (size_t)q->n * q->d);
    if (planes) {
        J->base.assign(q->base, q->base + (size_t)q->nplanes * q->d);
        J->normal.assign(q->normal, q->normal + (size_t)q->nplanes * q->d);
        if (q->bc) J->bc.assign(q->bc, q->bc + q->nplanes);
    } else {
        J->lo.assign(q->lo, q->lo + q->d);
        J->hi.assign(q->hi, q->hi + q->d);
    }
    double n_eff = (double)q->n;
    if (q->periodic) {
        bool any = false;
        for (int k = 0; k < q->d; ++k) any |= q->periodic[k] != 0;
        if (any) {
            J->periodic.assign(q->periodic, q->periodic + q->d);
            // images in a margin of a few spacings on each periodic face
            const double grow = std::pow(1.0 + 6.0 / std::pow(std::max<double>((double)q->n, 1.0), 1.0 / q->d), q->d);
            n_eff *= std::min(grow, std::pow(3.0, q->d));
        }
    }
    J->req.pts = nullptr; J->req.lo = nullptr; J->req.hi = nullptr;
    J->req.periodic = nullptr; J->req.base = nullptr; J->req.normal = nullptr; J->req.bc = nullptr;
    static const int kd[7] = {0, 0, 24, 64, 128, 256, 384};  // the library's default list lengths
    J->est = estimate_bytes(q->d, (int64_t)n_eff, q->params.knn > 0 ? q->params.knn : kd[q->d],
                            q->integrator == HV_INTEGRATOR_POLYGON);
    if (J->est > S->budget) return HV_E_OOM;
    J->t_submit = clk::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stopping) return HV_E_INVALID_ARG;
        *ticket = S->next_ticket++;
        S->jobs[*ticket] = std::move(J);
        S->pending.push_back(*ticket);
    }
    S->cv_work.notify_all();
    return HV_OK;
}

int hv_server_poll(hv_server* S, int64_t ticket, int* done) {
    if (!S || !done) return HV_E_INVALID_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->jobs.find(ticket);
    if (it == S->jobs.end()) return HV_E_INVALID_ARG;
    *done = it->second->state == 2;
    return HV_OK;
}

int hv_server_wait(hv_server* S, int64_t ticket, double timeout_ms, hv_result* out) {
    if (!S || !out) return HV_E_INVALID_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->jobs.find(ticket);
    if (it == S->jobs.end()) return HV_E_INVALID_ARG;
    Job* J = it->second.get();
    auto ready = [&] { return J->state == 2; };
    if (timeout_ms < 0) S->cv_done.wait(lk, ready);
    else if (!S->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready)) return HV_E_TIMEOUT;
    std::memset(out, 0, sizeof(*out));
    out->status = J->rc;
    out->d = J->req.d;
    out->n = J->req.n;
    out->nverts = J->nverts;
    out->nnbr = J->nnbr;
    if (J->rc == HV_OK) {
        out->sig = J->sig.data();
        out->r = J->r.data();
        out->offs = J->offs.data();
        out->nbr = J->nbr.data();
        out->vol = J->vol.empty() ? nullptr : J->vol.data();
        out->area = J->area.empty() ? nullptr : J->area.data();
        out->stats = J->stats;
        out->shift = J->shift.empty() ? nullptr : J->shift.data();
        out->sig_offs = J->sig_offs.empty() ? nullptr : J->sig_offs.data();
    }
    out->queue_ms = ms(J->t_submit, J->t_start);
    out->service_ms = ms(J->t_start, J->t_end);
    out->latency_ms = ms(J->t_submit, J->t_end);
    return HV_OK;
}

int hv_server_release(hv_server* S, int64_t ticket) {
    if (!S) return HV_E_INVALID_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->jobs.find(ticket);
    if (it == S->jobs.end() || it->second->state != 2) return HV_E_INVALID_ARG;
    S->jobs.erase(it);
    return HV_OK;
}

int hv_server_stop(hv_server* S) {
    if (!S) return HV_E_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stopping = true;
    }
    S->cv_work.notify_all();
    for (auto& t : S->workers) t.join();
    for (hv_ctx* c : S->ctxs) hv_ctx_destroy(c);
    delete S;
    return HV_OK;
}

}  // extern "C"
