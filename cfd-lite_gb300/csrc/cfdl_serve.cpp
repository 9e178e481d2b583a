// cfdl_serve.cpp -- a serving loop for cavity-solve requests with continuous
// batching.  No counterpart in the reference, which solves one case per run.
//
// Requests arrive from any host thread (cfdl_server_submit).  A pool of host
// threads prepares each one: the CGNS-shaped zone, the reference's mesh set-up
// (face numbering, geometry), the device-layout tables and the multigrid
// hierarchy -- everything but device memory.  One device thread owns a
// context and loops:
//   retire   cases whose run ended (converged, capped or failed): read their
//            statistics, keep their fields if asked, free their device memory;
//   admit    prepared requests in arrival order while a slot is free and the
//            case's device bytes fit both the HBM budget and the memory the
//            device reports free (less a reserve);
//   run      up to `chunk` outer iterations of every resident case as one
//            graph launch (cfdl_run's graph: a case whose run ends mid-launch
//            is skipped by every kernel from then on).
// Fields and matrices stay resident between outer iterations; a request's
// state leaves the device only when it is retired.  Every kernel works per
// case and every reduction sums a case's own partials in a fixed order, so a
// request's result does not depend on which requests shared its launches.
#include "cfdl_internal.h"
#include "cfdl_par.h"
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>

using namespace cfdl;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t id = 0;
    cfdl_request r{};
    double t_submit = 0, t_ready = 0, t_admit = 0;
    CasePrep prep;
    size_t est = 0;
    int status = CFDL_OK;
};

struct Resident {
    std::unique_ptr<Request> req;
    HostCase *hc = nullptr;
    int outer_seen = 0;
    size_t reserved = 0;     // bytes held against the budget: max(estimate, allocated)
};

struct Finished {
    cfdl_result res{};
    std::vector<double> u, v, w, p;
};

}  // namespace

struct cfdl_server {
    cfdl_server_config cfg{};
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_prep, cv_dev, cv_done;
    std::deque<std::unique_ptr<Request>> pending;            // submitted, not prepared
    std::map<int64_t, std::unique_ptr<Request>> ready;       // prepared, by arrival
    std::map<int64_t, Finished> finished;                     // retired
    std::deque<int64_t> unpolled;
    int64_t next_id = 0, submitted = 0, done = 0;
    int preparing = 0;
    bool stopping = false;
    std::vector<std::thread> preppers;
    std::thread device;
    // device-thread state (read under mu for cfdl_server_info)
    int resident = 0;
    size_t held_bytes = 0;
    int64_t launches = 0;
    double cell_iters = 0, busy_s = 0;
    int device_status = CFDL_OK;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

cfdl_config request_config(const cfdl_server_config &s, const cfdl_request &r) {
    cfdl_config c;
    cfdl_config_default(&c);
    c.rho = 1.0;
    c.mu = 1.0 / r.re;
    c.dt = INFINITY;
    c.alpha_u = s.alpha_u;
    c.alpha_p = s.alpha_p;
    c.precision = s.precision;
    c.precond = s.precond;
    return c;
}

// The host threads this preparation's parallel loops may use: the cores
// shared by the requests being prepared now (a lone request gets them all).
// Re-read before each parallel phase, so a request that started during a
// burst takes the cores back once the others are done; the loops give the
// same result on any number of threads.
void share_cores(cfdl_server *S) {
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    std::lock_guard<std::mutex> lk(S->mu);
    host_threads() = std::max(1, hw / std::max(1, S->preparing));
}

// Host preparation of one request: zone, mesh set-up, device-layout tables,
// multigrid hierarchy.
int prepare(cfdl_server *S, const cfdl_server_config &s, Request &q) {
    const cfdl_request &r = q.r;
    int nvx, nelem, nsec, m;
    int st = cfdl_box_zone_sizes(r.n, r.tet, &nvx, &nelem, &nsec, &m);
    if (st) return st;
    try {
        std::vector<double> x(nvx), y(nvx), z(nvx);
        std::vector<int> e2vx((size_t)m * nelem), etype(nsec), esec(2 * (size_t)nsec);
        std::vector<char> names(33 * (size_t)nsec + 1, 0);
        if ((st = cfdl_box_zone_fill(r.n, r.tet, r.jitter, r.seed, x.data(), y.data(), z.data(), e2vx.data(), etype.data(),
                                     esec.data(), names.data())))
            return st;
        cfdl_setup *su = nullptr;
        auto create = s.device_setup ? cfdl_setup_create_device : cfdl_setup_create;
        if ((st = create(nvx, x.data(), y.data(), z.data(), nsec, names.data(), etype.data(), esec.data(), m,
                         e2vx.data(), &su)))
            return st;
        cfdl_mesh mesh;
        st = cfdl_setup_mesh(su, 1.0, &mesh);
        share_cores(S);
        if (!st) st = prepare_case(&mesh, &q.prep);
        cfdl_setup_destroy(su);
        if (st) return st;
        share_cores(S);
        if (s.precond == 1 && (st = prepare_case_amg(&q.prep))) return st;
    } catch (const std::bad_alloc &) {
        return CFDL_ERR_OOM;
    }
    q.est = cfdl_case_bytes_estimate(q.prep.ne, q.prep.nf, q.prep.nbf, q.prep.W);
    return CFDL_OK;
}

void prep_loop(cfdl_server *S) {
    if (S->cfg.device_setup) cudaSetDevice(S->cfg.device);   // the set-up kernels' device
    for (;;) {
        std::unique_ptr<Request> q;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_prep.wait(lk, [&] { return S->stopping || !S->pending.empty(); });
            if (S->stopping) return;
            q = std::move(S->pending.front());
            S->pending.pop_front();
            S->preparing++;
        }
        share_cores(S);
        q->status = prepare(S, S->cfg, *q);
        std::lock_guard<std::mutex> lk(S->mu);
        S->preparing--;
        q->t_ready = S->now();
        const int64_t id = q->id;
        S->ready[id] = std::move(q);
        S->cv_dev.notify_one();
    }
}

void finish_request(cfdl_server *S, Request &q, int status, const SolveScalars *sc, HostCase *hc, Finished &&f) {
    f.res.id = q.id;
    f.res.status = status;
    f.res.ne = q.prep.ne ? q.prep.ne : (hc ? hc->ne : 0);
    if (sc) {
        f.res.outer_done = sc->outer_done;
        f.res.converged = sc->converged;
        f.res.mass_ratio = sc->mass_ratio;
    }
    f.res.t_submit = q.t_submit;
    f.res.t_ready = q.t_ready;
    f.res.t_admit = q.t_admit;
    std::lock_guard<std::mutex> lk(S->mu);
    f.res.t_done = S->now();
    S->finished[q.id] = std::move(f);
    S->unpolled.push_back(q.id);
    S->done++;
    S->cv_done.notify_all();
}

int set_run(HostCase *hc, int n_outer, double conv_tol) {
    SolveScalars sc;
    std::memset(&sc, 0, sizeof(sc));
    sc.run_left = n_outer;
    sc.conv_tol = conv_tol;
    return cuda_status(cudaMemcpy(hc->dev.sc, &sc, sizeof(sc), cudaMemcpyHostToDevice));
}

void device_loop(cfdl_server *S) {
    if (cudaSetDevice(S->cfg.device) != cudaSuccess) {
        std::lock_guard<std::mutex> lk(S->mu);
        S->device_status = CFDL_ERR_NO_DEVICE;
        S->stopping = true;
        S->cv_done.notify_all();
        return;
    }
    cfdl_ctx *ctx = ctx_new();
    if (!ctx) {
        std::lock_guard<std::mutex> lk(S->mu);
        S->device_status = CFDL_ERR_CUDA;
        S->cv_done.notify_all();
        return;
    }
    if (S->cfg.tile) { ctx->vec = S->cfg.tile; }
    std::vector<Resident> res;
    std::vector<SolveScalars> sc;
    for (;;) {
        bool changed = false;
        // ---- retire ----
        sc.resize(res.size());
        for (size_t c = 0; c < res.size(); c++)
            if (cudaMemcpyAsync(&sc[c], res[c].hc->dev.sc, sizeof(SolveScalars), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
                sc[c].run_left = -1;
        cudaStreamSynchronize(ctx->stream);
        double cell_iters = 0;
        for (size_t c = 0; c < res.size(); c++) {
            cell_iters += (double)(sc[c].outer_done - res[c].outer_seen) * res[c].hc->ne;
            res[c].outer_seen = sc[c].outer_done;
        }
        for (size_t c = res.size(); c-- > 0;) {
            if (sc[c].run_left > 0) continue;
            Resident &R = res[c];
            Finished f;
            int status = CFDL_OK;
            for (int q = 0; q < 3; q++) if (sc[c].status[q] == CFDL_ERR_NONFINITE) status = CFDL_ERR_NONFINITE;
            if (sc[c].status_p == CFDL_ERR_NONFINITE) status = CFDL_ERR_NONFINITE;
            if (R.req->r.keep_fields) {
                const size_t nc = (size_t)R.hc->ne + R.hc->nbf;
                std::vector<double> *dst[4] = {&f.u, &f.v, &f.w, &f.p};
                double *src[4] = {R.hc->dev.u, R.hc->dev.v, R.hc->dev.w, R.hc->dev.p};
                for (int k = 0; k < 4; k++) {
                    dst[k]->resize(nc);
                    cudaMemcpyAsync(dst[k]->data(), src[k], nc * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
                }
                if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) status = CFDL_ERR_CUDA;
            }
            const size_t bytes = R.reserved;
            destroy_case(R.hc);
            ctx->cases.erase(ctx->cases.begin() + c);
            finish_request(S, *R.req, status, &sc[c], nullptr, std::move(f));
            res.erase(res.begin() + c);
            std::lock_guard<std::mutex> lk(S->mu);
            S->held_bytes -= bytes;
            changed = true;
        }
        // ---- admit ----
        std::vector<std::unique_ptr<Request>> admit;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cell_iters += cell_iters;
            for (;;) {
                size_t planned = S->held_bytes;
                for (auto &a : admit) planned += a->est;
                while (!S->ready.empty() && (int)(res.size() + admit.size()) < S->cfg.max_cases) {
                    auto it = S->ready.begin();
                    if (it->second->status == CFDL_OK && planned + it->second->est > (size_t)S->cfg.hbm_budget &&
                        !(res.empty() && admit.empty()))
                        break;
                    planned += it->second->est;
                    admit.push_back(std::move(it->second));
                    S->ready.erase(it);
                }
                if (S->stopping) break;
                if (!res.empty() || !admit.empty()) break;
                S->cv_dev.wait(lk);
            }
            if (S->stopping) {
                lk.unlock();
                for (Resident &R : res) R.hc = nullptr;   // destroyed with the context below
                cfdl_ctx_destroy(ctx);
                return;
            }
        }
        for (auto &q : admit) {
            if (q->status != CFDL_OK) { finish_request(S, *q, q->status, nullptr, nullptr, Finished()); continue; }
            size_t free_b = 0, total_b = 0;
            cudaMemGetInfo(&free_b, &total_b);
            if (free_b < q->est + (size_t)S->cfg.hbm_reserve && !res.empty()) {
                // not now: back to the front of the queue
                std::lock_guard<std::mutex> lk(S->mu);
                const int64_t id = q->id;
                S->ready[id] = std::move(q);
                continue;
            }
            HostCase *hc = nullptr;
            const cfdl_config cfg = request_config(S->cfg, q->r);
            int st = upload_case(q->prep, &cfg, &hc);
            if (!st) st = set_run(hc, q->r.max_outer, q->r.conv_tol);
            if (st) {
                if (hc) destroy_case(hc);
                finish_request(S, *q, st, nullptr, nullptr, Finished());
                continue;
            }
            hc->id = ctx->next_id++;
            ctx->cases.push_back(hc);
            q->t_admit = S->now();
            q->prep.release_tables();   // host tables no longer needed
            // the budget holds the larger of the estimate and what was
            // allocated, so later allocations of the case stay covered
            const size_t reserved = std::max(q->est, hc->bytes);
            {
                std::lock_guard<std::mutex> lk(S->mu);
                S->held_bytes += reserved;
            }
            Resident R;
            R.req = std::move(q);
            R.hc = hc;
            R.reserved = reserved;
            res.push_back(std::move(R));
            changed = true;
        }
        if (res.empty()) continue;
        if (changed && rebuild_worklists(ctx) != CFDL_OK) {
            std::lock_guard<std::mutex> lk(S->mu);
            S->device_status = CFDL_ERR_CUDA;
        }
        // ---- run ----
        const auto t_run = Clock::now();
        int running = 0;
        int st = run_outer(ctx, S->cfg.chunk, &running);
        const double dt_run = std::chrono::duration<double>(Clock::now() - t_run).count();
        std::lock_guard<std::mutex> lk(S->mu);
        S->resident = (int)res.size();
        S->launches++;
        S->busy_s += dt_run;
        if (st) S->device_status = st;
    }
}

}  // namespace

extern "C" {

void cfdl_server_config_default(cfdl_server_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->device = 0;
    c->hbm_budget = 150e9;
    c->hbm_reserve = 4e9;
    c->max_cases = 64;
    c->chunk = 10;
    c->prep_threads = 8;
    c->precision = 1;
    c->precond = 1;
    c->tile = 0;
    c->alpha_u = 0.7;
    c->alpha_p = 0.3;
    c->device_setup = 1;
}

int cfdl_server_create(const cfdl_server_config *cfg, cfdl_server **out) {
    if (!cfg || !out) return CFDL_ERR_INVALID;
    *out = nullptr;
    if (cfg->max_cases <= 0 || cfg->chunk <= 0 || cfg->prep_threads <= 0 || !(cfg->hbm_budget > 0) ||
        !(cfg->hbm_reserve >= 0) || cfg->precision < 0 || cfg->precision > 3 || (cfg->precond != 0 && cfg->precond != 1) ||
        !(cfg->tile == 0 || cfg->tile == 1 || cfg->tile == 2 || cfg->tile == 4 || cfg->tile == 8) ||
        !(cfg->alpha_u > 0 && cfg->alpha_u <= 1) || !(cfg->alpha_p > 0 && cfg->alpha_p <= 1))
        return CFDL_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device) { cudaGetLastError(); return CFDL_ERR_NO_DEVICE; }
    cfdl_server *S = new (std::nothrow) cfdl_server;
    if (!S) return CFDL_ERR_OOM;
    S->cfg = *cfg;
    S->t0 = Clock::now();
    for (int i = 0; i < cfg->prep_threads; i++) S->preppers.emplace_back(prep_loop, S);
    S->device = std::thread(device_loop, S);
    *out = S;
    return CFDL_OK;
}

int cfdl_server_submit(cfdl_server *S, const cfdl_request *r, int64_t *id) {
    if (!S || !r) return CFDL_ERR_INVALID;
    if (r->n < 1 || (r->tet != 0 && r->tet != 1) || !(r->jitter >= 0 && r->jitter < 0.5) || !(r->re > 0) ||
        !(r->conv_tol >= 0) || r->max_outer <= 0)
        return CFDL_ERR_INVALID;
    auto q = std::make_unique<Request>();
    q->r = *r;
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stopping) return CFDL_ERR_INVALID;
    q->id = S->next_id++;
    q->t_submit = S->now();
    if (id) *id = q->id;
    S->pending.push_back(std::move(q));
    S->submitted++;
    S->cv_prep.notify_one();
    return CFDL_OK;
}

int cfdl_server_poll(cfdl_server *S, cfdl_result *out, int max, int *n, double wait_s) {
    if (!S || !n || (max > 0 && !out)) return CFDL_ERR_INVALID;
    std::unique_lock<std::mutex> lk(S->mu);
    if (S->unpolled.empty() && wait_s > 0)
        S->cv_done.wait_for(lk, std::chrono::duration<double>(wait_s), [&] { return !S->unpolled.empty(); });
    int k = 0;
    while (k < max && !S->unpolled.empty()) {
        out[k++] = S->finished[S->unpolled.front()].res;
        S->unpolled.pop_front();
    }
    *n = k;
    return S->device_status;
}

int cfdl_server_fields(cfdl_server *S, int64_t id, const char *name, double *host, int64_t *len) {
    if (!S || !name) return CFDL_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->finished.find(id);
    if (it == S->finished.end()) return CFDL_ERR_INVALID;
    const std::vector<double> *v = nullptr;
    if (!std::strcmp(name, "u")) v = &it->second.u;
    else if (!std::strcmp(name, "v")) v = &it->second.v;
    else if (!std::strcmp(name, "w")) v = &it->second.w;
    else if (!std::strcmp(name, "p")) v = &it->second.p;
    else return CFDL_ERR_NAME;
    if (len) *len = (int64_t)v->size();
    if (host && !v->empty()) std::memcpy(host, v->data(), v->size() * sizeof(double));
    return CFDL_OK;
}

int cfdl_server_drain(cfdl_server *S, double timeout_s) {
    if (!S) return CFDL_ERR_INVALID;
    std::unique_lock<std::mutex> lk(S->mu);
    auto all_done = [&] { return S->done == S->submitted || S->device_status != CFDL_OK; };
    if (timeout_s > 0) {
        if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), all_done)) return CFDL_ERR_ITER_CAP;
    } else {
        S->cv_done.wait(lk, all_done);
    }
    return S->device_status;
}

int cfdl_server_query(cfdl_server *S, cfdl_server_info *info) {
    if (!S || !info) return CFDL_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    info->submitted = S->submitted;
    info->done = S->done;
    info->queued = (int64_t)(S->pending.size() + S->ready.size()) + S->preparing;
    info->resident = S->resident;
    info->held_bytes = (double)S->held_bytes;
    info->launches = S->launches;
    info->cell_iters = S->cell_iters;
    info->busy_s = S->busy_s;
    info->now = S->now();
    return S->device_status;
}

double cfdl_server_now(cfdl_server *S) { return S ? S->now() : 0.0; }

int cfdl_server_destroy(cfdl_server *S) {
    if (!S) return CFDL_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stopping = true;
    }
    S->cv_prep.notify_all();
    S->cv_dev.notify_all();
    for (auto &t : S->preppers) t.join();
    if (S->device.joinable()) S->device.join();
    delete S;
    return CFDL_OK;
}

}  // extern "C"
