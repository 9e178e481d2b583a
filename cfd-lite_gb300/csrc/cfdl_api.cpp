// cfdl_api.cpp -- the C-ABI of libcfdgpu (declared in include/cfdl.h).
//
// The entry points mirror the reference's Fortran routines one for one; see
// the header for the citation of each.  All work is queued on the context's
// stream; entry points that return results to the host synchronise it.
#include "cfdl_internal.h"
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <atomic>
#include <algorithm>

using namespace cfdl;

namespace {

int check_ctx(const cfdl_ctx *ctx) { return ctx && !ctx->cases.empty() ? CFDL_OK : CFDL_ERR_INVALID; }

int validate_config(const cfdl_config *c) {
    if (!c) return CFDL_ERR_INVALID;
    if (!(c->rho > 0) || !(c->mu >= 0) || !(c->dt > 0) || !(c->alpha_u > 0 && c->alpha_u <= 1) ||
        !(c->alpha_p > 0 && c->alpha_p <= 1) || c->nit < 0 || c->tight_maxit < 0 ||
        (c->solve_mode != 0 && c->solve_mode != 1) || c->precision < 0 || c->precision > 3 ||
        (c->precision >= 2 && c->solve_mode != 0) ||
        !(c->rtol_u > 0) || !(c->rtol_p > 0) || !(c->tight_rtol > 0) || (c->precond != 0 && c->precond != 1))
        return CFDL_ERR_INVALID;
    return CFDL_OK;
}

struct Named { double *ptr; size_t n; bool ell; };

Named lookup(HostCase *hc, const char *name) {
    CaseDev &d = hc->dev;
    const size_t nc = (size_t)hc->ne + hc->nbf, ne = hc->ne, nf = hc->nf;
    std::string s(name ? name : "");
    struct E { const char *nm; double *p; size_t n; };
    const E tab[] = {
        {"u", d.u, nc}, {"v", d.v, nc}, {"w", d.w, nc}, {"p", d.p, nc},
        {"u0", d.u0, nc}, {"v0", d.v0, nc}, {"w0", d.w0, nc}, {"phic", d.phic, nc},
        {"gu", d.gu, 3 * nc}, {"gv", d.gv, 3 * nc}, {"gw", d.gw, 3 * nc}, {"gp", d.gp, 3 * nc}, {"gpc", d.gpc, 3 * nc},
        {"mip", d.mip, nf}, {"mip0", d.mip0, nf},
        {"b", d.b, ne}, {"bu", d.bu, ne}, {"bv", d.bv, ne}, {"bw", d.bw, ne},
        {"d", d.d, ne}, {"dc", d.dc, ne}, {"rho", d.rho, ne}, {"mu", d.mu, ne},
        // energy equation (null until cfdl_energy_init)
        {"t", d.et, nc}, {"e", d.ee, nc}, {"e0", d.ee0, nc}, {"gt", d.egt, 3 * nc}, {"ge", d.ege, 3 * nc},
        {"cp", d.ecp, ne}, {"tc", d.etc, ne},
    };
    for (const E &e : tab) if (s == e.nm) return {e.p, e.n, false};
    // ap/anb as the reference's phys_t holds them: the last assembly's (the
    // pressure matrix after calc_coef_p / solve_uvwp)
    if (s == "anb") return {hc->coef_is_pressure ? d.anb_p : d.anb, (size_t)hc->H, true};
    if (s == "ap") return {hc->coef_is_pressure ? d.ap_p : d.ap, ne, false};
    return {nullptr, 0, false};
}

int copy_named(cfdl_ctx *ctx, HostCase *hc, const char *name, double *host, bool to_host) {
    Named nm = lookup(hc, name);
    if (!nm.ptr) return CFDL_ERR_NAME;
    if (!host) return CFDL_ERR_INVALID;
    if (!to_host) ctx->host_writes++;
    if (!to_host && (nm.ptr == hc->dev.rho || nm.ptr == hc->dev.mu)) hc->props_dirty = true;
    if (!to_host && nm.ptr && (nm.ptr == hc->dev.ecp || nm.ptr == hc->dev.etc)) hc->eprops_dirty = true;
    if (!to_host && (nm.ptr == hc->dev.gu || nm.ptr == hc->dev.gv || nm.ptr == hc->dev.gw || nm.ptr == hc->dev.gp ||
                     nm.ptr == hc->dev.d))
        hc->g32_stale = true;
    cudaError_t e;
    if (!nm.ell) {
        e = cudaMemcpyAsync(to_host ? (void *)host : (void *)nm.ptr, to_host ? (const void *)nm.ptr : (const void *)host,
                            nm.n * sizeof(double), to_host ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        return cuda_status(e);
    }
    // anb: ELL [W][ne] <-> reference CSR half-face order
    const int ne = hc->ne, W = hc->W;
    std::vector<double> ell((size_t)W * ne, 0.0);
    if (to_host) {
        e = cudaMemcpyAsync(ell.data(), nm.ptr, ell.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_status(e);
        for (int c = 0; c < ne; c++)
            for (int idx = hc->ef2nb_idx[c]; idx < hc->ef2nb_idx[c + 1]; idx++)
                host[idx - 1] = ell[(size_t)(idx - hc->ef2nb_idx[c]) * ne + c];
        return CFDL_OK;
    }
    for (int c = 0; c < ne; c++)
        for (int idx = hc->ef2nb_idx[c]; idx < hc->ef2nb_idx[c + 1]; idx++)
            ell[(size_t)(idx - hc->ef2nb_idx[c]) * ne + c] = host[idx - 1];
    e = cudaMemcpyAsync(nm.ptr, ell.data(), ell.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return cuda_status(e);
}

int transfer_fields(cfdl_ctx *ctx, HostCase *hc, const cfdl_fields *f, bool to_host) {
    if (!f) return CFDL_ERR_INVALID;
    CaseDev &d = hc->dev;
    const size_t nc = (size_t)hc->ne + hc->nbf, nf = hc->nf;
    struct P { double *h; double *dv; size_t n; };
    const P list[] = {
        {f->u, d.u, nc}, {f->v, d.v, nc}, {f->w, d.w, nc}, {f->p, d.p, nc},
        {f->u0, d.u0, nc}, {f->v0, d.v0, nc}, {f->w0, d.w0, nc},
        {f->gu, d.gu, 3 * nc}, {f->gv, d.gv, 3 * nc}, {f->gw, d.gw, 3 * nc}, {f->gp, d.gp, 3 * nc}, {f->gpc, d.gpc, 3 * nc},
        {f->mip, d.mip, nf}, {f->mip0, d.mip0, nf},
    };
    if (!to_host && (f->gu || f->gv || f->gw || f->gp)) hc->g32_stale = true;   // precision 3 derives g32, gp32 from them
    for (const P &p : list) {
        if (!p.h) continue;
        if (!to_host) ctx->host_writes++;
        cudaError_t e = to_host ? cudaMemcpyAsync(p.h, p.dv, p.n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream)
                                : cudaMemcpyAsync(p.dv, p.h, p.n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return cuda_status(e);
    }
    return CFDL_OK;
}

int finish(cfdl_ctx *ctx, cfdl_stats *st) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e);
    if (st) {
        int s = read_stats(ctx, 0, st);
        if (s) return s;
        return st->status == CFDL_ERR_NONFINITE || st->status == CFDL_ERR_ITER_CAP ? st->status : CFDL_OK;
    }
    return CFDL_OK;
}

}  // namespace

namespace cfdl {
cfdl_ctx *ctx_new() {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return nullptr; }
    cfdl_ctx *ctx = new (std::nothrow) cfdl_ctx;
    if (!ctx) return nullptr;
    cudaGetDevice(&ctx->device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return nullptr; }
    return ctx;
}

int solve_uvwp_all(cfdl_ctx *ctx) {
    // solve_uvwp, src/equations/mod_uvwp.f90:95-134: as one graph launch unless
    // graphs are off or launches are being profiled one by one.  The pressure
    // matrix needs only dc of calc_coef_uvw, so it and the pressure solve's
    // operators are built right after it (in the graph: beside the momentum
    // solve); the right-hand side follows calc_mip.
    if (ctx->use_graph && !prof_active(ctx)) return solve_uvwp_graph(ctx);
    int st;
    if (ctx->cases[0]->cfg.precond == 1 && (st = ensure_amg(ctx))) return st;
    launch_coef_uvw(ctx);
    launch_coef_p_matrix(ctx);
    pressure_operators(ctx);
    if ((st = solve_momentum(ctx))) return st;
    launch_grad(ctx, 4);
    if (ctx->ev_mom) cudaEventRecord(ctx->ev_mom, ctx->stream);
    launch_calc_mip(ctx, 1);
    launch_coef_p_rhs(ctx);
    st = solve_pressure_prepared(ctx);
    if (st) return st;
    launch_adjust_pc(ctx);
    launch_grad(ctx, 3);
    launch_update_uvwp(ctx);
    return cuda_status(cudaGetLastError());
}
}  // namespace cfdl

extern "C" {

void cfdl_config_default(cfdl_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    // reference defaults: mod_physics.f90:15-19, mod_properties.f90:86-87
    c->rho = 5.0; c->mu = 0.01; c->dt = 0.01;
    c->alpha_u = 1.0; c->alpha_p = 1.0;
    c->nit = 100; c->solve_mode = 0; c->rtol_u = 0.1; c->rtol_p = 0.1;
    c->tight_rtol = 1e-13; c->tight_maxit = 20000;
    c->precision = 0; c->precond = 1;
}

const char *cfdl_status_string(int s) {
    switch (s) {
    case CFDL_OK: return "ok";
    case CFDL_ERR_INVALID: return "invalid argument";
    case CFDL_ERR_OOM: return "out of memory";
    case CFDL_ERR_NONFINITE: return "non-finite value in a solve";
    case CFDL_ERR_ITER_CAP: return "inner solve reached its iteration cap";
    case CFDL_ERR_CUDA: return "CUDA runtime error";
    case CFDL_ERR_MESH: return "mesh connectivity error";
    case CFDL_ERR_NO_DEVICE: return "no CUDA device";
    case CFDL_ERR_NAME: return "unknown array name";
    case CFDL_ERR_TOO_LARGE: return "problem larger than the fixed scratch of the allocation-free entry point";
    case CFDL_ERR_BREAKDOWN: return "Krylov breakdown: p.Ap <= 0 above the tolerance (matrix not positive definite)";
    default: return "unknown status";
    }
}

int cfdl_mesh_check(const cfdl_mesh *mesh) {
    cfdl::CasePrep p;
    return cfdl::prepare_case(mesh, &p);
}

int cfdl_ctx_create(const cfdl_mesh *mesh, const cfdl_config *cfg, cfdl_ctx **out) {
    if (!out) return CFDL_ERR_INVALID;
    *out = nullptr;
    int st = validate_config(cfg);
    if (st) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return CFDL_ERR_NO_DEVICE; }
    cfdl_ctx *ctx = new (std::nothrow) cfdl_ctx;
    if (!ctx) return CFDL_ERR_OOM;
    cudaGetDevice(&ctx->device);
    if ((st = cuda_status(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)))) { delete ctx; return st; }
    HostCase *hc = nullptr;
    if ((st = create_case(ctx, mesh, cfg, &hc))) { cfdl_ctx_destroy(ctx); return st; }
    hc->id = ctx->next_id++;
    ctx->cases.push_back(hc);
    if ((st = rebuild_worklists(ctx))) { cfdl_ctx_destroy(ctx); return st; }
    // construct_uvwp: mip = calc_mip(.false.) from the zero fields, mip0 = mip
    launch_calc_mip(ctx, 0);
    launch_set_mip0(ctx);
    if ((st = cuda_status(cudaStreamSynchronize(ctx->stream)))) { cfdl_ctx_destroy(ctx); return st; }
    *out = ctx;
    return CFDL_OK;
}

int cfdl_set_config(cfdl_ctx *ctx, const cfdl_config *cfg) {
    int st = check_ctx(ctx);
    if (st) return st;
    if ((st = validate_config(cfg))) return st;
    for (HostCase *hc : ctx->cases) {
        if (hc->cfg.rho != cfg->rho || hc->cfg.mu != cfg->mu) {
            hc->props_dirty = true;
            std::vector<double> rho(hc->ne, cfg->rho), mu(hc->ne, cfg->mu);
            if ((st = cuda_status(cudaMemcpy(hc->dev.rho, rho.data(), hc->ne * sizeof(double), cudaMemcpyHostToDevice)))) return st;
            if ((st = cuda_status(cudaMemcpy(hc->dev.mu, mu.data(), hc->ne * sizeof(double), cudaMemcpyHostToDevice)))) return st;
        }
        if (cfg->precision == 3 && (st = ensure_f32_assembly(hc, ctx->stream))) return st;
        if (cfg->precision == 3 && hc->cfg.precision != 3) hc->g32_stale = true;
        apply_config(hc, cfg);
    }
    return upload_case_table(ctx);
}

int cfdl_upload_fields(cfdl_ctx *ctx, const cfdl_fields *f) {
    int st = check_ctx(ctx);
    if (st) return st;
    if ((st = transfer_fields(ctx, ctx->cases[0], f, false))) return st;
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_download_fields(cfdl_ctx *ctx, cfdl_fields *f) {
    int st = check_ctx(ctx);
    if (st) return st;
    if ((st = transfer_fields(ctx, ctx->cases[0], f, true))) return st;
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_ctx_destroy(cfdl_ctx *ctx) {
    if (!ctx) return CFDL_ERR_INVALID;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (HostCase *hc : ctx->cases) destroy_case(hc);
    WorkList *wls[3] = {&ctx->cells, &ctx->faces, &ctx->halos};
    for (WorkList *wl : wls) free_worklist(*wl);
    free_worklist(ctx->cellsv);
    free_worklist(ctx->cellse);
    free_worklist(ctx->facesv);
    for (auto &wl : ctx->amg_cells) free_worklist(wl);
    for (auto &wl : ctx->amg_smooth) free_worklist(wl);
    for (auto &wl : ctx->amg_gcells) free_worklist(wl);
    for (auto &wl : ctx->amg_gsmooth) free_worklist(wl);
    for (auto &wl : ctx->amg_restr) free_worklist(wl);
    for (auto &wl : ctx->amg_grestr) free_worklist(wl);
    cudaFree(ctx->d_cases);
    cudaFree(ctx->d_partials);
    cudaFree(ctx->d_flags);
    if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    prof_destroy(ctx);
    destroy_graph(ctx);
    cudaFree(ctx->d_loop_passes);
    cudaFree(ctx->d_run_ctl);
    if (ctx->ev_mom) cudaEventDestroy(ctx->ev_mom);
    if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->h_run_ctl) cudaFreeHost(ctx->h_run_ctl);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return CFDL_OK;
}

int cfdl_update_boundaries(cfdl_ctx *ctx) {
    int st = check_ctx(ctx);
    if (st) return st;
    launch_bc(ctx);
    return cuda_status(cudaGetLastError());
}

int cfdl_solve_uvwp(cfdl_ctx *ctx, cfdl_stats *stats) {
    int st = check_ctx(ctx);
    if (st) return st;
    if ((st = solve_uvwp_all(ctx))) return st;
    return finish(ctx, stats);
}

int cfdl_update_time(cfdl_ctx *ctx) {
    int st = check_ctx(ctx);
    if (st) return st;
    launch_update_time(ctx);
    return cuda_status(cudaGetLastError());
}

int cfdl_step(cfdl_ctx *ctx, int n_outer, int ncoef, cfdl_stats *stats) {
    int st = check_ctx(ctx);
    if (st) return st;
    if (n_outer < 0) return CFDL_ERR_INVALID;
    for (int k = 1; k <= n_outer; k++) {
        launch_bc(ctx);
        if ((st = solve_uvwp_all(ctx))) return st;
        if ((st = solve_energy_all(ctx))) return st;    // main.f90:58, when set up
        if (ncoef > 0 && k % ncoef == 0) launch_update_time(ctx);
    }
    return finish(ctx, stats);
}

static int ensure_copy_stream(cfdl_ctx *ctx) {
    if (ctx->copy_stream) return CFDL_OK;
    int st;
    if ((st = cuda_status(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking)))) return st;
    if ((st = cuda_status(cudaEventCreateWithFlags(&ctx->ev_mom, cudaEventDisableTiming)))) return st;
    if ((st = cuda_status(cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming)))) return st;
    destroy_graph(ctx);   // rebuilt with a record of ev_mom after the momentum half
    return CFDL_OK;
}

// Downloads f after the last solve_uvwp queued on ctx->stream.  u, v, w and
// their gradients are final once the momentum solve and calc_grad(u,v,w) are
// done (update_uvwp corrects p, gp and mip only) and the old-time fields do
// not change, so they go back on the copy stream while the pressure
// correction runs; p, gp, gpc and mip follow on the main stream.
static int download_overlapped(cfdl_ctx *ctx, HostCase *hc, const cfdl_fields *f) {
    cfdl_fields early = {}, late = {};
    early.u = f->u; early.v = f->v; early.w = f->w; early.gu = f->gu; early.gv = f->gv; early.gw = f->gw;
    early.u0 = f->u0; early.v0 = f->v0; early.w0 = f->w0; early.mip0 = f->mip0;
    late.p = f->p; late.gp = f->gp; late.gpc = f->gpc; late.mip = f->mip;
    int st;
    cudaStream_t main_stream = ctx->stream;
    if ((st = cuda_status(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_mom, 0)))) return st;
    ctx->stream = ctx->copy_stream;
    st = transfer_fields(ctx, hc, &early, true);
    ctx->stream = main_stream;
    if (st) return st;
    if ((st = cuda_status(cudaEventRecord(ctx->ev_copy, ctx->copy_stream)))) return st;
    if ((st = transfer_fields(ctx, hc, &late, true))) return st;
    if ((st = cuda_status(cudaStreamWaitEvent(ctx->stream, ctx->ev_copy, 0)))) return st;
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

// The members of a cfdl_fields in CFDL_F_* bit order.
static double **field_slot(cfdl_fields *f, int k) {
    double **m[14] = {&f->u, &f->v, &f->w, &f->p, &f->u0, &f->v0, &f->w0,
                      &f->gu, &f->gv, &f->gw, &f->gp, &f->gpc, &f->mip, &f->mip0};
    return m[k];
}

// The host drop-in's upload: every non-NULL member of f, except those the
// caller declares unchanged (keep) whose host array is the one the last
// drop-in download filled while nothing has written the device since.
static int upload_changed(cfdl_ctx *ctx, HostCase *hc, const cfdl_fields *f, unsigned keep) {
    const bool clean = ctx->launches == ctx->synced_launches && ctx->graph_launches == ctx->synced_graphs &&
                       ctx->host_writes == ctx->synced_writes;
    cfdl_fields up = *f;
    for (int k = 0; k < 14; k++) {
        double **slot = field_slot(&up, k);
        if (clean && (keep >> k & 1u) && *slot && *slot == ctx->synced_ptr[k]) *slot = nullptr;
    }
    return transfer_fields(ctx, hc, &up, false);
}

// After the drop-in's download: which host arrays now equal the device's.
static void mark_synced(cfdl_ctx *ctx, cfdl_fields *f) {
    for (int k = 0; k < 14; k++) ctx->synced_ptr[k] = *field_slot(f, k);
    ctx->synced_launches = ctx->launches;
    ctx->synced_graphs = ctx->graph_launches;
    ctx->synced_writes = ctx->host_writes;
}

int cfdl_solve_uvwp_host(cfdl_ctx *ctx, cfdl_fields *f, cfdl_stats *stats) {
    int st = check_ctx(ctx);
    if (st) return st;
    if (!f) return CFDL_ERR_INVALID;
    HostCase *hc = ctx->cases[0];
    if ((st = ensure_copy_stream(ctx))) return st;
    if ((st = transfer_fields(ctx, hc, f, false))) return st;
    if ((st = solve_uvwp_all(ctx))) return st;
    if ((st = download_overlapped(ctx, hc, f))) return st;
    mark_synced(ctx, f);
    return finish(ctx, stats);
}

int cfdl_step_host_keep(cfdl_ctx *ctx, cfdl_fields *f, unsigned keep, int n_outer, int ncoef, cfdl_stats *stats) {
    int st = check_ctx(ctx);
    if (st) return st;
    if (!f || n_outer < 1 || (keep >> 14) != 0u) return CFDL_ERR_INVALID;
    HostCase *hc = ctx->cases[0];
    if ((st = ensure_copy_stream(ctx))) return st;
    if ((st = upload_changed(ctx, hc, f, keep))) return st;
    for (int k = 1; k <= n_outer; k++) {
        launch_bc(ctx);
        if ((st = solve_uvwp_all(ctx))) return st;
        if ((st = solve_energy_all(ctx))) return st;    // main.f90:58, when set up
        if (ncoef > 0 && k % ncoef == 0) launch_update_time(ctx);
    }
    if ((st = download_overlapped(ctx, hc, f))) return st;
    mark_synced(ctx, f);
    return finish(ctx, stats);
}

int cfdl_step_host(cfdl_ctx *ctx, cfdl_fields *f, int n_outer, int ncoef, cfdl_stats *stats) {
    return cfdl_step_host_keep(ctx, f, 0u, n_outer, ncoef, stats);
}

int cfdl_calc_coef_uvw(cfdl_ctx *ctx) {
    int st = check_ctx(ctx);
    if (st) return st;
    launch_coef_uvw(ctx);
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_solve_momentum(cfdl_ctx *ctx, cfdl_stats *stats) {
    int st = check_ctx(ctx);
    if (st) return st;
    if ((st = solve_momentum(ctx))) return st;
    return finish(ctx, stats);
}

int cfdl_calc_grad(cfdl_ctx *ctx, int field) {
    int st = check_ctx(ctx);
    if (st) return st;
    if (field < 0 || field > 5 || (field == 5 && !energy_on(ctx))) return CFDL_ERR_INVALID;
    launch_grad(ctx, field);
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_calc_mip(cfdl_ctx *ctx, int rhie_chow) {
    int st = check_ctx(ctx);
    if (st) return st;
    launch_calc_mip(ctx, rhie_chow ? 1 : 0);
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_calc_coef_p(cfdl_ctx *ctx) {
    int st = check_ctx(ctx);
    if (st) return st;
    launch_coef_p(ctx);
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_solve_pc(cfdl_ctx *ctx, cfdl_stats *stats) {
    int st = check_ctx(ctx);
    if (st) return st;
    if ((st = solve_pressure(ctx))) return st;
    return finish(ctx, stats);
}

int cfdl_adjust_pc(cfdl_ctx *ctx) {
    int st = check_ctx(ctx);
    if (st) return st;
    launch_adjust_pc(ctx);
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_update_uvwp(cfdl_ctx *ctx) {
    int st = check_ctx(ctx);
    if (st) return st;
    launch_update_uvwp(ctx);
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_energy_init(cfdl_ctx *ctx, double cp, double tc, double t_init) {
    int st = check_ctx(ctx);
    if (st) return st;
    if (!(cp > 0) || !(tc >= 0) || !std::isfinite(cp) || !std::isfinite(tc) || !std::isfinite(t_init))
        return CFDL_ERR_INVALID;
    for (HostCase *hc : ctx->cases)
        if (hc->h_temp.empty()) return CFDL_ERR_INVALID;   // the mesh carried no energy BCs
    for (HostCase *hc : ctx->cases)
        if ((st = energy_init_case(ctx, hc, cp, tc, t_init))) break;
    // the device table follows the host records even after a failure part way
    destroy_graph(ctx);   // graphs captured without (or with) the energy launches
    const int st2 = upload_case_table(ctx);
    if (st) return st;
    if (st2) return st2;
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_solve_energy(cfdl_ctx *ctx, cfdl_stats *stats) {
    int st = check_ctx(ctx);
    if (st) return st;
    if (!energy_on(ctx)) return CFDL_ERR_INVALID;
    if ((st = solve_energy_all(ctx))) return st;
    if ((st = finish(ctx, stats))) return st;
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_calc_coef_energy(cfdl_ctx *ctx) {
    int st = check_ctx(ctx);
    if (st) return st;
    if (!energy_on(ctx)) return CFDL_ERR_INVALID;
    launch_coef_energy(ctx);
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int cfdl_get_array(cfdl_ctx *ctx, const char *name, double *host) {
    int st = check_ctx(ctx);
    if (st) return st;
    return copy_named(ctx, ctx->cases[0], name, host, true);
}

int cfdl_set_array(cfdl_ctx *ctx, const char *name, const double *host) {
    int st = check_ctx(ctx);
    if (st) return st;
    return copy_named(ctx, ctx->cases[0], name, const_cast<double *>(host), false);
}

int64_t cfdl_launch_count(const cfdl_ctx *ctx) {
    if (!ctx) return -1;
    return ctx->launches + graph_loop_kernels(const_cast<cfdl_ctx *>(ctx));
}

// ---------------------------------------------------------------- batches
static int find_case(const cfdl_ctx *ctx, int id) {
    for (size_t c = 0; c < ctx->cases.size(); c++) if (ctx->cases[c]->id == id) return (int)c;
    return -1;
}

static bool same_form(const cfdl_config *a, const cfdl_config *b) {
    return a->precision == b->precision && a->precond == b->precond;
}

int cfdl_batch_create(int ncases, const cfdl_mesh *meshes, const cfdl_config *cfgs, cfdl_ctx **out) {
    if (!out || ncases <= 0 || !meshes || !cfgs) return CFDL_ERR_INVALID;
    *out = nullptr;
    for (int c = 0; c < ncases; c++) {
        int st = validate_config(&cfgs[c]);
        if (st) return st;
        if (!same_form(&cfgs[0], &cfgs[c])) return CFDL_ERR_INVALID;
    }
    cfdl_ctx *ctx = nullptr;
    int st = cfdl_ctx_create(&meshes[0], &cfgs[0], &ctx);
    if (st) return st;
    // host tables (and multigrid hierarchies) of the other cases on host threads
    std::vector<CasePrep> preps(ncases > 1 ? ncases - 1 : 0);
    std::vector<int> pst(preps.size(), CFDL_OK);
    {
        std::atomic<int> next{0};
        const int nthr = (int)std::min<size_t>(preps.size(), std::max(1u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (int t = 0; t < nthr; t++)
            pool.emplace_back([&] {
                for (int k; (k = next++) < (int)preps.size();) {
                    pst[k] = prepare_case(&meshes[k + 1], &preps[k]);
                    if (!pst[k] && cfgs[k + 1].precond == 1) pst[k] = prepare_case_amg(&preps[k]);
                }
            });
        for (auto &t : pool) t.join();
    }
    for (size_t k = 0; k < preps.size(); k++) {
        HostCase *hc = nullptr;
        if ((st = pst[k]) || (st = upload_case(preps[k], &cfgs[k + 1], &hc))) { cfdl_ctx_destroy(ctx); return st; }
        preps[k].release_tables();
        hc->id = ctx->next_id++;
        ctx->cases.push_back(hc);
    }
    if ((st = rebuild_worklists(ctx))) { cfdl_ctx_destroy(ctx); return st; }
    *out = ctx;
    return CFDL_OK;
}

int cfdl_case_add(cfdl_ctx *ctx, const cfdl_mesh *mesh, const cfdl_config *cfg, int *id) {
    int st = check_ctx(ctx);
    if (st) return st;
    if ((st = validate_config(cfg))) return st;
    if (!same_form(&ctx->cases[0]->cfg, cfg)) return CFDL_ERR_INVALID;
    if ((st = cuda_status(cudaStreamSynchronize(ctx->stream)))) return st;
    HostCase *hc = nullptr;
    if ((st = create_case(ctx, mesh, cfg, &hc))) return st;
    hc->id = ctx->next_id++;
    ctx->cases.push_back(hc);
    // construct_uvwp on zero fields leaves mip = mip0 = 0, as allocated
    if ((st = rebuild_worklists(ctx))) return st;
    if (id) *id = hc->id;
    return CFDL_OK;
}

int cfdl_case_remove(cfdl_ctx *ctx, int id) {
    int st = check_ctx(ctx);
    if (st) return st;
    int c = find_case(ctx, id);
    if (c < 0) return CFDL_ERR_INVALID;
    if (ctx->cases.size() == 1) return CFDL_ERR_INVALID;   // a context keeps at least one case
    if ((st = cuda_status(cudaStreamSynchronize(ctx->stream)))) return st;
    destroy_case(ctx->cases[c]);
    ctx->cases.erase(ctx->cases.begin() + c);
    return rebuild_worklists(ctx);
}

int cfdl_case_count(const cfdl_ctx *ctx) { return ctx ? (int)ctx->cases.size() : -1; }

int cfdl_case_ids(const cfdl_ctx *ctx, int *ids) {
    if (!ctx || !ids) return CFDL_ERR_INVALID;
    for (size_t c = 0; c < ctx->cases.size(); c++) ids[c] = ctx->cases[c]->id;
    return CFDL_OK;
}

int cfdl_case_get_array(cfdl_ctx *ctx, int id, const char *name, double *host) {
    int st = check_ctx(ctx);
    if (st) return st;
    int c = find_case(ctx, id);
    if (c < 0) return CFDL_ERR_INVALID;
    return copy_named(ctx, ctx->cases[c], name, host, true);
}

int cfdl_case_set_array(cfdl_ctx *ctx, int id, const char *name, const double *host) {
    int st = check_ctx(ctx);
    if (st) return st;
    int c = find_case(ctx, id);
    if (c < 0) return CFDL_ERR_INVALID;
    return copy_named(ctx, ctx->cases[c], name, const_cast<double *>(host), false);
}

int cfdl_case_stats(cfdl_ctx *ctx, int id, cfdl_stats *st_out) {
    int st = check_ctx(ctx);
    if (st) return st;
    int c = find_case(ctx, id);
    if (c < 0 || !st_out) return CFDL_ERR_INVALID;
    return read_stats(ctx, c, st_out);
}

int cfdl_case_info(const cfdl_ctx *ctx, int id, int *ne, size_t *device_bytes) {
    if (!ctx) return CFDL_ERR_INVALID;
    int c = find_case(ctx, id);
    if (c < 0) return CFDL_ERR_INVALID;
    if (ne) *ne = ctx->cases[c]->ne;
    if (device_bytes) *device_bytes = ctx->cases[c]->bytes;
    return CFDL_OK;
}

size_t cfdl_case_bytes_estimate(int ne, int nf, int nbf, int W) {
    const size_t c = (size_t)ne, f = (size_t)nf, b = (size_t)nbf, nc = c + b, w = (size_t)W;
    size_t bytes = 0;
    bytes += 2 * w * c * 4 + 3 * w * c * 8;          // ELL connectivity, gradient stencil
    bytes += 2 * f * 4 + 16 * f * 8;                 // face tables, geometry planes
    bytes += 3 * b * 4 + 3 * b * 8 + c * 8;          // halo tables, volume
    bytes += 4 * b * 8;                               // the BC loop's per-halo terms
    bytes += 8 * nc * 8 + 15 * nc * 8 + 2 * f * 8;   // cell fields, gradients, mip/mip0
    bytes += 9 * c * 8 + w * c * 8 + 4 * f * 8;      // coefficients, face intermediates
    bytes += 10 * f * 8;                              // property planes
    bytes += 24 * c * 8 + 8 * c * 4 + w * c * 4 + c * 8;   // Krylov and FP32 vectors
    bytes += 160 * c + w * c * 2;                     // multigrid hierarchy (bound), 16-bit mesh offsets
    bytes += 9 * c * 4 + 3 * w * c * 4 + 7 * f * 4;   // precision 3 FP32 gradients, stencil, face planes
    bytes += w * c * 12 + c * 24;                     // the pressure matrix's own storage and FP32 copies
    return bytes;
}

int cfdl_case_set_run(cfdl_ctx *ctx, int id, int n_outer, int ncoef, double conv_tol) {
    int st = check_ctx(ctx);
    if (st) return st;
    if (n_outer < 0 || ncoef < 0 || !(conv_tol >= 0)) return CFDL_ERR_INVALID;
    if (id != -1 && find_case(ctx, id) < 0) return CFDL_ERR_INVALID;
    if ((st = cuda_status(cudaStreamSynchronize(ctx->stream)))) return st;
    for (HostCase *hc : ctx->cases) {
        if (id != -1 && hc->id != id) continue;
        SolveScalars S;
        if ((st = cuda_status(cudaMemcpy(&S, hc->dev.sc, sizeof(S), cudaMemcpyDeviceToHost)))) return st;
        S.run_left = n_outer; S.outer_done = 0; S.ncoef = ncoef; S.halted = 0; S.time_due = 0; S.converged = 0;
        S.conv_tol = conv_tol; S.mip_abs = 0.0; S.mass_ratio = 0.0;
        if ((st = cuda_status(cudaMemcpy(hc->dev.sc, &S, sizeof(S), cudaMemcpyHostToDevice)))) return st;
    }
    return CFDL_OK;
}

int cfdl_run(cfdl_ctx *ctx, int max_outer, int *running) {
    int st = check_ctx(ctx);
    if (st) return st;
    if (max_outer < 0) return CFDL_ERR_INVALID;
    if ((st = run_outer(ctx, max_outer, running))) return st;
    return cuda_status(cudaGetLastError());
}

int cfdl_set_pdl(cfdl_ctx *ctx, int on) {
    int st = check_ctx(ctx);
    if (st) return st;
    if ((st = cuda_status(cudaStreamSynchronize(ctx->stream)))) return st;
    ctx->pdl = on != 0;
    destroy_graph(ctx);   // captured launches carry the launch mode
    return CFDL_OK;
}

int cfdl_set_index16(cfdl_ctx *ctx, int on) {
    int st = check_ctx(ctx);
    if (st) return st;
    if ((st = cuda_status(cudaStreamSynchronize(ctx->stream)))) return st;
    ctx->index16 = on != 0;
    ctx->amg_lmax = -1;   // the choice is made when the multigrid work lists are built
    destroy_graph(ctx);   // captured launches carry the kernel form
    return CFDL_OK;
}

int cfdl_set_graph_mode(cfdl_ctx *ctx, int on) {
    if (!ctx || on < 0 || on > 2) return CFDL_ERR_INVALID;
    const bool branches = on != 2;
    if (branches != ctx->graph_branches) {
        int st = cuda_status(cudaStreamSynchronize(ctx->stream));
        if (st) return st;
        destroy_graph(ctx);
    }
    ctx->use_graph = on != 0;
    ctx->graph_branches = branches;
    return CFDL_OK;
}

}  // extern "C"
