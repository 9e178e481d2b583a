// cfdl_tune.cpp -- the solver tile shape and its autotuner.
//
// The Krylov, multigrid-transfer and reduction kernels of the inner solves
// run over the "wide" cell work list, whose tiles hold kTile * vec cells (vec
// cells per thread).  Wide tiles mean fewer partial sums per reduction and
// more independent loads in flight per thread; narrow tiles mean more CTAs
// for small cases.  The best vec depends on the mix of case sizes, so the
// autotuner measures it: for each candidate it times a few outer iterations
// on the context's own cases, from a snapshot of their state that is put back
// afterwards, and keeps the fastest; with the energy equation set up, the
// tile shape of the energy solve is tuned the same way, on energy solves
// alone.  The tile shape changes the order of the
// partial sums, so results agree across shapes to rounding, not bit for bit;
// the shape is a property of the context, and cases compared bit for bit
// must share it.
#include "cfdl_internal.h"
#include <cstring>

using namespace cfdl;

namespace {

constexpr int kTileShapes[] = {1, 2, 4, 8};

struct Snap { double *p; size_t n; };

std::vector<Snap> state_arrays(HostCase *hc) {
    CaseDev &d = hc->dev;
    const size_t nc = (size_t)hc->ne + hc->nbf, nf = hc->nf;
    std::vector<Snap> v = {{d.u, nc}, {d.v, nc}, {d.w, nc}, {d.p, nc}, {d.u0, nc}, {d.v0, nc}, {d.w0, nc},
                           {d.gu, 3 * nc}, {d.gv, 3 * nc}, {d.gw, 3 * nc}, {d.gp, 3 * nc}, {d.gpc, 3 * nc},
                           {d.mip, nf}, {d.mip0, nf}};
    if (d.ee) {   // the energy equation's state
        const Snap e[] = {{d.et, nc}, {d.ee, nc}, {d.ee0, nc}, {d.egt, 3 * nc}, {d.ege, 3 * nc}};
        v.insert(v.end(), e, e + 5);
    }
    return v;
}

// Device copy of every case's outer-iteration state and solver scalars.
struct Snapshot {
    std::vector<char *> bufs;
    ~Snapshot() { for (char *b : bufs) cudaFree(b); }

    int take(cfdl_ctx *ctx) {
        for (HostCase *hc : ctx->cases) {
            size_t bytes = sizeof(SolveScalars);
            for (const Snap &s : state_arrays(hc)) bytes += s.n * sizeof(double);
            char *b = nullptr;
            int st = cuda_status(cudaMalloc(&b, bytes));
            if (st) return st;
            bufs.push_back(b);
            size_t off = 0;
            for (const Snap &s : state_arrays(hc)) {
                if ((st = cuda_status(cudaMemcpyAsync(b + off, s.p, s.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream)))) return st;
                off += s.n * sizeof(double);
            }
            if ((st = cuda_status(cudaMemcpyAsync(b + off, hc->dev.sc, sizeof(SolveScalars), cudaMemcpyDeviceToDevice, ctx->stream)))) return st;
        }
        return cuda_status(cudaStreamSynchronize(ctx->stream));
    }

    int restore(cfdl_ctx *ctx) {
        for (size_t c = 0; c < ctx->cases.size(); c++) {
            HostCase *hc = ctx->cases[c];
            size_t off = 0;
            int st;
            for (const Snap &s : state_arrays(hc)) {
                if ((st = cuda_status(cudaMemcpyAsync(s.p, bufs[c] + off, s.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream)))) return st;
                off += s.n * sizeof(double);
            }
            if ((st = cuda_status(cudaMemcpyAsync(hc->dev.sc, bufs[c] + off, sizeof(SolveScalars), cudaMemcpyDeviceToDevice, ctx->stream)))) return st;
            hc->g32_stale = true;    // precision 3: the FP32 gradients follow the restored gu, gv, gw
        }
        return cuda_status(cudaStreamSynchronize(ctx->stream));
    }
};

bool valid_shape(int vec) {
    for (int v : kTileShapes) if (v == vec) return true;
    return false;
}

}  // namespace

extern "C" {

int cfdl_set_tile(cfdl_ctx *ctx, int vec) {
    if (!ctx || ctx->cases.empty() || !valid_shape(vec)) return CFDL_ERR_INVALID;
    if (vec == ctx->vec) return CFDL_OK;
    int st = cuda_status(cudaStreamSynchronize(ctx->stream));
    if (st) return st;
    ctx->vec = vec;
    return rebuild_worklists(ctx);
}

int cfdl_get_tile(const cfdl_ctx *ctx) { return ctx ? ctx->vec : -1; }

int cfdl_set_energy_tile(cfdl_ctx *ctx, int vec) {
    if (!ctx || ctx->cases.empty() || !valid_shape(vec)) return CFDL_ERR_INVALID;
    if (vec == ctx->en_vec) return CFDL_OK;
    int st = cuda_status(cudaStreamSynchronize(ctx->stream));
    if (st) return st;
    ctx->en_vec = vec;
    return rebuild_worklists(ctx);
}

int cfdl_get_energy_tile(const cfdl_ctx *ctx) { return ctx ? ctx->en_vec : -1; }

int cfdl_set_coarse_group(cfdl_ctx *ctx, int lanes) {
    if (!ctx || ctx->cases.empty() || !(lanes == 1 || lanes == 2 || lanes == 4)) return CFDL_ERR_INVALID;
    if (lanes == ctx->cgroup) return CFDL_OK;
    int st = cuda_status(cudaStreamSynchronize(ctx->stream));
    if (st) return st;
    ctx->cgroup = lanes;
    ctx->amg_lmax = -1;      // multigrid work lists are rebuilt on the next solve
    destroy_graph(ctx);
    return CFDL_OK;
}

int cfdl_get_coarse_group(const cfdl_ctx *ctx) { return ctx ? ctx->cgroup : -1; }

// Times `outer` outer iterations from the snapshot; returns ms per iteration.
static int time_outer(cfdl_ctx *ctx, Snapshot &snap, int outer, cudaEvent_t e0, cudaEvent_t e1, double *ms) {
    int st;
    // warm-up: builds this shape's multigrid lists and graph
    if ((st = solve_uvwp_all(ctx)) || (st = snap.restore(ctx))) return st;
    cudaEventRecord(e0, ctx->stream);
    for (int i = 0; i < outer; i++) {
        launch_bc(ctx);
        if ((st = solve_uvwp_all(ctx))) return st;
    }
    cudaEventRecord(e1, ctx->stream);
    float f = 0.f;
    if ((st = cuda_status(cudaEventSynchronize(e1)))) return st;
    if ((st = cuda_status(cudaEventElapsedTime(&f, e0, e1)))) return st;
    *ms = f / outer;
    return snap.restore(ctx);
}

// Times `outer` energy solves from the snapshot; ms per solve.
static int time_energy(cfdl_ctx *ctx, Snapshot &snap, int outer, cudaEvent_t e0, cudaEvent_t e1, double *ms) {
    int st;
    if ((st = solve_energy_all(ctx)) || (st = snap.restore(ctx))) return st;
    cudaEventRecord(e0, ctx->stream);
    for (int i = 0; i < outer; i++)
        if ((st = solve_energy_all(ctx))) return st;
    cudaEventRecord(e1, ctx->stream);
    float f = 0.f;
    if ((st = cuda_status(cudaEventSynchronize(e1)))) return st;
    if ((st = cuda_status(cudaEventElapsedTime(&f, e0, e1)))) return st;
    *ms = f / outer;
    return snap.restore(ctx);
}

int cfdl_autotune(cfdl_ctx *ctx, int outer, int *best, double *ms) {
    if (!ctx || ctx->cases.empty() || outer <= 0) return CFDL_ERR_INVALID;
    Snapshot snap;
    int st = snap.take(ctx);
    if (st) return st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if ((st = cuda_status(cudaEventCreate(&e0)))) return st;
    if ((st = cuda_status(cudaEventCreate(&e1)))) { cudaEventDestroy(e0); return st; }
    // the solver tile shape first, then the lanes per row of the large coarse
    // multigrid levels at that shape
    const int n = (int)(sizeof(kTileShapes) / sizeof(kTileShapes[0]));
    int pick = ctx->vec;
    double best_ms = -1.0;
    for (int k = 0; k < n && !st; k++) {
        const int v = kTileShapes[k];
        double t = 0.0;
        if ((st = cfdl_set_tile(ctx, v)) || (st = time_outer(ctx, snap, outer, e0, e1, &t))) break;
        if (ms) ms[k] = t;
        if (best_ms < 0.0 || t < best_ms) { best_ms = t; pick = v; }
    }
    if (!st) st = cfdl_set_tile(ctx, pick);
    int gpick = ctx->cgroup;
    const int groups[] = {1, 2, 4};
    double gbest = -1.0;
    for (int k = 0; k < 3 && !st; k++) {
        double t = 0.0;
        if ((st = cfdl_set_coarse_group(ctx, groups[k])) || (st = time_outer(ctx, snap, outer, e0, e1, &t))) break;
        if (gbest < 0.0 || t < gbest) { gbest = t; gpick = groups[k]; }
    }
    if (!st) st = cfdl_set_coarse_group(ctx, gpick);
    // with the energy equation, the tile shape of its solve
    if (!st && energy_on(ctx)) {
        int epick = ctx->en_vec;
        double ebest = -1.0;
        for (int k = 0; k < n && !st; k++) {
            double t = 0.0;
            if ((st = cfdl_set_energy_tile(ctx, kTileShapes[k])) || (st = time_energy(ctx, snap, outer, e0, e1, &t))) break;
            if (ebest < 0.0 || t < ebest) { ebest = t; epick = kTileShapes[k]; }
        }
        if (!st) st = cfdl_set_energy_tile(ctx, epick);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    if (best) *best = pick;
    return snap.restore(ctx);
}

}  // extern "C"
