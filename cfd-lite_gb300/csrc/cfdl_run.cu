// cfdl_run.cu -- runs of many SIMPLE outer iterations for every case of a
// context, the reference's time loop (mod_physics.f90:23-36: update_boundaries,
// solve_uvwp, update_time every ncoef iterations) with per-case targets.
//
// Each case carries, in its device scalars, the outer iterations it has left,
// its update_time cadence and an optional convergence tolerance on the mass
// imbalance ratio ||b||_2 / sum_f |mip_f| (b = the pressure-correction source
// of calc_coef_p, the continuity error of the predicted fluxes).  At the top
// of each pass k_run_begin marks the cases with nothing left as halted, and
// every kernel of the outer iteration returns at once for a halted case, so a
// case's arithmetic is the same whichever other cases share the launch.  The
// graph form (cfdl_graph.cu) is one while node over all of this; the eager
// form below is the same sequence with a host check per pass.
#include "cfdl_device.cuh"

namespace cfdl {
namespace {

enum { CNT_RUN = 0 };

__global__ void k_run_begin(const CaseDev *__restrict__ cases, int ncases) {
    CFDL_PDL_WAIT();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncases) return;
    SolveScalars *S = cases[c].sc;
    const int h = S->run_left <= 0;
    S->halted = h;
    S->time_due = 0;
    if (h) {
        S->active[0] = S->active[1] = S->active[2] = 0;
        S->active_p = 0;
        S->active32 = 0;
        S->en.active[0] = 0;
    }
}

// sum |mip| over the case's faces, then the per-case bookkeeping of the pass
__global__ void __launch_bounds__(kTile) k_run_end(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                   const int *__restrict__ cfirst, const int *__restrict__ cnt,
                                                   double *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (S->halted) return;
    // several faces per thread (wide tiles), then one block tree: the FP64
    // reduction tree is paid once per kTile*kFaceVec faces
    double v[1] = {0.0};
    FOR_CELLS(t) v[0] += fabs(C.mip[i]);
    block_reduce<1>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_RUN], cnt[t.c])) {
        __shared__ double s[1];
        sum_partials<1>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            S->mip_abs = s[0];
            S->mass_ratio = s[0] > 0.0 ? S->mass_imbalance / s[0] : S->mass_imbalance;
            S->outer_done += 1;
            S->run_left -= 1;
            S->time_due = S->ncoef > 0 && S->outer_done % S->ncoef == 0;
            if (S->conv_tol > 0.0 && S->mass_imbalance <= S->conv_tol * s[0]) { S->converged = 1; S->run_left = 0; }
            const int bad = S->status[0] | S->status[1] | S->status[2] | S->status_p;
            if (bad == CFDL_ERR_NONFINITE || !isfinite(S->mass_imbalance)) S->run_left = 0;
        }
    }
}

// update_time (mod_uvwp.f90:74-93) for the cases whose cadence is due
__global__ void __launch_bounds__(kTile) k_run_time_cells(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    if (C.sc->halted || !C.sc->time_due) return;
    const int i = t.first + (int)threadIdx.x;
    if (i < t.last) { C.u0[i] = C.u[i]; C.v0[i] = C.v[i]; C.w0[i] = C.w[i]; }
}
__global__ void __launch_bounds__(kTile) k_run_time_halos(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    if (C.sc->halted || !C.sc->time_due) return;
    const int i = t.first + (int)threadIdx.x;
    if (i < t.last) { const int h = C.ne + i; C.u0[h] = C.u[h]; C.v0[h] = C.v[h]; C.w0[h] = C.w[h]; }
}
__global__ void __launch_bounds__(kTile) k_run_time_faces(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    if (C.sc->halted || !C.sc->time_due) return;
    const int i = t.first + (int)threadIdx.x;
    if (i < t.last) C.mip0[i] = C.mip[i];
}

// Run-loop condition: a case has iterations left and the launch's pass
// budget (ctl[0]) is not spent.  consume = 1 at the end of a pass.
// (one warp; lane l counts cases l, l+32, ...)
__device__ __forceinline__ int count_running(const CaseDev *__restrict__ cases, int ncases) {
    int running = 0;
    for (int c = (int)threadIdx.x; c < ncases; c += 32) running += cases[c].sc->run_left > 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) running += __shfl_xor_sync(0xffffffffu, running, o);
    return running;
}

__global__ void k_run_cond(const CaseDev *__restrict__ cases, int ncases, cudaGraphConditionalHandle h, int consume,
                           int *ctl, unsigned long long *passes) {
    CFDL_PDL_WAIT();
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    const int running = count_running(cases, ncases);
    if (threadIdx.x != 0) return;
    if (consume) { ctl[0] -= 1; if (passes) *passes += 1; }
    ctl[1] = running;
    cudaGraphSetConditional(h, (running > 0 && ctl[0] > 0) ? 1u : 0u);
}

// eager form of the condition: the same count, no graph handle
__global__ void k_run_count(const CaseDev *__restrict__ cases, int ncases, int *ctl) {
    CFDL_PDL_WAIT();
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    const int running = count_running(cases, ncases);
    if (threadIdx.x == 0) ctl[1] = running;
}

__global__ void k_run_finish(const CaseDev *__restrict__ cases, int ncases) {
    CFDL_PDL_WAIT();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncases) return;
    cases[c].sc->halted = 0;
}

}  // namespace

void launch_run_begin(cfdl_ctx *ctx) {
    const int n = (int)ctx->cases.size();
    k_run_begin<<<(n + 127) / 128, 128, 0, ctx->stream>>>(ctx->d_cases, n);
    ctx->launches++;
}

void launch_run_end(cfdl_ctx *ctx) {
    CFDL_LAUNCH("k_run_end", k_run_end, facesv, ctx->facesv.d_case_first, ctx->facesv.d_case_ntiles, ctx->d_partials);
    CFDL_LAUNCH("k_run_time_cells", k_run_time_cells, cells);
    CFDL_LAUNCH("k_run_time_halos", k_run_time_halos, halos);
    CFDL_LAUNCH("k_run_time_faces", k_run_time_faces, faces);
    launch_energy_time(ctx, true);
}

void launch_run_cond(cfdl_ctx *ctx, cudaGraphConditionalHandle h, int consume, unsigned long long *passes) {
    k_run_cond<<<1, 32, 0, ctx->stream>>>(ctx->d_cases, (int)ctx->cases.size(), h, consume, ctx->d_run_ctl, passes);
    ctx->launches++;
}

void launch_run_finish(cfdl_ctx *ctx) {
    const int n = (int)ctx->cases.size();
    k_run_finish<<<(n + 127) / 128, 128, 0, ctx->stream>>>(ctx->d_cases, n);
    ctx->launches++;
}

static int ensure_ctl(cfdl_ctx *ctx) {
    if (ctx->d_run_ctl) return CFDL_OK;
    int st = cuda_status(cudaMalloc(&ctx->d_run_ctl, 2 * sizeof(int)));
    if (!st) st = cuda_status(cudaMallocHost(&ctx->h_run_ctl, 2 * sizeof(int)));
    return st;
}

// Up to max_outer passes of the run loop; *running = cases with iterations
// left afterwards.
int run_outer(cfdl_ctx *ctx, int max_outer, int *running) {
    int st;
    if ((st = ensure_ctl(ctx))) return st;
    ctx->h_run_ctl[0] = max_outer;
    ctx->h_run_ctl[1] = 0;
    if ((st = cuda_status(cudaMemcpyAsync(ctx->d_run_ctl, ctx->h_run_ctl, 2 * sizeof(int), cudaMemcpyHostToDevice,
                                          ctx->stream))))
        return st;
    const int n = (int)ctx->cases.size();
    if (ctx->use_graph && !prof_active(ctx)) {
        if ((st = run_graph_launch(ctx))) return st;
    } else {
        for (int k = 0; k < max_outer; k++) {
            k_run_count<<<1, 32, 0, ctx->stream>>>(ctx->d_cases, n, ctx->d_run_ctl);
            ctx->launches++;
            if ((st = cuda_status(cudaMemcpyAsync(ctx->h_run_ctl + 1, ctx->d_run_ctl + 1, sizeof(int),
                                                  cudaMemcpyDeviceToHost, ctx->stream))))
                return st;
            if ((st = cuda_status(cudaStreamSynchronize(ctx->stream)))) return st;
            if (ctx->h_run_ctl[1] == 0) break;
            launch_run_begin(ctx);
            launch_bc(ctx);
            if ((st = solve_uvwp_all(ctx))) return st;
            if ((st = solve_energy_all(ctx))) return st;
            launch_run_end(ctx);
        }
        k_run_count<<<1, 32, 0, ctx->stream>>>(ctx->d_cases, n, ctx->d_run_ctl);
        ctx->launches++;
        launch_run_finish(ctx);
    }
    if ((st = cuda_status(cudaMemcpyAsync(ctx->h_run_ctl + 1, ctx->d_run_ctl + 1, sizeof(int), cudaMemcpyDeviceToHost,
                                          ctx->stream))))
        return st;
    if ((st = cuda_status(cudaStreamSynchronize(ctx->stream)))) return st;
    if (running) *running = ctx->h_run_ctl[1];
    return CFDL_OK;
}

}  // namespace cfdl
