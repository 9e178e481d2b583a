// cfdl_graph.cu -- one outer iteration (solve_uvwp) as one CUDA graph.
//
// The inner solves of solve_uvwp loop until a residual test passes
// (solve_gs / multi_subdomain_solver in the reference,
// src/modules/mod_solver.f90:124-327).  Here each such loop is a graph
// "while" node whose body is one Krylov iteration followed by a one-thread
// kernel that sets the loop condition from the per-case activity flags the
// iteration's reductions left on the device.  The whole outer iteration --
// momentum assembly, three-component BiCGStab loop, gradients, Rhie-Chow
// fluxes, pressure assembly, pressure-correction loop (nested loops for the
// mixed-precision form), correction -- is then a single cudaGraphLaunch with
// no host round trip.  The graph is built once per context and kernel
// sequence; coefficients, tolerances and fields are read from device memory
// at run time, so changing them does not rebuild it.
#include "cfdl_internal.h"
#include <cuda_runtime.h>

namespace cfdl {

void mom_init(cfdl_ctx *ctx);
void mom_iter(cfdl_ctx *ctx);
void mom_finish(cfdl_ctx *ctx);
void pcj_init(cfdl_ctx *ctx);
void pcj_iter(cfdl_ctx *ctx);
void apc_init(cfdl_ctx *ctx);
void apc_iter(cfdl_ctx *ctx);
void mx_init(cfdl_ctx *ctx);
void mx_start(cfdl_ctx *ctx);
void mx_inner_iter(cfdl_ctx *ctx);
void mx_finish(cfdl_ctx *ctx);

namespace {

enum { LOOP_MOM = 0, LOOP_P = 1, LOOP_INNER = 2, LOOP_OUTER = 3, LOOP_EN = 4 };

// Loop condition = any case still active for this loop kind; counts the pass.
// One warp: lane l reads cases l, l+32, ... and the warp votes.
__global__ void k_setcond(const CaseDev *__restrict__ cases, int ncases, cudaGraphConditionalHandle h, int kind,
                          unsigned long long *loop_passes) {
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    int any = 0;
    for (int c = (int)threadIdx.x; c < ncases; c += 32) {
        const SolveScalars *S = cases[c].sc;
        int a;
        if (kind == LOOP_MOM) a = S->active[0] | S->active[1] | S->active[2];
        else if (kind == LOOP_INNER) a = S->active32;
        else if (kind == LOOP_EN) a = S->en.active[0];
        else a = S->active_p;
        any |= (a != 0);
    }
    any = __any_sync(0xffffffffu, any);
    if (threadIdx.x == 0) {
        cudaGraphSetConditional(h, any ? 1u : 0u);
        loop_passes[kind == LOOP_EN ? 5 : kind] += 1;   // the run graph's energy slot is base + 5
    }
}

__global__ void k_setone(cudaGraphConditionalHandle h) {
    if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(h, 1u);
}

struct Builder {
    cfdl_ctx *ctx;
    unsigned long long *passes;   // this graph's loop-pass counters

    void setcond(cudaGraphConditionalHandle h, int kind) {
        k_setcond<<<1, 32, 0, ctx->stream>>>(ctx->d_cases, (int)ctx->cases.size(), h, kind, passes);
        ctx->launches++;
    }
    void setone(cudaGraphConditionalHandle h) {
        k_setone<<<1, 32, 0, ctx->stream>>>(h);
        ctx->launches++;
    }
    template <class F> int capture(F f, cudaGraph_t *out, int64_t *count) {
        const int64_t l0 = ctx->launches;
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_status(e);
        f();
        e = cudaStreamEndCapture(ctx->stream, out);
        *count = ctx->launches - l0;
        ctx->launches = l0;
        return cuda_status(e);
    }
    template <class F> int capture_into(cudaGraph_t body, F f, int64_t *count) {
        const int64_t l0 = ctx->launches;
        cudaError_t e = cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_status(e);
        f();
        cudaGraph_t out = nullptr;
        e = cudaStreamEndCapture(ctx->stream, &out);
        *count = ctx->launches - l0;
        ctx->launches = l0;
        return cuda_status(e);
    }
    // append a captured segment as a child-graph node after *prev
    template <class F> int segment(cudaGraph_t G, cudaGraphNode_t *prev, F f, int64_t *count) {
        cudaGraphNode_t dep[1] = {*prev};
        return segment_after(G, dep, *prev ? 1 : 0, f, count, prev);
    }
    // a captured segment as a child-graph node depending on deps[0..ndep)
    template <class F>
    int segment_after(cudaGraph_t G, const cudaGraphNode_t *deps, int ndep, F f, int64_t *count, cudaGraphNode_t *out) {
        cudaGraph_t child = nullptr;
        int st = capture(f, &child, count);
        if (st) return st;
        cudaGraphNode_t n;
        cudaError_t e = cudaGraphAddChildGraphNode(&n, G, ndep ? deps : nullptr, ndep, child);
        cudaGraphDestroy(child);
        if (e != cudaSuccess) return cuda_status(e);
        *out = n;
        return CFDL_OK;
    }
    // append a while node; fill(body) builds its body graph
    template <class F> int loop(cudaGraph_t G, cudaGraphNode_t *prev, cudaGraphConditionalHandle h, F fill) {
        cudaGraphNodeParams p = {};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t n;
        cudaError_t e = cudaGraphAddNode(&n, G, *prev ? prev : nullptr, nullptr, *prev ? 1 : 0, &p);
        if (e != cudaSuccess) return cuda_status(e);
        int st = fill(p.conditional.phGraph_out[0]);
        if (st) return st;
        *prev = n;
        return CFDL_OK;
    }
};

}  // namespace

static void drop_uvwp_graph(cfdl_ctx *ctx) {
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->graph) cudaGraphDestroy(ctx->graph);
    ctx->graph_exec = nullptr;
    ctx->graph = nullptr;
    ctx->graph_form = -1;
}

static void drop_run_graph(cfdl_ctx *ctx) {
    if (ctx->run_exec) cudaGraphExecDestroy(ctx->run_exec);
    if (ctx->run_graph) cudaGraphDestroy(ctx->run_graph);
    ctx->run_exec = nullptr;
    ctx->run_graph = nullptr;
    ctx->run_form = -1;
}

static void drop_energy_graph(cfdl_ctx *ctx) {
    if (ctx->energy_exec) cudaGraphExecDestroy(ctx->energy_exec);
    if (ctx->energy_graph) cudaGraphDestroy(ctx->energy_graph);
    ctx->energy_exec = nullptr;
    ctx->energy_graph = nullptr;
    ctx->energy_form = -1;
}

void destroy_graph(cfdl_ctx *ctx) {
    drop_uvwp_graph(ctx);
    drop_run_graph(ctx);
    drop_energy_graph(ctx);
}

static int graph_form(const cfdl_ctx *ctx) {
    const cfdl_config &c = ctx->cases[0]->cfg;
    return c.precision * 2 + c.precond + (energy_on(ctx) ? 8 : 0);
}

static int ensure_graph_state(cfdl_ctx *ctx) {
    int st;
    if (ctx->cases[0]->cfg.precond == 1 && (st = ensure_amg(ctx))) return st;
    if (!ctx->d_loop_passes) {
        const size_t bytes = kLoopSlots * sizeof(unsigned long long);
        if ((st = cuda_status(cudaMalloc(&ctx->d_loop_passes, bytes)))) return st;
        if ((st = cuda_status(cudaMemset(ctx->d_loop_passes, 0, bytes)))) return st;
    }
    return CFDL_OK;
}

// Appends the nodes of one solve_uvwp to G after *prev.  pre() is captured at
// the head of the first segment, post() at the tail of the last.  Loop
// handles are created in G and raised by a kernel before each loop, so the
// same nodes work at the top level and inside the body of an outer loop.
// static_k gets the kernels outside the loops, body[0..3] those of each
// loop's body.
template <class Pre, class Post>
static int append_uvwp(Builder &b, cudaGraph_t G, cudaGraphNode_t *prev, Pre pre, Post post, int64_t *static_k,
                       int64_t *body, bool mark) {
    cfdl_ctx *ctx = b.ctx;
    const cfdl_config &cfg = ctx->cases[0]->cfg;
    int st;
    int64_t k = 0;
    cudaGraphConditionalHandle hm, hp;
    if ((st = cuda_status(cudaGraphConditionalHandleCreate(&hm, G, 0, 0)))) return st;
    if ((st = cuda_status(cudaGraphConditionalHandleCreate(&hp, G, 0, 0)))) return st;
    // momentum assembly and BiCGStab
    if ((st = b.segment(G, prev, [&] {
             pre();
             launch_coef_uvw(ctx);
             mom_init(ctx);
             b.setone(hm);
         }, &k)))
        return st;
    *static_k += k;
    // beside the momentum solve: the pressure matrix (it needs only dc of
    // calc_coef_uvw) and the pressure solve's operators, in their own storage
    cudaGraphNode_t branch = nullptr;
    {
        const cudaGraphNode_t dep[1] = {*prev};
        if ((st = b.segment_after(G, dep, 1, [&] {
                 launch_coef_p_matrix(ctx);
                 pressure_operators(ctx);
             }, &k, &branch)))
            return st;
        *static_k += k;
        if (!ctx->graph_branches) *prev = branch;   // one chain: the momentum solve after it
    }
    st = b.loop(G, prev, hm, [&](cudaGraph_t body_g) {
        return b.capture_into(body_g, [&] { mom_iter(ctx); b.setcond(hm, LOOP_MOM); }, &body[LOOP_MOM]);
    });
    if (st) return st;
    // the FP32 correction of precision >= 2 completes u, v, w
    if (cfg.precision >= 2) {
        if ((st = b.segment(G, prev, [&] { mom_finish(ctx); }, &k))) return st;
        *static_k += k;
    }
    // the gradients of u, v, w are read only by the next outer iteration's
    // face terms, so they run beside the whole pressure part
    cudaGraphNode_t gradn = nullptr;
    {
        const cudaGraphNode_t dep[1] = {*prev};
        if ((st = b.segment_after(G, dep, 1, [&] { launch_grad(ctx, 4); }, &k, &gradn))) return st;
        *static_k += k;
        if (!ctx->graph_branches) *prev = gradn;
    }
    if (ctx->ev_mom && mark) {
        // u, v, w and their gradients are final here (cfdl_solve_uvwp_host
        // starts their download on this record)
        cudaGraphNode_t n;
        cudaError_t e = cudaGraphAddEventRecordNode(&n, G, &gradn, 1, ctx->ev_mom);
        if (e != cudaSuccess) return cuda_status(e);
    }
    // Rhie-Chow fluxes, the pressure right-hand side, the pressure-solve start
    {
        const cudaGraphNode_t deps[2] = {*prev, branch};
        if ((st = b.segment_after(G, deps, 2, [&] {
                 launch_calc_mip(ctx, 1);
                 launch_coef_p_rhs(ctx);
                 if (cfg.precision >= 1) mx_init(ctx);
                 else if (cfg.precond == 1) apc_init(ctx);
                 else pcj_init(ctx);
                 b.setone(hp);
             }, &k, prev)))
            return st;
        *static_k += k;
    }
    if (cfg.precision == 0) {
        st = b.loop(G, prev, hp, [&](cudaGraph_t body_g) {
            return b.capture_into(body_g, [&] {
                if (cfg.precond == 1) apc_iter(ctx);
                else pcj_iter(ctx);
                b.setcond(hp, LOOP_P);
            }, &body[LOOP_P]);
        });
    } else {
        // refinement loop around the FP32 inner loop
        st = b.loop(G, prev, hp, [&](cudaGraph_t outer) {
            cudaGraphConditionalHandle hi;
            int s2 = cuda_status(cudaGraphConditionalHandleCreate(&hi, outer, 0, 0));
            if (s2) return s2;
            cudaGraphNode_t op = nullptr;
            int64_t k1 = 0, k2 = 0;
            if ((s2 = b.segment(outer, &op, [&] { mx_start(ctx); b.setone(hi); }, &k1))) return s2;
            if ((s2 = b.loop(outer, &op, hi, [&](cudaGraph_t inner) {
                     return b.capture_into(inner, [&] { mx_inner_iter(ctx); b.setcond(hi, LOOP_INNER); }, &body[LOOP_INNER]);
                 })))
                return s2;
            if ((s2 = b.segment(outer, &op, [&] { mx_finish(ctx); b.setcond(hp, LOOP_OUTER); }, &k2))) return s2;
            body[LOOP_OUTER] = k1 + k2;
            return CFDL_OK;
        });
    }
    if (st) return st;
    // correction
    if ((st = b.segment(G, prev, [&] {
             launch_adjust_pc(ctx);
             launch_grad(ctx, 3);
             launch_update_uvwp(ctx);
             post();
         }, &k)))
        return st;
    *static_k += k;
    return CFDL_OK;
}

int build_graph(cfdl_ctx *ctx) {
    drop_uvwp_graph(ctx);
    int st;
    if ((st = ensure_graph_state(ctx))) return st;
    cudaGraph_t G = nullptr;
    if ((st = cuda_status(cudaGraphCreate(&G, 0)))) return st;
    Builder b{ctx, ctx->d_loop_passes};
    ctx->capturing = true;
    cudaGraphNode_t prev = nullptr;
    int64_t stat = 0, body[4] = {0, 0, 0, 0};
    st = append_uvwp(b, G, &prev, [] {}, [] {}, &stat, body, true);
    ctx->capturing = false;
    if (st) { cudaGraphDestroy(G); return st; }
    cudaGraphExec_t exec = nullptr;
    if ((st = cuda_status(cudaGraphInstantiate(&exec, G, 0)))) { cudaGraphDestroy(G); return st; }
    ctx->graph = G;
    ctx->graph_exec = exec;
    ctx->graph_form = graph_form(ctx);
    ctx->graph_static_kernels = stat;
    for (int i = 0; i < 4; i++) ctx->graph_body_kernels[i] = body[i];
    return CFDL_OK;
}

// solve_energy (mod_energy.f90:59-80) after *prev: gradients and assembly,
// the BiCGStab loop on the energy lane, calc_temperature, then post().
template <class Post>
static int append_energy(Builder &b, cudaGraph_t G, cudaGraphNode_t *prev, Post post, int64_t *static_k,
                         int64_t *body) {
    cfdl_ctx *ctx = b.ctx;
    int st;
    int64_t k = 0;
    cudaGraphConditionalHandle he;
    if ((st = cuda_status(cudaGraphConditionalHandleCreate(&he, G, 0, 0)))) return st;
    if ((st = b.segment(G, prev, [&] {
             launch_grad(ctx, 5);
             launch_coef_energy(ctx);
             energy_init_solve(ctx);
             b.setone(he);
         }, &k)))
        return st;
    *static_k += k;
    st = b.loop(G, prev, he, [&](cudaGraph_t body_g) {
        return b.capture_into(body_g, [&] { energy_iter(ctx); b.setcond(he, LOOP_EN); }, body);
    });
    if (st) return st;
    if ((st = b.segment(G, prev, [&] { energy_finish(ctx); launch_energy_temp(ctx); post(); }, &k))) return st;
    *static_k += k;
    return CFDL_OK;
}

// The run graph: while (a case has outer iterations left and the launch's
// budget is not spent) { per-case start; update_boundaries; solve_uvwp;
// solve_energy when set up; per-case end with the convergence test; gated
// update_time }.  Cases whose run is over are skipped by every kernel until
// the host gives them more.
int build_run_graph(cfdl_ctx *ctx) {
    drop_run_graph(ctx);
    int st;
    if ((st = ensure_graph_state(ctx))) return st;
    cudaGraph_t G = nullptr;
    if ((st = cuda_status(cudaGraphCreate(&G, 0)))) return st;
    Builder b{ctx, ctx->d_loop_passes + 4};
    ctx->capturing = true;
    cudaGraphNode_t prev = nullptr;
    int64_t stat = 0, k = 0, body[6] = {0, 0, 0, 0, 0, 0};
    cudaGraphConditionalHandle hr;
    auto fail = [&](int s) { ctx->capturing = false; cudaGraphDestroy(G); return s; };
    if ((st = cuda_status(cudaGraphConditionalHandleCreate(&hr, G, 0, 0)))) return fail(st);
    if ((st = b.segment(G, &prev, [&] { launch_run_cond(ctx, hr, 0, nullptr); }, &k))) return fail(st);
    stat += k;
    st = b.loop(G, &prev, hr, [&](cudaGraph_t outer) {
        cudaGraphNode_t op = nullptr;
        int64_t inner_static = 0;
        auto tail = [&] { launch_run_end(ctx); launch_run_cond(ctx, hr, 1, ctx->d_loop_passes + 8); };
        const bool energy = energy_on(ctx);
        int s2 = energy ? append_uvwp(b, outer, &op, [&] { launch_run_begin(ctx); launch_bc(ctx); }, [] {},
                                      &inner_static, body, false)
                        : append_uvwp(b, outer, &op, [&] { launch_run_begin(ctx); launch_bc(ctx); }, tail,
                                      &inner_static, body, false);
        if (!s2 && energy) s2 = append_energy(b, outer, &op, tail, &inner_static, &body[5]);
        body[4] = inner_static;
        return s2;
    });
    if (st) return fail(st);
    if ((st = b.segment(G, &prev, [&] { launch_run_finish(ctx); }, &k))) return fail(st);
    stat += k;
    ctx->capturing = false;
    cudaGraphExec_t exec = nullptr;
    if ((st = cuda_status(cudaGraphInstantiate(&exec, G, 0)))) { cudaGraphDestroy(G); return st; }
    ctx->run_graph = G;
    ctx->run_exec = exec;
    ctx->run_form = graph_form(ctx);
    ctx->run_static_kernels = stat;
    for (int i = 0; i < 6; i++) ctx->run_body_kernels[i] = body[i];
    return CFDL_OK;
}

// solve_energy alone as one graph: assembly, the BiCGStab loop on the device,
// calc_temperature (cfdl_solve_energy, cfdl_step)
static int build_energy_graph(cfdl_ctx *ctx) {
    drop_energy_graph(ctx);
    int st;
    if ((st = ensure_graph_state(ctx))) return st;
    cudaGraph_t G = nullptr;
    if ((st = cuda_status(cudaGraphCreate(&G, 0)))) return st;
    Builder b{ctx, ctx->d_loop_passes + 5};          // its loop counts in slot 10
    ctx->capturing = true;
    cudaGraphNode_t prev = nullptr;
    int64_t stat = 0, body = 0;
    st = append_energy(b, G, &prev, [] {}, &stat, &body);
    ctx->capturing = false;
    if (st) { cudaGraphDestroy(G); return st; }
    cudaGraphExec_t exec = nullptr;
    if ((st = cuda_status(cudaGraphInstantiate(&exec, G, 0)))) { cudaGraphDestroy(G); return st; }
    ctx->energy_graph = G;
    ctx->energy_exec = exec;
    ctx->energy_form = graph_form(ctx);
    ctx->energy_static_kernels = stat;
    ctx->energy_body_kernels = body;
    return CFDL_OK;
}

int solve_energy_graph(cfdl_ctx *ctx) {
    int st;
    ensure_energy_props(ctx);
    if (!ctx->energy_exec || ctx->energy_form != graph_form(ctx))
        if ((st = build_energy_graph(ctx))) return st;
    ctx->launches += ctx->energy_static_kernels;
    ctx->graph_launches++;
    return cuda_status(cudaGraphLaunch(ctx->energy_exec, ctx->stream));
}

int run_graph_launch(cfdl_ctx *ctx) {
    int st;
    ensure_face_props(ctx);
    ensure_g32(ctx);
    ensure_energy_props(ctx);
    if (!ctx->run_exec || ctx->run_form != graph_form(ctx))
        if ((st = build_run_graph(ctx))) return st;
    ctx->launches += ctx->run_static_kernels;
    ctx->graph_launches++;
    const bool pressure_last = !energy_on(ctx);
    for (HostCase *hc : ctx->cases) hc->coef_is_pressure = pressure_last;
    return cuda_status(cudaGraphLaunch(ctx->run_exec, ctx->stream));
}

// One solve_uvwp through the graph (built on first use, rebuilt when the
// kernel sequence changes).  Returns a status; falls back to nothing.
int solve_uvwp_graph(cfdl_ctx *ctx) {
    int st;
    ensure_face_props(ctx);
    ensure_g32(ctx);
    if (!ctx->graph_exec || ctx->graph_form != graph_form(ctx))
        if ((st = build_graph(ctx))) return st;
    ctx->launches += ctx->graph_static_kernels;
    ctx->graph_launches++;
    for (HostCase *hc : ctx->cases) hc->coef_is_pressure = true;
    return cuda_status(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
}

// Kernels the graph ran inside its loops so far (synchronises).
int64_t graph_loop_kernels(cfdl_ctx *ctx) {
    if (!ctx->d_loop_passes) return 0;
    unsigned long long passes[kLoopSlots] = {};
    if (cudaMemcpyAsync(passes, ctx->d_loop_passes, sizeof(passes), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return 0;
    int64_t n = 0;
    for (int i = 0; i < 4; i++) n += (int64_t)passes[i] * ctx->graph_body_kernels[i];
    for (int i = 0; i < 4; i++) n += (int64_t)passes[4 + i] * ctx->run_body_kernels[i];
    n += (int64_t)passes[8] * ctx->run_body_kernels[4];
    n += (int64_t)passes[9] * ctx->run_body_kernels[5];
    n += (int64_t)passes[10] * ctx->energy_body_kernels;
    return n;
}

}  // namespace cfdl
