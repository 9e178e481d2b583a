// cfdl_internal.h -- device data layout and launch plumbing of libcfdgpu.
//
// Layout in HBM (per case, all device pointers):
//   cells      0..ne-1 interior, ne..ne+nbf-1 halos (boundary faces): the
//              reference numbering shifted to 0-based;
//   half-faces ELL slots [W][ne] (W = max faces per cell, padding nb = -1),
//              slot k of cell e = local face k+1 of the reference CSR:
//              hf_nb = neighbour cell or halo, hf_fc = face id (owner side)
//              or ~face id (neighbour side), hf_G = least-squares gradient
//              stencil A^-1 * w * dr, planes [3][W][ne];
//   faces      reference face order fg-1: f_own, f_nb and precomputed
//              geometry planes fgeo[FG_*][nf];
//   halos      h_own (owner cell), h_face, h_kind, h_vel (wall velocity).
// Fields keep the reference layout (gradients xyz-interleaved) so uploads and
// downloads are plain copies.
//
// Every kernel walks a work list of tiles: tile = (case, first, last) over the
// cells, faces or halos of one case, one CTA per tile.  A single case is a list
// of one; the batched and served forms put many cases in one list, so one
// launch covers all of them.  Reductions write one partial per tile; the last
// tile of a case to finish sums that case's partials in tile order, so every
// result is deterministic run to run and needs no extra launch.
#pragma once
#include "cfdl.h"
#include <cuda_runtime.h>
#include "cfdl_par.h"
#include <cstdint>
#include <vector>

namespace cfdl {

constexpr int kTile = 256;        // cells / faces / halos per CTA
constexpr int kMaxW = 6;          // max faces per cell supported (HEXA_8)
constexpr short kNb16None = -32768; // CaseDev::nb16: the slot has no interior neighbour
constexpr int kNPart = 16;        // partial slots per tile
constexpr int kVec = 4;           // default cells per thread in the solver kernels
constexpr int kFaceVec = 8;       // faces per thread in the face reductions (their FP64 tree amortised)
constexpr int kMixedMaxOuter = 60;   // FP64 refinement cycles of the mixed pressure solve
// loop-pass counters: [0,4) loops of the solve_uvwp graph, [4,8) the same
// loops inside the run graph, [8] the run graph's outer loop, [9] its energy
// solve loop, [10] the loop of the solve_energy graph
constexpr int kLoopSlots = 11;

// Loop over the cells of a wide solver tile: thread t handles cells
// first+t, first+t+kTile, ... (coalesced); the tile's pad field holds how many
// cells each thread takes (the tile shape the autotuner chooses).
#define FOR_CELLS(t) \
    for (int j_ = 0, i = (t).first + (int)threadIdx.x; j_ < (t).pad; j_++, i += cfdl::kTile) if (i < (t).last)

// face geometry planes, precomputed once per mesh (cfdl_case.cpp)
enum FaceGeo {
    FG_WT = 0,              // vec_weight(rip, r_own, r_nb)
    FG_AX, FG_AY, FG_AZ,    // aip (area vector, outward from the owner)
    FG_AREA,                // |aip|
    FG_ADN,                 // area / (dr . n) (boundary faces: dr to the halo centre)
    FG_DRX, FG_DRY, FG_DRZ, // dr = r_nb - r_own
    FG_ADS,                 // area / ds
    FG_ADRX, FG_ADRY, FG_ADRZ,  // area * dr / ds
    FG_EX, FG_EY, FG_EZ,        // area * (dr_p/ds_p - dr/ds)
    FG_N
};

// energy property planes eprop[EP_*][nf], recomputed only when cp or tc change
enum EnergyProp {
    EP_D = 0,                   // tc_ip/cp_ip * area/(dr.n) (boundary faces: tc/cp of the owner * area/(dr.n))
    EP_TC,                      // tc_ip
    EP_TCR,                     // tc_ip/cp_ip
    EP_N
};

// property planes fprop[PR_*][nf]: the mesh planes scaled by the interpolated
// density and viscosity, recomputed only when rho or mu change
enum FaceProp {
    PR_FDIFF = 0,               // mu_ip * area/ds (boundary faces: mu_own * area/ds)
    PR_MAX, PR_MAY, PR_MAZ,     // mu_ip * area * dr/ds
    PR_MEX, PR_MEY, PR_MEZ,     // mu_ip * area * (dr_p/ds_p - dr/ds)
    PR_RHO,                     // rho_ip
    PR_RHOADN,                  // rho_ip * area/(dr.n)
    PR_RHOMADN,                 // (rho_own + rho_nb)/2 * area/(dr.n)  (update_uvwp's face density)
    PR_N
};

struct AmgLevelDev;
struct AmgHierarchy;

// BiCGStab scalars, one lane per right-hand side
struct KLanes {
    double rho[3], alpha[3], omega[3], beta[3];
    int half[3];
    double rnorm[3], r0norm[3], bnorm[3], tol[3];
    int active[3], iters[3], status[3];
};

// Per-case solver state on the device.  The base lanes are the momentum
// solve's (u, v, w); en lane 0 is the energy solve's.
struct SolveScalars : KLanes {
    KLanes en;
    // pressure CG
    double rz, rnorm_p, r0norm_p, tol_p, alpha_p, beta_p, mean_b, pref;
    int active_p, iters_p, status_p;
    // mixed-precision refinement
    double res64, res64_0, tol64;
    int outer_p;
    float rz32, tol32, alpha32, beta32, rnorm32;
    int active32, iters32;
    double mass_imbalance;
    // outer-iteration runs (cfdl_run.cu): per-case targets and progress
    int run_left, outer_done, ncoef, halted, time_due, converged;
    double conv_tol, mip_abs, mass_ratio;
};

struct CaseDev {
    int ne, nbf, nf, W;
    // mesh
    const int *hf_nb, *hf_fc;
    const double *hf_G;
    const int *f_own, *f_nb;
    const double *fgeo;
    const int *h_own, *h_face, *h_kind;
    const double *h_vel;
    const double *vol;
    // fields (reference layout)
    double *u, *v, *w, *p, *u0, *v0, *w0;
    double *gu, *gv, *gw, *gp, *gpc;
    double *mip, *mip0;
    double *bu, *bv, *bw, *d, *dc, *rho, *mu;
    double *ap, *anb, *b, *phic;          // phys_t scratch: ap[ne], anb ELL [W][ne], b[ne], phic[ne+nbf]
    // the pressure-correction matrix in its own storage (the reference shares
    // ap/anb): it depends only on dc, so it and the multigrid set-up are built
    // beside the momentum solve; its 1/ap scaling and FP32 copies likewise
    double *ap_p, *anb_p, *rap_p;
    float *fdiag_p, *fanb_p, *frap_p;
    // face intermediates of the assemblies
    double *fdiff, *fS;                   // [nf] pressure face coefficient, [3][nf] explicit momentum face terms
    double *hbc;                          // [4][nbf] per halo: the wall diffusion added to ap and anb, and the
                                          // three momentum sources of the BC loop (k_coef_uvw_halo)
    double *fprop;                        // [PR_N][nf] property planes
    // precision 3 (FP32 explicit momentum face terms); null otherwise:
    float *g32;                           // [3][ne][3] FP32 gradients of u, v, w
    float *G32;                           // [3][W][ne] FP32 copy of the gradient stencil hf_G
    float *fprop32;                       // [11][nf] FP32 weight, mu*area*dr/ds, mu*area*(dr_p/ds_p - dr/ds),
                                          // dr, rho_ip*area/(dr.n) (the Rhie-Chow term's planes)
    float *gp32;                          // [ne][3] FP32 copy of gp, and d32 [ne] of d (the FP32 Rhie-Chow term)
    float *d32;
    // Krylov work vectors, [3][ne] each (pressure uses plane 0)
    double *kr, *krh, *kp, *kph, *kv, *ks, *ksh, *kt;
    // FP32 work vectors for the mixed-precision pressure solve, [ne] each
    float *fr, *fz, *fp, *fq, *fx, *fdiag, *fanb;   // fanb ELL [W][ne]
    float *ft, *frap;
    // 1/ap of the operator being solved (momentum, then pressure), AMG levels, coarsest inverse
    double *rap;
    int nlev, ncoarse;                    // coarse levels; cells of the coarsest level
    int amg_tail;                         // first level the one-CTA V-cycle tail runs (k_v_tail)
    const AmgLevelDev *lev;               // [nlev] device array
    // [W][ne] the mesh level's interior neighbours as 16-bit offsets j - i
    // (kNb16None: no interior neighbour) for the mixed pressure solve's FP32
    // mesh-level kernels; null when an offset does not fit, or in FP64
    const short *nb16;
    double *cinv;                         // [ncoarse^2] dense inverse of the coarsest operator
    float *cinv32;
    SolveScalars *sc;
    int *counters;                        // [16] last-tile counters, zero between launches
    // energy equation (null until cfdl_energy_init): t, phi = cp*t, phi0
    // [ne+nbf]; their gradients [3(ne+nbf)]; cp, tc [ne]; wall temperature
    // of each halo [nbf]
    double *et, *ee, *ee0, *egt, *ege, *ecp, *etc;
    const double *eh_t;
    double *eprop;                        // [EP_N][nf] energy property planes
    // parameters
    double dt, alpha_u, alpha_p, rtol_u, rtol_p, tight_rtol;
    double rdt, ralpha_u;                 // 1/dt (0 when steady), 1/alpha_u
    int nit, solve_mode, tight_maxit, precision, precond;
    int steady;                           // dt = INFINITY: the transient terms vanish
};

// A tile of a work list: case c, entities [first, last); pad = entities per
// thread (1 for the kTile-entity lists, the solver tile shape for cellsv).
struct Tile { int c, first, last, pad; };

// One work list per entity type, with each case's tile range for reductions.
struct WorkList {
    int ntiles = 0;
    Tile *d_tiles = nullptr;
    int *d_case_first = nullptr, *d_case_ntiles = nullptr;
    std::vector<Tile> h_tiles;
    std::vector<int> case_first, case_ntiles;
};

// Host-side record of one case.
struct HostCase {
    int ne = 0, nf = 0, nbf = 0, W = 0, H = 0;
    cfdl_config cfg{};
    std::vector<int> ef2nb_idx;      // [ne+1], 1-based values
    std::vector<void *> allocs;      // device allocations owned by the case
    CaseDev dev{};                   // host mirror of the device struct
    AmgHierarchy *amg = nullptr;     // host hierarchy, built on first AMG use
    std::vector<void *> amg_allocs;  // device allocations of the hierarchy
    int id = 0;                      // stable case id within its context
    bool props_dirty = true;         // fprop must be recomputed (rho or mu changed)
    size_t bytes = 0;                // device bytes held (mesh, fields, solver, hierarchy)
    std::vector<double> h_temp;      // [nbf] energy wall temperature of each halo (empty: none)
    bool eprops_dirty = true;        // eprop must be recomputed (cp or tc changed)
    bool g32_stale = false;          // g32 must be rebuilt from gu, gv, gw (they were written from outside)
    bool coef_is_pressure = false;   // ap/anb as the reference's phys_t holds them: the pressure matrix last
};

}  // namespace cfdl

// A context: one or more cases resident on one device, one stream.
struct cfdl_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // host drop-in (cfdl_solve_uvwp_host): a copy stream that downloads the
    // momentum results while the pressure half of the iteration runs
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_mom = nullptr;        // recorded after the momentum solve and calc_grad(u,v,w)
    cudaEvent_t ev_copy = nullptr;
    std::vector<cfdl::HostCase *> cases;
    int next_id = 0;                     // id given to the next added case
    cfdl::CaseDev *d_cases = nullptr;
    int d_cases_cap = 0;
    cfdl::WorkList cells, faces, halos;
    cfdl::WorkList cellsv;               // wide tiles (kTile*vec cells) for the solver kernels
    int vec = cfdl::kVec;                // cells per thread in those tiles (autotuned)
    cfdl::WorkList cellse;               // tiles of the energy solve (kTile*en_vec cells)
    cfdl::WorkList facesv;               // wide face tiles (kTile*kFaceVec faces) for face reductions
    int en_vec = 1;                      // cells per thread in those tiles (autotuned with the energy equation)
    int last_iters_m = 0, last_iters_p = 0, last_iters_e = 0;   // previous inner iteration counts (poll scheduling)
    double *d_partials = nullptr;        // [max tiles][kNPart]
    int partials_cap = 0;                // tiles
    int64_t launches = 0;
    int64_t host_writes = 0;             // host-to-device copies into the fields (uploads, set_array)
    // the host drop-in's last download (cfdl_step_host*): the host array each
    // field went to, and the launch and write counters at that moment; a
    // field whose host array the caller declares unchanged is not uploaded
    // again while nothing has touched the device since (cfdl_step_host_keep)
    double *synced_ptr[14] = {};
    int64_t synced_launches = -1, synced_graphs = -1, synced_writes = -1;
    void *h_pinned = nullptr;            // pinned staging for host transfers
    size_t h_pinned_bytes = 0;
    int *h_flags = nullptr;              // pinned, per-case convergence flags
    int h_flags_cap = 0;
    int *d_flags = nullptr;
    void *prof = nullptr;                // event profiler state (cfdl_prof.cpp)
    // AMG work lists: amg_cells[l] = level-l cells of cases with nlev >= l
    // (the Galerkin operators), amg_smooth[l] = level-l cells of cases whose
    // V-cycle tail starts below level l (smoothed by per-level kernels);
    // amg_lmax = max nlev
    std::vector<cfdl::WorkList> amg_cells, amg_smooth;      // per level, kTile rows per tile
    std::vector<cfdl::WorkList> amg_gcells, amg_gsmooth;    // per small coarse level, kTile/8 rows per tile
    // restriction targets of the V-cycle's per-level kernels: level-l rows of
    // cases whose tail starts at level l or below (amg_restr), and grouped
    std::vector<cfdl::WorkList> amg_restr, amg_grestr;
    std::vector<int> amg_grouped;                           // lanes per row of each level (1: one thread per row)
    int cgroup = 1;                                          // lanes per row on the large coarse levels (autotuned)
    int amg_lmax = -1;
    bool amg_nb16 = false;                                   // every case has CaseDev::nb16 (the mesh kernels read it)
    bool index16 = true;                                     // cfdl_set_index16: allow amg_nb16
    // solve_uvwp as one CUDA graph with device-side loops (cfdl_graph.cu)
    bool use_graph = true, capturing = false;
    bool graph_branches = true;          // the outer-iteration graph's parallel branches (off: one chain)
    bool pdl = true;                     // launch with programmatic dependent launch (cfdl_set_pdl)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_form = -1;
    int64_t graph_static_kernels = 0, graph_body_kernels[4] = {0, 0, 0, 0}, graph_launches = 0;
    // solve_energy as one CUDA graph (cfdl_graph.cu)
    cudaGraph_t energy_graph = nullptr;
    cudaGraphExec_t energy_exec = nullptr;
    int energy_form = -1;
    int64_t energy_static_kernels = 0, energy_body_kernels = 0;
    unsigned long long *d_loop_passes = nullptr;   // passes of each loop kind, [kLoopSlots]
    // runs of many outer iterations as one graph launch (cfdl_run.cu)
    cudaGraph_t run_graph = nullptr;
    cudaGraphExec_t run_exec = nullptr;
    int run_form = -1;
    int64_t run_static_kernels = 0, run_body_kernels[6] = {0, 0, 0, 0, 0, 0};
    int *d_run_ctl = nullptr, *h_run_ctl = nullptr;   // [0] outer passes left, [1] cases still running
};

namespace cfdl {
int cuda_status(cudaError_t e);
int case_alloc(HostCase *hc, void **p, size_t bytes);
int rebuild_worklists(cfdl_ctx *ctx);
int upload_case_table(cfdl_ctx *ctx);
int create_case(cfdl_ctx *ctx, const cfdl_mesh *mesh, const cfdl_config *cfg, HostCase **out);
// create_case in two halves: host tables (any thread), then device upload
struct CasePrep {
    int ne = 0, nf = 0, nbf = 0, W = 0, H = 0;
    std::vector<int> ef2nb_idx, h_own, h_face, h_kind;
    FillVec<int> hf_nb, hf_fc, f_own, f_nb;   // every element written by prepare_case's parallel loops
    FillVec<double> hf_G, fgeo;
    std::vector<double> h_vel, vol;
    std::vector<double> h_temp;      // energy wall temperatures (empty when the mesh has none)
    AmgHierarchy *amg = nullptr;     // optional, built on the host by prepare_case_amg
    CasePrep() = default;
    CasePrep(const CasePrep &) = delete;
    CasePrep &operator=(const CasePrep &) = delete;
    ~CasePrep();
    void release_tables();           // frees the host tables, keeps the sizes
};
int prepare_case(const cfdl_mesh *mesh, CasePrep *p);
cfdl_ctx *ctx_new();                 // a context with no cases yet (the serving loop's)
int prepare_case_amg(CasePrep *p);
int upload_case(CasePrep &p, const cfdl_config *cfg, HostCase **out);
int upload_case_amg(HostCase *hc, AmgHierarchy *H);
void destroy_case(HostCase *hc);
void apply_config(HostCase *hc, const cfdl_config *cfg);

// kernel launchers (cfdl_kernels.cu): asynchronous on ctx->stream, all cases
void launch_bc(cfdl_ctx *ctx);
void ensure_face_props(cfdl_ctx *ctx);   // recompute the property planes of cases whose rho/mu changed
void ensure_g32(cfdl_ctx *ctx);          // precision 3: rebuild stale FP32 gradients from gu, gv, gw
int ensure_f32_assembly(HostCase *hc, cudaStream_t stream);   // precision 3 arrays (allocated once)
void launch_coef_uvw(cfdl_ctx *ctx);
void launch_grad(cfdl_ctx *ctx, int field);     // 0 u, 1 v, 2 w, 3 phic, 4 = u,v,w fused, 5 = energy t, phi
void launch_calc_mip(cfdl_ctx *ctx, int rhie_chow);
void launch_coef_p(cfdl_ctx *ctx);             // matrix and right-hand side
void launch_coef_p_matrix(cfdl_ctx *ctx);      // face coefficients, ap_p/anb_p (needs dc only)
void launch_coef_p_rhs(cfdl_ctx *ctx);         // b (needs the fluxes of calc_mip)
void launch_adjust_pc(cfdl_ctx *ctx);
void launch_update_uvwp(cfdl_ctx *ctx);
void launch_update_time(cfdl_ctx *ctx);
void launch_set_mip0(cfdl_ctx *ctx);

// energy equation (cfdl_energy.cu)
bool energy_on(const cfdl_ctx *ctx);          // some case of the context has it
void launch_energy_bc(cfdl_ctx *ctx);
void launch_energy_time(cfdl_ctx *ctx, bool run_due);   // run_due: only cases whose run cadence is due
void launch_coef_energy(cfdl_ctx *ctx);
void ensure_energy_props(cfdl_ctx *ctx);      // recompute eprop of cases whose cp/tc changed
int solve_energy_all(cfdl_ctx *ctx);
int solve_energy_phi(cfdl_ctx *ctx);          // the phi solve alone (cfdl_solvers.cu)
void energy_init_solve(cfdl_ctx *ctx);
void energy_iter(cfdl_ctx *ctx);
void energy_finish(cfdl_ctx *ctx);
void launch_energy_temp(cfdl_ctx *ctx);
int energy_init_case(cfdl_ctx *ctx, HostCase *hc, double cp, double tc, double t_init);

// event profiler (cfdl_prof.cpp)
bool prof_wants(cfdl_ctx *ctx, const char *name);
bool prof_active(cfdl_ctx *ctx);
void prof_begin(cfdl_ctx *ctx, const char *name);
void prof_end(cfdl_ctx *ctx);
void prof_destroy(cfdl_ctx *ctx);

#ifdef __CUDACC__
// Launch a kernel whose first statement is CFDL_PDL_WAIT with programmatic
// stream serialization: it may be scheduled while its predecessor in the
// stream drains (inside graphs too, as programmatic edges), which hides the
// gap between dependent launches; or the ordinary way when pdl is off.
template <class... KArgs, class... Args>
inline void launch_k(bool pdl, void (*k)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args... args) {
    if (!pdl) {
        k<<<grid, block, 0, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);
}
#endif

// Launch a tile kernel over work list WL of the context, with optional
// event bracketing for the profiler.
#define CFDL_LAUNCH(name, kern, WL, ...)                                                            \
    do {                                                                                            \
        if (ctx->WL.ntiles > 0) {                                                                   \
            const bool p_ = ctx->prof && cfdl::prof_wants(ctx, name);                               \
            if (p_) cfdl::prof_begin(ctx, name);                                                    \
            cfdl::launch_k(ctx->pdl, kern, (unsigned)ctx->WL.ntiles, (unsigned)cfdl::kTile, ctx->stream, \
                           (const cfdl::CaseDev *)ctx->d_cases, (const cfdl::Tile *)ctx->WL.d_tiles, ##__VA_ARGS__); \
            if (p_) cfdl::prof_end(ctx);                                                            \
            ctx->launches++;                                                                        \
        }                                                                                           \
    } while (0)

// solvers (cfdl_solvers.cu)
int solve_momentum(cfdl_ctx *ctx);
int solve_pressure(cfdl_ctx *ctx);              // operators (multigrid / FP32 copies) + solve
int solve_pressure_prepared(cfdl_ctx *ctx);     // the solve, operators already built
void pressure_operators(cfdl_ctx *ctx);         // what the pressure solve needs of its matrix
// AMG-preconditioned pressure solve (cfdl_amg.cu)
int ensure_amg(cfdl_ctx *ctx);
int solve_pressure_amg(cfdl_ctx *ctx);
int solve_pressure_mixed(cfdl_ctx *ctx);
void free_worklist(WorkList &wl);
int build_worklist(cfdl_ctx *ctx, WorkList &wl, const std::vector<int> &sizes, int tile = kTile);
int read_stats(cfdl_ctx *ctx, int c, cfdl_stats *st);
int poll_kind(cfdl_ctx *ctx, int kind, int *maxit);
int poll_chunk(int done, int expected);

void launch_pc_mean(cfdl_ctx *ctx);

// one outer iteration for every case of the context (cfdl_api.cpp)
int solve_uvwp_all(cfdl_ctx *ctx);

// graph form of solve_uvwp (cfdl_graph.cu)
int build_graph(cfdl_ctx *ctx);
void destroy_graph(cfdl_ctx *ctx);
int solve_uvwp_graph(cfdl_ctx *ctx);
int64_t graph_loop_kernels(cfdl_ctx *ctx);
int build_run_graph(cfdl_ctx *ctx);
int run_graph_launch(cfdl_ctx *ctx);
int solve_energy_graph(cfdl_ctx *ctx);

// runs of many outer iterations (cfdl_run.cu)
void launch_run_begin(cfdl_ctx *ctx);
void launch_run_end(cfdl_ctx *ctx);
void launch_run_cond(cfdl_ctx *ctx, cudaGraphConditionalHandle h, int consume, unsigned long long *passes);
void launch_run_finish(cfdl_ctx *ctx);
int run_outer(cfdl_ctx *ctx, int max_outer, int *running);
}  // namespace cfdl
