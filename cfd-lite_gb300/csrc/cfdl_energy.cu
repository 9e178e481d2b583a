// cfdl_energy.cu -- the energy equation of the reference
// (src/equations/mod_energy.f90) on the device; assembly in FP64 (the solve's
// FP32 correction form for precision >= 2 is in cfdl_solvers.cu).
//
// The equation is for phi = cp*t: upwind advection by the face mass fluxes of
// solve_uvwp, diffusion tc/cp with a deferred correction carrying the
// difference between grad t and grad(phi)/cp, the transient rho*vol/dt, and
// Dirichlet walls.  As in the momentum assembly, the per-face quantities that
// the reference computes from both sides of a face are computed once per face
// (k_en_face) and gathered by the cells in the reference's half-face order
// (k_en_cell); the boundary terms follow in the BC loop's order (ascending
// halo index).  The cp/tc-only face terms (the diffusion coefficients) are
// kept in property planes recomputed only when cp or tc change.  The assembly
// leaves ap, anb, b in the case's shared scratch, as the reference's
// phys%ap/anb/b, and uses the momentum face-term plane fS[0] as its face
// scratch.  The phi solve reuses the momentum BiCGStab kernels
// on one right-hand side (cfdl_solvers.cu).
//
// Every kernel returns at once for a case without the energy equation (its
// energy arrays are null) and for a case whose run has halted, so a batch may
// mix cases with and without it.
#include "cfdl_device.cuh"
#include <algorithm>

namespace cfdl {
namespace {

#define EN_PROLOGUE                               \
    const Tile t = tiles[blockIdx.x];             \
    const CaseDev &C = cases[t.c];                \
    if (!C.ee || C.sc->halted) return;            \
    const int i = t.first + (int)threadIdx.x;

// lid / dirichlet0 of the energy equation (mod_energy.f90:173-212): the halo
// takes the wall temperature and phi = cp(owner)*t.  One thread per halo.
__global__ void __launch_bounds__(kTile) k_en_bc(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    EN_PROLOGUE
    if (i >= t.last || C.h_kind[i] == 0) return;
    const int h = C.ne + i;
    const double tw = C.eh_t[i];
    C.et[h] = tw;
    C.ee[h] = C.ecp[C.h_own[i]] * tw;
}

// update_time's phi0 = phi (mod_physics.f90:111) over cells (halo = 0) or
// halos (halo = 1); run_due: only the cases whose run cadence is due.
__global__ void __launch_bounds__(kTile) k_en_time(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                   int halo, int run_due) {
    CFDL_PDL_WAIT();
    EN_PROLOGUE
    if (run_due && !C.sc->time_due) return;
    if (i >= t.last) return;
    const int j = halo ? C.ne + i : i;
    C.ee0[j] = C.ee[j];
}

// Energy property planes of every face (recomputed when cp or tc change):
// per interior face tc_ip, tc_ip/cp_ip and the diffusion coefficient
// tc_ip/cp_ip * area/(dr.n) of calc_coef_energy (mod_energy.f90:123-125, the
// same from both sides); per boundary face the Dirichlet coefficient
// tc*area/ds/cp of the BC loop (mod_energy.f90:157), where ds = dr.n (the
// momentum walls use |dr|).  The divisions are done here, once.
__global__ void __launch_bounds__(kTile) k_en_props(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    EN_PROLOGUE
    if (i >= t.last) return;
    const int nf = C.nf, o = C.f_own[i], n = C.f_nb[i];
    const double *g = C.fgeo;
    double *ep = C.eprop;
    if (n >= C.ne) {
        ep[EP_D * nf + i] = C.etc[o] * g[FG_ADN * nf + i] / C.ecp[o];
        ep[EP_TC * nf + i] = 0.0;
        ep[EP_TCR * nf + i] = 0.0;
        return;
    }
    const double wt = g[FG_WT * nf + i], omw = 1.0 - wt;
    const double tci = omw * C.etc[o] + wt * C.etc[n];
    const double cpi = omw * C.ecp[o] + wt * C.ecp[n];
    const double r = tci / cpi;
    ep[EP_D * nf + i] = r * g[FG_ADN * nf + i];
    ep[EP_TC * nf + i] = tci;
    ep[EP_TCR * nf + i] = r;
}

// calc_coef_energy, face part (mod_energy.f90:126-128): per interior face, from
// the owner's side, the deferred term
// tc_ip * area * (grad t_ip . n - grad phi_ip . n / cp_ip)
//   = tc_ip * (grad t_ip . A) - tc_ip/cp_ip * (grad phi_ip . A)
// (A the area vector; the neighbour sees the opposite normal and the
// complementary weight, so it takes the negative), into fS[0].
__global__ void __launch_bounds__(kTile) k_en_face(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    EN_PROLOGUE
    if (i >= t.last) return;
    const int nf = C.nf, o = C.f_own[i], n = C.f_nb[i];
    if (n >= C.ne) return;
    const double *g = C.fgeo;
    const double wt = g[FG_WT * nf + i], omw = 1.0 - wt;
    const double A[3] = {g[FG_AX * nf + i], g[FG_AY * nf + i], g[FG_AZ * nf + i]};
    double gtn = 0.0, ghn = 0.0;
#pragma unroll
    for (int m = 0; m < 3; m++) {
        gtn += (omw * C.egt[3 * o + m] + wt * C.egt[3 * n + m]) * A[m];
        ghn += (omw * C.ege[3 * o + m] + wt * C.ege[3 * n + m]) * A[m];
    }
    C.fS[i] = C.eprop[EP_TC * nf + i] * gtn - C.eprop[EP_TCR * nf + i] * ghn;
}

// calc_coef_energy, cell part (mod_energy.f90:92-143, then the BC loop
// :146-168): anb = d + max(f,0) with f = -sg*mip the inward flux,
// ap = sum anb + rho*vol/dt + the wall coefficients,
// b = ap0*phi0 + sumf*phi + sumdefc.
__global__ void __launch_bounds__(kTile) k_en_cell(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    EN_PROLOGUE
    if (i >= t.last) return;
    const int ne = C.ne, W = C.W;
    const double *fd = C.eprop + EP_D * C.nf, *fx = C.fS;
    double ap = 0.0, sumf = 0.0, sumdefc = 0.0;
    double a[kMaxW];
    int nbk[kMaxW], nb_cnt = 0;              // slot neighbours (-1: none), boundary slots
#pragma unroll
    for (int k = 0; k < kMaxW; k++) {
        a[k] = 0.0;
        nbk[k] = -1;
        if (k >= W) continue;
        const int nb = C.hf_nb[k * ne + i];
        nbk[k] = nb;
        if (nb < 0) continue;
        if (nb >= ne) { nb_cnt++; continue; }
        const int fc = C.hf_fc[k * ne + i], f = face_of(fc);
        const double fl = flip_sign(C.mip[f], fc >= 0);   // -sg * mip
        const double ak = fd[f] + positive_part(fl);
        sumf += fl;
        a[k] = ak;
        ap += ak;
        sumdefc += flip_sign(fx[f], fc < 0);              // sg * deferred term
    }
    const double phi = C.ee[i];
    double b;
    if (C.steady) {                                       // ap0 = rho*vol/dt = 0
        b = sumf * phi + sumdefc;
    } else {
        const double ap0 = C.rho[i] * C.vol[i] * C.rdt;
        ap = ap + ap0;
        b = ap0 * C.ee0[i] + sumf * phi + sumdefc;
    }
    // walls in BC-loop order (ascending halo index), the next boundary slot
    // picked by comparisons over the unrolled slots (the row stays in
    // registers); every bound BC is 'dirichlet'
    int prev = -1;
    for (int q = 0; q < nb_cnt; q++) {
        int k = 0, h = 0x7fffffff;
#pragma unroll
        for (int s = 0; s < kMaxW; s++)
            if (nbk[s] >= ne && nbk[s] > prev && nbk[s] < h) { h = nbk[s]; k = s; }
        prev = h;
        if (C.h_kind[h - ne] == 0) continue;
        const double d = fd[face_of(C.hf_fc[k * ne + i])];
        ap = ap + d;
#pragma unroll
        for (int s = 0; s < kMaxW; s++)
            if (s == k) a[s] = a[s] + d;
    }
    C.ap[i] = ap;
    C.b[i] = b;
#pragma unroll
    for (int k = 0; k < kMaxW; k++)
        if (k < W) C.anb[k * ne + i] = a[k];
}

// calc_temperature, mod_properties.f90:214-221: t = phi/cp on the cells
__global__ void __launch_bounds__(kTile) k_en_temp(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    EN_PROLOGUE
    if (i < t.last) C.et[i] = C.ee[i] / C.ecp[i];
}

// t = t_init, phi = cp*t, phi0 = phi over cells and halos (construct_energy,
// mod_energy.f90:33-37); the halos take the cp of their owner
__global__ void k_en_fill(double *t, double *e, double *e0, const double *cp, const int *h_own, int ne, int nbf,
                          double t_init) {
    CFDL_PDL_WAIT();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ne + nbf) return;
    const double c = cp[j < ne ? j : h_own[j - ne]];
    t[j] = t_init;
    e[j] = t_init * c;
    e0[j] = e[j];
}

__global__ void k_fill(double *x, size_t n, double v) {
    CFDL_PDL_WAIT();
    const size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j < n) x[j] = v;
}

}  // namespace

bool energy_on(const cfdl_ctx *ctx) {
    for (const HostCase *hc : ctx->cases)
        if (hc->dev.ee) return true;
    return false;
}

void launch_energy_bc(cfdl_ctx *ctx) {
    if (energy_on(ctx)) CFDL_LAUNCH("k_en_bc", k_en_bc, halos);
}

void launch_energy_time(cfdl_ctx *ctx, bool run_due) {
    if (!energy_on(ctx)) return;
    CFDL_LAUNCH("k_en_time", k_en_time, cells, 0, run_due ? 1 : 0);
    CFDL_LAUNCH("k_en_time_halo", k_en_time, halos, 1, run_due ? 1 : 0);
}

void ensure_energy_props(cfdl_ctx *ctx) {
    bool dirty = false;
    for (HostCase *hc : ctx->cases) dirty |= hc->dev.ee && hc->eprops_dirty;
    if (!dirty || ctx->capturing) return;
    CFDL_LAUNCH("k_en_props", k_en_props, faces);
    for (HostCase *hc : ctx->cases) hc->eprops_dirty = false;
}

void launch_coef_energy(cfdl_ctx *ctx) {
    ensure_energy_props(ctx);
    if (!ctx->capturing)
        for (HostCase *hc : ctx->cases) hc->coef_is_pressure = false;   // ap/anb hold the energy matrix
    CFDL_LAUNCH("k_en_face", k_en_face, faces);
    CFDL_LAUNCH("k_en_cell", k_en_cell, cells);
}

void launch_energy_temp(cfdl_ctx *ctx) { CFDL_LAUNCH("k_en_temp", k_en_temp, cells); }

// solve_energy, mod_energy.f90:59-80 (the run graph has the same sequence
// with the solve as a device-side loop, cfdl_graph.cu)
int solve_energy_all(cfdl_ctx *ctx) {
    if (!energy_on(ctx)) return CFDL_OK;
    if (ctx->use_graph && !prof_active(ctx)) return solve_energy_graph(ctx);
    launch_grad(ctx, 5);                  // calc_grad(t -> gt), calc_grad(phi -> grad), one pass
    launch_coef_energy(ctx);
    int st = solve_energy_phi(ctx);
    if (st) return st;
    launch_energy_temp(ctx);
    return cuda_status(cudaGetLastError());
}

// construct_energy for one case: allocates the energy arrays on first use and
// sets the initial state; the case table is uploaded by the caller.
int energy_init_case(cfdl_ctx *ctx, HostCase *hc, double cp, double tc, double t_init) {
    if (hc->h_temp.empty() || (int)hc->h_temp.size() < hc->nbf) return CFDL_ERR_INVALID;
    CaseDev &d = hc->dev;
    const size_t ne = hc->ne, nc = ne + hc->nbf;
    int st;
    if (!d.ee) {
        // allocate everything first: the case's energy pointers are set only
        // when all of it exists (a null d.ee means "no energy equation")
        CaseDev e = d;
        void *p;
        struct A { double **dst; size_t n; } list[] = {
            {&e.et, nc}, {&e.ee, nc}, {&e.ee0, nc}, {&e.egt, 3 * nc}, {&e.ege, 3 * nc}, {&e.ecp, ne}, {&e.etc, ne},
            {&e.eprop, (size_t)EP_N * hc->nf}};
        for (const A &a : list) {
            if ((st = case_alloc(hc, &p, a.n * sizeof(double)))) return st;
            *a.dst = (double *)p;
        }
        if ((st = case_alloc(hc, &p, std::max<size_t>(hc->nbf, 1) * sizeof(double)))) return st;
        e.eh_t = (const double *)p;
        if ((st = cuda_status(cudaMemcpyAsync(p, hc->h_temp.data(), hc->nbf * sizeof(double), cudaMemcpyHostToDevice,
                                              ctx->stream))))
            return st;
        d.et = e.et; d.ee0 = e.ee0; d.egt = e.egt; d.ege = e.ege; d.ecp = e.ecp; d.etc = e.etc;
        d.eprop = e.eprop; d.eh_t = e.eh_t;
        d.ee = e.ee;
    }
    const int tb = 256;
    k_fill<<<(unsigned)((ne + tb - 1) / tb), tb, 0, ctx->stream>>>(d.ecp, ne, cp);
    k_fill<<<(unsigned)((ne + tb - 1) / tb), tb, 0, ctx->stream>>>(d.etc, ne, tc);
    k_en_fill<<<(unsigned)((nc + tb - 1) / tb), tb, 0, ctx->stream>>>(d.et, d.ee, d.ee0, d.ecp, d.h_own, (int)ne,
                                                                       hc->nbf, t_init);
    ctx->launches += 3;
    hc->eprops_dirty = true;
    if ((st = cuda_status(cudaMemsetAsync(d.egt, 0, 3 * nc * sizeof(double), ctx->stream)))) return st;
    if ((st = cuda_status(cudaMemsetAsync(d.ege, 0, 3 * nc * sizeof(double), ctx->stream)))) return st;
    return cuda_status(cudaGetLastError());
}

}  // namespace cfdl
