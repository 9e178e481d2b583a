// cfdl_solvers.cu -- inner linear solves of solve_uvwp on the device (FP64).
//
// The reference solves each momentum component with symmetric Gauss-Seidel
// (solve_gs, src/modules/mod_solver.f90:255-327) and the pressure correction
// with 4-block Jacobi / SSOR sweeps (multi_subdomain_solver,
// mod_solver.f90:124-189), both stopping at a 10x residual drop or nit sweeps.
// Lexicographic Gauss-Seidel is sequential, so here:
//   momentum  Jacobi-preconditioned BiCGStab on the three components at once
//             (one matrix, three right-hand sides, independent scalars);
//   pressure  Jacobi-preconditioned CG on the singular Neumann system with
//             its right-hand side projected to zero mean (cfdl_precond.cu adds
//             the aggregation-AMG preconditioner and cfdl_mixed.cu the mixed-
//             precision form).
// Stopping: solve_mode 0 stops a component when ||r||2 <= rtol*||r0||2 (the
// reference's 10x drop with rtol = 0.1) or after nit iterations; solve_mode 1
// (tight, parity) stops at ||r||2 <= tight_rtol*||b||2.
//
// All scalars live on the device.  Each reduction writes one partial per tile;
// the last tile of a case to finish sums them in tile order and updates that
// case's scalars, so the iteration never waits for the host.  A component
// that has converged is frozen (its kernels return at once), so polling the
// flags every few iterations gives the same result as checking every one.
#include "cfdl_device.cuh"
#include <algorithm>

namespace cfdl {
namespace {

enum { CNT_M1 = 0, CNT_M2, CNT_M3, CNT_M4, CNT_M5, CNT_P0, CNT_P1, CNT_P2, CNT_P3 };

__device__ __forceinline__ double *comp_field(const CaseDev &C, int q) { return q == 0 ? C.u : q == 1 ? C.v : C.w; }
__device__ __forceinline__ const double *comp_rhs(const CaseDev &C, int q) { return q == 0 ? C.bu : q == 1 ? C.bv : C.bw; }

// (A x)_i for the pressure-correction operator: ap_i x_i - sum_{interior nb} anb x_nb
__device__ __forceinline__ double amul_row(const CaseDev &C, const double *x, int i) {
    double y[1];
    ell_row<1, double>(C.hf_nb, C.anb_p, C.ap_p[i], x, 0, C.ne, C.W, i, y);
    return y[0];
}

__device__ __forceinline__ bool any_active(const SolveScalars *S) { return (S->active[0] | S->active[1] | S->active[2]) != 0; }

#define TILE_HEAD                                             \
    const Tile t = tiles[blockIdx.x];                         \
    const CaseDev &C = cases[t.c];                            \
    SolveScalars *S = C.sc;                                   \
    if (S->halted) return;                                    \
    const int ne = C.ne;                                      \
    (void)ne;

// ------------------------------ momentum ----------------------------------
// init: b' = b + sum_bdry anb*phi_halo, r = b' - A phi, rh = r.
// The row's slot indices and coefficients are loaded once for the three
// components; sums run in slot order.  W is the compile-time slot bound
// (6, 4, or kMaxW for other widths, which stops at the case's C.W).
template <int W>
__device__ __forceinline__ void mom_init_row(const CaseDev &C, int i, int ne, double (&v)[6], bool m32) {
    int nb[W];
    double a[W];
    bool in[W], bd[W];
#pragma unroll
    for (int k = 0; k < W; k++) {
        const int j = k < C.W ? C.hf_nb[k * ne + i] : -1;
        in[k] = j >= 0 && j < ne;
        bd[k] = j >= ne;
        nb[k] = j >= 0 ? j : i;
        a[k] = j >= 0 ? C.anb[k * ne + i] : 0.0;
    }
    const double api = C.ap[i];
    if (m32) {                              // the operator in FP32 for the correction solve
        // integer-pipe conversion (cfdl_device.cuh); the FP32 solve's Jacobi
        // scaling is divided in FP32 (the FP64 1/ap would be one of the
        // kernel's costliest FP64 sequences, for a preconditioner)
        const float fa = narrow_f32(api);
        C.fdiag[i] = fa;
        C.frap[i] = 1.0f / fa;
#pragma unroll
        for (int k = 0; k < W; k++)
            if (k < C.W) C.fanb[k * ne + i] = narrow_f32(a[k]);
    } else {
        C.rap[i] = 1.0 / api;               // the Jacobi scaling of the whole FP64 solve, divided once
    }
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const double *__restrict__ phi = comp_field(C, q);
        double pv[W];
#pragma unroll
        for (int k = 0; k < W; k++) pv[k] = phi[nb[k]];
        double bb = comp_rhs(C, q)[i];
        double s = api * phi[i];
#pragma unroll
        for (int k = 0; k < W; k++) {
            if (bd[k]) bb += a[k] * pv[k];
            else if (in[k]) s -= a[k] * pv[k];
        }
        const double r = bb - s;
        // p and v need no clearing: the first iteration sets p = r (k_mom_p)
        if (m32) {
            // FP32 correction solve A d = r from d = 0 (first halves of kr, krh; d after kt's)
            const float rf = narrow_f32(r);
            ((float *)C.kr)[q * ne + i] = rf;
            ((float *)C.krh)[q * ne + i] = rf;
            ((float *)C.kt)[3 * (size_t)ne + q * ne + i] = 0.f;
        } else {
            C.kr[q * ne + i] = r;
            C.krh[q * ne + i] = r;
        }
        v[q] += bb * bb;
        v[3 + q] += r * r;
    }
}

__global__ void __launch_bounds__(kTile, 3) k_mom_init(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                    const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    double v[6] = {0, 0, 0, 0, 0, 0};
    const bool m32 = C.precision >= 2;
    if (C.W == 6) { FOR_CELLS(t) mom_init_row<6>(C, i, ne, v, m32); }
    else if (C.W == 4) { FOR_CELLS(t) mom_init_row<4>(C, i, ne, v, m32); }
    else { FOR_CELLS(t) mom_init_row<kMaxW>(C, i, ne, v, m32); }
    block_reduce<6>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_M1], cnt[t.c])) {
        __shared__ double s[6];
        sum_partials<6>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            const int cap = C.solve_mode == 0 ? C.nit : C.tight_maxit;
            for (int q = 0; q < 3; q++) {
                S->bnorm[q] = sqrt(s[q]);
                S->r0norm[q] = S->rnorm[q] = sqrt(s[3 + q]);
                S->rho[q] = s[3 + q];
                S->alpha[q] = 1.0; S->omega[q] = 1.0; S->beta[q] = 0.0; S->half[q] = 0;
                S->iters[q] = 0; S->status[q] = 0;
                S->tol[q] = C.solve_mode == 0 ? C.rtol_u * S->r0norm[q] : C.tight_rtol * S->bnorm[q];
                S->active[q] = (S->r0norm[q] > S->tol[q]) && cap > 0;
                if (!isfinite(S->r0norm[q]) || !isfinite(S->bnorm[q])) { S->active[q] = 0; S->status[q] = CFDL_ERR_NONFINITE; }
            }
        }
    }
}

// The BiCGStab vectors and operator of a case's solve, [NC][ne] per vector.
// NC = 3, the momentum solve: FP64 updates u, v, w in place; FP32
// (precision 2) finds the correction d of A d = r (r the FP64 residual of
// k_mom_init) in single precision, in the first halves of the FP64 vectors'
// storage, and k_mom_apply adds it to u, v, w in FP64.  NC = 1, the energy
// solve (cfdl_energy.cu): FP64, phi = C.ee in place, plane 0 of the vectors.
template <class T> struct MomVec {
    T *r, *rh, *p, *ph, *v, *s, *sh, *t;
    T *x[3];
    const T *a, *ap, *rap;
};
template <class T, int NC> __device__ __forceinline__ MomVec<T> mom_vec(const CaseDev &C);
template <> __device__ __forceinline__ MomVec<double> mom_vec<double, 3>(const CaseDev &C) {
    return {C.kr, C.krh, C.kp, C.kph, C.kv, C.ks, C.ksh, C.kt, {C.u, C.v, C.w}, C.anb, C.ap, C.rap};
}
template <> __device__ __forceinline__ MomVec<float> mom_vec<float, 3>(const CaseDev &C) {
    const int ne = C.ne;
    float *xf = (float *)C.kt + 3 * (size_t)ne;   // second half of kt's storage
    return {(float *)C.kr, (float *)C.krh, (float *)C.kp, (float *)C.kph, (float *)C.kv, (float *)C.ks,
            (float *)C.ksh, (float *)C.kt, {xf, xf + ne, xf + 2 * (size_t)ne}, C.fanb, C.fdiag, C.frap};
}
template <> __device__ __forceinline__ MomVec<double> mom_vec<double, 1>(const CaseDev &C) {
    return {C.kr, C.krh, C.kp, C.kph, C.kv, C.ks, C.ksh, C.kt, {C.ee, nullptr, nullptr}, C.anb, C.ap, C.rap};
}
// the energy solve's FP32 correction form (precision >= 2): as the momentum one
template <> __device__ __forceinline__ MomVec<float> mom_vec<float, 1>(const CaseDev &C) { return mom_vec<float, 3>(C); }

// the lanes of the solve: momentum u, v, w or the energy lane
template <int NC> __device__ __forceinline__ KLanes *lanes(SolveScalars *S) { return NC == 3 ? (KLanes *)S : &S->en; }
template <int NC> __device__ __forceinline__ bool lanes_active(const KLanes *L) {
    int a = 0;
#pragma unroll
    for (int q = 0; q < NC; q++) a |= L->active[q];
    return a != 0;
}

// p = r + beta (p - omega v); ph = p / ap
template <class T, int NC>
__global__ void __launch_bounds__(kTile) k_mom_p(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    const KLanes *L = lanes<NC>(S);
    if (!lanes_active<NC>(L)) return;
    const MomVec<T> M = mom_vec<T, NC>(C);
    // the iteration's scalars, read once
    int act[NC];
    bool first[NC];
    T be[NC], om[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) {
        act[q] = L->active[q]; first[q] = L->iters[q] == 0; be[q] = (T)L->beta[q]; om[q] = (T)L->omega[q];
    }
    FOR_CELLS(t) {
        const T rap = M.rap[i];
        T rr[NC], pp[NC], vv[NC];   // the row's loads, before its stores
#pragma unroll
        for (int q = 0; q < NC; q++) {
            const int j = q * ne + i;
            rr[q] = pp[q] = vv[q] = 0;
            if (!act[q]) continue;
            rr[q] = M.r[j];
            if (!first[q]) { pp[q] = M.p[j]; vv[q] = M.v[j]; }
        }
#pragma unroll
        for (int q = 0; q < NC; q++) {
            if (!act[q]) continue;
            const int j = q * ne + i;
            const T pn = first[q] ? rr[q] : rr[q] + be[q] * (pp[q] - om[q] * vv[q]);
            M.p[j] = pn;
            M.ph[j] = pn * rap;
        }
    }
}

// v = A ph; alpha = rho / (rh, v)
template <class T, int NC>
__global__ void __launch_bounds__(kTile, 4) k_mom_v(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                 const int *__restrict__ cfirst, const int *__restrict__ cnt, T *partials) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    KLanes *L = lanes<NC>(S);
    if (!lanes_active<NC>(L)) return;
    const MomVec<T> M = mom_vec<T, NC>(C);
    T v[NC];
    int act[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) { v[q] = 0; act[q] = L->active[q]; }
    FOR_CELLS(t) {
        T y[NC], rh[NC];   // one pass over the row for the components
        ell_row<NC, T>(C.hf_nb, M.a, M.ap[i], M.ph, ne, ne, C.W, i, y);
#pragma unroll
        for (int q = 0; q < NC; q++) rh[q] = act[q] ? M.rh[q * ne + i] : (T)0;   // loads before the stores
#pragma unroll
        for (int q = 0; q < NC; q++) {
            if (!act[q]) continue;
            M.v[q * ne + i] = y[q];
            v[q] += rh[q] * y[q];
        }
    }
    block_reduce<NC, T>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_M2], cnt[t.c])) {
        __shared__ T s[NC];
        sum_partials<NC, T>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0)
            for (int q = 0; q < NC; q++) {
                if (!L->active[q]) continue;
                const double sq = (double)s[q];
                const double a = L->rho[q] / sq;
                if (sq == 0.0 || !isfinite(a)) { L->active[q] = 0; L->status[q] = isfinite(a) || sq == 0.0 ? L->status[q] : CFDL_ERR_NONFINITE; continue; }
                L->alpha[q] = a;
            }
    }
}

// s = r - alpha v; sh = s / ap; early exit when ||s|| <= tol
template <class T, int NC>
__global__ void __launch_bounds__(kTile) k_mom_s(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                 const int *__restrict__ cfirst, const int *__restrict__ cnt, T *partials) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    KLanes *L = lanes<NC>(S);
    if (!lanes_active<NC>(L)) return;
    const MomVec<T> M = mom_vec<T, NC>(C);
    T v[NC], al[NC];
    int act[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) { v[q] = 0; act[q] = L->active[q]; al[q] = (T)L->alpha[q]; }
    FOR_CELLS(t) {
        const T rap = M.rap[i];
        if (sizeof(T) == 4) {
            // FP32: the row's loads, every component's, before its stores
            // (36 -> 27 us a launch at 128^3; the FP64 form measured slower
            // this way, 63 -> 68 us, and keeps one component at a time)
            T rr[NC], vv[NC];
#pragma unroll
            for (int q = 0; q < NC; q++) {
                rr[q] = act[q] ? M.r[q * ne + i] : (T)0;
                vv[q] = act[q] ? M.v[q * ne + i] : (T)0;
            }
#pragma unroll
            for (int q = 0; q < NC; q++) {
                if (!act[q]) continue;
                const int j = q * ne + i;
                const T sv = rr[q] - al[q] * vv[q];
                M.s[j] = sv;
                M.sh[j] = sv * rap;
                v[q] += sv * sv;
            }
        } else {
#pragma unroll
            for (int q = 0; q < NC; q++) {
                if (!act[q]) continue;
                const int j = q * ne + i;
                const T sv = M.r[j] - al[q] * M.v[j];
                M.s[j] = sv;
                M.sh[j] = sv * rap;
                v[q] += sv * sv;
            }
        }
    }
    block_reduce<NC, T>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_M3], cnt[t.c])) {
        __shared__ T s[NC];
        sum_partials<NC, T>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0)
            for (int q = 0; q < NC; q++) {
                if (!L->active[q]) continue;
                L->half[q] = sqrt((double)s[q]) <= L->tol[q];
            }
    }
}

// t = A sh; omega = (t,s)/(t,t)
template <class T, int NC>
__global__ void __launch_bounds__(kTile, 4) k_mom_t(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                 const int *__restrict__ cfirst, const int *__restrict__ cnt, T *partials) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    KLanes *L = lanes<NC>(S);
    if (!lanes_active<NC>(L)) return;
    const MomVec<T> M = mom_vec<T, NC>(C);
    T v[2 * NC];
    int act[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) { v[q] = v[NC + q] = 0; act[q] = L->active[q] && !L->half[q]; }
    FOR_CELLS(t) {
        T y[NC], sv[NC];
        ell_row<NC, T>(C.hf_nb, M.a, M.ap[i], M.sh, ne, ne, C.W, i, y);
#pragma unroll
        for (int q = 0; q < NC; q++) sv[q] = act[q] ? M.s[q * ne + i] : (T)0;   // loads before the stores
#pragma unroll
        for (int q = 0; q < NC; q++) {
            if (!act[q]) continue;
            const int j = q * ne + i;
            M.t[j] = y[q];
            v[q] += y[q] * sv[q];
            v[NC + q] += y[q] * y[q];
        }
    }
    block_reduce<2 * NC, T>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_M4], cnt[t.c])) {
        __shared__ T s[2 * NC];
        sum_partials<2 * NC, T>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0)
            for (int q = 0; q < NC; q++) {
                if (!L->active[q]) continue;
                const double ts = (double)s[q], tt = (double)s[NC + q];
                L->omega[q] = L->half[q] ? 0.0 : (tt > 0.0 ? ts / tt : 0.0);
            }
    }
}

// x += alpha ph + omega sh; r = s - omega t; rho' = (rh, r); beta
template <class T, int NC>
__global__ void __launch_bounds__(kTile, 4) k_mom_x(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                 const int *__restrict__ cfirst, const int *__restrict__ cnt, T *partials) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    KLanes *L = lanes<NC>(S);
    if (!lanes_active<NC>(L)) return;
    const MomVec<T> M = mom_vec<T, NC>(C);
    T v[2 * NC], al[NC], om[NC];
    int act[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) {
        v[q] = v[NC + q] = 0; act[q] = L->active[q]; al[q] = (T)L->alpha[q]; om[q] = (T)L->omega[q];
    }
    FOR_CELLS(t) {
        // the row's loads, every component's, before its stores
        T xv[NC], ph[NC], sh[NC], sv[NC], tv[NC], rh[NC];
#pragma unroll
        for (int q = 0; q < NC; q++) {
            const int j = q * ne + i;
            xv[q] = ph[q] = sh[q] = sv[q] = tv[q] = rh[q] = 0;
            if (!act[q]) continue;
            xv[q] = M.x[q][i]; ph[q] = M.ph[j]; sh[q] = M.sh[j]; sv[q] = M.s[j]; rh[q] = M.rh[j];
            if (om[q] != (T)0) tv[q] = M.t[j];
        }
#pragma unroll
        for (int q = 0; q < NC; q++) {
            if (!act[q]) continue;
            const int j = q * ne + i;
            M.x[q][i] = xv[q] + al[q] * ph[q] + om[q] * sh[q];
            const T r = om[q] == (T)0 ? sv[q] : sv[q] - om[q] * tv[q];
            M.r[j] = r;
            v[q] += r * r;
            v[NC + q] += rh[q] * r;
        }
    }
    block_reduce<2 * NC, T>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_M5], cnt[t.c])) {
        __shared__ T s[2 * NC];
        sum_partials<2 * NC, T>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            const int cap = C.solve_mode == 0 ? C.nit : C.tight_maxit;
            for (int q = 0; q < NC; q++) {
                if (!L->active[q]) continue;
                const double rn = sqrt((double)s[q]), rho_new = (double)s[NC + q];
                L->rnorm[q] = rn;
                L->iters[q] += 1;
                const double om = L->omega[q];
                L->beta[q] = (om != 0.0 && L->rho[q] != 0.0) ? (rho_new / L->rho[q]) * (L->alpha[q] / om) : 0.0;
                L->rho[q] = rho_new;
                int act = rn > L->tol[q];
                if (!isfinite(rn)) { act = 0; L->status[q] = CFDL_ERR_NONFINITE; }
                else if (act && (om == 0.0 || rho_new == 0.0)) act = 0;           // breakdown: stop here
                else if (act && L->iters[q] >= cap) { act = 0; if (C.solve_mode == 1) L->status[q] = CFDL_ERR_ITER_CAP; }
                L->active[q] = act;
            }
        }
    }
}

// ------------------------------- energy -----------------------------------
// init of the phi solve of solve_energy (mod_energy.f90:75): b' = b +
// sum_bdry anb*phi_halo, r = b' - A phi, rh = r; cases without the energy
// equation contribute nothing and stay inactive.  m32 (precision >= 2): the
// solve finds the correction d of A d = r in FP32 from d = 0, as the momentum
// solve does, on FP32 copies of the operator.
template <int W>
__device__ __forceinline__ void en_init_row(const CaseDev &C, int i, int ne, double (&v)[2], bool m32) {
    const double api = C.ap[i];
    if (m32) { const float fa = narrow_f32(api); C.fdiag[i] = fa; C.frap[i] = 1.0f / fa; }
    else C.rap[i] = 1.0 / api;
    const double *__restrict__ phi = C.ee;
    double bb = C.b[i], s = api * phi[i];
#pragma unroll
    for (int k = 0; k < W; k++) {
        const int j = k < C.W ? C.hf_nb[k * ne + i] : -1;
        if (j < 0) continue;
        const double a = C.anb[k * ne + i];
        if (m32) C.fanb[k * ne + i] = narrow_f32(a);
        if (j >= ne) bb += a * phi[j];
        else s -= a * phi[j];
    }
    const double r = bb - s;
    if (m32) {
        const float rf = narrow_f32(r);
        ((float *)C.kr)[i] = rf;
        ((float *)C.krh)[i] = rf;
        ((float *)C.kt)[3 * (size_t)ne + i] = 0.f;
    } else {
        C.kr[i] = r;
        C.krh[i] = r;
    }
    v[0] += bb * bb;
    v[1] += r * r;
}

__global__ void __launch_bounds__(kTile, 3) k_en_init(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                   const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    double v[2] = {0, 0};
    const bool m32 = C.precision >= 2;
    if (C.ee) {
        if (C.W == 6) { FOR_CELLS(t) en_init_row<6>(C, i, ne, v, m32); }
        else if (C.W == 4) { FOR_CELLS(t) en_init_row<4>(C, i, ne, v, m32); }
        else { FOR_CELLS(t) en_init_row<kMaxW>(C, i, ne, v, m32); }
    }
    block_reduce<2>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_M1], cnt[t.c])) {
        __shared__ double s[2];
        sum_partials<2>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            KLanes *L = &S->en;
            const int cap = C.solve_mode == 0 ? C.nit : C.tight_maxit;
            L->bnorm[0] = sqrt(s[0]);
            L->r0norm[0] = L->rnorm[0] = sqrt(s[1]);
            L->rho[0] = s[1];
            L->alpha[0] = 1.0; L->omega[0] = 1.0; L->beta[0] = 0.0; L->half[0] = 0;
            L->iters[0] = 0; L->status[0] = 0;
            L->tol[0] = C.solve_mode == 0 ? C.rtol_u * L->r0norm[0] : C.tight_rtol * L->bnorm[0];
            L->active[0] = C.ee != nullptr && L->r0norm[0] > L->tol[0] && cap > 0;
            if (!isfinite(L->r0norm[0]) || !isfinite(L->bnorm[0])) { L->active[0] = 0; L->status[0] = CFDL_ERR_NONFINITE; }
            L->active[1] = L->active[2] = 0;
        }
    }
}

// precision >= 2: phi += the FP32 correction of the energy solve
__global__ void __launch_bounds__(kTile) k_en_apply(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    if (!C.ee) return;
    const float *x = mom_vec<float, 1>(C).x[0];
    FOR_CELLS(t) C.ee[i] = C.ee[i] + widen_f64(x[i]);
}

// precision 2: u, v, w += the FP32 correction of the momentum solve
__global__ void __launch_bounds__(kTile) k_mom_apply(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    const MomVec<float> M = mom_vec<float, 3>(C);
    double *xs[3] = {C.u, C.v, C.w};
    FOR_CELLS(t) {
#pragma unroll
        for (int q = 0; q < 3; q++) xs[q][i] = xs[q][i] + widen_f64(M.x[q][i]);
    }
}

// ------------------------------ pressure ----------------------------------
// mean of b (the singular Neumann system is made consistent)
__global__ void __launch_bounds__(kTile) k_pc_mean(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                   const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    double v[1] = {0.0};
    FOR_CELLS(t) v[0] += C.b[i];
    block_reduce<1>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_P0], cnt[t.c])) {
        __shared__ double s[1];
        sum_partials<1>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) S->mean_b = s[0] / ne;
    }
}

// r = b - mean, z = r/ap, p = z, x = 0 (set_a_0(phic))
__global__ void __launch_bounds__(kTile) k_pc_init(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                   const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    double v[3] = {0, 0, 0};
    FOR_CELLS(t) {
        const double r = C.b[i] - S->mean_b, z = r / C.ap_p[i];
        C.kr[i] = r; C.ks[i] = z; C.kp[i] = z; C.phic[i] = 0.0;
        v[0] += r * r; v[1] += r * z; v[2] += C.b[i] * C.b[i];
    }
    block_reduce<3>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_P1], cnt[t.c])) {
        __shared__ double s[3];
        sum_partials<3>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            const int cap = C.solve_mode == 0 ? C.nit : C.tight_maxit;
            S->r0norm_p = S->rnorm_p = sqrt(s[0]);
            S->rz = s[1];
            S->mass_imbalance = sqrt(s[2]);
            S->iters_p = 0; S->status_p = 0;
            S->tol_p = (C.solve_mode == 0 ? C.rtol_p : C.tight_rtol) * S->r0norm_p;
            S->active_p = S->r0norm_p > S->tol_p && cap > 0;
            if (!isfinite(S->r0norm_p)) { S->active_p = 0; S->status_p = CFDL_ERR_NONFINITE; }
        }
    }
}

// q = A p; alpha = rz / (p, q)
__global__ void __launch_bounds__(kTile) k_pc_q(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    if (!S->active_p) return;
    double v[1] = {0};
    FOR_CELLS(t) {
        const double q = amul_row(C, C.kp, i);
        C.kv[i] = q;
        v[0] += C.kp[i] * q;
    }
    block_reduce<1>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_P2], cnt[t.c])) {
        __shared__ double s[1];
        sum_partials<1>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            if (!(s[0] > 0.0) || !isfinite(s[0])) {
                // runs only while ||r|| is above the tolerance, where p.Ap > 0 for the SPD system
                S->active_p = 0;
                S->status_p = isfinite(s[0]) ? CFDL_ERR_BREAKDOWN : CFDL_ERR_NONFINITE;
            }
            else S->alpha_p = S->rz / s[0];
        }
    }
}

// x += alpha p; r -= alpha q; z = r/ap; beta = (r,z)'/(r,z)
__global__ void __launch_bounds__(kTile) k_pc_x(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    if (!S->active_p) return;
    double v[2] = {0, 0};
    FOR_CELLS(t) {
        const double a = S->alpha_p;
        C.phic[i] = C.phic[i] + a * C.kp[i];
        const double r = C.kr[i] - a * C.kv[i], z = r / C.ap_p[i];
        C.kr[i] = r; C.ks[i] = z;
        v[0] += r * r; v[1] += r * z;
    }
    block_reduce<2>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_P3], cnt[t.c])) {
        __shared__ double s[2];
        sum_partials<2>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            const int cap = C.solve_mode == 0 ? C.nit : C.tight_maxit;
            const double rn = sqrt(s[0]);
            S->rnorm_p = rn;
            S->iters_p += 1;
            S->beta_p = S->rz != 0.0 ? s[1] / S->rz : 0.0;
            S->rz = s[1];
            int act = rn > S->tol_p;
            if (!isfinite(rn)) { act = 0; S->status_p = CFDL_ERR_NONFINITE; }
            else if (act && S->iters_p >= cap) { act = 0; if (C.solve_mode == 1) S->status_p = CFDL_ERR_ITER_CAP; }
            S->active_p = act;
        }
    }
}

// p = z + beta p
__global__ void __launch_bounds__(kTile) k_pc_p(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_HEAD
    if (!S->active_p) return;
    FOR_CELLS(t) C.kp[i] = C.ks[i] + S->beta_p * C.kp[i];
}

// Per-case activity flag and iteration count for the host poll.
// kind 0 momentum, 1 pressure CG, 2 mixed inner CG, 3 mixed outer refinement,
// 4 energy.
__global__ void k_poll(const CaseDev *__restrict__ cases, int ncases, int *flags, int kind) {
    CFDL_PDL_WAIT();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncases) return;
    const SolveScalars *S = cases[c].sc;
    int act = 0, its = 0;
    if (kind == 0) { act = any_active(S); its = max(S->iters[0], max(S->iters[1], S->iters[2])); }
    else if (kind == 1) { act = S->active_p; its = S->iters_p; }
    else if (kind == 2) { act = S->active32; its = S->iters32; }
    else if (kind == 3) { act = S->active_p; its = S->outer_p; }
    else { act = S->en.active[0]; its = S->en.iters[0]; }
    flags[2 * c] = act != 0;
    flags[2 * c + 1] = its;
}

}  // namespace

#define RED ctx->cellsv.d_case_first, ctx->cellsv.d_case_ntiles, ctx->d_partials

// Returns 1 if any case is still active, 0 if none, -1 on error; *maxit =
// the largest iteration count over the cases.
int poll_kind(cfdl_ctx *ctx, int kind, int *maxit) {
    const int n = (int)ctx->cases.size();
    k_poll<<<(n + 127) / 128, 128, 0, ctx->stream>>>(ctx->d_cases, n, ctx->d_flags, kind);
    ctx->launches++;
    cudaError_t e = cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, 2 * n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return -1;
    int any = 0, m = 0;
    for (int c = 0; c < n; c++) { any |= ctx->h_flags[2 * c]; m = std::max(m, ctx->h_flags[2 * c + 1]); }
    if (maxit) *maxit = m;
    return any;
}

// Iterations to issue before the next poll: first up to just short of the
// previous solve's count (consecutive outer iterations need similar counts),
// then one at a time.  Converged cases are frozen on the device, so the
// schedule changes only the number of idle launches, never the result.
int poll_chunk(int done, int expected) {
    if (done == 0) return std::max(1, expected - 1);
    return 1;
}

static int max_cap(cfdl_ctx *ctx) {
    int cap = 0;
    for (auto *hc : ctx->cases) cap = std::max(cap, hc->cfg.solve_mode == 0 ? hc->cfg.nit : hc->cfg.tight_maxit);
    return cap;
}

void mom_init(cfdl_ctx *ctx) { CFDL_LAUNCH("k_mom_init", k_mom_init, cellsv, RED); }

#define RED32 ctx->cellsv.d_case_first, ctx->cellsv.d_case_ntiles, (float *)ctx->d_partials

void mom_iter(cfdl_ctx *ctx) {
    if (ctx->cases[0]->cfg.precision >= 2) {
        CFDL_LAUNCH("k_mom_p", (k_mom_p<float, 3>), cellsv);
        CFDL_LAUNCH("k_mom_v", (k_mom_v<float, 3>), cellsv, RED32);
        CFDL_LAUNCH("k_mom_s", (k_mom_s<float, 3>), cellsv, RED32);
        CFDL_LAUNCH("k_mom_t", (k_mom_t<float, 3>), cellsv, RED32);
        CFDL_LAUNCH("k_mom_x", (k_mom_x<float, 3>), cellsv, RED32);
        return;
    }
    CFDL_LAUNCH("k_mom_p", (k_mom_p<double, 3>), cellsv);
    CFDL_LAUNCH("k_mom_v", (k_mom_v<double, 3>), cellsv, RED);
    CFDL_LAUNCH("k_mom_s", (k_mom_s<double, 3>), cellsv, RED);
    CFDL_LAUNCH("k_mom_t", (k_mom_t<double, 3>), cellsv, RED);
    CFDL_LAUNCH("k_mom_x", (k_mom_x<double, 3>), cellsv, RED);
}

// Jacobi-preconditioned BiCGStab on the energy system, with the momentum
// solve's kernels on one right-hand side and the energy lane
#define REDE ctx->cellse.d_case_first, ctx->cellse.d_case_ntiles, ctx->d_partials

void energy_init_solve(cfdl_ctx *ctx) { CFDL_LAUNCH("k_en_init", k_en_init, cellse, REDE); }

int solve_energy_phi(cfdl_ctx *ctx) {
    if (ctx->cells.ntiles == 0) return CFDL_OK;
    energy_init_solve(ctx);
    const int cap = max_cap(ctx);
    int it = 0, maxit = 0;
    while (it < cap) {
        const int chunk = poll_chunk(it, ctx->last_iters_e);
        for (int k = 0; k < chunk && it < cap; k++, it++) energy_iter(ctx);
        int a = poll_kind(ctx, 4, &maxit);
        if (a < 0) return CFDL_ERR_CUDA;
        if (a == 0) break;
    }
    ctx->last_iters_e = maxit;
    energy_finish(ctx);
    return cuda_status(cudaGetLastError());
}

// the end of the energy solve: precision >= 2 applies its FP32 correction
void energy_finish(cfdl_ctx *ctx) {
    if (ctx->cases[0]->cfg.precision >= 2) CFDL_LAUNCH("k_en_apply", k_en_apply, cellse);
}

// one BiCGStab iteration of the energy solve (one right-hand side; FP64, or
// FP32 on the correction for precision >= 2)
#define REDE32 ctx->cellse.d_case_first, ctx->cellse.d_case_ntiles, (float *)ctx->d_partials
void energy_iter(cfdl_ctx *ctx) {
    if (ctx->cases[0]->cfg.precision >= 2) {
        CFDL_LAUNCH("k_en_p", (k_mom_p<float, 1>), cellse);
        CFDL_LAUNCH("k_en_v", (k_mom_v<float, 1>), cellse, REDE32);
        CFDL_LAUNCH("k_en_s", (k_mom_s<float, 1>), cellse, REDE32);
        CFDL_LAUNCH("k_en_t", (k_mom_t<float, 1>), cellse, REDE32);
        CFDL_LAUNCH("k_en_x", (k_mom_x<float, 1>), cellse, REDE32);
        return;
    }
    CFDL_LAUNCH("k_en_p", (k_mom_p<double, 1>), cellse);
    CFDL_LAUNCH("k_en_v", (k_mom_v<double, 1>), cellse, REDE);
    CFDL_LAUNCH("k_en_s", (k_mom_s<double, 1>), cellse, REDE);
    CFDL_LAUNCH("k_en_t", (k_mom_t<double, 1>), cellse, REDE);
    CFDL_LAUNCH("k_en_x", (k_mom_x<double, 1>), cellse, REDE);
}

// the end of the momentum solve: precision 2 applies its FP32 correction
void mom_finish(cfdl_ctx *ctx) {
    if (ctx->cases[0]->cfg.precision >= 2) CFDL_LAUNCH("k_mom_apply", k_mom_apply, cellsv);
}

void pcj_init(cfdl_ctx *ctx) {
    CFDL_LAUNCH("k_pc_mean", k_pc_mean, cellsv, RED);
    CFDL_LAUNCH("k_pc_init", k_pc_init, cellsv, RED);
}

void pcj_iter(cfdl_ctx *ctx) {
    CFDL_LAUNCH("k_pc_q", k_pc_q, cellsv, RED);
    CFDL_LAUNCH("k_pc_x", k_pc_x, cellsv, RED);
    CFDL_LAUNCH("k_pc_p", k_pc_p, cellsv);
}

int solve_momentum(cfdl_ctx *ctx) {
    if (ctx->cells.ntiles == 0) return CFDL_OK;
    mom_init(ctx);
    const int cap = max_cap(ctx);
    int it = 0, maxit = 0;
    while (it < cap) {
        const int chunk = poll_chunk(it, ctx->last_iters_m);
        for (int k = 0; k < chunk && it < cap; k++, it++) mom_iter(ctx);
        int a = poll_kind(ctx, 0, &maxit);
        if (a < 0) return CFDL_ERR_CUDA;
        if (a == 0) break;
    }
    ctx->last_iters_m = maxit;
    mom_finish(ctx);
    return cuda_status(cudaGetLastError());
}

void launch_pc_mean(cfdl_ctx *ctx) { CFDL_LAUNCH("k_pc_mean", k_pc_mean, cellsv, RED); }

// the pressure solve with its operators (the per-routine entry point)
int solve_pressure(cfdl_ctx *ctx) {
    if (ctx->cells.ntiles == 0) return CFDL_OK;
    int st;
    if (ctx->cases[0]->cfg.precond == 1 && (st = ensure_amg(ctx))) return st;
    pressure_operators(ctx);
    return solve_pressure_prepared(ctx);
}

int solve_pressure_prepared(cfdl_ctx *ctx) {
    if (ctx->cells.ntiles == 0) return CFDL_OK;
    if (ctx->cases[0]->cfg.precision >= 1) return solve_pressure_mixed(ctx);
    if (ctx->cases[0]->cfg.precond == 1) return solve_pressure_amg(ctx);
    pcj_init(ctx);
    const int cap = max_cap(ctx);
    int it = 0, maxit = 0;
    while (it < cap) {
        const int chunk = poll_chunk(it, ctx->last_iters_p);
        for (int k = 0; k < chunk && it < cap; k++, it++) pcj_iter(ctx);
        int a = poll_kind(ctx, 1, &maxit);
        if (a < 0) return CFDL_ERR_CUDA;
        if (a == 0) break;
    }
    ctx->last_iters_p = maxit;
    return cuda_status(cudaGetLastError());
}

int read_stats(cfdl_ctx *ctx, int c, cfdl_stats *st) {
    SolveScalars S;
    cudaError_t e = cudaMemcpyAsync(&S, ctx->cases[c]->dev.sc, sizeof(S), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_status(e);
    st->it_u = S.iters[0]; st->it_v = S.iters[1]; st->it_w = S.iters[2]; st->it_p = S.iters_p;
    for (int q = 0; q < 3; q++) { st->res_i[q] = S.r0norm[q]; st->res_f[q] = S.rnorm[q]; }
    st->res_i[3] = S.r0norm_p; st->res_f[3] = S.rnorm_p;
    st->mass_imbalance = S.mass_imbalance;
    st->outer_done = S.outer_done;
    st->run_left = S.run_left;
    st->converged = S.converged;
    st->mass_ratio = S.mass_ratio;
    st->it_e = S.en.iters[0];
    st->res_e[0] = S.en.r0norm[0]; st->res_e[1] = S.en.rnorm[0];
    st->status = 0;
    for (int q = 0; q < 3; q++) if (S.status[q]) st->status = S.status[q];
    if (S.en.status[0]) st->status = S.en.status[0];
    if (S.status_p) st->status = S.status_p;
    return CFDL_OK;
}

}  // namespace cfdl
