// cfdl_amg.cu -- aggregation-AMG preconditioned CG for the pressure
// correction (FP64), and the mixed-precision form (FP32 AMG-PCG inner solve,
// FP64 residual and refinement).
//
// The reference solves the pressure correction with 4-block Jacobi / SSOR
// sweeps (multi_subdomain_solver, src/modules/mod_solver.f90:124-189), whose
// convergence degrades with the mesh size.  Here CG on the same singular
// Neumann system (right-hand side projected to zero mean) is preconditioned
// by one V-cycle of aggregation multigrid:
//   level l -> l+1   two damped-Jacobi sweeps, residual restricted by summing
//                    over each aggregate (P^T, P piecewise constant);
//   coarsest level   dense inverse of (A_L + c 11^T), which is A_L's
//                    pseudo-inverse on zero-sum right-hand sides;
//   level l+1 -> l   prolongation (injection, scaled by kOverCorrect) added
//                    in place, then two damped-Jacobi sweeps;
//   small levels     a case's levels of at most kTailRows rows and its
//                    coarsest solve run in one CTA (k_v_tail).
// Pre- and post-smoothing match, so the preconditioner is symmetric and
// positive semi-definite, as CG requires.  The coarse operators are rebuilt
// at every pressure solve from the current coefficients (A_c = P^T A P).
#include "cfdl_amg.h"
#include "cfdl_device.cuh"
#include "cfdl_par.h"
#include <algorithm>
#include <new>

namespace cfdl {
namespace {

// Damped-Jacobi weights of a level's two smoothing sweeps.  Pre-smoothing
// runs the kOmega sweep from zero (k_v_jac0) and then the kOmega2 sweep;
// post-smoothing runs the kOmega sweep from the prolongated value and then
// the kOmega2 sweep.  Either way the error propagator is
// (I - kOmega2 D^-1 A)(I - kOmega D^-1 A), the same polynomial in D^-1 A
// before and after the coarse correction, so the V-cycle stays symmetric.
// rd = kOmega / D is stored per level; the second sweep scales it by
// kOmega2 / kOmega.  The two weights are the reciprocals of the roots of the
// degree-2 Chebyshev polynomial on [0.6, 2] (D^-1 A of these zero-row-sum
// M-matrices has its spectrum in [0, 2]): the pair damps the upper part of
// the spectrum more than two sweeps of one weight.  Measured on the 128^3
// cavity against 0.8 / 0.8: 2% less time per outer iteration, FP64 and
// mixed alike (Chebyshev on [0.5, 2] 1%, [0.4, 2] 1% more; a coarse
// over-correction of 2 instead of 3: 22% more).
constexpr double kOmega = 0.557;   // first sweep
constexpr double kOmega2 = 1.242;  // second sweep
constexpr double kOverCorrect = 3.0;   // scaling of the prolongated coarse correction
constexpr int kG = 8;                  // lanes per row on the small coarse levels
constexpr int kGroupedRows = 65536;    // levels below this many rows (per case) run grouped
constexpr int kTailRows = 2048;        // a case's levels at or below this many rows run in its V-cycle tail
constexpr int kTailThreads = 1024;     // threads of the tail's one CTA per case
enum { CNT_A0 = 9, CNT_A1, CNT_A2, CNT_A3, CNT_A4, CNT_A5 };

template <class T> struct LP {
    int n, W;
    const int *nb;
    const T *a, *dg, *rd;   // rd = omega / diagonal (the damped Jacobi scaling)
    T *r, *z, *t;
    const int *len;         // coarse levels: valid slots of each row, packed first (null on the mesh level)
    const short *nb16;      // mesh level: the neighbours as 16-bit offsets (CaseDev::nb16), or null
};

template <class T> __device__ __forceinline__ LP<T> level(const CaseDev &C, int l);
template <> __device__ __forceinline__ LP<double> level<double>(const CaseDev &C, int l) {
    if (l == 0) return {C.ne, C.W, C.hf_nb, C.anb_p, C.ap_p, C.rap_p, C.kr, C.ks, C.ksh, nullptr, C.nb16};
    const AmgLevelDev &L = C.lev[l - 1];
    return {L.n, L.W, L.nb, L.a, L.dg, L.rd, L.r, L.z, L.t, L.len, nullptr};
}
template <> __device__ __forceinline__ LP<float> level<float>(const CaseDev &C, int l) {
    if (l == 0) return {C.ne, C.W, C.hf_nb, C.fanb_p, C.fdiag_p, C.frap_p, C.fr, C.fz, C.ft, nullptr, C.nb16};
    const AmgLevelDev &L = C.lev[l - 1];
    return {L.n, L.W, L.nb, L.a32, L.dg32, L.rd32, L.r32, L.z32, L.t32, L.len, nullptr};
}

// (A x)_i at a level; neighbours outside [0, n) (halos, padding) are skipped
template <class T> __device__ __forceinline__ T amul(const LP<T> &P, const T *x, int i) {
    T y[1];
    ell_row<1, T>(P.nb, P.a, P.dg[i], x, 0, P.n, P.W, i, y);
    return y[0];
}
// A thread's rows of a wide tile, two per step: rows i0 and i1, with ok0 and
// ok1 false past the tile's end.  The CG kernels issue both rows' loads
// before either row's stores: a store holds back every load after it (the
// compiler cannot tell that they do not alias), so one row per step made
// each row its own trip to memory.  Sums still run in row order.
#define FOR_ROW_PAIRS(t)                                                                            \
    for (int j_ = 0, i0 = (t).first + (int)threadIdx.x; j_ < (t).pad; j_ += 2, i0 += 2 * kTile)     \
        if (const int i1 = i0 + kTile, ok0 = i0 < (t).last, ok1 = j_ + 1 < (t).pad && i1 < (t).last; \
            true)

template <class T, bool k16> __device__ __forceinline__ T amul_mesh(const LP<T> &P, const T *x, int i);

// CG's q = A p over a thread's rows of a wide tile, returning its share of
// (p, q), two rows per step
template <class T, bool k16>
__device__ __forceinline__ T cg_aq_rows(const LP<T> &P, const T *p, T *q, const Tile &t) {
    T v = 0;
    FOR_ROW_PAIRS(t) {
        T q0 = 0, q1 = 0, p0 = 0, p1 = 0;
        // the int32 form keeps amul's guarded coefficient loads (measured
        // faster in these multi-row tiles than the mesh sweeps' eager ones)
        if (ok0) { q0 = k16 ? amul_mesh<T, true>(P, p, i0) : amul<T>(P, p, i0); p0 = p[i0]; }
        if (ok1) { q1 = k16 ? amul_mesh<T, true>(P, p, i1) : amul<T>(P, p, i1); p1 = p[i1]; }
        if (ok0) { q[i0] = q0; v += p0 * q0; }
        if (ok1) { q[i1] = q1; v += p1 * q1; }
    }
    return v;
}
// CG's (r, z), two rows per step
template <class T>
__device__ __forceinline__ T cg_rz_rows(const T *r, const T *z, const Tile &t) {
    T v = 0;
    FOR_ROW_PAIRS(t) {
        T r0 = 0, z0 = 0, r1 = 0, z1 = 0;
        if (ok0) { r0 = r[i0]; z0 = z[i0]; }
        if (ok1) { r1 = r[i1]; z1 = z[i1]; }
        if (ok0) v += r0 * z0;
        if (ok1) v += r1 * z1;
    }
    return v;
}
// CG's p = z (first iteration) or z + beta p, two rows per step
template <class T>
__device__ __forceinline__ void cg_p_rows(const T *z, T *p, bool first, T beta, const Tile &t) {
    FOR_ROW_PAIRS(t) {
        T z0 = 0, p0 = 0, z1 = 0, p1 = 0;
        if (ok0) { z0 = z[i0]; if (!first) p0 = p[i0]; }
        if (ok1) { z1 = z[i1]; if (!first) p1 = p[i1]; }
        if (ok0) p[i0] = first ? z0 : z0 + beta * p0;
        if (ok1) p[i1] = first ? z1 : z1 + beta * p1;
    }
}
// CG's x += alpha p; r -= alpha q, returning the share of (r, r), two rows
// per step
template <class T>
__device__ __forceinline__ T cg_x_rows(T *x, const T *p, T *r, const T *q, T a, const Tile &t) {
    T v = 0;
    FOR_ROW_PAIRS(t) {
        T x0 = 0, p0 = 0, r0 = 0, q0 = 0, x1 = 0, p1 = 0, r1 = 0, q1 = 0;
        if (ok0) { x0 = x[i0]; p0 = p[i0]; r0 = r[i0]; q0 = q[i0]; }
        if (ok1) { x1 = x[i1]; p1 = p[i1]; r1 = r[i1]; q1 = q[i1]; }
        if (ok0) { x[i0] = x0 + a * p0; const T rr = r0 - a * q0; r[i0] = rr; v += rr * rr; }
        if (ok1) { x[i1] = x1 + a * p1; const T rr = r1 - a * q1; r[i1] = rr; v += rr * rr; }
    }
    return v;
}
// Slots of a wide coarse row taken per step, their index, coefficient and
// vector loads issued together (sums stay in slot order): 8 for the FP32
// levels, 4 for FP64, where 8 took the sweeps from 48 to 64 registers and
// measured slower (the FP32 sweeps and tail measured 5-15% faster at 8)
template <class T> __host__ __device__ constexpr int coarse_chunk() { return sizeof(T) == 4 ? 8 : 4; }
// the same on a coarse level, over the row's valid slots only (the padding
// slots would subtract zero terms): kCh slots per step
template <class T> __device__ __forceinline__ T amul_coarse(const LP<T> &P, const T *x, int i) {
    if (P.W == 6 || P.W == 4 || !P.len) return amul<T>(P, x, i);
    constexpr int kCh = coarse_chunk<T>();
    const int len = P.len[i];
    T y = P.dg[i] * x[i];
    for (int k0 = 0; k0 < len; k0 += kCh) {
        int jj[kCh];
        T ak[kCh], xv[kCh];
#pragma unroll
        for (int u = 0; u < kCh; u++) jj[u] = k0 + u < len ? P.nb[(k0 + u) * P.n + i] : -1;
#pragma unroll
        for (int u = 0; u < kCh; u++) {
            const bool ok = (unsigned)jj[u] < (unsigned)P.n;
            ak[u] = ok ? P.a[(k0 + u) * P.n + i] : (T)0;
            if (!ok) jj[u] = i;
        }
#pragma unroll
        for (int u = 0; u < kCh; u++) xv[u] = x[jj[u]];
#pragma unroll
        for (int u = 0; u < kCh; u++) y -= ak[u] * xv[u];
    }
    return y;
}

// The first W slots of row i: neighbour j[k] (i itself for a slot outside
// [0, n)) and coefficient c[k] (0 there).  The coefficient's address does not
// depend on the index, so both loads are issued together: a load guarded by
// the index would wait for it, a second memory latency in the row's chain.
// kGuard: the row has P.W <= W slots (the mesh level, W = kMaxW); slots past
// P.W are not read.  kEager false: the coefficient load waits for the index
// (the coarse levels' kernels, where that form measured faster).
template <int W, class T, bool kGuard, bool kEager = true, bool k16 = false>
__device__ __forceinline__ void row_slots(const LP<T> &P, int i, int (&j)[W], T (&c)[W]) {
#pragma unroll
    for (int k = 0; k < W; k++) {
        const bool in = !kGuard || k < P.W;
        int jj;
        if (k16) {      // the mesh level's 16-bit offsets: half the index bytes
            const int d = in ? (int)P.nb16[k * P.n + i] : (int)kNb16None;
            jj = d == (int)kNb16None ? -1 : i + d;
        } else {
            jj = in ? P.nb[k * P.n + i] : -1;
        }
        const bool ok = (unsigned)jj < (unsigned)P.n;
        j[k] = ok ? jj : i;
        if (kEager) {
            const T ak = in ? P.a[k * P.n + i] : (T)0;
            c[k] = ok ? ak : (T)0;
        } else {
            c[k] = ok ? P.a[k * P.n + i] : (T)0;
        }
    }
}

// The vector a sweep reads: a stored one, or t = w D^-1 r formed on the fly
// for the first pre-smoothing sweep (the product k_v_jac0 would store; the
// same multiplication, so the same values)
template <class T> struct VecIn {
    const T *x;
    __device__ __forceinline__ T operator()(int j) const { return x[j]; }
};
template <class T> struct VecRdR {
    const T *rd, *r;
    __device__ __forceinline__ T operator()(int j) const { return rd[j] * r[j]; }
};

// sum_j a_ij x_j over the row's couplings inside the level (the ELL values
// are the off-diagonal magnitudes: A = D - offdiag)
template <int W, class T, bool kGuard = false, bool kEager = true, bool k16 = false, class X>
__device__ __forceinline__ T offsum_w(const LP<T> &P, const X &xv, int i) {
    int j[W];
    T c[W];
    row_slots<W, T, kGuard, kEager, k16>(P, i, j, c);
    T xj[W];
#pragma unroll
    for (int k = 0; k < W; k++) xj[k] = xv(j[k]);
    T s = 0;
#pragma unroll
    for (int k = 0; k < W; k++) s += c[k] * xj[k];
    return s;
}

// The mesh level (level 0): at most kMaxW slots a row, every width on the
// short fixed-width paths (no wide-row code in the kernels that use these)
// k16: the level's neighbours are read from P.nb16 (every case of the launch has them)
template <class T, bool k16, class X> __device__ __forceinline__ T offsum_mesh(const LP<T> &P, const X &x, int i) {
    if (P.W == 6) return offsum_w<6, T, false, true, k16>(P, x, i);
    if (P.W == 4) return offsum_w<4, T, false, true, k16>(P, x, i);
    return offsum_w<kMaxW, T, true, true, k16>(P, x, i);
}
template <int W, class T, bool kGuard = false, bool k16 = false> __device__ __forceinline__ T amul_w(const LP<T> &P, const T *x, int i) {
    int j[W];
    T c[W];
    row_slots<W, T, kGuard, true, k16>(P, i, j, c);
    T s = P.dg[i] * x[i];
#pragma unroll
    for (int k = 0; k < W; k++) s -= c[k] * x[j[k]];
    return s;
}
template <class T, bool k16> __device__ __forceinline__ T amul_mesh(const LP<T> &P, const T *x, int i) {
    if (P.W == 6) return amul_w<6, T, false, k16>(P, x, i);
    if (P.W == 4) return amul_w<4, T, false, k16>(P, x, i);
    return amul_w<kMaxW, T, true, k16>(P, x, i);
}
// Valid slots of row i: a coarse row's couplings are packed in its first
// len[i] slots (the rest is padding up to the level's widest row, W).
template <class T> __device__ __forceinline__ int row_len(const LP<T> &P, int i) {
    return P.len ? P.len[i] : P.W;
}

template <class T, class X> __device__ __forceinline__ T offsum_x(const LP<T> &P, const X &x, int i) {
    if (P.W == 6) return offsum_w<6, T, false, false>(P, x, i);
    if (P.W == 4) return offsum_w<4, T, false, false>(P, x, i);
    constexpr int kCh = coarse_chunk<T>();
    // wide coarse rows: kCh slots per step, loads issued together,
    // up to the row's own length (the padding would add zero terms)
    T s = 0;
    const int len = row_len(P, i);
    for (int k0 = 0; k0 < len; k0 += kCh) {
        int jj[kCh];
        T c[kCh], xv[kCh];
#pragma unroll
        for (int u = 0; u < kCh; u++) jj[u] = k0 + u < len ? P.nb[(k0 + u) * P.n + i] : -1;
#pragma unroll
        for (int u = 0; u < kCh; u++) {
            const bool ok = (unsigned)jj[u] < (unsigned)P.n;
            c[u] = ok ? P.a[(k0 + u) * P.n + i] : (T)0;
            xv[u] = x(ok ? jj[u] : i);
        }
#pragma unroll
        for (int u = 0; u < kCh; u++) s += c[u] * xv[u];
    }
    return s;
}
template <class T> __device__ __forceinline__ T offsum(const LP<T> &P, const T *x, int i) {
    return offsum_x<T>(P, VecIn<T>{x}, i);
}

// damped Jacobi sweep from x: x + w D^-1 (r - A x) = (1 - w) x + (w/D)(r + offsum);
// kSweep 1 with w = kOmega (wrd = rd as stored), 2 with w = kOmega2
template <class T, int kSweep = 2> __device__ __forceinline__ T jacobi_step(T x, T r, T wrd, T off) {
    if (kSweep == 1) return (T)(1.0 - kOmega) * x + wrd * (r + off);
    return (T)(1.0 - kOmega2) * x + (wrd * (T)(kOmega2 / kOmega)) * (r + off);
}

__device__ __forceinline__ bool pactive(const CaseDev &C) { return C.sc->active_p != 0; }
__device__ __forceinline__ bool mactive(const CaseDev &C) { return C.sc->active32 != 0; }

// ------------------------------------------------------------ Galerkin
// Coarse row I of A_c = P^T A P for unsmoothed aggregation (k_amg_galg below):
// each off-diagonal slot is the sum of the fine couplings between aggregate I
// and its neighbour, in a fixed order.  The pressure-correction matrix has
// zero row sums (calc_coef_p: ap = sum of anb), and so has A_c, whose
// diagonal is therefore the sum of its row's off-diagonal couplings -- no
// pass over the aggregate's members or its internal couplings.

// level-0 diagonal inverse and the FP32 copies the mixed form needs
__global__ void __launch_bounds__(kTile) k_amg_prep0(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    const int i = t.first + (int)threadIdx.x;
    if (i >= t.last || C.sc->halted) return;
    const double ap = C.ap_p[i];
    const bool mixed = C.precision >= 1;
    // the row's loads before its stores (a store holds back the loads after it)
    double a[kMaxW];
#pragma unroll
    for (int k = 0; k < kMaxW; k++) a[k] = mixed && k < C.W ? C.anb_p[k * C.ne + i] : 0.0;
    const double rd = kOmega / ap;
    C.rap_p[i] = rd;
    if (mixed) {
        // the FP32 copies converted in the integer pipe (GB300 runs the hardware
        // conversions at its FP64 rate)
        C.fdiag_p[i] = narrow_f32(ap);
        C.frap_p[i] = narrow_f32(rd);
#pragma unroll
        for (int k = 0; k < kMaxW; k++)
            if (k < C.W) C.fanb_p[k * C.ne + i] = narrow_f32(a[k]);
    }
}

// Dense inverse of A_L + c 11^T at each case's coarsest level (one CTA per
// case, Gauss-Jordan in shared memory; the matrix is SPD, no pivoting).  Per
// pivot k, the first n threads scale the pivot row into R (R[k] = 1/p, one
// division per column: FP64 division is a long instruction sequence on a
// single SM's FP64 pipe) and save the pivot column into Q; after a barrier
// every thread updates its own entries (up to four: n <= 64, so
// n^2 <= 4 * kInvThreads) from M, Q and R alone, so the update is in place;
// a second barrier ends the pivot.
constexpr int kInvThreads = 1024;
__global__ void __launch_bounds__(kInvThreads) k_amg_coarse_inv(const CaseDev *__restrict__ cases, int ncases) {
    CFDL_PDL_WAIT();
    const int c = blockIdx.x;
    if (c >= ncases) return;
    const CaseDev &C = cases[c];
    if (C.precond != 1 || C.sc->halted) return;
    __shared__ double M[kAmgCoarsest * kAmgCoarsest];
    __shared__ double R[kAmgCoarsest], Q[kAmgCoarsest];
    const LP<double> P = level<double>(C, C.nlev);
    const int n = P.n;
    if (n > kAmgCoarsest) return;   // cannot happen: the builder coarsens to <= kAmgCoarsest
    double dmax = 0.0;
    for (int i = 0; i < n; i++) dmax = fmax(dmax, fabs(P.dg[i]));
    const double cc = dmax > 0.0 ? dmax / n : 1.0;
    constexpr int kPer = kAmgCoarsest * kAmgCoarsest / kInvThreads;
    int ei[kPer], ej[kPer];
#pragma unroll
    for (int q = 0; q < kPer; q++) {
        const int e = (int)threadIdx.x + q * kInvThreads;
        ei[q] = e < n * n ? e / n : -1;
        ej[q] = e < n * n ? e % n : -1;
        if (ei[q] >= 0) M[e] = cc + (ei[q] == ej[q] ? P.dg[ei[q]] : 0.0);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        for (int k = 0; k < P.W; k++) {
            const int j = P.nb[k * n + e];
            if (j >= 0 && j < n) M[e * n + j] -= P.a[k * n + e];
        }
    }
    __syncthreads();
    for (int k = 0; k < n; k++) {
        const int t = (int)threadIdx.x;
        if (t < n) {
            const double p = M[k * n + k];
            R[t] = (t == k ? 1.0 : M[k * n + t]) / p;     // the pivot row, scaled
            Q[t] = M[t * n + k];                          // the pivot column, before the update
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kPer; q++) {
            const int i = ei[q], j = ej[q];
            if (i < 0) continue;
            double &m = M[i * n + j];
            if (i == k) m = R[j];
            else if (j == k) m = -Q[i] * R[k];
            else m -= Q[i] * R[j];
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < kPer; q++) {
        if (ei[q] < 0) continue;
        const int e = ei[q] * n + ej[q];
        C.cinv[e] = M[e];
        if (C.precision >= 1) C.cinv32[e] = (float)M[e];
    }
}

// ------------------------------------------------------------ V-cycle
// t = w D^-1 r
template <class T>
__global__ void __launch_bounds__(kTile) k_v_jac0(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    const Tile tl = tiles[blockIdx.x];
    const CaseDev &C = cases[tl.c];
    if (sizeof(T) == 8 ? !pactive(C) : !mactive(C)) return;
    const int i = tl.first + (int)threadIdx.x;
    if (i >= tl.last) return;
    const LP<T> P = level<T>(C, l);
    P.t[i] = P.rd[i] * P.r[i];
}

// z = t + w D^-1 (r - A t).  kMesh: launched on the mesh level only.
// kToT: the sweep from z into t instead (the first post-smoothing sweep,
// after k_v_lift has added the prolongated coarse correction to z).
// kFromR: the first pre-smoothing sweep, from t = w D^-1 r formed on the fly
// for the row and its neighbours instead of read from k_v_jac0's pass (the
// same products, so the same z; one pass over the level fewer)
template <class T, bool kMesh, bool kToT, bool kFromR = false, bool k16 = false>
__device__ __forceinline__ void v_jac_row(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    const Tile tl = tiles[blockIdx.x];
    const CaseDev &C = cases[tl.c];
    if (sizeof(T) == 8 ? !pactive(C) : !mactive(C)) return;
    const int i = tl.first + (int)threadIdx.x;
    if (i >= tl.last) return;
    const LP<T> P = level<T>(C, l);
    if (kFromR) {
        const VecRdR<T> tv{P.rd, P.r};
        const T ri = P.r[i], rdi = P.rd[i];
        const T off = kMesh ? offsum_mesh<T, k16>(P, tv, i) : offsum_x<T>(P, tv, i);
        P.z[i] = jacobi_step<T, 2>(rdi * ri, ri, rdi, off);
        return;
    }
    const T *x = kToT ? P.z : P.t;
    T *y = kToT ? P.t : P.z;
    if (kMesh) {
        const T off = offsum_mesh<T, k16>(P, VecIn<T>{x}, i);
        y[i] = jacobi_step<T, kToT ? 1 : 2>(x[i], P.r[i], P.rd[i], off);
    } else {
        // the row's own values first: measured faster on the coarse levels
        y[i] = jacobi_step<T, kToT ? 1 : 2>(x[i], P.r[i], P.rd[i], offsum<T>(P, x, i));
    }
}
template <class T, bool kToT = false, bool kFromR = false>
__global__ void __launch_bounds__(kTile) k_v_jac(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    v_jac_row<T, false, kToT, kFromR>(cases, tiles, l);
}
// The mesh-level sweeps (one row per thread, two dependent trips to memory
// a row) are kernels of their own, so that their register cap, and with it
// the resident warps and the loads in flight, is set apart from the coarse
// levels' sweeps: 32 registers, 8 CTAs per SM (the FP64 forms keep one
// 8-byte spill slot), measured 2-4% faster at 128^3 than the 40 registers
// and 6 CTAs the compiler picks unbounded; the coarse sweeps would spill
// 100+ bytes under the same cap.
template <class T, bool k16, bool kToT = false, bool kFromR = false>
__global__ void __launch_bounds__(kTile, 8) k_v_jac_mesh(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    v_jac_row<T, true, kToT, kFromR, k16>(cases, tiles, l);
}

// z = z + s P z_{l+1}: the prolongated coarse correction, added in place.
// With it as its own streaming pass, the sweep after it gathers each
// neighbour's corrected value once instead of the neighbour's aggregate and
// then the coarse value: the same values, a shorter load chain.
template <class T>
__global__ void __launch_bounds__(kTile) k_v_lift(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    const Tile tl = tiles[blockIdx.x];
    const CaseDev &C = cases[tl.c];
    if (sizeof(T) == 8 ? !pactive(C) : !mactive(C)) return;
    const int i = tl.first + (int)threadIdx.x;
    if (i >= tl.last) return;
    const LP<T> P = level<T>(C, l);
    const AmgLevelDev &L = C.lev[l];
    const T *zc = sizeof(T) == 8 ? (const T *)L.z : (const T *)L.z32;
    P.z[i] = P.z[i] + (T)kOverCorrect * zc[L.agg[i]];
}

// t = r - A z (the smoothed residual, one thread per cell, coalesced)
template <class T, bool kMesh, bool k16 = false>
__device__ __forceinline__ void v_resid_row(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    const Tile tl = tiles[blockIdx.x];
    const CaseDev &C = cases[tl.c];
    if (sizeof(T) == 8 ? !pactive(C) : !mactive(C)) return;
    const int i = tl.first + (int)threadIdx.x;
    if (i >= tl.last) return;
    const LP<T> P = level<T>(C, l);
    P.t[i] = P.r[i] - (kMesh ? amul_mesh<T, k16>(P, P.z, i) : amul_coarse<T>(P, P.z, i));
}
template <class T>
__global__ void __launch_bounds__(kTile) k_v_resid(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    v_resid_row<T, false>(cases, tiles, l);
}
// the mesh level's residual, with the mesh sweeps' register cap
template <class T, bool k16>
__global__ void __launch_bounds__(kTile, 8) k_v_resid_mesh(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    v_resid_row<T, true, k16>(cases, tiles, l);
}

// sum of t over the members of aggregate I of the level below L: four
// members per step, their indices and then their values loaded side by side,
// summed in member order (one member per step made every member two
// dependent trips to memory)
template <class T>
__device__ __forceinline__ T restrict_row(const AmgLevelDev &L, const T *t, int I) {
    const int m0 = L.mem_ptr[I], m1 = L.mem_ptr[I + 1];
    T s = 0;
    for (int m = m0; m < m1; m += 4) {
        int j[4];
        T x[4];
#pragma unroll
        for (int u = 0; u < 4; u++) j[u] = m + u < m1 ? L.mem[m + u] : -1;
#pragma unroll
        for (int u = 0; u < 4; u++) x[u] = j[u] >= 0 ? t[j[u]] : (T)0;
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (j[u] >= 0) s += x[u];
    }
    return s;
}

// r_{l1}[I] = sum of the residual t over the members of aggregate I (one
// thread per coarse row: the large levels, where rows outnumber lanes)
template <class T>
__global__ void __launch_bounds__(kTile) k_v_restrict(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l1) {
    CFDL_PDL_WAIT();
    const Tile tl = tiles[blockIdx.x];
    const CaseDev &C = cases[tl.c];
    if (sizeof(T) == 8 ? !pactive(C) : !mactive(C)) return;
    const int I = tl.first + (int)threadIdx.x;
    if (I >= tl.last) return;
    const AmgLevelDev &L = C.lev[l1 - 1];
    const LP<T> F = level<T>(C, l1 - 1);
    T *rc = sizeof(T) == 8 ? (T *)L.r : (T *)L.r32;
    rc[I] = restrict_row<T>(L, F.t, I);
}

// Galerkin row I, one thread per row (large levels)
__global__ void __launch_bounds__(kTile) k_amg_gal(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    const int I = t.first + (int)threadIdx.x;
    if (I >= t.last || C.sc->halted) return;
    const AmgLevelDev &L = C.lev[l - 1];
    const double *af = l == 1 ? C.anb_p : C.lev[l - 2].a;
    const bool mixed = C.precision >= 1;
    const int n = L.n;
    double dsum = 0.0;
    // padding slots (k >= len) keep the zeros they were created with
    const int len = L.len[I];
    for (int k = 0; k < len; k++) {
        const int s = k * n + I;
        double v = 0.0;
        for (int q = L.g_ptr[s]; q < L.g_ptr[s + 1]; q++) v += af[L.g_src[q]];
        L.a[s] = v;
        if (mixed) L.a32[s] = narrow_f32(v);
        dsum += v;
    }
    L.dg[I] = dsum;
    L.rd[I] = kOmega / dsum;
    if (mixed) { L.dg32[I] = narrow_f32(dsum); L.rd32[I] = narrow_f32(kOmega / dsum); }
}

// ------------------------------------------------- the V-cycle's tail
// The small coarse levels of a case, from its tail level (the first level of
// at most kTailRows rows) down to the coarsest and back, in one CTA: the
// steps of k_v_jac0 / k_v_jac / k_v_resid / k_v_restrict, the coarsest solve
// and k_v_lift / k_v_jac, one row per thread per pass, with a block
// barrier between steps.  Each step is a few microseconds of dependent loads
// from L2; launched one by one, every step costs a kernel launch instead.
// The CTA waits only at __syncthreads, on its own threads.
template <class T>
__global__ void __launch_bounds__(kTailThreads) k_v_tail(const CaseDev *__restrict__ cases, int ncases) {
    CFDL_PDL_WAIT();
    const int c = blockIdx.x;
    if (c >= ncases) return;
    const CaseDev &C = cases[c];
    if (C.precond != 1 || (sizeof(T) == 8 ? !pactive(C) : !mactive(C))) return;
    const int L = C.nlev, lt = C.amg_tail, nt = (int)blockDim.x;
    for (int l = lt; l < L; l++) {
        const LP<T> P = level<T>(C, l);
        for (int i = threadIdx.x; i < P.n; i += nt) P.t[i] = P.rd[i] * P.r[i];
        __syncthreads();
        for (int i = threadIdx.x; i < P.n; i += nt) P.z[i] = jacobi_step<T>(P.t[i], P.r[i], P.rd[i], offsum<T>(P, P.t, i));
        __syncthreads();
        for (int i = threadIdx.x; i < P.n; i += nt) P.t[i] = P.r[i] - amul_coarse<T>(P, P.z, i);
        __syncthreads();
        const AmgLevelDev &Lc = C.lev[l];                  // level l + 1
        T *rc = sizeof(T) == 8 ? (T *)Lc.r : (T *)Lc.r32;
        for (int I = threadIdx.x; I < Lc.n; I += nt) rc[I] = restrict_row<T>(Lc, P.t, I);
        __syncthreads();
    }
    {   // coarsest: z_L = Minv r_L
        const LP<T> P = level<T>(C, L);
        const T *Mi = sizeof(T) == 8 ? (const T *)C.cinv : (const T *)C.cinv32;
        const int n = P.n;
        for (int i = threadIdx.x; i < n; i += nt) {
            T sum = 0;
            for (int j = 0; j < n; j++) sum += Mi[i * n + j] * P.r[j];
            P.z[i] = sum;
        }
        __syncthreads();
    }
    const T sc = (T)kOverCorrect;
    constexpr int kCh = coarse_chunk<T>();
    for (int l = L - 1; l >= lt; l--) {
        const LP<T> P = level<T>(C, l);
        const AmgLevelDev &Lc = C.lev[l];
        const T *zc = sizeof(T) == 8 ? (const T *)Lc.z : (const T *)Lc.z32;
        for (int i = threadIdx.x; i < P.n; i += nt) {
            const T xi = P.z[i] + sc * zc[Lc.agg[i]];
            // the neighbours' lifted values, kCh slots per step with
            // each step's loads issued together, summed in slot order
            T off = 0;
            const int len = row_len(P, i);
            for (int k0 = 0; k0 < len; k0 += kCh) {
                int jj[kCh], ag[kCh];
                bool ok[kCh];
                T ak[kCh], zj[kCh];
#pragma unroll
                for (int u = 0; u < kCh; u++) jj[u] = k0 + u < len ? P.nb[(k0 + u) * P.n + i] : -1;
#pragma unroll
                for (int u = 0; u < kCh; u++) {
                    ok[u] = (unsigned)jj[u] < (unsigned)P.n;
                    ak[u] = ok[u] ? P.a[(k0 + u) * P.n + i] : (T)0;
                    zj[u] = ok[u] ? P.z[jj[u]] : (T)0;
                    ag[u] = ok[u] ? Lc.agg[jj[u]] : 0;
                }
#pragma unroll
                for (int u = 0; u < kCh; u++)
                    if (ok[u]) off += ak[u] * (zj[u] + sc * zc[ag[u]]);
            }
            P.t[i] = jacobi_step<T, 1>(xi, P.r[i], P.rd[i], off);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < P.n; i += nt) P.z[i] = jacobi_step<T>(P.t[i], P.r[i], P.rd[i], offsum<T>(P, P.t, i));
        __syncthreads();
    }
}

// ------------------------------------------------- coarse levels, grouped
// Coarse rows are wide (up to ~30 couplings) and a thread that walked one
// alone would issue its index -> value -> vector loads one slot after the
// other: a chain of dependent loads that left the small levels latency-bound.
// On small levels each row is handled by G lanes that split its slots (and
// the Galerkin and restriction gather lists) and combine their partial sums
// with shuffles, in a fixed order.  Tiles hold kTile / G rows.
#define GROUP_HEAD                                                   \
    const Tile tl = tiles[blockIdx.x];                               \
    const CaseDev &C = cases[tl.c];                                  \
    const int g = (int)threadIdx.x & (G - 1);                        \
    const int i = tl.first + (int)threadIdx.x / G;                   \
    const bool ok = i < tl.last;

template <int G, class T> __device__ __forceinline__ T group_sum(T v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// sum_k a_ik x_j over the row's couplings inside the level, split over the group
template <int G, class T> __device__ __forceinline__ T group_offdiag(const LP<T> &P, const T *x, int i, bool ok, int g) {
    T s = 0;
    if (ok) {
        const int len = row_len(P, i);
        for (int k = g; k < len; k += G) {
            const int j = P.nb[k * P.n + i];
            if ((unsigned)j < (unsigned)P.n) s += P.a[k * P.n + i] * x[j];
        }
    }
    return group_sum<G>(s);
}

// z = t + w D^-1 (r - A t)
template <class T, int G>
__global__ void __launch_bounds__(kTile) k_vg_jac(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    GROUP_HEAD
    if (sizeof(T) == 8 ? !pactive(C) : !mactive(C)) return;
    const LP<T> P = level<T>(C, l);
    const T off = group_offdiag<G, T>(P, P.t, i, ok, g);
    if (ok && g == 0) P.z[i] = jacobi_step<T>(P.t[i], P.r[i], P.rd[i], off);
}

// t = r - A z
template <class T, int G>
__global__ void __launch_bounds__(kTile) k_vg_resid(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    GROUP_HEAD
    if (sizeof(T) == 8 ? !pactive(C) : !mactive(C)) return;
    const LP<T> P = level<T>(C, l);
    const T off = group_offdiag<G, T>(P, P.z, i, ok, g);
    if (ok && g == 0) P.t[i] = P.r[i] - (P.dg[i] * P.z[i] - off);
}

// r_{l1}[I] = sum of the residual t_{l1-1} over the members of aggregate I
template <class T, int G>
__global__ void __launch_bounds__(kTile) k_vg_restrict(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l1) {
    CFDL_PDL_WAIT();
    GROUP_HEAD
    if (sizeof(T) == 8 ? !pactive(C) : !mactive(C)) return;
    const AmgLevelDev &L = C.lev[l1 - 1];
    const LP<T> F = level<T>(C, l1 - 1);
    T s = 0;
    if (ok)
        for (int m = L.mem_ptr[i] + g; m < L.mem_ptr[i + 1]; m += G) s += F.t[L.mem[m]];
    s = group_sum<G>(s);
    T *rc = sizeof(T) == 8 ? (T *)L.r : (T *)L.r32;
    if (ok && g == 0) rc[i] = s;
}

// t = x + w D^-1 (r - A x) with x = z + s P z_{l+1}
template <class T, int G>
__global__ void __launch_bounds__(kTile) k_vg_prolong(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    GROUP_HEAD
    if (sizeof(T) == 8 ? !pactive(C) : !mactive(C)) return;
    const LP<T> P = level<T>(C, l);
    const AmgLevelDev &L = C.lev[l];
    const T *zc = sizeof(T) == 8 ? (const T *)L.z : (const T *)L.z32;
    const T sc = (T)kOverCorrect;
    T off = 0;
    if (ok) {
        const int len = row_len(P, i);
        for (int k = g; k < len; k += G) {
            const int j = P.nb[k * P.n + i];
            if ((unsigned)j < (unsigned)P.n) off += P.a[k * P.n + i] * (P.z[j] + sc * zc[L.agg[j]]);
        }
    }
    off = group_sum<G>(off);
    if (ok && g == 0) {
        const T xi = P.z[i] + sc * zc[L.agg[i]];
        P.t[i] = jacobi_step<T, 1>(xi, P.r[i], P.rd[i], off);
    }
}

// Galerkin row I of level l: each lane sums the gather lists of its slots
template <int G>
__global__ void __launch_bounds__(kTile) k_amg_galg(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int l) {
    CFDL_PDL_WAIT();
    GROUP_HEAD
    if (C.sc->halted) return;
    const AmgLevelDev &L = C.lev[l - 1];
    const double *af = l == 1 ? C.anb_p : C.lev[l - 2].a;
    const bool mixed = C.precision >= 1;
    const int n = L.n;
    double dsum = 0.0;
    if (ok)
        for (int k = g, len = L.len[i]; k < len; k += G) {
            const int sl = k * n + i;
            double v = 0.0;
            for (int q = L.g_ptr[sl]; q < L.g_ptr[sl + 1]; q++) v += af[L.g_src[q]];
            L.a[sl] = v;
            if (mixed) L.a32[sl] = narrow_f32(v);
            dsum += v;
        }
    dsum = group_sum<G>(dsum);
    if (ok && g == 0) {
        L.dg[i] = dsum;
        L.rd[i] = kOmega / dsum;
        if (mixed) { L.dg32[i] = narrow_f32(dsum); L.rd32[i] = narrow_f32(kOmega / dsum); }
    }
}

// ------------------------------------------------------------ CG (FP64)
// r = b - mean, x = 0; ||r0||
__global__ void __launch_bounds__(kTile) k_apc_init(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                    const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (S->halted) return;
    double v[2] = {0, 0};
    FOR_CELLS(t) {
        const double r = C.b[i] - S->mean_b;
        C.kr[i] = r; C.phic[i] = 0.0;
        v[0] += r * r; v[1] += C.b[i] * C.b[i];
    }
    block_reduce<2>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_A0], cnt[t.c])) {
        __shared__ double s[2];
        sum_partials<2>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            const int cap = C.solve_mode == 0 ? C.nit : C.tight_maxit;
            S->r0norm_p = S->rnorm_p = sqrt(s[0]);
            S->mass_imbalance = sqrt(s[1]);
            S->iters_p = 0; S->status_p = 0; S->rz = 0.0;
            S->tol_p = (C.solve_mode == 0 ? C.rtol_p : C.tight_rtol) * S->r0norm_p;
            S->active_p = S->r0norm_p > S->tol_p && cap > 0;
            if (!isfinite(S->r0norm_p)) { S->active_p = 0; S->status_p = CFDL_ERR_NONFINITE; }
        }
    }
}

// beta = (r,z)/(r,z)_old (0 on the first iteration)
__global__ void __launch_bounds__(kTile) k_apc_rz(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                  const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (!S->active_p) return;
    // one row per step in FP64: the paired form (cg_rz_rows) measured slower
    // here (21.4 against 18.8 us a launch at 128^3)
    double v[1] = {0.0};
    FOR_CELLS(t) v[0] += C.kr[i] * C.ks[i];
    block_reduce<1>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_A1], cnt[t.c])) {
        __shared__ double s[1];
        sum_partials<1>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            S->beta_p = S->iters_p == 0 || S->rz == 0.0 ? 0.0 : s[0] / S->rz;
            S->rz = s[0];
            if (!isfinite(s[0])) { S->active_p = 0; S->status_p = CFDL_ERR_NONFINITE; }
        }
    }
}

// p = z + beta p; q = A p needs every p, so it is the next kernel
__global__ void __launch_bounds__(kTile) k_apc_p(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    const SolveScalars *S = C.sc;
    if (!S->active_p) return;
    cg_p_rows<double>(C.ks, C.kp, S->iters_p == 0, S->beta_p, t);
}

// q = A p; alpha = rz / (p, q)
__global__ void __launch_bounds__(kTile) k_apc_q(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                 const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (!S->active_p) return;
    double v[1] = {cg_aq_rows<double, false>(level<double>(C, 0), C.kp, C.kv, t)};
    block_reduce<1>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_A2], cnt[t.c])) {
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

// x += alpha p; r -= alpha q; ||r||
__global__ void __launch_bounds__(kTile) k_apc_x(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                 const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (!S->active_p) return;
    // one row per step in FP64: the paired form (cg_x_rows, 48 registers
    // against 32) measured slower here (31.9 against 28.5 us a launch)
    double v[1] = {0};
    FOR_CELLS(t) {
        const double a = S->alpha_p;
        C.phic[i] = C.phic[i] + a * C.kp[i];
        const double r = C.kr[i] - a * C.kv[i];
        C.kr[i] = r;
        v[0] += r * r;
    }
    block_reduce<1>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_A3], cnt[t.c])) {
        __shared__ double s[1];
        sum_partials<1>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            const int cap = C.solve_mode == 0 ? C.nit : C.tight_maxit;
            const double rn = sqrt(s[0]);
            S->rnorm_p = rn;
            S->iters_p += 1;
            int act = rn > S->tol_p;
            if (!isfinite(rn)) { act = 0; S->status_p = CFDL_ERR_NONFINITE; }
            else if (act && S->iters_p >= cap) { act = 0; if (C.solve_mode == 1) S->status_p = CFDL_ERR_ITER_CAP; }
            S->active_p = act;
        }
    }
}

// the mesh level's neighbour offsets for CaseDev::nb16; overflow is set when
// an offset does not fit in 16 bits
__global__ void k_nb16(const int *__restrict__ nb, short *__restrict__ out, int ne, int W, unsigned *overflow) {
    const size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (s >= (size_t)W * ne) return;
    const int i = (int)(s % (size_t)ne);
    const int j = nb[s];
    short v = kNb16None;
    if (j >= 0 && j < ne) {
        const int d = j - i;
        if (d < -32767 || d > 32767) atomicOr(overflow, 1u);
        else v = (short)d;
    }
    out[s] = v;
}

}  // namespace

// ------------------------------------------------------------------ host
namespace {

template <class T, class A> int dupload(HostCase *hc, T **d, const std::vector<T, A> &h) {
    size_t bytes = std::max<size_t>(1, h.size()) * sizeof(T);
    cudaError_t e = cudaMalloc((void **)d, bytes);
    if (e != cudaSuccess) { cudaGetLastError(); return cuda_status(e); }
    hc->amg_allocs.push_back(*d);
    hc->bytes += bytes;
    if (h.empty()) return CFDL_OK;
    return cuda_status(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}
template <class T> int dzeros(HostCase *hc, T **d, size_t n) {
    cudaError_t e = cudaMalloc((void **)d, std::max<size_t>(1, n) * sizeof(T));
    if (e != cudaSuccess) { cudaGetLastError(); return cuda_status(e); }
    hc->amg_allocs.push_back(*d);
    hc->bytes += std::max<size_t>(1, n) * sizeof(T);
    return cuda_status(cudaMemset(*d, 0, std::max<size_t>(1, n) * sizeof(T)));
}

// strength of each ELL slot = |area/(dr.n)| of its face; -1 marks the slots
// that are not interior couplings
void amg_strength(int ne, int W, const int *nb_in, const int *fc, const double *adn, FillVec<int> &nb,
                  FillVec<double> &strength) {
    nb.resize((size_t)W * ne);          // every slot written below (first touch in parallel)
    strength.resize((size_t)W * ne);
    parallel_for((long)nb.size(), [&](long b, long e) {
        for (long s = b; s < e; s++) {
            const int j = nb_in[s];
            if (j < 0 || j >= ne) { nb[s] = -1; strength[s] = 0.0; continue; }
            const int f = fc[s] >= 0 ? fc[s] : ~fc[s];
            nb[s] = j;
            strength[s] = std::fabs(adn[f]);
        }
    });
}

// Build and upload the hierarchy of one case (mesh-only, once).
int build_case_amg(HostCase *hc) {
    if (hc->amg) return CFDL_OK;
    CaseDev &d = hc->dev;
    const int ne = hc->ne, W = hc->W, nf = hc->nf;
    // the slot tables and face planes, read back from the device
    std::vector<int> nb0((size_t)W * ne), fc((size_t)W * ne);
    std::vector<double> adn(nf);
    int st;
    if ((st = cuda_status(cudaMemcpy(nb0.data(), d.hf_nb, nb0.size() * sizeof(int), cudaMemcpyDeviceToHost)))) return st;
    if ((st = cuda_status(cudaMemcpy(fc.data(), d.hf_fc, fc.size() * sizeof(int), cudaMemcpyDeviceToHost)))) return st;
    if ((st = cuda_status(cudaMemcpy(adn.data(), d.fgeo + (size_t)FG_ADN * nf, nf * sizeof(double), cudaMemcpyDeviceToHost)))) return st;
    FillVec<int> nb;
    FillVec<double> strength;
    amg_strength(ne, W, nb0.data(), fc.data(), adn.data(), nb, strength);
    AmgHierarchy *H = new AmgHierarchy;
    AmgFineView fv{ne, W, nb.data(), strength.data()};
    if ((st = build_amg_hierarchy(fv, *H))) { delete H; return st; }
    return upload_case_amg(hc, H);
}

}  // namespace

int prepare_case_amg(CasePrep *p) {
    if (!p || p->amg) return p ? CFDL_OK : CFDL_ERR_INVALID;
    FillVec<int> nb;
    FillVec<double> strength;
    amg_strength(p->ne, p->W, p->hf_nb.data(), p->hf_fc.data(), p->fgeo.data() + (size_t)FG_ADN * p->nf, nb, strength);
    AmgHierarchy *H = new (std::nothrow) AmgHierarchy;
    if (!H) return CFDL_ERR_OOM;
    AmgFineView fv{p->ne, p->W, nb.data(), strength.data()};
    int st = build_amg_hierarchy(fv, *H);
    if (st) { delete H; return st; }
    p->amg = H;
    return CFDL_OK;
}

// Upload a host-built hierarchy into the case, which takes ownership of it.
int upload_case_amg(HostCase *hc, AmgHierarchy *H) {
    CaseDev &d = hc->dev;
    const int ne = hc->ne;
    int st;
    hc->amg = H;
    const int nlev = (int)H->levels.size();
    std::vector<AmgLevelDev> devl(nlev);
    for (int l = 0; l < nlev; l++) {
        const AmgHostLevel &L = H->levels[l];
        AmgLevelDev &D = devl[l];
        D.n = L.n; D.W = L.W; D.n_fine = L.n_fine; D.W_fine = L.W_fine;
        if ((st = dupload(hc, (int **)&D.nb, L.nb))) return st;
        if ((st = dupload(hc, (int **)&D.agg, L.agg))) return st;
        if ((st = dupload(hc, (int **)&D.mem_ptr, L.mem_ptr))) return st;
        if ((st = dupload(hc, (int **)&D.mem, L.mem))) return st;
        if ((st = dupload(hc, (int **)&D.g_ptr, L.g_ptr))) return st;
        if ((st = dupload(hc, (int **)&D.g_src, L.g_src))) return st;
        {
            // valid slots of each row: the builder packs a row's couplings first
            std::vector<int> len((size_t)L.n, 0);
            for (int k = 0; k < L.W; k++)
                for (int c = 0; c < L.n; c++)
                    if (L.nb[(size_t)k * L.n + c] >= 0) len[c] = k + 1;
            if ((st = dupload(hc, (int **)&D.len, len))) return st;
        }
        if ((st = dzeros(hc, &D.a, (size_t)L.W * L.n))) return st;
        if ((st = dzeros(hc, &D.a32, (size_t)L.W * L.n))) return st;
        double **v64[] = {&D.dg, &D.rd, &D.r, &D.z, &D.t};
        for (double **p : v64) if ((st = dzeros(hc, p, (size_t)L.n))) return st;
        float **v32[] = {&D.dg32, &D.rd32, &D.r32, &D.z32, &D.t32};
        for (float **p : v32) if ((st = dzeros(hc, p, (size_t)L.n))) return st;
    }
    AmgLevelDev *dlev = nullptr;
    if ((st = dupload(hc, &dlev, devl))) return st;
    const int ncoarse = nlev ? H->levels.back().n : ne;
    if (ncoarse > kAmgCoarsest) return CFDL_ERR_MESH;
    if ((st = dzeros(hc, &d.cinv, (size_t)ncoarse * ncoarse))) return st;
    if ((st = dzeros(hc, &d.cinv32, (size_t)ncoarse * ncoarse))) return st;
    if (hc->cfg.precision >= 1) {   // the FP32 mesh kernels' 16-bit neighbour offsets, used when every one fits
        const size_t nslot = (size_t)hc->W * ne;
        short *nb16 = nullptr;
        unsigned *flag = nullptr, over = 0;
        if ((st = dzeros(hc, &nb16, nslot)) || (st = dzeros(hc, &flag, 1))) return st;
        k_nb16<<<(unsigned)((nslot + kTile - 1) / kTile), kTile>>>(d.hf_nb, nb16, ne, hc->W, flag);
        if ((st = cuda_status(cudaGetLastError()))) return st;
        if ((st = cuda_status(cudaMemcpy(&over, flag, sizeof(unsigned), cudaMemcpyDeviceToHost)))) return st;
        d.nb16 = over ? nullptr : nb16;
    }
    d.nlev = nlev;
    d.ncoarse = ncoarse;
    d.lev = dlev;
    return CFDL_OK;
}


int ensure_amg(cfdl_ctx *ctx) {
    bool changed = false;
    for (HostCase *hc : ctx->cases) {
        if (!hc->amg) {
            int st = build_case_amg(hc);
            if (st) return st;
            changed = true;
        }
    }
    bool all16 = ctx->index16;
    for (HostCase *hc : ctx->cases) all16 = all16 && hc->dev.nb16 != nullptr;
    if (all16 != ctx->amg_nb16) { ctx->amg_nb16 = all16; destroy_graph(ctx); }
    if (!changed && ctx->amg_lmax >= 0) return CFDL_OK;
    int lmax = 0;
    for (HostCase *hc : ctx->cases) lmax = std::max(lmax, hc->dev.nlev);
    for (auto &wl : ctx->amg_cells) free_worklist(wl);
    for (auto &wl : ctx->amg_smooth) free_worklist(wl);
    for (auto &wl : ctx->amg_gcells) free_worklist(wl);
    for (auto &wl : ctx->amg_gsmooth) free_worklist(wl);
    for (auto &wl : ctx->amg_restr) free_worklist(wl);
    for (auto &wl : ctx->amg_grestr) free_worklist(wl);
    ctx->amg_cells.assign(lmax + 1, WorkList());
    ctx->amg_smooth.assign(lmax + 1, WorkList());
    ctx->amg_gcells.assign(lmax + 1, WorkList());
    ctx->amg_gsmooth.assign(lmax + 1, WorkList());
    ctx->amg_restr.assign(lmax + 1, WorkList());
    ctx->amg_grestr.assign(lmax + 1, WorkList());
    ctx->amg_grouped.assign(lmax + 1, 0);
    // each case's tail level: its first coarse level of at most kTailRows rows
    // (the coarsest always qualifies); a case without coarse levels solves its
    // mesh level directly (tail level 0)
    for (HostCase *hc : ctx->cases) {
        int lt = 0;
        for (int l = 1; l <= hc->dev.nlev; l++)
            if (hc->amg->levels[l - 1].n <= kTailRows) { lt = l; break; }
        hc->dev.amg_tail = lt;
    }
    for (int l = 0; l <= lmax; l++) {
        std::vector<int> cells, smooth, restr;
        for (HostCase *hc : ctx->cases) {
            int n = l == 0 ? hc->ne : (l <= hc->dev.nlev ? hc->amg->levels[l - 1].n : 0);
            cells.push_back(l <= hc->dev.nlev ? n : 0);
            smooth.push_back(l < hc->dev.amg_tail ? n : 0);
            restr.push_back(l >= 1 && l <= hc->dev.amg_tail ? n : 0);
        }
        int st;
        if ((st = build_worklist(ctx, ctx->amg_cells[l], cells))) return st;
        if ((st = build_worklist(ctx, ctx->amg_smooth[l], smooth))) return st;
        if ((st = build_worklist(ctx, ctx->amg_restr[l], restr))) return st;
        // lanes per row: 8 when every case's level is small, else the tuned
        // cgroup (1 = one thread per row); the mesh level is always 1
        const int nmax = *std::max_element(cells.begin(), cells.end());
        const int G = l == 0 ? 1 : nmax < kGroupedRows ? kG : ctx->cgroup;
        ctx->amg_grouped[l] = G;
        if (G > 1) {
            if ((st = build_worklist(ctx, ctx->amg_gcells[l], cells, kTile / G))) return st;
            if ((st = build_worklist(ctx, ctx->amg_gsmooth[l], smooth, kTile / G))) return st;
            if ((st = build_worklist(ctx, ctx->amg_grestr[l], restr, kTile / G))) return st;
        }
    }
    ctx->amg_lmax = lmax;
    return upload_case_table(ctx);
}

#define ALAUNCH(name, kern, WL, ...)                                                                 \
    do {                                                                                             \
        if ((WL).ntiles > 0) {                                                                       \
            const bool p_ = ctx->prof && prof_wants(ctx, name);                                      \
            if (p_) prof_begin(ctx, name);                                                           \
            launch_k(ctx->pdl, kern, (unsigned)(WL).ntiles, (unsigned)kTile, ctx->stream,                 \
                     (const CaseDev *)ctx->d_cases, (const Tile *)(WL).d_tiles, ##__VA_ARGS__);          \
            if (p_) prof_end(ctx);                                                                   \
            ctx->launches++;                                                                         \
        }                                                                                            \
    } while (0)
#define CLAUNCH(name, kern, threads)                                                                 \
    do {                                                                                             \
        const int nc_ = (int)ctx->cases.size();                                                      \
        const bool p_ = ctx->prof && prof_wants(ctx, name);                                          \
        if (p_) prof_begin(ctx, name);                                                               \
        launch_k(ctx->pdl, kern, (unsigned)nc_, (unsigned)(threads), ctx->stream,                    \
                 (const CaseDev *)ctx->d_cases, nc_);                                                \
        if (p_) prof_end(ctx);                                                                       \
        ctx->launches++;                                                                             \
    } while (0)

// Coarse operators of every level and the coarsest inverse.
static void amg_setup_operators(cfdl_ctx *ctx) {
    ALAUNCH("k_amg_prep0", k_amg_prep0, ctx->cells);
    for (int l = 1; l <= ctx->amg_lmax; l++) {
        switch (ctx->amg_grouped[l]) {
        case 8: ALAUNCH("k_amg_gal", k_amg_galg<8>, ctx->amg_gcells[l], l); break;
        case 4: ALAUNCH("k_amg_gal", k_amg_galg<4>, ctx->amg_gcells[l], l); break;
        case 2: ALAUNCH("k_amg_gal", k_amg_galg<2>, ctx->amg_gcells[l], l); break;
        default: ALAUNCH("k_amg_gal", k_amg_gal, ctx->amg_cells[l], l);
        }
    }
    CLAUNCH("k_amg_coarse_inv", k_amg_coarse_inv, kInvThreads);
}

// One V-cycle z_0 = M^-1 r_0 on every active case.
// The kernels of one coarse-level step at a group size (1: one thread per row)
#define GROUPED(NAME, K, WLG, WL1, ...)                                          \
    switch (G) {                                                                \
    case 8: { auto kf_ = K<T, 8>; ALAUNCH(NAME, kf_, WLG, ##__VA_ARGS__); } break; \
    case 4: { auto kf_ = K<T, 4>; ALAUNCH(NAME, kf_, WLG, ##__VA_ARGS__); } break; \
    case 2: { auto kf_ = K<T, 2>; ALAUNCH(NAME, kf_, WLG, ##__VA_ARGS__); } break; \
    default: break;                                                             \
    }

template <class T> static void vcycle(cfdl_ctx *ctx) {
    // Large levels run one thread per row (G = 1) or a few lanes per row
    // (the autotuned cgroup); small levels run 8 lanes per row, which
    // shortens each thread's chain of loads (amg_grouped[l] = G).
    const int L = ctx->amg_lmax;
    // the FP32 mesh-level kernels read 16-bit neighbour offsets when every
    // case has them: 52 B a row instead of 64, 8% faster at 128^3; the FP64
    // sweeps gained 3% for 12% fewer bytes (latency-bound) and keep int32
    const bool n16 = sizeof(T) == 4 && ctx->amg_nb16;
    for (int l = 0; l < L; l++) {
        int G = ctx->amg_grouped[l];
        if (G > 1) {
            ALAUNCH(l ? "k_v_jac0_c" : "k_v_jac0_f", k_v_jac0<T>, ctx->amg_smooth[l], l);
            GROUPED("k_v_jac_c", k_vg_jac, ctx->amg_gsmooth[l], 0, l)
            GROUPED("k_v_resid_c", k_vg_resid, ctx->amg_gsmooth[l], 0, l)
        } else if (l == 0 && sizeof(T) == 4) {
            // FP32 mesh level: t = w D^-1 r and the first sweep from it in one
            // pass (46.6 -> 33.2 us at 128^3).  The FP64 form keeps the two
            // passes: there the fused sweep measured slower (65.0 -> 74.7 us),
            // and so did the coarse levels' in both forms.
            if (n16) {
                ALAUNCH("k_v_jacr_f", (k_v_jac_mesh<T, true, false, true>), ctx->amg_smooth[l], l);
                ALAUNCH("k_v_resid_f", (k_v_resid_mesh<T, true>), ctx->amg_smooth[l], l);
            } else {
                ALAUNCH("k_v_jacr_f", (k_v_jac_mesh<T, false, false, true>), ctx->amg_smooth[l], l);
                ALAUNCH("k_v_resid_f", (k_v_resid_mesh<T, false>), ctx->amg_smooth[l], l);
            }
        } else {
            ALAUNCH(l ? "k_v_jac0_c" : "k_v_jac0_f", k_v_jac0<T>, ctx->amg_smooth[l], l);
            if (l == 0 && n16) {
                ALAUNCH("k_v_jac_f", (k_v_jac_mesh<T, true>), ctx->amg_smooth[l], l);
                ALAUNCH("k_v_resid_f", (k_v_resid_mesh<T, true>), ctx->amg_smooth[l], l);
            } else if (l == 0) {
                ALAUNCH("k_v_jac_f", (k_v_jac_mesh<T, false>), ctx->amg_smooth[l], l);
                ALAUNCH("k_v_resid_f", (k_v_resid_mesh<T, false>), ctx->amg_smooth[l], l);
            } else {
                ALAUNCH("k_v_jac_c", (k_v_jac<T>), ctx->amg_smooth[l], l);
                ALAUNCH("k_v_resid_c", (k_v_resid<T>), ctx->amg_smooth[l], l);
            }
        }
        G = ctx->amg_grouped[l + 1];
        if (G > 1) { GROUPED(l ? "k_v_restrict_c" : "k_v_restrict_f", k_vg_restrict, ctx->amg_grestr[l + 1], 0, l + 1) }
        else ALAUNCH(l ? "k_v_restrict_c" : "k_v_restrict_f", k_v_restrict<T>, ctx->amg_restr[l + 1], l + 1);
    }
    // each case's small levels and its coarsest solve, one CTA per case
    CLAUNCH("k_v_tail", k_v_tail<T>, kTailThreads);
    for (int l = L - 1; l >= 0; l--) {
        const int G = ctx->amg_grouped[l];
        if (G > 1) {
            GROUPED("k_v_prolong_c", k_vg_prolong, ctx->amg_gsmooth[l], 0, l)
            GROUPED("k_v_jac_c", k_vg_jac, ctx->amg_gsmooth[l], 0, l)
        } else {
            // z += s P z_{l+1}; t = J(z); z = J(t)
            ALAUNCH(l ? "k_v_lift_c" : "k_v_lift_f", k_v_lift<T>, ctx->amg_smooth[l], l);
            if (l == 0 && n16) {
                ALAUNCH("k_v_jac_f", (k_v_jac_mesh<T, true, true>), ctx->amg_smooth[l], l);
                ALAUNCH("k_v_jac_f", (k_v_jac_mesh<T, true>), ctx->amg_smooth[l], l);
            } else if (l == 0) {
                ALAUNCH("k_v_jac_f", (k_v_jac_mesh<T, false, true>), ctx->amg_smooth[l], l);
                ALAUNCH("k_v_jac_f", (k_v_jac_mesh<T, false>), ctx->amg_smooth[l], l);
            } else {
                ALAUNCH("k_v_jac_c", (k_v_jac<T, true>), ctx->amg_smooth[l], l);
                ALAUNCH("k_v_jac_c", (k_v_jac<T>), ctx->amg_smooth[l], l);
            }
        }
    }
}

void launch_pc_mean(cfdl_ctx *ctx);

#define RED ctx->cellsv.d_case_first, ctx->cellsv.d_case_ntiles, ctx->d_partials
#define RED32 ctx->cellsv.d_case_first, ctx->cellsv.d_case_ntiles, (float *)ctx->d_partials

// What the pressure solve needs of its matrix, once the matrix exists: the
// multigrid operators (AMG), or the level-0 FP32 copies and 1/ap (mixed
// Jacobi); the FP64 Jacobi form needs nothing.  In solve_uvwp this runs
// beside the momentum solve (cfdl_graph.cu): it depends on dc only.
void pressure_operators(cfdl_ctx *ctx) {
    const cfdl_config &c = ctx->cases[0]->cfg;
    if (c.precond == 1) amg_setup_operators(ctx);
    else if (c.precision >= 1) ALAUNCH("k_amg_prep0", k_amg_prep0, ctx->cells);
}

// FP64 AMG-PCG: zero-mean right-hand side, x = 0 (operators already built)
void apc_init(cfdl_ctx *ctx) {
    launch_pc_mean(ctx);
    ALAUNCH("k_apc_init", k_apc_init, ctx->cellsv, RED);
}

// one preconditioned CG iteration
void apc_iter(cfdl_ctx *ctx) {
    vcycle<double>(ctx);
    ALAUNCH("k_apc_rz", k_apc_rz, ctx->cellsv, RED);
    ALAUNCH("k_apc_p", k_apc_p, ctx->cellsv);
    ALAUNCH("k_apc_q", k_apc_q, ctx->cellsv, RED);
    ALAUNCH("k_apc_x", k_apc_x, ctx->cellsv, RED);
}

int solve_pressure_amg(cfdl_ctx *ctx) {
    int st = ensure_amg(ctx);
    if (st) return st;
    apc_init(ctx);
    int cap = 0;
    for (auto *hc : ctx->cases) cap = std::max(cap, hc->cfg.solve_mode == 0 ? hc->cfg.nit : hc->cfg.tight_maxit);
    int it = 0, maxit = 0;
    while (it < cap) {
        const int chunk = poll_chunk(it, ctx->last_iters_p);
        for (int k = 0; k < chunk && it < cap; k++, it++) apc_iter(ctx);
        int a = poll_kind(ctx, 1, &maxit);
        if (a < 0) return CFDL_ERR_CUDA;
        if (a == 0) break;
    }
    ctx->last_iters_p = maxit;
    return cuda_status(cudaGetLastError());
}


// ------------------------------------------------------------------------
// Mixed precision: FP64 outer residual and refinement around an FP32 inner
// PCG (FP32 SpMV, preconditioner, vectors and dot-product accumulation).
// ------------------------------------------------------------------------
namespace {

enum { CNT_M0 = 15 };   // shares the last counter slot only with itself

// outer start: r64 = b - mean, x = 0
__global__ void __launch_bounds__(kTile) k_mx_init(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                   const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (S->halted) return;
    double v[2] = {0, 0};
    FOR_CELLS(t) {
        const double r = C.b[i] - S->mean_b;
        C.kr[i] = r; C.phic[i] = 0.0;
        v[0] += r * r; v[1] += C.b[i] * C.b[i];
    }
    block_reduce<2>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_A0], cnt[t.c])) {
        __shared__ double s[2];
        sum_partials<2>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            S->r0norm_p = S->rnorm_p = sqrt(s[0]);
            S->mass_imbalance = sqrt(s[1]);
            S->iters_p = 0; S->status_p = 0; S->outer_p = 0;
            S->tol_p = (C.solve_mode == 0 ? C.rtol_p : C.tight_rtol) * S->r0norm_p;
            S->active_p = S->r0norm_p > S->tol_p && (C.solve_mode == 0 ? C.nit : C.tight_maxit) > 0;
            if (!isfinite(S->r0norm_p)) { S->active_p = 0; S->status_p = CFDL_ERR_NONFINITE; }
        }
    }
}

// inner start: fr = (float) r64, fx = 0; ||fr|| in FP32
__global__ void __launch_bounds__(kTile) k_mx_start(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                    const int *__restrict__ cfirst, const int *__restrict__ cnt, float *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (!S->active_p) return;
    float v[1] = {0.f};
    FOR_CELLS(t) {
        const float r = narrow_f32(C.kr[i]);
        C.fr[i] = r; C.fx[i] = 0.f;
        v[0] += r * r;
    }
    block_reduce<1, float>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_A1], cnt[t.c])) {
        __shared__ float s[1];
        sum_partials<1, float>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            const float rn = sqrtf(s[0]);
            // inner tolerance: the reference's drop in mode 0; when tight, half the
            // drop still needed to reach the FP64 target, but no finer than FP32
            // iterates track the true residual (1e-5) and no coarser than 0.5
            const float need = rn > 0.f ? (float)(S->tol_p / (double)rn) : 1.f;
            const float eps = C.solve_mode == 0 ? (float)C.rtol_p : fminf(0.5f, fmaxf(1e-5f, 0.5f * need));
            S->rnorm32 = rn;
            S->tol32 = eps * rn;
            S->rz32 = 0.f;
            S->iters32 = 0;
            S->active32 = rn > 0.f && isfinite(rn);
        }
    }
}

// z = M^-1 r for the Jacobi preconditioner (the AMG form uses the V-cycle)
__global__ void __launch_bounds__(kTile) k_mx_jacobi(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    if (!C.sc->active32) return;
    FOR_CELLS(t) C.fz[i] = C.fr[i] * C.frap_p[i];
}

__global__ void __launch_bounds__(kTile) k_mx_rz(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                 const int *__restrict__ cfirst, const int *__restrict__ cnt, float *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (!S->active32) return;
    float v[1] = {cg_rz_rows<float>(C.fr, C.fz, t)};
    block_reduce<1, float>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_A2], cnt[t.c])) {
        __shared__ float s[1];
        sum_partials<1, float>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            S->beta32 = S->iters32 == 0 || S->rz32 == 0.f ? 0.f : s[0] / S->rz32;
            S->rz32 = s[0];
            if (!isfinite(s[0])) S->active32 = 0;
        }
    }
}

__global__ void __launch_bounds__(kTile) k_mx_p(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    const SolveScalars *S = C.sc;
    if (!S->active32) return;
    cg_p_rows<float>(C.fz, C.fp, S->iters32 == 0, S->beta32, t);
}

template <bool k16>
__global__ void __launch_bounds__(kTile) k_mx_q(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                const int *__restrict__ cfirst, const int *__restrict__ cnt, float *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (!S->active32) return;
    float v[1] = {cg_aq_rows<float, k16>(level<float>(C, 0), C.fp, C.fq, t)};
    block_reduce<1, float>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_A3], cnt[t.c])) {
        __shared__ float s[1];
        sum_partials<1, float>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            if (!(s[0] > 0.f) || !isfinite(s[0])) S->active32 = 0;
            else S->alpha32 = S->rz32 / s[0];
        }
    }
}

__global__ void __launch_bounds__(kTile) k_mx_x(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                const int *__restrict__ cfirst, const int *__restrict__ cnt, float *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (!S->active32) return;
    float v[1] = {cg_x_rows<float>(C.fx, C.fp, C.fr, C.fq, S->alpha32, t)};
    block_reduce<1, float>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_A4], cnt[t.c])) {
        __shared__ float s[1];
        sum_partials<1, float>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            const float rn = sqrtf(s[0]);
            S->rnorm32 = rn;
            S->iters32 += 1;
            const int cap = C.solve_mode == 0 ? C.nit : C.tight_maxit;
            S->active32 = rn > S->tol32 && isfinite(rn) && S->iters32 < cap;
        }
    }
}

// x += (double) fx
__global__ void __launch_bounds__(kTile) k_mx_apply(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    if (!C.sc->active_p) return;
    FOR_CELLS(t) C.phic[i] = C.phic[i] + widen_f64(C.fx[i]);
}

// FP64 true residual r = (b - mean) - A x and the outer stopping test
__global__ void __launch_bounds__(kTile) k_mx_res(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles,
                                                  const int *__restrict__ cfirst, const int *__restrict__ cnt, double *partials) {
    CFDL_PDL_WAIT();
    const Tile t = tiles[blockIdx.x];
    const CaseDev &C = cases[t.c];
    SolveScalars *S = C.sc;
    if (!S->active_p) return;
    // two rows per step, both rows' loads before either store
    double v[1] = {0};
    const LP<double> P = level<double>(C, 0);
    const double mb = S->mean_b;
    FOR_ROW_PAIRS(t) {
        double r0 = 0.0, r1 = 0.0;
        if (ok0) r0 = (C.b[i0] - mb) - amul<double>(P, C.phic, i0);
        if (ok1) r1 = (C.b[i1] - mb) - amul<double>(P, C.phic, i1);
        if (ok0) { C.kr[i0] = r0; v[0] += r0 * r0; }
        if (ok1) { C.kr[i1] = r1; v[0] += r1 * r1; }
    }
    block_reduce<1>(v, &partials[(size_t)blockIdx.x * kNPart]);
    if (last_tile_of_case(&C.counters[CNT_M0], cnt[t.c])) {
        __shared__ double s[1];
        sum_partials<1>(partials, cfirst[t.c], cnt[t.c], s);
        if (threadIdx.x == 0) {
            const double rn = sqrt(s[0]);
            S->rnorm_p = rn;
            S->outer_p += 1;
            S->iters_p += S->iters32;
            int act = rn > S->tol_p;
            if (!isfinite(rn)) { act = 0; S->status_p = CFDL_ERR_NONFINITE; }
            else if (act && S->outer_p >= kMixedMaxOuter) { act = 0; if (C.solve_mode == 1) S->status_p = CFDL_ERR_ITER_CAP; }
            S->active_p = act;
        }
    }
}

}  // namespace

// mixed form: FP32 operator copies (+ coarse operators), FP64 start
void mx_init(cfdl_ctx *ctx) {
    launch_pc_mean(ctx);
    ALAUNCH("k_mx_init", k_mx_init, ctx->cellsv, RED);
}
void mx_start(cfdl_ctx *ctx) { ALAUNCH("k_mx_start", k_mx_start, ctx->cellsv, RED32); }
void mx_inner_iter(cfdl_ctx *ctx) {
    if (ctx->cases[0]->cfg.precond == 1) vcycle<float>(ctx);
    else ALAUNCH("k_mx_jacobi", k_mx_jacobi, ctx->cellsv);
    ALAUNCH("k_mx_rz", k_mx_rz, ctx->cellsv, RED32);
    ALAUNCH("k_mx_p", k_mx_p, ctx->cellsv);
    if (ctx->amg_nb16) ALAUNCH("k_mx_q", k_mx_q<true>, ctx->cellsv, RED32);
    else ALAUNCH("k_mx_q", k_mx_q<false>, ctx->cellsv, RED32);
    ALAUNCH("k_mx_x", k_mx_x, ctx->cellsv, RED32);
}
void mx_finish(cfdl_ctx *ctx) {
    ALAUNCH("k_mx_apply", k_mx_apply, ctx->cellsv);
    ALAUNCH("k_mx_res", k_mx_res, ctx->cellsv, RED);
}

int solve_pressure_mixed(cfdl_ctx *ctx) {
    int st;
    if (ctx->cases[0]->cfg.precond == 1 && (st = ensure_amg(ctx))) return st;
    mx_init(ctx);
    int cap = 0;
    for (auto *hc : ctx->cases) cap = std::max(cap, hc->cfg.solve_mode == 0 ? hc->cfg.nit : hc->cfg.tight_maxit);
    for (int outer = 0; outer < kMixedMaxOuter; outer++) {
        mx_start(ctx);
        int it = 0, maxit = 0;
        while (it < cap) {
            const int chunk = poll_chunk(it, ctx->last_iters_p);
            for (int k = 0; k < chunk && it < cap; k++, it++) mx_inner_iter(ctx);
            int a = poll_kind(ctx, 2, &maxit);
            if (a < 0) return CFDL_ERR_CUDA;
            if (a == 0) break;
        }
        ctx->last_iters_p = maxit;
        mx_finish(ctx);
        int a = poll_kind(ctx, 3, nullptr);
        if (a < 0) return CFDL_ERR_CUDA;
        if (a == 0) break;
    }
    return cuda_status(cudaGetLastError());
}
#undef RED
#undef RED32

}  // namespace cfdl

extern "C" int cfdl_amg_index_bytes(const cfdl_ctx *ctx) {
    return ctx ? (ctx->amg_nb16 && !ctx->cases.empty() && ctx->cases[0]->cfg.precision >= 1 ? 2 : 4) : -1;
}

extern "C" int cfdl_amg_info(cfdl_ctx *ctx, int maxlev, int *nlev, int *n, int *W) {
    using namespace cfdl;
    if (!ctx || ctx->cases.empty() || !nlev || maxlev < 0) return CFDL_ERR_INVALID;
    const HostCase *hc = ctx->cases[0];
    const int L = hc->amg ? (int)hc->amg->levels.size() : 0;
    *nlev = L;
    for (int l = 0; l <= L && l <= maxlev; l++) {
        if (n) n[l] = l == 0 ? hc->ne : hc->amg->levels[l - 1].n;
        if (W) W[l] = l == 0 ? hc->W : hc->amg->levels[l - 1].W;
    }
    return CFDL_OK;
}
