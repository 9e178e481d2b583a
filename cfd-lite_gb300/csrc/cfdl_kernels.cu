// cfdl_kernels.cu -- assembly, gradient, flux and correction kernels of one
// SIMPLE outer iteration (FP64), one CTA per tile of the work list.
//
// Each kernel restates a reference routine (cited per kernel).  Per-face
// quantities that the reference computes twice (once from each side of a
// face) are computed once per face here and gathered by the cells, and every
// mesh-only sub-expression comes from the precomputed face planes; the
// remaining FP64 arithmetic is what the fields require.  Cell-side sums run in
// the reference's CSR half-face order, and boundary contributions in the
// reference's BC-loop order (ascending halo index), so the only differences
// from the reference are the roundings of the reassociated face terms.
#include "cfdl_device.cuh"

namespace cfdl {
namespace {

#define TILE_PROLOGUE(WL)                         \
    const Tile t = tiles[blockIdx.x];             \
    const CaseDev &C = cases[t.c];                \
    if (C.sc->halted) return;                     \
    const int i = t.first + (int)threadIdx.x;

// ---------------------------------------------------------------------------
// update_boundaries -> lid / dirichlet0 / symmetry, mod_physics.f90:38-50,
// mod_uvwp.f90:493-570.  One thread per halo.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTile) k_bc(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(halos)
    if (i >= t.last) return;
    const int kind = C.h_kind[i];
    if (kind == 0) return;
    const int e = C.h_own[i], f = C.h_face[i], h = C.ne + i;
    if (kind == CFDL_BC_WALL) {
        C.u[h] = C.h_vel[3 * i];
        C.v[h] = C.h_vel[3 * i + 1];
        C.w[h] = C.h_vel[3 * i + 2];
    } else {  // symmetry: velt - 2*veln of the owner velocity
        const double *g = C.fgeo;
        const int nf = C.nf;
        double area = g[FG_AREA * nf + f];
        double n0 = g[FG_AX * nf + f] / area, n1 = g[FG_AY * nf + f] / area, n2 = g[FG_AZ * nf + f] / area;
        double vu = C.u[e], vv = C.v[e], vw = C.w[e];
        double vn = vu * n0 + vv * n1 + vw * n2;
        double a0 = vn * n0, a1 = vn * n1, a2 = vn * n2;
        C.u[h] = (vu - a0) - 2 * a0;
        C.v[h] = (vv - a1) - 2 * a1;
        C.w[h] = (vw - a2) - 2 * a2;
    }
    C.p[h] = C.p[e];
    C.mip[f] = 0.0;
}

// ---------------------------------------------------------------------------
// calc_coef_uvw, face part (mod_uvwp.f90:183-226): per interior face the
// diffusion coefficient muip*area/ds and the secondary-stress (sumss) and
// deferred non-orthogonal correction (sumdefc) terms, from the owner's side;
// the neighbour takes them with the opposite sign.  Boundary faces: the wall
// diffusion mu*area/ds of the BC loop (mod_uvwp.f90:257).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTile) k_coef_uvw_face(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(faces)
    if (i >= t.last) return;
    const int nf = C.nf, o = C.f_own[i], n = C.f_nb[i];
    if (n >= C.ne) return;                  // boundary faces: only their (precomputed) diffusion
    const double *g = C.fgeo, *pr = C.fprop;
    const double wt = g[FG_WT * nf + i], omw = 1.0 - wt;
    const double A0 = pr[PR_MAX * nf + i], A1 = pr[PR_MAY * nf + i], A2 = pr[PR_MAZ * nf + i];
    const double E0 = pr[PR_MEX * nf + i], E1 = pr[PR_MEY * nf + i], E2 = pr[PR_MEZ * nf + i];
    double gi[3][3];   // gi[q][m]: component m of grad(u_q) at the face
    const double *gq[3] = {C.gu, C.gv, C.gw};
#pragma unroll
    for (int q = 0; q < 3; q++)
#pragma unroll
        for (int m = 0; m < 3; m++) gi[q][m] = omw * gq[q][3 * o + m] + wt * gq[q][3 * n + m];
    // the two explicit face terms of component m, which the cell sums add to
    // the same right-hand side, stored as one value:
    //   sumss(m):   mu_ip (du/dx_m, dv/dx_m, dw/dx_m) . dr
    //   sumdefc(m): mu_ip grad(u_m) . (dr_p/ds_p - dr/ds)
    // (mu_ip is folded into the property planes)
#pragma unroll
    for (int m = 0; m < 3; m++)
        C.fS[m * nf + i] = (gi[0][m] * A0 + gi[1][m] * A1 + gi[2][m] * A2) + (gi[m][0] * E0 + gi[m][1] * E1 + gi[m][2] * E2);
}

// Property planes of every face (recomputed when rho or mu change): the mesh
// planes scaled by the interpolated viscosity and density.
__global__ void __launch_bounds__(kTile) k_face_props(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(faces)
    if (i >= t.last) return;
    const int nf = C.nf, o = C.f_own[i], n = C.f_nb[i];
    const double *g = C.fgeo;
    double *pr = C.fprop;
    if (n >= C.ne) {
        pr[PR_FDIFF * nf + i] = C.mu[o] * g[FG_ADS * nf + i];
        for (int k = PR_MAX; k < PR_N; k++) pr[k * nf + i] = 0.0;
        return;
    }
    const double wt = g[FG_WT * nf + i], omw = 1.0 - wt;
    const double muip = omw * C.mu[o] + wt * C.mu[n];
    const double rhoip = C.rho[o] * omw + C.rho[n] * wt;
    const double adn = g[FG_ADN * nf + i];
    pr[PR_FDIFF * nf + i] = muip * g[FG_ADS * nf + i];
    for (int m = 0; m < 3; m++) {
        pr[(PR_MAX + m) * nf + i] = muip * g[(FG_ADRX + m) * nf + i];
        pr[(PR_MEX + m) * nf + i] = muip * g[(FG_EX + m) * nf + i];
    }
    pr[PR_RHO * nf + i] = rhoip;
    pr[PR_RHOADN * nf + i] = rhoip * adn;
    pr[PR_RHOMADN * nf + i] = (C.rho[o] + C.rho[n]) / 2.0 * adn;
    if (C.fprop32) {   // precision 3: the planes of the FP32 explicit face terms and Rhie-Chow term
        float *pf = C.fprop32;
        pf[i] = narrow_f32(wt);
        for (int m = 0; m < 3; m++) {
            pf[(1 + m) * nf + i] = narrow_f32(pr[(PR_MAX + m) * nf + i]);
            pf[(4 + m) * nf + i] = narrow_f32(pr[(PR_MEX + m) * nf + i]);
            pf[(7 + m) * nf + i] = narrow_f32(g[(FG_DRX + m) * nf + i]);
        }
        pf[10 * nf + i] = narrow_f32(pr[PR_RHOADN * nf + i]);
    }
}

// calc_coef_uvw face part in FP32 (precision 3): the same two explicit terms
// as k_coef_uvw_face -- sumss and the deferred non-orthogonal correction, the
// deferred-correction sources of the momentum equations -- from the FP32
// gradients and planes, with no FP64 instruction; fS holds them as FP32.
__global__ void __launch_bounds__(kTile) k_coef_uvw_face_f32(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(faces)
    if (i >= t.last) return;
    const int nf = C.nf, ne = C.ne, o = C.f_own[i], n = C.f_nb[i];
    if (n >= ne) return;
    const float *pf = C.fprop32;
    const float wt = pf[i], omw = 1.0f - wt;
    const float A0 = pf[nf + i], A1 = pf[2 * nf + i], A2 = pf[3 * nf + i];
    const float E0 = pf[4 * nf + i], E1 = pf[5 * nf + i], E2 = pf[6 * nf + i];
    float gi[3][3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const float *g = C.g32 + (size_t)q * 3 * ne;
#pragma unroll
        for (int m = 0; m < 3; m++) gi[q][m] = omw * g[3 * o + m] + wt * g[3 * n + m];
    }
    float *fS = (float *)C.fS;
#pragma unroll
    for (int m = 0; m < 3; m++)
        fS[m * nf + i] = (gi[0][m] * A0 + gi[1][m] * A1 + gi[2][m] * A2) + (gi[m][0] * E0 + gi[m][1] * E1 + gi[m][2] * E2);
}

// calc_coef_uvw, boundary-condition loop (mod_uvwp.f90:242-273), one thread
// per halo: the wall diffusion mu*area/ds it adds to the owner's ap and to
// the slot's anb, and for a wall ('dirichlet') the momentum source
// d*(u_wall - u_tangential) - d*u of each component; a symmetry plane
// ('zero_flux') adds the diffusion only.  The cell kernel gathers them.
__global__ void __launch_bounds__(kTile) k_coef_uvw_halo(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(halos)
    if (i >= t.last) return;
    const int nbf = C.nbf, nf = C.nf, kind = C.h_kind[i];
    double dbc = 0.0, s0 = 0.0, s1 = 0.0, s2 = 0.0;
    if (kind != 0) {
        const int e = C.h_own[i], f = C.h_face[i], h = C.ne + i;
        dbc = C.fprop[PR_FDIFF * nf + f];
        if (kind == CFDL_BC_WALL) {
            const double ue = C.u[e], ve = C.v[e], we = C.w[e];
            const double area = C.fgeo[FG_AREA * nf + f];
            const double n0 = C.fgeo[FG_AX * nf + f] / area, n1 = C.fgeo[FG_AY * nf + f] / area,
                         n2 = C.fgeo[FG_AZ * nf + f] / area;
            const double tn = ue * n0 + ve * n1 + we * n2;
            const double r0 = C.u[h] - (ue - tn * n0), r1 = C.v[h] - (ve - tn * n1), r2 = C.w[h] - (we - tn * n2);
            s0 = dbc * r0 - dbc * ue;
            s1 = dbc * r1 - dbc * ve;
            s2 = dbc * r2 - dbc * we;
        }
    }
    C.hbc[i] = dbc;
    C.hbc[nbf + i] = s0;
    C.hbc[2 * nbf + i] = s1;
    C.hbc[3 * nbf + i] = s2;
}

// calc_coef_uvw, cell part (mod_uvwp.f90:174-284) + implicit relaxation.
// Interior slots first (their faces' terms), then the boundary slots' terms
// of k_coef_uvw_halo, summed apart and added after the right-hand sides as
// the reference's BC loop adds them after its cell loop.  Every slot is
// indexed by an unrolled loop counter, so the row stays in registers.
// F32 (precision 3): the explicit face terms are FP32 and summed in FP32.
template <bool F32>
__global__ void __launch_bounds__(kTile) k_coef_uvw_cell(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(cells)
    if (i >= t.last) return;
    const int ne = C.ne, nf = C.nf, nbf = C.nbf, W = C.W;
    double ap = 0.0, sumf = 0.0, ss0 = 0.0, ss1 = 0.0, ss2 = 0.0;
    double bap = 0.0, bs0 = 0.0, bs1 = 0.0, bs2 = 0.0;   // the boundary slots' terms
    float fs0 = 0.f, fs1 = 0.f, fs2 = 0.f;
    const float *fS32 = (const float *)C.fS;
    double a[kMaxW];
#pragma unroll
    for (int k = 0; k < kMaxW; k++) {
        a[k] = 0.0;
        if (k >= W) continue;
        const int nb = C.hf_nb[k * ne + i];
        if (nb < 0) continue;
        if (nb >= ne) {
            const int q = nb - ne;
            const double dbc = C.hbc[q];
            a[k] = dbc;                 // anb of a boundary slot is 0 before the BC loop: 0 + d = d
            bap += dbc;
            bs0 += C.hbc[nbf + q]; bs1 += C.hbc[2 * nbf + q]; bs2 += C.hbc[3 * nbf + q];
            continue;
        }
        const int fc = C.hf_fc[k * ne + i], f = face_of(fc);
        // inward flux f = -sg*mip and upwind max(f,0): sign and comparison on
        // the bit pattern, so they cost no FP64 instruction
        const double fl = flip_sign(C.mip[f], fc >= 0);
        const double ak = C.fprop[PR_FDIFF * nf + f] + positive_part(fl);
        sumf += fl;
        a[k] = ak;
        ap += ak;
        // sg * x as a sign-bit flip: no FP64 multiply
        const bool ng = fc < 0;
        if (F32) {
            fs0 += flip_sign_f(fS32[f], ng); fs1 += flip_sign_f(fS32[nf + f], ng); fs2 += flip_sign_f(fS32[2 * nf + f], ng);
        } else {
            ss0 += flip_sign(C.fS[f], ng); ss1 += flip_sign(C.fS[nf + f], ng); ss2 += flip_sign(C.fS[2 * nf + f], ng);
        }
    }
    if (F32) { ss0 = widen_f64(fs0); ss1 = widen_f64(fs1); ss2 = widen_f64(fs2); }
    double asum = ap;                       // sum of the anb of this row so far
    const double vol = C.vol[i];
    const double ue = C.u[i], ve = C.v[i], we = C.w[i];
    double bu, bv, bw;
    if (C.steady) {                         // ap0 = rho*vol/dt = 0
        bu = sumf * ue - vol * C.gp[3 * i] + ss0;
        bv = sumf * ve - vol * C.gp[3 * i + 1] + ss1;
        bw = sumf * we - vol * C.gp[3 * i + 2] + ss2;
    } else {
        const double ap0 = C.rho[i] * vol * C.rdt;
        ap = ap + ap0;
        bu = ap0 * C.u0[i] + sumf * ue - vol * C.gp[3 * i] + ss0;
        bv = ap0 * C.v0[i] + sumf * ve - vol * C.gp[3 * i + 1] + ss1;
        bw = ap0 * C.w0[i] + sumf * we - vol * C.gp[3 * i + 2] + ss2;
    }
    // the boundary-condition loop's additions
    ap = ap + bap;
    asum = asum + bap;
    bu = bu + bs0; bv = bv + bs1; bw = bw + bs2;
    if (C.alpha_u != 1.0) {
        const double apr = ap * C.ralpha_u, f1 = (1.0 - C.alpha_u) * apr;
        bu = bu + f1 * ue; bv = bv + f1 * ve; bw = bw + f1 * we;
        ap = apr;
    }
    C.ap[i] = ap;
    C.bu[i] = bu; C.bv[i] = bv; C.bw[i] = bw;
    const double dd = vol / ap;
    C.d[i] = dd;
    if (F32) C.d32[i] = narrow_f32(dd);
#pragma unroll
    for (int k = 0; k < kMaxW; k++)
        if (k < W) C.anb[k * ne + i] = a[k];
    C.dc[i] = vol / (ap - asum);            // SIMPLEC: vol / (ap - sum anb)
}

// ---------------------------------------------------------------------------
// calc_grad, mod_solver.f90:40-81, as the stencil sum grad = sum_k G_k dphi_k.
// NF fields at once (u,v,w or the energy equation's t and phi share the
// stencil loads).
// ---------------------------------------------------------------------------
template <int NF>
__global__ void __launch_bounds__(kTile) k_grad(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int field) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(cells)
    if (i >= t.last) return;
    const int ne = C.ne, W = C.W;
    const double *phi[NF];
    double *grad[NF];
    if (NF == 3) { phi[0] = C.u; phi[1 % NF] = C.v; phi[2 % NF] = C.w; grad[0] = C.gu; grad[1 % NF] = C.gv; grad[2 % NF] = C.gw; }
    else if (NF == 2) {
        if (!C.ee) return;                  // no energy equation in this case
        phi[0] = C.et; phi[1 % NF] = C.ee; grad[0] = C.egt; grad[1 % NF] = C.ege;
    } else {
        phi[0] = field == 0 ? C.u : field == 1 ? C.v : field == 2 ? C.w : C.phic;
        grad[0] = field == 0 ? C.gu : field == 1 ? C.gv : field == 2 ? C.gw : C.gpc;
    }
    double pe[NF], g[NF][3];
#pragma unroll
    for (int q = 0; q < NF; q++) { pe[q] = phi[q][i]; g[q][0] = g[q][1] = g[q][2] = 0.0; }
#pragma unroll
    for (int k = 0; k < kMaxW; k++) {
        if (k >= W) break;
        const int nb = C.hf_nb[k * ne + i];
        if (nb < 0) break;
        const double G0 = C.hf_G[(0 * W + k) * ne + i], G1 = C.hf_G[(1 * W + k) * ne + i], G2 = C.hf_G[(2 * W + k) * ne + i];
#pragma unroll
        for (int q = 0; q < NF; q++) {
            const double dphi = phi[q][nb] - pe[q];
            g[q][0] += G0 * dphi; g[q][1] += G1 * dphi; g[q][2] += G2 * dphi;
        }
    }
#pragma unroll
    for (int q = 0; q < NF; q++) { grad[q][3 * i] = g[q][0]; grad[q][3 * i + 1] = g[q][1]; grad[q][3 * i + 2] = g[q][2]; }
}

// calc_grad of u, v, w for the FP32 explicit face terms (precision 3): the
// neighbour differences in FP64, narrowed in the integer pipe, the stencil
// sums in FP32; the gradients go to g32 and, widened, to gu, gv, gw.
__global__ void __launch_bounds__(kTile, 3) k_grad3_f32(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(cells)
    if (i >= t.last) return;
    const int ne = C.ne, W = C.W;
    const double *phi[3] = {C.u, C.v, C.w};
    double *grad[3] = {C.gu, C.gv, C.gw};
    double pe[3];
    float g[3][3];
#pragma unroll
    for (int q = 0; q < 3; q++) { pe[q] = phi[q][i]; g[q][0] = g[q][1] = g[q][2] = 0.f; }
    // Every slot's loads are issued before the first is used: a loop that
    // stopped at the first padding slot had to wait for each slot's index
    // before it could load the next slot, six dependent trips to memory.  A
    // row's slots end at its first padding slot (live), as that loop did.
    // With 3 CTAs per SM (80 registers) this measured 203 -> 151 us at 128^3.
    int nb[kMaxW];
    bool live[kMaxW];
    float G[3][kMaxW];
    bool on = true;
#pragma unroll
    for (int k = 0; k < kMaxW; k++) {
        const int j = k < W ? C.hf_nb[k * ne + i] : -1;
#pragma unroll
        for (int m = 0; m < 3; m++) G[m][k] = k < W ? C.G32[(m * W + k) * ne + i] : 0.f;
        on = on && j >= 0;
        live[k] = on;
        nb[k] = on ? j : i;
    }
    double pn[3][kMaxW];
#pragma unroll
    for (int k = 0; k < kMaxW; k++)
#pragma unroll
        for (int q = 0; q < 3; q++) pn[q][k] = phi[q][nb[k]];
#pragma unroll
    for (int k = 0; k < kMaxW; k++) {
        if (!live[k]) continue;
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const float d = narrow_f32(pn[q][k] - pe[q]);
            g[q][0] += G[0][k] * d; g[q][1] += G[1][k] * d; g[q][2] += G[2][k] * d;
        }
    }
#pragma unroll
    for (int q = 0; q < 3; q++) {
        float *g32 = C.g32 + (size_t)q * 3 * ne + 3 * i;
#pragma unroll
        for (int m = 0; m < 3; m++) { g32[m] = g[q][m]; grad[q][3 * i + m] = widen_f64(g[q][m]); }
    }
}

// precision 3: g32 from gu, gv, gw after they were written from outside
// (uploads, set_array, a restored snapshot)
__global__ void __launch_bounds__(kTile) k_narrow_grad(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(cells)
    if (i >= t.last || !C.g32) return;
    const double *grad[3] = {C.gu, C.gv, C.gw};
#pragma unroll
    for (int q = 0; q < 3; q++)
#pragma unroll
        for (int m = 0; m < 3; m++) C.g32[(size_t)q * 3 * C.ne + 3 * i + m] = narrow_f32(grad[q][3 * i + m]);
#pragma unroll
    for (int m = 0; m < 3; m++) C.gp32[3 * i + m] = narrow_f32(C.gp[3 * i + m]);
    C.d32[i] = narrow_f32(C.d[i]);
}

__global__ void k_narrow_array(const double *__restrict__ in, float *__restrict__ out, size_t n) {
    CFDL_PDL_WAIT();
    const size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j < n) out[j] = narrow_f32(in[j]);
}

// narrow_f32 / widen_f64 against the hardware conversions on n values drawn
// from every binary64 exponent (bit patterns from a 64-bit mix of the
// index) plus signed zeros, infinities and NaN.  Differences are counted
// except where the definitions differ on purpose: values whose binary32
// result is subnormal (flushed to a signed zero here).
__global__ void k_check_conversions(int n, unsigned *bad) {
    CFDL_PDL_WAIT();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    unsigned long long z = 0x9e3779b97f4a7c15ull * (unsigned long long)(j + 1);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    // exponents concentrated near the binary32 range so that rounding, carries and
    // the range limits are all exercised
    const unsigned long long e = 1023 - 140 + (z >> 52) % 290;
    unsigned long long bits = (z & 0x800fffffffffffffull) | (e << 52);
    if (j < 8) {
        const unsigned long long special[8] = {0x0ull, 0x8000000000000000ull, 0x7ff0000000000000ull, 0xfff0000000000000ull,
                                               0x7ff8000000000000ull, 0x3ff0000010000000ull, 0x3ff0000030000000ull,
                                               0x47efffffefffffffull};
        bits = special[j];
    }
    const double x = __longlong_as_double((long long)bits);
    const float mine = narrow_f32(x), ref = __double2float_rn(x);
    const unsigned mu = __float_as_uint(mine), ru = __float_as_uint(ref);
    const bool ref_sub = (ru & 0x7f800000u) == 0 && (ru & 0x7fffffu) != 0;
    const bool nan_both = (ru & 0x7fffffffu) > 0x7f800000u && (mu & 0x7fffffffu) > 0x7f800000u;
    if (mu != ru && !nan_both && !(ref_sub && (mu & 0x7fffffffu) == 0)) atomicAdd(&bad[0], 1u);
    // widening: exact for every normal binary32
    const float f = __uint_as_float((unsigned)(z >> 11));
    const unsigned fe = (__float_as_uint(f) >> 23) & 0xffu;
    if (fe != 0 && fe != 0xffu) {
        if (__double_as_longlong(widen_f64(f)) != __double_as_longlong((double)f)) atomicAdd(&bad[1], 1u);
    }
}

// ---------------------------------------------------------------------------
// calc_mip, mod_uvwp.f90:438-490.  One thread per face; boundary faces keep
// the value their BC set.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTile) k_calc_mip(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int rc) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(faces)
    if (i >= t.last) return;
    const int nf = C.nf, o = C.f_own[i], n = C.f_nb[i];
    if (n >= C.ne) return;
    const double *g = C.fgeo;
    const double wt = g[FG_WT * nf + i], omw = 1.0 - wt;
    const double A0 = g[FG_AX * nf + i], A1 = g[FG_AY * nf + i], A2 = g[FG_AZ * nf + i];
    const double vx = omw * C.u[o] + wt * C.u[n], vy = omw * C.v[o] + wt * C.v[n], vz = omw * C.w[o] + wt * C.w[n];
    const double rhoip = C.fprop[PR_RHO * nf + i];
    double mip = (vx * A0 + vy * A1 + vz * A2) * rhoip;
    if (rc) {
        const double D0 = g[FG_DRX * nf + i], D1 = g[FG_DRY * nf + i], D2 = g[FG_DRZ * nf + i];
        const double gx = omw * C.gp[3 * o] + wt * C.gp[3 * n];
        const double gy = omw * C.gp[3 * o + 1] + wt * C.gp[3 * n + 1];
        const double gz = omw * C.gp[3 * o + 2] + wt * C.gp[3 * n + 2];
        const double dip = omw * C.d[o] + wt * C.d[n];
        mip = mip - dip * C.fprop[PR_RHOADN * nf + i] * ((C.p[n] - C.p[o]) - (gx * D0 + gy * D1 + gz * D2));
        if (!C.steady) {   // the transient term carries 1/dt and vanishes when steady
            const double ux = omw * C.u0[o] + wt * C.u0[n], uy = omw * C.v0[o] + wt * C.v0[n], uz = omw * C.w0[o] + wt * C.w0[n];
            mip = mip - rhoip * dip * C.rdt * (C.mip0[i] - (ux * A0 + uy * A1 + uz * A2) * rhoip);
        }
    }
    C.mip[i] = mip;
}

// calc_mip in precision 3: the flux (rho_ip v_ip . A) in FP64, the Rhie-Chow
// pressure-smoothing term -rho_ip A/(dr.n) d_ip ((p_nb - p_P) - gp_ip . dr)
// in FP32 from the FP64 pressure difference and FP32 copies of gp, d and the
// planes (it is a correction to the flux, well inside FP32's range and
// relative precision), widened and subtracted in FP64.  The transient term
// of an unsteady case stays FP64.
__global__ void __launch_bounds__(kTile) k_calc_mip_f32(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles, int rc) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(faces)
    if (i >= t.last) return;
    const int nf = C.nf, o = C.f_own[i], n = C.f_nb[i];
    if (n >= C.ne) return;
    const double *g = C.fgeo;
    const double wt = g[FG_WT * nf + i], omw = 1.0 - wt;
    const double A0 = g[FG_AX * nf + i], A1 = g[FG_AY * nf + i], A2 = g[FG_AZ * nf + i];
    const double vx = omw * C.u[o] + wt * C.u[n], vy = omw * C.v[o] + wt * C.v[n], vz = omw * C.w[o] + wt * C.w[n];
    const double rhoip = C.fprop[PR_RHO * nf + i];
    double mip = (vx * A0 + vy * A1 + vz * A2) * rhoip;
    if (rc) {
        const float *pf = C.fprop32;
        const float wf = pf[i], omf = 1.0f - wf;
        const float D0 = pf[7 * nf + i], D1 = pf[8 * nf + i], D2 = pf[9 * nf + i];
        const float *gp = C.gp32;
        const float gx = omf * gp[3 * o] + wf * gp[3 * n];
        const float gy = omf * gp[3 * o + 1] + wf * gp[3 * n + 1];
        const float gz = omf * gp[3 * o + 2] + wf * gp[3 * n + 2];
        const float dip = omf * C.d32[o] + wf * C.d32[n];
        const float dp = narrow_f32(C.p[n] - C.p[o]);
        const float corr = dip * pf[10 * nf + i] * (dp - (gx * D0 + gy * D1 + gz * D2));
        mip = mip - widen_f64(corr);
        if (!C.steady) {
            const double dip64 = omw * C.d[o] + wt * C.d[n];
            const double ux = omw * C.u0[o] + wt * C.u0[n], uy = omw * C.v0[o] + wt * C.v0[n], uz = omw * C.w0[o] + wt * C.w0[n];
            mip = mip - rhoip * dip64 * C.rdt * (C.mip0[i] - (ux * A0 + uy * A1 + uz * A2) * rhoip);
        }
    }
    C.mip[i] = mip;
}

// ---------------------------------------------------------------------------
// calc_coef_p, mod_uvwp.f90:289-368: face coefficient
// rho_ip * dc_ip * area/(dr.n), symmetric, then per cell ap = sum anb and
// b = net inflow - boundary mass flux.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTile) k_coef_p_face(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(faces)
    if (i >= t.last) return;
    const int nf = C.nf, o = C.f_own[i], n = C.f_nb[i];
    if (n >= C.ne) { C.fdiff[i] = 0.0; return; }
    const double wt = C.fgeo[FG_WT * nf + i], omw = 1.0 - wt;
    C.fdiff[i] = (omw * C.dc[o] + wt * C.dc[n]) * C.fprop[PR_RHOADN * nf + i];
}

// the matrix: anb = the face coefficient on interior slots (0 on walls,
// mod_uvwp.f90:354-363), ap = their sum.  Every slot's index loads, then
// every coefficient gather, are issued before the stores (a store in the
// slot loop held back the next slot's loads: three dependent trips to
// memory a slot).
__global__ void __launch_bounds__(kTile) k_coef_p_mat(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(cells)
    if (i >= t.last) return;
    const int ne = C.ne, W = C.W;
    int nb[kMaxW], fc[kMaxW];
#pragma unroll
    for (int k = 0; k < kMaxW; k++) {
        nb[k] = k < W ? C.hf_nb[k * ne + i] : -1;
        fc[k] = k < W ? C.hf_fc[k * ne + i] : 0;
    }
    double a[kMaxW];
#pragma unroll
    for (int k = 0; k < kMaxW; k++) a[k] = nb[k] >= 0 && nb[k] < ne ? C.fdiff[face_of(fc[k])] : 0.0;
    double ap = 0.0;
#pragma unroll
    for (int k = 0; k < kMaxW; k++)
        if (nb[k] >= 0 && nb[k] < ne) ap += a[k];
#pragma unroll
    for (int k = 0; k < kMaxW; k++)
        if (k < W) C.anb_p[k * ne + i] = a[k];
    C.ap_p[i] = ap;
}

// the right-hand side: b = net inflow over the interior faces, minus the
// boundary mass fluxes in BC-loop order (ascending halo index).  The slots'
// loads are issued together; the boundary slots are then taken in halo
// order by selection over the row's registers.
__global__ void __launch_bounds__(kTile) k_coef_p_rhs(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(cells)
    if (i >= t.last) return;
    const int ne = C.ne, W = C.W;
    int nb[kMaxW], fc[kMaxW];
#pragma unroll
    for (int k = 0; k < kMaxW; k++) {
        nb[k] = k < W ? C.hf_nb[k * ne + i] : -1;
        fc[k] = k < W ? C.hf_fc[k * ne + i] : 0;
    }
    double m[kMaxW];
    int kind[kMaxW];
#pragma unroll
    for (int k = 0; k < kMaxW; k++) {
        m[k] = nb[k] >= 0 ? C.mip[face_of(fc[k])] : 0.0;
        kind[k] = nb[k] >= ne ? C.h_kind[nb[k] - ne] : 0;
    }
    double sumf = 0.0;
#pragma unroll
    for (int k = 0; k < kMaxW; k++)
        if (nb[k] >= 0 && nb[k] < ne) sumf += flip_sign(m[k], fc[k] >= 0);   // -sg * mip
    int prev = ne - 1;
    for (int q = 0; q < kMaxW; q++) {       // the boundary slot of the next larger halo index
        int best = 0x7fffffff, bkind = 0;
        double bm = 0.0;
#pragma unroll
        for (int k = 0; k < kMaxW; k++)
            if (nb[k] > prev && nb[k] < best) { best = nb[k]; bm = m[k]; bkind = kind[k]; }
        if (best == 0x7fffffff) break;
        prev = best;
        if (bkind != 0) sumf = sumf - bm;
    }
    C.b[i] = sumf;
}

// ---------------------------------------------------------------------------
// adjust_pc, mod_uvwp.f90:136-158: pc -= pc(1); halo pc = owner pc.
// ---------------------------------------------------------------------------
__global__ void k_save_pref(const CaseDev *__restrict__ cases, int ncases) {
    CFDL_PDL_WAIT();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncases) cases[c].sc->pref = cases[c].phic[0];
}

__global__ void __launch_bounds__(kTile) k_adjust_pc(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(cells)
    if (i >= t.last) return;
    const int ne = C.ne, W = C.W;
    // the row's loads before its stores (a store holds back the loads after it)
    int nb[kMaxW];
#pragma unroll
    for (int k = 0; k < kMaxW; k++) nb[k] = k < W ? C.hf_nb[k * ne + i] : -1;
    const double v = C.phic[i] - C.sc->pref;
    C.phic[i] = v;
#pragma unroll
    for (int k = 0; k < kMaxW; k++)
        if (nb[k] >= ne) C.phic[nb[k]] = v;
}

// ---------------------------------------------------------------------------
// update_uvwp, mod_uvwp.f90:370-436: p += alpha_p*pc, gp += alpha_p*gpc on
// cells; mip -= rho_ip*A*dc_ip*(pc_nb-pc_P)/(dr.n) on interior faces.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTile) k_update_cells(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(cells)
    if (i >= t.last) return;
    const double a = C.alpha_p;
    double g[3];
    if (a == 1.0) {
        C.p[i] = C.p[i] + C.phic[i];
#pragma unroll
        for (int q = 0; q < 3; q++) C.gp[3 * i + q] = g[q] = C.gp[3 * i + q] + C.gpc[3 * i + q];
    } else {
        C.p[i] = C.p[i] + a * C.phic[i];
#pragma unroll
        for (int q = 0; q < 3; q++) C.gp[3 * i + q] = g[q] = C.gp[3 * i + q] + a * C.gpc[3 * i + q];
    }
    if (C.gp32) {   // precision 3: the FP32 copy the Rhie-Chow term reads, from the new values in registers
#pragma unroll
        for (int q = 0; q < 3; q++) C.gp32[3 * i + q] = narrow_f32(g[q]);
    }
}

__global__ void __launch_bounds__(kTile) k_update_faces(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(faces)
    if (i >= t.last) return;
    const int nf = C.nf, o = C.f_own[i], n = C.f_nb[i];
    if (n >= C.ne) return;
    const double wt = C.fgeo[FG_WT * nf + i], omw = 1.0 - wt;
    const double dip = omw * C.dc[o] + wt * C.dc[n];
    C.mip[i] = C.mip[i] - C.fprop[PR_RHOMADN * nf + i] * dip * (C.phic[n] - C.phic[o]);
}

// update_time, mod_physics.f90:101-112
__global__ void __launch_bounds__(kTile) k_update_time(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(cells)
    if (i < t.last) { C.u0[i] = C.u[i]; C.v0[i] = C.v[i]; C.w0[i] = C.w[i]; }
}
__global__ void __launch_bounds__(kTile) k_update_time_halo(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(halos)
    if (i < t.last) { const int h = C.ne + i; C.u0[h] = C.u[h]; C.v0[h] = C.v[h]; C.w0[h] = C.w[h]; }
}
__global__ void __launch_bounds__(kTile) k_copy_mip0(const CaseDev *__restrict__ cases, const Tile *__restrict__ tiles) {
    CFDL_PDL_WAIT();
    TILE_PROLOGUE(faces)
    if (i < t.last) C.mip0[i] = C.mip[i];
}

}  // namespace

void launch_bc(cfdl_ctx *ctx) {
    CFDL_LAUNCH("k_bc", k_bc, halos);
    launch_energy_bc(ctx);                  // mod_physics.f90:47
}
void ensure_face_props(cfdl_ctx *ctx) {
    bool dirty = false;
    for (HostCase *hc : ctx->cases) dirty |= hc->props_dirty;
    if (!dirty || ctx->capturing) return;
    CFDL_LAUNCH("k_face_props", k_face_props, faces);
    for (HostCase *hc : ctx->cases) hc->props_dirty = false;
}
static bool f32_assembly(const cfdl_ctx *ctx) { return ctx->cases[0]->cfg.precision == 3; }

void ensure_g32(cfdl_ctx *ctx) {
    bool stale = false;
    for (HostCase *hc : ctx->cases) stale |= hc->g32_stale;
    if (!stale || ctx->capturing || !f32_assembly(ctx)) return;
    CFDL_LAUNCH("k_narrow_grad", k_narrow_grad, cells);
    for (HostCase *hc : ctx->cases) hc->g32_stale = false;
}
void launch_coef_uvw(cfdl_ctx *ctx) {
    ensure_face_props(ctx);
    for (HostCase *hc : ctx->cases) hc->coef_is_pressure = false;
    if (f32_assembly(ctx)) {
        ensure_g32(ctx);
        CFDL_LAUNCH("k_coef_uvw_halo", k_coef_uvw_halo, halos);
        CFDL_LAUNCH("k_coef_uvw_face_f32", k_coef_uvw_face_f32, faces);
        CFDL_LAUNCH("k_coef_uvw_cell", k_coef_uvw_cell<true>, cells);
        return;
    }
    CFDL_LAUNCH("k_coef_uvw_halo", k_coef_uvw_halo, halos);
    CFDL_LAUNCH("k_coef_uvw_face", k_coef_uvw_face, faces);
    CFDL_LAUNCH("k_coef_uvw_cell", k_coef_uvw_cell<false>, cells);
}
void launch_grad(cfdl_ctx *ctx, int field) {
    if (field == 4 && f32_assembly(ctx)) CFDL_LAUNCH("k_grad3_f32", k_grad3_f32, cells);
    else if (field == 4) CFDL_LAUNCH("k_grad3", k_grad<3>, cells, 0);
    else if (field == 5) CFDL_LAUNCH("k_grad2", k_grad<2>, cells, 0);
    else CFDL_LAUNCH("k_grad1", k_grad<1>, cells, field);
}
void launch_calc_mip(cfdl_ctx *ctx, int rc) {
    ensure_face_props(ctx);
    if (rc && f32_assembly(ctx)) {
        ensure_g32(ctx);
        CFDL_LAUNCH("k_calc_mip", k_calc_mip_f32, faces, rc);
        return;
    }
    CFDL_LAUNCH("k_calc_mip", k_calc_mip, faces, rc);
}
void launch_coef_p_matrix(cfdl_ctx *ctx) {
    ensure_face_props(ctx);
    CFDL_LAUNCH("k_coef_p_face", k_coef_p_face, faces);
    CFDL_LAUNCH("k_coef_p_mat", k_coef_p_mat, cells);
}
void launch_coef_p_rhs(cfdl_ctx *ctx) {
    CFDL_LAUNCH("k_coef_p_rhs", k_coef_p_rhs, cells);
    for (HostCase *hc : ctx->cases) hc->coef_is_pressure = true;
}
void launch_coef_p(cfdl_ctx *ctx) {
    launch_coef_p_matrix(ctx);
    launch_coef_p_rhs(ctx);
}
void launch_adjust_pc(cfdl_ctx *ctx) {
    int n = (int)ctx->cases.size();
    if (n == 0) return;
    const bool p_ = ctx->prof && prof_wants(ctx, "k_save_pref");
    if (p_) prof_begin(ctx, "k_save_pref");
    k_save_pref<<<(n + 127) / 128, 128, 0, ctx->stream>>>(ctx->d_cases, n);
    if (p_) prof_end(ctx);
    ctx->launches++;
    CFDL_LAUNCH("k_adjust_pc", k_adjust_pc, cells);
}
void launch_update_uvwp(cfdl_ctx *ctx) {
    ensure_face_props(ctx);
    CFDL_LAUNCH("k_update_cells", k_update_cells, cells);
    CFDL_LAUNCH("k_update_faces", k_update_faces, faces);
}
void launch_update_time(cfdl_ctx *ctx) {
    CFDL_LAUNCH("k_update_time", k_update_time, cells);
    CFDL_LAUNCH("k_update_time_halo", k_update_time_halo, halos);
    CFDL_LAUNCH("k_copy_mip0", k_copy_mip0, faces);
    launch_energy_time(ctx, false);         // mod_physics.f90:111
}
void launch_set_mip0(cfdl_ctx *ctx) { CFDL_LAUNCH("k_copy_mip0", k_copy_mip0, faces); }

// precision 3 arrays of a case: FP32 gradients, the FP32 gradient stencil
// (narrowed from hf_G once) and the FP32 face planes (filled with the
// property planes, which are marked for recomputation)
int ensure_f32_assembly(HostCase *hc, cudaStream_t stream) {
    CaseDev &d = hc->dev;
    if (d.g32) return CFDL_OK;
    const size_t ne = hc->ne, nf = hc->nf, nG = 3 * (size_t)hc->W * ne;
    void *g = nullptr, *G = nullptr, *pf = nullptr;
    int st;
    // g32: the FP32 gradients of u, v, w [9 ne], then gp32 [3 ne] and d32 [ne]
    if ((st = case_alloc(hc, &g, 13 * ne * sizeof(float)))) return st;
    if ((st = case_alloc(hc, &G, nG * sizeof(float)))) return st;
    if ((st = case_alloc(hc, &pf, 11 * nf * sizeof(float)))) return st;
    const int tb = 256;
    k_narrow_array<<<(unsigned)((nG + tb - 1) / tb), tb, 0, stream>>>(d.hf_G, (float *)G, nG);
    if ((st = cuda_status(cudaGetLastError()))) return st;
    if ((st = cuda_status(cudaMemsetAsync(pf, 0, 11 * nf * sizeof(float), stream)))) return st;
    if ((st = cuda_status(cudaStreamSynchronize(stream)))) return st;
    d.g32 = (float *)g; d.G32 = (float *)G; d.fprop32 = (float *)pf;
    d.gp32 = d.g32 + 9 * ne; d.d32 = d.g32 + 12 * ne;
    hc->props_dirty = true;      // k_face_props fills fprop32
    hc->g32_stale = true;        // k_narrow_grad fills g32, gp32, d32 from gu, gv, gw, gp, d
    return CFDL_OK;
}

}  // namespace cfdl

extern "C" int cfdl_check_conversions(int n, unsigned *mismatches) {
    if (n <= 0 || !mismatches) return CFDL_ERR_INVALID;
    unsigned *d = nullptr;
    int st = cfdl::cuda_status(cudaMalloc(&d, 2 * sizeof(unsigned)));
    if (st) return st;
    st = cfdl::cuda_status(cudaMemset(d, 0, 2 * sizeof(unsigned)));
    if (!st) {
        cfdl::k_check_conversions<<<(n + 255) / 256, 256>>>(n, d);
        st = cfdl::cuda_status(cudaGetLastError());
    }
    if (!st) st = cfdl::cuda_status(cudaMemcpy(mismatches, d, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost));
    cudaFree(d);
    return st;
}
