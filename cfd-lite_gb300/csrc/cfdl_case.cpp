// cfdl_case.cpp -- host side of a case: validation of the reference-layout
// mesh arrays, conversion to the device layout (ELL half-faces, face
// geometry planes, halo tables), geometry precomputation, and the tile work
// lists.  Compiled without floating-point contraction.
//
// The precomputed face quantities are the sub-expressions the reference
// evaluates per half-face in calc_coef_uvw, calc_coef_p, calc_mip and
// update_uvwp (src/equations/mod_uvwp.f90:161-436): area, unit normal, wt
// (vec_weight, src/modules/mod_util.f90:729-743), dr, ds, the projected
// distance dr_p/ds_p, and dr.n.  They depend only on the mesh, so the device
// never recomputes a square root or a division for them.  The least-squares
// gradient of calc_grad (src/modules/mod_solver.f90:40-81) is folded into a
// per-half-face stencil A^-1 * (dr/|dr|^2), with A inverted by matinv3
// (mod_solver.f90:8-38) including its trace fallback.
#include "cfdl_internal.h"
#include "cfdl_amg.h"
#include "cfdl_par.h"
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cfloat>
#include <cstring>
#include <new>

namespace cfdl {

void delete_amg(HostCase *hc) {
    delete hc->amg;
    hc->amg = nullptr;
}

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return CFDL_OK;
    if (e == cudaErrorMemoryAllocation) return CFDL_ERR_OOM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return CFDL_ERR_NO_DEVICE;
    return CFDL_ERR_CUDA;
}

int case_alloc(HostCase *hc, void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) { *p = nullptr; cudaGetLastError(); return cuda_status(e); }
    hc->allocs.push_back(*p);
    hc->bytes += bytes;
    return CFDL_OK;
}

void destroy_case(HostCase *hc) {
    if (!hc) return;
    for (void *p : hc->allocs) cudaFree(p);
    for (void *p : hc->amg_allocs) cudaFree(p);
    delete_amg(hc);
    delete hc;
}

void free_worklist(WorkList &wl) {
    cudaFree(wl.d_tiles); cudaFree(wl.d_case_first); cudaFree(wl.d_case_ntiles);
    wl.d_tiles = nullptr; wl.d_case_first = nullptr; wl.d_case_ntiles = nullptr;
    wl.ntiles = 0;
}

// Tile list over per-case entity counts (sizes[c] = 0 leaves case c out).
int build_worklist(cfdl_ctx *ctx, WorkList &wl, const std::vector<int> &sizes, int tile) {
    free_worklist(wl);
    wl.h_tiles.clear(); wl.case_first.clear(); wl.case_ntiles.clear();
    for (size_t c = 0; c < sizes.size(); c++) {
        wl.case_first.push_back((int)wl.h_tiles.size());
        int cnt = 0;
        for (int s = 0; s < sizes[c]; s += tile, cnt++)
            wl.h_tiles.push_back({(int)c, s, std::min(sizes[c], s + tile), (tile + kTile - 1) / kTile});
        wl.case_ntiles.push_back(cnt);
    }
    wl.ntiles = (int)wl.h_tiles.size();
    size_t nt = std::max<size_t>(1, wl.h_tiles.size()), ncs = std::max<size_t>(1, sizes.size());
    int st;
    if ((st = cuda_status(cudaMalloc(&wl.d_tiles, nt * sizeof(Tile))))) return st;
    if ((st = cuda_status(cudaMalloc(&wl.d_case_first, ncs * sizeof(int))))) return st;
    if ((st = cuda_status(cudaMalloc(&wl.d_case_ntiles, ncs * sizeof(int))))) return st;
    if (!wl.h_tiles.empty()) {
        if ((st = cuda_status(cudaMemcpy(wl.d_tiles, wl.h_tiles.data(), wl.h_tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice)))) return st;
        if ((st = cuda_status(cudaMemcpy(wl.d_case_first, wl.case_first.data(), wl.case_first.size() * sizeof(int), cudaMemcpyHostToDevice)))) return st;
        if ((st = cuda_status(cudaMemcpy(wl.d_case_ntiles, wl.case_ntiles.data(), wl.case_ntiles.size() * sizeof(int), cudaMemcpyHostToDevice)))) return st;
    }
    (void)ctx;
    return CFDL_OK;
}

void apply_config(HostCase *hc, const cfdl_config *cfg) {
    hc->cfg = *cfg;
    CaseDev &d = hc->dev;
    d.dt = cfg->dt; d.alpha_u = cfg->alpha_u; d.alpha_p = cfg->alpha_p;
    d.rtol_u = cfg->rtol_u; d.rtol_p = cfg->rtol_p; d.tight_rtol = cfg->tight_rtol;
    d.nit = cfg->nit; d.solve_mode = cfg->solve_mode; d.tight_maxit = cfg->tight_maxit;
    d.precision = cfg->precision;
    d.precond = cfg->precond;
    d.steady = std::isinf(cfg->dt) ? 1 : 0;
    d.rdt = d.steady ? 0.0 : 1.0 / cfg->dt;
    d.ralpha_u = 1.0 / cfg->alpha_u;
}

namespace {

inline void get_idx(int idx, int &g, int &s) { s = (int)((unsigned)idx & 31u); g = (int)((unsigned)idx >> 5); }

// matinv3, src/modules/mod_solver.f90:8-38
void matinv3(const double A[3][3], double B[3][3]) {
    double det = (A[0][0]*A[1][1]*A[2][2] - A[0][0]*A[1][2]*A[2][1]
                - A[0][1]*A[1][0]*A[2][2] + A[0][1]*A[1][2]*A[2][0]
                + A[0][2]*A[1][0]*A[2][1] - A[0][2]*A[1][1]*A[2][0]);
    if (std::fabs(det) > DBL_MIN) {
        double di = 1.0 / det;
        B[0][0] = +di * (A[1][1]*A[2][2] - A[1][2]*A[2][1]);
        B[1][0] = -di * (A[1][0]*A[2][2] - A[1][2]*A[2][0]);
        B[2][0] = +di * (A[1][0]*A[2][1] - A[1][1]*A[2][0]);
        B[0][1] = -di * (A[0][1]*A[2][2] - A[0][2]*A[2][1]);
        B[1][1] = +di * (A[0][0]*A[2][2] - A[0][2]*A[2][0]);
        B[2][1] = -di * (A[0][0]*A[2][1] - A[0][1]*A[2][0]);
        B[0][2] = +di * (A[0][1]*A[1][2] - A[0][2]*A[1][1]);
        B[1][2] = -di * (A[0][0]*A[1][2] - A[0][2]*A[1][0]);
        B[2][2] = +di * (A[0][0]*A[1][1] - A[0][1]*A[1][0]);
    } else {
        std::memset(B, 0, 9 * sizeof(double));
        double di = 1.0 / (A[0][0] + A[1][1] + A[2][2]);
        B[0][0] = di; B[1][1] = di; B[2][2] = di;
    }
}

double vec_weight(const double *r0, const double *r1, const double *r2) {
    double ra[3], rb[3];
    for (int i = 0; i < 3; i++) { ra[i] = r1[i] - r0[i]; rb[i] = r2[i] - r0[i]; }
    double la = std::sqrt(ra[0]*ra[0] + ra[1]*ra[1] + ra[2]*ra[2]);
    double lb = std::sqrt(rb[0]*rb[0] + rb[1]*rb[1] + rb[2]*rb[2]);
    return la + lb > 0. ? la / (la + lb) : 0.5;
}

template <class T, class A> int upload(HostCase *hc, T **dptr, const std::vector<T, A> &h) {
    int st = case_alloc(hc, (void **)dptr, h.size() * sizeof(T));
    if (st) return st;
    return cuda_status(cudaMemcpy(*dptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}
template <class T> int zeros(HostCase *hc, T **dptr, size_t n) {
    int st = case_alloc(hc, (void **)dptr, n * sizeof(T));
    if (st) return st;
    return cuda_status(cudaMemset(*dptr, 0, n * sizeof(T)));
}

int upload_all(HostCase *hc, const cfdl_config *cfg, const FillVec<int> &hf_nb, const FillVec<int> &hf_fc,
               const FillVec<double> &hf_G, const FillVec<int> &f_own, const FillVec<int> &f_nb,
               const FillVec<double> &fgeo, const std::vector<int> &h_own, const std::vector<int> &h_face,
               const std::vector<int> &h_kind, const std::vector<double> &h_vel, const std::vector<double> &vol) {
    CaseDev &d = hc->dev;
    const int ne = hc->ne, nf = hc->nf, nbf = hc->nbf, W = hc->W, nc = ne + nbf;
    d.ne = ne; d.nbf = nbf; d.nf = nf; d.W = W;
    int st;
    if ((st = upload(hc, (int **)&d.hf_nb, hf_nb))) return st;
    if ((st = upload(hc, (int **)&d.hf_fc, hf_fc))) return st;
    if ((st = upload(hc, (double **)&d.hf_G, hf_G))) return st;
    if ((st = upload(hc, (int **)&d.f_own, f_own))) return st;
    if ((st = upload(hc, (int **)&d.f_nb, f_nb))) return st;
    if ((st = upload(hc, (double **)&d.fgeo, fgeo))) return st;
    if ((st = upload(hc, (int **)&d.h_own, h_own))) return st;
    if ((st = upload(hc, (int **)&d.h_face, h_face))) return st;
    if ((st = upload(hc, (int **)&d.h_kind, h_kind))) return st;
    if ((st = upload(hc, (double **)&d.h_vel, h_vel))) return st;
    if ((st = upload(hc, (double **)&d.vol, vol))) return st;
    double **cellf[] = {&d.u, &d.v, &d.w, &d.p, &d.u0, &d.v0, &d.w0, &d.phic};
    for (double **pp : cellf) if ((st = zeros(hc, pp, (size_t)nc))) return st;
    double **gradf[] = {&d.gu, &d.gv, &d.gw, &d.gp, &d.gpc};
    for (double **pp : gradf) if ((st = zeros(hc, pp, 3 * (size_t)nc))) return st;
    if ((st = zeros(hc, &d.mip, (size_t)nf))) return st;
    if ((st = zeros(hc, &d.mip0, (size_t)nf))) return st;
    double **ef[] = {&d.bu, &d.bv, &d.bw, &d.d, &d.dc, &d.rho, &d.mu, &d.ap, &d.b};
    for (double **pp : ef) if ((st = zeros(hc, pp, (size_t)ne))) return st;
    if ((st = zeros(hc, &d.anb, (size_t)W * ne))) return st;
    if ((st = zeros(hc, &d.anb_p, (size_t)W * ne))) return st;
    if ((st = zeros(hc, &d.ap_p, (size_t)ne))) return st;
    if ((st = zeros(hc, &d.rap_p, (size_t)ne))) return st;
    if ((st = zeros(hc, &d.fanb_p, (size_t)W * ne))) return st;
    if ((st = zeros(hc, &d.fdiag_p, (size_t)ne))) return st;
    if ((st = zeros(hc, &d.frap_p, (size_t)ne))) return st;
    if ((st = zeros(hc, &d.fdiff, (size_t)nf))) return st;
    if ((st = zeros(hc, &d.fS, 3 * (size_t)nf))) return st;
    if ((st = zeros(hc, &d.hbc, 4 * (size_t)nbf))) return st;
    if ((st = zeros(hc, &d.fprop, (size_t)PR_N * nf))) return st;
    double **kv[] = {&d.kr, &d.krh, &d.kp, &d.kph, &d.kv, &d.ks, &d.ksh, &d.kt};
    for (double **pp : kv) if ((st = zeros(hc, pp, 3 * (size_t)ne))) return st;
    float **fv[] = {&d.fr, &d.fz, &d.fp, &d.fq, &d.fx, &d.fdiag, &d.ft, &d.frap};
    for (float **pp : fv) if ((st = zeros(hc, pp, (size_t)ne))) return st;
    if ((st = zeros(hc, &d.fanb, (size_t)W * ne))) return st;
    if ((st = zeros(hc, &d.rap, (size_t)ne))) return st;
    if ((st = zeros(hc, &d.sc, 1))) return st;
    if ((st = zeros(hc, &d.counters, 16))) return st;
    std::vector<double> rho(ne, cfg->rho), mu(ne, cfg->mu);
    if ((st = cuda_status(cudaMemcpy(d.rho, rho.data(), ne * sizeof(double), cudaMemcpyHostToDevice)))) return st;
    return cuda_status(cudaMemcpy(d.mu, mu.data(), ne * sizeof(double), cudaMemcpyHostToDevice));
}

}  // namespace

CasePrep::~CasePrep() { delete amg; }

void CasePrep::release_tables() {
    std::vector<int>().swap(ef2nb_idx); FillVec<int>().swap(hf_nb); FillVec<int>().swap(hf_fc);
    FillVec<int>().swap(f_own); FillVec<int>().swap(f_nb); std::vector<int>().swap(h_own);
    std::vector<int>().swap(h_face); std::vector<int>().swap(h_kind);
    FillVec<double>().swap(hf_G); FillVec<double>().swap(fgeo); std::vector<double>().swap(h_vel);
    std::vector<double>().swap(vol); std::vector<double>().swap(h_temp);
    delete amg;
    amg = nullptr;
}

// Host half of create_case: validates the reference-layout arrays and builds
// every device-layout table.  Touches no device state, so it may run on any
// host thread (the serving loop prepares meshes ahead of admission).
int prepare_case(const cfdl_mesh *m, CasePrep *p) {
    if (!m || !p) return CFDL_ERR_INVALID;
    const int ne = m->ne, nf = m->nf, nbf = m->nbf;
    if (ne <= 0 || nf <= 0 || nbf < 0 || !m->ef2nb1 || !m->ef2nb2 || !m->ef2nb_idx || !m->s2g ||
        (nbf > 0 && !m->bs) || !m->aip || !m->rip || !m->xc || !m->yc || !m->zc || !m->vol)
        return CFDL_ERR_INVALID;
    if ((long long)ne + nbf >= (1LL << 26)) return CFDL_ERR_INVALID;
    const int H = 2 * nf - nbf;
    if (H <= 0 || m->ef2nb_idx[0] != 1 || m->ef2nb_idx[ne] != H + 1) return CFDL_ERR_INVALID;
    const int nc = ne + nbf;
    try {
        p->ne = ne; p->nf = nf; p->nbf = nbf; p->H = H;
        p->ef2nb_idx.assign(m->ef2nb_idx, m->ef2nb_idx + ne + 1);
        int W = 0;
        for (int e = 0; e < ne; e++) {
            int cnt = m->ef2nb_idx[e + 1] - m->ef2nb_idx[e];
            if (cnt <= 0 || cnt > kMaxW) return CFDL_ERR_INVALID;
            W = std::max(W, cnt);
        }
        p->W = W;
        // ---- ELL half-faces + validation of every index ----
        // In parallel over cells: each cell writes its own slots, and the
        // owner side of each face records (owner, neighbour).  Two owner
        // claims on one face (an invalid mesh) are found by the second pass:
        // every owner-side half-face must be the one recorded.
        FillVec<int> &hf_nb = p->hf_nb, &hf_fc = p->hf_fc, &f_own = p->f_own, &f_nb = p->f_nb;
        hf_nb.resize((size_t)W * ne); hf_fc.resize((size_t)W * ne);
        f_own.resize(nf); f_nb.resize(nf);
        parallel_for(nf, [&](long fb, long fe) {
            for (long f = fb; f < fe; f++) { f_own[f] = -1; f_nb[f] = -1; }
        });
        std::atomic<int> bad{0};
        parallel_for(ne, [&](long cb, long ce) {
            for (int e = (int)cb; e < (int)ce; e++) {
                const int b0 = m->ef2nb_idx[e], cnt = m->ef2nb_idx[e + 1] - b0;
                for (int k = 0; k < W; k++) {
                    const size_t sl = (size_t)k * ne + e;
                    hf_nb[sl] = -1; hf_fc[sl] = 0;          // padding past the cell's faces
                    if (k >= cnt) continue;
                    int enb, lfnb;
                    get_idx(m->ef2nb1[b0 + k - 1], enb, lfnb);
                    const int fg = m->ef2nb2[b0 + k - 1];
                    const int fa = fg >= 0 ? fg : -fg;
                    if (enb < 1 || enb > nc || fa < 1 || fa > nf || (lfnb == 0) != (enb > ne)) {
                        bad.store(1, std::memory_order_relaxed);
                        continue;
                    }
                    hf_nb[sl] = enb - 1;
                    hf_fc[sl] = fg > 0 ? fa - 1 : ~(fa - 1);
                    if (fg > 0) {
                        __atomic_store_n(&f_own[fa - 1], e, __ATOMIC_RELAXED);
                        __atomic_store_n(&f_nb[fa - 1], enb - 1, __ATOMIC_RELAXED);
                    }
                }
            }
        });
        if (bad.load()) return CFDL_ERR_INVALID;
        parallel_for(ne, [&](long cb, long ce) {
            for (int e = (int)cb; e < (int)ce; e++)
                for (int idx = m->ef2nb_idx[e]; idx < m->ef2nb_idx[e + 1]; idx++) {
                    const int fg = m->ef2nb2[idx - 1];
                    const int k = idx - m->ef2nb_idx[e];
                    if (fg > 0 && (f_own[fg - 1] != e || f_nb[fg - 1] != hf_nb[(size_t)k * ne + e]))
                        bad.store(1, std::memory_order_relaxed);
                }
        });
        if (bad.load()) return CFDL_ERR_INVALID;
        for (int f = 0; f < nf; f++) {
            if (f_own[f] < 0) return CFDL_ERR_INVALID;
            int e, lf;
            get_idx(m->s2g[f], e, lf);           // s2g names the owner side
            if (e - 1 != f_own[f]) return CFDL_ERR_INVALID;
        }
        // ---- halos and boundary conditions ----
        std::vector<int> &h_own = p->h_own, &h_face = p->h_face, &h_kind = p->h_kind;
        std::vector<double> &h_vel = p->h_vel;
        h_own.assign(std::max(nbf, 1), 0); h_face.assign(std::max(nbf, 1), 0); h_kind.assign(std::max(nbf, 1), 0);
        h_vel.assign(3 * (size_t)std::max(nbf, 1), 0.0);
        for (int h = 0; h < nbf; h++) {
            int b = m->bs[h] < 0 ? -m->bs[h] : m->bs[h], e, lf;
            get_idx(b, e, lf);
            if (e < 1 || e > ne || lf < 1 || lf > m->ef2nb_idx[e] - m->ef2nb_idx[e - 1]) return CFDL_ERR_INVALID;
            int fg = m->ef2nb2[m->ef2nb_idx[e - 1] + lf - 1 - 1];
            if (fg < 1 || f_nb[fg - 1] != ne + h) return CFDL_ERR_INVALID;
            h_own[h] = e - 1; h_face[h] = fg - 1;
        }
        for (int bc = 0; bc < m->nbc; bc++) {
            int a = m->bc_esec[2 * bc], z = m->bc_esec[2 * bc + 1];
            if (a < ne + 1 || z > nc || a > z + 1) return CFDL_ERR_INVALID;
            int kind = m->bc_kind[bc];
            if (kind != CFDL_BC_WALL && kind != CFDL_BC_SYMMETRY) return CFDL_ERR_INVALID;
            for (int el = a; el <= z; el++) {
                int h = el - ne - 1;
                h_kind[h] = kind;
                for (int q = 0; q < 3; q++) h_vel[3 * (size_t)h + q] = m->bc_vel[3 * bc + q];
            }
        }
        // energy wall temperatures, when the mesh carries them
        p->h_temp.clear();
        if (m->bc_temp) {
            p->h_temp.assign(std::max(nbf, 1), 0.0);
            for (int bc = 0; bc < m->nbc; bc++)
                for (int el = m->bc_esec[2 * bc]; el <= m->bc_esec[2 * bc + 1]; el++) p->h_temp[el - ne - 1] = m->bc_temp[bc];
        }
        // ---- face geometry planes ----
        FillVec<double> &fgeo = p->fgeo;
        fgeo.resize((size_t)FG_N * nf);       // every plane of every face is written below
        auto G = [&](int plane, int f) -> double & { return fgeo[(size_t)plane * nf + f]; };
        parallel_for(nf, [&](long fb, long fe) {
        for (int f = (int)fb; f < (int)fe; f++) {
            int e = f_own[f], n = f_nb[f];
            const double *a = &m->aip[3 * (size_t)f], *ri = &m->rip[3 * (size_t)f];
            double rp[3] = {m->xc[e], m->yc[e], m->zc[e]}, rn[3] = {m->xc[n], m->yc[n], m->zc[n]};
            double area = std::sqrt(a[0]*a[0] + a[1]*a[1] + a[2]*a[2]);
            double nrm[3] = {a[0] / area, a[1] / area, a[2] / area};
            double dr[3] = {rn[0] - rp[0], rn[1] - rp[1], rn[2] - rp[2]};
            double ds = std::sqrt(dr[0]*dr[0] + dr[1]*dr[1] + dr[2]*dr[2]);
            G(FG_AX, f) = a[0]; G(FG_AY, f) = a[1]; G(FG_AZ, f) = a[2];
            G(FG_AREA, f) = area;
            G(FG_DRX, f) = dr[0]; G(FG_DRY, f) = dr[1]; G(FG_DRZ, f) = dr[2];
            G(FG_ADS, f) = area / ds;
            // boundary faces too: the energy equation's wall coefficient uses it
            const double dn = dr[0]*nrm[0] + dr[1]*nrm[1] + dr[2]*nrm[2];
            G(FG_ADN, f) = area / dn;
            if (n >= ne) {
                // boundary faces: no interpolation weight, no non-orthogonal terms
                G(FG_WT, f) = 0.0;
                for (int q = 0; q < 3; q++) G(FG_ADRX + q, f) = G(FG_EX + q, f) = 0.0;
            } else {
                G(FG_WT, f) = vec_weight(ri, rp, rn);
                double drip[3], t, rpp[3], rnp[3], drp[3];
                for (int q = 0; q < 3; q++) drip[q] = ri[q] - rp[q];
                t = drip[0]*nrm[0] + drip[1]*nrm[1] + drip[2]*nrm[2];
                for (int q = 0; q < 3; q++) rpp[q] = ri[q] - t * nrm[q];
                for (int q = 0; q < 3; q++) drip[q] = ri[q] - rn[q];
                t = drip[0]*nrm[0] + drip[1]*nrm[1] + drip[2]*nrm[2];
                for (int q = 0; q < 3; q++) rnp[q] = ri[q] - t * nrm[q];
                for (int q = 0; q < 3; q++) drp[q] = rnp[q] - rpp[q];
                double dsp = std::sqrt(drp[0]*drp[0] + drp[1]*drp[1] + drp[2]*drp[2]);
                for (int q = 0; q < 3; q++) {
                    G(FG_ADRX + q, f) = area * dr[q] / ds;
                    G(FG_EX + q, f) = area * (drp[q] / dsp - dr[q] / ds);
                }
            }
        }
        });
        // ---- least-squares gradient stencil ----
        FillVec<double> &hf_G = p->hf_G;
        hf_G.resize(3 * (size_t)W * ne);      // every slot written below (0 past a cell's faces)
        parallel_for(ne, [&](long cb, long ce) {
        for (int e = (int)cb; e < (int)ce; e++) {
            double A[3][3] = {{0}}, Ai[3][3], wdr[kMaxW][3];
            int cnt = m->ef2nb_idx[e + 1] - m->ef2nb_idx[e];
            for (int k = 0; k < cnt; k++) {
                int n = hf_nb[(size_t)k * ne + e];
                double dr[3] = {m->xc[n] - m->xc[e], m->yc[n] - m->yc[e], m->zc[n] - m->zc[e]};
                double wt = 1. / (dr[0]*dr[0] + dr[1]*dr[1] + dr[2]*dr[2]);
                for (int q = 0; q < 3; q++) wdr[k][q] = wt * dr[q];
                A[0][0] = A[0][0] + wt*dr[0]*dr[0];
                A[0][1] = A[0][1] + wt*dr[0]*dr[1];
                A[0][2] = A[0][2] + wt*dr[0]*dr[2];
                A[1][1] = A[1][1] + wt*dr[1]*dr[1];
                A[1][2] = A[1][2] + wt*dr[1]*dr[2];
                A[2][2] = A[2][2] + wt*dr[2]*dr[2];
            }
            A[1][0] = A[0][1]; A[2][0] = A[0][2]; A[2][1] = A[1][2];
            matinv3(A, Ai);
            for (int k = 0; k < W; k++)
                for (int q = 0; q < 3; q++)
                    hf_G[((size_t)q * W + k) * ne + e] =
                        k < cnt ? Ai[q][0]*wdr[k][0] + Ai[q][1]*wdr[k][1] + Ai[q][2]*wdr[k][2] : 0.0;
        }
        });
        p->vol.assign(m->vol, m->vol + ne);
    } catch (const std::bad_alloc &) {
        return CFDL_ERR_OOM;
    }
    return CFDL_OK;
}

// Device half: allocates and uploads the case (and a host-built multigrid
// hierarchy, whose ownership moves to the case).
int upload_case(CasePrep &p, const cfdl_config *cfg, HostCase **out) {
    *out = nullptr;
    if (!cfg) return CFDL_ERR_INVALID;
    HostCase *hc = new (std::nothrow) HostCase;
    if (!hc) return CFDL_ERR_OOM;
    int st;
    try {
        hc->ne = p.ne; hc->nf = p.nf; hc->nbf = p.nbf; hc->H = p.H; hc->W = p.W;
        hc->ef2nb_idx = p.ef2nb_idx;
        hc->h_temp = p.h_temp;
        st = upload_all(hc, cfg, p.hf_nb, p.hf_fc, p.hf_G, p.f_own, p.f_nb, p.fgeo, p.h_own, p.h_face, p.h_kind,
                        p.h_vel, p.vol);
        if (!st && p.amg) {
            st = upload_case_amg(hc, p.amg);   // takes the hierarchy
            p.amg = nullptr;
        }
        if (!st && cfg->precision == 3) st = ensure_f32_assembly(hc, 0);
        if (st) { destroy_case(hc); return st; }
        apply_config(hc, cfg);
    } catch (const std::bad_alloc &) {
        destroy_case(hc);
        return CFDL_ERR_OOM;
    }
    *out = hc;
    return CFDL_OK;
}

int create_case(cfdl_ctx *ctx, const cfdl_mesh *m, const cfdl_config *cfg, HostCase **out) {
    *out = nullptr;
    if (!cfg) return CFDL_ERR_INVALID;
    CasePrep p;
    int st = prepare_case(m, &p);
    if (st) return st;
    (void)ctx;
    return upload_case(p, cfg, out);
}

// Tile work lists over every case of the context.
int rebuild_worklists(cfdl_ctx *ctx) {
    std::vector<int> nc, nfc, nh;
    for (const HostCase *hc : ctx->cases) { nc.push_back(hc->ne); nfc.push_back(hc->nf); nh.push_back(hc->nbf); }
    int st;
    if ((st = build_worklist(ctx, ctx->cells, nc))) return st;
    if ((st = build_worklist(ctx, ctx->faces, nfc))) return st;
    if ((st = build_worklist(ctx, ctx->facesv, nfc, kTile * kFaceVec))) return st;
    if ((st = build_worklist(ctx, ctx->halos, nh))) return st;
    if ((st = build_worklist(ctx, ctx->cellsv, nc, kTile * ctx->vec))) return st;
    if ((st = build_worklist(ctx, ctx->cellse, nc, kTile * ctx->en_vec))) return st;
    for (auto &wl : ctx->amg_cells) free_worklist(wl);
    for (auto &wl : ctx->amg_smooth) free_worklist(wl);
    for (auto &wl : ctx->amg_gcells) free_worklist(wl);
    for (auto &wl : ctx->amg_gsmooth) free_worklist(wl);
    for (auto &wl : ctx->amg_restr) free_worklist(wl);
    for (auto &wl : ctx->amg_grestr) free_worklist(wl);
    ctx->amg_cells.clear(); ctx->amg_smooth.clear(); ctx->amg_gcells.clear(); ctx->amg_gsmooth.clear();
    ctx->amg_restr.clear(); ctx->amg_grestr.clear(); ctx->amg_lmax = -1;
    destroy_graph(ctx);   // captured launch arguments refer to the old lists
    int need = std::max({ctx->cells.ntiles, ctx->faces.ntiles, ctx->halos.ntiles, 1});
    if (need > ctx->partials_cap) {
        cudaFree(ctx->d_partials);
        ctx->d_partials = nullptr;
        int st = cuda_status(cudaMalloc(&ctx->d_partials, (size_t)need * kNPart * sizeof(double)));
        if (st) { ctx->partials_cap = 0; return st; }
        ctx->partials_cap = need;
    }
    int ncases = (int)ctx->cases.size();
    if (ncases > ctx->h_flags_cap) {
        cudaFreeHost(ctx->h_flags); cudaFree(ctx->d_flags);
        ctx->h_flags = nullptr; ctx->d_flags = nullptr;
        int cap = std::max(ncases, 8);
        int st = cuda_status(cudaMallocHost(&ctx->h_flags, (size_t)cap * 4 * sizeof(int)));
        if (!st) st = cuda_status(cudaMalloc(&ctx->d_flags, (size_t)cap * 4 * sizeof(int)));
        if (st) { ctx->h_flags_cap = 0; return st; }
        ctx->h_flags_cap = cap;
    }
    return upload_case_table(ctx);
}

int upload_case_table(cfdl_ctx *ctx) {
    int n = (int)ctx->cases.size();
    if (n > ctx->d_cases_cap) {
        cudaFree(ctx->d_cases);
        ctx->d_cases = nullptr;
        int cap = std::max(n, 8);
        int st = cuda_status(cudaMalloc(&ctx->d_cases, (size_t)cap * sizeof(CaseDev)));
        if (st) { ctx->d_cases_cap = 0; return st; }
        ctx->d_cases_cap = cap;
    }
    std::vector<CaseDev> tab(n);
    for (int c = 0; c < n; c++) tab[c] = ctx->cases[c]->dev;
    if (n == 0) return CFDL_OK;
    int st = cuda_status(cudaMemcpyAsync(ctx->d_cases, tab.data(), n * sizeof(CaseDev), cudaMemcpyHostToDevice, ctx->stream));
    if (st) return st;
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

}  // namespace cfdl
