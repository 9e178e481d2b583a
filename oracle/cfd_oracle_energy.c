/*
 * cfd_oracle_energy.c -- CPU oracle (test infrastructure only): restatement of
 * the reference's energy equation, src/equations/mod_energy.f90.
 *
 *   construct_energy          mod_energy.f90:14-47
 *   solve_energy              mod_energy.f90:59-80
 *   calc_coef_energy          mod_energy.f90:82-169
 *   lid, dirichlet0 (energy)  mod_energy.f90:173-212
 *   calc_temperature          src/modules/mod_properties.f90:214-221
 *   init_properties (cp, tc)  src/modules/mod_properties.f90:83-89
 *
 * The equation is for phi = cp*t: upwind advection by the face mass fluxes
 * mip of solve_uvwp, diffusion tc/cp with a deferred correction that carries
 * the difference between grad(t) and grad(phi)/cp, the transient rho*vol/dt,
 * and Dirichlet walls.  solve mode 0 uses solve_gs (sor = 1, 10x drop or nit
 * sweeps), mode 1 the tight BiCGStab of the momentum solves.
 */
#include "cfd_oracle_int.h"
#include <stdlib.h>
#include <string.h>
#include <math.h>

static inline double dot3e(const double *a, const double *b) { return a[0]*b[0] + a[1]*b[1] + a[2]*b[2]; }

int or_energy_init(ocase *c, double cp, double tc, double t_init, double t_lid, double t_wall) {
    if (!c->phys_ready) return -1;
    const size_t nc = (size_t)c->ne + c->nbf;
    o_energy_free(c);
    c->t = o_alloc(nc + 1, sizeof(double));
    c->ephi = o_alloc(nc + 1, sizeof(double));
    c->ephi0 = o_alloc(nc + 1, sizeof(double));
    c->gt = o_alloc(3 * nc + 1, sizeof(double));
    c->gephi = o_alloc(3 * nc + 1, sizeof(double));
    c->cp = o_alloc((size_t)c->ne + 1, sizeof(double));
    c->tc = o_alloc((size_t)c->ne + 1, sizeof(double));
    c->ebc_t = o_alloc((size_t)c->nintf_c2b + 1, sizeof(double));
    for (int e = 1; e <= c->ne; e++) { c->cp[e] = cp; c->tc[e] = tc; }
    /* eqn%t = 273; eqn%phi = eqn%t*prop%cp; phi0 = phi; grad = gt = 0.  The
     * reference multiplies the (ne+nbf)-long t by the ne-long cp; the halo
     * values it gets are overwritten by update_boundaries before any use, so
     * here the halos take the uniform cp. */
    for (size_t e = 1; e <= nc; e++) {
        c->t[e] = t_init;
        c->ephi[e] = c->t[e] * cp;
        c->ephi0[e] = c->ephi[e];
    }
    /* BC binding by name, as construct_uvwp's: 'top' -> lid, the rest -> dirichlet0 */
    for (int i = 1; i <= c->nintf_c2b; i++)
        c->ebc_t[i] = c->bcs[i].kind == BC_LID ? t_lid : t_wall;
    c->energy_on = 1;
    return 0;
}

void o_energy_free(ocase *c) {
    free(c->t); free(c->ephi); free(c->ephi0); free(c->gt); free(c->gephi);
    free(c->cp); free(c->tc); free(c->ebc_t);
    c->t = c->ephi = c->ephi0 = c->gt = c->gephi = c->cp = c->tc = c->ebc_t = NULL;
    c->energy_on = 0;
}

/* lid / dirichlet0 of the energy equation, mod_energy.f90:173-212 */
void o_energy_bc(ocase *c) {
    for (int i = 1; i <= c->nintf_c2b; i++) {
        const obc *bc = &c->bcs[i];
        if (bc->kind == BC_NONE) continue;
        for (int e = bc->esec1; e <= bc->esec2; e++) {
            int enb, lfnb;
            o_get_idx(abs(BS(c, e)), &enb, &lfnb);
            c->t[e] = c->ebc_t[i];
            c->ephi[e] = c->cp[enb] * c->t[e];
        }
    }
}

/* update_time's phys%energy%phi0 = phys%energy%phi, mod_physics.f90:111 */
void o_energy_time(ocase *c) {
    memcpy(c->ephi0 + 1, c->ephi + 1, ((size_t)c->ne + c->nbf) * sizeof(double));
}

/* calc_coef_energy, mod_energy.f90:82-169 */
void or_calc_coef_energy(ocase *c) {
    const double dt = c->cfg.dt;
    double *ap = c->ap, *anb = c->anb, *b = c->b;
    for (int e = 1; e <= c->ne; e++) {
        ap[e] = 0.;
        double sumf = 0., sumdefc = 0.;
        const double rp[3] = {c->xc[e], c->yc[e], c->zc[e]};
        for (int idx = c->ef2nb_idx[e]; idx <= c->ef2nb_idx[e+1] - 1; idx++) {
            anb[idx] = 0.;
            int enb, lfnb;
            o_get_idx(c->ef2nb1[idx], &enb, &lfnb);
            if (lfnb == 0) continue;
            int fg = c->ef2nb2[idx];
            const int sg = o_sgn(fg);
            fg = abs(fg);
            const int i = 3*fg - 2;
            const double area = sqrt(c->aip[i]*c->aip[i] + c->aip[i+1]*c->aip[i+1] + c->aip[i+2]*c->aip[i+2]);
            const double norm[3] = {sg*c->aip[i]/area, sg*c->aip[i+1]/area, sg*c->aip[i+2]/area};
            const double rip[3] = {c->rip[i], c->rip[i+1], c->rip[i+2]};
            const double rpnb[3] = {c->xc[enb], c->yc[enb], c->zc[enb]};
            const double dr[3] = {rpnb[0] - rp[0], rpnb[1] - rp[1], rpnb[2] - rp[2]};
            const double wt = o_vec_weight(rip, rp, rpnb);
            /* advection: inward flux, upwind */
            const double f = -sg * c->mip[fg];
            const double fnb = fmax(f, 0.);
            sumf = sumf + f;
            /* diffusion */
            const double tci = (1. - wt)*c->tc[e] + wt*c->tc[enb];
            const double cpi = (1. - wt)*c->cp[e] + wt*c->cp[enb];
            const double d = tci / cpi / dot3e(dr, norm) * area;
            double ghi[3], gti[3];
            for (int k = 0; k < 3; k++) {
                ghi[k] = (1. - wt)*c->gephi[3*e-2+k] + wt*c->gephi[3*enb-2+k];
                gti[k] = (1. - wt)*c->gt[3*e-2+k] + wt*c->gt[3*enb-2+k];
            }
            sumdefc = sumdefc + tci*area*(dot3e(gti, norm) - dot3e(ghi, norm)/cpi);
            anb[idx] = d + fnb;
            ap[e] = ap[e] + d + fnb;
        }
        const double ap0 = c->rho[e]*c->vol[e]/dt;
        ap[e] = ap[e] + ap0;
        b[e] = ap0*c->ephi0[e] + sumf*c->ephi[e] + sumdefc;
    }
    /* boundary conditions: every bound energy BC is 'dirichlet' */
    for (int ibc = 1; ibc <= c->nintf_c2b; ibc++) {
        const obc *bc = &c->bcs[ibc];
        if (bc->kind == BC_NONE) continue;
        for (int enb = bc->esec1; enb <= bc->esec2; enb++) {
            int e, lf;
            o_get_idx(abs(BS(c, enb)), &e, &lf);
            const int idx = c->ef2nb_idx[e] + lf - 1;
            const int fg = c->ef2nb2[idx];            /* outward on the boundary */
            const int i = 3*fg - 2;
            const double area = sqrt(c->aip[i]*c->aip[i] + c->aip[i+1]*c->aip[i+1] + c->aip[i+2]*c->aip[i+2]);
            const double norm[3] = {c->aip[i]/area, c->aip[i+1]/area, c->aip[i+2]/area};
            const double dr[3] = {c->xc[enb] - c->xc[e], c->yc[enb] - c->yc[e], c->zc[enb] - c->zc[e]};
            const double ds = dot3e(dr, norm);
            const double f = 0.;
            const double d = c->tc[e]*area/ds/c->cp[e];
            ap[e] = ap[e] + d + f;
            anb[idx] = anb[idx] + d + f;
        }
    }
}

/* solve_energy, mod_energy.f90:59-80 */
void or_solve_energy(ocase *c, or_stats *st) {
    if (!c->energy_on) return;
    o_calc_grad(c, c->t, c->gt);
    o_calc_grad(c, c->ephi, c->gephi);
    or_calc_coef_energy(c);
    int it; double ri, rf, rm = 0.;
    if (c->cfg.mode == 0)
        o_solve_gs(0, c->ephi, c->ap, c->anb, c->b, c->ef2nb_idx, c->ef2nb1, c->ne, c->cfg.nit, &it, &ri, &rf, &rm);
    else
        it = o_bicgstab(c, c->ap, c->anb, c->b, c->ephi, c->cfg.tight_rtol, c->cfg.tight_maxit, &ri, &rf);
    /* calc_temperature, mod_properties.f90:214-221 */
    for (int e = 1; e <= c->ne; e++) c->t[e] = c->ephi[e] / c->cp[e];
    if (st) { st->it_e = it; st->res_e[0] = ri; st->res_e[1] = rf; st->res_e[2] = rm; }
}
