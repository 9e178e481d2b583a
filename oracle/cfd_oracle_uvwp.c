/*
 * cfd_oracle_uvwp.c -- CPU oracle (test infrastructure only): restatement of
 * one SIMPLE outer iteration of the reference (solve_uvwp) and its callers.
 *
 *   construct_physics / update_boundaries / update_time
 *                               src/modules/mod_physics.f90:38-112
 *   make_bc                     src/modules/mod_eqn_setup.f90:46-68
 *   construct_uvwp, solve_uvwp, adjust_pc, calc_coef_uvw, calc_coef_p,
 *   update_uvwp, calc_mip, lid, dirichlet0, symmetry
 *                               src/equations/mod_uvwp.f90:20-570
 *   matinv3, calc_grad, multi_subdomain_solver, smoother_gs, calc_residual,
 *   solve_gs, solve             src/modules/mod_solver.f90:8-344
 *   assemble_coef, update_halos, update_phi
 *                               src/modules/mod_subdomains.f90:162-229
 *   vec_weight                  src/modules/mod_util.f90:729-743
 *
 * Two solve modes.  mode 0 ("ref") is the literal reference: symmetric
 * Gauss-Seidel to a 10x residual drop (momentum) and the 4-block Jacobi /
 * SSOR(1.02) pressure solve with its residual-accumulation quirk.  mode 1
 * ("tight") keeps the discretisation and replaces each inner solve by a Krylov
 * solve to ||r||2 <= tight_rtol*||b||2, so that the iterates no longer depend
 * on the sweep order; it is the parity mode for the GPU.
 *
 * Extensions (absent from the reference, identical in the GPU library):
 * rho, mu, lid speed, dt are parameters; dt = INFINITY gives a steady form
 * (ap0 = 0 and the Rhie-Chow transient term vanish through IEEE arithmetic);
 * alpha_u applies Patankar implicit relaxation after the boundary loop of
 * calc_coef_uvw (apr = ap/alpha_u, b += (1-alpha_u)*apr*phi) and alpha_p
 * scales the pressure update p += alpha_p*pc, gp += alpha_p*gpc.
 */
#define _POSIX_C_SOURCE 199309L
#include "cfd_oracle_int.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* host threads the parallel loops use (1 when built without OpenMP) */
int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* threads for the parallel loops from now on (no effect without OpenMP) */
void or_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

double or_wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static inline double dot3(const double *a, const double *b) { return a[0]*b[0] + a[1]*b[1] + a[2]*b[2]; }

/* vec_weight, mod_util.f90:729-743 */
static double vec_weight(const double *r0, const double *r1, const double *r2) {
    double ra[3], rb[3], la, lb;
    for (int i = 0; i < 3; i++) { ra[i] = r1[i] - r0[i]; rb[i] = r2[i] - r0[i]; }
    la = sqrt(ra[0]*ra[0] + ra[1]*ra[1] + ra[2]*ra[2]);
    lb = sqrt(rb[0]*rb[0] + rb[1]*rb[1] + rb[2]*rb[2]);
    if (la + lb > 0.) return la / (la + lb);
    return 0.5;
}

/* ------------------------------------------------------------------------ */
ocase *or_create(int nvx, const double *x, const double *y, const double *z,
                 int nsec, const char *names, const int *etype, const int *esec,
                 int ne2vxmax, const int *e2vx, int n_subdomains) {
    ocase *c = o_alloc(1, sizeof(ocase));
    int s, cvs1 = 0, cvs2 = 0, cvs3 = 0;
    static const int nface[21] = {0,6,0,0,0,1,1,1,1,1, 4, 4, 5, 5, 5, 5, 5, 6, 6, 6,0};
    c->nvx = nvx; c->nsec = nsec; c->ne2vxmax = ne2vxmax;
    c->esec = o_alloc(2 * (size_t)nsec, sizeof(int));
    c->etype = o_alloc((size_t)nsec + 1, sizeof(int));
    c->secname = o_alloc((size_t)nsec + 1, 33);
    c->sec2intf = o_alloc((size_t)nsec + 1, sizeof(int));
    c->bs_idx = o_alloc((size_t)nsec + 2, sizeof(int));
    /* section sizes, cell_input.f90:55-81 */
    for (s = 1; s <= nsec; s++) {
        c->etype[s] = etype[s-1];
        c->esec[2*(s-1)] = esec[2*(s-1)];
        c->esec[2*(s-1)+1] = esec[2*(s-1)+1];
        memcpy(c->secname[s], names + 33*(s-1), 32);
        c->secname[s][32] = 0;
        int cnt = esec[2*(s-1)+1] - esec[2*(s-1)] + 1;
        if (etype[s-1] >= 10 && etype[s-1] <= 20) { cvs1 += cnt; cvs2 += nface[etype[s-1]] * cnt; }
        else cvs3 += cnt;
    }
    cvs2 = (cvs2 + cvs3) / 2;
    c->ne = cvs1; c->nf = cvs2; c->nbf = cvs3; c->nelem = cvs1 + cvs3;
    c->H = 2 * c->nf - c->nbf;
    c->x = o_alloc((size_t)nvx + 1, sizeof(double));
    c->y = o_alloc((size_t)nvx + 1, sizeof(double));
    c->z = o_alloc((size_t)nvx + 1, sizeof(double));
    memcpy(c->x + 1, x, (size_t)nvx * sizeof(double));
    memcpy(c->y + 1, y, (size_t)nvx * sizeof(double));
    memcpy(c->z + 1, z, (size_t)nvx * sizeof(double));
    c->e2vx = o_alloc((size_t)ne2vxmax * c->nelem, sizeof(int));
    memcpy(c->e2vx, e2vx, (size_t)ne2vxmax * c->nelem * sizeof(int));
    c->ef2nb1 = o_alloc((size_t)c->H + 1, sizeof(int));
    c->ef2nb2 = o_alloc((size_t)c->H + 1, sizeof(int));
    c->ef2nb_idx = o_alloc((size_t)c->ne + 2, sizeof(int));
    c->s2g = o_alloc((size_t)c->nf + 2, sizeof(int));
    c->bs_store = o_alloc((size_t)c->nbf + 1, sizeof(int));
    c->red = o_alloc((size_t)c->ne + 2, sizeof(int));
    c->aip = o_alloc(3 * (size_t)c->nf + 1, sizeof(double));
    c->rip = o_alloc(3 * (size_t)c->nf + 1, sizeof(double));
    c->xc = o_alloc((size_t)c->nelem + 1, sizeof(double));
    c->yc = o_alloc((size_t)c->nelem + 1, sizeof(double));
    c->zc = o_alloc((size_t)c->nelem + 1, sizeof(double));
    c->vol = o_alloc((size_t)c->ne + 1, sizeof(double));
    if (o_build_mesh(c)) { or_destroy(c); return NULL; }
    c->nsubd = 1;
    if (n_subdomains > 1 && o_build_partition(c, n_subdomains)) { or_destroy(c); return NULL; }
    return c;
}

ocase *or_create_from_arrays(int ne, int nf, int nbf, int nsec, const char *names, const int *etype,
                             const int *esec, const int *ef2nb1, const int *ef2nb2, const int *ef2nb_idx,
                             const int *s2g, const int *bs, const double *aip, const double *rip,
                             const double *xc, const double *yc, const double *zc, const double *vol,
                             int n_subdomains) {
    ocase *c = o_alloc(1, sizeof(ocase));
    c->ne = ne; c->nf = nf; c->nbf = nbf; c->nelem = ne + nbf; c->nsec = nsec;
    c->H = 2 * nf - nbf;
    c->esec = o_alloc(2 * (size_t)nsec, sizeof(int));
    c->etype = o_alloc((size_t)nsec + 1, sizeof(int));
    c->secname = o_alloc((size_t)nsec + 1, 33);
    c->sec2intf = o_alloc((size_t)nsec + 1, sizeof(int));
    c->bs_idx = o_alloc((size_t)nsec + 2, sizeof(int));
    for (int s = 1; s <= nsec; s++) {
        c->etype[s] = etype[s-1];
        c->esec[2*(s-1)] = esec[2*(s-1)]; c->esec[2*(s-1)+1] = esec[2*(s-1)+1];
        memcpy(c->secname[s], names + 33*(s-1), 32);
        c->secname[s][32] = 0;
    }
    /* sections are taken as already ordered (add_meshds); interfaces = 2D sections */
    c->bs_idx[1] = 1;
    int n = 0;
    for (int s = 1; s <= nsec; s++) {
        c->bs_idx[s+1] = c->esec[2*(s-1)+1] + 1;
        if (c->etype[s] < 10) { n++; c->sec2intf[s] = n; }
    }
    c->nintf_c2b = n;
    c->intf2sec = o_alloc((size_t)n + 1, sizeof(int));
    for (int s = 1; s <= nsec; s++) if (c->sec2intf[s] > 0) c->intf2sec[c->sec2intf[s]] = s;
    const size_t nc = (size_t)ne + nbf;
#define COPYI(dst, src, cnt) do { dst = o_alloc((size_t)(cnt) + 2, sizeof(int)); memcpy(dst + 1, src, (size_t)(cnt) * sizeof(int)); } while (0)
#define COPYD(dst, src, cnt) do { dst = o_alloc((size_t)(cnt) + 1, sizeof(double)); memcpy(dst + 1, src, (size_t)(cnt) * sizeof(double)); } while (0)
    COPYI(c->ef2nb1, ef2nb1, c->H); COPYI(c->ef2nb2, ef2nb2, c->H); COPYI(c->ef2nb_idx, ef2nb_idx, ne + 1);
    COPYI(c->s2g, s2g, nf);
    c->bs_store = o_alloc((size_t)nbf + 1, sizeof(int));
    memcpy(c->bs_store + 1, bs, (size_t)nbf * sizeof(int));
    COPYD(c->aip, aip, 3 * (size_t)nf); COPYD(c->rip, rip, 3 * (size_t)nf);
    COPYD(c->xc, xc, nc); COPYD(c->yc, yc, nc); COPYD(c->zc, zc, nc); COPYD(c->vol, vol, ne);
#undef COPYI
#undef COPYD
    c->red = o_alloc((size_t)ne + 2, sizeof(int));
    c->nsubd = 1;
    if (n_subdomains > 1 && o_build_partition(c, n_subdomains)) { or_destroy(c); return NULL; }
    return c;
}

void or_destroy(ocase *c) {
    if (!c) return;
    free(c->x); free(c->y); free(c->z); free(c->e2vx); free(c->esec); free(c->etype);
    free(c->secname); free(c->sec2intf); free(c->intf2sec); free(c->bs_idx);
    free(c->ef2nb1); free(c->ef2nb2); free(c->ef2nb_idx); free(c->s2g); free(c->bs_store);
    free(c->red); free(c->aip); free(c->rip); free(c->xc); free(c->yc); free(c->zc); free(c->vol);
    free(c->gf2g); free(c->g2gf); free(c->g2gf_idx);
    if (c->sd) {
        for (int k = 1; k <= c->nsubd; k++) {
            free(c->sd[k].ef2nb); free(c->sd[k].ef2nb_idx); free(c->sd[k].ap);
            free(c->sd[k].anb); free(c->sd[k].b); free(c->sd[k].phic);
        }
        free(c->sd);
    }
    if (c->intf) {
        for (int k = 0; k < c->nsubd * c->nsubd; k++) free(c->intf[k].index1);
        free(c->intf);
    }
    free(c->rho); free(c->mu); free(c->u); free(c->v); free(c->w); free(c->p);
    free(c->u0); free(c->v0); free(c->w0); free(c->gu); free(c->gv); free(c->gw);
    free(c->gp); free(c->gpc); free(c->mip); free(c->mip0); free(c->bu); free(c->bv);
    free(c->bw); free(c->d); free(c->dc); free(c->ap); free(c->b); free(c->anb); free(c->phic);
    free(c->bcs);
    o_energy_free(c);
    free(c);
}

void or_sizes(const ocase *c, int *o) {
    o[0] = c->ne; o[1] = c->nf; o[2] = c->nbf; o[3] = c->nvx; o[4] = c->nelem;
    o[5] = c->nsec; o[6] = c->nred; o[7] = c->nsubd; o[8] = c->nintf_c2b;
}

int or_get_int(const ocase *c, const char *name, int *out) {
#define CP(nm, arr, n) if (!strcmp(name, nm)) { memcpy(out, (arr) + 1, (size_t)(n) * sizeof(int)); return 0; }
    CP("ef2nb1", c->ef2nb1, c->H)
    CP("ef2nb2", c->ef2nb2, c->H)
    CP("ef2nb_idx", c->ef2nb_idx, c->ne + 1)
    CP("s2g", c->s2g, c->nf)
    CP("bs", c->bs_store, c->nbf)
    CP("bs_idx", c->bs_idx, c->nsec + 1)
    CP("etype", c->etype, c->nsec)
    CP("red", c->red, c->ne)
    CP("sec2intf", c->sec2intf, c->nsec)
    if (!strcmp(name, "esec")) { memcpy(out, c->esec, 2 * (size_t)c->nsec * sizeof(int)); return 0; }
    if (c->nsubd > 1) {
        CP("gf2g", c->gf2g, c->ne)
        CP("g2gf", c->g2gf, c->ne)
        CP("g2gf_idx", c->g2gf_idx, c->nsubd + 1)
    }
#undef CP
    return -1;
}

static double **dbl_field(ocase *c, const char *name, size_t *n) {
    const size_t nc = (size_t)c->ne + c->nbf;
#define F(nm, arr, len) if (!strcmp(name, nm)) { *n = (len); return &c->arr; }
    F("aip", aip, 3 * (size_t)c->nf) F("rip", rip, 3 * (size_t)c->nf)
    F("xc", xc, nc) F("yc", yc, nc) F("zc", zc, nc) F("vol", vol, c->ne)
    F("u", u, nc) F("v", v, nc) F("w", w, nc) F("p", p, nc)
    F("u0", u0, nc) F("v0", v0, nc) F("w0", w0, nc)
    F("gu", gu, 3 * nc) F("gv", gv, 3 * nc) F("gw", gw, 3 * nc) F("gp", gp, 3 * nc) F("gpc", gpc, 3 * nc)
    F("mip", mip, c->nf) F("mip0", mip0, c->nf)
    F("bu", bu, c->ne) F("bv", bv, c->ne) F("bw", bw, c->ne) F("d", d, c->ne) F("dc", dc, c->ne)
    F("ap", ap, c->ne) F("b", b, c->ne) F("anb", anb, c->H) F("phic", phic, nc)
    F("rho", rho, c->ne) F("mu", mu, c->ne)
    F("t", t, nc) F("e", ephi, nc) F("e0", ephi0, nc) F("gt", gt, 3 * nc) F("ge", gephi, 3 * nc)
    F("cp", cp, c->ne) F("tc", tc, c->ne)
#undef F
    return NULL;
}
int or_get_dbl(const ocase *c, const char *name, double *out) {
    size_t n; double **f = dbl_field((ocase *)c, name, &n);
    if (!f || !*f) return -1;
    memcpy(out, *f + 1, n * sizeof(double));
    return 0;
}
int or_set_dbl(ocase *c, const char *name, const double *in) {
    size_t n; double **f = dbl_field(c, name, &n);
    if (!f || !*f) return -1;
    memcpy(*f + 1, in, n * sizeof(double));
    return 0;
}
int or_subdomain_sizes(const ocase *c, int sd, int *o) {
    if (sd < 1 || sd > c->nsubd || !c->sd) return -1;
    o[0] = c->sd[sd].ne; o[1] = c->sd[sd].nf; o[2] = c->sd[sd].nbf;
    return 0;
}
int or_subdomain_get(const ocase *c, int sd, int *idx, int *ef) {
    if (sd < 1 || sd > c->nsubd || !c->sd) return -1;
    const osubd *S = &c->sd[sd];
    memcpy(idx, S->ef2nb_idx + 1, ((size_t)S->ne + 1) * sizeof(int));
    memcpy(ef, S->ef2nb + 1, (size_t)(2 * S->nf - S->nbf) * sizeof(int));
    return 0;
}

/* ------------------------------------------------------------------------
 * Boundary conditions (mod_uvwp.f90:493-570), bound by section name as in
 * construct_uvwp (mod_uvwp.f90:73-78) through make_bc (mod_eqn_setup.f90:46-68):
 * 'top' -> lid, the other five walls -> dirichlet0.  make_bc compares against
 * sectionName in file order indexed by the sorted section number, as the
 * reference does.
 * ---------------------------------------------------------------------- */
static void make_bc(ocase *c, const char *secname, obc_kind kind) {
    int found = 0;
    for (int i = 1; i <= c->nintf_c2b; i++) {
        int s = c->intf2sec[i];
        char nm[33]; memcpy(nm, c->secname[s], 33);
        int L = (int)strlen(nm); while (L > 0 && nm[L-1] == ' ') nm[--L] = 0;
        if (L > 0 && strstr(secname, nm) != NULL) {
            c->bcs[i].kind = kind;
            c->bcs[i].esec1 = c->esec[2*(s-1)];
            c->bcs[i].esec2 = c->esec[2*(s-1)+1];
            found = 1;
        }
    }
    if (!found) fprintf(stderr, "oracle: BC %s not found!\n", secname);
}

static void apply_bc(ocase *c, obc *bc) {
    int e, enb, lfnb, idx, fg;
    for (e = bc->esec1; e <= bc->esec2; e++) {
        o_get_idx(abs(BS(c, e)), &enb, &lfnb);
        idx = c->ef2nb_idx[enb] + lfnb - 1;
        fg = c->ef2nb2[idx];
        if (bc->kind == BC_LID || bc->kind == BC_DIRICHLET0) {
            bc->is_dirichlet = 1;
            c->u[e] = bc->kind == BC_LID ? c->cfg.u_lid : 0.;
            c->v[e] = 0.;
            c->w[e] = 0.;
            c->p[e] = c->p[enb];
            c->mip[fg] = 0.;
        } else if (bc->kind == BC_SYMMETRY) {      /* mod_uvwp.f90:517-546 */
            bc->is_dirichlet = 2;
            double area = sqrt(c->aip[3*fg-2]*c->aip[3*fg-2] + c->aip[3*fg-1]*c->aip[3*fg-1] + c->aip[3*fg]*c->aip[3*fg]);
            double nrm[3] = {c->aip[3*fg-2]/area, c->aip[3*fg-1]/area, c->aip[3*fg]/area};
            double vel[3] = {c->u[enb], c->v[enb], c->w[enb]}, vn = dot3(vel, nrm), veln[3], velt[3];
            for (int k = 0; k < 3; k++) { veln[k] = vn*nrm[k]; velt[k] = vel[k] - veln[k]; }
            c->u[e] = velt[0] - 2*veln[0]; c->v[e] = velt[1] - 2*veln[1]; c->w[e] = velt[2] - 2*veln[2];
            c->p[e] = c->p[enb];
            c->mip[fg] = 0.;
        }
    }
}

void or_update_boundaries(ocase *c) {
    for (int i = 1; i <= c->nintf_c2b; i++) apply_bc(c, &c->bcs[i]);
    if (c->energy_on) o_energy_bc(c);        /* mod_physics.f90:47 */
}

void or_update_time(ocase *c) {
    const size_t nc = (size_t)c->ne + c->nbf;
    memcpy(c->u0 + 1, c->u + 1, nc * sizeof(double));
    memcpy(c->v0 + 1, c->v + 1, nc * sizeof(double));
    memcpy(c->w0 + 1, c->w + 1, nc * sizeof(double));
    memcpy(c->mip0 + 1, c->mip + 1, (size_t)c->nf * sizeof(double));
    if (c->energy_on) o_energy_time(c);      /* mod_physics.f90:111 */
}

int or_set_bc_kind(ocase *c, int i, int kind) {
    if (!c->bcs || i < 1 || i > c->nintf_c2b || c->bcs[i].kind == BC_NONE) return -1;
    if (kind == 1) c->bcs[i].kind = BC_LID;
    else if (kind == 2) c->bcs[i].kind = BC_DIRICHLET0;
    else if (kind == 3) c->bcs[i].kind = BC_SYMMETRY;
    else return -1;
    return 0;
}

void or_set_config(ocase *c, const or_config *cfg) {
    c->cfg = *cfg;
    if (c->rho) for (int e = 1; e <= c->ne; e++) { c->rho[e] = cfg->rho; c->mu[e] = cfg->mu; }
}

int or_physics_init(ocase *c, const or_config *cfg) {
    const size_t nc = (size_t)c->ne + c->nbf;
    c->cfg = *cfg;
    /* construct_physics, mod_physics.f90:58-63 */
    c->ap = o_alloc((size_t)c->ne + 1, sizeof(double));
    c->b = o_alloc((size_t)c->ne + 1, sizeof(double));
    c->anb = o_alloc((size_t)c->H + 1, sizeof(double));
    c->phic = o_alloc(nc + 1, sizeof(double));
    /* init_properties, mod_properties.f90:76-89 */
    c->rho = o_alloc((size_t)c->ne + 1, sizeof(double));
    c->mu = o_alloc((size_t)c->ne + 1, sizeof(double));
    for (int e = 1; e <= c->ne; e++) { c->rho[e] = cfg->rho; c->mu[e] = cfg->mu; }
    /* construct_uvwp, mod_uvwp.f90:30-82 */
    c->u = o_alloc(nc + 1, sizeof(double)); c->v = o_alloc(nc + 1, sizeof(double));
    c->w = o_alloc(nc + 1, sizeof(double)); c->p = o_alloc(nc + 1, sizeof(double));
    c->u0 = o_alloc(nc + 1, sizeof(double)); c->v0 = o_alloc(nc + 1, sizeof(double));
    c->w0 = o_alloc(nc + 1, sizeof(double));
    c->gu = o_alloc(3*nc + 1, sizeof(double)); c->gv = o_alloc(3*nc + 1, sizeof(double));
    c->gw = o_alloc(3*nc + 1, sizeof(double)); c->gp = o_alloc(3*nc + 1, sizeof(double));
    c->gpc = o_alloc(3*nc + 1, sizeof(double));
    c->mip = o_alloc((size_t)c->nf + 1, sizeof(double)); c->mip0 = o_alloc((size_t)c->nf + 1, sizeof(double));
    c->bu = o_alloc((size_t)c->ne + 1, sizeof(double)); c->bv = o_alloc((size_t)c->ne + 1, sizeof(double));
    c->bw = o_alloc((size_t)c->ne + 1, sizeof(double)); c->d = o_alloc((size_t)c->ne + 1, sizeof(double));
    c->dc = o_alloc((size_t)c->ne + 1, sizeof(double));
    c->bcs = o_alloc((size_t)c->nintf_c2b + 1, sizeof(obc));
    make_bc(c, "top", BC_LID);
    make_bc(c, "west", BC_DIRICHLET0);
    make_bc(c, "east", BC_DIRICHLET0);
    make_bc(c, "south", BC_DIRICHLET0);
    make_bc(c, "north", BC_DIRICHLET0);
    make_bc(c, "bottom", BC_DIRICHLET0);
    or_calc_mip(c, 0);
    memcpy(c->mip0 + 1, c->mip + 1, (size_t)c->nf * sizeof(double));
    c->phys_ready = 1;
    return 0;
}

/* ------------------------------------------------------------------------
 * matinv3 + calc_grad, mod_solver.f90:8-81
 * ---------------------------------------------------------------------- */
static void matinv3(const double A[3][3], double B[3][3]) {
    double det = (A[0][0]*A[1][1]*A[2][2] - A[0][0]*A[1][2]*A[2][1]
                - A[0][1]*A[1][0]*A[2][2] + A[0][1]*A[1][2]*A[2][0]
                + A[0][2]*A[1][0]*A[2][1] - A[0][2]*A[1][1]*A[2][0]);
    if (fabs(det) > DBL_MIN) {
        double detinv = 1.0 / det;
        B[0][0] = +detinv * (A[1][1]*A[2][2] - A[1][2]*A[2][1]);
        B[1][0] = -detinv * (A[1][0]*A[2][2] - A[1][2]*A[2][0]);
        B[2][0] = +detinv * (A[1][0]*A[2][1] - A[1][1]*A[2][0]);
        B[0][1] = -detinv * (A[0][1]*A[2][2] - A[0][2]*A[2][1]);
        B[1][1] = +detinv * (A[0][0]*A[2][2] - A[0][2]*A[2][0]);
        B[2][1] = -detinv * (A[0][0]*A[2][1] - A[0][1]*A[2][0]);
        B[0][2] = +detinv * (A[0][1]*A[1][2] - A[0][2]*A[1][1]);
        B[1][2] = -detinv * (A[0][0]*A[1][2] - A[0][2]*A[1][0]);
        B[2][2] = +detinv * (A[0][0]*A[1][1] - A[0][1]*A[1][0]);
    } else {
        memset(B, 0, 9 * sizeof(double));
        det = A[0][0] + A[1][1] + A[2][2];
        double detinv = 1.0 / det;
        B[0][0] = detinv; B[1][1] = detinv; B[2][2] = detinv;
    }
}

static void calc_grad(ocase *c, const double *phi, double *grad) {
    /* phi [1..ne+nbf], grad [1..3(ne+nbf)] */
    O_PAR
    for (int e = 1; e <= c->ne; e++) {
        double A[3][3] = {{0}}, Ai[3][3], g[3] = {0, 0, 0};
        for (int idx = c->ef2nb_idx[e]; idx <= c->ef2nb_idx[e+1] - 1; idx++) {
            int enb, lfnb;
            o_get_idx(c->ef2nb1[idx], &enb, &lfnb);
            double dr[3] = {c->xc[enb] - c->xc[e], c->yc[enb] - c->yc[e], c->zc[enb] - c->zc[e]};
            double wt = 1. / (dr[0]*dr[0] + dr[1]*dr[1] + dr[2]*dr[2]);
            double dphi = phi[enb] - phi[e];
            for (int k = 0; k < 3; k++) g[k] = g[k] + wt*dphi*dr[k];
            A[0][0] = A[0][0] + wt*dr[0]*dr[0];
            A[0][1] = A[0][1] + wt*dr[0]*dr[1];
            A[0][2] = A[0][2] + wt*dr[0]*dr[2];
            A[1][1] = A[1][1] + wt*dr[1]*dr[1];
            A[1][2] = A[1][2] + wt*dr[1]*dr[2];
            A[2][2] = A[2][2] + wt*dr[2]*dr[2];
        }
        A[1][0] = A[0][1]; A[2][0] = A[0][2]; A[2][1] = A[1][2];
        matinv3(A, Ai);
        for (int k = 0; k < 3; k++) grad[3*e-2+k] = Ai[k][0]*g[0] + Ai[k][1]*g[1] + Ai[k][2]*g[2];
    }
}

void or_calc_grad(ocase *c, const double *phi0, double *grad0) {
    const size_t nc = (size_t)c->ne + c->nbf;
    double *phi = o_alloc(nc + 1, sizeof(double)), *g = o_alloc(3*nc + 1, sizeof(double));
    memcpy(phi + 1, phi0, nc * sizeof(double));
    memcpy(g + 1, grad0, 3*nc * sizeof(double));
    calc_grad(c, phi, g);
    memcpy(grad0, g + 1, 3*nc * sizeof(double));
    free(phi); free(g);
}

/* ------------------------------------------------------------------------
 * calc_coef_uvw, mod_uvwp.f90:161-286 (+ relaxation extension)
 * ---------------------------------------------------------------------- */
void or_calc_coef_uvw(ocase *c) {
    const double dt = c->cfg.dt;
    double *ap = c->ap, *anb = c->anb;
    O_PAR
    for (int e = 1; e <= c->ne; e++) {
        double rp[3] = {c->xc[e], c->yc[e], c->zc[e]};
        double sumf = 0., sumss[3] = {0, 0, 0}, sumdefc[3] = {0, 0, 0};
        ap[e] = 0.;
        for (int idx = c->ef2nb_idx[e]; idx <= c->ef2nb_idx[e+1] - 1; idx++) {
            int enb, lfnb, fg, fg_sgn, i;
            double f = 0., fnb = 0., d = 0.;
            anb[idx] = 0.;
            o_get_idx(c->ef2nb1[idx], &enb, &lfnb);
            if (lfnb > 0) {
                double area, norm[3], rip[3], rpnb[3], dr[3], ds, wt, drip[3], rp_p[3], rpnb_p[3], dr_p[3], ds_p, muip, gip[3], t;
                fg = c->ef2nb2[idx];
                fg_sgn = o_sgn(fg);
                fg = abs(fg);
                i = 3*fg - 2;
                area = sqrt(c->aip[i]*c->aip[i] + c->aip[i+1]*c->aip[i+1] + c->aip[i+2]*c->aip[i+2]);
                for (int k = 0; k < 3; k++) norm[k] = fg_sgn*c->aip[i+k] / area;
                for (int k = 0; k < 3; k++) rip[k] = c->rip[i+k];
                rpnb[0] = c->xc[enb]; rpnb[1] = c->yc[enb]; rpnb[2] = c->zc[enb];
                for (int k = 0; k < 3; k++) dr[k] = rpnb[k] - rp[k];
                ds = sqrt(dot3(dr, dr));
                wt = vec_weight(rip, rp, rpnb);
                for (int k = 0; k < 3; k++) drip[k] = rip[k] - rp[k];
                t = dot3(drip, norm);
                for (int k = 0; k < 3; k++) rp_p[k] = rip[k] - t*norm[k];
                for (int k = 0; k < 3; k++) drip[k] = rip[k] - rpnb[k];
                t = dot3(drip, norm);
                for (int k = 0; k < 3; k++) rpnb_p[k] = rip[k] - t*norm[k];
                for (int k = 0; k < 3; k++) dr_p[k] = rpnb_p[k] - rp_p[k];
                ds_p = sqrt(dot3(dr_p, dr_p));
                f = -fg_sgn*c->mip[fg];
                fnb = fmax(f, 0.);
                sumf = sumf + f;
                muip = (1. - wt)*c->mu[e] + wt*c->mu[enb];
                d = muip*area/ds;
                for (int m = 1; m <= 3; m++) {
                    gip[0] = (1. - wt)*c->gu[3*e-3+m] + wt*c->gu[3*enb-3+m];
                    gip[1] = (1. - wt)*c->gv[3*e-3+m] + wt*c->gv[3*enb-3+m];
                    gip[2] = (1. - wt)*c->gw[3*e-3+m] + wt*c->gw[3*enb-3+m];
                    sumss[m-1] = sumss[m-1] + muip*area*dot3(gip, dr)/ds;
                }
                const double *gfld[3] = {c->gu, c->gv, c->gw};
                for (int q = 0; q < 3; q++) {
                    for (int k = 0; k < 3; k++) gip[k] = (1. - wt)*gfld[q][3*e-2+k] + wt*gfld[q][3*enb-2+k];
                    sumdefc[q] = sumdefc[q] + muip*area*(dot3(gip, dr_p)/ds_p - dot3(gip, dr)/ds);
                }
            }
            anb[idx] = d + fnb;
            ap[e] = ap[e] + d + fnb;
        }
        double ap0 = c->rho[e]*c->vol[e]/dt;
        ap[e] = ap[e] + ap0;
        c->bu[e] = ap0*c->u0[e] + sumf*c->u[e] - c->vol[e]*c->gp[3*e-2] + sumss[0] + sumdefc[0];
        c->bv[e] = ap0*c->v0[e] + sumf*c->v[e] - c->vol[e]*c->gp[3*e-1] + sumss[1] + sumdefc[1];
        c->bw[e] = ap0*c->w0[e] + sumf*c->w[e] - c->vol[e]*c->gp[3*e]   + sumss[2] + sumdefc[2];
    }
    /* boundary conditions, mod_uvwp.f90:242-273 */
    for (int ibc = 1; ibc <= c->nintf_c2b; ibc++) {
        obc *bc = &c->bcs[ibc];
        for (int enb = bc->esec1; enb <= bc->esec2; enb++) {
            int e, lf, idx, fg, i;
            double area, norm[3], dr[3], ds, f = 0., d = 0.;
            o_get_idx(abs(BS(c, enb)), &e, &lf);
            idx = c->ef2nb_idx[e] + lf - 1;
            fg = c->ef2nb2[idx];
            i = 3*fg - 2;
            area = sqrt(c->aip[i]*c->aip[i] + c->aip[i+1]*c->aip[i+1] + c->aip[i+2]*c->aip[i+2]);
            for (int k = 0; k < 3; k++) norm[k] = c->aip[i+k] / area;
            dr[0] = c->xc[enb] - c->xc[e]; dr[1] = c->yc[enb] - c->yc[e]; dr[2] = c->zc[enb] - c->zc[e];
            ds = sqrt(dot3(dr, dr));
            if (bc->is_dirichlet == 1) {
                double vbnc[3] = {c->u[enb], c->v[enb], c->w[enb]}, vrel[3] = {c->u[e], c->v[e], c->w[e]}, t;
                f = 0.;
                d = c->mu[e]*area/ds;
                t = dot3(vrel, norm);
                for (int k = 0; k < 3; k++) vrel[k] = vrel[k] - t*norm[k];
                for (int k = 0; k < 3; k++) vrel[k] = vbnc[k] - vrel[k];
                c->bu[e] = c->bu[e] + d*vrel[0] - d*c->u[e];
                c->bv[e] = c->bv[e] + d*vrel[1] - d*c->v[e];
                c->bw[e] = c->bw[e] + d*vrel[2] - d*c->w[e];
            } else if (bc->is_dirichlet == 2) {
                f = 0.;
                d = c->mu[e]*area/ds;
            }
            ap[e] = ap[e] + d + f;
            anb[idx] = anb[idx] + d + f;
        }
    }
    /* implicit under-relaxation (extension) */
    if (c->cfg.alpha_u != 1.0) {
        const double a = c->cfg.alpha_u;
        O_PAR
        for (int e = 1; e <= c->ne; e++) {
            double apr = ap[e] / a;
            c->bu[e] = c->bu[e] + (1.0 - a)*apr*c->u[e];
            c->bv[e] = c->bv[e] + (1.0 - a)*apr*c->v[e];
            c->bw[e] = c->bw[e] + (1.0 - a)*apr*c->w[e];
            ap[e] = apr;
        }
    }
    /* Rhie-Chow and SIMPLEC coefficients, mod_uvwp.f90:275-284 */
    O_PAR
    for (int e = 1; e <= c->ne; e++) {
        c->d[e] = c->vol[e]/ap[e];
        double dc = ap[e];
        for (int idx = c->ef2nb_idx[e]; idx <= c->ef2nb_idx[e+1] - 1; idx++) dc = dc - anb[idx];
        c->dc[e] = c->vol[e]/dc;
    }
}

/* ------------------------------------------------------------------------
 * calc_coef_p, mod_uvwp.f90:289-368
 * ---------------------------------------------------------------------- */
void or_calc_coef_p(ocase *c) {
    double *ap = c->ap, *anb = c->anb, *b = c->b;
    O_PAR
    for (int e = 1; e <= c->ne; e++) {
        double sumf = 0., rp[3] = {c->xc[e], c->yc[e], c->zc[e]};
        ap[e] = 0.;
        for (int idx = c->ef2nb_idx[e]; idx <= c->ef2nb_idx[e+1] - 1; idx++) {
            int enb, lfnb, fg, fg_sgn, i;
            double d = 0.;
            anb[idx] = 0.;
            o_get_idx(c->ef2nb1[idx], &enb, &lfnb);
            if (lfnb > 0) {
                double area, norm[3], rip[3], rpnb[3], dr[3], wt, f, rhoip;
                fg = c->ef2nb2[idx];
                fg_sgn = o_sgn(fg);
                fg = abs(fg);
                i = 3*fg - 2;
                area = sqrt(c->aip[i]*c->aip[i] + c->aip[i+1]*c->aip[i+1] + c->aip[i+2]*c->aip[i+2]);
                for (int k = 0; k < 3; k++) norm[k] = fg_sgn*c->aip[i+k] / area;
                for (int k = 0; k < 3; k++) rip[k] = c->rip[i+k];
                rpnb[0] = c->xc[enb]; rpnb[1] = c->yc[enb]; rpnb[2] = c->zc[enb];
                for (int k = 0; k < 3; k++) dr[k] = rpnb[k] - rp[k];
                wt = vec_weight(rip, rp, rpnb);
                f = -fg_sgn*c->mip[fg];
                sumf = sumf + f;
                rhoip = (1. - wt)*c->rho[e] + wt*c->rho[enb];
                d = ((1. - wt)*c->dc[e] + wt*c->dc[enb]) / dot3(dr, norm)*rhoip*area;
            }
            anb[idx] = d;
            ap[e] = ap[e] + d;
        }
        b[e] = sumf;
    }
    for (int ibc = 1; ibc <= c->nintf_c2b; ibc++) {
        obc *bc = &c->bcs[ibc];
        for (int enb = bc->esec1; enb <= bc->esec2; enb++) {
            int e, lf, idx, fg;
            o_get_idx(abs(BS(c, enb)), &e, &lf);
            idx = c->ef2nb_idx[e] + lf - 1;
            fg = c->ef2nb2[idx];
            double d = 0.;
            ap[e] = ap[e] + d;
            anb[idx] = anb[idx] + d;
            b[e] = b[e] - c->mip[fg];
        }
    }
}

/* ------------------------------------------------------------------------
 * calc_mip, mod_uvwp.f90:438-490
 * ---------------------------------------------------------------------- */
void or_calc_mip(ocase *c, int lRhieChow) {
    const double dt = c->cfg.dt;
    O_PAR
    for (int fg = 1; fg <= c->nf; fg++) {
        int e, lf, idx, enb, lfnb, i;
        o_get_idx(c->s2g[fg], &e, &lf);
        idx = c->ef2nb_idx[e] + lf - 1;
        o_get_idx(c->ef2nb1[idx], &enb, &lfnb);
        if (lfnb == 0) continue;
        double rp[3] = {c->xc[e], c->yc[e], c->zc[e]}, rpnb[3] = {c->xc[enb], c->yc[enb], c->zc[enb]};
        double area, norm[3], rip[3], wt, vec1[3], vec2[3], velip[3], rhoip;
        i = 3*fg - 2;
        area = sqrt(c->aip[i]*c->aip[i] + c->aip[i+1]*c->aip[i+1] + c->aip[i+2]*c->aip[i+2]);
        for (int k = 0; k < 3; k++) norm[k] = c->aip[i+k] / area;
        for (int k = 0; k < 3; k++) rip[k] = c->rip[i+k];
        wt = vec_weight(rip, rp, rpnb);
        vec1[0] = c->u[e]; vec1[1] = c->v[e]; vec1[2] = c->w[e];
        vec2[0] = c->u[enb]; vec2[1] = c->v[enb]; vec2[2] = c->w[enb];
        for (int k = 0; k < 3; k++) velip[k] = (1. - wt)*vec1[k] + wt*vec2[k];
        rhoip = c->rho[e]*(1. - wt) + c->rho[enb]*wt;
        c->mip[fg] = dot3(velip, norm)*rhoip*area;
        if (lRhieChow) {
            double dr[3], gpip[3], dip, velip0[3];
            for (int k = 0; k < 3; k++) dr[k] = rpnb[k] - rp[k];
            for (int k = 0; k < 3; k++) gpip[k] = (1. - wt)*c->gp[3*e-2+k] + wt*c->gp[3*enb-2+k];
            dip = (1. - wt)*c->d[e] + wt*c->d[enb];
            vec1[0] = c->u0[e]; vec1[1] = c->v0[e]; vec1[2] = c->w0[e];
            vec2[0] = c->u0[enb]; vec2[1] = c->v0[enb]; vec2[2] = c->w0[enb];
            for (int k = 0; k < 3; k++) velip0[k] = (1. - wt)*vec1[k] + wt*vec2[k];
            c->mip[fg] = c->mip[fg] - rhoip*area*dip/dot3(dr, norm)*(c->p[enb] - c->p[e] - dot3(gpip, dr))
                       - rhoip/dt*dip*(c->mip0[fg] - dot3(velip0, norm)*rhoip*area);
        }
    }
}

/* ------------------------------------------------------------------------
 * update_uvwp, mod_uvwp.f90:370-436 (+ alpha_p extension)
 * ---------------------------------------------------------------------- */
static void update_uvwp(ocase *c, const double *pc) {
    const double ap_ = c->cfg.alpha_p;
    O_PAR
    for (int e = 1; e <= c->ne; e++) {
        if (ap_ == 1.0) {
            c->p[e] = c->p[e] + pc[e];
            for (int k = 0; k < 3; k++) c->gp[3*e-2+k] = c->gp[3*e-2+k] + c->gpc[3*e-2+k];
        } else {
            c->p[e] = c->p[e] + ap_*pc[e];
            for (int k = 0; k < 3; k++) c->gp[3*e-2+k] = c->gp[3*e-2+k] + ap_*c->gpc[3*e-2+k];
        }
    }
    O_PAR
    for (int fg = 1; fg <= c->nf; fg++) {
        int e, lf, idx, enb, lfnb, i;
        o_get_idx(c->s2g[fg], &e, &lf);
        idx = c->ef2nb_idx[e] + lf - 1;
        o_get_idx(c->ef2nb1[idx], &enb, &lfnb);
        if (lfnb == 0) continue;
        double area, norm[3], dr[3], rip[3], wt, dip, rhoip, dmip;
        i = 3*fg - 2;
        area = sqrt(c->aip[i]*c->aip[i] + c->aip[i+1]*c->aip[i+1] + c->aip[i+2]*c->aip[i+2]);
        for (int k = 0; k < 3; k++) norm[k] = c->aip[i+k] / area;
        double rp[3] = {c->xc[e], c->yc[e], c->zc[e]}, rpnb[3] = {c->xc[enb], c->yc[enb], c->zc[enb]};
        for (int k = 0; k < 3; k++) dr[k] = rpnb[k] - rp[k];
        for (int k = 0; k < 3; k++) rip[k] = c->rip[i+k];
        wt = vec_weight(rip, rp, rpnb);
        dip = (1. - wt)*c->dc[e] + wt*c->dc[enb];
        rhoip = (c->rho[e] + c->rho[enb]) / 2.;
        dmip = rhoip*area*dip*(pc[enb] - pc[e]) / dot3(dr, norm);
        c->mip[fg] = c->mip[fg] - dmip;
    }
}
void or_update_uvwp(ocase *c) { update_uvwp(c, c->phic); }

/* adjust_pc, mod_uvwp.f90:136-158 */
static void adjust_pc(ocase *c, double *pc, double pref) {
    O_PAR
    for (int e = 1; e <= c->ne; e++) pc[e] = pc[e] - pref;
    O_PAR
    for (int enb = c->ne + 1; enb <= c->ne + c->nbf; enb++) {
        int e, lf;
        o_get_idx(abs(BS(c, enb)), &e, &lf);
        pc[enb] = pc[e];
    }
}
void or_adjust_pc(ocase *c) { adjust_pc(c, c->phic, c->phic[1]); }

/* ------------------------------------------------------------------------
 * Linear solvers.
 * ---------------------------------------------------------------------- */
/* calc_residual, mod_solver.f90:230-253 */
static void calc_residual(const double *phi, const double *ap, const double *anb, const double *b,
                          const int *ef2nb_idx, const int *ef2nb, int ne, double *res, double *res_max) {
    double r;
    *res = 0.; *res_max = 0.;
    for (int e = 1; e <= ne; e++) {
        double sumnb = b[e];
        for (int idx = ef2nb_idx[e]; idx <= ef2nb_idx[e+1] - 1; idx++) {
            int enb, lfnb; o_get_idx(ef2nb[idx], &enb, &lfnb);
            sumnb = sumnb + anb[idx]*phi[enb];
        }
        r = sumnb - ap[e]*phi[e];
        *res_max = fmax(r, *res_max);
        *res = *res + r*r;
    }
    *res = sqrt(*res / ne);
}

/* smoother_gs, mod_solver.f90:191-228 */
static void smoother_gs(int is_pc, double *phi, const double *ap, const double *anb, const double *b,
                        const int *ef2nb_idx, const int *ef2nb, int ne, int nit) {
    const double sor = is_pc ? 1.02 : 1.;
    for (int it = 1; it <= nit; it++) {
        for (int e = 1; e <= ne; e++) {
            double sumnb = b[e];
            for (int idx = ef2nb_idx[e]; idx <= ef2nb_idx[e+1] - 1; idx++) {
                int enb, lfnb; o_get_idx(ef2nb[idx], &enb, &lfnb);
                sumnb = sumnb + anb[idx]*phi[enb];
            }
            phi[e] = (sumnb + (sor - 1.)*ap[e]*phi[e]) / ap[e] / sor;
        }
        for (int e = ne; e >= 1; e--) {
            double sumnb = b[e];
            for (int idx = ef2nb_idx[e]; idx <= ef2nb_idx[e+1] - 1; idx++) {
                int enb, lfnb; o_get_idx(ef2nb[idx], &enb, &lfnb);
                sumnb = sumnb + anb[idx]*phi[enb];
            }
            phi[e] = (sumnb + (sor - 1.)*ap[e]*phi[e]) / ap[e] / sor;
        }
    }
}

/* solve_gs, mod_solver.f90:255-327 */
static void solve_gs(int is_pc, double *phi, const double *ap, const double *anb, const double *b,
                     const int *ef2nb_idx, const int *ef2nb, int ne, int nit,
                     int *it_out, double *ri, double *rf, double *rmax) {
    const double sor = is_pc ? 1.02 : 1.;
    double res_i = 0., res_f, res_target, res_max = 0., r;
    for (int e = 1; e <= ne; e++) {
        double sumnb = b[e];
        for (int idx = ef2nb_idx[e]; idx <= ef2nb_idx[e+1] - 1; idx++) {
            int enb, lfnb; o_get_idx(ef2nb[idx], &enb, &lfnb);
            sumnb = sumnb + anb[idx]*phi[enb];
        }
        r = sumnb - ap[e]*phi[e];
        res_i = res_i + r*r;
    }
    res_i = sqrt(res_i / ne);
    int it = 0;
    res_f = res_i;
    res_target = res_i / 10.;
    while (it < nit && res_f > res_target) {
        it++;
        for (int e = 1; e <= ne; e++) {
            double sumnb = b[e];
            for (int idx = ef2nb_idx[e]; idx <= ef2nb_idx[e+1] - 1; idx++) {
                int enb, lfnb; o_get_idx(ef2nb[idx], &enb, &lfnb);
                sumnb = sumnb + anb[idx]*phi[enb];
            }
            phi[e] = (sumnb + (sor - 1.)*ap[e]*phi[e]) / ap[e] / sor;
        }
        for (int e = ne; e >= 1; e--) {
            double sumnb = b[e];
            for (int idx = ef2nb_idx[e]; idx <= ef2nb_idx[e+1] - 1; idx++) {
                int enb, lfnb; o_get_idx(ef2nb[idx], &enb, &lfnb);
                sumnb = sumnb + anb[idx]*phi[enb];
            }
            phi[e] = (sumnb + (sor - 1.)*ap[e]*phi[e]) / ap[e] / sor;
        }
        res_max = 0.;
        res_f = 0.;
        for (int e = 1; e <= ne; e++) {
            double sumnb = b[e];
            for (int idx = ef2nb_idx[e]; idx <= ef2nb_idx[e+1] - 1; idx++) {
                int enb, lfnb; o_get_idx(ef2nb[idx], &enb, &lfnb);
                sumnb = sumnb + anb[idx]*phi[enb];
            }
            r = fabs(sumnb - ap[e]*phi[e]);
            res_max = fmax(r, res_max);
            res_f = res_f + r*r;
        }
        res_f = sqrt(res_f / ne);
    }
    *it_out = it; *ri = res_i; *rf = res_f; *rmax = res_max;
}

/* assemble_coef, update_halos, update_phi: mod_subdomains.f90:162-229 */
static void assemble_coef(ocase *c, const double *ap, const double *anb, const double *b, const double *phi) {
    O_PAR
    for (int cc = 1; cc <= c->nsubd; cc++) {
        osubd *S = &c->sd[cc];
        for (int e = 1; e <= S->ne; e++) {
            int g = c->g2gf[c->g2gf_idx[cc] + e - 1];
            S->ap[e] = ap[g]; S->b[e] = b[g]; S->phic[e] = phi[g];
            for (int idx = S->ef2nb_idx[e]; idx <= S->ef2nb_idx[e+1] - 1; idx++) {
                int enb, lfnb, lf, idx2, gnb, lfg;
                o_get_idx(S->ef2nb[idx], &enb, &lfnb);
                lf = idx - S->ef2nb_idx[e] + 1;
                idx2 = c->ef2nb_idx[g] + lf - 1;
                S->anb[idx] = anb[idx2];
                if (lfnb == 0) {
                    o_get_idx(c->ef2nb1[idx2], &gnb, &lfg);
                    S->phic[enb] = phi[gnb];
                }
            }
        }
    }
}
static void update_halos(ointf *it, osubd *s1, osubd *s2) {
    if (it->c1 == it->c2) return;
    for (int cs = 1; cs <= it->ncs; cs++) {
        int g1, lf1, g2, lf2, gnb1, gnb2, tmp, idx;
        o_get_idx(it->index1[cs], &g1, &lf1);
        idx = s1->ef2nb_idx[g1] + lf1 - 1;
        o_get_idx(s1->ef2nb[idx], &gnb1, &tmp);
        o_get_idx(it->index2[cs], &g2, &lf2);
        idx = s2->ef2nb_idx[g2] + lf2 - 1;
        o_get_idx(s2->ef2nb[idx], &gnb2, &tmp);
        s1->phic[gnb1] = s2->phic[g2];
        s2->phic[gnb2] = s1->phic[g1];
    }
}
/* multi_subdomain_solver, mod_solver.f90:124-189 */
static void multi_subdomain_solver(ocase *c, const double *ap, const double *anb, const double *b, double *phi,
                                   int nit, int *it_out, double *ri, double *rf, double *rmax) {
    const int nsd = c->nsubd;
    double res, res_max, res_i_tot = 0., res_f_tot = 0., res_max_tot = 0., res_target;
    double *sres = o_alloc((size_t)nsd + 1, sizeof(double)), *sres_max = o_alloc((size_t)nsd + 1, sizeof(double));
    assemble_coef(c, ap, anb, b, phi);
    O_PAR
    for (int cc = 1; cc <= nsd; cc++) {
        osubd *S = &c->sd[cc];
        calc_residual(S->phic, S->ap, S->anb, S->b, S->ef2nb_idx, S->ef2nb, S->ne, &sres[cc], &sres_max[cc]);
    }
    for (int cc = 1; cc <= nsd; cc++) {
        res = sres[cc]; res_max = sres_max[cc];
        res_i_tot = res_i_tot + res*res;
        res_max_tot = fmax(res_max_tot, res_max);
    }
    res_i_tot = sqrt(res_i_tot / nsd);
    int it = 0;
    res_f_tot = res_i_tot;
    res_target = res_i_tot / 10.;
    while (it < nit && res_f_tot > res_target) {
        /* each block sweeps its own cells and reads only its own halo copies */
        O_PAR
        for (int cc = 1; cc <= nsd; cc++) {
            osubd *S = &c->sd[cc];
            smoother_gs(1, S->phic, S->ap, S->anb, S->b, S->ef2nb_idx, S->ef2nb, S->ne, 2);
        }
        it = it + 2;
        for (int i = 1; i <= nsd; i++)
            for (int j = i + 1; j <= nsd; j++)
                update_halos(&c->intf[(j-1)*nsd + i-1], &c->sd[i], &c->sd[j]);
        if (it % 10 == 0) {
            O_PAR
            for (int cc = 1; cc <= nsd; cc++) {
                osubd *S = &c->sd[cc];
                calc_residual(S->phic, S->ap, S->anb, S->b, S->ef2nb_idx, S->ef2nb, S->ne, &sres[cc], &sres_max[cc]);
            }
            for (int cc = 1; cc <= nsd; cc++) {
                res = sres[cc]; res_max = sres_max[cc];
                res_f_tot = res_f_tot + res*res;    /* not reset: reference quirk */
                res_max_tot = fmax(res_max_tot, res_max);
            }
            res_f_tot = sqrt(res_f_tot / nsd);
        }
    }
    for (int cc = 1; cc <= nsd; cc++) {
        osubd *S = &c->sd[cc];
        for (int e = 1; e <= S->ne; e++) phi[c->g2gf[c->g2gf_idx[cc] + e - 1]] = S->phic[e];
    }
    free(sres); free(sres_max);
    *it_out = it; *ri = res_i_tot; *rf = res_f_tot; *rmax = res_max_tot;
}

/* ---- tight mode: Krylov inner solves (parity mode) -------------------- */
/* y = A x for the interior operator: (A x)_e = ap_e x_e - sum_interior anb x_nb */
static void amul(const ocase *c, const double *ap, const double *anb, const double *x, double *y) {
    O_PAR
    for (int e = 1; e <= c->ne; e++) {
        double s = ap[e]*x[e];
        for (int idx = c->ef2nb_idx[e]; idx <= c->ef2nb_idx[e+1] - 1; idx++) {
            int enb, lfnb; o_get_idx(c->ef2nb1[idx], &enb, &lfnb);
            if (lfnb > 0) s = s - anb[idx]*x[enb];
        }
        y[e] = s;
    }
}
/* Dot product over fixed blocks of O_DOT_BLOCK elements: each block is summed
 * in order, then the block sums in order, so the result does not depend on
 * the number of threads (a single block is the plain serial sum). */
#define O_DOT_BLOCK 4096
static double vdot(int n, const double *a, const double *b) {
    const int nb = (n + O_DOT_BLOCK - 1) / O_DOT_BLOCK;
    if (nb <= 1) {
        double s = 0.;
        for (int e = 1; e <= n; e++) s = s + a[e]*b[e];
        return s;
    }
    double *part = o_alloc((size_t)nb, sizeof(double));
    O_PAR
    for (int k = 0; k < nb; k++) {
        const int e1 = 1 + k*O_DOT_BLOCK, e2 = (k + 1)*O_DOT_BLOCK < n ? (k + 1)*O_DOT_BLOCK : n;
        double s = 0.;
        for (int e = e1; e <= e2; e++) s = s + a[e]*b[e];
        part[k] = s;
    }
    double s = 0.;
    for (int k = 0; k < nb; k++) s = s + part[k];
    free(part);
    return s;
}
/* RHS including the known halo terms: b'_e = b_e + sum_boundary anb*phi_halo */
static void full_rhs(const ocase *c, const double *anb, const double *b, const double *phi, double *bb) {
    O_PAR
    for (int e = 1; e <= c->ne; e++) {
        double s = b[e];
        for (int idx = c->ef2nb_idx[e]; idx <= c->ef2nb_idx[e+1] - 1; idx++) {
            int enb, lfnb; o_get_idx(c->ef2nb1[idx], &enb, &lfnb);
            if (lfnb == 0) s = s + anb[idx]*phi[enb];
        }
        bb[e] = s;
    }
}
/* Jacobi-preconditioned BiCGStab on A phi = b' from the current phi. */
static int bicgstab(const ocase *c, const double *ap, const double *anb, const double *b, double *phi,
                    double rtol, int maxit, double *r0n, double *rfn) {
    const int n = c->ne;
    double *bb = o_alloc(n + 1, 8), *r = o_alloc(n + 1, 8), *rh = o_alloc(n + 1, 8), *pp = o_alloc(n + 1, 8);
    double *vv = o_alloc(n + 1, 8), *ph = o_alloc(n + 1, 8), *s = o_alloc(n + 1, 8), *sh = o_alloc(n + 1, 8);
    double *t = o_alloc(n + 1, 8);
    full_rhs(c, anb, b, phi, bb);
    amul(c, ap, anb, phi, t);
    O_PAR
    for (int e = 1; e <= n; e++) { r[e] = bb[e] - t[e]; rh[e] = r[e]; }
    double bn = sqrt(vdot(n, bb, bb)), rn = sqrt(vdot(n, r, r));
    double rho = 1., alpha = 1., omega = 1., rho1;
    int it = 0;
    *r0n = rn;
    double tol = rtol * bn;
    while (rn > tol && it < maxit) {
        it++;
        rho1 = vdot(n, rh, r);
        if (rho1 == 0.) break;
        if (it == 1) {
            O_PAR
            for (int e = 1; e <= n; e++) pp[e] = r[e];
        } else {
            double beta = (rho1/rho)*(alpha/omega);
            O_PAR
            for (int e = 1; e <= n; e++) pp[e] = r[e] + beta*(pp[e] - omega*vv[e]);
        }
        O_PAR
        for (int e = 1; e <= n; e++) ph[e] = pp[e]/ap[e];
        amul(c, ap, anb, ph, vv);
        alpha = rho1 / vdot(n, rh, vv);
        O_PAR
        for (int e = 1; e <= n; e++) s[e] = r[e] - alpha*vv[e];
        double sn = sqrt(vdot(n, s, s));
        if (sn <= tol) {
            O_PAR
            for (int e = 1; e <= n; e++) phi[e] = phi[e] + alpha*ph[e];
            rn = sn;
            break;
        }
        O_PAR
        for (int e = 1; e <= n; e++) sh[e] = s[e]/ap[e];
        amul(c, ap, anb, sh, t);
        double tt = vdot(n, t, t);
        omega = tt > 0. ? vdot(n, t, s)/tt : 0.;
        O_PAR
        for (int e = 1; e <= n; e++) phi[e] = phi[e] + alpha*ph[e] + omega*sh[e];
        O_PAR
        for (int e = 1; e <= n; e++) r[e] = s[e] - omega*t[e];
        rn = sqrt(vdot(n, r, r));
        rho = rho1;
        if (omega == 0.) break;
    }
    *rfn = rn;
    free(bb); free(r); free(rh); free(pp); free(vv); free(ph); free(s); free(sh); free(t);
    return it;
}
/* Jacobi-preconditioned CG on the singular Neumann pressure system, from 0,
 * with the RHS projected to zero mean (consistent system). */
static int pcg(const ocase *c, const double *ap, const double *anb, const double *b, double *x,
               double rtol, int maxit, double *r0n, double *rfn) {
    const int n = c->ne;
    double *r = o_alloc(n + 1, 8), *z = o_alloc(n + 1, 8), *pp = o_alloc(n + 1, 8), *q = o_alloc(n + 1, 8);
    double mean = 0.;
    for (int e = 1; e <= n; e++) mean = mean + b[e];
    mean = mean / n;
    O_PAR
    for (int e = 1; e <= n; e++) { r[e] = b[e] - mean; x[e] = 0.; }
    double bn = sqrt(vdot(n, r, r)), rn = bn, rz, rz1, alpha, beta;
    *r0n = bn;
    double tol = rtol * bn;
    int it = 0;
    O_PAR
    for (int e = 1; e <= n; e++) { z[e] = r[e]/ap[e]; pp[e] = z[e]; }
    rz = vdot(n, r, z);
    while (rn > tol && it < maxit) {
        it++;
        amul(c, ap, anb, pp, q);
        double pq = vdot(n, pp, q);
        if (pq <= 0.) break;
        alpha = rz / pq;
        O_PAR
        for (int e = 1; e <= n; e++) { x[e] = x[e] + alpha*pp[e]; r[e] = r[e] - alpha*q[e]; }
        rn = sqrt(vdot(n, r, r));
        O_PAR
        for (int e = 1; e <= n; e++) z[e] = r[e]/ap[e];
        rz1 = vdot(n, r, z);
        beta = rz1 / rz;
        rz = rz1;
        O_PAR
        for (int e = 1; e <= n; e++) pp[e] = z[e] + beta*pp[e];
    }
    *rfn = rn;
    free(r); free(z); free(pp); free(q);
    return it;
}

void or_solve_momentum(ocase *c, int comp, or_stats *st) {
    double *phi = comp == 0 ? c->u : comp == 1 ? c->v : c->w;
    const double *b = comp == 0 ? c->bu : comp == 1 ? c->bv : c->bw;
    int it; double ri, rf, rm = 0.;
    if (c->cfg.mode == 0)
        solve_gs(0, phi, c->ap, c->anb, b, c->ef2nb_idx, c->ef2nb1, c->ne, c->cfg.nit, &it, &ri, &rf, &rm);
    else
        it = bicgstab(c, c->ap, c->anb, b, phi, c->cfg.tight_rtol, c->cfg.tight_maxit, &ri, &rf);
    if (st) {
        if (comp == 0) st->it_u = it; else if (comp == 1) st->it_v = it; else st->it_w = it;
        st->res_i[comp] = ri; st->res_f[comp] = rf; st->res_max[comp] = rm;
    }
}

/* set_a_0(phic) + solve('pc'), mod_uvwp.f90:126-127, mod_solver.f90:329-344 */
void or_solve_pc(ocase *c, or_stats *st) {
    int it; double ri, rf, rm = 0.;
    for (int e = 1; e <= c->ne + c->nbf; e++) c->phic[e] = 0.;
    if (c->cfg.mode == 0) {
        if (c->nsubd == 1)
            solve_gs(1, c->phic, c->ap, c->anb, c->b, c->ef2nb_idx, c->ef2nb1, c->ne, c->cfg.nit, &it, &ri, &rf, &rm);
        else
            multi_subdomain_solver(c, c->ap, c->anb, c->b, c->phic, c->cfg.nit, &it, &ri, &rf, &rm);
    } else {
        it = pcg(c, c->ap, c->anb, c->b, c->phic, c->cfg.tight_rtol, c->cfg.tight_maxit, &ri, &rf);
    }
    if (st) { st->it_p = it; st->res_i[3] = ri; st->res_f[3] = rf; st->res_max[3] = rm; }
}

/* solve_uvwp, mod_uvwp.f90:95-134 */
void or_solve_uvwp(ocase *c, or_stats *st) {
    const size_t nc = (size_t)c->ne + c->nbf;
    or_stats dummy;
    if (!st) st = &dummy;
    or_calc_coef_uvw(c);
    or_solve_momentum(c, 0, st);
    or_solve_momentum(c, 1, st);
    or_solve_momentum(c, 2, st);
    calc_grad(c, c->u, c->gu);
    calc_grad(c, c->v, c->gv);
    calc_grad(c, c->w, c->gw);
    or_calc_mip(c, 1);
    or_calc_coef_p(c);
    or_solve_pc(c, st);
    adjust_pc(c, c->phic, c->phic[1]);
    calc_grad(c, c->phic, c->gpc);
    update_uvwp(c, c->phic);
    (void)nc;
}

/* main.f90:50-63; with the energy equation set up, its solve follows
 * solve_uvwp where main.f90:58 has it (commented out in the reference). */
void or_run(ocase *c, int n_outer, int ncoef, or_stats *last) {
    for (int k = 1; k <= n_outer; k++) {
        or_update_boundaries(c);
        or_solve_uvwp(c, last);
        if (c->energy_on) or_solve_energy(c, last);
        if (ncoef > 0 && k % ncoef == 0) or_update_time(c);
    }
}

/* the routines the energy equation shares with solve_uvwp */
double o_vec_weight(const double *r0, const double *r1, const double *r2) { return vec_weight(r0, r1, r2); }
void o_calc_grad(ocase *c, const double *phi, double *grad) { calc_grad(c, phi, grad); }
void o_solve_gs(int is_pc, double *phi, const double *ap, const double *anb, const double *b,
                const int *ef2nb_idx, const int *ef2nb, int ne, int nit,
                int *it_out, double *ri, double *rf, double *rmax) {
    solve_gs(is_pc, phi, ap, anb, b, ef2nb_idx, ef2nb, ne, nit, it_out, ri, rf, rmax);
}
int o_bicgstab(const ocase *c, const double *ap, const double *anb, const double *b, double *phi,
               double rtol, int maxit, double *r0n, double *rfn) {
    return bicgstab(c, ap, anb, b, phi, rtol, maxit, r0n, rfn);
}
