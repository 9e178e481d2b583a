/*
 * cfd_oracle.h -- CPU oracle for the CFD-Lite SIMPLE hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a line-by-line restatement, in plain C,
 * of the reference Fortran (serial, FP64) that the GPU library is checked
 * against.  Only the test suite, the smoke check and the CPU-baseline leg of
 * the benchmark may load it; the product library never links or calls it.
 *
 * Parity unpinned: the reference ships no tests, golden vectors or sample
 * mesh and cannot be compiled in this environment (no Fortran compiler, no
 * libcgns), so no output of the reference itself checks this restatement.
 * It is held instead by hand-derivable invariants (exact gradients of linear
 * fields, symmetric zero-row-sum pressure matrices, closed-form face
 * numbering, mass conservation) and by the hash fixtures under tests/golden/,
 * which this oracle produced and the product's independent C++ mesh builder
 * reproduces bit for bit.
 *
 * Conventions follow the reference: all indices are 1-based, packed
 * half-face indices use index_t(e,lf)=e<<5|lf (src/modules/mod_util.f90:1428),
 * reals are double (the reference is built with -r8, build.py:35), integers
 * are int32.
 */
#ifndef CFD_ORACLE_H
#define CFD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ocase ocase;

/* Physics / solver configuration.  The reference hard-codes these
 * (src/modules/mod_physics.f90:15-19, src/modules/mod_properties.f90:86-87,
 * src/equations/mod_uvwp.f90:560); here they are parameters. */
typedef struct {
    double rho;        /* density (reference: 5)                         */
    double mu;         /* viscosity (reference: 0.01)                    */
    double u_lid;      /* lid speed on section 'top' (reference: 1)      */
    double dt;         /* time step; INFINITY = steady (reference: 0.01) */
    double alpha_u;    /* momentum under-relaxation (reference: none = 1) */
    double alpha_p;    /* pressure under-relaxation (reference: none = 1) */
    int    nit;        /* inner sweep cap (reference: 100)               */
    int    mode;       /* 0 = ref (literal GS/SSOR), 1 = tight (Krylov)  */
    double tight_rtol; /* tight mode: ||r||2 <= rtol*||b||2              */
    int    tight_maxit;
} or_config;

typedef struct {
    int    it_u, it_v, it_w, it_p;          /* inner iterations           */
    double res_i[4], res_f[4], res_max[4];  /* u,v,w,pc residual norms    */
    int    it_e;                            /* energy solve (or_solve_energy) */
    double res_e[3];                        /* its initial, final, max residual */
} or_stats;

/* Build the mesh data structures from a CGNS-shaped zone (what cell_input
 * reads, src/setup/cell_input.f90:10-165).  names: nsec blocks of 33 chars.
 * e2vx: ne2vxmax ints per element, element-major, 1-based vertex ids.
 * n_subdomains > 1 builds the oct-tree partition and subdomains. */
ocase *or_create(int nvx, const double *x, const double *y, const double *z,
                 int nsec, const char *names, const int *etype, const int *esec,
                 int ne2vxmax, const int *e2vx, int n_subdomains);
/* Same, from set-up arrays that were already built (what a host that ran
 * cell_input holds): skips find_element_nb and the geometry, keeps the
 * oct-tree partition and subdomains.  Arrays are 0-offset copies of the
 * reference's 1-based-valued arrays; esec/etype/names as in or_create. */
ocase *or_create_from_arrays(int ne, int nf, int nbf, int nsec, const char *names, const int *etype,
                             const int *esec, const int *ef2nb1, const int *ef2nb2, const int *ef2nb_idx,
                             const int *s2g, const int *bs, const double *aip, const double *rip,
                             const double *xc, const double *yc, const double *zc, const double *vol,
                             int n_subdomains);
void or_destroy(ocase *c);

/* sizes: ne, nf, nbf, nvx, nelem, nsec, nred, nsubd, nintf_c2b */
void or_sizes(const ocase *c, int *out9);

/* Copy named arrays out / in.  Integer names: ef2nb1, ef2nb2 (H), ef2nb_idx
 * (ne+1), s2g (nf), bs (nbf, halo ne+1..ne+nbf), bs_idx (nsec+1), esec
 * (2*nsec), etype (nsec), red (ne: red then black), gf2g (ne), g2gf (ne),
 * g2gf_idx (nsubd+1), sec2intf (nsec).
 * Real names: aip, rip (3nf), xc, yc, zc (ne+nbf), vol (ne), u v w p u0 v0 w0
 * (ne+nbf), gu gv gw gp gpc (3(ne+nbf)), mip mip0 (nf), ap b d dc bu bv bw
 * (ne), anb (H), phic (ne+nbf).  Return 0 on success, -1 for unknown name. */
int or_get_int(const ocase *c, const char *name, int *out);
int or_get_dbl(const ocase *c, const char *name, double *out);
int or_set_dbl(ocase *c, const char *name, const double *in);
/* subdomain c (1-based) arrays: ne,nf,nbf then ef2nb_idx, ef2nb */
int or_subdomain_sizes(const ocase *c, int sd, int *out3);
int or_subdomain_get(const ocase *c, int sd, int *ef2nb_idx, int *ef2nb);

/* construct_physics + construct_uvwp (src/modules/mod_physics.f90:52-75,
 * src/equations/mod_uvwp.f90:20-84). */
int  or_physics_init(ocase *c, const or_config *cfg);
void or_set_config(ocase *c, const or_config *cfg);
/* Rebind boundary condition i (1-based, eqn%bcs order) to another of the
 * reference's BC procedures, as an edited construct_uvwp would:
 * 1 lid, 2 dirichlet0, 3 symmetry (mod_uvwp.f90:493-570). */
int  or_set_bc_kind(ocase *c, int i, int kind);
void or_update_boundaries(ocase *c);                 /* mod_physics.f90:38  */
void or_solve_uvwp(ocase *c, or_stats *st);          /* mod_uvwp.f90:95     */
void or_update_time(ocase *c);                       /* mod_physics.f90:101 */
/* n_outer outer iterations of main.f90:50-63: update_boundaries + solve_uvwp,
 * with update_time after every ncoef of them. */
void or_run(ocase *c, int n_outer, int ncoef, or_stats *last);

/* Individual routines (operate on the case state) for per-kernel parity. */
void or_calc_grad(ocase *c, const double *phi, double *grad);  /* mod_solver.f90:40 */
void or_calc_coef_uvw(ocase *c);                               /* mod_uvwp.f90:161  */
void or_calc_mip(ocase *c, int rhie_chow);                     /* mod_uvwp.f90:438  */
void or_calc_coef_p(ocase *c);                                 /* mod_uvwp.f90:289  */
void or_solve_pc(ocase *c, or_stats *st);     /* set_a_0 + solve('pc') mod_uvwp.f90:126-127 */
void or_adjust_pc(ocase *c);                                   /* mod_uvwp.f90:136  */
void or_update_uvwp(ocase *c);                                 /* mod_uvwp.f90:370  */
/* one momentum component solve: comp 0,1,2 = u,v,w; mod_solver.f90:255 */
void or_solve_momentum(ocase *c, int comp, or_stats *st);

/* Energy equation, src/equations/mod_energy.f90 (its solve is commented out
 * of the reference's time loop, main.f90:58; here it runs after solve_uvwp in
 * or_run once set up).  or_energy_init = construct_energy (:14-47) with the
 * properties of init_properties (mod_properties.f90:83-89): cp, tc per cell,
 * t = t_init (reference 273), phi = cp*t, phi0 = phi; the BCs are bound by
 * section name like the uvwp ones: 'top' -> lid (t_lid, reference 373), the
 * other walls -> dirichlet0 (t_wall, reference 273).  After it,
 * or_update_boundaries applies the energy BCs (:173-212) and or_update_time
 * copies phi0 = phi (mod_physics.f90:111).  Field names for or_get_dbl /
 * or_set_dbl: t, e (phi), e0 (phi0) [ne+nbf], gt, ge [3(ne+nbf)], cp, tc [ne].
 * The assembly leaves ap, anb, b in the shared phys_t scratch, as the
 * reference does. */
int  or_energy_init(ocase *c, double cp, double tc, double t_init, double t_lid, double t_wall);
void or_calc_coef_energy(ocase *c);                  /* mod_energy.f90:82-169 */
void or_solve_energy(ocase *c, or_stats *st);        /* mod_energy.f90:59-80  */

/* Timing helper for the CPU baseline: monotonic seconds. */
/* the hex cavity zone in CGNS shape (cfd_oracle_zone.c); sizes = nvx, nelem, nsec, ne2vxmax */
int or_box_zone_sizes(int n, int *sizes);
int or_box_zone_fill(int n, double jitter, uint64_t seed, double *x, double *y, double *z, int *e2vx,
                     int *etype, int *esec, char *names);
double or_wtime(void);
int or_num_threads(void);
void or_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
