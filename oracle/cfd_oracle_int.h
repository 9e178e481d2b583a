/* Internal state of the CPU oracle (test infrastructure only).
 * Arrays are allocated with one extra slot and indexed 1-based, exactly like
 * the Fortran they restate. */
#ifndef CFD_ORACLE_INT_H
#define CFD_ORACLE_INT_H
#include "cfd_oracle.h"
#include <stddef.h>

/* CGNS element type codes, src/modules/mod_util.f90:18-39 */
enum { O_TRI_3 = 5, O_QUAD_4 = 7, O_TETRA_4 = 10, O_PYRA_5 = 12, O_PENTA_6 = 14, O_HEXA_8 = 17 };

typedef struct {
    int ne, nf, nbf;
    int *ef2nb;      /* [1..2nf-nbf] packed index_t(enb,lfnb) (1 column)   */
    int *ef2nb_idx;  /* [1..ne+1]                                            */
    double *ap, *anb, *b, *phic;
} osubd;

typedef struct {
    int c1, c2, ncs;
    int *index1;     /* [1..ncs] owned */
    int *index2;     /* alias of intf(c2,c1)%index1 */
} ointf;

typedef enum { BC_NONE = 0, BC_LID, BC_DIRICHLET0, BC_SYMMETRY } obc_kind;

typedef struct {
    obc_kind kind;
    int esec1, esec2;
    int is_dirichlet;   /* bc_type: 1 dirichlet, 2 zero_flux, 0 unset */
} obc;

struct ocase {
    /* ---- mesh (mod_mg_lvl_uns.f90:12-58) ---- */
    int nvx, nelem, ne, nf, nbf, nsec, ne2vxmax, H;
    double *x, *y, *z;          /* [1..nvx] */
    int *e2vx;                  /* e2vx(j,e) = e2vx[(e-1)*ne2vxmax + j-1] */
    int *esec;                  /* esec(k,s) = esec[2*(s-1)+k-1], sorted */
    int *etype;                 /* [1..nsec] sorted */
    char (*secname)[33];        /* [1..nsec] sorted */
    int *sec2intf, *intf2sec, nintf_c2b;
    int *bs_idx;                /* [1..nsec+1] */
    int *ef2nb1, *ef2nb2;       /* gs2nb(:,1), gs2nb(:,2) [1..H] */
    int *ef2nb_idx;             /* [1..ne+1] */
    int *s2g;                   /* [1..nf] */
    int *bs_store;              /* bs(e) for e in ne+1..ne+nbf: bs_store[e-ne] */
    int *red; int nred;         /* [1..ne] red then black (calc_redblack) */
    double *aip, *rip;          /* [1..3nf] */
    double *xc, *yc, *zc;       /* [1..nelem] */
    double *vol;                /* [1..ne] */
    /* ---- partition (level 1) ---- */
    int nsubd;
    int *gf2g;                  /* [1..ne] */
    int *g2gf, *g2gf_idx;       /* [1..ne], [1..nsubd+1] */
    osubd *sd;                  /* [1..nsubd] */
    ointf *intf;                /* intf(c,cnb) = intf[(cnb-1)*nsubd + c-1] */
    /* ---- physics ---- */
    or_config cfg;
    int phys_ready;
    double *rho, *mu;           /* [1..ne] */
    double *u, *v, *w, *p, *u0, *v0, *w0;    /* [1..ne+nbf] */
    double *gu, *gv, *gw, *gp, *gpc;         /* [1..3(ne+nbf)] */
    double *mip, *mip0;                      /* [1..nf] */
    double *bu, *bv, *bw, *d, *dc;           /* [1..ne] */
    double *ap, *b, *anb, *phic;             /* scratch of phys_t */
    obc *bcs;                                /* [1..nintf_c2b] */
    /* ---- energy equation (mod_energy.f90:5-9), set up by or_energy_init ---- */
    int energy_on;
    double *t, *ephi, *ephi0;                /* [1..ne+nbf] temperature, phi = cp*t, phi0 */
    double *gt, *gephi;                      /* [1..3(ne+nbf)] grad t, grad phi */
    double *cp, *tc;                         /* [1..ne] properties (mod_properties.f90:83-89) */
    double *ebc_t;                           /* [1..nintf_c2b] wall temperature of each bound BC */
};

#define BS(c, e) ((c)->bs_store[(e) - (c)->ne])
#define E2VX(c, j, e) ((c)->e2vx[((size_t)(e) - 1) * (c)->ne2vxmax + (j) - 1])

/* index_t / get_idx at lvl 0: 5-bit side field (mod_util.f90:1428-1448) */
static inline int o_index_t(int g, int s) { return (int)(((unsigned)g << 5) | (unsigned)s); }
static inline void o_get_idx(int idx, int *g, int *s) {
    *s = (int)((unsigned)idx & 31u);
    *g = (int)((unsigned)idx >> 5);
}
/* sgn, mod_util.f90:832-843 */
static inline int o_sgn(int x) { return x >= 0 ? 1 : -1; }

/* Host threads.  Loops whose iterations write only their own cell or face
 * (the assembly, gradient, flux and correction loops, the per-subdomain
 * sweeps of the 4-block pressure solve, the Krylov vector updates) run in
 * parallel: each element's arithmetic is unchanged, so results do not depend
 * on the thread count.  The reference's sequential Gauss-Seidel sweeps stay
 * serial.  Built without OpenMP, O_PAR is empty and everything is serial. */
#ifdef _OPENMP
#define O_PAR _Pragma("omp parallel for schedule(static)")
#else
#define O_PAR
#endif

void *o_alloc(size_t n, size_t sz);
/* shared with the energy equation (cfd_oracle_energy.c) */
double o_vec_weight(const double *r0, const double *r1, const double *r2);
void o_calc_grad(ocase *c, const double *phi, double *grad);
void o_solve_gs(int is_pc, double *phi, const double *ap, const double *anb, const double *b,
                const int *ef2nb_idx, const int *ef2nb, int ne, int nit,
                int *it_out, double *ri, double *rf, double *rmax);
int o_bicgstab(const ocase *c, const double *ap, const double *anb, const double *b, double *phi,
               double rtol, int maxit, double *r0n, double *rfn);
void o_energy_bc(ocase *c);
void o_energy_time(ocase *c);
void o_energy_free(ocase *c);
int o_build_mesh(ocase *c);
int o_build_partition(ocase *c, int nsubd);

#endif
