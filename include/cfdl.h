/*
 * cfdl.h -- C-ABI of libcfdgpu, the GB300 (sm_103a) implementation of the
 * CFD-Lite SIMPLE outer iteration (solve_uvwp and its callees).
 *
 * The boundary mirrors the reference's Fortran interfaces.  Arrays use the
 * reference layouts (1-based index values, Fortran column order, xyz
 * interleaving), real = double, integer = int32, and every array is passed as
 * a plain pointer to its first element, like the reference's existing
 * bind(C) crossings (src/VTK/mod_vtk.f90:4-29).  The caller keeps ownership
 * of all host arrays.  Every entry point returns a status code (CFDL_OK = 0).
 *
 * Threading: one CUDA stream per context; a context is not thread-safe;
 * different contexts may be used from different threads.  A set-up object is
 * read-only after creation except for cfdl_setup_mesh, which fills the
 * boundary-condition tables the returned cfdl_mesh points into: call it from
 * one thread at a time per set-up.
 */
#ifndef CFDL_H
#define CFDL_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define CFDL_OK             0
#define CFDL_ERR_INVALID    1   /* bad argument or size                     */
#define CFDL_ERR_OOM        2   /* device or host allocation failed         */
#define CFDL_ERR_NONFINITE  3   /* NaN/Inf detected in a solve              */
#define CFDL_ERR_ITER_CAP   4   /* inner solve hit its iteration cap (tight) */
#define CFDL_ERR_CUDA       5   /* CUDA runtime error                        */
#define CFDL_ERR_MESH       6   /* connectivity could not be built           */
#define CFDL_ERR_NO_DEVICE  7   /* no CUDA device                            */
#define CFDL_ERR_NAME       8   /* unknown array name                        */
#define CFDL_ERR_BREAKDOWN 10   /* CG breakdown: p.Ap <= 0 above the tolerance
                                   (the matrix is not positive definite)     */

/* CGNS element type codes (src/modules/mod_util.f90:18-39) */
#define CFDL_TRI_3    5
#define CFDL_QUAD_4   7
#define CFDL_TETRA_4 10
#define CFDL_PYRA_5  12
#define CFDL_PENTA_6 14
#define CFDL_HEXA_8  17

/* Boundary condition kinds, the procedures the reference binds per section
 * in construct_uvwp (src/equations/mod_uvwp.f90:73-78, 493-570). */
#define CFDL_BC_WALL      1   /* dirichlet0 / lid: halo velocity = wall velocity, bc_type 'dirichlet' */
#define CFDL_BC_SYMMETRY  2   /* symmetry: reflected velocity, bc_type 'zero_flux' */

/* ======================================================================
 * 1. Synthetic CGNS-shaped zone (the input the reference reads with
 *    cell_input, src/setup/cell_input.f90:36-99).  Unit cube of n^3 cubes;
 *    `tet` is the element kind: 0 one HEXA_8 per cube, 1 six Kuhn TETRA_4,
 *    2 two PENTA_6 (split along the x-y diagonal), 3 six PYRA_5 with the
 *    apex at the cube centre (an extra vertex per cube), 4 HEXA_8 and
 *    6-pyramid cubes in a checkerboard (two volume sections).  Sections:
 *    volume, then bottom, top, south, north, west, east (QUAD_4, or TRI_3
 *    where the cubes' faces are split).  Interior lattice vertices are
 *    jittered by U(-jitter,jitter)*h per coordinate, drawn from
 *    SplitMix64(seed) in vertex order; an apex is the mean of its cube's
 *    corners.  names: nsec blocks of 33 chars.
 * ====================================================================== */
int cfdl_box_zone_sizes(int n, int tet, int *nvx, int *nelem, int *nsec, int *ne2vxmax);
int cfdl_box_zone_fill(int n, int tet, double jitter, uint64_t seed,
                       double *x, double *y, double *z, int *e2vx,
                       int *etype, int *esec, char *names);

/* ======================================================================
 * 2. Mesh set-up: the connectivity and geometry arrays that the reference's
 *    cell_input builds (find_element_nb, calc_aip_xyzip_uns,
 *    calc_vol_cv_centers_uns; src/setup/mod_mg_lvl_uns.f90:283-488,
 *    src/setup/calc_aip_xyzip.f90:7-74, src/setup/calc_vol_cv_centers.f90:4-61),
 *    with the same face numbering, orientation and ordering.  A Fortran host
 *    that already ran cell_input skips this and fills cfdl_mesh from geom.
 * ====================================================================== */
typedef struct cfdl_setup cfdl_setup;

typedef struct cfdl_mesh {
    int ne, nf, nbf;             /* cells, faces, boundary faces (= halos)   */
    const int *ef2nb1;           /* [2nf-nbf] geom%ef2nb(:,1): enb<<5|lfnb    */
    const int *ef2nb2;           /* [2nf-nbf] geom%ef2nb(:,2): +-fg           */
    const int *ef2nb_idx;        /* [ne+1]    geom%ef2nb_idx                  */
    const int *s2g;              /* [nf]      fine_lvl%s2g: owner<<5|lf       */
    const int *bs;               /* [nbf]     fine_lvl%bs(ne+1:ne+nbf)        */
    const double *aip, *rip;     /* [3nf]                                     */
    const double *xc, *yc, *zc;  /* [ne+nbf]                                  */
    const double *vol;           /* [ne]                                      */
    int nbc;                     /* boundary conditions, eqn%bcs order        */
    const int *bc_esec;          /* [2nbc] halo element range of each bc      */
    const int *bc_kind;          /* [nbc]  CFDL_BC_*                          */
    const double *bc_vel;        /* [3nbc] wall velocity (lid: (U,0,0))       */
    const double *bc_temp;       /* [nbc] wall temperature of the energy BCs
                                    (lid 373, dirichlet0 273; mod_energy.f90:
                                    173-212); NULL: no energy equation        */
} cfdl_mesh;

int cfdl_setup_create(int nvx, const double *x, const double *y, const double *z,
                      int nsec, const char *names, const int *etype, const int *esec,
                      int ne2vxmax, const int *e2vx, cfdl_setup **out);
/* The same set-up with the face matching, face numbering and geometry on
 * the current CUDA device (bucketed by smallest vertex instead of a global
 * sort); the arrays equal cfdl_setup_create's bit for bit.  The reference's
 * counterpart is the same cell_input path (next item of the hot-path scope:
 * the connectivity builder for large meshes). */
int cfdl_setup_create_device(int nvx, const double *x, const double *y, const double *z,
                             int nsec, const char *names, const int *etype, const int *esec,
                             int ne2vxmax, const int *e2vx, cfdl_setup **out);
/* sizes[0..4] = ne, nf, nbf, nsec, nred */
int cfdl_setup_sizes(const cfdl_setup *s, int *sizes);
/* Fill a cfdl_mesh whose pointers stay valid until cfdl_setup_destroy.
 * Boundary conditions are bound by section name as construct_uvwp does:
 * 'top' -> moving wall (u_lid,0,0), every other 2D section -> wall at rest;
 * the energy BCs as construct_energy binds them: 'top' -> lid (373), every
 * other section -> dirichlet0 (273). */
int cfdl_setup_mesh(const cfdl_setup *s, double u_lid, cfdl_mesh *mesh);
/* Copy out named integer arrays: ef2nb1, ef2nb2, ef2nb_idx, s2g, bs, esec,
 * etype, red (calc_redblack order, src/setup/mod_meshds_uns.f90:134-204). */
int cfdl_setup_get_int(const cfdl_setup *s, const char *name, int *out);
/* Copy out named real arrays: aip, rip (3nf), xc, yc, zc (ne+nbf), vol (ne). */
int cfdl_setup_get_dbl(const cfdl_setup *s, const char *name, double *out);
int cfdl_setup_destroy(cfdl_setup *s);

/* ======================================================================
 * 3. Device context: mesh and fields resident in HBM.
 * ====================================================================== */
typedef struct cfdl_ctx cfdl_ctx;

typedef struct cfdl_config {
    double rho, mu;        /* properties (reference: 5, 0.01; mod_properties.f90:86-87) */
    double dt;             /* time step (reference 0.01; INFINITY = steady)             */
    double alpha_u;        /* momentum under-relaxation (1 = none, as the reference)    */
    double alpha_p;        /* pressure under-relaxation (1 = none)                      */
    int    nit;            /* inner iteration cap (reference phys%nit = 100)            */
    int    solve_mode;     /* 0: stop each inner solve at a residual drop of rtol_*;
                              1: tight, ||r||2 <= tight_rtol*||b||2 (parity mode)        */
    double rtol_u, rtol_p; /* mode 0 residual drop (reference: 0.1)                      */
    double tight_rtol;     /* mode 1 tolerance                                           */
    int    tight_maxit;    /* mode 1 iteration cap                                       */
    int    precision;      /* 0: FP64 throughout; 1: mixed pressure solve (FP32 SpMV,
                              preconditioner and inner CG, FP64 residual/refinement);
                              2: as 1, and each momentum solve (and the energy
                              solve) finds its correction to the FP64 residual with
                              FP32 BiCGStab (solve_mode 0 only: the reference's 10x
                              drop, no refinement needed);
                              3: as 2, and the explicit momentum face terms (sumss and
                              the deferred non-orthogonal correction of calc_coef_uvw)
                              and the gradients of u, v, w they use are FP32, as is
                              the Rhie-Chow term of calc_mip; the implicit
                              coefficients, the fluxes themselves and the pressure
                              equation stay FP64 (solve_mode 0 only)                   */
    int    precond;        /* pressure preconditioner: 0 Jacobi, 1 aggregation AMG      */
} cfdl_config;

typedef struct cfdl_stats {
    int    it_u, it_v, it_w, it_p;   /* inner iterations of the last solve_uvwp       */
    double res_i[4], res_f[4];       /* initial/final residual 2-norms (u,v,w,pc)     */
    double mass_imbalance;           /* ||b||2 of calc_coef_p (net inflow per cell)   */
    int    status;
    /* progress of cfdl_run (zero until a run target is set) */
    int    outer_done;               /* outer iterations run since cfdl_case_set_run  */
    int    run_left;                 /* outer iterations still to run                 */
    int    converged;                /* 1 once mass_ratio <= the run's tolerance      */
    double mass_ratio;               /* mass_imbalance / sum_f |mip_f| after the pass */
    /* the last energy solve (cfdl_solve_energy) */
    int    it_e;                     /* inner iterations                              */
    double res_e[2];                 /* initial and final residual 2-norms            */
} cfdl_stats;

/* Fields in reference layout (host pointers; NULL members are skipped). */
typedef struct cfdl_fields {
    double *u, *v, *w, *p;           /* [ne+nbf]      */
    double *u0, *v0, *w0;            /* [ne+nbf]      */
    double *gu, *gv, *gw, *gp, *gpc; /* [3(ne+nbf)]   */
    double *mip, *mip0;              /* [nf]          */
} cfdl_fields;

void cfdl_config_default(cfdl_config *cfg);
/* construct_physics + construct_uvwp (mod_physics.f90:52-75, mod_uvwp.f90:20-84):
 * upload the mesh, zero the fields, set rho/mu, bind BCs, mip = calc_mip(.false.),
 * mip0 = mip. */
int cfdl_ctx_create(const cfdl_mesh *mesh, const cfdl_config *cfg, cfdl_ctx **out);
/* The host-side checks cfdl_ctx_create makes of a mesh before it touches the
 * device (sizes, CSR offsets, every neighbour and face index, one owner per
 * face agreeing with s2g, halos against bs, boundary-condition ranges and
 * kinds): CFDL_OK, CFDL_ERR_INVALID or CFDL_ERR_OOM.  Needs no GPU.  The
 * reference trusts its mesh reader (cell_input.f90) and checks nothing. */
int cfdl_mesh_check(const cfdl_mesh *mesh);
int cfdl_set_config(cfdl_ctx *ctx, const cfdl_config *cfg);
int cfdl_upload_fields(cfdl_ctx *ctx, const cfdl_fields *f);
int cfdl_download_fields(cfdl_ctx *ctx, cfdl_fields *f);
int cfdl_ctx_destroy(cfdl_ctx *ctx);

/* ---- the hot path (device-resident state) ---- */
int cfdl_update_boundaries(cfdl_ctx *ctx);               /* mod_physics.f90:38-50  */
int cfdl_solve_uvwp(cfdl_ctx *ctx, cfdl_stats *st);      /* mod_uvwp.f90:95-134    */
int cfdl_update_time(cfdl_ctx *ctx);                     /* mod_physics.f90:101-112 */
/* n_outer iterations of main.f90:50-63 (update_boundaries + solve_uvwp,
 * update_time after every ncoef of them). */
int cfdl_step(cfdl_ctx *ctx, int n_outer, int ncoef, cfdl_stats *st);

/* Drop-in for the Fortran solve_uvwp with host arrays: uploads the fields
 * solve_uvwp reads, runs it, downloads what it writes (NULL members are
 * skipped both ways).  u, v, w and their gradients are downloaded while the
 * pressure correction still runs. */
int cfdl_solve_uvwp_host(cfdl_ctx *ctx, cfdl_fields *f, cfdl_stats *st);
/* cfdl_step with host arrays: upload, n_outer passes of update_boundaries +
 * solve_uvwp (+ update_time every ncoef), download as above. */
int cfdl_step_host(cfdl_ctx *ctx, cfdl_fields *f, int n_outer, int ncoef, cfdl_stats *st);
/* cfdl_step_host for a host that leaves some fields alone between calls:
 * keep is a set of CFDL_F_* bits naming the members of f whose host arrays
 * the caller has not modified since the previous cfdl_step_host* call
 * downloaded into them.  Such a member is not uploaded again -- the device
 * copy already equals it -- provided its pointer is the one that call
 * downloaded into and nothing has written the context's device state since
 * (no kernel launch, upload or set_array in between); otherwise it is
 * uploaded as usual.  Every non-NULL member is still downloaded.  A Fortran
 * host whose gradients and face fluxes are only the solver's own state
 * (solve_uvwp's callees write them, the host reads them for output) keeps
 * CFDL_F_GU|GV|GW|GP|GPC|MIP and uploads only u, v, w, p. */
#define CFDL_F_U    (1u << 0)
#define CFDL_F_V    (1u << 1)
#define CFDL_F_W    (1u << 2)
#define CFDL_F_P    (1u << 3)
#define CFDL_F_U0   (1u << 4)
#define CFDL_F_V0   (1u << 5)
#define CFDL_F_W0   (1u << 6)
#define CFDL_F_GU   (1u << 7)
#define CFDL_F_GV   (1u << 8)
#define CFDL_F_GW   (1u << 9)
#define CFDL_F_GP   (1u << 10)
#define CFDL_F_GPC  (1u << 11)
#define CFDL_F_MIP  (1u << 12)
#define CFDL_F_MIP0 (1u << 13)
int cfdl_step_host_keep(cfdl_ctx *ctx, cfdl_fields *f, unsigned keep, int n_outer, int ncoef, cfdl_stats *st);

/* ---- individual routines, for per-routine replacement and parity ---- */
int cfdl_calc_coef_uvw(cfdl_ctx *ctx);                   /* mod_uvwp.f90:161-286   */
int cfdl_solve_momentum(cfdl_ctx *ctx, cfdl_stats *st);  /* mod_uvwp.f90:114-116 (solve_gs x3) */
/* field: 0 u, 1 v, 2 w, 3 phic, 5 energy t and phi; gradient into gu/gv/gw/gpc
 * or gt/ge (mod_solver.f90:40-81) */
int cfdl_calc_grad(cfdl_ctx *ctx, int field);
int cfdl_calc_mip(cfdl_ctx *ctx, int rhie_chow);         /* mod_uvwp.f90:438-490   */
int cfdl_calc_coef_p(cfdl_ctx *ctx);                     /* mod_uvwp.f90:289-368   */
int cfdl_solve_pc(cfdl_ctx *ctx, cfdl_stats *st);        /* mod_uvwp.f90:126-127 + mod_solver.f90:329-344 */
int cfdl_adjust_pc(cfdl_ctx *ctx);                       /* mod_uvwp.f90:136-158   */
int cfdl_update_uvwp(cfdl_ctx *ctx);                     /* mod_uvwp.f90:370-436   */

/* ---- energy equation (src/equations/mod_energy.f90) ----
 * The reference builds it (construct_energy, :14-47) and applies its BCs in
 * update_boundaries, but its solve is commented out of the time loop
 * (main.f90:58).  cfdl_energy_init is construct_energy for every case of the
 * context (cases whose mesh has no bc_temp are refused): properties cp, tc
 * per cell (reference 1000, 5; mod_properties.f90:88-89), t = t_init
 * (reference 273), phi = cp*t, phi0 = phi.  From then on
 * cfdl_update_boundaries also applies the energy BCs (t = wall temperature,
 * phi = cp(owner)*t on the halos), cfdl_update_time also copies phi0 = phi
 * (mod_physics.f90:111), and every outer pass of cfdl_step, cfdl_step_host and
 * cfdl_run solves the energy equation after solve_uvwp, where main.f90:58
 * has the call.  cfdl_solve_energy is solve_energy (:59-80): calc_grad of t
 * and phi, calc_coef_energy (:82-169) into ap/anb/b, the phi solve (mode 0:
 * BiCGStab to the reference's 10x residual drop, mode 1: to tight_rtol), and
 * calc_temperature t = phi/cp (mod_properties.f90:214-221).  The assembly
 * is FP64 in every precision form; precision >= 2 solves for the correction
 * of the FP64 residual in FP32, as the momentum solve does. */
int cfdl_energy_init(cfdl_ctx *ctx, double cp, double tc, double t_init);
int cfdl_solve_energy(cfdl_ctx *ctx, cfdl_stats *st);
int cfdl_calc_coef_energy(cfdl_ctx *ctx);                /* mod_energy.f90:82-169  */

/* Copy a named device array to/from a host buffer in reference layout.
 * Names: u v w p u0 v0 w0 phic (ne+nbf), gu gv gw gp gpc (3(ne+nbf)),
 * mip mip0 (nf), ap b bu bv bw d dc rho mu (ne), anb (2nf-nbf); after
 * cfdl_energy_init also t, e (phi = cp*t), e0 (phi0) (ne+nbf), gt, ge
 * (3(ne+nbf)), cp, tc (ne). */
int cfdl_get_array(cfdl_ctx *ctx, const char *name, double *host);
int cfdl_set_array(cfdl_ctx *ctx, const char *name, const double *host);

/* ---- measurement (CUDA events on the context's stream) ---- */
/* Make device `device` current for the contexts created afterwards on this
 * thread (one process per GPU). */
int cfdl_select_device(int device);
int cfdl_timer_begin(cfdl_ctx *ctx);
int cfdl_timer_end(cfdl_ctx *ctx, double *ms);      /* synchronises */
/* Bracket every launch (kernel = NULL or "") or the launches of one named
 * kernel with events until cfdl_profile_stop, which returns the number of
 * distinct kernels seen; cfdl_profile_get reads kernel i's name (64 chars),
 * launch count and summed device time. */
int cfdl_profile_start(cfdl_ctx *ctx, const char *kernel);
int cfdl_profile_stop(cfdl_ctx *ctx, int *nkernels);
int cfdl_profile_get(cfdl_ctx *ctx, int i, char *name64, int64_t *launches, double *total_ms);
/* The current device's FP64 FMA rate (thread-instructions per second;
 * multiply by 2 for flop/s), measured by a probe kernel of independent DFMA
 * chains on every SM, timed with CUDA events; *ms (optional) receives the
 * probe's duration.  No counterpart in the reference: it is the ceiling of
 * the FP64-bound kernels' roofline. */
int cfdl_probe_fp64(double *fma_per_s, double *ms);

/* ---- allocation-free pressure-correction solve --------------------------
 * No counterpart in the reference.  For callers that cannot allocate GPU
 * memory themselves or let a library do it: a Fortran host whose device
 * arrays belong to another runtime or memory pool, a process held to a fixed
 * device-memory budget, or a time-stepping loop in which allocation is not
 * allowed.  It solves the pressure-correction system A pc = b (the
 * Jacobi-preconditioned CG of cfdl_solve_pc, from pc = 0, right-hand side
 * projected to zero mean, stop at ||r||2 <= rtol*||r0||2 or maxit) on arrays
 * the caller already holds in device memory, in the reference layout:
 *   ef2nb1 [nh], ef2nb_idx [ne+1]: geom%ef2nb(:,1) and geom%ef2nb_idx;
 *   ap [ne], anb [nh], b [ne]: calc_coef_p's coefficients (nh = 2nf-nbf);
 *   phic [ne]: output, the interior cells of the pressure correction.
 * It allocates nothing, on the device or the host: its Krylov vectors,
 * reduction partials and scalars live in one file-scope device array sized
 * for CFDL_NOALLOC_MAX_CELLS cells (about 4.2 MB), which every GPU that loads
 * the library holds until the process exits.  Larger systems are rejected
 * with CFDL_ERR_TOO_LARGE.  Each call asks the runtime for that array's
 * device address with the device current (so a cudaDeviceReset between calls
 * is harmless); the first call on a device also loads the library's device
 * code there, so make it before any stream capture.  Every call shares the
 * one array (the call clears what must start at zero), so calls that overlap
 * on the GPU -- from several host threads, or on one device at the same time
 * -- race.  Work is queued on the legacy default stream and the call returns
 * after synchronising it; iters and rnorm (optional) receive the CG
 * iterations and the final ||r||2.  Status: CFDL_OK when ||r||2 <= rtol*||r0||2;
 * CFDL_ERR_ITER_CAP when CG stopped at maxit above it (as cfdl_solve_pc in
 * tight mode); CFDL_ERR_BREAKDOWN when p.Ap <= 0 above it; CFDL_ERR_NONFINITE
 * for a non-finite value (a zero diagonal entry, say); CFDL_ERR_INVALID for an
 * index outside the arrays (that access is skipped on the device). */
#define CFDL_ERR_TOO_LARGE      9
#define CFDL_NOALLOC_MAX_CELLS  131072
int cfdl_solve_pc_noalloc(int ne, int nh, const int *ef2nb1, const int *ef2nb_idx, const double *ap,
                          const double *anb, const double *b, double *phic, double rtol, int maxit,
                          int *iters, double *rnorm);

/* solve_uvwp runs as one CUDA graph (inner solve loops as device-side while
 * nodes) when on (1, the default), or as individually launched kernels with
 * host polling of the inner convergence when off (0); 2 is the graph with
 * its nodes in one chain instead of the parallel branches (the pressure
 * matrix and multigrid set-up beside the momentum solve, the velocity
 * gradients beside the pressure part).  The results are the same in every
 * mode.  Per-kernel profiling always uses the eager form. */
int cfdl_set_graph_mode(cfdl_ctx *ctx, int on);
/* Programmatic dependent launch of the solver kernels (default on): each
 * kernel may be scheduled while the one before it drains, and waits for it
 * on the device.  Results do not depend on it. */
int cfdl_set_pdl(cfdl_ctx *ctx, int on);
/* 16-bit neighbour offsets in the mixed form's FP32 mesh-level kernels
 * (default on; used only where every case's offsets fit, see
 * cfdl_amg_index_bytes).  Off, those kernels read the int32 indices; the
 * results are the same either way. */
int cfdl_set_index16(cfdl_ctx *ctx, int on);

/* Multigrid hierarchy of case 0 (built on the first AMG pressure solve):
 * *nlev coarse levels; n[0..nlev] cells and W[0..nlev] ELL widths per level
 * (level 0 = the mesh); at most maxlev+1 entries are written. */
int cfdl_amg_info(cfdl_ctx *ctx, int maxlev, int *nlev, int *n, int *W);

/* Bytes per neighbour index that the mixed (precision >= 1) AMG pressure
 * solve's FP32 mesh-level kernels read: 2 when every case's mesh neighbours
 * fit in 16-bit offsets from their cell (checked when the multigrid
 * hierarchy is set up), else 4; 4 for the FP64 form (its kernels read int32
 * indices) and before the first AMG pressure solve.  -1 for a null context. */
int cfdl_amg_index_bytes(const cfdl_ctx *ctx);

/* ---- batches: many independent cases in one context ---------------------
 * No counterpart in the reference, which holds one case per process.  Every
 * case of a context is advanced by the same launches (each kernel's work list
 * holds tiles of all cases; reductions are per case and deterministic), so a
 * case's results do not depend on the other cases sharing the context.  All
 * cases share the pressure-solve form (precision, precond); the other
 * configuration members are per case.  Cases are named by the ids these calls
 * return (the context's first case has id 0); the context-level entry points
 * above address the first case for fields and statistics and advance all of
 * them. */
int cfdl_batch_create(int ncases, const cfdl_mesh *meshes, const cfdl_config *cfgs, cfdl_ctx **ctx);
int cfdl_case_add(cfdl_ctx *ctx, const cfdl_mesh *mesh, const cfdl_config *cfg, int *id);
int cfdl_case_remove(cfdl_ctx *ctx, int id);       /* the last case cannot be removed */
int cfdl_case_count(const cfdl_ctx *ctx);
int cfdl_case_ids(const cfdl_ctx *ctx, int *ids);  /* ids[cfdl_case_count()] */
int cfdl_case_get_array(cfdl_ctx *ctx, int id, const char *name, double *host);
int cfdl_case_set_array(cfdl_ctx *ctx, int id, const char *name, const double *host);
int cfdl_case_stats(cfdl_ctx *ctx, int id, cfdl_stats *stats);
/* cells and device bytes held by one case */
int cfdl_case_info(const cfdl_ctx *ctx, int id, int *ne, size_t *device_bytes);
/* upper estimate of the device bytes of a case, before it is created */
size_t cfdl_case_bytes_estimate(int ne, int nf, int nbf, int W);

/* ---- runs: many outer iterations per launch ------------------------------
 * The reference's time loop (src/modules/mod_physics.f90:23-36:
 * update_boundaries, solve_uvwp, update_time every ncoef outer iterations)
 * with a target per case.  cfdl_case_set_run gives case `id` (-1: every
 * case) n_outer iterations to run, the update_time cadence ncoef (0: never)
 * and a tolerance conv_tol on mass_imbalance / sum_f |mip_f| at which the
 * case stops early (0: none), and resets its progress counters.  cfdl_run
 * then runs up to max_outer passes; in each pass every case with iterations
 * left does one outer iteration and the others are left untouched.  With
 * graphs on (the default) the whole call is one CUDA graph launch.  *running
 * (optional) receives the number of cases with iterations left. */
int cfdl_case_set_run(cfdl_ctx *ctx, int id, int n_outer, int ncoef, double conv_tol);
int cfdl_run(cfdl_ctx *ctx, int max_outer, int *running);

/* ---- solver tile shape and its autotuner ---------------------------------
 * No counterpart in the reference.  The inner-solve kernels give each CTA
 * 256 * vec cells (vec = 1, 2, 4 or 8; default 4).  cfdl_autotune times
 * `outer` outer iterations of the context's own cases with each vec, from a
 * snapshot of their state that it restores afterwards, keeps the fastest and
 * returns it in *best; ms[4] (optional) receives the time per outer
 * iteration of each candidate.  The shape changes the order of the partial
 * sums, so results agree across shapes to rounding, not bit for bit. */
int cfdl_set_tile(cfdl_ctx *ctx, int vec);
int cfdl_get_tile(const cfdl_ctx *ctx);
/* Lanes per row (1, 2 or 4; default 1) on the large coarse multigrid levels
 * (small levels always use 8).  cfdl_autotune also picks this, after vec. */
int cfdl_set_coarse_group(cfdl_ctx *ctx, int lanes);
int cfdl_get_coarse_group(const cfdl_ctx *ctx);
int cfdl_autotune(cfdl_ctx *ctx, int outer, int *best, double *ms);
/* Tile shape (cells per thread: 1, 2, 4, 8) of the energy solve's kernels;
 * cfdl_autotune tunes it too when the energy equation is set up. */
int cfdl_set_energy_tile(cfdl_ctx *ctx, int vec);
int cfdl_get_energy_tile(const cfdl_ctx *ctx);

/* ---- serving loop ---------------------------------------------------------
 * No counterpart in the reference.  Solves lid-driven-cavity requests with
 * continuous batching on one device: host threads prepare each request's mesh
 * (zone, set-up, device tables, multigrid hierarchy) while the device runs;
 * one device thread admits prepared requests in arrival order while a slot is
 * free and their device bytes fit both hbm_budget and the memory the device
 * reports free (less hbm_reserve), runs every resident case `chunk` outer
 * iterations per graph launch (steady SIMPLE, alpha_u/alpha_p, rho = 1,
 * u_lid = 1, mu = 1/re), and retires a case when its mass ratio reaches
 * conv_tol or it has run max_outer iterations.  State stays on the device
 * between outer iterations.  A request's result does not depend on the
 * requests that shared its launches (same tile shape assumed). */
typedef struct cfdl_request {
    int      n;             /* mesh edge: n^3 hexes, or 6 n^3 tets             */
    int      tet;           /* 1: every hex split into 6 tets                  */
    double   jitter;        /* interior-node jitter, fraction of the spacing   */
    uint64_t seed;          /* jitter seed                                     */
    double   re;            /* Reynolds number                                 */
    double   conv_tol;      /* stop at mass_imbalance / sum|mip| <= conv_tol   */
    int      max_outer;     /* outer-iteration cap                             */
    int      keep_fields;   /* 1: keep u, v, w, p for cfdl_server_fields       */
} cfdl_request;

typedef struct cfdl_server_config {
    int    device;
    double hbm_budget;      /* device bytes the resident cases may hold        */
    double hbm_reserve;     /* device bytes always left free                   */
    int    max_cases;       /* resident-case slots                             */
    int    chunk;           /* outer iterations per launch between admissions  */
    int    prep_threads;    /* host threads preparing meshes                   */
    int    precision, precond;   /* pressure-solve form (cfdl_config)          */
    int    tile;            /* solver tile shape (0: the default)              */
    double alpha_u, alpha_p;
    int    device_setup;    /* 1: mesh set-up on the GPU (cfdl_setup_create_device) */
} cfdl_server_config;

typedef struct cfdl_result {
    int64_t id;
    int     status, ne, outer_done, converged;
    double  mass_ratio;
    double  t_submit, t_ready, t_admit, t_done;   /* seconds on the server clock */
} cfdl_result;

typedef struct cfdl_server_info {
    int64_t submitted, done, queued, launches;
    int     resident;
    double  held_bytes, cell_iters, busy_s, now;
} cfdl_server_info;

typedef struct cfdl_server cfdl_server;
void   cfdl_server_config_default(cfdl_server_config *cfg);
int    cfdl_server_create(const cfdl_server_config *cfg, cfdl_server **srv);
int    cfdl_server_submit(cfdl_server *srv, const cfdl_request *req, int64_t *id);  /* thread-safe */
/* up to max finished results not yet returned; waits up to wait_s for one */
int    cfdl_server_poll(cfdl_server *srv, cfdl_result *out, int max, int *n, double wait_s);
/* u, v, w or p [ne+nbf] of a finished request with keep_fields; *len = size */
int    cfdl_server_fields(cfdl_server *srv, int64_t id, const char *name, double *host, int64_t *len);
/* wait until every submitted request is finished (timeout_s <= 0: no limit) */
int    cfdl_server_drain(cfdl_server *srv, double timeout_s);
int    cfdl_server_query(cfdl_server *srv, cfdl_server_info *info);
double cfdl_server_now(cfdl_server *srv);
/* stops at once: unfinished requests are dropped */
int    cfdl_server_destroy(cfdl_server *srv);

/* ---- output --------------------------------------------------------------
 * write_vtubin (src/modules/mod_vtu_output.f90:6-328) for the uvwp equation:
 * the case's u, v, w, p, gpc and net cell mass flux ("mip") read from the
 * device, with the mesh of `setup`, in the reference's VTU byte layout (XML
 * header, raw appended data with UInt64 counts).  path is the file to write
 * (the reference's VTK/output-<iout>/uvwp.vtu; the caller makes the folder). */
int cfdl_write_vtu(cfdl_ctx *ctx, int case_id, const cfdl_setup *setup, const char *path);
/* write_vtubin for the energy equation (mod_vtu_output.f90:124-132): enthalpy
 * (phi), grad_enthalpy, temperature, grad_temperature; the reference's
 * VTK/output-<iout>/energy.vtu.  Needs cfdl_energy_init. */
int cfdl_write_vtu_energy(cfdl_ctx *ctx, int case_id, const cfdl_setup *setup, const char *path);

/* Self-check of the integer-pipe FP64 <-> FP32 conversions of the precision-3
 * kernels against the hardware conversions on n generated values (every
 * binary64 exponent near the binary32 range, ties, signed zeros, infinities,
 * NaN).  mismatches[0]: narrowing differences (binary32 subnormal results,
 * flushed to zero by design, are not counted); mismatches[1]: widening
 * differences on normal binary32 values. */
int cfdl_check_conversions(int n, unsigned *mismatches);

/* Number of kernel launches issued by this context since creation. */
int64_t cfdl_launch_count(const cfdl_ctx *ctx);
/* Human-readable text for a status code. */
const char *cfdl_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif
