/*
 * A host program in plain C that drives libcfdgpu through its C-ABI the way
 * the reference's Fortran host does through ISO_C_BINDING (main.f90:50-63):
 * it builds the cavity zone and its set-up, attaches a device context, keeps
 * the fields in its own arrays and calls cfdl_step_host once per outer pass
 * (update_boundaries + solve_uvwp, update_time every ncoef passes), then
 * writes the fields it holds as raw little-endian doubles for the test to
 * compare.
 *
 * usage: step_host <n> <tet 0/1> <jitter> <seed> <n_outer> <ncoef> <out.bin>
 */
#include "cfdl.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#define CHECK(call)                                                                      \
    do {                                                                                 \
        int st_ = (call);                                                                \
        if (st_ != CFDL_OK) {                                                            \
            fprintf(stderr, "%s failed: %s\n", #call, cfdl_status_string(st_));          \
            return 1;                                                                    \
        }                                                                                \
    } while (0)

int main(int argc, char **argv) {
    if (argc != 8) {
        fprintf(stderr, "usage: %s n tet jitter seed n_outer ncoef out.bin\n", argv[0]);
        return 2;
    }
    const int n = atoi(argv[1]), tet = atoi(argv[2]), n_outer = atoi(argv[5]), ncoef = atoi(argv[6]);
    const double jitter = atof(argv[3]);
    const uint64_t seed = (uint64_t)strtoull(argv[4], NULL, 10);
    int nvx, nelem, nsec, m;
    CHECK(cfdl_box_zone_sizes(n, tet, &nvx, &nelem, &nsec, &m));
    double *x = malloc(sizeof(double) * nvx), *y = malloc(sizeof(double) * nvx), *z = malloc(sizeof(double) * nvx);
    int *e2vx = malloc(sizeof(int) * (size_t)m * nelem), *etype = malloc(sizeof(int) * nsec), *esec = malloc(sizeof(int) * 2 * nsec);
    char *names = malloc((size_t)33 * nsec);
    if (!x || !y || !z || !e2vx || !etype || !esec || !names) return 3;
    CHECK(cfdl_box_zone_fill(n, tet, jitter, seed, x, y, z, e2vx, etype, esec, names));
    cfdl_setup *s = NULL;
    CHECK(cfdl_setup_create(nvx, x, y, z, nsec, names, etype, esec, m, e2vx, &s));
    cfdl_mesh mesh;
    CHECK(cfdl_setup_mesh(s, 1.0, &mesh));
    cfdl_config cfg;
    cfdl_config_default(&cfg);
    cfg.rho = 1.0; cfg.mu = 0.01; cfg.dt = INFINITY;              /* steady */
    cfg.alpha_u = 0.7; cfg.alpha_p = 0.3;
    cfdl_ctx *ctx = NULL;
    CHECK(cfdl_ctx_create(&mesh, &cfg, &ctx));
    /* the host's own field arrays, as the Fortran uvwp_t holds them */
    const size_t nc = (size_t)mesh.ne + mesh.nbf, nf = (size_t)mesh.nf;
    double *u = calloc(nc, 8), *v = calloc(nc, 8), *w = calloc(nc, 8), *p = calloc(nc, 8);
    double *u0 = calloc(nc, 8), *v0 = calloc(nc, 8), *w0 = calloc(nc, 8);
    double *gu = calloc(3 * nc, 8), *gv = calloc(3 * nc, 8), *gw = calloc(3 * nc, 8), *gp = calloc(3 * nc, 8),
           *gpc = calloc(3 * nc, 8);
    double *mip = calloc(nf, 8), *mip0 = calloc(nf, 8);
    if (!u || !v || !w || !p || !u0 || !v0 || !w0 || !gu || !gv || !gw || !gp || !gpc || !mip || !mip0) return 3;
    cfdl_fields f = {u, v, w, p, u0, v0, w0, gu, gv, gw, gp, gpc, mip, mip0};
    CHECK(cfdl_download_fields(ctx, &f));                           /* construct_uvwp's state */
    cfdl_stats st;
    for (int k = 1; k <= n_outer; k++) {
        /* one pass per call, as a host that owns the time loop would make it */
        CHECK(cfdl_step_host(ctx, &f, 1, 0, &st));
        if (ncoef > 0 && k % ncoef == 0) {                          /* update_time on the host's arrays */
            for (size_t i = 0; i < nc; i++) { u0[i] = u[i]; v0[i] = v[i]; w0[i] = w[i]; }
            for (size_t i = 0; i < nf; i++) mip0[i] = mip[i];
        }
    }
    FILE *fo = fopen(argv[7], "wb");
    if (!fo) return 4;
    double *out[4] = {u, v, w, p};
    for (int q = 0; q < 4; q++)
        if (fwrite(out[q], 8, nc, fo) != nc) return 4;
    if (fwrite(mip, 8, nf, fo) != nf) return 4;
    fclose(fo);
    printf("%d outer passes on %d cells: it_p %d, mass imbalance %.3e\n", n_outer, mesh.ne, st.it_p, st.mass_imbalance);
    CHECK(cfdl_ctx_destroy(ctx));
    CHECK(cfdl_setup_destroy(s));
    return 0;
}
