/*
 * cfd_oracle_zone.c -- CPU oracle (test infrastructure only): the hex
 * lid-driven-cavity zone in the CGNS shape the reference's cell_input reads
 * (src/setup/cell_input.f90:36-99, src/modules/mod_cgns.f90:31-148), so that
 * an oracle run can be set up without the GPU library.
 *
 * The zone is the benchmark's synthetic input, not a reference routine: the
 * unit cube of n^3 HEXA_8 cells, vertex (i,j,k) at (i,j,k)/n numbered
 * 1 + i + (n+1)(j + (n+1)k), interior vertices jittered per coordinate by
 * U(-jitter, jitter) * h drawn from SplitMix64(seed) in vertex order (x, y, z
 * of one vertex, then the next); one volume section 'Elem' of the cubes in
 * i-fastest order with the CGNS HEXA_8 corner order, then the boundary
 * sections bottom, top, south, north, west, east of QUAD_4 faces, each face's
 * corners ordered so that its normal points out of the cube.  The product's
 * generator makes the same zone (a CPU test compares the two bit for bit).
 */
#include "cfd_oracle.h"
#include <stdint.h>
#include <string.h>

static uint64_t splitmix64(uint64_t *s) {
    uint64_t z = (*s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static double uniform01(uint64_t *s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

static int vid(int n, int i, int j, int k) { return 1 + i + (n + 1) * (j + (n + 1) * k); }

/* sizes[0..3] = nvx, nelem, nsec, ne2vxmax */
int or_box_zone_sizes(int n, int *sizes) {
    if (n < 1 || n > 400) return -1;
    sizes[0] = (n + 1) * (n + 1) * (n + 1);
    sizes[1] = n * n * n + 6 * n * n;
    sizes[2] = 7;
    sizes[3] = 8;
    return 0;
}

static void put(int *e2vx, size_t *e, const int *vs, int cnt) {
    for (int q = 0; q < cnt; q++) e2vx[*e * 8 + q] = vs[q];
    (*e)++;
}

int or_box_zone_fill(int n, double jitter, uint64_t seed, double *x, double *y, double *z, int *e2vx,
                     int *etype, int *esec, char *names) {
    int sz[4];
    if (or_box_zone_sizes(n, sz)) return -1;
    const double h = 1.0 / n;
    uint64_t rng = seed;
    for (int k = 0; k <= n; k++)
        for (int j = 0; j <= n; j++)
            for (int i = 0; i <= n; i++) {
                const int v = vid(n, i, j, k) - 1;
                double px = (double)i / n, py = (double)j / n, pz = (double)k / n;
                const int interior = i > 0 && i < n && j > 0 && j < n && k > 0 && k < n;
                if (interior && jitter != 0.0) {
                    px += (2.0 * uniform01(&rng) - 1.0) * jitter * h;
                    py += (2.0 * uniform01(&rng) - 1.0) * jitter * h;
                    pz += (2.0 * uniform01(&rng) - 1.0) * jitter * h;
                }
                x[v] = px; y[v] = py; z[v] = pz;
            }
    memset(e2vx, 0, sizeof(int) * 8 * (size_t)sz[1]);
    size_t e = 0;
    for (int k = 0; k < n; k++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) {
                const int c[8] = {vid(n, i, j, k), vid(n, i + 1, j, k), vid(n, i + 1, j + 1, k), vid(n, i, j + 1, k),
                                  vid(n, i, j, k + 1), vid(n, i + 1, j, k + 1), vid(n, i + 1, j + 1, k + 1),
                                  vid(n, i, j + 1, k + 1)};
                put(e2vx, &e, c, 8);
            }
    const int ne = (int)e;
    int start[6], stop[6], q[4];
    start[0] = (int)e + 1;   /* bottom z = 0, outward -z */
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
        q[0] = vid(n, i, j, 0); q[1] = vid(n, i, j + 1, 0); q[2] = vid(n, i + 1, j + 1, 0); q[3] = vid(n, i + 1, j, 0);
        put(e2vx, &e, q, 4);
    }
    stop[0] = (int)e; start[1] = (int)e + 1;   /* top z = 1, outward +z */
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
        q[0] = vid(n, i, j, n); q[1] = vid(n, i + 1, j, n); q[2] = vid(n, i + 1, j + 1, n); q[3] = vid(n, i, j + 1, n);
        put(e2vx, &e, q, 4);
    }
    stop[1] = (int)e; start[2] = (int)e + 1;   /* south y = 0, outward -y */
    for (int k = 0; k < n; k++) for (int i = 0; i < n; i++) {
        q[0] = vid(n, i, 0, k); q[1] = vid(n, i + 1, 0, k); q[2] = vid(n, i + 1, 0, k + 1); q[3] = vid(n, i, 0, k + 1);
        put(e2vx, &e, q, 4);
    }
    stop[2] = (int)e; start[3] = (int)e + 1;   /* north y = 1, outward +y */
    for (int k = 0; k < n; k++) for (int i = 0; i < n; i++) {
        q[0] = vid(n, i, n, k); q[1] = vid(n, i, n, k + 1); q[2] = vid(n, i + 1, n, k + 1); q[3] = vid(n, i + 1, n, k);
        put(e2vx, &e, q, 4);
    }
    stop[3] = (int)e; start[4] = (int)e + 1;   /* west x = 0, outward -x */
    for (int k = 0; k < n; k++) for (int j = 0; j < n; j++) {
        q[0] = vid(n, 0, j, k); q[1] = vid(n, 0, j, k + 1); q[2] = vid(n, 0, j + 1, k + 1); q[3] = vid(n, 0, j + 1, k);
        put(e2vx, &e, q, 4);
    }
    stop[4] = (int)e; start[5] = (int)e + 1;   /* east x = 1, outward +x */
    for (int k = 0; k < n; k++) for (int j = 0; j < n; j++) {
        q[0] = vid(n, n, j, k); q[1] = vid(n, n, j + 1, k); q[2] = vid(n, n, j + 1, k + 1); q[3] = vid(n, n, j, k + 1);
        put(e2vx, &e, q, 4);
    }
    stop[5] = (int)e;
    if ((int)e != sz[1]) return -1;
    static const char *bc[6] = {"bottom", "top", "south", "north", "west", "east"};
    memset(names, 0, 33 * 7);
    strncpy(names, "Elem", 32);
    etype[0] = 17;            /* HEXA_8 */
    esec[0] = 1; esec[1] = ne;
    for (int b = 0; b < 6; b++) {
        etype[1 + b] = 7;     /* QUAD_4 */
        esec[2 * (1 + b)] = start[b];
        esec[2 * (1 + b) + 1] = stop[b];
        strncpy(names + 33 * (1 + b), bc[b], 32);
    }
    return 0;
}
