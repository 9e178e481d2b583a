// cfdl_zone.cpp -- synthetic CGNS-shaped zone for the lid-driven cavity.
//
// Produces exactly what the reference's cell_input reads from a CGNS file
// (src/setup/cell_input.f90:36-99, src/modules/mod_cgns.f90:31-148): vertex
// coordinates, one volume section followed by six boundary sections named
// bottom, top, south, north, west, east, and element-to-vertex lists in CGNS
// node order (HEXA_8 / TETRA_4 / QUAD_4 / TRI_3).  The reference's own
// sample mesh is not available, so this generator stands in for it.
#include "cfdl.h"
#include <cstring>
#include <cstdint>

namespace {

struct SplitMix64 {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

inline int vid(int n, int i, int j, int k) { return 1 + i + (n + 1) * (j + (n + 1) * k); }

const char *kSecNames[7] = {"Elem", "bottom", "top", "south", "north", "west", "east"};

}  // namespace

extern "C" int cfdl_box_zone_sizes(int n, int tet, int *nvx, int *nelem, int *nsec, int *ne2vxmax) {
    if (n < 1 || n > 1024) return CFDL_ERR_INVALID;
    long long nv = (long long)(n + 1) * (n + 1) * (n + 1);
    long long ne = (long long)n * n * n * (tet ? 6 : 1);
    long long nb = 6LL * n * n * (tet ? 2 : 1);
    if (ne + nb > (1LL << 26) - 1) return CFDL_ERR_INVALID;  // index_t packs e<<5 into int32
    if (nvx) *nvx = (int)nv;
    if (nelem) *nelem = (int)(ne + nb);
    if (nsec) *nsec = 7;
    if (ne2vxmax) *ne2vxmax = tet ? 4 : 8;
    return CFDL_OK;
}

extern "C" int cfdl_box_zone_fill(int n, int tet, double jitter, uint64_t seed,
                                  double *x, double *y, double *z, int *e2vx,
                                  int *etype, int *esec, char *names) {
    int nvx, nelem, nsec, m;
    int st = cfdl_box_zone_sizes(n, tet, &nvx, &nelem, &nsec, &m);
    if (st) return st;
    if (!x || !y || !z || !e2vx || !etype || !esec || !names) return CFDL_ERR_INVALID;
    const double h = 1.0 / n;
    SplitMix64 rng{seed};
    for (int k = 0; k <= n; k++)
        for (int j = 0; j <= n; j++)
            for (int i = 0; i <= n; i++) {
                int v = vid(n, i, j, k) - 1;
                double px = (double)i / n, py = (double)j / n, pz = (double)k / n;
                bool interior = i > 0 && i < n && j > 0 && j < n && k > 0 && k < n;
                if (interior && jitter != 0.0) {
                    px += (2.0 * rng.uniform() - 1.0) * jitter * h;
                    py += (2.0 * rng.uniform() - 1.0) * jitter * h;
                    pz += (2.0 * rng.uniform() - 1.0) * jitter * h;
                }
                x[v] = px; y[v] = py; z[v] = pz;
            }
    std::memset(e2vx, 0, sizeof(int) * (size_t)m * nelem);
    size_t e = 0;  // 0-based element counter
    auto put = [&](const int *vs, int cnt) {
        for (int q = 0; q < cnt; q++) e2vx[e * m + q] = vs[q];
        e++;
    };
    // volume section
    for (int k = 0; k < n; k++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) {
                int c[8] = {vid(n, i, j, k), vid(n, i + 1, j, k), vid(n, i + 1, j + 1, k), vid(n, i, j + 1, k),
                            vid(n, i, j, k + 1), vid(n, i + 1, j, k + 1), vid(n, i + 1, j + 1, k + 1), vid(n, i, j + 1, k + 1)};
                if (!tet) { put(c, 8); continue; }
                // Kuhn split along (i,j,k)-(i+1,j+1,k+1): one tet per axis order.
                static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
                for (int t = 0; t < 6; t++) {
                    int o[3] = {0, 0, 0}, p[4][3];
                    for (int q = 0; q < 3; q++) p[0][q] = 0;
                    for (int s = 0; s < 3; s++) {
                        o[perm[t][s]] = 1;
                        for (int q = 0; q < 3; q++) p[s + 1][q] = o[q];
                    }
                    // orientation from the lattice: (p1-p0)x(p2-p0).(p3-p0) > 0
                    int a[3], b[3], cc[3];
                    for (int q = 0; q < 3; q++) { a[q] = p[1][q] - p[0][q]; b[q] = p[2][q] - p[0][q]; cc[q] = p[3][q] - p[0][q]; }
                    int det = (a[1] * b[2] - a[2] * b[1]) * cc[0] + (a[2] * b[0] - a[0] * b[2]) * cc[1] + (a[0] * b[1] - a[1] * b[0]) * cc[2];
                    int vv[4];
                    for (int s = 0; s < 4; s++) vv[s] = vid(n, i + p[s][0], j + p[s][1], k + p[s][2]);
                    if (det < 0) { int t2 = vv[1]; vv[1] = vv[2]; vv[2] = t2; }
                    put(vv, 4);
                }
            }
    const int ne = (int)e;
    // boundary sections: quads given as (00,10,11,01) in-plane corners, outward
    auto quad = [&](int a0, int a1, int a2, int a3) {
        if (!tet) { int q[4] = {a0, a1, a2, a3}; put(q, 4); return; }
        // split along the in-plane (0,0)-(1,1) diagonal, matching the Kuhn faces
        int t1[3] = {a0, a1, a2}, t2[3] = {a0, a2, a3};
        put(t1, 3); put(t2, 3);
    };
    int start[7], stop[7];
    start[0] = 1; stop[0] = ne;
    // bottom z=0 (outward -z): corners (i,j),(i,j+1),(i+1,j+1),(i+1,j)
    start[1] = (int)e + 1;
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++)
        quad(vid(n, i, j, 0), vid(n, i, j + 1, 0), vid(n, i + 1, j + 1, 0), vid(n, i + 1, j, 0));
    stop[1] = (int)e;
    start[2] = (int)e + 1;  // top z=1 (outward +z)
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++)
        quad(vid(n, i, j, n), vid(n, i + 1, j, n), vid(n, i + 1, j + 1, n), vid(n, i, j + 1, n));
    stop[2] = (int)e;
    start[3] = (int)e + 1;  // south y=0 (outward -y)
    for (int k = 0; k < n; k++) for (int i = 0; i < n; i++)
        quad(vid(n, i, 0, k), vid(n, i + 1, 0, k), vid(n, i + 1, 0, k + 1), vid(n, i, 0, k + 1));
    stop[3] = (int)e;
    start[4] = (int)e + 1;  // north y=1 (outward +y)
    for (int k = 0; k < n; k++) for (int i = 0; i < n; i++)
        quad(vid(n, i, n, k), vid(n, i, n, k + 1), vid(n, i + 1, n, k + 1), vid(n, i + 1, n, k));
    stop[4] = (int)e;
    start[5] = (int)e + 1;  // west x=0 (outward -x)
    for (int k = 0; k < n; k++) for (int j = 0; j < n; j++)
        quad(vid(n, 0, j, k), vid(n, 0, j, k + 1), vid(n, 0, j + 1, k + 1), vid(n, 0, j + 1, k));
    stop[5] = (int)e;
    start[6] = (int)e + 1;  // east x=1 (outward +x)
    for (int k = 0; k < n; k++) for (int j = 0; j < n; j++)
        quad(vid(n, n, j, k), vid(n, n, j + 1, k), vid(n, n, j + 1, k + 1), vid(n, n, j, k + 1));
    stop[6] = (int)e;
    if ((int)e != nelem) return CFDL_ERR_MESH;
    for (int s = 0; s < 7; s++) {
        etype[s] = s == 0 ? (tet ? CFDL_TETRA_4 : CFDL_HEXA_8) : (tet ? CFDL_TRI_3 : CFDL_QUAD_4);
        esec[2 * s] = start[s];
        esec[2 * s + 1] = stop[s];
        std::memset(names + 33 * s, 0, 33);
        std::strncpy(names + 33 * s, kSecNames[s], 32);
    }
    return CFDL_OK;
}
