// cfdl_zone.cpp -- synthetic CGNS-shaped zone for the lid-driven cavity.
//
// Produces exactly what the reference's cell_input reads from a CGNS file
// (src/setup/cell_input.f90:36-99, src/modules/mod_cgns.f90:31-148): vertex
// coordinates, the volume section(s) followed by six boundary sections named
// bottom, top, south, north, west, east, and element-to-vertex lists in CGNS
// node order.  Element kinds (the `tet` argument): 0 HEXA_8; 1 TETRA_4 (six
// Kuhn tets per cube); 2 PENTA_6 (two prisms per cube, split along the
// cube's (0,0)-(1,1) diagonal in x-y, so top and bottom are TRI_3); 3 PYRA_5
// (six pyramids per cube with their apex at the cube centre, an extra
// vertex); 4 mixed: HEXA_8 cubes and 6-pyramid cubes in a checkerboard, two
// volume sections (every face between cubes is a quad, so the mesh is
// conformal).  The reference's own sample mesh is not available, so this
// generator stands in for it.
#include "cfdl.h"
#include <cstring>
#include <cstdint>
#include <vector>

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

enum { K_HEX = 0, K_TET = 1, K_PRISM = 2, K_PYRA = 3, K_MIXED = 4 };

const char *kBcNames[6] = {"bottom", "top", "south", "north", "west", "east"};

// cubes split into pyramids: all of them (K_PYRA), the odd ones (K_MIXED)
inline bool pyra_cube(int kind, int i, int j, int k) { return kind == K_PYRA || (kind == K_MIXED && ((i + j + k) & 1)); }
inline long long n_pyra_cubes(int kind, long long n) {
    if (kind == K_PYRA) return n * n * n;
    if (kind == K_MIXED) return n * n * n / 2;   // (i+j+k) odd: floor(n^3/2)
    return 0;
}

}  // namespace

extern "C" int cfdl_box_zone_sizes(int n, int tet, int *nvx, int *nelem, int *nsec, int *ne2vxmax) {
    if (n < 1 || n > 1024 || tet < 0 || tet > K_MIXED) return CFDL_ERR_INVALID;
    const int kind = tet;
    const long long cubes = (long long)n * n * n, npy = n_pyra_cubes(kind, n);
    long long nv = (long long)(n + 1) * (n + 1) * (n + 1) + npy;   // + the pyramid apexes
    long long ne;
    switch (kind) {
    case K_TET: ne = 6 * cubes; break;
    case K_PRISM: ne = 2 * cubes; break;
    default: ne = (cubes - npy) + 6 * npy;
    }
    long long nb = kind == K_TET ? 12LL * n * n : kind == K_PRISM ? 8LL * n * n : 6LL * n * n;
    if (ne + nb > (1LL << 26) - 1) return CFDL_ERR_INVALID;  // index_t packs e<<5 into int32
    if (nvx) *nvx = (int)nv;
    if (nelem) *nelem = (int)(ne + nb);
    if (nsec) *nsec = kind == K_MIXED ? 8 : 7;
    if (ne2vxmax) *ne2vxmax = kind == K_TET ? 4 : kind == K_PRISM ? 6 : kind == K_PYRA ? 5 : 8;
    return CFDL_OK;
}

extern "C" int cfdl_box_zone_fill(int n, int tet, double jitter, uint64_t seed,
                                  double *x, double *y, double *z, int *e2vx,
                                  int *etype, int *esec, char *names) {
    int nvx, nelem, nsec, m;
    int st = cfdl_box_zone_sizes(n, tet, &nvx, &nelem, &nsec, &m);
    if (st) return st;
    const int kind = tet;
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
    // pyramid apexes: the mean of the cube's corners, numbered after the lattice
    const int nlat = (n + 1) * (n + 1) * (n + 1);
    std::vector<int> apex;
    if (n_pyra_cubes(kind, n) > 0) {
        apex.assign((size_t)n * n * n, 0);
        int next = nlat;
        for (int k = 0; k < n; k++)
            for (int j = 0; j < n; j++)
                for (int i = 0; i < n; i++) {
                    if (!pyra_cube(kind, i, j, k)) continue;
                    double sx = 0, sy = 0, sz = 0;
                    for (int c = 0; c < 8; c++) {
                        int v = vid(n, i + (c & 1), j + ((c >> 1) & 1), k + (c >> 2)) - 1;
                        sx += x[v]; sy += y[v]; sz += z[v];
                    }
                    x[next] = sx / 8; y[next] = sy / 8; z[next] = sz / 8;
                    apex[(size_t)i + (size_t)n * (j + (size_t)n * k)] = ++next;   // 1-based id
                }
        if (next != nvx) return CFDL_ERR_MESH;
    }
    std::memset(e2vx, 0, sizeof(int) * (size_t)m * nelem);
    size_t e = 0;  // 0-based element counter
    auto put = [&](const int *vs, int cnt) {
        for (int q = 0; q < cnt; q++) e2vx[e * m + q] = vs[q];
        e++;
    };
    // volume section(s); the mixed kind writes its hex cubes, then its pyramid cubes
    auto corners = [&](int i, int j, int k, int *c) {
        const int cc[8] = {vid(n, i, j, k), vid(n, i + 1, j, k), vid(n, i + 1, j + 1, k), vid(n, i, j + 1, k),
                           vid(n, i, j, k + 1), vid(n, i + 1, j, k + 1), vid(n, i + 1, j + 1, k + 1), vid(n, i, j + 1, k + 1)};
        for (int q = 0; q < 8; q++) c[q] = cc[q];
    };
    int vol_stop[2] = {0, 0};
    for (int pass = 0; pass < (kind == K_MIXED ? 2 : 1); pass++) {
        for (int k = 0; k < n; k++)
            for (int j = 0; j < n; j++)
                for (int i = 0; i < n; i++) {
                    int c[8];
                    corners(i, j, k, c);
                    const bool py = pyra_cube(kind, i, j, k);
                    if (kind == K_MIXED && py != (pass == 1)) continue;
                    if (kind == K_HEX || (kind == K_MIXED && !py)) { put(c, 8); continue; }
                    if (kind == K_PRISM) {
                        // bottom triangles (0,0)(1,0)(1,1) and (0,0)(1,1)(0,1), counterclockwise seen from +z
                        const int a[6] = {c[0], c[1], c[2], c[4], c[5], c[6]}, b[6] = {c[0], c[2], c[3], c[4], c[6], c[7]};
                        put(a, 6); put(b, 6);
                        continue;
                    }
                    if (py) {
                        // one pyramid per cube face: base = the face in reverse of its outward
                        // (faces_hexa8) order, so the pyramid's own base face points outward
                        static const int hf[6][4] = {{1, 4, 3, 2}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 4, 8, 7}, {1, 5, 8, 4}, {5, 6, 7, 8}};
                        const int ap = apex[(size_t)i + (size_t)n * (j + (size_t)n * k)];
                        for (int f = 0; f < 6; f++) {
                            const int q[5] = {c[hf[f][0] - 1], c[hf[f][3] - 1], c[hf[f][2] - 1], c[hf[f][1] - 1], ap};
                            put(q, 5);
                        }
                        continue;
                    }
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
        vol_stop[pass] = (int)e;
    }
    const int ne = (int)e;
    const int nvol = kind == K_MIXED ? 2 : 1;
    const bool tri_tb = kind == K_TET || kind == K_PRISM;   // triangulated top and bottom
    const bool tri_side = kind == K_TET;
    // boundary sections: quads given as (00,10,11,01) in-plane corners, outward
    bool tri = false;
    auto quad = [&](int a0, int a1, int a2, int a3) {
        if (!tri) { int q[4] = {a0, a1, a2, a3}; put(q, 4); return; }
        // split along the in-plane (0,0)-(1,1) diagonal, matching the Kuhn and prism faces
        int t1[3] = {a0, a1, a2}, t2[3] = {a0, a2, a3};
        put(t1, 3); put(t2, 3);
    };
    int start[7], stop[7];
    start[0] = 1; stop[0] = ne;
    // bottom z=0 (outward -z): corners (i,j),(i,j+1),(i+1,j+1),(i+1,j)
    tri = tri_tb;
    start[1] = (int)e + 1;
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++)
        quad(vid(n, i, j, 0), vid(n, i, j + 1, 0), vid(n, i + 1, j + 1, 0), vid(n, i + 1, j, 0));
    stop[1] = (int)e;
    start[2] = (int)e + 1;  // top z=1 (outward +z)
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++)
        quad(vid(n, i, j, n), vid(n, i + 1, j, n), vid(n, i + 1, j + 1, n), vid(n, i, j + 1, n));
    stop[2] = (int)e;
    tri = tri_side;
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
    static const int vtype[5] = {CFDL_HEXA_8, CFDL_TETRA_4, CFDL_PENTA_6, CFDL_PYRA_5, CFDL_HEXA_8};
    // volume sections
    etype[0] = vtype[kind];
    esec[0] = 1;
    esec[1] = nvol == 2 ? vol_stop[0] : ne;
    std::memset(names, 0, 33);
    std::strncpy(names, "Elem", 32);
    if (nvol == 2) {
        etype[1] = CFDL_PYRA_5;
        esec[2] = vol_stop[0] + 1;
        esec[3] = ne;
        std::memset(names + 33, 0, 33);
        std::strncpy(names + 33, "Pyra", 32);
    }
    for (int b = 0; b < 6; b++) {
        const int s = nvol + b;
        const bool t = b < 2 ? tri_tb : tri_side;
        etype[s] = t ? CFDL_TRI_3 : CFDL_QUAD_4;
        esec[2 * s] = start[b + 1];
        esec[2 * s + 1] = stop[b + 1];
        std::memset(names + 33 * s, 0, 33);
        std::strncpy(names + 33 * s, kBcNames[b], 32);
    }
    return CFDL_OK;
}
