// cfdl_setup_int.h -- private to the mesh set-up (cfdl_setup.cpp on the host,
// cfdl_gsetup.cu on the device): the element face tables, index packing, the
// set-up object and its build phases.
#pragma once
#include "cfdl.h"
#include "cfdl_par.h"
#include <string>
#include <vector>

#ifdef __CUDACC__
#define CFDL_HD __host__ __device__
#else
#define CFDL_HD
#endif

namespace cfdl_setup_detail {

// element tables, src/modules/mod_util.f90:54-169
CFDL_HD inline const int *faces_tetra4(int f) {
    static constexpr int t[4][4] = {{1, 3, 2, 0}, {1, 2, 4, 0}, {2, 3, 4, 0}, {3, 1, 4, 0}};
    return t[f - 1];
}
CFDL_HD inline const int *faces_pyra5(int f) {
    static constexpr int t[5][4] = {{1, 4, 3, 2}, {1, 2, 5, 0}, {2, 3, 5, 0}, {3, 4, 5, 0}, {4, 1, 5, 0}};
    return t[f - 1];
}
CFDL_HD inline const int *faces_penta6(int f) {
    static constexpr int t[5][4] = {{1, 2, 5, 4}, {2, 3, 6, 5}, {3, 1, 4, 6}, {1, 3, 2, 0}, {4, 5, 6, 0}};
    return t[f - 1];
}
CFDL_HD inline const int *faces_hexa8(int f) {
    static constexpr int t[6][4] = {{1, 4, 3, 2}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 4, 8, 7}, {1, 5, 8, 4}, {5, 6, 7, 8}};
    return t[f - 1];
}
CFDL_HD inline int element_nface(int t) {
    constexpr int n[21] = {0, 6, 0, 0, 0, 1, 1, 1, 1, 1, 4, 4, 5, 5, 5, 5, 5, 6, 6, 6, 0};
    return t >= 0 && t <= 20 ? n[t] : 0;
}
CFDL_HD inline int element_nvx(int t) {
    constexpr int n[21] = {0, 8, 1, 2, 3, 3, 6, 4, 8, 9, 4, 10, 5, 14, 6, 15, 18, 8, 20, 27, 0};
    return t >= 0 && t <= 20 ? n[t] : 0;
}

CFDL_HD inline int index_t(int g, int s) { return (int)(((unsigned)g << 5) | (unsigned)s); }
CFDL_HD inline void get_idx(int idx, int &g, int &s) { s = (int)((unsigned)idx & 31u); g = (int)((unsigned)idx >> 5); }

// face_vxlist, src/modules/mod_util.f90:1361-1423
CFDL_HD inline bool face_vxlist(const int *vx, int t, int f, int *lst, int &nl) {
    switch (t) {
    case CFDL_TETRA_4: { nl = 3; const int *q = faces_tetra4(f); for (int l = 0; l < 3; l++) lst[l] = vx[q[l] - 1]; return true; }
    case 12: { const int *q = faces_pyra5(f); nl = f == 1 ? 4 : 3; for (int l = 0; l < nl; l++) lst[l] = vx[q[l] - 1]; return true; }
    case 14: { const int *q = faces_penta6(f); nl = f <= 3 ? 4 : 3; for (int l = 0; l < nl; l++) lst[l] = vx[q[l] - 1]; return true; }
    case CFDL_HEXA_8: { nl = 4; const int *q = faces_hexa8(f); for (int l = 0; l < 4; l++) lst[l] = vx[q[l] - 1]; return true; }
    case CFDL_TRI_3: nl = 3; for (int l = 0; l < 3; l++) lst[l] = vx[l]; return true;
    case CFDL_QUAD_4: nl = 4; for (int l = 0; l < 4; l++) lst[l] = vx[l]; return true;
    default: return false;
    }
}

}  // namespace cfdl_setup_detail

struct cfdl_setup {
    int nvx = 0, nelem = 0, ne = 0, nf = 0, nbf = 0, nsec = 0, m = 0, nred = 0, nintf = 0;
    std::vector<double> x, y, z;
    std::vector<int> e2vx, esec, etype, sec2intf, intf2sec;
    std::vector<std::string> names;          // file order, as mg%sectionName
    std::vector<int> ef2nb1, ef2nb2, ef2nb_idx, s2g, bs, red;
    cfdl::FillVec<double> aip, rip, xc, yc, zc, vol;   // written in full by the geometry phase
    // boundary-condition binding produced by cfdl_setup_mesh
    mutable std::vector<int> bc_esec, bc_kind;
    mutable std::vector<double> bc_vel, bc_temp;
};

namespace cfdl_setup_detail {
// build phases (status codes); the matching and geometry phases have host
// (cfdl_setup.cpp) and device (cfdl_gsetup.cu) forms with identical results
int init_setup(cfdl_setup &S, int nvx, const double *x, const double *y, const double *z, int nsec,
               const char *names, const int *etype, const int *esec, int ne2vxmax, const int *e2vx);
int order_sections(cfdl_setup &S);
int match_faces_host(cfdl_setup &S);
int match_faces_device(cfdl_setup &S);
int finish_topology(cfdl_setup &S);
int geometry_host(cfdl_setup &S);
int geometry_device(cfdl_setup &S);
int sec_of(const cfdl_setup &S, int e);
}  // namespace cfdl_setup_detail
