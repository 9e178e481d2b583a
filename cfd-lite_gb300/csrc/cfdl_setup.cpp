// cfdl_setup.cpp -- host-side mesh set-up: from a CGNS-shaped zone to the
// connectivity and geometry arrays the SIMPLE hot path consumes, with the
// reference's exact face numbering, orientation and halo bookkeeping.
//
// The reference builds these in cell_input (src/setup/cell_input.f90:10-165)
// with find_element_nb (src/setup/mod_mg_lvl_uns.f90:283-488), an
// O(nvx*k^2) vertex-pair search.  Its numbering has a closed form: a face is
// numbered at its smallest vertex, and among the faces first met at one vertex
// in the order of (lower element id, local face) of the pair's first entry.
// This builder matches faces with a sort on sorted vertex tuples and numbers
// them by (min vertex, owner element, owner local face), which gives the
// same ef2nb/ef2nb_idx/s2g/bs arrays in O(F log F).  Geometry follows
// calc_aip_xyzip_uns (src/setup/calc_aip_xyzip.f90:7-74) and
// calc_vol_cv_centers_uns (src/setup/calc_vol_cv_centers.f90:4-61) operation
// by operation (compiled without FP contraction), so the doubles are the
// reference's bit for bit.
#include "cfdl_setup_int.h"
#include "cfdl_par.h"
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

namespace cfdl_setup_detail {
namespace {

struct FaceKey {
    int v[4];     // sorted vertex ids, 0-padded at the front for triangles
    int minv;
    int e, f;     // element (1-based) and local face
    bool operator<(const FaceKey &o) const {
        for (int q = 0; q < 4; q++) if (v[q] != o.v[q]) return v[q] < o.v[q];
        if (e != o.e) return e < o.e;
        return f < o.f;
    }
};

}  // namespace

int sec_of(const cfdl_setup &S, int e) {
    for (int s = 0; s < S.nsec; s++) if (e <= S.esec[2 * s + 1]) return s;
    return S.nsec - 1;
}

// Section order and the half-face CSR.
int order_sections(cfdl_setup &S) {
    const int ng = S.ne;
    // order section ranges (add_meshds, mod_mg_lvl_uns.f90:154-168)
    {
        std::vector<int> es = S.esec, et = S.etype;
        int bs_next = 1;
        for (int n = 0; n < S.nsec; n++) {
            bool found = false;
            for (int s = 0; s < S.nsec; s++)
                if (es[2 * s] == bs_next) {
                    S.esec[2 * n] = es[2 * s]; S.esec[2 * n + 1] = es[2 * s + 1]; S.etype[n] = et[s];
                    bs_next = es[2 * s + 1] + 1; found = true; break;
                }
            if (!found) return CFDL_ERR_MESH;
        }
        if (bs_next != S.nelem + 1) return CFDL_ERR_MESH;
        S.sec2intf.assign(S.nsec, 0);
        S.intf2sec.clear();
        for (int s = 0; s < S.nsec; s++)
            if (S.etype[s] < 10) { S.intf2sec.push_back(s + 1); S.sec2intf[s] = (int)S.intf2sec.size(); }
        S.nintf = (int)S.intf2sec.size();
    }
    // CSR (gs2nb_idx) and element faces
    S.ef2nb_idx.assign(ng + 1, 0);
    S.ef2nb_idx[0] = 1;
    for (int e = 1; e <= ng; e++) {
        int t = S.etype[sec_of(S, e)];
        if (t < 10 || t > 20) return CFDL_ERR_MESH;  // volume elements must come first
        S.ef2nb_idx[e] = S.ef2nb_idx[e - 1] + element_nface(t);
    }
    const int H = S.ef2nb_idx[ng] - 1;
    if (H != 2 * S.nf - S.nbf) return CFDL_ERR_MESH;
    return CFDL_OK;
}

// Face matching and numbering: ef2nb1, ef2nb2, s2g, bs.
int match_faces_host(cfdl_setup &S) {
    const int ng = S.ne, m = S.m, H = S.ef2nb_idx[ng] - 1;
    // one key per element face: volume element e's faces at its CSR slots,
    // each 2D element's single face after them (disjoint writes, any order)
    const size_t nk = (size_t)H + (S.nelem - ng);
    std::unique_ptr<FaceKey[]> keys(new FaceKey[nk]);   // every key written below
    std::atomic<int> bad{0};
    cfdl::parallel_for(S.nelem, [&](long b, long e_end) {
        for (long e0 = b; e0 < e_end; e0++) {
            const int e = (int)e0 + 1;
            const int t = S.etype[sec_of(S, e)];
            const size_t base = e <= ng ? (size_t)S.ef2nb_idx[e - 1] - 1 : (size_t)H + (e - ng - 1);
            if (e > ng && element_nface(t) != 1) { bad = 1; return; }
            for (int f = 1; f <= element_nface(t); f++) {
                int lst[4], nl;
                if (!face_vxlist(&S.e2vx[(size_t)(e - 1) * m], t, f, lst, nl)) { bad = 1; return; }
                FaceKey k;
                k.v[0] = 0;
                for (int q = 0; q < nl; q++) k.v[4 - nl + q] = lst[q];
                std::sort(k.v + 4 - nl, k.v + 4);
                k.minv = k.v[4 - nl];
                k.e = e; k.f = f;
                keys[base + f - 1] = k;
            }
        }
    });
    if (bad) return CFDL_ERR_MESH;
    // The two keys of a face share its smallest vertex.  The keys are
    // bucketed by it (a counting sort), and each bucket is sorted and paired
    // on its own: pairs of (lower, higher) element, each bucket's pairs in
    // (element, local face) order.  Buckets in vertex order then give the
    // faces in (smallest vertex, element, local face) order, the numbering of
    // find_element_nb, with no global sort.
    const int nv = S.nvx;
    if (nk % 2 != 0 || (long long)(nk / 2) != S.nf) return CFDL_ERR_MESH;   // some face unmatched
    std::vector<int> start((size_t)nv + 2, 0);     // bucket v: keys order[start[v] .. start[v+1])
    cfdl::parallel_for((long)nk, [&](long b, long e_end) {
        for (long i = b; i < e_end; i++) {
            const int v = keys[i].minv;
            if (v < 1 || v > nv) { bad = 1; continue; }
            __atomic_fetch_add(&start[v + 1], 1, __ATOMIC_RELAXED);
        }
    });
    if (bad) return CFDL_ERR_MESH;
    for (int v = 0; v <= nv; v++) start[v + 1] += start[v];
    std::vector<int> order(nk);
    {
        std::vector<int> fill(start.begin(), start.end() - 1);
        cfdl::parallel_for((long)nk, [&](long b, long e_end) {
            for (long i = b; i < e_end; i++) order[__atomic_fetch_add(&fill[keys[i].minv], 1, __ATOMIC_RELAXED)] = (int)i;
        });
    }
    struct Pair { int minv, e1, f1, e2, f2; };
    std::unique_ptr<Pair[]> pairs(new Pair[nk / 2]);   // every pair written below
    cfdl::parallel_for((long)nv + 1, [&](long vb, long ve) {
        for (long v = vb; v < ve && !bad; v++) {
            const int a = start[v], cnt = start[v + 1] - a;
            if (cnt == 0) continue;
            if (cnt % 2 != 0 || a % 2 != 0) { bad = 1; return; }
            int *o = &order[a];
            std::sort(o, o + cnt, [&](int p, int q) { return keys[p] < keys[q]; });
            Pair *out = &pairs[a / 2];
            for (int i = 0; i < cnt; i += 2) {
                const FaceKey &k1 = keys[o[i]], &k2 = keys[o[i + 1]];   // k1.e < k2.e
                // exactly two keys per face: non-conforming or unmatched otherwise
                if (!std::equal(k1.v, k1.v + 4, k2.v) ||
                    (i + 2 < cnt && std::equal(k2.v, k2.v + 4, keys[o[i + 2]].v)) || k1.e > ng) {   // k1.e > ng: two 2D elements
                    bad = 1;
                    return;
                }
                out[i / 2] = {k1.minv, k1.e, k1.f, k2.e, k2.f};
            }
            std::sort(out, out + cnt / 2, [](const Pair &p, const Pair &q) {
                return p.e1 != q.e1 ? p.e1 < q.e1 : p.f1 < q.f1;
            });
        }
    }, 4096);
    if (bad) return CFDL_ERR_MESH;
    S.ef2nb1.assign(H, 0); S.ef2nb2.assign(H, 0); S.s2g.assign(S.nf, 0); S.bs.assign(S.nbf, 0);
    cfdl::parallel_for(S.nf, [&](long b, long e_end) {
    for (int fg = (int)b + 1; fg <= (int)e_end; fg++) {
        const Pair &p = pairs[fg - 1];
        int idx1 = S.ef2nb_idx[p.e1 - 1] + p.f1 - 1;
        if (p.e2 > ng) {
            S.ef2nb1[idx1 - 1] = index_t(p.e2, 0);
            S.ef2nb2[idx1 - 1] = fg;
            S.s2g[fg - 1] = index_t(p.e1, p.f1);
            S.bs[p.e2 - ng - 1] = index_t(p.e1, p.f1);
        } else {
            int idx2 = S.ef2nb_idx[p.e2 - 1] + p.f2 - 1;
            S.ef2nb1[idx1 - 1] = index_t(p.e2, p.f2);
            S.ef2nb1[idx2 - 1] = index_t(p.e1, p.f1);
            S.ef2nb2[idx1 - 1] = fg;
            S.ef2nb2[idx2 - 1] = -fg;
            S.s2g[fg - 1] = index_t(p.e1, p.f1);
        }
    }
    });
    return CFDL_OK;
}

// Edge boundary marking and the red/black order (sequential in the reference
// and here: both depend on visiting order).
int finish_topology(cfdl_setup &S) {
    const int ng = S.ne;
    // edge boundary faces (mod_mg_lvl_uns.f90:421-433)
    for (int e1 = ng + 1; e1 <= S.nelem; e1++) {
        int &b1 = S.bs[e1 - ng - 1];
        if (b1 < 0) continue;
        int ee, ff;
        get_idx(b1, ee, ff);
        for (int idx = S.ef2nb_idx[ee - 1]; idx <= S.ef2nb_idx[ee] - 1; idx++) {
            if (idx - S.ef2nb_idx[ee - 1] + 1 == ff) continue;
            int e2, f2;
            get_idx(S.ef2nb1[idx - 1], e2, f2);
            if (f2 == 0) {
                b1 = -std::abs(b1);
                S.bs[e2 - ng - 1] = -S.bs[e2 - ng - 1];
            }
        }
    }
    // calc_redblack (mod_meshds_uns.f90:134-204)
    {
        std::vector<int> rb(ng + 1, 0);
        int nred = 0, g = 1;
        bool lexit = false;
        while (g <= ng) {
            while (rb[g] != 0) { if (g == ng) { lexit = true; break; } g++; }
            if (lexit) break;
            bool lfound = true;
            for (int idx = S.ef2nb_idx[g - 1]; idx <= S.ef2nb_idx[g] - 1; idx++) {
                int gnb, fl; get_idx(S.ef2nb1[idx - 1], gnb, fl);
                if (fl != 0 && rb[gnb] == 2) { lfound = false; break; }
            }
            if (lfound) {
                for (int idx = S.ef2nb_idx[g - 1]; idx <= S.ef2nb_idx[g] - 1; idx++) {
                    int gnb, fl; get_idx(S.ef2nb1[idx - 1], gnb, fl);
                    if (fl != 0 && rb[gnb] == 0) { nred++; rb[gnb] = 1; }
                }
                rb[g] = 2;
            } else { nred++; rb[g] = 1; }
            g++;
        }
        S.red.assign(ng, 0);
        int b = nred, r = 0;
        for (g = 1; g <= ng; g++) {
            if (rb[g] == 1) S.red[r++] = g;
            else if (rb[g] == 2) S.red[b++] = g;
        }
        S.nred = nred;
    }
    return CFDL_OK;
}

// Face areas and centroids, cell volumes and centres.
int geometry_host(cfdl_setup &S) {
    const int ng = S.ne, m = S.m;
    // calc_aip_xyzip_uns (calc_aip_xyzip.f90:7-74)
    S.aip.resize(3 * (size_t)S.nf); S.rip.resize(3 * (size_t)S.nf);   // every face written below
    cfdl::parallel_for(S.nf, [&](long b, long e_end) {
    for (int fg = (int)b + 1; fg <= (int)e_end; fg++) {
        int e, fl; get_idx(S.s2g[fg - 1], e, fl);
        int t = S.etype[sec_of(S, e)], lst[4], nl;
        face_vxlist(&S.e2vx[(size_t)(e - 1) * m], t, fl, lst, nl);
        double r[4][3], dr1[3], dr2[3], av[3], sub[3], sumc[3][3];
        double *a = &S.aip[3 * (size_t)(fg - 1)], *ri = &S.rip[3 * (size_t)(fg - 1)];
        for (int q = 0; q < nl; q++) { r[q][0] = S.x[lst[q] - 1]; r[q][1] = S.y[lst[q] - 1]; r[q][2] = S.z[lst[q] - 1]; }
        auto tri = [&](int i0, int i1, int i2, bool first) {
            for (int q = 0; q < 3; q++) { dr1[q] = r[i1][q] - r[i0][q]; dr2[q] = r[i2][q] - r[i0][q]; }
            av[0] = dr1[1] * dr2[2] - dr1[2] * dr2[1];
            av[1] = dr1[2] * dr2[0] - dr1[0] * dr2[2];
            av[2] = dr1[0] * dr2[1] - dr1[1] * dr2[0];
            for (int q = 0; q < 3; q++) av[q] = 0.5 * av[q];
            for (int q = 0; q < 3; q++) sub[q] = (r[i0][q] + r[i1][q] + r[i2][q]) / 3.0;
            for (int q = 0; q < 3; q++) a[q] = first ? av[q] : a[q] + av[q];
            for (int q = 0; q < 3; q++)
                for (int p = 0; p < 3; p++) sumc[q][p] = first ? sub[q] * av[p] : sumc[q][p] + sub[q] * av[p];
        };
        if (nl == 3) tri(0, 1, 2, true);
        else { tri(0, 1, 2, true); tri(0, 2, 3, false); }
        double dd = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
        for (int q = 0; q < 3; q++) ri[q] = (sumc[q][0] * a[0] + sumc[q][1] * a[1] + sumc[q][2] * a[2]) / dd;
    }
    });
    // calc_vol_cv_centers_uns (calc_vol_cv_centers.f90:4-61)
    // every cell below, every halo through its one boundary face
    S.xc.resize(S.nelem); S.yc.resize(S.nelem); S.zc.resize(S.nelem); S.vol.resize(ng);
    std::atomic<int> flat{0};
    cfdl::parallel_for(ng, [&](long b, long e_end) {
    for (int e = (int)b + 1; e <= (int)e_end; e++) {
        int t = S.etype[sec_of(S, e)], nv = element_nvx(t);
        double gc[3] = {0, 0, 0}, rc[3] = {0, 0, 0}, sum_vol = 0;
        for (int q = 1; q <= nv; q++) {
            int v = S.e2vx[(size_t)(e - 1) * m + q - 1];
            gc[0] = gc[0] + S.x[v - 1]; gc[1] = gc[1] + S.y[v - 1]; gc[2] = gc[2] + S.z[v - 1];
        }
        for (int q = 0; q < 3; q++) gc[q] = gc[q] / nv;
        for (int idx = S.ef2nb_idx[e - 1]; idx <= S.ef2nb_idx[e] - 1; idx++) {
            int gf = S.ef2nb2[idx - 1], sg = gf >= 0 ? 1 : -1, enb, lf;
            gf = std::abs(gf);
            const double *cs = &S.rip[3 * (size_t)(gf - 1)], *ai = &S.aip[3 * (size_t)(gf - 1)];
            get_idx(S.ef2nb1[idx - 1], enb, lf);
            if (lf == 0) { S.xc[enb - 1] = cs[0]; S.yc[enb - 1] = cs[1]; S.zc[enb - 1] = cs[2]; }
            double h[3] = {cs[0] - gc[0], cs[1] - gc[1], cs[2] - gc[2]};
            double sub_vol = ((sg * ai[0]) * h[0] + (sg * ai[1]) * h[1] + (sg * ai[2]) * h[2]) / 3.0;
            sum_vol = sum_vol + sub_vol;
            for (int q = 0; q < 3; q++) rc[q] = rc[q] + (0.25 * gc[q] + 0.75 * cs[q]) * sub_vol;
        }
        for (int q = 0; q < 3; q++) rc[q] = rc[q] / sum_vol;
        S.xc[e - 1] = rc[0]; S.yc[e - 1] = rc[1]; S.zc[e - 1] = rc[2];
        S.vol[e - 1] = sum_vol;
        if (!(sum_vol > 1e-20)) flat = 1;  // the reference only warns here
    }
    });
    return flat ? CFDL_ERR_MESH : CFDL_OK;
}

// Argument checks and the copies of the zone arrays.
int init_setup(cfdl_setup &S, int nvx, const double *x, const double *y, const double *z, int nsec,
               const char *names, const int *etype, const int *esec, int ne2vxmax, const int *e2vx) {
    S.nvx = nvx; S.nsec = nsec; S.m = ne2vxmax;
    int cvs1 = 0, cvs2 = 0, cvs3 = 0;  // cell_input.f90:55-72
    for (int s = 0; s < nsec; s++) {
        int t = etype[s], cnt = esec[2 * s + 1] - esec[2 * s] + 1;
        if (t < 0 || t > 20 || cnt <= 0) return CFDL_ERR_INVALID;
        if (t >= 10 && t <= 20) { cvs1 += cnt; cvs2 += element_nface(t) * cnt; } else cvs3 += cnt;
        S.names.emplace_back(std::string(names + 33 * s, strnlen(names + 33 * s, 32)));
    }
    S.ne = cvs1; S.nbf = cvs3; S.nf = (cvs2 + cvs3) / 2; S.nelem = cvs1 + cvs3;
    if ((long long)S.nelem >= (1LL << 26)) return CFDL_ERR_INVALID;
    S.x.assign(x, x + nvx); S.y.assign(y, y + nvx); S.z.assign(z, z + nvx);
    S.e2vx.assign(e2vx, e2vx + (size_t)ne2vxmax * S.nelem);
    for (size_t q = 0; q < S.e2vx.size(); q++)
        if (S.e2vx[q] < 0 || S.e2vx[q] > nvx) return CFDL_ERR_INVALID;
    S.esec.assign(esec, esec + 2 * nsec);
    S.etype.assign(etype, etype + nsec);
    return CFDL_OK;
}

}  // namespace cfdl_setup_detail

using namespace cfdl_setup_detail;

static int create_setup(int nvx, const double *x, const double *y, const double *z, int nsec, const char *names,
                        const int *etype, const int *esec, int ne2vxmax, const int *e2vx, cfdl_setup **out,
                        bool device) {
    if (!out || nvx <= 0 || nsec <= 0 || ne2vxmax <= 0 || !x || !y || !z || !names || !etype || !esec || !e2vx)
        return CFDL_ERR_INVALID;
    *out = nullptr;
    cfdl_setup *S = new (std::nothrow) cfdl_setup;
    if (!S) return CFDL_ERR_OOM;
    int st;
    try {
        st = init_setup(*S, nvx, x, y, z, nsec, names, etype, esec, ne2vxmax, e2vx);
        if (!st) st = order_sections(*S);
        if (!st) st = device ? match_faces_device(*S) : match_faces_host(*S);
        if (!st) st = finish_topology(*S);
        if (!st) st = device ? geometry_device(*S) : geometry_host(*S);
    } catch (const std::bad_alloc &) {
        st = CFDL_ERR_OOM;
    }
    if (st) { delete S; return st; }
    *out = S;
    return CFDL_OK;
}

extern "C" int cfdl_setup_create(int nvx, const double *x, const double *y, const double *z,
                                 int nsec, const char *names, const int *etype, const int *esec,
                                 int ne2vxmax, const int *e2vx, cfdl_setup **out) {
    return create_setup(nvx, x, y, z, nsec, names, etype, esec, ne2vxmax, e2vx, out, false);
}

extern "C" int cfdl_setup_create_device(int nvx, const double *x, const double *y, const double *z,
                                        int nsec, const char *names, const int *etype, const int *esec,
                                        int ne2vxmax, const int *e2vx, cfdl_setup **out) {
    return create_setup(nvx, x, y, z, nsec, names, etype, esec, ne2vxmax, e2vx, out, true);
}

extern "C" int cfdl_setup_sizes(const cfdl_setup *s, int *sz) {
    if (!s || !sz) return CFDL_ERR_INVALID;
    sz[0] = s->ne; sz[1] = s->nf; sz[2] = s->nbf; sz[3] = s->nsec; sz[4] = s->nred;
    return CFDL_OK;
}

extern "C" int cfdl_setup_mesh(const cfdl_setup *s, double u_lid, cfdl_mesh *mesh) {
    if (!s || !mesh) return CFDL_ERR_INVALID;
    // make_bc (mod_eqn_setup.f90:46-68) as bound in construct_uvwp
    // (mod_uvwp.f90:73-78): a section is bound when its name is a substring of
    // the BC name; names are looked up in file order by sorted section number.
    static const char *kBc[6] = {"top", "west", "east", "south", "north", "bottom"};
    s->bc_esec.assign(2 * (size_t)s->nintf, 0);
    s->bc_kind.assign(s->nintf, 0);
    s->bc_vel.assign(3 * (size_t)s->nintf, 0.0);
    s->bc_temp.assign(s->nintf, 0.0);
    for (int b = 0; b < 6; b++) {
        for (int i = 0; i < s->nintf; i++) {
            int sec = s->intf2sec[i];
            const std::string &nm = s->names[sec - 1];
            std::string t = nm;
            while (!t.empty() && t.back() == ' ') t.pop_back();
            if (!t.empty() && std::string(kBc[b]).find(t) != std::string::npos) {
                s->bc_esec[2 * i] = s->esec[2 * (sec - 1)];
                s->bc_esec[2 * i + 1] = s->esec[2 * (sec - 1) + 1];
                s->bc_kind[i] = CFDL_BC_WALL;
                s->bc_vel[3 * i] = b == 0 ? u_lid : 0.0;
                s->bc_vel[3 * i + 1] = 0.0;
                s->bc_vel[3 * i + 2] = 0.0;
                // construct_energy's binding (mod_energy.f90:40-45): lid 373, dirichlet0 273
                s->bc_temp[i] = b == 0 ? 373.0 : 273.0;
            }
        }
    }
    mesh->ne = s->ne; mesh->nf = s->nf; mesh->nbf = s->nbf;
    mesh->ef2nb1 = s->ef2nb1.data(); mesh->ef2nb2 = s->ef2nb2.data(); mesh->ef2nb_idx = s->ef2nb_idx.data();
    mesh->s2g = s->s2g.data(); mesh->bs = s->bs.data();
    mesh->aip = s->aip.data(); mesh->rip = s->rip.data();
    mesh->xc = s->xc.data(); mesh->yc = s->yc.data(); mesh->zc = s->zc.data(); mesh->vol = s->vol.data();
    mesh->nbc = s->nintf; mesh->bc_esec = s->bc_esec.data(); mesh->bc_kind = s->bc_kind.data();
    mesh->bc_vel = s->bc_vel.data();
    mesh->bc_temp = s->bc_temp.data();
    return CFDL_OK;
}

extern "C" int cfdl_setup_get_int(const cfdl_setup *s, const char *name, int *out) {
    if (!s || !name || !out) return CFDL_ERR_INVALID;
    const std::vector<int> *v = nullptr;
    std::string n(name);
    if (n == "ef2nb1") v = &s->ef2nb1;
    else if (n == "ef2nb2") v = &s->ef2nb2;
    else if (n == "ef2nb_idx") v = &s->ef2nb_idx;
    else if (n == "s2g") v = &s->s2g;
    else if (n == "bs") v = &s->bs;
    else if (n == "esec") v = &s->esec;
    else if (n == "etype") v = &s->etype;
    else if (n == "red") v = &s->red;
    if (!v) return CFDL_ERR_NAME;
    std::copy(v->begin(), v->end(), out);
    return CFDL_OK;
}

extern "C" int cfdl_setup_get_dbl(const cfdl_setup *s, const char *name, double *out) {
    if (!s || !name || !out) return CFDL_ERR_INVALID;
    const cfdl::FillVec<double> *v = nullptr;
    std::string n(name);
    if (n == "aip") v = &s->aip;
    else if (n == "rip") v = &s->rip;
    else if (n == "xc") v = &s->xc;
    else if (n == "yc") v = &s->yc;
    else if (n == "zc") v = &s->zc;
    else if (n == "vol") v = &s->vol;
    if (!v) return CFDL_ERR_NAME;
    std::copy(v->begin(), v->end(), out);
    return CFDL_OK;
}

extern "C" int cfdl_setup_destroy(cfdl_setup *s) {
    delete s;
    return CFDL_OK;
}
