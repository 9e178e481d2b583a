/*
 * cfd_oracle_mesh.c -- CPU oracle (test infrastructure only): restatement of
 * the reference's mesh set-up, which produces every integer and geometry
 * array the SIMPLE hot path consumes.
 *
 *   cell_input                 src/setup/cell_input.f90:10-165
 *   add_meshds (fine branch)   src/setup/mod_mg_lvl_uns.f90:120-233
 *   find_element_nb            src/setup/mod_mg_lvl_uns.f90:283-488
 *   calc_redblack              src/setup/mod_meshds_uns.f90:134-204
 *   calc_aip_xyzip_uns         src/setup/calc_aip_xyzip.f90:7-74
 *   calc_vol_cv_centers_uns    src/setup/calc_vol_cv_centers.f90:4-61
 *   seed_gen_t / grow          src/setup/mod_agglomeration.f90:331-561
 *   add_transformation_bt      src/setup/mod_mg_lvl_uns.f90:873-903 (level-1 g2gf)
 *   qsort_key_nRec             src/modules/mod_util.f90:1683-1730
 *   qsort_key                  src/modules/mod_util.f90:1602-1625
 *   construct_subdomains       src/modules/mod_subdomains.f90:18-160
 *
 * Element quality (esm, mod_mg_lvl_uns.f90:435-454) and the coarse
 * multigrid levels (find_group_nb and the level-2 transformation) are not
 * restated: the hot path never reads them.
 */
#include "cfd_oracle_int.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

void *o_alloc(size_t n, size_t sz) {
    void *p = calloc(n ? n : 1, sz);
    if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    return p;
}

/* ---- element tables, src/modules/mod_util.f90:54-169 (CGNS conventions) ---- */
static const int faces_tetra4[4][4] = {{1,3,2,0},{1,2,4,0},{2,3,4,0},{3,1,4,0}};
static const int nfaces_tetra4[4] = {3,3,3,3};
static const int faces_pyra5[5][4] = {{1,4,3,2},{1,2,5,0},{2,3,5,0},{3,4,5,0},{4,1,5,0}};
static const int nfaces_pyra5[5] = {4,3,3,3,3};
static const int faces_penta6[5][4] = {{1,2,5,4},{2,3,6,5},{3,1,4,6},{1,3,2,0},{4,5,6,0}};
static const int nfaces_penta6[5] = {4,4,4,3,3};
static const int faces_hexa8[6][4] = {{1,4,3,2},{1,2,6,5},{2,3,7,6},{3,4,8,7},{1,5,8,4},{5,6,7,8}};
static const int nfaces_hexa8[6] = {4,4,4,4,4,4};
/*                               1 2 3 4 5 6 7 8 9 10 11 12 13 14 15 16 17 18 19 20 */
static const int element_nface[21] = {0,6,0,0,0,1,1,1,1,1, 4, 4, 5, 5, 5, 5, 5, 6, 6, 6,0};
static const int element_nvx[21]   = {0,8,1,2,3,3,6,4,8,9, 4,10, 5,14, 6,15,18, 8,20,27,0};

/* face_vxlist, src/modules/mod_util.f90:1361-1423 */
static void face_vxlist(const int *vx, int t, int f, int *lst, int *nl) {
    int l;
    if (t == O_TETRA_4) {
        *nl = nfaces_tetra4[f-1];
        for (l = 0; l < *nl; l++) lst[l] = vx[faces_tetra4[f-1][l]-1];
    } else if (t == O_PYRA_5) {
        *nl = nfaces_pyra5[f-1];
        for (l = 0; l < *nl; l++) lst[l] = vx[faces_pyra5[f-1][l]-1];
    } else if (t == O_PENTA_6) {
        *nl = nfaces_penta6[f-1];
        for (l = 0; l < *nl; l++) lst[l] = vx[faces_penta6[f-1][l]-1];
    } else if (t == O_HEXA_8) {
        *nl = nfaces_hexa8[f-1];
        for (l = 0; l < *nl; l++) lst[l] = vx[faces_hexa8[f-1][l]-1];
    } else if (t == O_TRI_3) {
        *nl = 3;
        for (l = 0; l < 3; l++) lst[l] = vx[l];
    } else if (t == O_QUAD_4) {
        *nl = 4;
        for (l = 0; l < 4; l++) lst[l] = vx[l];
    } else {
        fprintf(stderr, "oracle: unsupported element type in face_vxlist %d\n", t);
        abort();
    }
}

/* face_compare, src/modules/mod_util.f90:1450-1479 */
static int face_compare(int e1, int f1, int t1, const int *vx1, int e2, int f2, int t2, const int *vx2) {
    int lst1[4], lst2[4], nl1, nl2, i, j, cnt;
    if (e1 == e2) return 0;
    face_vxlist(vx1, t1, f1, lst1, &nl1);
    face_vxlist(vx2, t2, f2, lst2, &nl2);
    if (nl1 != nl2) return 0;
    cnt = 0;
    for (i = 0; i < nl1; i++)
        for (j = 0; j < nl2; j++)
            if (lst1[i] == lst2[j]) { cnt++; break; }
    return cnt == nl1;
}

/* vec_a_bcrossc, src/modules/mod_util.f90:692-704 */
static void cross3(double *a, const double *b, const double *c) {
    a[0] = b[1]*c[2] - b[2]*c[1];
    a[1] = b[2]*c[0] - b[0]*c[2];
    a[2] = b[0]*c[1] - b[1]*c[0];
}

/* ---------------------------------------------------------------------------
 * find_element_nb, src/setup/mod_mg_lvl_uns.f90:283-488
 * ------------------------------------------------------------------------- */
static int find_element_nb(ocase *c) {
    const int ng = c->ne, nvx = c->nvx, nsec = c->nsec;
    int s, e, j, v, t, fmax = 0, emax, tmp, tmp2, idx1, idx2, n, l, m, f, nl1, nf = 0;
    int *vx2e_idx = o_alloc((size_t)nvx + 2, sizeof(int));
    int *gs2nb_idx = c->ef2nb_idx;
    size_t vx2e_size = 0;

    gs2nb_idx[1] = 1;
    for (s = 1; s <= nsec; s++) {
        for (e = c->bs_idx[s]; e <= c->bs_idx[s+1] - 1; e++) {
            t = c->etype[s];
            if (e < ng + 1) gs2nb_idx[e+1] = gs2nb_idx[e] + element_nface[t];
            if (element_nface[t] > fmax) fmax = element_nface[t];
            for (j = 1; j <= element_nvx[t]; j++) {
                v = E2VX(c, j, e);
                vx2e_idx[v] += 1;
                vx2e_size++;
            }
        }
    }
    tmp = vx2e_idx[1];
    vx2e_idx[1] = 1;
    emax = tmp;
    for (v = 2; v <= nvx + 1; v++) {
        tmp2 = vx2e_idx[v];
        if (tmp2 > emax) emax = tmp2;
        vx2e_idx[v] = vx2e_idx[v-1] + tmp;
        tmp = tmp2;
    }
    int *vx2e = o_alloc(vx2e_size + 2, sizeof(int));
    int *indices = o_alloc((size_t)emax * fmax + 1, sizeof(int));
    int *f2s = o_alloc((size_t)emax * fmax + 1, sizeof(int));

    for (s = 1; s <= nsec; s++) {
        int n1 = c->bs_idx[s], n2 = c->bs_idx[s+1] - 1;
        for (e = n1; e <= n2; e++) {
            for (j = 1; j <= element_nvx[c->etype[s]]; j++) {
                v = E2VX(c, j, e);
                idx1 = vx2e_idx[v];
                while (vx2e[idx1] != 0 && idx1 < vx2e_idx[v+1]) idx1++;
                vx2e[idx1] = e;
            }
        }
    }

    for (v = 1; v <= nvx; v++) {
        int lst1[4];
        n = 0;
        for (idx1 = vx2e_idx[v]; idx1 <= vx2e_idx[v+1] - 1; idx1++) {
            e = vx2e[idx1];
            for (s = 1; s <= nsec; s++) if (e < c->bs_idx[s+1]) break;
            t = c->etype[s];
            for (f = 1; f <= element_nface[t]; f++) {
                face_vxlist(&E2VX(c, 1, e), t, f, lst1, &nl1);
                for (l = 0; l < nl1; l++) {
                    if (lst1[l] == v) {
                        n++;
                        indices[n] = o_index_t(e, f);
                        f2s[n] = s;
                    }
                }
            }
        }
        for (l = 1; l <= n; l++) {
            for (m = l + 1; m <= n; m++) {
                int t1 = c->etype[f2s[l]], t2 = c->etype[f2s[m]], e1, f1, e2, f2;
                o_get_idx(indices[l], &e1, &f1);
                o_get_idx(indices[m], &e2, &f2);
                if (!face_compare(e1, f1, t1, &E2VX(c, 1, e1), e2, f2, t2, &E2VX(c, 1, e2))) continue;
                if (e1 > ng && e2 <= ng) {
                    idx2 = gs2nb_idx[e2] + f2 - 1;
                    if (c->ef2nb1[idx2] != 0) continue;
                    nf++;
                    c->ef2nb1[idx2] = o_index_t(e1, 0);
                    c->ef2nb2[idx2] = nf;
                    c->s2g[nf] = indices[m];
                    BS(c, e1) = o_index_t(e2, f2);
                } else if (e2 > ng && e1 <= ng) {
                    idx1 = gs2nb_idx[e1] + f1 - 1;
                    if (c->ef2nb1[idx1] != 0) continue;
                    nf++;
                    c->ef2nb1[idx1] = o_index_t(e2, 0);
                    c->ef2nb2[idx1] = nf;
                    c->s2g[nf] = indices[l];
                    BS(c, e2) = o_index_t(e1, f1);
                } else if (e1 <= ng && e2 <= ng) {
                    idx1 = gs2nb_idx[e1] + f1 - 1;
                    idx2 = gs2nb_idx[e2] + f2 - 1;
                    if (c->ef2nb1[idx1] != 0 && c->ef2nb1[idx2] != 0) continue;
                    nf++;
                    c->ef2nb1[idx1] = indices[m];
                    c->ef2nb1[idx2] = indices[l];
                    c->ef2nb2[idx1] = nf;
                    c->s2g[nf] = indices[l];
                    if (e1 > e2) {
                        c->ef2nb2[idx1] = -nf;
                        c->s2g[nf] = indices[m];
                    }
                    c->ef2nb2[idx2] = -c->ef2nb2[idx1];
                }
                /* else: two 2D elements matched; the reference only warns */
            }
        }
    }
    /* edge boundary faces, mod_mg_lvl_uns.f90:421-433 */
    for (int e1 = ng + 1; e1 <= c->nelem; e1++) {
        int ee, ff, idx, e2, f2;
        if (BS(c, e1) < 0) continue;
        o_get_idx(BS(c, e1), &ee, &ff);
        for (idx = gs2nb_idx[ee]; idx <= gs2nb_idx[ee+1] - 1; idx++) {
            if (idx - gs2nb_idx[ee] + 1 == ff) continue;
            o_get_idx(c->ef2nb1[idx], &e2, &f2);
            if (f2 == 0) {
                BS(c, e1) = -abs(BS(c, e1));
                BS(c, e2) = -BS(c, e2);
            }
        }
    }
    free(vx2e_idx); free(vx2e); free(indices); free(f2s);
    if (nf != c->nf) {
        fprintf(stderr, "oracle: error in creation of element neighbour list %d %d\n", nf, c->nf);
        return -1;
    }
    return 0;
}

/* calc_redblack, src/setup/mod_meshds_uns.f90:134-204 (fine level) */
static void calc_redblack(ocase *c) {
    const int ng = c->ne;
    int g, gnb, idx, fl, b, lexit = 0, lfound;
    int *rb = o_alloc((size_t)ng + 1, sizeof(int));
    c->nred = 0;
    g = 1;
    while (g <= ng) {
        while (rb[g] != 0) {
            if (g == ng) { lexit = 1; break; }
            g++;
        }
        if (lexit) break;
        lfound = 1;
        for (idx = c->ef2nb_idx[g]; idx <= c->ef2nb_idx[g+1] - 1; idx++) {
            o_get_idx(c->ef2nb1[idx], &gnb, &fl);
            if (fl != 0 && rb[gnb] == 2) { lfound = 0; break; }
        }
        if (lfound) {
            for (idx = c->ef2nb_idx[g]; idx <= c->ef2nb_idx[g+1] - 1; idx++) {
                o_get_idx(c->ef2nb1[idx], &gnb, &fl);
                if (fl != 0 && rb[gnb] == 0) { c->nred++; rb[gnb] = 1; }
            }
            rb[g] = 2;
        } else {
            c->nred++;
            rb[g] = 1;
        }
        g++;
    }
    b = c->nred;
    c->nred = 0;
    for (g = 1; g <= ng; g++) {
        if (rb[g] == 1) { c->nred++; c->red[c->nred] = g; }
        else if (rb[g] == 2) { b++; c->red[b] = g; }
    }
    free(rb);
}

/* calc_aip_xyzip_uns, src/setup/calc_aip_xyzip.f90:7-74 */
static void calc_aip_xyzip(ocase *c) {
    int fg, e, fl, s, t, nl, i, j, lst[4];
    for (fg = 1; fg <= c->nf; fg++) {
        double r1[3], r2[3], r3[3], r4[3], dr1[3], dr2[3], sub[3], av[3], sumc[3][3], a[3];
        o_get_idx(c->s2g[fg], &e, &fl);
        for (s = 1; s <= c->nsec; s++)
            if (e >= c->esec[2*(s-1)] && e <= c->esec[2*(s-1)+1]) break;
        t = c->etype[s];
        face_vxlist(&E2VX(c, 1, e), t, fl, lst, &nl);
        double *aip = &c->aip[3*fg-2], *rip = &c->rip[3*fg-2];
#define LOADV(r, k) do { r[0] = c->x[lst[k]]; r[1] = c->y[lst[k]]; r[2] = c->z[lst[k]]; } while (0)
        if (nl == 3) {
            LOADV(r1, 0); LOADV(r2, 1); LOADV(r3, 2);
            for (i = 0; i < 3; i++) sub[i] = (r1[i] + r2[i] + r3[i]) / 3.0;
            for (i = 0; i < 3; i++) { dr1[i] = r2[i] - r1[i]; dr2[i] = r3[i] - r1[i]; }
            cross3(av, dr1, dr2);
            for (i = 0; i < 3; i++) av[i] = 0.5 * av[i];
            for (i = 0; i < 3; i++) aip[i] = av[i];
            for (i = 0; i < 3; i++) for (j = 0; j < 3; j++) sumc[i][j] = sub[i] * av[j];
        } else if (nl == 4) {
            LOADV(r1, 0); LOADV(r2, 1); LOADV(r3, 2); LOADV(r4, 3);
            for (i = 0; i < 3; i++) { dr1[i] = r2[i] - r1[i]; dr2[i] = r3[i] - r1[i]; }
            cross3(av, dr1, dr2);
            for (i = 0; i < 3; i++) av[i] = 0.5 * av[i];
            for (i = 0; i < 3; i++) aip[i] = av[i];
            for (i = 0; i < 3; i++) sub[i] = (r1[i] + r2[i] + r3[i]) / 3.0;
            for (i = 0; i < 3; i++) for (j = 0; j < 3; j++) sumc[i][j] = sub[i] * av[j];
            for (i = 0; i < 3; i++) { dr1[i] = r3[i] - r1[i]; dr2[i] = r4[i] - r1[i]; }
            cross3(av, dr1, dr2);
            for (i = 0; i < 3; i++) av[i] = 0.5 * av[i];
            for (i = 0; i < 3; i++) aip[i] = aip[i] + av[i];
            for (i = 0; i < 3; i++) sub[i] = (r1[i] + r3[i] + r4[i]) / 3.0;
            for (i = 0; i < 3; i++) for (j = 0; j < 3; j++) sumc[i][j] = sumc[i][j] + sub[i] * av[j];
        } else {
            fprintf(stderr, "oracle: unsupported face in calc_xyzip_uns\n");
            abort();
        }
#undef LOADV
        for (i = 0; i < 3; i++) a[i] = aip[i];
        double dd = a[0]*a[0] + a[1]*a[1] + a[2]*a[2];
        for (i = 0; i < 3; i++) rip[i] = (sumc[i][0]*a[0] + sumc[i][1]*a[1] + sumc[i][2]*a[2]) / dd;
    }
}

/* calc_vol_cv_centers_uns, src/setup/calc_vol_cv_centers.f90:4-61 */
static void calc_vol_cv_centers(ocase *c) {
    int s, e, idx, t, nv, gf, gf_sgn, enb, lf, k;
    for (s = 1; s <= c->nsec; s++) {
        for (e = c->esec[2*(s-1)]; e <= c->esec[2*(s-1)+1]; e++) {
            if (e > c->nelem - c->nbf) continue;
            double gc[3] = {0, 0, 0}, cs[3], h[3], sub_c[3], rc[3] = {0, 0, 0}, sum_vol = 0, sub_vol;
            t = c->etype[s];
            nv = element_nvx[t];
            for (idx = 1; idx <= nv; idx++) {
                int vv = E2VX(c, idx, e);
                gc[0] = gc[0] + c->x[vv]; gc[1] = gc[1] + c->y[vv]; gc[2] = gc[2] + c->z[vv];
            }
            for (k = 0; k < 3; k++) gc[k] = gc[k] / nv;
            for (idx = c->ef2nb_idx[e]; idx <= c->ef2nb_idx[e+1] - 1; idx++) {
                gf = c->ef2nb2[idx];
                gf_sgn = o_sgn(gf);
                gf = abs(gf);
                for (k = 0; k < 3; k++) cs[k] = c->rip[3*gf-2+k];
                o_get_idx(c->ef2nb1[idx], &enb, &lf);
                if (lf == 0) {
                    c->xc[enb] = c->rip[3*gf-2]; c->yc[enb] = c->rip[3*gf-1]; c->zc[enb] = c->rip[3*gf];
                }
                for (k = 0; k < 3; k++) h[k] = cs[k] - gc[k];
                sub_vol = ((gf_sgn*c->aip[3*gf-2])*h[0] + (gf_sgn*c->aip[3*gf-1])*h[1] + (gf_sgn*c->aip[3*gf])*h[2]) / 3.0;
                for (k = 0; k < 3; k++) sub_c[k] = 0.25*gc[k] + 0.75*cs[k];
                sum_vol = sum_vol + sub_vol;
                for (k = 0; k < 3; k++) rc[k] = rc[k] + sub_c[k]*sub_vol;
            }
            for (k = 0; k < 3; k++) rc[k] = rc[k] / sum_vol;
            c->xc[e] = rc[0]; c->yc[e] = rc[1]; c->zc[e] = rc[2];
            c->vol[e] = sum_vol;
            if (c->vol[e] <= 1e-20)
                fprintf(stderr, "oracle: negative or zero volume at element %d: %g\n", e, c->vol[e]);
        }
    }
}

/* cell_input (sizes) + add_meshds (fine branch) + geometry */
int o_build_mesh(ocase *c) {
    /* order section ranges, mod_mg_lvl_uns.f90:154-168 */
    int nsec = c->nsec, n, s;
    int *esec0 = o_alloc(2 * (size_t)nsec, sizeof(int)), *etype0 = o_alloc((size_t)nsec + 1, sizeof(int));
    memcpy(esec0, c->esec, 2 * (size_t)nsec * sizeof(int));
    memcpy(etype0, c->etype, ((size_t)nsec + 1) * sizeof(int));
    c->bs_idx[1] = 1;
    for (n = 1; n <= nsec; n++) {
        for (s = 1; s <= nsec; s++) {
            if (c->bs_idx[n] == esec0[2*(s-1)]) {
                c->bs_idx[n+1] = esec0[2*(s-1)+1] + 1;
                c->etype[n] = etype0[s];
                c->esec[2*(n-1)] = esec0[2*(s-1)];
                c->esec[2*(n-1)+1] = esec0[2*(s-1)+1];
                break;
            }
        }
    }
    free(esec0); free(etype0);
    /* boundary interfaces = 2D sections, mod_mg_lvl_uns.f90:169-182 */
    n = 0;
    for (s = 1; s <= nsec; s++) if (c->etype[s] < 10) { n++; c->sec2intf[s] = n; }
    c->nintf_c2b = n;
    c->intf2sec = o_alloc((size_t)n + 1, sizeof(int));
    for (s = 1; s <= nsec; s++) if (c->sec2intf[s] > 0) c->intf2sec[c->sec2intf[s]] = s;

    if (find_element_nb(c)) return -1;
    calc_redblack(c);
    calc_aip_xyzip(c);
    calc_vol_cv_centers(c);
    return 0;
}

/* ---------------------------------------------------------------------------
 * Oct-tree seed generation, src/setup/mod_agglomeration.f90.  The threaded
 * binary tree is modelled by its in-order node sequence, which is all its
 * iterators observe; cell lists keep push order (the doubly-linked list pops
 * from the head, mod_util.f90:2149-2206).
 * ------------------------------------------------------------------------- */
typedef struct {
    int parent_group_id, group_id;
    double rmin[3], rmax[3], group_vol;
    int *list, len;
    int leaf;
} obb;

typedef struct {
    obb *nodes; int nnodes, cap;
    int *order; int norder;   /* in-order sequence of node ids */
    const double *vol, *xc, *yc, *zc;
    double vol_ave;
    int target_ncv, nleaf;
} oseed;

static int seq_pos(const oseed *sg, int id) {
    for (int i = 0; i < sg->norder; i++) if (sg->order[i] == id) return i;
    return -1;
}
/* goto_next_leaf: next leaf after sequence position pos, -1 if none */
static int next_leaf_pos(const oseed *sg, int pos) {
    for (int i = pos + 1; i < sg->norder; i++) if (sg->nodes[sg->order[i]].leaf) return i;
    return -1;
}
static int first_leaf_pos(const oseed *sg) {
    if (sg->norder == 0) return -1;
    if (sg->nodes[sg->order[0]].leaf) return 0;
    return next_leaf_pos(sg, 0);
}
static int new_node(oseed *sg) {
    if (sg->nnodes == sg->cap) {
        sg->cap = sg->cap ? 2 * sg->cap : 16;
        sg->nodes = realloc(sg->nodes, (size_t)sg->cap * sizeof(obb));
        sg->order = realloc(sg->order, (size_t)sg->cap * sizeof(int));
    }
    memset(&sg->nodes[sg->nnodes], 0, sizeof(obb));
    sg->nodes[sg->nnodes].group_id = -1;
    sg->nodes[sg->nnodes].leaf = 1;
    return sg->nnodes++;
}
static void seq_insert(oseed *sg, int pos, int id) {
    memmove(&sg->order[pos + 1], &sg->order[pos], (size_t)(sg->norder - pos) * sizeof(int));
    sg->order[pos] = id;
    sg->norder++;
}

/* split_leaf, mod_agglomeration.f90:380-498 */
static int split_leaf(oseed *sg, int pos, double threshold_density, int *nchild) {
    int id = sg->order[pos];
    obb *bb = &sg->nodes[id];
    int i, isplit = 0, k;
    double d = 0.;
    *nchild = 0;
    if (!bb->leaf) return 0;
    if (bb->group_vol / sg->vol_ave < threshold_density) return 0;
    if (bb->len == 1) return 0;
    for (i = 0; i < 3; i++) {
        if (fabs(bb->rmin[i] - bb->rmax[i]) > d) { d = fabs(bb->rmin[i] - bb->rmax[i]); isplit = i + 1; }
    }
    if (isplit == 0) return 0;
    d = (bb->rmin[isplit-1] + bb->rmax[isplit-1]) / 2.;
    const double *pos_arr = isplit == 1 ? sg->xc : (isplit == 2 ? sg->yc : sg->zc);
    int *ll = o_alloc((size_t)bb->len, sizeof(int)), *rl = o_alloc((size_t)bb->len, sizeof(int)), nl = 0, nr = 0;
    double lrmin[3] = {1e20, 1e20, 1e20}, lrmax[3] = {-1e20, -1e20, -1e20};
    double rrmin[3] = {1e20, 1e20, 1e20}, rrmax[3] = {-1e20, -1e20, -1e20};
    double vol_l = 0., vol_r = 0.;
    for (k = 0; k < bb->len; k++) {
        int e = bb->list[k];
        double r[3] = {sg->xc[e], sg->yc[e], sg->zc[e]};
        if (pos_arr[e] < d) {
            ll[nl++] = e;
            vol_l = vol_l + sg->vol[e] * 1.0;
            for (i = 0; i < 3; i++) { lrmin[i] = fmin(lrmin[i], r[i]); lrmax[i] = fmax(lrmax[i], r[i]); }
        } else {
            rl[nr++] = e;
            vol_r = vol_r + sg->vol[e] * 1.0;
            for (i = 0; i < 3; i++) { rrmin[i] = fmin(rrmin[i], r[i]); rrmax[i] = fmax(rrmax[i], r[i]); }
        }
    }
    int parent = bb->group_id == -1 ? bb->parent_group_id : bb->group_id;
    free(bb->list); bb->list = NULL; bb->len = 0;
    int p = seq_pos(sg, id);
    if (nl > 0) {
        int lid = new_node(sg);
        obb *L = &sg->nodes[lid];
        L->list = ll; L->len = nl; L->group_vol = vol_l; L->parent_group_id = parent;
        memcpy(L->rmin, lrmin, sizeof lrmin); memcpy(L->rmax, lrmax, sizeof lrmax);
        seq_insert(sg, p, lid); p++;
    } else free(ll);
    if (nr > 0) {
        int rid = new_node(sg);
        obb *R = &sg->nodes[rid];
        R->list = rl; R->len = nr; R->group_vol = vol_r; R->parent_group_id = parent;
        memcpy(R->rmin, rrmin, sizeof rrmin); memcpy(R->rmax, rrmax, sizeof rrmax);
        seq_insert(sg, p + 1, rid);
    } else free(rl);
    sg->nodes[id].leaf = 0;
    *nchild = (nl > 0) + (nr > 0);
    return 1;
}

/* grow, mod_agglomeration.f90:500-561 */
static void seed_grow(oseed *sg, int new_target, int *gf2g, int lvl) {
    int nleaf0 = sg->nleaf, nchild, pos;
    double threshold_density = 2.;
    sg->vol_ave = sg->vol_ave * (double)sg->target_ncv / (double)new_target;
    sg->target_ncv = new_target;
    if (lvl > 1) {
        while (sg->nleaf < new_target) {
            pos = first_leaf_pos(sg);
            if (pos >= 0) {
                for (;;) {
                    int node = sg->order[pos];
                    if (split_leaf(sg, pos, threshold_density, &nchild)) {
                        /* the iterator stays on the split node; step to the next leaf */
                        pos = next_leaf_pos(sg, seq_pos(sg, node));
                        sg->nleaf = sg->nleaf + nchild - 1;
                        if (sg->nleaf == new_target) break;
                        if (pos < 0) break;
                    }
                    pos = next_leaf_pos(sg, pos);
                    if (pos < 0) break;
                }
            }
            if (sg->nleaf == nleaf0) threshold_density = threshold_density * 0.75;
            nleaf0 = sg->nleaf;
        }
        int nleaf = 0;
        pos = first_leaf_pos(sg);
        while (pos >= 0) {
            obb *leaf = &sg->nodes[sg->order[pos]];
            nleaf++;
            if (leaf->group_id != -1) leaf->parent_group_id = leaf->group_id;
            leaf->group_id = nleaf;
            gf2g[nleaf] = leaf->parent_group_id;
            pos = next_leaf_pos(sg, pos);
        }
    } else if (lvl == 1) {
        pos = first_leaf_pos(sg);
        while (pos >= 0) {
            obb *leaf = &sg->nodes[sg->order[pos]];
            for (int k = 0; k < leaf->len; k++) gf2g[leaf->list[k]] = leaf->group_id;
            pos = next_leaf_pos(sg, pos);
        }
    }
}

/* qsort_key_nRec, src/modules/mod_util.f90:1683-1730 (0-based views) */
static void qsort_key_nrec(int *key, int *b, int n) {
    enum { max_levels = 1000 };
    int beg[max_levels], end[max_levels];
    int i = 0, L, R, piv, b0, t;
    beg[0] = 0; end[0] = n;
    while (i >= 0) {
        L = beg[i]; R = end[i] - 1;
        if (L < R) {
            piv = key[L]; b0 = b[L];
            while (L < R) {
                while (key[R] >= piv && L < R) R--;
                if (L < R) { key[L] = key[R]; b[L] = b[R]; L++; }
                while (key[L] <= piv && L < R) L++;
                if (L < R) { key[R] = key[L]; b[R] = b[L]; R--; }
            }
            key[L] = piv; b[L] = b0;
            beg[i+1] = L + 1; end[i+1] = end[i]; end[i] = L;
            i++;
            if (end[i] - beg[i] > end[i-1] - beg[i-1]) {
                t = beg[i]; beg[i] = beg[i-1]; beg[i-1] = t;
                t = end[i]; end[i] = end[i-1]; end[i-1] = t;
            }
        } else {
            i--;
        }
    }
}

/* qsort_key, src/modules/mod_util.f90:1602-1625 (1-based, keys unique here) */
static void qsort_key(int *key, int *b, int i, int f) {
    int n, p, t;
    if (i >= f) return;
    n = i; p = f;
    while (n < p) {
        if (key[n] > key[p]) {
            t = key[n]; key[n] = key[p]; key[p] = t;
            t = b[n]; b[n] = b[p]; b[p] = t;
            p--;
            if (p > n) {
                t = key[n]; key[n] = key[p]; key[p] = t;
                t = b[n]; b[n] = b[p]; b[p] = t;
            }
        } else n++;
    }
    qsort_key(key, b, i, p - 1);
    qsort_key(key, b, p + 1, f);
}

/* construct_subdomains, src/modules/mod_subdomains.f90:18-160 */
static void construct_subdomains(ocase *c) {
    const int nsd = c->nsubd;
    int cc, cnb, n, g, gf, idx, gfnb, lfnb, lf, nl, idx2, cs, ncs;
    c->sd = o_alloc((size_t)nsd + 1, sizeof(osubd));
    c->intf = o_alloc((size_t)nsd * nsd, sizeof(ointf));
    ointf *tmpi = o_alloc((size_t)nsd * nsd, sizeof(ointf));
#define INTF(a, b) c->intf[((b)-1)*nsd + (a)-1]
#define TMPI(a, b) tmpi[((b)-1)*nsd + (a)-1]
    int *ef2nb_tmp = o_alloc((size_t)c->H + 1, sizeof(int));
    for (cc = 1; cc <= nsd; cc++) {
        osubd *S = &c->sd[cc];
        S->ne = c->g2gf_idx[cc+1] - c->g2gf_idx[cc];
        int nf = 0, nbf = 0;
        for (n = c->g2gf_idx[cc]; n <= c->g2gf_idx[cc+1] - 1; n++) {
            gf = c->g2gf[n];
            for (idx = c->ef2nb_idx[gf]; idx <= c->ef2nb_idx[gf+1] - 1; idx++) {
                o_get_idx(c->ef2nb1[idx], &gfnb, &lfnb);
                cnb = 0;
                if (lfnb != 0) cnb = c->gf2g[gfnb];
                if (cnb == 0) { INTF(cc, cc).ncs++; nbf++; }
                else if (cc != cnb) { INTF(cc, cnb).ncs++; nbf++; }
                nf++;
            }
        }
        nf = (nf + nbf) / 2;
        S->nbf = nbf; S->nf = nf;
        S->ap = o_alloc((size_t)S->ne + 1, sizeof(double));
        S->b = o_alloc((size_t)S->ne + 1, sizeof(double));
        S->anb = o_alloc((size_t)(2*nf - nbf) + 1, sizeof(double));
        S->phic = o_alloc((size_t)(S->ne + nbf) + 1, sizeof(double));
        S->ef2nb = o_alloc((size_t)(2*nf - nbf) + 1, sizeof(int));
        S->ef2nb_idx = o_alloc((size_t)S->ne + 2, sizeof(int));
        for (cnb = 1; cnb <= nsd; cnb++) {
            ncs = INTF(cc, cnb).ncs;
            INTF(cc, cnb).c1 = cc; INTF(cc, cnb).c2 = cnb;
            INTF(cc, cnb).index1 = o_alloc((size_t)ncs + 1, sizeof(int));
            if (cc != cnb) TMPI(cc, cnb).index1 = o_alloc((size_t)ncs + 1, sizeof(int));
        }
    }
    for (cc = 1; cc <= nsd; cc++)
        for (cnb = 1; cnb <= nsd; cnb++) {
            if (cc != cnb) INTF(cc, cnb).index2 = INTF(cnb, cc).index1;
            INTF(cc, cnb).ncs = 0;
        }
    for (cc = 1; cc <= nsd; cc++) {
        osubd *S = &c->sd[cc];
        int nbf = 0, ne = S->ne;
        S->ef2nb_idx[1] = 1;
        for (n = c->g2gf_idx[cc]; n <= c->g2gf_idx[cc+1] - 1; n++) {
            g = n - c->g2gf_idx[cc] + 1;
            gf = c->g2gf[n];
            nl = c->ef2nb_idx[gf+1] - c->ef2nb_idx[gf];
            S->ef2nb_idx[g+1] = S->ef2nb_idx[g] + nl;
            for (idx = c->ef2nb_idx[gf]; idx <= c->ef2nb_idx[gf+1] - 1; idx++) {
                lf = idx - c->ef2nb_idx[gf] + 1;
                o_get_idx(c->ef2nb1[idx], &gfnb, &lfnb);
                cnb = 0;
                if (lfnb != 0) cnb = c->gf2g[gfnb];
                if (cc == cnb) {
                    idx2 = c->ef2nb_idx[gfnb] + lfnb - 1;
                    ef2nb_tmp[idx2] = o_index_t(g, lf);
                } else {
                    nbf++;
                    ef2nb_tmp[idx] = o_index_t(ne + nbf, 0);
                }
            }
        }
    }
    for (cc = 1; cc <= nsd; cc++) {
        osubd *S = &c->sd[cc];
        for (n = c->g2gf_idx[cc]; n <= c->g2gf_idx[cc+1] - 1; n++) {
            g = n - c->g2gf_idx[cc] + 1;
            gf = c->g2gf[n];
            for (idx = c->ef2nb_idx[gf]; idx <= c->ef2nb_idx[gf+1] - 1; idx++) {
                lf = idx - c->ef2nb_idx[gf] + 1;
                o_get_idx(c->ef2nb1[idx], &gfnb, &lfnb);
                cnb = 0;
                if (lfnb != 0) cnb = c->gf2g[gfnb];
                idx2 = S->ef2nb_idx[g] + lf - 1;
                S->ef2nb[idx2] = ef2nb_tmp[idx];
                if (cnb == 0) {
                    INTF(cc, cc).ncs++;
                    INTF(cc, cc).index1[INTF(cc, cc).ncs] = o_index_t(g, lf);
                } else if (cc != cnb) {
                    INTF(cc, cnb).ncs++;
                    cs = INTF(cc, cnb).ncs;
                    INTF(cc, cnb).index1[cs] = o_index_t(g, lf);
                    if (cc < cnb) TMPI(cc, cnb).index1[cs] = o_index_t(gfnb, lfnb);
                    else TMPI(cc, cnb).index1[cs] = o_index_t(gf, lf);
                }
            }
        }
    }
    for (cc = 1; cc <= nsd; cc++)
        for (cnb = 1; cnb <= nsd; cnb++) {
            if (cc == cnb) continue;
            ncs = INTF(cc, cnb).ncs;
            qsort_key(TMPI(cc, cnb).index1, INTF(cc, cnb).index1, 1, ncs);
            free(TMPI(cc, cnb).index1);
        }
#undef INTF
#undef TMPI
    free(tmpi); free(ef2nb_tmp);
}

/* generate_seeds + add_transformation_bt (level 1) + construct_subdomains,
 * cell_input.f90:123-151, mod_mg_lvl_uns.f90:95-118,873-903 */
int o_build_partition(ocase *c, int nsubd) {
    const int ne = c->ne;
    int e, k;
    c->nsubd = nsubd;
    oseed sg; memset(&sg, 0, sizeof sg);
    sg.vol = c->vol; sg.xc = c->xc; sg.yc = c->yc; sg.zc = c->zc;
    /* construct_seed_gen, mod_agglomeration.f90:331-378 */
    int root = new_node(&sg);
    seq_insert(&sg, 0, root);
    obb *rb = &sg.nodes[root];
    rb->list = o_alloc((size_t)ne, sizeof(int)); rb->len = ne;
    rb->rmin[0] = rb->rmax[0] = c->xc[1];
    rb->rmin[1] = rb->rmax[1] = c->yc[1];
    rb->rmin[2] = rb->rmax[2] = c->zc[1];
    for (e = 1; e <= ne; e++) {
        rb->rmin[0] = fmin(rb->rmin[0], c->xc[e]); rb->rmax[0] = fmax(rb->rmax[0], c->xc[e]);
        rb->rmin[1] = fmin(rb->rmin[1], c->yc[e]); rb->rmax[1] = fmax(rb->rmax[1], c->yc[e]);
        rb->rmin[2] = fmin(rb->rmin[2], c->zc[e]); rb->rmax[2] = fmax(rb->rmax[2], c->zc[e]);
    }
    sg.vol_ave = 0.;
    for (e = 1; e <= ne; e++) { rb->list[e-1] = e; sg.vol_ave = sg.vol_ave + c->vol[e] * 1.0; }
    rb->group_vol = 2.1 * sg.vol_ave;
    rb->group_id = 1;
    rb->parent_group_id = 0;
    sg.target_ncv = 1; sg.nleaf = 1;
    /* generate_seeds with nl=(nsubd,1): p=2 then p=1 */
    int *gf2g2 = o_alloc((size_t)nsubd + 1, sizeof(int));
    seed_grow(&sg, nsubd, gf2g2, 2);
    c->gf2g = o_alloc((size_t)ne + 1, sizeof(int));
    seed_grow(&sg, ne, c->gf2g, 1);
    free(gf2g2);
    for (k = 0; k < sg.nnodes; k++) free(sg.nodes[k].list);
    free(sg.nodes); free(sg.order);
    /* add_transformation_bt, mod_mg_lvl_uns.f90:883-902 */
    c->g2gf = o_alloc((size_t)ne + 1, sizeof(int));
    int *key = o_alloc((size_t)ne + 1, sizeof(int));
    for (e = 1; e <= ne; e++) { c->g2gf[e] = e; key[e] = c->gf2g[e]; }
    qsort_key_nrec(&key[1], &c->g2gf[1], ne);
    int ngr = key[ne];
    if (ngr != nsubd) { fprintf(stderr, "oracle: partition produced %d groups\n", ngr); free(key); return -1; }
    c->g2gf_idx = o_alloc((size_t)ngr + 2, sizeof(int));
    int g = 0;
    for (int idx = 1; idx <= ne; idx++) {
        if (g != key[idx]) { g = key[idx]; c->g2gf_idx[g] = idx; }
    }
    c->g2gf_idx[ngr + 1] = ne + 1;
    free(key);
    construct_subdomains(c);
    return 0;
}
