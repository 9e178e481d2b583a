// cfdl_vtu.cpp -- headless VTU output of a case's fields, in the format of
// the reference's write_vtubin (src/modules/mod_vtu_output.f90:6-328).
//
// The fields are read from the device (u, v, w, p, gpc, mip); the file is the
// reference's byte layout: an XML header naming each DataArray's offset into
// the appended block, then, after '_', each array as a UInt64 byte count and
// its raw little-endian values.  Cell data, in order: u, v, w, p (Float64),
// gpc (3 components), and under the name "mip" the net face mass flux of each
// cell (sum over its half-faces of mip(fg) times the sign of fg; the reference
// computes it into eqn%dc, mod_vtu_output.f90:113-123 -- here it goes to the
// file only and the device coefficients are left alone).  Then the vertices,
// the volume elements' connectivity (0-based), offsets and VTK cell types.
#include "cfdl_internal.h"
#include "cfdl_setup_int.h"
#include <cstdio>
#include <cstring>
#include <string>

using namespace cfdl;

namespace {

// Fortran I12: right-justified in 12 columns
std::string i12(long long v) {
    char b[32];
    snprintf(b, sizeof b, "%12lld", v);
    return b;
}

int vtk_type(int cgns_type) {
    switch (cgns_type) {
    case 10: return 10;   // tetrahedron
    case 17: return 12;   // hexahedron
    case 12: return 14;   // pyramid
    case 14: return 13;   // prism / wedge
    default: return -1;
    }
}

struct Out {
    FILE *f;
    bool ok = true;
    void str(const std::string &s) { ok &= fwrite(s.data(), 1, s.size(), f) == s.size(); }
    template <class T> void raw(const T *p, size_t n) { ok &= fwrite(p, sizeof(T), n, f) == n; }
    void u64(unsigned long long v) { raw(&v, 1); }
};

}  // namespace

extern "C" int cfdl_write_vtu(cfdl_ctx *ctx, int case_id, const cfdl_setup *s, const char *path) {
    if (!ctx || !s || !path) return CFDL_ERR_INVALID;
    int c = -1;
    for (size_t k = 0; k < ctx->cases.size(); k++) if (ctx->cases[k]->id == case_id) c = (int)k;
    if (c < 0) return CFDL_ERR_INVALID;
    HostCase *hc = ctx->cases[c];
    if (hc->ne != s->ne || hc->nf != s->nf || hc->nbf != s->nbf) return CFDL_ERR_INVALID;
    const int ne = s->ne, nc = ne + s->nbf;
    for (int q = 0; q < s->nsec; q++)
        if (s->etype[q] >= 10 && vtk_type(s->etype[q]) < 0) return CFDL_ERR_INVALID;   // the reference stops here
    // the case's fields, from the device
    std::vector<double> u(nc), v(nc), w(nc), p(nc), gpc(3 * (size_t)nc), mip(s->nf);
    const CaseDev &d = hc->dev;
    struct Cp { double *h; const double *dv; size_t n; } cps[] = {
        {u.data(), d.u, (size_t)nc}, {v.data(), d.v, (size_t)nc}, {w.data(), d.w, (size_t)nc}, {p.data(), d.p, (size_t)nc},
        {gpc.data(), d.gpc, 3 * (size_t)nc}, {mip.data(), d.mip, (size_t)s->nf}};
    for (const Cp &q : cps) {
        cudaError_t e = cudaMemcpyAsync(q.h, q.dv, q.n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
        if (e != cudaSuccess) return cuda_status(e);
    }
    int st = cuda_status(cudaStreamSynchronize(ctx->stream));
    if (st) return st;
    // net face mass flux per cell, in half-face order (mod_vtu_output.f90:113-123)
    std::vector<double> net(ne, 0.0);
    for (int e = 0; e < ne; e++)
        for (int idx = s->ef2nb_idx[e]; idx <= s->ef2nb_idx[e + 1] - 1; idx++) {
            int fg = s->ef2nb2[idx - 1];
            const int sg = fg / std::abs(fg);
            fg = std::abs(fg);
            net[e] = net[e] + mip[fg - 1] * sg;
        }
    struct Var { const char *name; int dim; const double *a; } vars[6] = {
        {"u", 1, u.data()}, {"v", 1, v.data()}, {"w", 1, w.data()}, {"p", 1, p.data()}, {"gpc", 3, gpc.data()},
        {"mip", 1, net.data()}};
    // volume sections, as the reference walks them
    long long nconn = 0, ncell = 0;
    for (int q = 0; q < s->nsec; q++) {
        if (s->etype[q] < 10) continue;
        const long long cnt = s->esec[2 * q + 1] - s->esec[2 * q] + 1;
        nconn += cnt * cfdl_setup_detail::element_nvx(s->etype[q]);
        ncell += cnt;
    }
    FILE *f = fopen(path, "wb");
    if (!f) return CFDL_ERR_INVALID;
    Out o{f};
    const std::string lf = "\n";
    long long noffset = 0;
    o.str("<?xml version=\"1.0\"?>" + lf);
    o.str("<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">" + lf);
    o.str(" <UnstructuredGrid>" + lf);
    o.str("  <Piece NumberOfPoints=\"" + std::to_string(s->nvx) + "\" NumberOfCells=\"" + std::to_string(ne) + "\">" + lf);
    o.str("   <CellData Scalars=\"scalars\">" + lf);
    unsigned long long nbytes[6];
    for (int k = 0; k < 6; k++) {
        o.str("    <DataArray type=\"Float64\" Name=\"" + std::string(vars[k].name) + "\" NumberOfComponents=\"" +
              std::to_string(vars[k].dim) + "\" format=\"appended\" offset=\"" + i12(noffset) + "\" />" + lf);
        nbytes[k] = (unsigned long long)ne * vars[k].dim * 8;
        noffset += 8 + (long long)nbytes[k];
    }
    o.str("   </CellData>" + lf);
    o.str("   <Points>" + lf);
    o.str("    <DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"appended\" offset=\"" + i12(noffset) + "\" />" + lf);
    const unsigned long long nb_pts = 3ull * s->nvx * 8, nb_conn = (unsigned long long)nconn * 4,
                             nb_off = (unsigned long long)ncell * 4, nb_typ = (unsigned long long)ne * 4;
    noffset += 8 + (long long)nb_pts;
    o.str("   </Points>" + lf);
    o.str("   <Cells>" + lf);
    o.str("    <DataArray type=\"Int32\" Name=\"connectivity\" format=\"appended\" offset=\"" + i12(noffset) + "\" />" + lf);
    noffset += 8 + (long long)nb_conn;
    o.str("    <DataArray type=\"Int32\" Name=\"offsets\" format=\"appended\" offset=\"" + i12(noffset) + "\" />" + lf);
    noffset += 8 + (long long)nb_off;
    o.str("    <DataArray type=\"Int32\" Name=\"types\" format=\"appended\" offset=\"" + i12(noffset) + "\" />" + lf);
    o.str("   </Cells>" + lf);
    o.str("  </Piece>" + lf);
    o.str(" </UnstructuredGrid>" + lf);
    o.str(" <AppendedData encoding=\"raw\">" + lf);
    o.str("_");
    for (int k = 0; k < 6; k++) {
        o.u64(nbytes[k]);
        for (int q = 0; q < s->nsec; q++) {
            if (s->etype[q] < 10) continue;
            for (int m = s->esec[2 * q]; m <= s->esec[2 * q + 1]; m++)
                o.raw(vars[k].a + (size_t)(m - 1) * vars[k].dim, vars[k].dim);
        }
    }
    o.u64(nb_pts);
    for (int j = 0; j < s->nvx; j++) { const double xyz[3] = {s->x[j], s->y[j], s->z[j]}; o.raw(xyz, 3); }
    o.u64(nb_conn);
    std::vector<int> row;
    for (int q = 0; q < s->nsec; q++) {
        if (s->etype[q] < 10) continue;
        const int l = cfdl_setup_detail::element_nvx(s->etype[q]);
        for (int m = s->esec[2 * q]; m <= s->esec[2 * q + 1]; m++) {
            row.assign(s->e2vx.begin() + (size_t)(m - 1) * s->m, s->e2vx.begin() + (size_t)(m - 1) * s->m + l);
            for (int &x : row) x -= 1;   // 0-based vertex ids
            o.raw(row.data(), row.size());
        }
    }
    o.u64(nb_off);
    int l = 0;
    for (int q = 0; q < s->nsec; q++) {
        if (s->etype[q] < 10) continue;
        for (int m = s->esec[2 * q]; m <= s->esec[2 * q + 1]; m++) { l += cfdl_setup_detail::element_nvx(s->etype[q]); o.raw(&l, 1); }
    }
    o.u64(nb_typ);
    for (int q = 0; q < s->nsec; q++) {
        if (s->etype[q] < 10) continue;
        const int t = vtk_type(s->etype[q]);
        for (int m = s->esec[2 * q]; m <= s->esec[2 * q + 1]; m++) o.raw(&t, 1);
    }
    o.str(lf + " </AppendedData>" + lf);
    o.str("</VTKFile>" + lf);
    const bool ok = o.ok && fclose(f) == 0;
    return ok ? CFDL_OK : CFDL_ERR_INVALID;
}
