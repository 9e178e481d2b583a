// cfdl_vtu.cpp -- headless VTU output of a case's fields, in the format of
// the reference's write_vtubin (src/modules/mod_vtu_output.f90:6-328).
//
// The fields are read from the device; the file is the reference's byte
// layout: an XML header naming each DataArray's offset into the appended
// block, then, after '_', each array as a UInt64 byte count and its raw
// little-endian values.  Cell data of the uvwp equation, in order: u, v, w, p
// (Float64), gpc (3 components), and under the name "mip" the net face mass
// flux of each cell (sum over its half-faces of mip(fg) times the sign of fg;
// the reference computes it into eqn%dc, mod_vtu_output.f90:113-123 -- here
// it goes to the file only and the device coefficients are left alone).  Cell
// data of the energy equation (mod_vtu_output.f90:124-132): enthalpy (phi),
// grad_enthalpy, temperature, grad_temperature.  Then the vertices, the volume
// elements' connectivity (0-based), offsets and VTK cell types.
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

struct Var { const char *name; int dim; const double *a; };

HostCase *find_case(cfdl_ctx *ctx, int case_id, const cfdl_setup *s) {
    for (HostCase *hc : ctx->cases)
        if (hc->id == case_id)
            return hc->ne == s->ne && hc->nf == s->nf && hc->nbf == s->nbf ? hc : nullptr;
    return nullptr;
}

bool sections_writable(const cfdl_setup *s) {
    for (int q = 0; q < s->nsec; q++)
        if (s->etype[q] >= 10 && vtk_type(s->etype[q]) < 0) return false;   // the reference stops here
    return true;
}

// device arrays -> host vectors, one copy each
int fetch(cfdl_ctx *ctx, std::vector<std::vector<double> *> dst, std::vector<const double *> src) {
    for (size_t k = 0; k < dst.size(); k++) {
        cudaError_t e = cudaMemcpyAsync(dst[k]->data(), src[k], dst[k]->size() * sizeof(double), cudaMemcpyDeviceToHost,
                                        ctx->stream);
        if (e != cudaSuccess) return cuda_status(e);
    }
    return cuda_status(cudaStreamSynchronize(ctx->stream));
}

int write_vtubin(const cfdl_setup *s, const Var *vars, int nvar, const char *path);

}  // namespace

extern "C" int cfdl_write_vtu(cfdl_ctx *ctx, int case_id, const cfdl_setup *s, const char *path) {
    if (!ctx || !s || !path) return CFDL_ERR_INVALID;
    HostCase *hc = find_case(ctx, case_id, s);
    if (!hc || !sections_writable(s)) return CFDL_ERR_INVALID;
    const int ne = s->ne, nc = ne + s->nbf;
    // the case's fields, from the device
    std::vector<double> u(nc), v(nc), w(nc), p(nc), gpc(3 * (size_t)nc), mip(s->nf);
    const CaseDev &d = hc->dev;
    int st = fetch(ctx, {&u, &v, &w, &p, &gpc, &mip}, {d.u, d.v, d.w, d.p, d.gpc, d.mip});
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
    const Var vars[6] = {
        {"u", 1, u.data()}, {"v", 1, v.data()}, {"w", 1, w.data()}, {"p", 1, p.data()}, {"gpc", 3, gpc.data()},
        {"mip", 1, net.data()}};
    return write_vtubin(s, vars, 6, path);
}

extern "C" int cfdl_write_vtu_energy(cfdl_ctx *ctx, int case_id, const cfdl_setup *s, const char *path) {
    if (!ctx || !s || !path) return CFDL_ERR_INVALID;
    HostCase *hc = find_case(ctx, case_id, s);
    if (!hc || !hc->dev.ee || !sections_writable(s)) return CFDL_ERR_INVALID;
    const size_t nc = (size_t)s->ne + s->nbf;
    std::vector<double> e(nc), ge(3 * nc), t(nc), gt(3 * nc);
    const CaseDev &d = hc->dev;
    int st = fetch(ctx, {&e, &ge, &t, &gt}, {d.ee, d.ege, d.et, d.egt});
    if (st) return st;
    const Var vars[4] = {{"enthalpy", 1, e.data()}, {"grad_enthalpy", 3, ge.data()}, {"temperature", 1, t.data()},
                         {"grad_temperature", 3, gt.data()}};
    return write_vtubin(s, vars, 4, path);
}

namespace {

int write_vtubin(const cfdl_setup *s, const Var *vars, int nvar, const char *path) {
    const int ne = s->ne;
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
    std::vector<unsigned long long> nbytes(nvar);
    for (int k = 0; k < nvar; k++) {
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
    for (int k = 0; k < nvar; k++) {
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

}  // namespace
