// cfdl_phys.hpp -- CFD-Lite's physics interface for a C++ host, over the C-ABI.
//
// The reference's host drives a case through mod_physics and mod_uvwp
// (src/modules/mod_physics.f90, src/equations/mod_uvwp.f90): phys_t holds the
// time-stepping parameters, the properties and the equations' fields;
// construct_physics allocates them; the time loop of src/main.f90:50-63 calls
// update_boundaries and solve_uvwp ncoef times per time step, then
// update_time.  This header gives a C++ host the same names and argument
// meaning.  The fields live in host arrays in the reference's layouts
// (phys.uvwp.u, ...); each call moves them through libcfdgpu's C-ABI
// (include/cfdl.h) and the work runs on the GPU.  A failing call stops the
// program, as the reference's print + stop does: it throws
// cfdl_host::stop_error, which ends the program when nothing catches it.
//
// Header-only; link with -lcfdgpu.
#pragma once
#include "cfdl.h"
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace cfdl_host {

struct stop_error : std::runtime_error {
    int status;
    stop_error(const std::string &where, int st)
        : std::runtime_error(where + ": " + cfdl_status_string(st)), status(st) {}
};

inline void check(int st, const char *where) {
    if (st != CFDL_OK) throw stop_error(where, st);
}

// geometry_t (src/setup/cell_input.f90, src/setup/mod_mg_lvl_uns.f90): the
// connectivity and geometry of one zone in the reference's arrays.
class geometry_t {
  public:
    // From the CGNS-shaped zone arrays cell_input reads (cell_input.f90:55-72):
    // vertex coordinates, sections (names, element types, element ranges) and
    // the element-vertex table; u_lid is the lid velocity bound to 'top'.
    geometry_t(int nvx, const double *x, const double *y, const double *z, int nsec, const char *names,
               const int *etype, const int *esec, int ne2vxmax, const int *e2vx, double u_lid = 1.0) {
        check(cfdl_setup_create(nvx, x, y, z, nsec, names, etype, esec, ne2vxmax, e2vx, &s_), "cell_input");
        const int st = cfdl_setup_mesh(s_, u_lid, &mesh_);
        if (st != CFDL_OK) {
            cfdl_setup_destroy(s_);
            throw stop_error("make_bc", st);
        }
    }
    // The synthetic lid-driven cavity zone: the unit cube on n^3 cubes of
    // kind 0 hex, 1 tet (6 per cube), 2 prism, 3 pyramid, 4 mixed, interior
    // vertices jittered by U(-jitter, jitter) of the spacing (seeded).
    static geometry_t box(int n, int kind, double jitter, uint64_t seed, double u_lid = 1.0) {
        int nvx = 0, nelem = 0, nsec = 0, m = 0;
        check(cfdl_box_zone_sizes(n, kind, &nvx, &nelem, &nsec, &m), "box zone");
        std::vector<double> x(nvx), y(nvx), z(nvx);
        std::vector<int> e2vx((size_t)m * nelem), etype(nsec), esec(2 * (size_t)nsec);
        std::vector<char> names(33 * (size_t)nsec + 1, 0);
        check(cfdl_box_zone_fill(n, kind, jitter, seed, x.data(), y.data(), z.data(), e2vx.data(), etype.data(),
                                 esec.data(), names.data()),
              "box zone");
        return geometry_t(nvx, x.data(), y.data(), z.data(), nsec, names.data(), etype.data(), esec.data(), m,
                          e2vx.data(), u_lid);
    }
    geometry_t(geometry_t &&o) noexcept : s_(o.s_), mesh_(o.mesh_) { o.s_ = nullptr; }
    geometry_t(const geometry_t &) = delete;
    geometry_t &operator=(const geometry_t &) = delete;
    ~geometry_t() {
        if (s_) cfdl_setup_destroy(s_);
    }
    int ne() const { return mesh_.ne; }     // cells
    int nf() const { return mesh_.nf; }     // faces
    int nbf() const { return mesh_.nbf; }   // boundary faces (= halo cells)
    const cfdl_mesh &mesh() const { return mesh_; }
    const cfdl_setup *setup() const { return s_; }

  private:
    cfdl_setup *s_ = nullptr;
    cfdl_mesh mesh_{};
};

// properties_t (src/modules/mod_properties.f90:76-89): homogeneous density
// and viscosity, 5 and 0.01 in the reference.
struct properties_t {
    double rho = 5.0, mu = 0.01;
};

// uvwp_t (src/equations/mod_uvwp.f90:20-55): the fields of the momentum and
// pressure-correction equations in the reference's layouts, and the device
// context that solves them.
struct uvwp_t {
    std::vector<double> u, v, w, p, u0, v0, w0;    // [ne+nbf], halos after the cells
    std::vector<double> gu, gv, gw, gp, gpc;        // [3(ne+nbf)], xyz-interleaved
    std::vector<double> mip, mip0;                  // [nf] face mass fluxes
    cfdl_ctx *ctx = nullptr;
    cfdl_config cfg{};

    cfdl_fields fields() {
        return {u.data(), v.data(), w.data(), p.data(), u0.data(), v0.data(), w0.data(),
                gu.data(), gv.data(), gw.data(), gp.data(), gpc.data(), mip.data(), mip0.data()};
    }
};

// phys_t (src/modules/mod_physics.f90:13-35): time stepping, properties and
// the uvwp equation.  The relaxation factors, the inner-solve mode and the
// precision form are the C-ABI's additions (cfdl_config); their defaults are
// the reference's behaviour.
struct phys_t {
    double dt = 0.01;
    int ntstep = 10, ncoef = 3, nit = 100;
    double alpha_u = 1.0, alpha_p = 1.0;
    int solve_mode = 0, precision = 0;
    properties_t prop;
    uvwp_t uvwp;

    phys_t() = default;
    phys_t(const phys_t &) = delete;
    phys_t &operator=(const phys_t &) = delete;
    ~phys_t() {
        if (uvwp.ctx) cfdl_ctx_destroy(uvwp.ctx);
    }
};

// The context's configuration follows the arguments of each call, as the
// reference's routines take dt, nit and the properties per call.
inline void configure(uvwp_t &eqn, const properties_t &prop, double dt, int nit) {
    if (eqn.cfg.rho == prop.rho && eqn.cfg.mu == prop.mu && eqn.cfg.dt == dt && eqn.cfg.nit == nit) return;
    cfdl_config c = eqn.cfg;
    c.rho = prop.rho;
    c.mu = prop.mu;
    c.dt = dt;
    c.nit = nit;
    check(cfdl_set_config(eqn.ctx, &c), "solve_uvwp");
    eqn.cfg = c;
}

// construct_physics (mod_physics.f90:52-75) with construct_uvwp
// (mod_uvwp.f90:30-84): zero fields, bound boundary conditions, the initial
// face fluxes mip = calc_mip(.false.) and mip0 = mip.
inline void construct_physics(phys_t &phys, const geometry_t &geom) {
    cfdl_config c;
    cfdl_config_default(&c);
    c.rho = phys.prop.rho;
    c.mu = phys.prop.mu;
    c.dt = phys.dt;
    c.nit = phys.nit;
    c.alpha_u = phys.alpha_u;
    c.alpha_p = phys.alpha_p;
    c.solve_mode = phys.solve_mode;
    c.precision = phys.precision;
    uvwp_t &q = phys.uvwp;
    if (q.ctx) {
        cfdl_ctx_destroy(q.ctx);
        q.ctx = nullptr;
    }
    check(cfdl_ctx_create(&geom.mesh(), &c, &q.ctx), "construct_physics");
    q.cfg = c;
    const size_t nc = (size_t)geom.ne() + geom.nbf(), nf = (size_t)geom.nf();
    for (std::vector<double> *a : {&q.u, &q.v, &q.w, &q.p, &q.u0, &q.v0, &q.w0}) a->assign(nc, 0.0);
    for (std::vector<double> *a : {&q.gu, &q.gv, &q.gw, &q.gp, &q.gpc}) a->assign(3 * nc, 0.0);
    q.mip.assign(nf, 0.0);
    q.mip0.assign(nf, 0.0);
    cfdl_fields f = q.fields();
    check(cfdl_download_fields(q.ctx, &f), "construct_physics");
}

// update_boundaries(phys, geom) (mod_physics.f90:38-50): the halo values of
// u, v, w, p and the boundary face fluxes from the boundary conditions.
inline void update_boundaries(phys_t &phys, const geometry_t &) {
    cfdl_fields f = phys.uvwp.fields();
    check(cfdl_upload_fields(phys.uvwp.ctx, &f), "update_boundaries");
    check(cfdl_update_boundaries(phys.uvwp.ctx), "update_boundaries");
    check(cfdl_download_fields(phys.uvwp.ctx, &f), "update_boundaries");
}

// solve_uvwp(eqn, prop, geom, dt, nit) (mod_uvwp.f90:95-134): one SIMPLE
// outer iteration on the host arrays of eqn.  The reference's scratch arrays
// (ap, anb, b, phic) and subdomain partition have no counterpart: the GPU
// keeps its own.  Returns the inner iteration counts and residuals.  An inner
// solve that stops at nit is the reference's stopping rule, not an error.
inline cfdl_stats solve_uvwp(uvwp_t &eqn, const properties_t &prop, const geometry_t &, double dt, int nit) {
    configure(eqn, prop, dt, nit);
    cfdl_fields f = eqn.fields();
    cfdl_stats st{};
    const int s = cfdl_solve_uvwp_host(eqn.ctx, &f, &st);
    if (s != CFDL_ERR_ITER_CAP) check(s, "solve_uvwp");
    return st;
}

// update_time(phys) (mod_physics.f90:101-112): the old time level takes the
// new one.
inline void update_time(phys_t &phys) {
    uvwp_t &q = phys.uvwp;
    q.u0 = q.u;
    q.v0 = q.v;
    q.w0 = q.w;
    q.mip0 = q.mip;
}

}  // namespace cfdl_host
