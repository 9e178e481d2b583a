// A C++ host shaped like the reference's main program (src/main.f90:50-63),
// through the cfdl_host mirror of mod_physics / mod_uvwp
// (cfd-lite_gb300/host/cfdl_phys.hpp): it builds the cavity zone, constructs
// the physics, runs ntstep time steps of ncoef (update_boundaries,
// solve_uvwp) passes followed by update_time, and writes u, v, w, p and mip
// as raw little-endian doubles for the test to compare.  A stop_error ends it
// with exit status 10 + the C-ABI status.
//
// usage: phys_host <n> <kind> <jitter> <seed> <ntstep> <ncoef> <out.bin>
#include "cfdl_phys.hpp"
#include <cmath>
#include <cstdio>
#include <cstdlib>

int main(int argc, char **argv) {
    if (argc != 8) {
        std::fprintf(stderr, "usage: %s n kind jitter seed ntstep ncoef out.bin\n", argv[0]);
        return 2;
    }
    const int n = std::atoi(argv[1]), kind = std::atoi(argv[2]);
    const double jitter = std::atof(argv[3]);
    const uint64_t seed = std::strtoull(argv[4], nullptr, 10);
    try {
        cfdl_host::geometry_t geom = cfdl_host::geometry_t::box(n, kind, jitter, seed);
        cfdl_host::phys_t phys;
        phys.prop.rho = 1.0;           // Re 100 on the unit cavity with a unit lid
        phys.prop.mu = 0.01;
        phys.dt = INFINITY;            // steady SIMPLE, under-relaxed
        phys.alpha_u = 0.7;
        phys.alpha_p = 0.3;
        phys.ntstep = std::atoi(argv[5]);
        phys.ncoef = std::atoi(argv[6]);
        cfdl_host::construct_physics(phys, geom);
        cfdl_stats st{};
        for (int tstep = 1; tstep <= phys.ntstep; tstep++) {
            for (int icoef = 1; icoef <= phys.ncoef; icoef++) {
                cfdl_host::update_boundaries(phys, geom);
                st = cfdl_host::solve_uvwp(phys.uvwp, phys.prop, geom, phys.dt, phys.nit);
            }
            cfdl_host::update_time(phys);
        }
        std::FILE *fo = std::fopen(argv[7], "wb");
        if (!fo) return 4;
        const cfdl_host::uvwp_t &q = phys.uvwp;
        for (const std::vector<double> *a : {&q.u, &q.v, &q.w, &q.p, &q.mip})
            if (std::fwrite(a->data(), 8, a->size(), fo) != a->size()) return 4;
        std::fclose(fo);
        std::printf("%d time steps x %d passes on %d cells: it_p %d, mass imbalance %.3e\n", phys.ntstep, phys.ncoef,
                    geom.ne(), st.it_p, st.mass_imbalance);
    } catch (const cfdl_host::stop_error &e) {
        std::fprintf(stderr, "stop: %s\n", e.what());
        return 10 + e.status;
    }
    return 0;
}
