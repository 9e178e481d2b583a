// cfdl_amg_setup.cpp -- host set-up of the aggregation multigrid hierarchy
// used to precondition the pressure-correction CG.
//
// The reference builds an agglomeration hierarchy of the mesh at start-up
// (generate_seeds / add_transformation, src/setup/mod_agglomeration.f90,
// src/setup/mod_mg_lvl_uns.f90:552-1001) but its solver never uses more than
// the fine level.  Here the coarse levels are real: cells are grouped into
// aggregates by a greedy, deterministic pass over the cell graph (a cell whose
// neighbours are all free seeds an aggregate with them; leftover cells join
// their most strongly connected aggregate; the rest group with their free
// neighbours), with face strength area/(dr.n), the geometric factor of the
// pressure coefficient.  The aggregation depends only on the mesh, so it is
// built once; every pressure solve then forms the Galerkin coarse operators
// A_c = P^T A P (P piecewise constant) from gather lists prepared here, so the
// coarse coefficients are sums in a fixed order (deterministic).
#include "cfdl_amg.h"
#include "cfdl_par.h"
#include <algorithm>
#include <cstring>
#include <numeric>

namespace cfdl {
namespace {

// The large arrays below are sized without a fill (FillVec) and written in
// full by the parallel loops that follow, which first-touch their pages.
struct Graph {
    int n = 0, W = 0;
    FillVec<int> nb;            // [W][n] neighbour or -1
    FillVec<double> w;          // [W][n] strength
};

// greedy aggregation of one level
int aggregate(const Graph &g, FillVec<int> &agg) {
    const int n = g.n, W = g.W;
    agg.assign(n, -1);
    int nagg = 0;
    for (int i = 0; i < n; i++) {                       // phase 1: free seeds with free neighbourhoods
        if (agg[i] != -1) continue;
        bool free_nbhd = true;
        for (int k = 0; k < W; k++) {
            int j = g.nb[(size_t)k * n + i];
            if (j >= 0 && agg[j] != -1) { free_nbhd = false; break; }
        }
        if (!free_nbhd) continue;
        agg[i] = nagg;
        for (int k = 0; k < W; k++) {
            int j = g.nb[(size_t)k * n + i];
            if (j >= 0) agg[j] = nagg;
        }
        nagg++;
    }
    std::vector<int> join(n, -1);                       // phase 2: join the strongest aggregated neighbour
    for (int i = 0; i < n; i++) {
        if (agg[i] != -1) continue;
        double best = -1.0;
        for (int k = 0; k < W; k++) {
            int j = g.nb[(size_t)k * n + i];
            if (j >= 0 && agg[j] != -1 && g.w[(size_t)k * n + i] > best) { best = g.w[(size_t)k * n + i]; join[i] = agg[j]; }
        }
    }
    for (int i = 0; i < n; i++) if (agg[i] == -1 && join[i] != -1) agg[i] = join[i];
    for (int i = 0; i < n; i++) {                       // phase 3: what is left groups with free neighbours
        if (agg[i] != -1) continue;
        agg[i] = nagg;
        for (int k = 0; k < W; k++) {
            int j = g.nb[(size_t)k * n + i];
            if (j >= 0 && agg[j] == -1) agg[j] = nagg;
        }
        nagg++;
    }
    return nagg;
}

}  // namespace

int build_amg_hierarchy(const AmgFineView &fine, AmgHierarchy &H) {
    H.levels.clear();
    Graph g;
    g.n = fine.n; g.W = fine.W;
    g.nb.resize((size_t)g.W * g.n);
    g.w.resize((size_t)g.W * g.n);
    parallel_for((long)g.W * g.n, [&](long b, long e) {
        for (long s = b; s < e; s++) {
            const int j = fine.nb[s];
            const bool in = j >= 0 && j < g.n;
            g.nb[s] = in ? j : -1;
            g.w[s] = in ? fine.strength[s] : 0.0;
        }
    });
    while (g.n > kAmgCoarsest && (int)H.levels.size() < kAmgMaxLevels) {
        FillVec<int> agg_new;
        int nc = aggregate(g, agg_new);
        if (nc >= g.n) break;                           // no coarsening possible
        AmgHostLevel L;
        L.n_fine = g.n; L.n = nc; L.W_fine = g.W;
        L.agg = std::move(agg_new);
        const FillVec<int> &agg = L.agg;
        // members CSR (fine cells in increasing order per aggregate)
        L.mem_ptr.assign(nc + 1, 0);
        for (int i = 0; i < g.n; i++) L.mem_ptr[agg[i] + 1]++;
        for (int c = 0; c < nc; c++) L.mem_ptr[c + 1] += L.mem_ptr[c];
        L.mem.resize(g.n);                              // each fine cell filed once below
        {
            std::vector<int> fill(L.mem_ptr.begin(), L.mem_ptr.end() - 1);
            for (int i = 0; i < g.n; i++) L.mem[fill[agg[i]]++] = i;
        }
        // Coarse neighbours of each aggregate in first-met order (members in
        // increasing order, slots in increasing k), and the fine slots feeding
        // each coarse slot, built in two parallel passes over flat arrays:
        // pass 1 finds each aggregate's neighbours, slot counts and strength
        // sums (in a region sized by its members' slots), pass 2 files the
        // slots once the coarse slot offsets are known.
        std::vector<long> cap(nc + 1, 0);
        for (int c = 0; c < nc; c++) cap[c + 1] = cap[c] + (long)(L.mem_ptr[c + 1] - L.mem_ptr[c]) * g.W;
        FillVec<int> nbr(cap[nc]), cntq(cap[nc]), ncnb(nc);   // read only where pass 1 wrote
        FillVec<double> wq(cap[nc]);
        parallel_for(nc, [&](long cb, long ce) {
            for (int c = (int)cb; c < (int)ce; c++) {
                int *nb_c = &nbr[cap[c]], *cn_c = &cntq[cap[c]];
                double *w_c = &wq[cap[c]];
                int nq = 0;
                for (int m = L.mem_ptr[c]; m < L.mem_ptr[c + 1]; m++) {
                    const int i = L.mem[m];
                    for (int k = 0; k < g.W; k++) {
                        const int j = g.nb[(size_t)k * g.n + i];
                        if (j < 0) continue;
                        const int cj = agg[j];
                        if (cj == c) continue;           // internal coupling: not a coarse slot
                        int q = 0;
                        while (q < nq && nb_c[q] != cj) q++;
                        if (q == nq) { nb_c[q] = cj; cn_c[q] = 0; w_c[q] = 0.0; nq++; }
                        cn_c[q]++;
                        w_c[q] += g.w[(size_t)k * g.n + i];
                    }
                }
                ncnb[c] = nq;
            }
        }, 2048);
        int Wc = 1;
        for (int c = 0; c < nc; c++) Wc = std::max(Wc, ncnb[c]);
        L.W = Wc;
        L.nb.resize((size_t)Wc * nc);                   // every slot written below
        L.g_ptr.resize((size_t)Wc * nc + 1);
        L.g_ptr[0] = 0;
        // slot-major offsets: each slot plane k scanned on its own, then the
        // planes' totals carried over in order
        std::vector<long> plane_total(Wc + 1, 0);
        parallel_for(Wc, [&](long kb, long ke) {
            for (int k = (int)kb; k < (int)ke; k++) {
                long run = 0;
                for (int c = 0; c < nc; c++) {
                    const size_t sl = (size_t)k * nc + c;
                    const bool has = k < ncnb[c];
                    run += has ? cntq[cap[c] + k] : 0;
                    L.g_ptr[sl + 1] = (int)run;
                    L.nb[sl] = has ? nbr[cap[c] + k] : -1;
                }
                plane_total[k + 1] = run;
            }
        }, 1);
        for (int k = 0; k < Wc; k++) plane_total[k + 1] += plane_total[k];
        parallel_for(Wc, [&](long kb, long ke) {
            for (int k = (int)kb; k < (int)ke; k++)
                for (int c = 0; c < nc; c++) L.g_ptr[(size_t)k * nc + c + 1] += (int)plane_total[k];
        }, 1);
        L.g_src.resize(L.g_ptr.back());                 // each fine slot filed once below
        parallel_for(nc, [&](long cb, long ce) {
            std::vector<int> fill;
            for (int c = (int)cb; c < (int)ce; c++) {
                const int *nb_c = &nbr[cap[c]], nq = ncnb[c];
                fill.assign(nq, 0);
                for (int m = L.mem_ptr[c]; m < L.mem_ptr[c + 1]; m++) {
                    const int i = L.mem[m];
                    for (int k = 0; k < g.W; k++) {
                        const int j = g.nb[(size_t)k * g.n + i];
                        if (j < 0) continue;
                        const int cj = agg[j];
                        if (cj == c) continue;
                        int q = 0;
                        while (nb_c[q] != cj) q++;
                        L.g_src[L.g_ptr[(size_t)q * nc + c] + fill[q]++] = k * g.n + i;
                    }
                }
            }
        }, 2048);
        // next graph
        Graph ng;
        ng.n = nc; ng.W = Wc;
        ng.nb.resize((size_t)Wc * nc);
        ng.w.resize((size_t)Wc * nc);
        parallel_for(nc, [&](long cb, long ce) {
            for (int c = (int)cb; c < (int)ce; c++)
                for (int k = 0; k < Wc; k++) {
                    const size_t sl = (size_t)k * nc + c;
                    ng.nb[sl] = L.nb[sl];
                    ng.w[sl] = k < ncnb[c] ? wq[cap[c] + k] : 0.0;
                }
        });
        H.levels.push_back(std::move(L));
        g = std::move(ng);
    }
    return CFDL_OK;
}

}  // namespace cfdl
