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

struct Graph {
    int n = 0, W = 0;
    std::vector<int> nb;        // [W][n] neighbour or -1
    std::vector<double> w;      // [W][n] strength
};

// greedy aggregation of one level
int aggregate(const Graph &g, std::vector<int> &agg) {
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
    g.nb.assign((size_t)g.W * g.n, -1);
    g.w.assign((size_t)g.W * g.n, 0.0);
    for (int k = 0; k < g.W; k++)
        for (int i = 0; i < g.n; i++) {
            int j = fine.nb[(size_t)k * g.n + i];
            if (j >= 0 && j < g.n) { g.nb[(size_t)k * g.n + i] = j; g.w[(size_t)k * g.n + i] = fine.strength[(size_t)k * g.n + i]; }
        }
    while (g.n > kAmgCoarsest && (int)H.levels.size() < kAmgMaxLevels) {
        std::vector<int> agg;
        int nc = aggregate(g, agg);
        if (nc >= g.n) break;                           // no coarsening possible
        AmgHostLevel L;
        L.n_fine = g.n; L.n = nc; L.W_fine = g.W;
        L.agg = agg;
        // members CSR (fine cells in increasing order per aggregate)
        L.mem_ptr.assign(nc + 1, 0);
        for (int i = 0; i < g.n; i++) L.mem_ptr[agg[i] + 1]++;
        for (int c = 0; c < nc; c++) L.mem_ptr[c + 1] += L.mem_ptr[c];
        L.mem.assign(g.n, 0);
        {
            std::vector<int> fill(L.mem_ptr.begin(), L.mem_ptr.end() - 1);
            for (int i = 0; i < g.n; i++) L.mem[fill[agg[i]]++] = i;
        }
        // coarse neighbours in first-met order, and the fine slots feeding each
        std::vector<std::vector<int>> cnb(nc);
        std::vector<std::vector<std::vector<int>>> src(nc);
        std::vector<std::vector<double>> cw(nc);
        parallel_for(nc, [&](long cb, long ce) {
        for (int c = (int)cb; c < (int)ce; c++) {
            for (int m = L.mem_ptr[c]; m < L.mem_ptr[c + 1]; m++) {
                int i = L.mem[m];
                for (int k = 0; k < g.W; k++) {
                    int j = g.nb[(size_t)k * g.n + i];
                    if (j < 0) continue;
                    int slot = k * g.n + i;
                    int cj = agg[j];
                    if (cj == c) continue;           // internal coupling: not a coarse slot
                    size_t q = 0;
                    while (q < cnb[c].size() && cnb[c][q] != cj) q++;
                    if (q == cnb[c].size()) { cnb[c].push_back(cj); src[c].emplace_back(); cw[c].push_back(0.0); }
                    src[c][q].push_back(slot);
                    cw[c][q] += g.w[(size_t)slot];
                }
            }
        }
        }, 2048);
        int Wc = 1;
        for (int c = 0; c < nc; c++) Wc = std::max<int>(Wc, (int)cnb[c].size());
        L.W = Wc;
        L.nb.assign((size_t)Wc * nc, -1);
        L.g_ptr.assign((size_t)Wc * nc + 1, 0);
        for (int k = 0; k < Wc; k++)
            for (int c = 0; c < nc; c++) {
                size_t s = (size_t)k * nc + c;
                int cnt = k < (int)cnb[c].size() ? (int)src[c][k].size() : 0;
                L.g_ptr[s + 1] = L.g_ptr[s] + cnt;
                if (k < (int)cnb[c].size()) L.nb[s] = cnb[c][k];
            }
        L.g_src.assign(L.g_ptr.back(), 0);
        for (int k = 0; k < Wc; k++)
            for (int c = 0; c < nc; c++)
                if (k < (int)cnb[c].size()) {
                    size_t s = (size_t)k * nc + c;
                    std::copy(src[c][k].begin(), src[c][k].end(), L.g_src.begin() + L.g_ptr[s]);
                }
        // next graph
        Graph ng;
        ng.n = nc; ng.W = Wc;
        ng.nb = L.nb;
        ng.w.assign((size_t)Wc * nc, 0.0);
        for (int k = 0; k < Wc; k++)
            for (int c = 0; c < nc; c++)
                if (k < (int)cnb[c].size()) ng.w[(size_t)k * nc + c] = cw[c][k];
        H.levels.push_back(std::move(L));
        g = std::move(ng);
    }
    return CFDL_OK;
}

}  // namespace cfdl
