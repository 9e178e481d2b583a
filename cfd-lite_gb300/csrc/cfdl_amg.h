// cfdl_amg.h -- aggregation multigrid hierarchy (host build, device view).
#pragma once
#include "cfdl_internal.h"

namespace cfdl {

constexpr int kAmgCoarsest = 64;     // dense (pseudo-)inverse at or below this many cells
constexpr int kAmgMaxLevels = 12;

// Level-0 (mesh) graph handed to the builder: ELL neighbours (-1 or >= n for
// "no interior neighbour") and the strength of each slot.
struct AmgFineView {
    int n, W;
    const int *nb;
    const double *strength;
};

// One coarse level, host side.  Slots are ELL slot indices k*n + i of the
// finer level; "fine" means the level just above.
struct AmgHostLevel {
    int n_fine = 0, n = 0, W_fine = 0, W = 0;
    FillVec<int> agg;                  // [n_fine] coarse cell of each fine cell
    FillVec<int> mem_ptr, mem;         // members of each coarse cell
    FillVec<int> nb;                   // [W][n] coarse neighbours, -1 padded
    FillVec<int> g_ptr, g_src;         // fine slots summed into coarse slot s = k*n + c
};

struct AmgHierarchy {
    std::vector<AmgHostLevel> levels;
};

int build_amg_hierarchy(const AmgFineView &fine, AmgHierarchy &H);

// One coarse level, device side (all pointers device).
struct AmgLevelDev {
    int n, W, n_fine, W_fine;
    const int *nb, *agg, *mem_ptr, *mem, *g_ptr, *g_src;
    const int *len;                           // [n] couplings of each row (its slots k < len are the valid ones)
    double *a, *dg, *rd, *r, *z, *t;          // FP64 operator and V-cycle vectors
    float *a32, *dg32, *rd32, *r32, *z32, *t32; // FP32 copies (mixed-precision form)
};

}  // namespace cfdl
