// cfdl_noalloc.cu -- pressure-correction solve that allocates nothing.
//
// Some hosts cannot call cudaMalloc: a Fortran code whose device memory is
// owned by another runtime or pool, a process that runs under a fixed memory
// budget, or a caller inside a loop where allocation is not allowed.  For
// them cfdl_solve_pc_noalloc solves the pressure-correction system with
// arrays the caller already holds on the device, in the reference's CSR
// layout, and keeps all of its own working storage (Krylov vectors, reduction
// partials, scalars) in one file-scope __device__ array of fixed size.
//
// Algorithm: the Jacobi-preconditioned CG of the context path (set_a_0 then
// CG from zero on the zero-mean right-hand side), one thread per cell over
// the CSR rows, deterministic tile reductions.
#include "cfdl_internal.h"
#include "cfdl_device.cuh"
#include <cstddef>

namespace cfdl {
namespace {

constexpr int kNaMaxCells = 131072;                 // CFDL_NOALLOC_MAX_CELLS
constexpr int kNaMaxTiles = kNaMaxCells / kTile;

struct NoAllocScratch {
    double r[kNaMaxCells], z[kNaMaxCells], p[kNaMaxCells], q[kNaMaxCells];
    double partials[kNaMaxTiles * kNPart];
    double mean, rz, alpha, beta, rnorm, r0, tol;
    int counter[4];
    int active, iters, bad;
    int fail;           // why CG stopped early: 0 it did not, 1 a non-finite value, 2 p.Ap <= 0
};

// Shared by every call on a device and kept between calls.
static __device__ __align__(256) NoAllocScratch g_na_scratch;

// Row i of the pressure operator from the caller's CSR arrays.  Indices are
// checked against ne and nh; a bad one is recorded and its access skipped.
__device__ __forceinline__ double csr_amul(NoAllocScratch *S, int ne, int nh, const int *ef1, const int *idx,
                                           const double *ap, const double *anb, const double *x, int i) {
    double s = ap[i] * x[i];
    int h0 = idx[i] - 1, h1 = idx[i + 1] - 1;
    if (h0 < 0 || h1 > nh || h0 > h1) { S->bad = 1; return s; }
    for (int h = h0; h < h1; h++) {
        const int enb = (int)((unsigned)ef1[h] >> 5), lf = ef1[h] & 31;
        if (!lf) continue;
        if (enb < 1 || enb > ne) { S->bad = 1; continue; }
        s -= anb[h] * x[enb - 1];
    }
    return s;
}

__device__ __forceinline__ bool na_last(NoAllocScratch *S, int which, int ntiles) {
    return last_tile_of_case(&S->counter[which], ntiles);
}

__global__ void __launch_bounds__(kTile) k_na_mean(NoAllocScratch *S, int ne, const double *b) {
    const int i = blockIdx.x * kTile + threadIdx.x;
    double v[1] = {i < ne ? b[i] : 0.0};
    block_reduce<1>(v, &S->partials[(size_t)blockIdx.x * kNPart]);
    if (na_last(S, 0, gridDim.x)) {
        __shared__ double s[1];
        sum_partials<1>(S->partials, 0, gridDim.x, s);
        if (threadIdx.x == 0) S->mean = s[0] / ne;
    }
}

__global__ void __launch_bounds__(kTile) k_na_init(NoAllocScratch *S, int ne, const double *ap, const double *b,
                                                  double *x, double rtol, int maxit) {
    const int i = blockIdx.x * kTile + threadIdx.x;
    double v[2] = {0, 0};
    if (i < ne) {
        const double r = b[i] - S->mean, z = r / ap[i];
        S->r[i] = r; S->z[i] = z; S->p[i] = z; x[i] = 0.0;
        v[0] = r * r; v[1] = r * z;
    }
    block_reduce<2>(v, &S->partials[(size_t)blockIdx.x * kNPart]);
    if (na_last(S, 1, gridDim.x)) {
        __shared__ double s[2];
        sum_partials<2>(S->partials, 0, gridDim.x, s);
        if (threadIdx.x == 0) {
            S->r0 = S->rnorm = sqrt(s[0]);
            S->rz = s[1];
            S->tol = rtol * S->r0;
            S->iters = 0;
            S->bad = 0;
            // a zero or non-finite diagonal entry makes z = r/ap, and so (r, z), non-finite
            S->fail = isfinite(S->r0) && isfinite(S->rz) ? 0 : 1;
            S->active = S->r0 > S->tol && maxit > 0 && !S->fail;
        }
    }
}

__global__ void __launch_bounds__(kTile) k_na_q(NoAllocScratch *S, int ne, int nh, const int *ef1, const int *idx,
                                               const double *ap, const double *anb) {
    if (!S->active) return;
    const int i = blockIdx.x * kTile + threadIdx.x;
    double v[1] = {0};
    if (i < ne) {
        const double q = csr_amul(S, ne, nh, ef1, idx, ap, anb, S->p, i);
        S->q[i] = q;
        v[0] = S->p[i] * q;
    }
    block_reduce<1>(v, &S->partials[(size_t)blockIdx.x * kNPart]);
    if (na_last(S, 2, gridDim.x)) {
        __shared__ double s[1];
        sum_partials<1>(S->partials, 0, gridDim.x, s);
        if (threadIdx.x == 0) {
            // only runs while ||r|| is above the tolerance, where an SPD system has p.Ap > 0
            if (S->bad) S->active = 0;
            else if (!isfinite(s[0])) { S->active = 0; S->fail = 1; }
            else if (!(s[0] > 0.0)) { S->active = 0; S->fail = 2; }
            else S->alpha = S->rz / s[0];
        }
    }
}

__global__ void __launch_bounds__(kTile) k_na_x(NoAllocScratch *S, int ne, const double *ap, double *x, int maxit) {
    if (!S->active) return;
    const int i = blockIdx.x * kTile + threadIdx.x;
    double v[2] = {0, 0};
    if (i < ne) {
        const double a = S->alpha;
        x[i] = x[i] + a * S->p[i];
        const double r = S->r[i] - a * S->q[i], z = r / ap[i];
        S->r[i] = r; S->z[i] = z;
        v[0] = r * r; v[1] = r * z;
    }
    block_reduce<2>(v, &S->partials[(size_t)blockIdx.x * kNPart]);
    if (na_last(S, 3, gridDim.x)) {
        __shared__ double s[2];
        sum_partials<2>(S->partials, 0, gridDim.x, s);
        if (threadIdx.x == 0) {
            S->rnorm = sqrt(s[0]);
            S->iters += 1;
            S->beta = S->rz != 0.0 ? s[1] / S->rz : 0.0;
            S->rz = s[1];
            if (!isfinite(S->rnorm) || !isfinite(S->rz)) S->fail = 1;
            S->active = S->rnorm > S->tol && S->iters < maxit && !S->fail;
        }
    }
}

__global__ void __launch_bounds__(kTile) k_na_p(NoAllocScratch *S, int ne) {
    if (!S->active) return;
    const int i = blockIdx.x * kTile + threadIdx.x;
    if (i < ne) S->p[i] = S->z[i] + S->beta * S->p[i];
}

// Device address of the scratch array on the current device.  The host-side
// symbol is only a stand-in, not a device address, so the address is asked
// of the runtime with the device current.  The first call on a device loads
// the library's device code there (make it before any stream capture); later
// calls only read the runtime's table.  Asking on every call, rather than
// keeping the first answer, keeps the address right after a cudaDeviceReset,
// which gives the device a new context and may place the array elsewhere.
int na_scratch(NoAllocScratch **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e);
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_na_scratch);
    if (e != cudaSuccess) return cuda_status(e);
    *out = static_cast<NoAllocScratch *>(ptr);
    return CFDL_OK;
}

}  // namespace
}  // namespace cfdl

using namespace cfdl;

extern "C" int cfdl_solve_pc_noalloc(int ne, int nh, const int *ef2nb1, const int *ef2nb_idx, const double *ap,
                                     const double *anb, const double *b, double *phic, double rtol, int maxit,
                                     int *iters, double *rnorm) {
    if (ne <= 0 || nh <= 0 || !ef2nb1 || !ef2nb_idx || !ap || !anb || !b || !phic || !(rtol > 0) || maxit < 0)
        return CFDL_ERR_INVALID;
    if (ne > kNaMaxCells) return CFDL_ERR_TOO_LARGE;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return CFDL_ERR_NO_DEVICE; }
    NoAllocScratch *S = nullptr;
    int st = na_scratch(&S);
    if (st) return st;
    const cudaStream_t s0 = 0;
    const int grid = (ne + kTile - 1) / kTile;
    // the last-tile counters must start at zero on every call
    cudaError_t e = cudaMemsetAsync(S->counter, 0, sizeof(S->counter), s0);
    if (e != cudaSuccess) return cuda_status(e);
    k_na_mean<<<grid, kTile, 0, s0>>>(S, ne, b);
    k_na_init<<<grid, kTile, 0, s0>>>(S, ne, ap, b, phic, rtol, maxit);
    int it = 0, active = 1, chunk = 4;
    while (it < maxit) {
        for (int k = 0; k < chunk && it < maxit; k++, it++) {
            k_na_q<<<grid, kTile, 0, s0>>>(S, ne, nh, ef2nb1, ef2nb_idx, ap, anb);
            k_na_x<<<grid, kTile, 0, s0>>>(S, ne, ap, phic, maxit);
            k_na_p<<<grid, kTile, 0, s0>>>(S, ne);
        }
        e = cudaMemcpyAsync(&active, &S->active, sizeof(int), cudaMemcpyDeviceToHost, s0);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s0);
        if (e != cudaSuccess) return cuda_status(e);
        if (!active) break;
        chunk = chunk < 64 ? chunk * 2 : 64;
    }
    // iters, bad and fail are adjacent ints; rnorm and tol are read alone
    int flags[3] = {0, 0, 0};
    double rn = 0.0, tol = 0.0;
    static_assert(offsetof(NoAllocScratch, bad) == offsetof(NoAllocScratch, iters) + sizeof(int) &&
                  offsetof(NoAllocScratch, fail) == offsetof(NoAllocScratch, bad) + sizeof(int),
                  "iters, bad, fail must be adjacent");
    e = cudaMemcpyAsync(flags, &S->iters, sizeof(flags), cudaMemcpyDeviceToHost, s0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&rn, &S->rnorm, sizeof(double), cudaMemcpyDeviceToHost, s0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tol, &S->tol, sizeof(double), cudaMemcpyDeviceToHost, s0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s0);
    if (e != cudaSuccess) return cuda_status(e);
    const int it_dev = flags[0], bad = flags[1], fail = flags[2];
    if (iters) *iters = it_dev;
    if (rnorm) *rnorm = rn;
    if (bad) return CFDL_ERR_INVALID;
    if (fail == 1 || !isfinite(rn)) return CFDL_ERR_NONFINITE;
    if (fail == 2) return CFDL_ERR_BREAKDOWN;
    if (rn > tol) return CFDL_ERR_ITER_CAP;       // stopped at maxit above the tolerance
    return CFDL_OK;
}
