// cfdl_device.cuh -- device helpers shared by the kernels of libcfdgpu.
#pragma once
#include "cfdl_internal.h"

namespace cfdl {

// First statement of every kernel the launch macros start with programmatic
// dependent launch: the grid may be scheduled while its predecessor in the
// stream is finishing, and waits here until that predecessor has completed
// and its writes are visible (a no-op when launched the ordinary way).
#define CFDL_PDL_WAIT() asm volatile("griddepcontrol.wait;" ::: "memory")

// Deterministic block reduction of K doubles (kTile threads): a fixed
// shuffle tree per warp, then warp partials summed in warp order by one
// thread.  The result lands in out[0..K-1].
template <int K, class T = double>
__device__ __forceinline__ void block_reduce(T (&v)[K], T *out) {
    __shared__ T sm[K][kTile / 32];
#pragma unroll
    for (int k = 0; k < K; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; k++) sm[k][wid] = v[k];
    __syncthreads();
    if (threadIdx.x < K) {
        T s = 0;
        for (int w = 0; w < kTile / 32; w++) s += sm[threadIdx.x][w];
        out[threadIdx.x] = s;
    }
    __syncthreads();
}

// Sum the K partials of tiles [first, first+n) in tile order (whole block),
// result broadcast in shared memory res[0..K-1].
template <int K, class T = double>
__device__ __forceinline__ void sum_partials(const T *partials, int first, int n, T *res) {
    T v[K];
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = 0;
    // thread-strided in a fixed order with four independent accumulators (so
    // the loads overlap instead of forming one dependent chain), then the
    // fixed tree
    T a1[K], a2[K], a3[K];
#pragma unroll
    for (int k = 0; k < K; k++) a1[k] = a2[k] = a3[k] = 0;
    int i = threadIdx.x;
    for (; i + 3 * kTile < n; i += 4 * kTile)
#pragma unroll
        for (int k = 0; k < K; k++) {
            v[k] += __ldcg(&partials[(size_t)(first + i) * kNPart + k]);
            a1[k] += __ldcg(&partials[(size_t)(first + i + kTile) * kNPart + k]);
            a2[k] += __ldcg(&partials[(size_t)(first + i + 2 * kTile) * kNPart + k]);
            a3[k] += __ldcg(&partials[(size_t)(first + i + 3 * kTile) * kNPart + k]);
        }
    for (; i < n; i += kTile)
#pragma unroll
        for (int k = 0; k < K; k++) v[k] += __ldcg(&partials[(size_t)(first + i) * kNPart + k]);
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = (v[k] + a1[k]) + (a2[k] + a3[k]);
    __shared__ T tmp[K];
    block_reduce<K, T>(v, tmp);
    if (threadIdx.x < K) res[threadIdx.x] = tmp[threadIdx.x];
    __syncthreads();
}

// "Last tile of the case finalises": every tile of case c publishes its
// partials, then increments the case counter; the tile that brings it to
// ntiles sums all partials (in tile order, so the result does not depend on
// which tile came last) and resets the counter.
__device__ __forceinline__ bool last_tile_of_case(int *counter, int ntiles) {
    __shared__ int is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        int prev = atomicAdd(counter, 1);
        is_last = (prev == ntiles - 1);
        if (is_last) *counter = 0;
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last != 0;
}

__device__ __forceinline__ int face_of(int fc) { return fc >= 0 ? fc : ~fc; }

// Row i of an ELL operator, y_c = diag*x_c[i] - sum_k a[k][i]*x_c[nb[k][i]]
// for NC vectors x_c = x + c*stride.  Neighbours outside [0, n) (halos,
// padding) contribute nothing.  W is a compile-time width so the index and
// coefficient loads of all slots are issued before any arithmetic; invalid
// slots read x[i] with a zero coefficient instead of branching.
template <int W, int NC, class T>
__device__ __forceinline__ void ell_row_w(const int *__restrict__ nb, const T *__restrict__ a, T diag,
                                          const T *x, int stride, int n, int i, T (&y)[NC]) {
    int j[W];
    T c[W];
#pragma unroll
    for (int k = 0; k < W; k++) {
        const int jj = __ldg(&nb[k * n + i]);
        const bool ok = (unsigned)jj < (unsigned)n;
        j[k] = ok ? jj : i;
        c[k] = ok ? a[k * n + i] : (T)0;
    }
#pragma unroll
    for (int q = 0; q < NC; q++) {
        const T *xq = x + q * stride;
        T s = diag * xq[i];
#pragma unroll
        for (int k = 0; k < W; k++) s -= c[k] * xq[j[k]];
        y[q] = s;
    }
}

template <int NC, class T>
__device__ __forceinline__ void ell_row(const int *__restrict__ nb, const T *__restrict__ a, T diag, const T *x,
                                        int stride, int n, int W, int i, T (&y)[NC]) {
    if (W == 6) { ell_row_w<6, NC, T>(nb, a, diag, x, stride, n, i, y); return; }
    if (W == 4) { ell_row_w<4, NC, T>(nb, a, diag, x, stride, n, i, y); return; }
#pragma unroll
    for (int q = 0; q < NC; q++) y[q] = diag * x[q * stride + i];
    // wide rows (coarse levels): four slots per step, their index, coefficient
    // and vector loads issued together instead of one dependent chain per slot
    for (int k0 = 0; k0 < W; k0 += 4) {
        int jj[4];
        T ak[4];
#pragma unroll
        for (int u = 0; u < 4; u++) jj[u] = k0 + u < W ? nb[(k0 + u) * n + i] : -1;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const bool ok = (unsigned)jj[u] < (unsigned)n;
            ak[u] = ok ? a[(k0 + u) * n + i] : (T)0;
            if (!ok) jj[u] = i;
        }
#pragma unroll
        for (int q = 0; q < NC; q++) {
            T xv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) xv[u] = x[q * stride + jj[u]];
#pragma unroll
            for (int u = 0; u < 4; u++) y[q] -= ak[u] * xv[u];
        }
    }
}

// -x when neg, else x: a sign-bit flip in the integer pipe (no FP64 op)
__device__ __forceinline__ double flip_sign(double x, bool neg) {
    return __longlong_as_double(__double_as_longlong(x) ^ ((long long)neg << 63));
}
// max(x, 0) for non-NaN x, decided on the bit pattern (no FP64 op); -0 -> 0
__device__ __forceinline__ double positive_part(double x) {
    return __double_as_longlong(x) > 0 ? x : 0.0;
}
// -x when neg, else x, for FP32
__device__ __forceinline__ float flip_sign_f(float x, bool neg) {
    return __uint_as_float(__float_as_uint(x) ^ ((unsigned)neg << 31));
}

// FP64 <-> FP32 from the IEEE 754 binary64 / binary32 bit layouts, in the
// integer pipe: GB300 executes the hardware conversion instructions at its
// FP64 rate (2 per SM per clock), so a kernel that is meant to spend no FP64
// work converts this way.
//
// binary64 -> binary32, rounded to nearest (ties to even) on the 29 dropped
// mantissa bits; results below the binary32 normal range become a signed
// zero, overflow gives infinity, NaN stays NaN.
__device__ __forceinline__ float narrow_f32(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ffu);
    const unsigned long long m = b & 0xfffffffffffffull;
    if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u));
    const int fe = e - 1023 + 127;
    if (fe <= 0) return __uint_as_float(sign);
    if (fe >= 255) return __uint_as_float(sign | 0x7f800000u);
    unsigned r = ((unsigned)fe << 23) | (unsigned)(m >> 29);
    const unsigned rem = (unsigned)(m & 0x1fffffffu);
    if (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) r += 1u;   // a carry moves into the exponent
    return __uint_as_float(sign | r);
}
// binary32 -> binary64: exact for normal values; a binary32 subnormal gives a
// signed zero
__device__ __forceinline__ double widen_f64(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    if (e == 0) return __longlong_as_double((long long)sign);
    const unsigned long long de = e == 0xffu ? 0x7ffull : (unsigned long long)(e - 127 + 1023);
    return __longlong_as_double((long long)(sign | (de << 52) | ((unsigned long long)m << 29)));
}

}  // namespace cfdl
