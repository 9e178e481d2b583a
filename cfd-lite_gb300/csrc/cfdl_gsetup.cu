// cfdl_gsetup.cu -- the mesh set-up's face matching, face numbering and
// geometry on the GPU, with the host builder's results bit for bit
// (cfdl_setup_create_device; the host form is cfdl_setup.cpp).
//
// Matching.  Every element face gets a key: its vertex ids sorted (0-padded
// at the front for triangles) and its smallest vertex minv.  The reference
// numbers a face at its smallest vertex and, among the faces first met at that
// vertex, in the order of the owner (lower element, local face)
// (find_element_nb, src/setup/mod_mg_lvl_uns.f90:283-488).  So the keys are
// bucketed by minv (counting sort: per-vertex counts, a scan, a scatter), each
// bucket -- a few dozen keys -- is put in (element, local face) order and its
// keys are paired by vertex tuple in one thread, and a scan over the buckets'
// pair counts gives every face its number.  No comparison sort over all faces.
//
// Geometry.  calc_aip_xyzip_uns (src/setup/calc_aip_xyzip.f90:7-74) per face
// and calc_vol_cv_centers_uns (src/setup/calc_vol_cv_centers.f90:4-61) per
// cell, operation by operation in the host builder's order.  This file is
// compiled without FMA contraction, and FP64 add, multiply and divide are
// correctly rounded, so the doubles equal the host's.
//
// The edge-boundary marking and the red/black order depend on visiting order
// and stay on the host (cfdl_setup.cpp: finish_topology).
#include "cfdl_setup_int.h"
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>

namespace cfdl_setup_detail {
namespace {

constexpr int kThreads = 256;

inline int blocks(long n) { return (int)((n + kThreads - 1) / kThreads); }

// per element: its section's type (sections are few; linear search)
__device__ __forceinline__ int elem_type(const int *esec, const int *etype, int nsec, int e) {
    for (int s = 0; s < nsec; s++) if (e <= esec[2 * s + 1]) return etype[s];
    return etype[nsec - 1];
}

// one key per element face: volume element e's faces at its CSR slots, each
// 2D element's face after them -- the (element, local face) order
__global__ void k_face_keys(int nelem, int ng, int H, int m, const int *__restrict__ e2vx, const int *__restrict__ esec,
                            const int *__restrict__ etype, int nsec, const int *__restrict__ ef2nb_idx, int4 *kv,
                            int *ke, int *kf, int *kmin, int *bad) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (e > nelem) return;
    const int t = elem_type(esec, etype, nsec, e);
    const int nfc = element_nface(t);
    const long base = e <= ng ? (long)ef2nb_idx[e - 1] - 1 : (long)H + (e - ng - 1);
    if (e > ng && nfc != 1) { *bad = 1; return; }
    for (int f = 1; f <= nfc; f++) {
        int lst[4], nl;
        if (!face_vxlist(&e2vx[(size_t)(e - 1) * m], t, f, lst, nl)) { *bad = 1; return; }
        int v[4] = {0, 0, 0, 0};
        for (int q = 0; q < nl; q++) v[4 - nl + q] = lst[q];
        // sort the nl ids (insertion sort; at most 4)
        for (int a = 4 - nl + 1; a < 4; a++) {
            const int x = v[a];
            int b = a - 1;
            while (b >= 4 - nl && v[b] > x) { v[b + 1] = v[b]; b--; }
            v[b + 1] = x;
        }
        const long p = base + f - 1;
        kv[p] = make_int4(v[0], v[1], v[2], v[3]);
        ke[p] = e;
        kf[p] = f;
        kmin[p] = v[4 - nl];
    }
}

__global__ void k_count(long nk, const int *__restrict__ kmin, int *cnt) {
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < nk) atomicAdd(&cnt[kmin[p]], 1);
}

// exclusive scan of n ints in three launches: per-block sums, a one-block
// scan of the sums, per-block scans with the carried offset
constexpr int kScanBlock = 1024;
__global__ void k_scan_sums(const int *__restrict__ in, long n, int *bsum) {
    __shared__ int sh[kScanBlock];
    const long i = (long)blockIdx.x * kScanBlock + threadIdx.x;
    sh[threadIdx.x] = i < n ? in[i] : 0;
    __syncthreads();
    for (int o = kScanBlock / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = sh[0];
}
__global__ void k_scan_top(int *bsum, int nb, int *total) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int run = 0;
    for (int b = 0; b < nb; b++) { const int x = bsum[b]; bsum[b] = run; run += x; }
    *total = run;
}
__global__ void k_scan_apply(const int *__restrict__ in, long n, const int *__restrict__ bsum, int *out) {
    __shared__ int sh[kScanBlock];
    const long i = (long)blockIdx.x * kScanBlock + threadIdx.x;
    const int x = i < n ? in[i] : 0;
    sh[threadIdx.x] = x;
    __syncthreads();
    // Hillis-Steele inclusive scan in shared memory
    for (int o = 1; o < kScanBlock; o <<= 1) {
        const int y = (int)threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += y;
        __syncthreads();
    }
    if (i < n) out[i] = bsum[blockIdx.x] + sh[threadIdx.x] - x;
}

__global__ void k_scatter(long nk, const int *__restrict__ kmin, const int *__restrict__ start, int *fill, int *perm) {
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nk) return;
    const int v = kmin[p];
    perm[start[v] + atomicAdd(&fill[v], 1)] = (int)p;
}

// Per vertex bucket: (element, local face) order, then pairs by vertex tuple.
// Key position p is already the (element, local face) rank, so the bucket is
// sorted by p.  Pairs are written at the bucket's start in first-met order.
__global__ void k_bucket_pairs(int nv, int ng, const int *__restrict__ start, int *perm, const int4 *__restrict__ kv,
                               const int *__restrict__ ke, int *pair_a, int *pair_b, int *npairs, int *bad) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v > nv) return;
    const int b0 = start[v], b1 = start[v + 1], n = b1 - b0;
    int *P = perm + b0;
    for (int a = 1; a < n; a++) {
        const int x = P[a];
        int b = a - 1;
        while (b >= 0 && P[b] > x) { P[b + 1] = P[b]; b--; }
        P[b + 1] = x;
    }
    int np = 0;
    for (int a = 0; a < n; a++) {
        const int pa = P[a];
        if (pa < 0) continue;                       // already paired
        const int4 va = kv[pa];
        int partner = -1, matches = 0;
        for (int c = a + 1; c < n; c++) {
            const int pc = P[c];
            if (pc < 0) continue;
            const int4 vc = kv[pc];
            if (vc.x == va.x && vc.y == va.y && vc.z == va.z && vc.w == va.w) {
                if (partner < 0) partner = c;
                matches++;
            }
        }
        if (matches != 1 || ke[pa] > ng) { *bad = 1; return; }   // unmatched, non-conforming, or two 2D elements
        pair_a[b0 + np] = pa;
        pair_b[b0 + np] = P[partner];
        np++;
        P[partner] = -1;
    }
    npairs[v] = np;
}

// Face fg = (pairs before this bucket) + rank in the bucket + 1.
__global__ void k_fill_faces(int nv, int ng, int H, const int *__restrict__ start, const int *__restrict__ pstart,
                             const int *__restrict__ npairs, const int *__restrict__ pair_a, const int *__restrict__ pair_b,
                             const int *__restrict__ ke, const int *__restrict__ kf, const int *__restrict__ ef2nb_idx,
                             int *ef2nb1, int *ef2nb2, int *s2g, int *bs) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v > nv) return;
    const int b0 = start[v];
    for (int q = 0; q < npairs[v]; q++) {
        const int fg = pstart[v] + q + 1;
        const int pa = pair_a[b0 + q], pb = pair_b[b0 + q];
        const int e1 = ke[pa], f1 = kf[pa], e2 = ke[pb], f2 = kf[pb];
        const int idx1 = ef2nb_idx[e1 - 1] + f1 - 1;
        if (e2 > ng) {
            ef2nb1[idx1 - 1] = index_t(e2, 0);
            ef2nb2[idx1 - 1] = fg;
            s2g[fg - 1] = index_t(e1, f1);
            bs[e2 - ng - 1] = index_t(e1, f1);
        } else {
            const int idx2 = ef2nb_idx[e2 - 1] + f2 - 1;
            ef2nb1[idx1 - 1] = index_t(e2, f2);
            ef2nb1[idx2 - 1] = index_t(e1, f1);
            ef2nb2[idx1 - 1] = fg;
            ef2nb2[idx2 - 1] = -fg;
            s2g[fg - 1] = index_t(e1, f1);
        }
    }
    (void)H;
}

// calc_aip_xyzip_uns, per face, in the host builder's operation order
__global__ void k_face_geometry(int nf, int m, const int *__restrict__ s2g, const int *__restrict__ e2vx,
                                const int *__restrict__ esec, const int *__restrict__ etype, int nsec,
                                const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                                double *aip, double *rip) {
    const int fg = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (fg > nf) return;
    int e, fl;
    get_idx(s2g[fg - 1], e, fl);
    const int t = elem_type(esec, etype, nsec, e);
    int lst[4], nl;
    face_vxlist(&e2vx[(size_t)(e - 1) * m], t, fl, lst, nl);
    double r[4][3], a[3], sumc[3][3];
    for (int q = 0; q < nl; q++) { r[q][0] = x[lst[q] - 1]; r[q][1] = y[lst[q] - 1]; r[q][2] = z[lst[q] - 1]; }
    for (int tr = 0; tr < (nl == 3 ? 1 : 2); tr++) {
        const int i0 = 0, i1 = tr == 0 ? 1 : 2, i2 = tr == 0 ? 2 : 3;
        double dr1[3], dr2[3], av[3], sub[3];
        for (int q = 0; q < 3; q++) { dr1[q] = r[i1][q] - r[i0][q]; dr2[q] = r[i2][q] - r[i0][q]; }
        av[0] = dr1[1] * dr2[2] - dr1[2] * dr2[1];
        av[1] = dr1[2] * dr2[0] - dr1[0] * dr2[2];
        av[2] = dr1[0] * dr2[1] - dr1[1] * dr2[0];
        for (int q = 0; q < 3; q++) av[q] = 0.5 * av[q];
        for (int q = 0; q < 3; q++) sub[q] = (r[i0][q] + r[i1][q] + r[i2][q]) / 3.0;
        for (int q = 0; q < 3; q++) a[q] = tr == 0 ? av[q] : a[q] + av[q];
        for (int q = 0; q < 3; q++)
            for (int p = 0; p < 3; p++) sumc[q][p] = tr == 0 ? sub[q] * av[p] : sumc[q][p] + sub[q] * av[p];
    }
    const double dd = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    double *ao = &aip[3 * (size_t)(fg - 1)], *ro = &rip[3 * (size_t)(fg - 1)];
    for (int q = 0; q < 3; q++) ao[q] = a[q];
    for (int q = 0; q < 3; q++) ro[q] = (sumc[q][0] * a[0] + sumc[q][1] * a[1] + sumc[q][2] * a[2]) / dd;
}

// calc_vol_cv_centers_uns, per cell (halo centres = their face's centroid)
__global__ void k_cell_geometry(int ng, int m, const int *__restrict__ e2vx, const int *__restrict__ esec,
                                const int *__restrict__ etype, int nsec, const double *__restrict__ x,
                                const double *__restrict__ y, const double *__restrict__ z,
                                const int *__restrict__ ef2nb_idx, const int *__restrict__ ef2nb1,
                                const int *__restrict__ ef2nb2, const double *__restrict__ aip,
                                const double *__restrict__ rip, double *xc, double *yc, double *zc, double *vol,
                                int *flat) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (e > ng) return;
    const int t = elem_type(esec, etype, nsec, e), nv = element_nvx(t);
    double gc[3] = {0, 0, 0}, rc[3] = {0, 0, 0}, sum_vol = 0;
    for (int q = 1; q <= nv; q++) {
        const int vx = e2vx[(size_t)(e - 1) * m + q - 1];
        gc[0] = gc[0] + x[vx - 1]; gc[1] = gc[1] + y[vx - 1]; gc[2] = gc[2] + z[vx - 1];
    }
    for (int q = 0; q < 3; q++) gc[q] = gc[q] / nv;
    for (int idx = ef2nb_idx[e - 1]; idx <= ef2nb_idx[e] - 1; idx++) {
        int gf = ef2nb2[idx - 1], enb, lf;
        const int sg = gf >= 0 ? 1 : -1;
        gf = gf >= 0 ? gf : -gf;
        const double *cs = &rip[3 * (size_t)(gf - 1)], *ai = &aip[3 * (size_t)(gf - 1)];
        get_idx(ef2nb1[idx - 1], enb, lf);
        if (lf == 0) { xc[enb - 1] = cs[0]; yc[enb - 1] = cs[1]; zc[enb - 1] = cs[2]; }
        const double h[3] = {cs[0] - gc[0], cs[1] - gc[1], cs[2] - gc[2]};
        const double sub_vol = ((sg * ai[0]) * h[0] + (sg * ai[1]) * h[1] + (sg * ai[2]) * h[2]) / 3.0;
        sum_vol = sum_vol + sub_vol;
        for (int q = 0; q < 3; q++) rc[q] = rc[q] + (0.25 * gc[q] + 0.75 * cs[q]) * sub_vol;
    }
    for (int q = 0; q < 3; q++) rc[q] = rc[q] / sum_vol;
    xc[e - 1] = rc[0]; yc[e - 1] = rc[1]; zc[e - 1] = rc[2];
    vol[e - 1] = sum_vol;
    if (!(sum_vol > 1e-20)) *flat = 1;
}

// device buffers of one set-up, freed on scope exit
struct DevBufs {
    std::vector<void *> p;
    ~DevBufs() { for (void *q : p) cudaFree(q); }
    template <class T> T *alloc(size_t n) {
        void *d = nullptr;
        if (cudaMalloc(&d, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        p.push_back(d);
        return (T *)d;
    }
};

int cuda_st(cudaError_t e) {
    if (e == cudaSuccess) return CFDL_OK;
    if (e == cudaErrorMemoryAllocation) return CFDL_ERR_OOM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return CFDL_ERR_NO_DEVICE;
    return CFDL_ERR_CUDA;
}

template <class T> int upload(DevBufs &B, T **d, const std::vector<T> &h) {
    *d = B.alloc<T>(h.size());
    if (!*d) return CFDL_ERR_OOM;
    return cuda_st(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}

template <class T, class A> int download(std::vector<T, A> &h, const T *d, size_t n) {
    h.resize(n);
    return cuda_st(cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost));
}

// exclusive scan of n ints from in to out (out[n] = total)
int scan(DevBufs &B, const int *in, long n, int *out) {
    const int nb = (int)((n + kScanBlock - 1) / kScanBlock);
    int *bsum = B.alloc<int>(nb);
    if (!bsum) return CFDL_ERR_OOM;
    k_scan_sums<<<nb, kScanBlock>>>(in, n, bsum);
    k_scan_top<<<1, 32>>>(bsum, nb, out + n);
    k_scan_apply<<<nb, kScanBlock>>>(in, n, bsum, out);
    return cuda_st(cudaGetLastError());
}

}  // namespace

int match_faces_device(cfdl_setup &S) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return CFDL_ERR_NO_DEVICE; }
    const int ng = S.ne, m = S.m, H = S.ef2nb_idx[ng] - 1, nv = S.nvx;
    const long nk = (long)H + (S.nelem - ng);
    DevBufs B;
    int *d_e2vx, *d_esec, *d_etype, *d_idx, st;
    if ((st = upload(B, &d_e2vx, S.e2vx)) || (st = upload(B, &d_esec, S.esec)) || (st = upload(B, &d_etype, S.etype)) ||
        (st = upload(B, &d_idx, S.ef2nb_idx)))
        return st;
    int4 *kv = B.alloc<int4>(nk);
    int *ke = B.alloc<int>(nk), *kf = B.alloc<int>(nk), *kmin = B.alloc<int>(nk), *perm = B.alloc<int>(nk);
    int *cnt = B.alloc<int>(nv + 2), *start = B.alloc<int>(nv + 3), *fill = B.alloc<int>(nv + 2);
    int *pair_a = B.alloc<int>(nk), *pair_b = B.alloc<int>(nk), *npairs = B.alloc<int>(nv + 2),
        *pstart = B.alloc<int>(nv + 3), *bad = B.alloc<int>(1);
    int *d_ef1 = B.alloc<int>(H), *d_ef2 = B.alloc<int>(H), *d_s2g = B.alloc<int>(S.nf), *d_bs = B.alloc<int>(S.nbf);
    if (!kv || !ke || !kf || !kmin || !perm || !cnt || !start || !fill || !pair_a || !pair_b || !npairs || !pstart ||
        !bad || !d_ef1 || !d_ef2 || !d_s2g || !d_bs)
        return CFDL_ERR_OOM;
    cudaMemset(cnt, 0, (nv + 2) * sizeof(int));
    cudaMemset(fill, 0, (nv + 2) * sizeof(int));
    cudaMemset(npairs, 0, (nv + 2) * sizeof(int));
    cudaMemset(bad, 0, sizeof(int));
    k_face_keys<<<blocks(S.nelem), kThreads>>>(S.nelem, ng, H, m, d_e2vx, d_esec, d_etype, S.nsec, d_idx, kv, ke, kf,
                                               kmin, bad);
    k_count<<<blocks(nk), kThreads>>>(nk, kmin, cnt);
    if ((st = scan(B, cnt, nv + 2, start))) return st;          // start[v], v = 0..nv+1
    k_scatter<<<blocks(nk), kThreads>>>(nk, kmin, start, fill, perm);
    k_bucket_pairs<<<blocks(nv + 1), kThreads>>>(nv, ng, start, perm, kv, ke, pair_a, pair_b, npairs, bad);
    if ((st = scan(B, npairs, nv + 2, pstart))) return st;
    int h_bad = 0, npair_total = 0;
    if ((st = cuda_st(cudaMemcpy(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost)))) return st;
    if ((st = cuda_st(cudaMemcpy(&npair_total, pstart + nv + 2, sizeof(int), cudaMemcpyDeviceToHost)))) return st;
    if (h_bad || npair_total != S.nf) return CFDL_ERR_MESH;
    k_fill_faces<<<blocks(nv + 1), kThreads>>>(nv, ng, H, start, pstart, npairs, pair_a, pair_b, ke, kf, d_idx, d_ef1,
                                               d_ef2, d_s2g, d_bs);
    if ((st = cuda_st(cudaGetLastError()))) return st;
    if ((st = download(S.ef2nb1, d_ef1, H)) || (st = download(S.ef2nb2, d_ef2, H)) || (st = download(S.s2g, d_s2g, S.nf)) ||
        (st = download(S.bs, d_bs, S.nbf)))
        return st;
    return CFDL_OK;
}

int geometry_device(cfdl_setup &S) {
    const int ng = S.ne, m = S.m, H = S.ef2nb_idx[ng] - 1;
    DevBufs B;
    int *d_e2vx, *d_esec, *d_etype, *d_idx, *d_ef1, *d_ef2, *d_s2g, st;
    double *dx, *dy, *dz;
    if ((st = upload(B, &d_e2vx, S.e2vx)) || (st = upload(B, &d_esec, S.esec)) || (st = upload(B, &d_etype, S.etype)) ||
        (st = upload(B, &d_idx, S.ef2nb_idx)) || (st = upload(B, &d_ef1, S.ef2nb1)) || (st = upload(B, &d_ef2, S.ef2nb2)) ||
        (st = upload(B, &d_s2g, S.s2g)) || (st = upload(B, &dx, S.x)) || (st = upload(B, &dy, S.y)) ||
        (st = upload(B, &dz, S.z)))
        return st;
    double *aip = B.alloc<double>(3 * (size_t)S.nf), *rip = B.alloc<double>(3 * (size_t)S.nf);
    double *xc = B.alloc<double>(S.nelem), *yc = B.alloc<double>(S.nelem), *zc = B.alloc<double>(S.nelem),
           *vol = B.alloc<double>(ng);
    int *flat = B.alloc<int>(1);
    if (!aip || !rip || !xc || !yc || !zc || !vol || !flat) return CFDL_ERR_OOM;
    cudaMemset(xc, 0, S.nelem * sizeof(double));
    cudaMemset(yc, 0, S.nelem * sizeof(double));
    cudaMemset(zc, 0, S.nelem * sizeof(double));
    cudaMemset(flat, 0, sizeof(int));
    k_face_geometry<<<blocks(S.nf), kThreads>>>(S.nf, m, d_s2g, d_e2vx, d_esec, d_etype, S.nsec, dx, dy, dz, aip, rip);
    k_cell_geometry<<<blocks(ng), kThreads>>>(ng, m, d_e2vx, d_esec, d_etype, S.nsec, dx, dy, dz, d_idx, d_ef1, d_ef2,
                                              aip, rip, xc, yc, zc, vol, flat);
    if ((st = cuda_st(cudaGetLastError()))) return st;
    int h_flat = 0;
    if ((st = download(S.aip, aip, 3 * (size_t)S.nf)) || (st = download(S.rip, rip, 3 * (size_t)S.nf)) ||
        (st = download(S.xc, xc, S.nelem)) || (st = download(S.yc, yc, S.nelem)) || (st = download(S.zc, zc, S.nelem)) ||
        (st = download(S.vol, vol, ng)) || (st = cuda_st(cudaMemcpy(&h_flat, flat, sizeof(int), cudaMemcpyDeviceToHost))))
        return st;
    (void)H;
    return h_flat ? CFDL_ERR_MESH : CFDL_OK;
}

}  // namespace cfdl_setup_detail
