// cfdl_prof.cpp -- CUDA-event timing on a context's own stream.
//
// cfdl_timer_begin/end bracket any span of work; the kernel profiler
// brackets individual launches (all kernels, or one named kernel) so a caller
// can attribute device time per kernel.  Events are recorded on ctx->stream,
// the stream every kernel of the context is launched on.
#include "cfdl_internal.h"
#include <cstring>
#include <string>

namespace cfdl {

struct ProfRec { std::string name; cudaEvent_t a, b; };
struct Prof {
    int mode = 0;                 // 0 off, 1 all kernels, 2 one kernel
    std::string only;
    std::vector<ProfRec> recs;
    size_t used = 0;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    // results
    std::vector<std::string> names;
    std::vector<int64_t> counts;
    std::vector<double> totals;
};

static Prof *prof_of(cfdl_ctx *ctx) {
    if (!ctx->prof) ctx->prof = new Prof;
    return static_cast<Prof *>(ctx->prof);
}

void prof_destroy(cfdl_ctx *ctx) {
    Prof *p = static_cast<Prof *>(ctx->prof);
    if (!p) return;
    for (auto &r : p->recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    if (p->t0) cudaEventDestroy(p->t0);
    if (p->t1) cudaEventDestroy(p->t1);
    delete p;
    ctx->prof = nullptr;
}

bool prof_wants(cfdl_ctx *ctx, const char *name) {
    Prof *p = static_cast<Prof *>(ctx->prof);
    if (!p || p->mode == 0 || ctx->capturing) return false;
    return p->mode == 1 || p->only == name;
}

bool prof_active(cfdl_ctx *ctx) {
    Prof *p = static_cast<Prof *>(ctx->prof);
    return p && p->mode != 0;
}

void prof_begin(cfdl_ctx *ctx, const char *name) {
    Prof *p = static_cast<Prof *>(ctx->prof);
    if (p->used == p->recs.size()) {
        ProfRec r;
        cudaEventCreate(&r.a);
        cudaEventCreate(&r.b);
        p->recs.push_back(r);
    }
    p->recs[p->used].name = name;
    cudaEventRecord(p->recs[p->used].a, ctx->stream);
}

void prof_end(cfdl_ctx *ctx) {
    Prof *p = static_cast<Prof *>(ctx->prof);
    cudaEventRecord(p->recs[p->used].b, ctx->stream);
    p->used++;
}

}  // namespace cfdl

using namespace cfdl;

extern "C" {

int cfdl_select_device(int device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { cudaGetLastError(); return CFDL_ERR_NO_DEVICE; }
    if (device < 0 || device >= n) return CFDL_ERR_INVALID;
    return cuda_status(cudaSetDevice(device));
}

int cfdl_timer_begin(cfdl_ctx *ctx) {
    if (!ctx) return CFDL_ERR_INVALID;
    Prof *p = prof_of(ctx);
    if (!p->t0) { cudaEventCreate(&p->t0); cudaEventCreate(&p->t1); }
    return cuda_status(cudaEventRecord(p->t0, ctx->stream));
}

int cfdl_timer_end(cfdl_ctx *ctx, double *ms) {
    if (!ctx || !ms) return CFDL_ERR_INVALID;
    Prof *p = prof_of(ctx);
    if (!p->t0) return CFDL_ERR_INVALID;
    cudaError_t e = cudaEventRecord(p->t1, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(p->t1);
    float f = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&f, p->t0, p->t1);
    *ms = f;
    return cuda_status(e);
}

int cfdl_profile_start(cfdl_ctx *ctx, const char *kernel) {
    if (!ctx) return CFDL_ERR_INVALID;
    Prof *p = prof_of(ctx);
    p->mode = (kernel && kernel[0]) ? 2 : 1;
    p->only = (kernel && kernel[0]) ? kernel : "";
    p->used = 0;
    p->names.clear(); p->counts.clear(); p->totals.clear();
    return CFDL_OK;
}

int cfdl_profile_stop(cfdl_ctx *ctx, int *nkernels) {
    if (!ctx) return CFDL_ERR_INVALID;
    Prof *p = prof_of(ctx);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_status(e);
    for (size_t i = 0; i < p->used; i++) {
        float f = 0.f;
        cudaEventElapsedTime(&f, p->recs[i].a, p->recs[i].b);
        size_t k = 0;
        while (k < p->names.size() && p->names[k] != p->recs[i].name) k++;
        if (k == p->names.size()) { p->names.push_back(p->recs[i].name); p->counts.push_back(0); p->totals.push_back(0.0); }
        p->counts[k]++;
        p->totals[k] += f;
    }
    p->mode = 0;
    p->used = 0;
    if (nkernels) *nkernels = (int)p->names.size();
    return CFDL_OK;
}

int cfdl_profile_get(cfdl_ctx *ctx, int i, char *name64, int64_t *launches, double *total_ms) {
    if (!ctx || !ctx->prof) return CFDL_ERR_INVALID;
    Prof *p = static_cast<Prof *>(ctx->prof);
    if (i < 0 || i >= (int)p->names.size()) return CFDL_ERR_INVALID;
    if (name64) { std::strncpy(name64, p->names[i].c_str(), 63); name64[63] = 0; }
    if (launches) *launches = p->counts[i];
    if (total_ms) *total_ms = p->totals[i];
    return CFDL_OK;
}

}  // extern "C"
