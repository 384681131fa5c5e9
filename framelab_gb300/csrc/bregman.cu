// bregman.cu -- split Bregman driver (solveSplitBregman.m:15-41) over the
// native CGLS and the fused framelet step; everything stays on the device.
// fl_sb_create keeps the framelet, the CGLS workspace and the coefficient
// sets of one plan for repeated solves; fl_sb_solve is the one-shot form.
#include <cmath>
#include <new>

#include "fl_trace.h"
#include "fl_common.cuh"
#include "fl_plan.h"

namespace {
__global__ void k_diff(float* __restrict__ d, const float* __restrict__ a,
                       const float* __restrict__ b, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        d[i] = a[i] - b[i];
}
}  // namespace

struct fl_sb {
    fl_plan* plan;
    fl_framelet* fw;
    fl_cgls* cg;
    long long n, nc;
    float *Atf, *b, *v, *t, *prev;
    double* dsum;
};

extern "C" void fl_sb_destroy(fl_sb* sb)
{
    if (!sb) return;
    void* bufs[] = {sb->Atf, sb->b, sb->v, sb->t, sb->prev, sb->dsum};
    for (void* q : bufs)
        if (q) cudaFree(q);
    if (sb->cg) fl_cgls_destroy(sb->cg);
    if (sb->fw) fl_framelet_destroy(sb->fw);
    delete sb;
}

extern "C" int fl_sb_create(fl_plan* plan, int levels, int kind, int mode, fl_sb** out)
{
    FL_RANGE("fl_sb_create");
    if (!plan || !out) return fl_set_error(FL_ERR_INVALID, "fl_sb_create: null argument");
    *out = nullptr;
    fl_sb* sb = new (std::nothrow) fl_sb();
    if (!sb) return fl_set_error(FL_ERR_ALLOC, "out of host memory");
    sb->plan = plan;
    const fl_scan& sc = plan->s;
    int st = fl_framelet_create(sc.nx, sc.ny, sc.nz, levels, kind, &sb->fw);
    if (!st) st = fl_cgls_create(plan, mode, &sb->cg);
    if (st) { fl_sb_destroy(sb); return st; }
    sb->n = plan->n_vox;
    sb->nc = fl_framelet_ncoef(sb->fw);
    auto alloc = [&](float** p, long long elems) {
        if (!st) st = fl_check_cuda(fl_malloc((void**)p, elems * sizeof(float)),
                                    "fl_malloc(split Bregman)");
    };
    alloc(&sb->Atf, sb->n); alloc(&sb->b, sb->n); alloc(&sb->v, sb->nc); alloc(&sb->t, sb->nc);
    alloc(&sb->prev, sb->n);
    if (!st) st = fl_check_cuda(fl_malloc((void**)&sb->dsum, 2 * sizeof(double)),
                                "fl_malloc(split Bregman)");
    if (st) { fl_sb_destroy(sb); return st; }
    *out = sb;
    return fl_set_error(FL_OK, "");
}

extern "C" int fl_sb_run(fl_sb* sb, const float* f, float* u, float lam, float mu, int outer,
                         int cg_iters, double cg_tol, double* history, void* stream)
{
    FL_RANGE("fl_sb_run");
    if (!sb || !f || !u || outer < 0 || cg_iters < 0 || !(mu > 0))
        return fl_set_error(FL_ERR_INVALID, "fl_sb_run: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = sb->n;
    int st = fl_adjoint(sb->plan, FL_MODEL_MATCHED, f, FL_F32, sb->Atf, FL_F32, stream);  // A^T f
    // alpha = v = W u0 ; b = Atf + mu W^T(alpha - v) = Atf
    if (!st) st = fl_framelet_analysis(sb->fw, u, sb->v, stream);
    if (!st) st = fl_check_cuda(cudaMemcpyAsync(sb->b, sb->Atf, n * 4, cudaMemcpyDeviceToDevice, s),
                                "copy");
    for (int k = 0; k < outer && !st; k++) {
        st = fl_check_cuda(cudaMemcpyAsync(sb->prev, u, n * 4, cudaMemcpyDeviceToDevice, s), "copy");
        // u = CGLS(A, At, b, u, mu, cg_iters, cg_tol)  (warm start: A_loc(u) - b)
        if (!st) st = fl_cgls_solve(sb->cg, sb->b, u, mu, cg_iters, cg_tol, 10, 0, nullptr, nullptr,
                                    stream);
        if (!st) st = fl_framelet_bregman(sb->fw, u, sb->v, sb->t, sb->Atf, mu, lam / mu, sb->b,
                                          stream);
        if (!st && history) {
            k_diff<<<1024, 256, 0, s>>>(sb->prev, u, sb->prev, n);
            double* d = sb->dsum;
            if (!(st = fl_check_launch("split Bregman diff")) &&
                !(st = fl_dot(sb->prev, sb->prev, n, d, stream)) &&
                !(st = fl_dot(u, u, n, d + 1, stream))) {
                double h[2];
                st = fl_check_cuda(cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, s), "D2H");
                if (!st) st = fl_check_cuda(cudaStreamSynchronize(s), "sync");
                if (!st) history[k] = h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
            }
        }
    }
    if (st) return st;
    return fl_set_error(FL_OK, "");
}

extern "C" int fl_sb_solve(fl_plan* plan, const float* f, float* u, float lam, float mu,
                           int outer, int cg_iters, double cg_tol, int levels, int kind, int mode,
                           double* history, void* stream)
{
    FL_RANGE("fl_sb_solve");
    if (!plan || !f || !u || outer < 0 || cg_iters < 0 || !(mu > 0))
        return fl_set_error(FL_ERR_INVALID, "fl_sb_solve: bad argument");
    fl_sb* sb = nullptr;
    int st = fl_sb_create(plan, levels, kind, mode, &sb);
    if (st) return st;
    st = fl_sb_run(sb, f, u, lam, mu, outer, cg_iters, cg_tol, history, stream);
    cudaError_t se = cudaStreamSynchronize((cudaStream_t)stream);   // buffers are freed next
    if (!st) st = fl_check_cuda(se, "cudaStreamSynchronize");
    fl_sb_destroy(sb);
    if (st) return st;
    return fl_set_error(FL_OK, "");
}
