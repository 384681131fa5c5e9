// bregman.cu -- split Bregman driver (solveSplitBregman.m:15-41) over the
// native CGLS and the fused framelet step; everything stays on the device.
#include <cmath>

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

struct DevMem {
    void* p = nullptr;
    ~DevMem() { if (p) cudaFree(p); }
};
}  // namespace

extern "C" int fl_sb_solve(fl_plan* plan, const float* f, float* u, float lam, float mu,
                           int outer, int cg_iters, double cg_tol, int levels, int kind, int mode,
                           double* history, void* stream)
{
    FL_RANGE("fl_sb_solve");
    if (!plan || !f || !u || outer < 0 || cg_iters < 0 || !(mu > 0))
        return fl_set_error(FL_ERR_INVALID, "fl_sb_solve: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    const fl_scan& sc = plan->s;
    int st;
    fl_framelet* fw = nullptr;
    if ((st = fl_framelet_create(sc.nx, sc.ny, sc.nz, levels, kind, &fw))) return st;
    fl_cgls* cg = nullptr;
    if ((st = fl_cgls_create(plan, mode, &cg))) { fl_framelet_destroy(fw); return st; }
    const long long n = plan->n_vox;
    const long long nc = fl_framelet_ncoef(fw);
    DevMem Atf, b, v, t, prev, dsum;
    auto alloc = [&](DevMem& m, size_t bytes) {
        return st ? st : (st = fl_check_cuda(fl_malloc(&m.p, bytes), "fl_malloc(split Bregman)"));
    };
    alloc(Atf, n * 4); alloc(b, n * 4); alloc(v, nc * 4); alloc(t, nc * 4); alloc(prev, n * 4);
    alloc(dsum, 2 * sizeof(double));
    if (!st) st = fl_adjoint(plan, FL_MODEL_MATCHED, f, FL_F32, Atf.p, FL_F32, stream);   // A^T f
    // alpha = v = W u0 ; b = Atf + mu W^T(alpha - v) = Atf
    if (!st) st = fl_framelet_analysis(fw, u, (float*)v.p, stream);
    if (!st) st = fl_check_cuda(cudaMemcpyAsync(b.p, Atf.p, n * 4, cudaMemcpyDeviceToDevice, s), "copy");
    for (int k = 0; k < outer && !st; k++) {
        st = fl_check_cuda(cudaMemcpyAsync(prev.p, u, n * 4, cudaMemcpyDeviceToDevice, s), "copy");
        // u = CGLS(A, At, b, u, mu, cg_iters, cg_tol)  (warm start: A_loc(u) - b)
        if (!st) st = fl_cgls_solve(cg, (const float*)b.p, u, mu, cg_iters, cg_tol, 10, 0, nullptr,
                                    nullptr, stream);
        if (!st) st = fl_framelet_bregman(fw, u, (float*)v.p, (float*)t.p, (const float*)Atf.p, mu,
                                          lam / mu, (float*)b.p, stream);
        if (!st && history) {
            k_diff<<<1024, 256, 0, s>>>((float*)prev.p, u, (const float*)prev.p, n);
            double* d = (double*)dsum.p;
            if (!(st = fl_check_launch("split Bregman diff")) &&
                !(st = fl_dot((const float*)prev.p, (const float*)prev.p, n, d, stream)) &&
                !(st = fl_dot(u, u, n, d + 1, stream))) {
                double h[2];
                st = fl_check_cuda(cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, s), "D2H");
                if (!st) st = fl_check_cuda(cudaStreamSynchronize(s), "sync");
                if (!st) history[k] = h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
            }
        }
    }
    cudaError_t se = cudaStreamSynchronize(s);   // buffers below are freed on return
    if (!st) st = fl_check_cuda(se, "cudaStreamSynchronize");
    fl_cgls_destroy(cg);
    fl_framelet_destroy(fw);
    if (st) return st;
    return fl_set_error(FL_OK, "");
}
