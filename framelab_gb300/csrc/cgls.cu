// cgls.cu -- CGLS on the normal equations (A^T A + lam I) u = b and the vector
// algebra it needs (solveCGLS.m:6-31, ObjectData.objdot/plus/mtimes).
//
// Inner products and the step lengths alpha/beta are FP64. Two drivers:
//  * FL_CGLS_PLAIN: FP32 storage, one kernel per vector operation, every
//    scalar brought back to the host (the reference's loop, with the
//    projector on the GPU).
//  * FL_CGLS_GRAPH: FP32 storage; axpy/dot work fused into three kernels that
//    keep alpha, beta and gamma in device memory; one iteration captured as a
//    CUDA graph and replayed.
//  * FL_CGLS_MIXED: as FL_CGLS_GRAPH, with FP16 storage of the two operands
//    the projectors read: the search direction (scaled, gathered along each
//    ray with FP32 accumulation) and, on a cone plan, the forward projection
//    that feeds the backprojection (scaled by the plan's y16_scale, gathered
//    with FP32 accumulation). u, r and the step lengths stay FP32 / FP64, so
//    the residual is updated in FP32 every iteration; every `refresh`
//    iterations it is recomputed in FP32 from u (r = (A^T A + lam) u - b).
// Both stop early once gamma < tol, like the reference; in the graph this is a
// device flag that turns the remaining replays into no-ops.
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "fl_trace.h"
#include "fl_common.cuh"
#include "fl_plan.h"

struct CgScalars {
    double gamma;      // <r, r>
    double alpha, beta;
    double tol;
    float lam;
    float p_scale;     // p16 = p * p_scale
    float p_unscale;   // 1 / p_scale
    float y_scale;     // mixed: scale of the FP16 forward projection (plan y16_scale, or 1)
    float q_unscale;   // mixed: q = q_unscale * (the backprojection of it); else 1
    int mixed;         // the direction is read in FP16
    int done;          // 1 once gamma < tol, or at a breakdown (see status)
    int iter;          // iterations completed
    int status;        // 1: a non-finite gamma or <p, q> (NaN / Inf in b, u0 or A) stopped it
    unsigned ticket;   // last-block detection for the fused reductions
};

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block sum -> partials[blockIdx.x]; returns true in the block that arrives
// last, after which `total` holds the sum of all partials (fixed order, so the
// result is the same on every run).
__device__ bool grid_sum(double v, double* partials, unsigned* ticket, double& total)
{
    __shared__ double sw[kThreads / 32];
    __shared__ bool last;
    v = warp_sum(v);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sw[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int k = 0; k < kThreads / 32; k++) b += sw[k];
        partials[blockIdx.x] = b;
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += kThreads) s += ((volatile double*)partials)[k];
    s = warp_sum(s);
    if (lane == 0) sw[w] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kThreads / 32; k++) t += sw[k];
        total = t;
        *ticket = 0u;
    }
    return true;
}

__global__ void __launch_bounds__(kThreads)
k_dot(const float* __restrict__ a, const float* __restrict__ b, long long n,
      double* __restrict__ partials, unsigned* ticket, double* out)
{
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads)
        s += (double)a[i] * (double)b[i];
    double tot;
    if (grid_sum(s, partials, ticket, tot) && threadIdx.x == 0) *out = tot;
}

// y = a*x + b*y (plain driver's building block)
__global__ void k_axpby(float* __restrict__ y, const float* __restrict__ x, float a, float b,
                        long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        y[i] = a * x[i] + b * y[i];
}

// r = q - b (q may be null: r = -b); p = -r; gamma = <r, r>
__global__ void __launch_bounds__(kThreads)
k_cg_init(const float* __restrict__ bvec, const float* __restrict__ q, float* __restrict__ r,
          float* __restrict__ p, long long n, CgScalars* S, double* partials)
{
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        float ri = (q ? q[i] : 0.0f) - bvec[i];
        r[i] = ri;
        p[i] = -ri;
        s += (double)ri * ri;
    }
    double tot;
    if (grid_sum(s, partials, &S->ticket, tot) && threadIdx.x == 0) {
        S->gamma = tot;
        S->done = 0;
        S->iter = 0;
        // a zero residual is already the solution (the reference loop would go
        // on to 0/0); a non-finite one stops with status 1
        if (!isfinite(tot)) { S->done = 1; S->status = 1; }
        else if (tot == 0.0) S->done = 1;
        double rms = sqrt(tot / (double)n);
        S->p_scale = rms > 0 ? (float)(1.0 / (8.0 * rms)) : 1.0f;
        S->p_unscale = 1.0f / S->p_scale;
        S->q_unscale = S->mixed ? S->p_unscale / S->y_scale : 1.0f;
    }
}

// p16 = p * p_scale
__global__ void k_cg_p16(const float* __restrict__ p, __half* __restrict__ p16, long long n,
                         const CgScalars* S)
{
    if (S->done) return;
    float sc = S->p_scale;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        p16[i] = __float2half_rn(p[i] * sc);
}

// q = q_unscale q + lam p ; alpha = gamma / <p, q>  (q_unscale = 1 outside
// the mixed form: the same bits as q + lam p)
__global__ void __launch_bounds__(kThreads)
k_cg_pq(const float* __restrict__ p, float* __restrict__ q, long long n, CgScalars* S,
        double* partials)
{
    if (S->done) return;
    float lam = S->lam, qs = S->q_unscale;
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        float pi = p[i];
        float qi = fmaf(lam, pi, q[i] * qs);
        q[i] = qi;
        s += (double)pi * qi;
    }
    double tot;
    if (grid_sum(s, partials, &S->ticket, tot) && threadIdx.x == 0) {
        const double a = S->gamma / tot;
        if (tot > 0.0 && isfinite(a)) {
            S->alpha = a;
        } else {                       // breakdown: stop before u is touched
            S->done = 1;
            if (!isfinite(tot) || !isfinite(S->gamma)) S->status = 1;
        }
    }
}

// u += alpha p ; r += alpha q ; gamma' = <r, r> ; beta = gamma'/gamma ; stop test
__global__ void __launch_bounds__(kThreads)
k_cg_update(float* __restrict__ u, float* __restrict__ r, const float* __restrict__ p,
            const float* __restrict__ q, long long n, CgScalars* S, double* partials,
            double* hist, int hist_cap)
{
    if (S->done) return;
    float a = (float)S->alpha;
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        u[i] = fmaf(a, p[i], u[i]);
        float ri = fmaf(a, q[i], r[i]);
        r[i] = ri;
        s += (double)ri * ri;
    }
    double tot;
    if (grid_sum(s, partials, &S->ticket, tot) && threadIdx.x == 0) {
        if (!isfinite(tot)) { S->done = 1; S->status = 1; return; }
        S->beta = tot / S->gamma;
        S->gamma = tot;
        if (hist && S->iter < hist_cap) hist[S->iter] = tot;
        S->iter += 1;
        double rms = sqrt(tot / (double)n);
        S->p_scale = rms > 0 ? (float)(1.0 / (8.0 * rms)) : 1.0f;
        S->p_unscale = 1.0f / S->p_scale;
        S->q_unscale = S->mixed ? S->p_unscale / S->y_scale : 1.0f;
        if (tot < S->tol) S->done = 1;
    }
}

// p = -r + beta p ; p16 = p * p_scale (mixed)
__global__ void k_cg_dir(const float* __restrict__ r, float* __restrict__ p,
                         __half* __restrict__ p16, long long n, const CgScalars* S)
{
    if (S->done) return;
    float b = (float)S->beta, sc = S->p_scale;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float pi = fmaf(b, p[i], -r[i]);
        p[i] = pi;
        if (p16) p16[i] = __float2half_rn(pi * sc);
    }
}

// residual refresh: r = q - b, gamma = <r, r> (keeps p, beta)
__global__ void __launch_bounds__(kThreads)
k_cg_refresh(const float* __restrict__ bvec, const float* __restrict__ q, float* __restrict__ r,
             long long n, CgScalars* S, double* partials)
{
    if (S->done) return;
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        float ri = q[i] - bvec[i];
        r[i] = ri;
        s += (double)ri * ri;
    }
    double tot;
    if (grid_sum(s, partials, &S->ticket, tot) && threadIdx.x == 0) {
        S->gamma = tot;
        if (!isfinite(tot)) { S->done = 1; S->status = 1; }
    }
}

int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
            n = 132;
    }
    return n;
}

unsigned grid_for(long long n)
{
    long long want = (n + kThreads - 1) / kThreads;
    long long cap = 4LL * sm_count();
    return (unsigned)(want < cap ? (want > 0 ? want : 1) : cap);
}

}  // namespace

// ---------------------------------------------------------------------------
// Shared scratch for the stand-alone FP64 dot product (per device, grown once)
// ---------------------------------------------------------------------------
namespace {
struct DotScratch {
    double* partials = nullptr;
    unsigned* ticket = nullptr;
    int cap = 0;
};
DotScratch g_dot[64];
}

extern "C" int fl_axpby(float* y, const float* x, float a, float b, int64_t n, void* stream)
{
    if (!y || (!x && a != 0.0f) || n < 0) return fl_set_error(FL_ERR_INVALID, "fl_axpby: bad argument");
    if (n == 0) return fl_set_error(FL_OK, "");
    k_axpby<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(y, x ? x : y, x ? a : 0.0f, b, n);
    int st = fl_check_launch("fl_axpby");
    return st ? st : fl_set_error(FL_OK, "");
}

extern "C" int fl_dot(const float* a, const float* b, int64_t n, double* out, void* stream)
{
    if (!a || !b || !out || n < 0) return fl_set_error(FL_ERR_INVALID, "fl_dot: bad argument");
    int dev = 0;
    FL_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fl_set_error(FL_ERR_UNSUPPORTED, "device index %d", dev);
    DotScratch& d = g_dot[dev];
    unsigned g = grid_for(n);
    if (d.cap < (int)g) {
        if (d.partials) cudaFree(d.partials);
        if (d.ticket) cudaFree(d.ticket);
        d.partials = nullptr; d.ticket = nullptr; d.cap = 0;
        FL_CUDA(fl_malloc((void**)&d.partials, sizeof(double) * 4 * sm_count()));
        FL_CUDA(fl_malloc((void**)&d.ticket, sizeof(unsigned)));
        FL_CUDA(cudaMemset(d.ticket, 0, sizeof(unsigned)));
        d.cap = 4 * sm_count();
    }
    k_dot<<<g, kThreads, 0, (cudaStream_t)stream>>>(a, b, n, d.partials, d.ticket, out);
    return fl_check_launch("fl_dot");
}

// ---------------------------------------------------------------------------
// CGLS workspace
// ---------------------------------------------------------------------------
struct fl_cgls {
    fl_plan* plan;
    int mode;
    long long n, nr;
    float *r, *p, *q, *tmp;     // tmp: sinogram (C^2 W p in the fused drivers)
    __half* p16;
    __half* tmp16;              // mixed form on a cone plan: the FP16 sinogram
    CgScalars* S;
    double* partials;
    double* hist;
    int hist_cap;
    unsigned grid;
    cudaStream_t cs;            // capture/replay stream
    cudaEvent_t ev0, ev1;
    cudaGraphExec_t exec;
    bool captured;
    const float* cap_u;         // pointers baked into the captured graph
    float* cap_uw;
    float *hb, *hu;             // device copies for the host-buffer entry point
    int fold;                   // fused forms on a z-mirror plan: vectors kept z-folded
    int rot;                    // fl_plan_form when the graph was captured
    float *bf, *uf;             // folded copies of b and u
};

static void cgls_free(fl_cgls* c)
{
    void* ptrs[] = {c->r,    c->p,        c->q,    c->tmp, c->p16, c->tmp16, c->S,
                    c->partials, c->hist, c->hb, c->hu,  c->bf,  c->uf};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    if (c->exec) cudaGraphExecDestroy(c->exec);
    if (c->cs) cudaStreamDestroy(c->cs);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
}

extern "C" int fl_cgls_create(fl_plan* plan, int mode, fl_cgls** out)
{
    FL_RANGE("fl_cgls_create");
    if (!plan || !out) return fl_set_error(FL_ERR_INVALID, "fl_cgls_create: null argument");
    if (mode != FL_CGLS_PLAIN && mode != FL_CGLS_MIXED && mode != FL_CGLS_GRAPH)
        return fl_set_error(FL_ERR_INVALID, "unknown CGLS mode %d", mode);
    int st = fl_matched_ready(plan);
    if (st) return st;
    *out = nullptr;
    fl_cgls* c = new (std::nothrow) fl_cgls;
    if (!c) return fl_set_error(FL_ERR_ALLOC, "out of host memory");
    std::memset((void*)c, 0, sizeof *c);
    c->plan = plan; c->mode = mode;
    c->n = plan->n_vox; c->nr = plan->n_rays;
    c->grid = grid_for(c->n);
    c->hist_cap = 4096;
    auto M = [&](void** ptr, size_t bytes) {
        return st ? st : (st = fl_check_cuda(fl_malloc(ptr, bytes), "fl_malloc(cgls)"));
    };
    M((void**)&c->r, c->n * 4); M((void**)&c->p, c->n * 4); M((void**)&c->q, c->n * 4);
    M((void**)&c->tmp, c->nr * 4);
    if (mode == FL_CGLS_MIXED) M((void**)&c->p16, c->n * 2);
    if (mode == FL_CGLS_MIXED && plan->s.ndim == 3) M((void**)&c->tmp16, c->nr * 2);
    // the fused forms keep every vector z-folded on a z-mirror plan (the
    // algebra is elementwise, so only b in and u out change layout); whether
    // the plan uses the mirror is read again at every solve
    c->fold = (plan->zmirror && mode != FL_CGLS_PLAIN) ? 1 : 0;
    c->rot = fl_plan_form(plan);
    if (c->fold) { M((void**)&c->bf, c->n * 4); M((void**)&c->uf, c->n * 4); }
    M((void**)&c->S, sizeof(CgScalars));
    M((void**)&c->partials, sizeof(double) * c->grid);
    M((void**)&c->hist, sizeof(double) * c->hist_cap);
    if (!st) st = fl_check_cuda(cudaMemset(c->S, 0, sizeof(CgScalars)), "cudaMemset");
    if (!st) st = fl_check_cuda(cudaStreamCreateWithFlags(&c->cs, cudaStreamNonBlocking), "stream");
    if (!st) st = fl_check_cuda(cudaEventCreateWithFlags(&c->ev0, cudaEventDisableTiming), "event");
    if (!st) st = fl_check_cuda(cudaEventCreateWithFlags(&c->ev1, cudaEventDisableTiming), "event");
    if (st) { cgls_free(c); delete c; return st; }
    *out = c;
    return fl_set_error(FL_OK, "");
}

extern "C" void fl_cgls_destroy(fl_cgls* c)
{
    if (!c) return;
    cgls_free(c);
    delete c;
}

// q = (A^T A + lam I) x with FP32 storage (matched model); x and q in the
// workspace's vector layout
static int normal_apply(fl_cgls* c, const float* x, float* q, float lam, cudaStream_t s)
{
    fl_plan* P = c->plan;
    const int lay = c->fold ? FL_LAY_X_FOLDED : 0;
    int st;
    if ((st = fl_matched_forward(P, x, FL_F32, c->tmp, FL_F32, 2, nullptr, nullptr,
                                 lay | FL_LAY_Y_ADJ, s)))
        return st;
    if ((st = fl_matched_adjoint_w(P, c->tmp, q, FL_F32, nullptr, lay, s))) return st;
    if (lam != 0.0f) {
        k_axpby<<<c->grid, kThreads, 0, s>>>(q, x, lam, 1.0f, c->n);
        if ((st = fl_check_launch("normal_apply"))) return st;
    }
    return FL_OK;
}

extern "C" int fl_normal_apply(fl_plan* plan, const float* x, float* q, float lam, void* stream)
{
    FL_RANGE("fl_normal_apply");
    if (!plan || !x || !q) return fl_set_error(FL_ERR_INVALID, "fl_normal_apply: null argument");
    int st = fl_matched_ready(plan);
    if (st) return st;
    float* w;
    if ((st = fl_plan_work(plan, &w))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if ((st = fl_matched_forward(plan, x, FL_F32, w, FL_F32, 2, nullptr, nullptr, FL_LAY_Y_ADJ,
                                 s)))
        return st;
    if ((st = fl_matched_adjoint_w(plan, w, q, FL_F32, nullptr, 0, s))) return st;
    if (lam != 0.0f) {
        k_axpby<<<grid_for(plan->n_vox), kThreads, 0, s>>>(q, x, lam, 1.0f, plan->n_vox);
        return fl_check_launch("fl_normal_apply");
    }
    return FL_OK;
}

static int plain_dot(fl_cgls* c, const float* a, const float* b, double* host, cudaStream_t s)
{
    int st = fl_dot(a, b, c->n, &c->S->alpha, s);   // S->alpha used as a scratch slot
    if (st) return st;
    FL_CUDA(cudaMemcpyAsync(host, &c->S->alpha, sizeof(double), cudaMemcpyDeviceToHost, s));
    return fl_check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}

static int nonfinite(int it, int* done_iters)
{
    if (done_iters) *done_iters = it;
    return fl_set_error(FL_ERR_NUMERIC,
                        "fl_cgls_solve: non-finite residual or curvature after %d iterations "
                        "(NaN or Inf in b, u0 or the operator)", it);
}

static int solve_plain(fl_cgls* c, const float* b, float* u, float lam, int iters, double tol,
                       int flags, double* hist, int* done_iters, cudaStream_t s)
{
    const long long n = c->n;
    const unsigned g = c->grid;
    int st;
    // r = A_loc(u0) - b ; p = -r
    if (!(flags & FL_CGLS_ZERO_START)) {
        if ((st = normal_apply(c, u, c->q, lam, s))) return st;
        FL_CUDA(cudaMemcpyAsync(c->r, c->q, n * 4, cudaMemcpyDeviceToDevice, s));
        k_axpby<<<g, kThreads, 0, s>>>(c->r, b, -1.0f, 1.0f, n);
    } else {
        FL_CUDA(cudaMemsetAsync(c->r, 0, n * 4, s));
        k_axpby<<<g, kThreads, 0, s>>>(c->r, b, -1.0f, 1.0f, n);
    }
    FL_CUDA(cudaMemsetAsync(c->p, 0, n * 4, s));
    k_axpby<<<g, kThreads, 0, s>>>(c->p, c->r, -1.0f, 0.0f, n);
    if ((st = fl_check_launch("cgls init"))) return st;
    double gamma;
    if ((st = plain_dot(c, c->r, c->r, &gamma, s))) return st;
    int it = 0;
    if (!std::isfinite(gamma)) return nonfinite(0, done_iters);
    if (gamma == 0.0) iters = 0;                 // u0 already solves it
    while (it < iters) {
        if ((st = normal_apply(c, c->p, c->q, lam, s))) return st;
        double pq;
        if ((st = plain_dot(c, c->p, c->q, &pq, s))) return st;
        if (!std::isfinite(pq)) return nonfinite(it, done_iters);
        if (!(pq > 0.0)) break;                  // breakdown: stop before u is touched
        it++;
        float alpha = (float)(gamma / pq);
        k_axpby<<<g, kThreads, 0, s>>>(u, c->p, alpha, 1.0f, n);
        k_axpby<<<g, kThreads, 0, s>>>(c->r, c->q, alpha, 1.0f, n);
        double gnew;
        if ((st = plain_dot(c, c->r, c->r, &gnew, s))) return st;
        if (!std::isfinite(gnew)) return nonfinite(it, done_iters);
        float beta = (float)(gnew / gamma);
        k_axpby<<<g, kThreads, 0, s>>>(c->p, c->r, -1.0f, beta, n);
        if ((st = fl_check_launch("cgls iteration"))) return st;
        gamma = gnew;
        if (hist) hist[it - 1] = gnew;
        if (gamma < tol) break;
    }
    if (done_iters) *done_iters = it;
    return FL_OK;
}

// one fused iteration: fwd(p or p16) -> tmp -> adj -> q ; fused updates
static int mixed_iteration(fl_cgls* c, float* u, cudaStream_t s)
{
    fl_plan* P = c->plan;
    CgScalars* S = c->S;
    const int lay = c->fold ? FL_LAY_X_FOLDED : 0;
    int st;
    if (c->p16) {
        // y = y_scale C^2 W p16 (FP16 on a cone plan), q' = W^T y; k_cg_pq
        // rescales q' by p_unscale / y_scale
        void* y = c->tmp16 ? (void*)c->tmp16 : (void*)c->tmp;
        const int yt = c->tmp16 ? FL_F16 : FL_F32;
        st = fl_matched_forward(P, c->p16, FL_F16, y, yt, 2, &S->done, &S->y_scale,
                                lay | FL_LAY_Y_ADJ, s);
        if (st) return st;
        st = fl_matched_adjoint_wt(P, y, yt, c->q, FL_F32, &S->done, lay, s);
    } else {
        st = fl_matched_forward(P, c->p, FL_F32, c->tmp, FL_F32, 2, &S->done, nullptr,
                                lay | FL_LAY_Y_ADJ, s);
        if (st) return st;
        st = fl_matched_adjoint_w(P, c->tmp, c->q, FL_F32, &S->done, lay, s);
    }
    if (st) return st;
    k_cg_pq<<<c->grid, kThreads, 0, s>>>(c->p, c->q, c->n, S, c->partials);
    k_cg_update<<<c->grid, kThreads, 0, s>>>(u, c->r, c->p, c->q, c->n, S, c->partials, c->hist,
                                             c->hist_cap);
    k_cg_dir<<<c->grid, kThreads, 0, s>>>(c->r, c->p, c->p16, c->n, S);
    return fl_check_launch("cgls mixed iteration");
}

static int solve_mixed(fl_cgls* c, const float* b, float* u, float lam, int iters, double tol,
                       int refresh, int flags, double* hist, int* done_iters, cudaStream_t us)
{
    cudaStream_t s = c->cs;
    int st;
    // layout of the workspace vectors follows the plan's current mirror option
    const int fold = c->plan->zmirror ? 1 : 0;
    if (fold && (!c->bf || !c->uf)) {        // both folded copies, or neither
        int e = c->bf ? FL_OK : fl_check_cuda(fl_malloc((void**)&c->bf, c->n * 4), "fl_malloc(cgls)");
        if (!e && !c->uf) e = fl_check_cuda(fl_malloc((void**)&c->uf, c->n * 4), "fl_malloc(cgls)");
        if (e) {
            if (c->bf) cudaFree(c->bf);
            if (c->uf) cudaFree(c->uf);
            c->bf = c->uf = nullptr;
            return e;
        }
    }
    if (fold != c->fold) { c->fold = fold; c->captured = false; }
    const int rot = fl_plan_form(c->plan);                // kernels in the graph
    if (rot != c->rot) { c->rot = rot; c->captured = false; }
    FL_CUDA(cudaEventRecord(c->ev0, us));
    FL_CUDA(cudaStreamWaitEvent(s, c->ev0, 0));
    CgScalars init;
    std::memset(&init, 0, sizeof init);
    init.tol = tol; init.lam = lam;
    init.mixed = c->p16 ? 1 : 0;
    init.y_scale = c->tmp16 ? c->plan->y16_scale : 1.0f;
    init.q_unscale = 1.0f;
    FL_CUDA(cudaMemcpyAsync(c->S, &init, sizeof init, cudaMemcpyHostToDevice, s));
    // the user's b and u (standard layout) or their z-folded copies
    const float* bb = b;
    float* uu = u;
    if (c->fold) {
        if ((st = fl_matched_fold(c->plan, b, c->bf, FL_F32, 0, s))) return st;
        if (flags & FL_CGLS_ZERO_START)
            FL_CUDA(cudaMemsetAsync(c->uf, 0, c->n * 4, s));
        else if ((st = fl_matched_fold(c->plan, u, c->uf, FL_F32, 0, s)))
            return st;
        bb = c->bf;
        uu = c->uf;
    }
    const float* q0 = nullptr;
    if (!(flags & FL_CGLS_ZERO_START)) {
        if ((st = normal_apply(c, uu, c->q, lam, s))) return st;
        q0 = c->q;
    }
    k_cg_init<<<c->grid, kThreads, 0, s>>>(bb, q0, c->r, c->p, c->n, c->S, c->partials);
    if (c->p16) k_cg_p16<<<c->grid, kThreads, 0, s>>>(c->p, c->p16, c->n, c->S);
    if ((st = fl_check_launch("cgls mixed init"))) return st;

    if (!c->captured || c->cap_uw != uu) {
        if (c->exec) { cudaGraphExecDestroy(c->exec); c->exec = nullptr; }
        cudaGraph_t g;
        FL_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int cst = mixed_iteration(c, uu, s);
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (cst) return cst;
        FL_CUDA(e);
        e = cudaGraphInstantiate(&c->exec, g, 0);
        cudaGraphDestroy(g);
        FL_CUDA(e);
        c->captured = true;
        c->cap_uw = uu;
    }
    for (int it = 0; it < iters; it++) {
        FL_CUDA(cudaGraphLaunch(c->exec, s));
        if (c->p16 && refresh > 0 && (it + 1) % refresh == 0 && it + 1 < iters) {
            if ((st = normal_apply(c, uu, c->q, lam, s))) return st;
            k_cg_refresh<<<c->grid, kThreads, 0, s>>>(bb, c->q, c->r, c->n, c->S, c->partials);
            if ((st = fl_check_launch("cgls refresh"))) return st;
        }
    }
    if (c->fold && (st = fl_matched_fold(c->plan, c->uf, u, FL_F32, 1, s))) return st;
    CgScalars fin;
    FL_CUDA(cudaMemcpyAsync(&fin, c->S, sizeof fin, cudaMemcpyDeviceToHost, s));
    std::vector<double> h(c->hist_cap);
    int nh = iters < c->hist_cap ? iters : c->hist_cap;
    if (hist && nh > 0)
        FL_CUDA(cudaMemcpyAsync(h.data(), c->hist, sizeof(double) * nh, cudaMemcpyDeviceToHost, s));
    FL_CUDA(cudaEventRecord(c->ev1, s));
    FL_CUDA(cudaStreamWaitEvent(us, c->ev1, 0));
    FL_CUDA(cudaStreamSynchronize(s));
    if (hist) for (int k = 0; k < nh && k < fin.iter; k++) hist[k] = h[k];
    if (done_iters) *done_iters = fin.iter;
    if (fin.status) return nonfinite(fin.iter, done_iters);
    return FL_OK;
}

extern "C" int fl_cgls_solve(fl_cgls* c, const float* b, float* u, float lam, int iters,
                             double tol, int refresh, int flags, double* gamma_history,
                             int* iters_done, void* stream)
{
    FL_RANGE("fl_cgls_solve");
    if (!c || !b || !u || iters < 0)
        return fl_set_error(FL_ERR_INVALID, "fl_cgls_solve: bad argument");
    int st = (c->mode == FL_CGLS_PLAIN)
                 ? solve_plain(c, b, u, lam, iters, tol, flags, gamma_history, iters_done,
                               (cudaStream_t)stream)
                 : solve_mixed(c, b, u, lam, iters, tol, refresh, flags, gamma_history, iters_done,
                               (cudaStream_t)stream);
    if (!st || st == FL_ERR_NUMERIC) {   // a forward's TMA wait gave up: the cause of any NaN
        const int t = fl_plan_take_timeouts(c->plan, (cudaStream_t)stream);
        if (t) return t;
    }
    if (st) return st;
    return fl_set_error(FL_OK, "");
}

// The device's address of a host buffer it can reach (pinned by
// cudaHostAlloc or registered by cudaHostRegister), or null (pageable memory,
// device memory, or a failed query).
static void* host_view(const void* h)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

extern "C" int fl_cgls_solve_host(fl_cgls* c, const float* b_host, float* u_host, float lam,
                                  int iters, double tol, int refresh, int flags,
                                  double* gamma_history, int* iters_done, void* stream)
{
    FL_RANGE("fl_cgls_solve_host");
    if (!c || !b_host || !u_host || iters < 0)
        return fl_set_error(FL_ERR_INVALID, "fl_cgls_solve_host: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    // A z-folded workspace in the graph or mixed form touches b and u once
    // each: the fold reads b (and u0), the unfold writes u. Where both host
    // buffers are pinned or registered, those passes read and write them in
    // place over the host link and nothing is staged. (A copy-engine transfer
    // of a 512^3 volume from pinned memory was measured to slow the projector
    // kernels that run after it by 4-5 % for seconds; reads and writes by the
    // fold kernels leave them at full speed.) Otherwise b and u are copied.
    if (c->mode != FL_CGLS_PLAIN && c->plan->zmirror) {
        const float* bd = static_cast<const float*>(host_view(b_host));
        float* ud = static_cast<float*>(host_view(u_host));
        if (bd && ud) {
            int st = fl_cgls_solve(c, bd, ud, lam, iters, tol, refresh, flags, gamma_history,
                                   iters_done, stream);
            if (st) return st;
            return fl_check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        }
    }
    size_t bytes = (size_t)c->n * sizeof(float);
    if (!c->hb) FL_CUDA(fl_malloc((void**)&c->hb, bytes));
    if (!c->hu) FL_CUDA(fl_malloc((void**)&c->hu, bytes));
    FL_CUDA(cudaMemcpyAsync(c->hb, b_host, bytes, cudaMemcpyHostToDevice, s));
    if (!(flags & FL_CGLS_ZERO_START))
        FL_CUDA(cudaMemcpyAsync(c->hu, u_host, bytes, cudaMemcpyHostToDevice, s));
    else
        FL_CUDA(cudaMemsetAsync(c->hu, 0, bytes, s));
    int st = fl_cgls_solve(c, c->hb, c->hu, lam, iters, tol, refresh, flags, gamma_history,
                           iters_done, stream);
    if (st) return st;
    FL_CUDA(cudaMemcpyAsync(u_host, c->hu, bytes, cudaMemcpyDeviceToHost, s));
    return fl_check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}
