// batch.cu -- many independent fan-beam scans of different sizes (slices with
// their own nx, ny, detector and view count) projected and solved together.
//
// The slices' matched-model tables stay where their plans put them; a batch
// holds one descriptor per slice and three work lists:
//  * rays:   chunks of 128 consecutive rays of one slice (forward, weighting),
//  * pixels: chunks of 2 image rows x 256 columns of one slice (adjoint),
//  * vector: chunks of kVecChunk elements of one slice's image (CGLS algebra).
// Each operator is ONE launch over its list, whatever the mix of sizes; the ray
// and pixel lists are ordered by decreasing per-item cost (walk length, view
// count) so the largest slices start first and the tail is made of the
// cheapest chunks. The forward and adjoint are the matched model of the
// single-scan kernels (the same device code, matched_dev.cuh), so each slice's
// result is bit-identical to its own plan's. A slice whose plan uses the half
// or quarter turn (fl_plan_turns when the batch is created) goes through the
// plan's turn kernels instead, on two more lists (32 rays of the views
// iv < nv/G; 32 primary pixels); its adjoint input is packed per orbit, as
// the plan's. So does a slice whose plan uses a reflection form (with or
// without a turn): walked rays and primary pixels of that form.
//
// CGLS (solveCGLS.m:6-31) runs per slice, all slices in lockstep: every slice
// has its own FP64 gamma/alpha/beta and stop flag, the inner products are
// segmented by slice (per-chunk FP64 partials; the last chunk of a slice to
// finish sums that slice's partials in a fixed order, so results do not depend
// on scheduling). One iteration = 3 launches (q += lam p with <p,q>, updates
// with <r,r>, direction) plus a forward with c_r^2 and an adjoint for each
// kind of slice present (general, turn, reflection; parallel branches) and
// the transposed copy of the direction the forwards read, captured once as a
// CUDA graph and replayed.
// A stopped slice's chunks return at once.
#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "fl_trace.h"
#include "fl_common.cuh"
#include "fl_plan.h"
#include "matched_dev.cuh"

namespace {

constexpr int kRayChunk = 128;
constexpr int kPixChunk = 128;
constexpr int kVecThreads = 256;
constexpr int kVecChunk = kVecThreads * 16;

struct BatchSlice {
    const ColEntry* col;
    const float* colr;
    const ViewEntry* view;
    const int* views;      // the frame's view list (id_Y column 0)
    int nvf;               // its length (Nv[0])
    DetGrid G;
    int nx, ny, na, nv;
    int turns;             // fl_plan_turns of the slice's plan at batch creation
    int refl;              // fl_plan_refl of it (1, 2, 4: a fan reflection form; 0: none)
    int pblk;              // its backprojection's pixel block side (fan_refl_pblock)
    int lanes;             // parts per walked ray (fl_plan_fan_lanes of the slice's plan)
    float scale;
    long long xoff, yoff;  // offsets of the slice in the concatenated image / sinogram
    long long woff;        // its offset in the batch's sinogram scratch (a multiple of
                           // 4 floats: turn slices' packed orbits are read as vectors)
    int vc0, vc1;          // its vector chunks [vc0, vc1)
};

struct BatchScal {
    double gamma, alpha, beta;
    int done, iter;
    int status;            // 1: stopped by a non-finite gamma or <p, q>
};

struct VecChunk {
    int slice, start, len, pad;
};

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block sum of v into partials[blockIdx.x]; returns true in the last block of
// the slice to arrive, where `total` is then the slice's sum over its chunks
// [c0, c1) in a fixed order.
__device__ bool slice_sum(double v, int slice, int c0, int c1, double* partials,
                          unsigned* tickets, double& total)
{
    __shared__ double sw[kVecThreads / 32];
    __shared__ bool last;
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sw[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int k = 0; k < kVecThreads / 32; k++) b += sw[k];
        partials[blockIdx.x] = b;
        __threadfence();
        unsigned t = atomicAdd(tickets + slice, 1u);
        last = (t == (unsigned)(c1 - c0 - 1));
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s = 0.0;
    for (int k = c0 + threadIdx.x; k < c1; k += kVecThreads) s += ((volatile double*)partials)[k];
    s = warp_sum(s);
    if (lane == 0) sw[w] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kVecThreads / 32; k++) t += sw[k];
        total = t;
        tickets[slice] = 0u;
    }
    return true;
}

// y = c_r^cr_power * (sum of w x along each ray), one block per ray chunk
__global__ void __launch_bounds__(kRayChunk, 8)
k_batch_fwd(const float* __restrict__ X, const float* __restrict__ XT, float* __restrict__ Y,
            const BatchSlice* __restrict__ sl, const int2* __restrict__ chunks, int cr_power,
            int scratch, const BatchScal* __restrict__ S)
{
    const int2 ch = chunks[blockIdx.x];
    if (S && S[ch.x].done) return;
    const BatchSlice& b = sl[ch.x];
    const int r = ch.y + threadIdx.x;
    if (r >= b.na * b.nv) return;
    float a1[1];
    walk_fan<float, 1>(X + b.xoff, XT + b.xoff, &b.col[r].x, &b.col[r].y, b.nx, b.ny, a1,
                       (long long)b.nx * b.ny);
    const float acc = a1[0];
    float cr = ray_cr(b.scale, b.colr[r], 0.0f);
    float out = cr * acc;
    if (cr_power == 2) out = cr * out;
    Y[(scratch ? b.woff : b.yoff) + r] = out;
}

// Turn slices: the plan's turn forward, one block of kFanBlock threads per
// chunk (slice, r0) of the rays iv < nv/G (kFanBlock / lanes rays). ypack:
// into the batch's scratch (woff), packed per orbit; else the standard
// layout at yoff.
__global__ void __launch_bounds__(kFanBlock, 3)
k_batch_fwd_turn(const float* __restrict__ X, const float* __restrict__ XT, float* __restrict__ Y,
                 const BatchSlice* __restrict__ sl, const int2* __restrict__ chunks,
                 int cr_power, int ypack, const BatchScal* __restrict__ S)
{
    const int2 ch = chunks[blockIdx.x];
    if (S && S[ch.x].done) return;            // uniform in the block
    const BatchSlice& b = sl[ch.x];
    float* y = Y + (ypack ? b.woff : b.yoff);
    if (b.turns == 4)
        fan_turn_forward_block<float, float, 4>(X + b.xoff, XT + b.xoff, y, b.col, b.colr, b.nx,
                                                b.ny, b.na, b.nv, b.scale, cr_power, nullptr,
                                                ypack, ch.y, b.lanes);
    else
        fan_turn_forward_block<float, float, 2>(X + b.xoff, XT + b.xoff, y, b.col, b.colr, b.nx,
                                                b.ny, b.na, b.nv, b.scale, cr_power, nullptr,
                                                ypack, ch.y, b.lanes);
}

// Transposed copy of every slice's image (XT[xoff + x ny + y] = X[xoff + y nx
// + x]) over the vector chunks, for the forwards (walk_fan).
__global__ void __launch_bounds__(kVecThreads)
k_batch_transpose(const float* __restrict__ X, float* __restrict__ XT,
                  const BatchSlice* __restrict__ sl, const VecChunk* __restrict__ chunks)
{
    const VecChunk ch = chunks[blockIdx.x];
    const BatchSlice& b = sl[ch.slice];
    for (int k = threadIdx.x; k < ch.len; k += kVecThreads) {
        const int i = ch.start + k, iy = i / b.nx, ix = i - iy * b.nx;
        XT[b.xoff + (long long)ix * b.ny + iy] = X[b.xoff + i];
    }
}

// Reflection slices: the plan's reflection forward (fan_refl_forward_block),
// one block of kFanBlock threads per chunk (slice, r0) of the walked rays
// (slots x columns of FanReflGeom; kFanBlock / lanes rays). ypack as above.
__global__ void __launch_bounds__(kFanBlock, 3)
k_batch_fwd_refl(const float* __restrict__ X, const float* __restrict__ XT, float* __restrict__ Y,
                 const BatchSlice* __restrict__ sl, const int2* __restrict__ chunks,
                 int cr_power, int ypack, const BatchScal* __restrict__ S)
{
    const int2 ch = chunks[blockIdx.x];
    if (S && S[ch.x].done) return;            // uniform in the block
    const BatchSlice& b = sl[ch.x];
    float* y = Y + (ypack ? b.woff : b.yoff);
#define FL_BATCH_REFL(NN)                                                                      \
    fan_refl_forward_block<float, float, NN>(X + b.xoff, XT + b.xoff, y, b.col, b.colr, b.nx,    \
                                             b.ny, b.na, b.nv, b.scale, cr_power, nullptr, ypack, \
                                             ch.y, b.lanes)
    if (b.refl == 4) FL_BATCH_REFL(4);
    else if (b.refl == 2) FL_BATCH_REFL(2);
    else FL_BATCH_REFL(1);
#undef FL_BATCH_REFL
}

// yw = c_r * y over the ray chunks of all slices (input of the stand-alone
// adjoint, in the batch's scratch); a turn slice's yw is packed per orbit
// with c_r of view iv < nv/G (the single plan's k_weight_fan_packed values)
__global__ void __launch_bounds__(kRayChunk)
k_batch_weight(float* __restrict__ YW, const float* __restrict__ Y,
               const BatchSlice* __restrict__ sl, const int2* __restrict__ chunks)
{
    const int2 ch = chunks[blockIdx.x];
    const BatchSlice& b = sl[ch.x];
    const int r = ch.y + threadIdx.x;
    if (r >= b.na * b.nv) return;
    if (b.refl) {                             // r: a walked ray (slot, column)
        const int NR = b.refl;
        const FanReflGeom g = fan_refl_geom(NR, b.nv, b.na);
        const int s = r / b.na, ia = r - s * b.na;
        int v, vt, a, stride;
        long long off;
        if (s >= g.slots || !refl_slot(g, s, ia, v, vt, a, off, stride)) return;
        const float cr = ray_cr(b.scale, b.colr[(long long)vt * b.na + a], 0.0f);
        for (int k = 0; k < 2 * NR; k++) {
            long long vk; int ak;
            if (NR == 4) refl_image<4>(k, v, a, b.na, b.nv, vk, ak);
            else if (NR == 2) refl_image<2>(k, v, a, b.na, b.nv, vk, ak);
            else refl_image<1>(k, v, a, b.na, b.nv, vk, ak);
            YW[b.woff + off + (long long)(2 * NR) * ia + k] = cr * Y[b.yoff + vk * b.na + ak];
        }
        return;
    }
    if (b.turns > 1) {
        const int gv = b.nv / b.turns, iv = r / b.na, ia = r - iv * b.na;
        const int rp = (iv % gv) * b.na + ia;
        const float cr = ray_cr(b.scale, b.colr[rp], 0.0f);
        YW[b.woff + (long long)b.turns * rp + iv / gv] = cr * Y[b.yoff + r];
        return;
    }
    float cr = ray_cr(b.scale, b.colr[r], 0.0f);
    YW[b.woff + r] = cr * Y[b.yoff + r];
}

// Turn slices: the plan's turn backprojection, one block of 32 blocks of 2 x 2
// primary pixels x kTurnGroups view groups per chunk (slice, iy0, ix0).
__global__ void __launch_bounds__(kFanX * kTurnGroups)
k_batch_adj_turn(float* __restrict__ X, const float* __restrict__ YW,
                 const BatchSlice* __restrict__ sl, const int4* __restrict__ chunks,
                 const BatchScal* __restrict__ S)
{
    const int4 ch = chunks[blockIdx.x];       // (slice, iy, ix0, -)
    if (S && S[ch.x].done) return;            // uniform in the block
    const BatchSlice& b = sl[ch.x];
    if (b.turns == 4)
        fan_turn_adjoint_block<float, 4, 2>(X + b.xoff, YW + b.woff, b.col, b.view, b.G, b.nx,
                                            b.ny, b.na, b.nv, ch.z, ch.y);
    else
        fan_turn_adjoint_block<float, 2, 2>(X + b.xoff, YW + b.woff, b.col, b.view, b.G, b.nx,
                                            b.ny, b.na, b.nv, ch.z, ch.y);
}

// Reflection slices: the plan's reflection backprojection, one block of
// kFanX primary pixel blocks of one block row x kTurnGroups view groups per
// chunk (slice, block row, first block column).
__global__ void __launch_bounds__(kFanX * kTurnGroups, 3)
k_batch_adj_refl(float* __restrict__ X, const float* __restrict__ YW,
                 const BatchSlice* __restrict__ sl, const int4* __restrict__ chunks,
                 const BatchScal* __restrict__ S)
{
    const int4 ch = chunks[blockIdx.x];       // (slice, iy, ix0, -)
    if (S && S[ch.x].done) return;            // uniform in the block
    const BatchSlice& b = sl[ch.x];
    __shared__ float smem[kFanReflShared];
#define FL_BATCH_ADJ_REFL(NN, PP)                                                              \
    fan_refl_adjoint_block<float, NN, PP>(X + b.xoff, YW + b.woff, b.col, b.view, b.G, b.nx, b.ny, \
                                          b.na, b.nv, ch.z, ch.y, smem)
    if (b.refl == 4 && b.pblk == 2) FL_BATCH_ADJ_REFL(4, 2);
    else if (b.refl == 4) FL_BATCH_ADJ_REFL(4, 1);
    else if (b.refl == 2 && b.pblk == 2) FL_BATCH_ADJ_REFL(2, 2);
    else if (b.refl == 2) FL_BATCH_ADJ_REFL(2, 1);
    else if (b.pblk == 2) FL_BATCH_ADJ_REFL(1, 2);
    else FL_BATCH_ADJ_REFL(1, 1);
#undef FL_BATCH_ADJ_REFL
}

// x = A^T (pre-weighted yw), one block per chunk of 2 image rows x
// 2*kPixChunk columns, one thread per 2 x 2 pixel block (all view groups in
// the thread: the single-scan kernel's bits)
__global__ void __launch_bounds__(kPixChunk)
k_batch_adj(float* __restrict__ X, const float* __restrict__ YW,
            const BatchSlice* __restrict__ sl, const int4* __restrict__ chunks,
            const BatchScal* __restrict__ S)
{
    const int4 ch = chunks[blockIdx.x];       // (slice, iy0, ix0, -)
    if (S && S[ch.x].done) return;
    const BatchSlice& b = sl[ch.x];
    const int ix0 = ch.z + 2 * threadIdx.x, iy0 = ch.y;
    if (ix0 >= b.nx) return;
    float acc[2][2];
    fan_block_gather_all<2, 2>(acc, YW + b.woff, b.col, b.view, b.views, b.nvf, b.G, ix0, iy0,
                               b.nx, b.ny, b.na);
    float* xs = X + b.xoff;
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
        for (int i = 0; i < 2; i++)
            if (iy0 + j < b.ny && ix0 + i < b.nx)
                xs[(long long)(iy0 + j) * b.nx + ix0 + i] = acc[j][i];
}

// r = q + lam u - b (q null: r = -b) ; p = -r ; gamma = <r, r>
__global__ void __launch_bounds__(kVecThreads)
k_batch_init(const float* __restrict__ bvec, const float* __restrict__ q,
             const float* __restrict__ u, float lam, float* __restrict__ r,
             float* __restrict__ p, const BatchSlice* __restrict__ sl,
             const VecChunk* __restrict__ vc, BatchScal* S, double* partials,
             unsigned* tickets)
{
    const VecChunk c = vc[blockIdx.x];
    const BatchSlice& b = sl[c.slice];
    const long long o = b.xoff + c.start;
    double s = 0.0;
    for (int k = threadIdx.x; k < c.len; k += kVecThreads) {
        const long long i = o + k;
        float ri = q ? fmaf(lam, u[i], q[i]) - bvec[i] : -bvec[i];
        r[i] = ri;
        p[i] = -ri;
        s += (double)ri * ri;
    }
    double tot;
    if (slice_sum(s, c.slice, b.vc0, b.vc1, partials, tickets, tot) && threadIdx.x == 0) {
        BatchScal& z = S[c.slice];
        z.gamma = tot; z.alpha = 0.0; z.beta = 0.0; z.iter = 0;
        z.done = 0; z.status = 0;
        if (!isfinite(tot)) { z.done = 1; z.status = 1; }
    }
}

// q += lam p ; alpha = gamma / <p, q>  (a slice whose <p, q> is zero stops)
__global__ void __launch_bounds__(kVecThreads)
k_batch_pq(const float* __restrict__ p, float* __restrict__ q, float lam,
           const BatchSlice* __restrict__ sl, const VecChunk* __restrict__ vc, BatchScal* S,
           double* partials, unsigned* tickets)
{
    const VecChunk c = vc[blockIdx.x];
    if (S[c.slice].done) return;
    const BatchSlice& b = sl[c.slice];
    const long long o = b.xoff + c.start;
    double s = 0.0;
    for (int k = threadIdx.x; k < c.len; k += kVecThreads) {
        const long long i = o + k;
        float pi = p[i];
        float qi = fmaf(lam, pi, q[i]);
        q[i] = qi;
        s += (double)pi * qi;
    }
    double tot;
    if (slice_sum(s, c.slice, b.vc0, b.vc1, partials, tickets, tot) && threadIdx.x == 0) {
        BatchScal& z = S[c.slice];
        const double a = z.gamma / tot;
        if (tot > 0.0 && isfinite(a)) {
            z.alpha = a;
        } else {
            z.alpha = 0.0; z.done = 1;
            if (!isfinite(tot) || !isfinite(z.gamma)) z.status = 1;
        }
    }
}

// u += alpha p ; r += alpha q ; gamma' = <r, r> ; beta = gamma'/gamma ; stop test
__global__ void __launch_bounds__(kVecThreads)
k_batch_update(float* __restrict__ u, float* __restrict__ r, const float* __restrict__ p,
               const float* __restrict__ q, double tol, const BatchSlice* __restrict__ sl,
               const VecChunk* __restrict__ vc, BatchScal* S, double* partials,
               unsigned* tickets, double* hist, int hist_cap)
{
    const VecChunk c = vc[blockIdx.x];
    if (S[c.slice].done) return;
    const BatchSlice& b = sl[c.slice];
    const long long o = b.xoff + c.start;
    const float a = (float)S[c.slice].alpha;
    double s = 0.0;
    for (int k = threadIdx.x; k < c.len; k += kVecThreads) {
        const long long i = o + k;
        u[i] = fmaf(a, p[i], u[i]);
        float ri = fmaf(a, q[i], r[i]);
        r[i] = ri;
        s += (double)ri * ri;
    }
    double tot;
    if (slice_sum(s, c.slice, b.vc0, b.vc1, partials, tickets, tot) && threadIdx.x == 0) {
        BatchScal& z = S[c.slice];
        if (!isfinite(tot)) { z.done = 1; z.status = 1; return; }
        z.beta = tot / z.gamma;
        z.gamma = tot;
        if (hist && z.iter < hist_cap) hist[(long long)c.slice * hist_cap + z.iter] = tot;
        z.iter += 1;
        if (tot < tol) z.done = 1;
    }
}

// p = -r + beta p
__global__ void __launch_bounds__(kVecThreads)
k_batch_dir(const float* __restrict__ r, float* __restrict__ p,
            const BatchSlice* __restrict__ sl, const VecChunk* __restrict__ vc,
            const BatchScal* __restrict__ S)
{
    const VecChunk c = vc[blockIdx.x];
    if (S[c.slice].done) return;
    const BatchSlice& b = sl[c.slice];
    const long long o = b.xoff + c.start;
    const float be = (float)S[c.slice].beta;
    for (int k = threadIdx.x; k < c.len; k += kVecThreads) {
        const long long i = o + k;
        p[i] = fmaf(be, p[i], -r[i]);
    }
}

}  // namespace

struct fl_batch {
    int n;
    long long n_vox, n_rays;
    std::vector<long long> xoff, yoff;   // [n + 1]
    BatchSlice* d_sl;
    int2* d_rays;  int n_ray_chunks;       // general slices' rays (forward)
    int2* d_rays_t; int n_ray_t_chunks;    // turn slices' walked rays (forward)
    int2* d_wrays; int n_wray_chunks;      // every slice's rays (weighting)
    int4* d_pix;   int n_pix_chunks;       // general slices' pixel blocks
    int4* d_pix_t; int n_pix_t_chunks;     // turn slices' primary pixels
    int2* d_rays_r; int n_ray_r_chunks;    // reflection slices' walked rays (forward)
    int4* d_pix_r; int n_pix_r_chunks;     // reflection slices' primary pixels
    VecChunk* d_vec; int n_vec_chunks;
    float *r, *p, *q, *tmp;
    float* xt;                         // transposed copies of a forward's input (walk_fan)
    BatchScal* S;
    double* partials;
    unsigned* tickets;
    double* hist;
    int hist_cap;
    cudaStream_t cs;
    cudaEvent_t ev0, ev1;
    cudaStream_t cs2;                  // the turn slices' branch of a forward / adjoint
    cudaEvent_t evf, evj;              // its fork and join
    cudaStream_t cs3;                  // the reflection slices' branch
    cudaEvent_t evf3, evj3;
    cudaGraphExec_t exec;
    float* cap_u;
    float cap_lam;
    double cap_tol;
    std::vector<BatchSlice> h_sl;      // host copy of d_sl
    std::vector<int> by_walk;          // slices, costliest walks first
    int cap_rays_t, cap_rays_r;        // capacities of d_rays_t, d_rays_r (chunks)
};

// Chunks (slice, r0) of the walked rays of the turn slices (refl false) or of
// the reflection slices (refl true), kFanBlock / lanes rays each.
static std::vector<int2> turn_ray_chunks(const std::vector<BatchSlice>& sl,
                                         const std::vector<int>& by_walk, bool refl)
{
    std::vector<int2> rays_t;
    for (int i : by_walk) {
        const BatchSlice& c = sl[i];
        if (c.turns > 1 && (c.refl != 0) == refl) {
            const int walks = c.refl ? c.na * fan_refl_geom(c.refl, c.nv, c.na).slots
                                     : c.na * (c.nv / c.turns);
            for (int r = 0; r < walks; r += kFanBlock / c.lanes) rays_t.push_back(make_int2(i, r));
        }
    }
    return rays_t;
}

static void batch_free(fl_batch* b)
{
    void* ptrs[] = {b->d_sl, b->d_rays, b->d_rays_t, b->d_wrays, b->d_pix, b->d_pix_t, b->d_vec,
                    b->d_rays_r, b->d_pix_r,
                    b->r, b->p, b->q, b->tmp, b->xt, b->S, b->partials, b->tickets, b->hist};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->cs) cudaStreamDestroy(b->cs);
    if (b->cs2) cudaStreamDestroy(b->cs2);
    if (b->evf) cudaEventDestroy(b->evf);
    if (b->evj) cudaEventDestroy(b->evj);
    if (b->cs3) cudaStreamDestroy(b->cs3);
    if (b->evf3) cudaEventDestroy(b->evf3);
    if (b->evj3) cudaEventDestroy(b->evj3);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
}

template <typename T>
static int upload_vec(T** d, const std::vector<T>& h)
{
    FL_CUDA(fl_malloc((void**)d, sizeof(T) * (h.empty() ? 1 : h.size())));
    if (!h.empty()) FL_CUDA(cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
    return FL_OK;
}

extern "C" int fl_batch_create(fl_plan* const* plans, int32_t n_plans, fl_batch** out)
{
    FL_RANGE("fl_batch_create");
    if (!plans || !out || n_plans < 1)
        return fl_set_error(FL_ERR_INVALID, "fl_batch_create: bad argument");
    *out = nullptr;
    std::vector<BatchSlice> sl(n_plans);
    std::vector<long long> xoff(n_plans + 1, 0), yoff(n_plans + 1, 0), woff(n_plans + 1, 0);
    for (int i = 0; i < n_plans; i++) {
        fl_plan* p = plans[i];
        if (!p) return fl_set_error(FL_ERR_INVALID, "fl_batch_create: plan %d is null", i);
        const fl_scan& s = p->s;
        if (s.ndim != 2)
            return fl_set_error(FL_ERR_UNSUPPORTED, "fl_batch_create: plan %d is not fan-beam", i);
        if (s.nt != 1)
            return fl_set_error(FL_ERR_UNSUPPORTED, "fl_batch_create: plan %d has %d frames "
                                "(batched slices are single-frame)", i, s.nt);
        int st = fl_matched_ready(p);
        if (st) return st;
        if (p->det_kind < 0)
            return fl_set_error(FL_ERR_UNSUPPORTED, "fl_batch_create: plan %d needs a uniform "
                                "flat or equiangular detector", i);
        int nvf = 0;
        FL_CUDA(cudaMemcpy(&nvf, p->d_Nv, sizeof(int), cudaMemcpyDeviceToHost));
        if ((long long)s.na * s.nv >= (1LL << 31) || (long long)s.nx * s.ny >= (1LL << 31))
            return fl_set_error(FL_ERR_UNSUPPORTED, "fl_batch_create: plan %d too large", i);
        BatchSlice& b = sl[i];
        std::memset(&b, 0, sizeof b);
        b.col = p->d_col; b.colr = p->d_colr; b.view = p->d_view;
        b.views = p->d_idY; b.nvf = nvf;
        b.G.kind = p->det_kind; b.G.u0 = p->u0; b.G.du = p->du; b.G.g0 = p->g0; b.G.dg = p->dg;
        b.G.v0 = p->v0; b.G.dv = p->dv; b.G.SO = s.SO; b.G.SD = p->SD;
        b.G.rdu = 1.0f / p->du; b.G.rdg = p->dg != 0.0f ? 1.0f / p->dg : 0.0f;
        b.nx = s.nx; b.ny = s.ny; b.na = s.na; b.nv = s.nv; b.scale = s.scale;
        b.turns = fl_plan_turns(p);
        b.refl = fl_plan_refl(p);
        b.pblk = b.refl ? fan_refl_pblock(b.refl, s.nx, s.ny) : 0;
        b.lanes = b.turns > 1 ? fl_plan_fan_lanes(p) : 1;
        xoff[i + 1] = xoff[i] + (long long)s.nx * s.ny;
        yoff[i + 1] = yoff[i] + (long long)s.na * s.nv;
        woff[i + 1] = woff[i] + ((long long)s.na * s.nv + 3) / 4 * 4;
        b.xoff = xoff[i]; b.yoff = yoff[i]; b.woff = woff[i];
    }
    // work lists, costliest slices first
    std::vector<int> by_walk(n_plans), by_views(n_plans);
    std::iota(by_walk.begin(), by_walk.end(), 0);
    std::iota(by_views.begin(), by_views.end(), 0);
    std::stable_sort(by_walk.begin(), by_walk.end(), [&](int a, int c) {
        return sl[a].nx + sl[a].ny > sl[c].nx + sl[c].ny;
    });
    std::stable_sort(by_views.begin(), by_views.end(), [&](int a, int c) {
        return sl[a].nvf > sl[c].nvf;
    });
    std::vector<int2> rays, wrays;
    for (int i : by_walk) {
        const BatchSlice& c = sl[i];
        for (int r = 0; r < c.na * c.nv; r += kRayChunk) wrays.push_back(make_int2(i, r));
        if (c.turns == 1)
            for (int r = 0; r < c.na * c.nv; r += kRayChunk) rays.push_back(make_int2(i, r));
    }
    // room for the largest walked-ray lists (16 parts per ray), which
    // fl_batch_autotune may choose
    std::vector<int2> rays_t = turn_ray_chunks(sl, by_walk, false);
    std::vector<int2> rays_r = turn_ray_chunks(sl, by_walk, true);
    size_t cap_t = rays_t.size(), cap_r = rays_r.size();
    {
        std::vector<BatchSlice> s16 = sl;
        for (BatchSlice& c : s16)
            if (c.turns > 1) c.lanes = kFanLanes;
        cap_t = std::max(cap_t, turn_ray_chunks(s16, by_walk, false).size());
        cap_r = std::max(cap_r, turn_ray_chunks(s16, by_walk, true).size());
    }
    std::vector<int4> pix, pix_t, pix_r;
    for (int i : by_views) {
        const BatchSlice& c = sl[i];
        if (c.turns == 1) {
            for (int iy = 0; iy < c.ny; iy += 2)
                for (int ix = 0; ix < c.nx; ix += 2 * kPixChunk)
                    pix.push_back(make_int4(i, iy, ix, 0));
        } else if (c.refl) {              // kFanX primary pixel blocks per chunk (block units)
            const int hxb = (c.refl == 1 ? c.nx : c.nx / 2) / c.pblk, hyb = (c.ny / 2) / c.pblk;
            for (int by = 0; by < hyb; by++)
                for (int bx = 0; bx < hxb && (c.refl != 4 || bx <= by); bx += kFanX)
                    pix_r.push_back(make_int4(i, by, bx, 0));
        } else {                          // the primary pixels: rows y < ny/2 (and x < nx/2)
            const int hx = c.turns == 2 ? c.nx : c.nx / 2;
            for (int iy = 0; iy < c.ny / 2; iy += 2)
                for (int ix = 0; ix < hx; ix += 2 * kFanX) pix_t.push_back(make_int4(i, iy, ix, 0));
        }
    }
    std::vector<VecChunk> vec;
    for (int i = 0; i < n_plans; i++) {
        sl[i].vc0 = (int)vec.size();
        long long n = (long long)sl[i].nx * sl[i].ny;
        for (long long k = 0; k < n; k += kVecChunk)
            vec.push_back(VecChunk{i, (int)k, (int)std::min<long long>(kVecChunk, n - k), 0});
        sl[i].vc1 = (int)vec.size();
    }
    if (wrays.size() > 0x7fffffffu || pix.size() + pix_t.size() + pix_r.size() > 0x7fffffffu ||
        vec.size() > 0x7fffffffu || cap_t + cap_r > 0x7fffffffu)
        return fl_set_error(FL_ERR_UNSUPPORTED, "fl_batch_create: batch too large");

    fl_batch* b = new (std::nothrow) fl_batch;
    if (!b) return fl_set_error(FL_ERR_ALLOC, "out of host memory");
    b->n = n_plans; b->n_vox = xoff[n_plans]; b->n_rays = yoff[n_plans];
    b->xoff = xoff; b->yoff = yoff;
    b->d_sl = nullptr; b->d_rays = nullptr; b->d_pix = nullptr; b->d_vec = nullptr;
    b->d_rays_t = nullptr; b->d_wrays = nullptr; b->d_pix_t = nullptr;
    b->r = b->p = b->q = b->tmp = b->xt = nullptr; b->S = nullptr; b->partials = nullptr;
    b->tickets = nullptr; b->hist = nullptr; b->hist_cap = 4096;
    b->cs = nullptr; b->ev0 = b->ev1 = nullptr; b->exec = nullptr; b->cap_u = nullptr;
    b->cs2 = nullptr; b->evf = b->evj = nullptr;
    b->cs3 = nullptr; b->evf3 = b->evj3 = nullptr;
    b->d_rays_r = nullptr; b->d_pix_r = nullptr;
    b->cap_lam = 0.0f; b->cap_tol = 0.0;
    b->h_sl = sl; b->by_walk = by_walk; b->cap_rays_t = (int)cap_t; b->cap_rays_r = (int)cap_r;
    b->n_ray_r_chunks = (int)rays_r.size(); b->n_pix_r_chunks = (int)pix_r.size();
    b->n_ray_chunks = (int)rays.size(); b->n_pix_chunks = (int)pix.size();
    b->n_ray_t_chunks = (int)rays_t.size(); b->n_wray_chunks = (int)wrays.size();
    b->n_pix_t_chunks = (int)pix_t.size();
    b->n_vec_chunks = (int)vec.size();
    int st = upload_vec(&b->d_sl, sl);
    if (!st) st = upload_vec(&b->d_rays, rays);
    auto upload_room = [&](int2** d, const std::vector<int2>& h, size_t cap) {
        if (st) return;
        st = fl_check_cuda(fl_malloc((void**)d, sizeof(int2) * (cap ? cap : 1)), "fl_malloc(batch)");
        if (!st && !h.empty())
            st = fl_check_cuda(cudaMemcpy(*d, h.data(), sizeof(int2) * h.size(),
                                          cudaMemcpyHostToDevice), "upload");
    };
    upload_room(&b->d_rays_t, rays_t, cap_t);
    upload_room(&b->d_rays_r, rays_r, cap_r);
    if (!st) st = upload_vec(&b->d_pix_r, pix_r);
    if (!st) st = upload_vec(&b->d_wrays, wrays);
    if (!st) st = upload_vec(&b->d_pix, pix);
    if (!st) st = upload_vec(&b->d_pix_t, pix_t);
    if (!st) st = upload_vec(&b->d_vec, vec);
    auto M = [&](void** ptr, size_t bytes) {
        if (!st) st = fl_check_cuda(fl_malloc(ptr, bytes), "fl_malloc(batch)");
    };
    M((void**)&b->r, b->n_vox * 4); M((void**)&b->p, b->n_vox * 4); M((void**)&b->q, b->n_vox * 4);
    M((void**)&b->tmp, woff[n_plans] * 4);
    M((void**)&b->xt, b->n_vox * 4);
    M((void**)&b->S, sizeof(BatchScal) * n_plans);
    M((void**)&b->partials, sizeof(double) * b->n_vec_chunks);
    M((void**)&b->tickets, sizeof(unsigned) * n_plans);
    M((void**)&b->hist, sizeof(double) * (size_t)b->hist_cap * n_plans);
    if (!st) st = fl_check_cuda(cudaMemset(b->tickets, 0, sizeof(unsigned) * n_plans), "memset");
    if (!st) st = fl_check_cuda(cudaMemset(b->S, 0, sizeof(BatchScal) * n_plans), "memset");
    if (!st) st = fl_check_cuda(cudaStreamCreateWithFlags(&b->cs, cudaStreamNonBlocking), "stream");
    if (!st) st = fl_check_cuda(cudaEventCreateWithFlags(&b->ev0, cudaEventDisableTiming), "event");
    if (!st) st = fl_check_cuda(cudaEventCreateWithFlags(&b->ev1, cudaEventDisableTiming), "event");
    if (!st) st = fl_check_cuda(cudaStreamCreateWithFlags(&b->cs2, cudaStreamNonBlocking), "stream");
    if (!st) st = fl_check_cuda(cudaEventCreateWithFlags(&b->evf, cudaEventDisableTiming), "event");
    if (!st) st = fl_check_cuda(cudaEventCreateWithFlags(&b->evj, cudaEventDisableTiming), "event");
    if (!st) st = fl_check_cuda(cudaStreamCreateWithFlags(&b->cs3, cudaStreamNonBlocking), "stream");
    if (!st) st = fl_check_cuda(cudaEventCreateWithFlags(&b->evf3, cudaEventDisableTiming), "event");
    if (!st) st = fl_check_cuda(cudaEventCreateWithFlags(&b->evj3, cudaEventDisableTiming), "event");
    if (st) { batch_free(b); delete b; return st; }
    *out = b;
    return fl_set_error(FL_OK, "");
}

extern "C" void fl_batch_destroy(fl_batch* b)
{
    if (!b) return;
    batch_free(b);
    delete b;
}

extern "C" int fl_batch_layout(const fl_batch* b, int64_t* vox_offsets, int64_t* ray_offsets)
{
    if (!b) return fl_set_error(FL_ERR_INVALID, "fl_batch_layout: null batch");
    for (int i = 0; i <= b->n; i++) {
        if (vox_offsets) vox_offsets[i] = b->xoff[i];
        if (ray_offsets) ray_offsets[i] = b->yoff[i];
    }
    return fl_set_error(FL_OK, "");
}

// ypack: y is the batch's scratch (slice offsets woff), turn and reflection
// slices packed per orbit, as batch_adj_w reads it; else the caller's
// sinogram (offsets yoff).
// Each kind of slice present (general, turn, reflection) is one launch; the
// first present runs on s, every further one on a stream of its own forked
// from s and joined back (branches of a captured graph): they write
// different slices, and each fills the others' tails.
static cudaStream_t fork_to(cudaStream_t s, cudaStream_t cs, cudaEvent_t ev)
{
    if (cudaEventRecord(ev, s) != cudaSuccess || cudaStreamWaitEvent(cs, ev, 0) != cudaSuccess)
        return s;
    return cs;
}

static int join_from(cudaStream_t s, cudaStream_t s2, cudaEvent_t ev)
{
    if (s2 == s) return FL_OK;
    FL_CUDA(cudaEventRecord(ev, s2));
    FL_CUDA(cudaStreamWaitEvent(s, ev, 0));
    return FL_OK;
}

static int batch_fwd(fl_batch* b, const float* x, float* y, int cr_power, int ypack,
                     const BatchScal* S, cudaStream_t s)
{
    const bool g = b->n_ray_chunks, t = b->n_ray_t_chunks, r = b->n_ray_r_chunks;
    k_batch_transpose<<<b->n_vec_chunks, kVecThreads, 0, s>>>(x, b->xt, b->d_sl, b->d_vec);
    const cudaStream_t s2 = (t && g) ? fork_to(s, b->cs2, b->evf) : s;
    const cudaStream_t s3 = (r && (g || t)) ? fork_to(s, b->cs3, b->evf3) : s;
    if (r)
        k_batch_fwd_refl<<<b->n_ray_r_chunks, kFanBlock, 0, s3>>>(
            x, b->xt, y, b->d_sl, b->d_rays_r, cr_power, ypack, S);
    if (t)
        k_batch_fwd_turn<<<b->n_ray_t_chunks, kFanBlock, 0, s2>>>(
            x, b->xt, y, b->d_sl, b->d_rays_t, cr_power, ypack, S);
    if (g)
        k_batch_fwd<<<b->n_ray_chunks, kRayChunk, 0, s>>>(x, b->xt, y, b->d_sl, b->d_rays,
                                                          cr_power, ypack, S);
    int st = fl_check_launch("batched forward");
    if (!st) st = join_from(s, s2, b->evj);
    if (!st) st = join_from(s, s3, b->evj3);
    return st;
}

static int batch_adj_w(fl_batch* b, const float* yw, float* x, const BatchScal* S, cudaStream_t s)
{
    const bool g = b->n_pix_chunks, t = b->n_pix_t_chunks, r = b->n_pix_r_chunks;
    const cudaStream_t s2 = (t && g) ? fork_to(s, b->cs2, b->evf) : s;
    const cudaStream_t s3 = (r && (g || t)) ? fork_to(s, b->cs3, b->evf3) : s;
    if (r)
        k_batch_adj_refl<<<b->n_pix_r_chunks, dim3(kFanX, kTurnGroups), 0, s3>>>(
            x, yw, b->d_sl, b->d_pix_r, S);
    if (t)
        k_batch_adj_turn<<<b->n_pix_t_chunks, dim3(kFanX, kTurnGroups), 0, s2>>>(
            x, yw, b->d_sl, b->d_pix_t, S);
    if (g)
        k_batch_adj<<<b->n_pix_chunks, kPixChunk, 0, s>>>(x, yw, b->d_sl, b->d_pix, S);
    int st = fl_check_launch("batched adjoint");
    if (!st) st = join_from(s, s2, b->evj);
    if (!st) st = join_from(s, s3, b->evj3);
    return st;
}

extern "C" int fl_batch_forward(fl_batch* b, const float* x, float* y, void* stream)
{
    FL_RANGE("fl_batch_forward");
    if (!b || !x || !y) return fl_set_error(FL_ERR_INVALID, "fl_batch_forward: null argument");
    int st = batch_fwd(b, x, y, 1, 0, nullptr, (cudaStream_t)stream);
    return st ? st : fl_set_error(FL_OK, "");
}

// Uses the batch's sinogram scratch: calls on one batch are stream-ordered.
extern "C" int fl_batch_adjoint(fl_batch* b, const float* y, float* x, void* stream)
{
    FL_RANGE("fl_batch_adjoint");
    if (!b || !x || !y) return fl_set_error(FL_ERR_INVALID, "fl_batch_adjoint: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    k_batch_weight<<<b->n_wray_chunks, kRayChunk, 0, s>>>(b->tmp, y, b->d_sl, b->d_wrays);
    int st = fl_check_launch("batched weighting");
    if (!st) st = batch_adj_w(b, b->tmp, x, nullptr, s);
    return st ? st : fl_set_error(FL_OK, "");
}

// Sets every turn slice's parts per walked ray to L and rebuilds the turn
// forward's work list (kFanBlock / L rays per chunk).
static int batch_set_lanes(fl_batch* b, int L, cudaStream_t s)
{
    for (BatchSlice& c : b->h_sl)
        if (c.turns > 1) c.lanes = L;
    const std::vector<int2> rays_t = turn_ray_chunks(b->h_sl, b->by_walk, false);
    const std::vector<int2> rays_r = turn_ray_chunks(b->h_sl, b->by_walk, true);
    if ((long long)rays_t.size() > b->cap_rays_t || (long long)rays_r.size() > b->cap_rays_r)
        return fl_set_error(FL_ERR_INVALID, "fl_batch_autotune: work list beyond its room");
    FL_CUDA(cudaMemcpyAsync(b->d_sl, b->h_sl.data(), sizeof(BatchSlice) * b->h_sl.size(),
                            cudaMemcpyHostToDevice, s));
    if (!rays_t.empty())
        FL_CUDA(cudaMemcpyAsync(b->d_rays_t, rays_t.data(), sizeof(int2) * rays_t.size(),
                                cudaMemcpyHostToDevice, s));
    if (!rays_r.empty())
        FL_CUDA(cudaMemcpyAsync(b->d_rays_r, rays_r.data(), sizeof(int2) * rays_r.size(),
                                cudaMemcpyHostToDevice, s));
    FL_CUDA(cudaStreamSynchronize(s));         // the host vectors go out of scope
    b->n_ray_t_chunks = (int)rays_t.size();
    b->n_ray_r_chunks = (int)rays_r.size();
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }   // recaptured
    return FL_OK;
}

// Parts per walked ray of the batch's turn slices: each count (1, 4, 16) is
// timed on the batch's own forward of a CGLS iteration (CUDA events, one
// launch after one untimed; the batch's q and scratch as input and output)
// and the fastest kept for every turn slice. Alone, a small scan needs parts
// to fill the GPU; in a batch its neighbours may already fill it.
extern "C" int fl_batch_autotune(fl_batch* b, void* stream, int32_t* parts)
{
    FL_RANGE("fl_batch_autotune");
    if (!b) return fl_set_error(FL_ERR_INVALID, "fl_batch_autotune: null batch");
    bool any = false;
    for (const BatchSlice& c : b->h_sl) any |= c.turns > 1;
    if (parts) *parts = 0;
    if (!any) return fl_set_error(FL_OK, "");
    cudaStream_t s = (cudaStream_t)stream;
    FL_CUDA(cudaMemsetAsync(b->q, 0, sizeof(float) * b->n_vox, s));
    cudaEvent_t e0, e1;
    FL_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fl_set_error(FL_ERR_CUDA, "fl_batch_autotune: cudaEventCreate failed");
    }
    static const int cand[3] = {1, 4, kFanLanes};
    float best = 3.0e38f;
    int bi = -1, st = FL_OK;
    for (int c = 0; c < 3 && !st; c++) {
        if ((st = batch_set_lanes(b, cand[c], s))) break;
        for (int rep = 0; rep < 2 && !st; rep++) {
            if (rep == 1 && cudaEventRecord(e0, s) != cudaSuccess) st = FL_ERR_CUDA;
            if (!st) st = batch_fwd(b, b->q, b->tmp, 2, 1, nullptr, s);
        }
        float ms = 0.0f;
        if (!st && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                    cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
            st = fl_set_error(FL_ERR_CUDA, "fl_batch_autotune: timing failed");
        if (!st && ms < best) { best = ms; bi = c; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    if ((st = batch_set_lanes(b, cand[bi], s))) return st;
    if (parts) *parts = cand[bi];
    return fl_set_error(FL_OK, "");
}

static int batch_iteration(fl_batch* b, float* u, float lam, double tol, cudaStream_t s)
{
    int st = batch_fwd(b, b->p, b->tmp, 2, 1, b->S, s);
    if (!st) st = batch_adj_w(b, b->tmp, b->q, b->S, s);
    if (st) return st;
    const int g = b->n_vec_chunks;
    k_batch_pq<<<g, kVecThreads, 0, s>>>(b->p, b->q, lam, b->d_sl, b->d_vec, b->S, b->partials,
                                         b->tickets);
    k_batch_update<<<g, kVecThreads, 0, s>>>(u, b->r, b->p, b->q, tol, b->d_sl, b->d_vec, b->S,
                                             b->partials, b->tickets, b->hist, b->hist_cap);
    k_batch_dir<<<g, kVecThreads, 0, s>>>(b->r, b->p, b->d_sl, b->d_vec, b->S);
    return fl_check_launch("batched CGLS iteration");
}

extern "C" int fl_batch_cgls(fl_batch* b, const float* rhs, float* u, float lam, int32_t iters,
                             double tol, int32_t flags, double* gamma_history,
                             int32_t* iters_done, void* stream)
{
    FL_RANGE("fl_batch_cgls");
    if (!b || !rhs || !u || iters < 0)
        return fl_set_error(FL_ERR_INVALID, "fl_batch_cgls: bad argument");
    cudaStream_t us = (cudaStream_t)stream, s = b->cs;
    int st;
    FL_CUDA(cudaEventRecord(b->ev0, us));
    FL_CUDA(cudaStreamWaitEvent(s, b->ev0, 0));
    const float* q0 = nullptr;
    if (!(flags & FL_CGLS_ZERO_START)) {
        if ((st = batch_fwd(b, u, b->tmp, 2, 1, nullptr, s))) return st;
        if ((st = batch_adj_w(b, b->tmp, b->q, nullptr, s))) return st;
        q0 = b->q;
    }
    k_batch_init<<<b->n_vec_chunks, kVecThreads, 0, s>>>(rhs, q0, u, lam, b->r, b->p, b->d_sl,
                                                         b->d_vec, b->S, b->partials, b->tickets);
    if ((st = fl_check_launch("batched CGLS init"))) return st;
    if (!b->exec || b->cap_u != u || b->cap_lam != lam || b->cap_tol != tol) {
        if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
        cudaGraph_t g;
        FL_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int cst = batch_iteration(b, u, lam, tol, s);
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (cst) return cst;
        FL_CUDA(e);
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        FL_CUDA(e);
        b->cap_u = u; b->cap_lam = lam; b->cap_tol = tol;
    }
    for (int it = 0; it < iters; it++) FL_CUDA(cudaGraphLaunch(b->exec, s));
    std::vector<BatchScal> fin(b->n);
    FL_CUDA(cudaMemcpyAsync(fin.data(), b->S, sizeof(BatchScal) * b->n, cudaMemcpyDeviceToHost, s));
    const int nh = std::min(iters, b->hist_cap);
    std::vector<double> h;
    if (gamma_history && nh > 0) {
        h.resize((size_t)b->hist_cap * b->n);
        FL_CUDA(cudaMemcpyAsync(h.data(), b->hist, sizeof(double) * h.size(),
                                cudaMemcpyDeviceToHost, s));
    }
    FL_CUDA(cudaEventRecord(b->ev1, s));
    FL_CUDA(cudaStreamWaitEvent(us, b->ev1, 0));
    FL_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < b->n; i++) {
        if (iters_done) iters_done[i] = fin[i].iter;
        if (gamma_history)
            for (int k = 0; k < iters; k++)
                gamma_history[(size_t)i * iters + k] =
                    (k < nh && k < fin[i].iter) ? h[(size_t)i * b->hist_cap + k] : 0.0;
    }
    for (int i = 0; i < b->n; i++)
        if (fin[i].status)
            return fl_set_error(FL_ERR_NUMERIC,
                                "fl_batch_cgls: slice %d stopped on a non-finite residual or "
                                "curvature after %d iterations (the other slices completed)",
                                i, fin[i].iter);
    return fl_set_error(FL_OK, "");
}

FL_OOB_ACCESSOR(fl_oob_batch)
