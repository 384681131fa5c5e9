// framelet.cu -- undecimated tensor-product framelets (Haar, piecewise linear,
// piecewise cubic), soft-shrinkage and the fused split-Bregman update.
//
// Semantics (FraDecMultiLevel3D.m:14-47, FraRecMultiLevel3D.m:14-48,
// ConvSymAsym3D.m:18-34, GenerateFrameletFilter.m:2-30, softThreshold.m:47-80):
//  * every 1-D filter is a circular correlation, taps at offsets
//    (t - c) * 2^(level-1) around the output sample (imfilter 'circular');
//  * 3-D band (i, j, k): D_i along y, D_j along x, D_k along z; 2-D band
//    (i, j): D_i along x, D_j along y (FraDecMultiLevel2D.m:43-52);
//  * level l+1 decomposes the low band (0,0[,0]) of level l; the synthesis
//    replaces that low band by the reconstruction of level l+1, so the low
//    band of every level but the last is never stored here;
//  * soft-shrink sign(a) max(|a| - tau, 0) applies to every stored band except
//    the low band of the last level.
// Coefficient layout: level-major; inside a level, band index = base-nf digits
// in pass order (nf filters per axis; linear 3-D: 9i + 3j + k, 2-D: 3i + j),
// band 0 omitted below the last level; each band is one volume (x fastest).
//
// Every pass is a streaming circular stencil along one axis. The last analysis
// pass computes each band value in registers and applies the Bregman update
// (v, alpha, alpha - v) without storing W u; the last synthesis pass writes
// b = base + mu * W^T t directly.
#include <cstring>
#include <new>
#include <vector>

#include "fl_trace.h"
#include "fl_common.cuh"

namespace {

constexpr int kMaxBands = 125;   // cubic bank in 3-D: 5^3 bands

struct Filters {
    float f[5][5];   // up to 5 filters x 5 taps (linear 3 x 3, haar 2 x 3, cubic 5 x 5)
    int nf, nt;      // filters, taps
};

struct BandPtrs {
    float* p[kMaxBands];   // per band: coefficient array (nullptr: not stored)
};

// j mod n for a tap index; |j - [0, n)| is almost always below n, so one add
// or subtract wraps it (the modulo only runs for volumes smaller than a tap
// offset)
__device__ __forceinline__ int wrapi(int j, int n)
{
    if (j < 0) {
        j += n;
        if (j < 0) { j %= n; if (j < 0) j += n; }
    } else if (j >= n) {
        j -= n;
        if (j >= n) j %= n;
    }
    return j;
}

// index of the neighbour at offset d along AXIS (0 x, 1 y, 2 z), circular
template <int AXIS>
__device__ __forceinline__ long long nb(int ix, int iy, int iz, int nx, int ny, int nz, int d)
{
    if (AXIS == 0) ix = wrapi(ix + d, nx);
    else if (AXIS == 1) iy = wrapi(iy + d, ny);
    else iz = wrapi(iz + d, nz);
    return ((long long)iz * ny + iy) * nx + ix;
}

// Every pass runs on the grid (x in blocks of 128, y, z * channel): no index
// arithmetic per element beyond the wrap of the taps. NF filters of NT taps.
constexpr int kPassThreads = 128;

// out[NF*c + f] = F_f (*) in[c] along AXIS   (analysis split pass)
template <int NF, int NT, int AXIS>
__global__ void __launch_bounds__(kPassThreads)
k_split(const float* __restrict__ in, long long in_stride, float* __restrict__ out,
        long long out_stride, int nx, int ny, int nz, int step, Filters F)
{
    const int ix = blockIdx.x * kPassThreads + threadIdx.x;
    if (ix >= nx) return;
    const int iy = blockIdx.y, iz = blockIdx.z % nz, c = blockIdx.z / nz;
    const long long q = ((long long)iz * ny + iy) * nx + ix;
    const float* src = in + (long long)c * in_stride;
    constexpr int ctr = (NT - 1) / 2;
    float v[NT];
#pragma unroll
    for (int t = 0; t < NT; t++) v[t] = __ldg(src + nb<AXIS>(ix, iy, iz, nx, ny, nz, (t - ctr) * step));
#pragma unroll
    for (int f = 0; f < NF; f++) {
        float s = 0.0f;
#pragma unroll
        for (int t = 0; t < NT; t++) s = fmaf(F.f[f][t], v[t], s);
        out[(long long)(NF * c + f) * out_stride + q] = s;
    }
}

// Last analysis pass. band = NF*c + f. mode 0: coef[band] = w (skipping band 0
// below the last level, which goes to `low`); mode 1: split-Bregman update on
// v and t = alpha - v_new with soft threshold tau (no shrink on band 0 of the
// last level).
template <int NF, int NT, int AXIS>
__global__ void __launch_bounds__(kPassThreads)
k_split_last(const float* __restrict__ in, long long in_stride, int nx, int ny, int nz,
             int step, Filters F, BandPtrs coef, BandPtrs tout, float* __restrict__ low,
             int last, int mode, float tau)
{
    const int ix = blockIdx.x * kPassThreads + threadIdx.x;
    if (ix >= nx) return;
    const int iy = blockIdx.y, iz = blockIdx.z % nz, c = blockIdx.z / nz;
    const long long q = ((long long)iz * ny + iy) * nx + ix;
    const float* src = in + (long long)c * in_stride;
    constexpr int ctr = (NT - 1) / 2;
    float v[NT];
#pragma unroll
    for (int t = 0; t < NT; t++) v[t] = __ldg(src + nb<AXIS>(ix, iy, iz, nx, ny, nz, (t - ctr) * step));
#pragma unroll
    for (int f = 0; f < NF; f++) {
        float w = 0.0f;
#pragma unroll
        for (int t = 0; t < NT; t++) w = fmaf(F.f[f][t], v[t], w);
        const int band = NF * c + f;
        if (band == 0 && !last) {
            if (low) low[q] = w;
            continue;
        }
        if (mode == 0) {
            coef.p[band][q] = w;
        } else {
            const float s = coef.p[band][q] + w;           // v + W u
            float a = s;                                   // alpha
            if (!(band == 0 && last)) {
                const float m = fabsf(s) - tau;
                a = m > 0.0f ? copysignf(m, s) : 0.0f;
            }
            const float vn = s - a;                        // v + W u - alpha
            coef.p[band][q] = vn;
            tout.p[band][q] = a - vn;                      // alpha - v_new
        }
    }
}

// out[c] = sum_f F_f (*) in[NF*c + f] along AXIS (synthesis merge pass); input
// arrays come from `bands` (band pointer per index) -- with band 0 replaced by
// `low` when non-null. final: out = base + scale * result.
template <int NF, int NT, int AXIS>
__global__ void __launch_bounds__(kPassThreads)
k_merge(BandPtrs bands, const float* __restrict__ low, float* __restrict__ out,
        long long out_stride, int nx, int ny, int nz, int step, Filters F,
        const float* __restrict__ base, float scale, int final_)
{
    const int ix = blockIdx.x * kPassThreads + threadIdx.x;
    if (ix >= nx) return;
    const int iy = blockIdx.y, iz = blockIdx.z % nz, c = blockIdx.z / nz;
    const long long q = ((long long)iz * ny + iy) * nx + ix;
    constexpr int ctr = (NT - 1) / 2;
    float s = 0.0f;
#pragma unroll
    for (int f = 0; f < NF; f++) {
        const int band = NF * c + f;
        const float* src = (band == 0 && low) ? low : bands.p[band];
#pragma unroll
        for (int t = 0; t < NT; t++)
            s = fmaf(F.f[f][t], __ldg(src + nb<AXIS>(ix, iy, iz, nx, ny, nz, (t - ctr) * step)), s);
    }
    if (final_) s = (base ? __ldg(base + q) : 0.0f) + scale * s;
    out[(long long)c * out_stride + q] = s;
}

// launchers: filter bank (NF, NT) and axis as template arguments
template <int NF, int NT>
struct Pass {
    static void split(int axis, dim3 g, cudaStream_t s, const float* in, long long is, float* out,
                      long long os, int nx, int ny, int nz, int step, const Filters& F)
    {
        if (axis == 0) k_split<NF, NT, 0><<<g, kPassThreads, 0, s>>>(in, is, out, os, nx, ny, nz, step, F);
        else if (axis == 1) k_split<NF, NT, 1><<<g, kPassThreads, 0, s>>>(in, is, out, os, nx, ny, nz, step, F);
        else k_split<NF, NT, 2><<<g, kPassThreads, 0, s>>>(in, is, out, os, nx, ny, nz, step, F);
    }
    static void split_last(int axis, dim3 g, cudaStream_t s, const float* in, long long is,
                           int nx, int ny, int nz, int step, const Filters& F, const BandPtrs& cb,
                           const BandPtrs& tb, float* low, int last, int mode, float tau)
    {
        if (axis == 0)
            k_split_last<NF, NT, 0><<<g, kPassThreads, 0, s>>>(in, is, nx, ny, nz, step, F, cb, tb, low, last, mode, tau);
        else if (axis == 1)
            k_split_last<NF, NT, 1><<<g, kPassThreads, 0, s>>>(in, is, nx, ny, nz, step, F, cb, tb, low, last, mode, tau);
        else
            k_split_last<NF, NT, 2><<<g, kPassThreads, 0, s>>>(in, is, nx, ny, nz, step, F, cb, tb, low, last, mode, tau);
    }
    static void merge(int axis, dim3 g, cudaStream_t s, const BandPtrs& b, const float* low,
                      float* out, long long os, int nx, int ny, int nz, int step,
                      const Filters& F, const float* base, float scale, int final_)
    {
        if (axis == 0)
            k_merge<NF, NT, 0><<<g, kPassThreads, 0, s>>>(b, low, out, os, nx, ny, nz, step, F, base, scale, final_);
        else if (axis == 1)
            k_merge<NF, NT, 1><<<g, kPassThreads, 0, s>>>(b, low, out, os, nx, ny, nz, step, F, base, scale, final_);
        else
            k_merge<NF, NT, 2><<<g, kPassThreads, 0, s>>>(b, low, out, os, nx, ny, nz, step, F, base, scale, final_);
    }
};

unsigned grid_for(long long n)
{
    long long g = (n + 255) / 256;
    return (unsigned)(g < 4096 ? (g > 0 ? g : 1) : 4096);
}

}  // namespace

// ---------------------------------------------------------------------------
// out = sign(a) max(|a| - tau, 0) for coefficients outside [keep0, keep1)
// (the unshrunk low band), out = a inside
__global__ void k_shrink(const float* __restrict__ a, float* __restrict__ out, long long n,
                         long long keep0, long long keep1, float tau)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float v = a[i];
        if (i >= keep0 && i < keep1) { out[i] = v; continue; }
        const float m = fmaxf(fabsf(v) - tau, 0.0f);
        out[i] = v > 0.0f ? m : (v < 0.0f ? -m : 0.0f);
    }
}

struct fl_framelet {
    int nx, ny, nz, dim, levels, kind;
    int nf, nbands;                 // filters per axis, bands per level (nf^dim)
    long long N;
    Filters D, R;
    int axes[3];                    // analysis pass order
    float* work;                    // intermediates: nf^(dim-1) + nf^(dim-2) arrays + low
    long long work_elems;
    std::vector<long long> level_base;   // first coefficient band of each level
    long long ncoef_bands;
};

static void set_filters(fl_framelet* w, int kind)
{
    std::memset(&w->D, 0, sizeof w->D);
    std::memset(&w->R, 0, sizeof w->R);
    const float r2 = 1.41421356237309505f;
    if (kind == 1) {   // piecewise linear (GenerateFrameletFilter.m:9-17)
        const float d[3][3] = {{0.25f, 0.5f, 0.25f}, {-r2 / 4, 0.0f, r2 / 4}, {-0.25f, 0.5f, -0.25f}};
        const float r[3][3] = {{0.25f, 0.5f, 0.25f}, {r2 / 4, 0.0f, -r2 / 4}, {-0.25f, 0.5f, -0.25f}};
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) { w->D.f[a][b] = d[a][b]; w->R.f[a][b] = r[a][b]; }
        w->D.nf = w->R.nf = 3; w->D.nt = w->R.nt = 3;
    } else if (kind == 3) {   // piecewise cubic (GenerateFrameletFilter.m:18-30)
        const float r6 = 2.44948974278317810f;
        const float d[5][5] = {{1 / 16.f, 4 / 16.f, 6 / 16.f, 4 / 16.f, 1 / 16.f},
                               {-1 / 8.f, -2 / 8.f, 0.f, 2 / 8.f, 1 / 8.f},
                               {-r6 / 16, 0.f, 2 * r6 / 16, 0.f, -r6 / 16},
                               {-1 / 8.f, 2 / 8.f, 0.f, -2 / 8.f, 1 / 8.f},
                               {-1 / 16.f, 4 / 16.f, -6 / 16.f, 4 / 16.f, -1 / 16.f}};
        const float r[5][5] = {{1 / 16.f, 4 / 16.f, 6 / 16.f, 4 / 16.f, 1 / 16.f},
                               {1 / 8.f, 2 / 8.f, 0.f, -2 / 8.f, -1 / 8.f},
                               {-r6 / 16, 0.f, 2 * r6 / 16, 0.f, -r6 / 16},
                               {1 / 8.f, -2 / 8.f, 0.f, 2 / 8.f, -1 / 8.f},
                               {-1 / 16.f, 4 / 16.f, -6 / 16.f, 4 / 16.f, -1 / 16.f}};
        for (int a = 0; a < 5; a++)
            for (int b = 0; b < 5; b++) { w->D.f[a][b] = d[a][b]; w->R.f[a][b] = r[a][b]; }
        w->D.nf = w->R.nf = 5; w->D.nt = w->R.nt = 5;
    } else {           // Haar (GenerateFrameletFilter.m:2-8)
        const float d[2][3] = {{0.0f, 0.5f, 0.5f}, {0.0f, -0.5f, 0.5f}};
        const float r[2][3] = {{0.5f, 0.5f, 0.0f}, {0.5f, -0.5f, 0.0f}};
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 3; b++) { w->D.f[a][b] = d[a][b]; w->R.f[a][b] = r[a][b]; }
        w->D.nf = w->R.nf = 2; w->D.nt = w->R.nt = 3;
    }
}

extern "C" int fl_framelet_create(int nx, int ny, int nz, int levels, int kind, fl_framelet** out)
{
    FL_RANGE("fl_framelet_create");
    if (!out || nx < 1 || ny < 1 || nz < 1 || levels < 1 || levels > 8)
        return fl_set_error(FL_ERR_INVALID, "fl_framelet_create: bad size or levels");
    if (kind != FL_FRAMELET_LINEAR && kind != FL_FRAMELET_HAAR && kind != FL_FRAMELET_CUBIC)
        return fl_set_error(FL_ERR_INVALID, "fl_framelet_create: unknown filter bank %d", kind);
    {   // the passes run on the grid (x blocks, y, z * channels)
        const long long maxch = (kind == FL_FRAMELET_CUBIC ? 25 : 9);
        if (ny > 65535 || (long long)nz * maxch > 65535)
            return fl_set_error(FL_ERR_UNSUPPORTED,
                                "fl_framelet_create: ny must be <= 65535 and nz <= %lld",
                                65535 / maxch);
    }
    *out = nullptr;
    fl_framelet* w = new (std::nothrow) fl_framelet;
    if (!w) return fl_set_error(FL_ERR_ALLOC, "out of host memory");
    w->nx = nx; w->ny = ny; w->nz = nz; w->dim = (nz > 1) ? 3 : 2; w->levels = levels;
    w->kind = kind; w->N = (long long)nx * ny * nz;
    set_filters(w, kind);
    w->nf = w->D.nf;
    w->nbands = w->dim == 3 ? w->nf * w->nf * w->nf : w->nf * w->nf;
    if (w->dim == 3) { w->axes[0] = 1; w->axes[1] = 0; w->axes[2] = 2; }   // y, x, z
    else { w->axes[0] = 0; w->axes[1] = 1; w->axes[2] = -1; }              // x, y
    long long b = 0;
    for (int l = 0; l < levels; l++) {
        w->level_base.push_back(b);
        b += (l == levels - 1) ? w->nbands : w->nbands - 1;
    }
    w->ncoef_bands = b;
    long long inter = (w->dim == 3) ? (w->nf + w->nf * w->nf) : w->nf;
    w->work_elems = (inter + 2) * w->N;   // pass intermediates + two low-band volumes
    int st = fl_check_cuda(fl_malloc((void**)&w->work, w->work_elems * sizeof(float)),
                           "fl_malloc(framelet)");
    if (st) { delete w; return st; }
    *out = w;
    return fl_set_error(FL_OK, "");
}

extern "C" void fl_framelet_destroy(fl_framelet* w)
{
    if (!w) return;
    if (w->work) cudaFree(w->work);
    delete w;
}

extern "C" int64_t fl_framelet_ncoef(const fl_framelet* w)
{
    return w ? w->ncoef_bands * w->N : 0;
}

// band pointers of one level inside a coefficient set (band 0 below the last
// level is absent)
static BandPtrs level_bands(const fl_framelet* w, float* coef, int l)
{
    BandPtrs B;
    for (int b = 0; b < kMaxBands; b++) B.p[b] = nullptr;
    if (!coef) return B;
    const bool last = (l == w->levels - 1);
    long long base = w->level_base[l];
    for (int b = 0; b < w->nbands; b++) {
        if (b == 0 && !last) continue;
        long long idx = base + (last ? b : b - 1);
        B.p[b] = coef + idx * w->N;
    }
    return B;
}

static dim3 pass_grid(const fl_framelet* w, int channels)
{
    return dim3(fl_div_up(w->nx, kPassThreads), w->ny, (unsigned)(w->nz * channels));
}

// One analysis level: the separable passes along the three (two) axes, the
// last one fused with the coefficient write or the Bregman update.
template <int NF, int NT>
static void analysis_level(fl_framelet* w, const float* in, int step, const BandPtrs& cb,
                           const BandPtrs& tb, float* low_out, int last, int mode, float tau,
                           cudaStream_t s)
{
    using P = Pass<NF, NT>;
    const long long N = w->N;
    float* A = w->work;                          // NF arrays
    float* Bm = A + (long long)NF * N;           // NF^2 arrays (3-D)
    if (w->dim == 3) {
        P::split(w->axes[0], pass_grid(w, 1), s, in, N, A, N, w->nx, w->ny, w->nz, step, w->D);
        P::split(w->axes[1], pass_grid(w, NF), s, A, N, Bm, N, w->nx, w->ny, w->nz, step, w->D);
        P::split_last(w->axes[2], pass_grid(w, NF * NF), s, Bm, N, w->nx, w->ny, w->nz, step,
                      w->D, cb, tb, low_out, last, mode, tau);
    } else {
        P::split(w->axes[0], pass_grid(w, 1), s, in, N, A, N, w->nx, w->ny, w->nz, step, w->D);
        P::split_last(w->axes[1], pass_grid(w, NF), s, A, N, w->nx, w->ny, w->nz, step, w->D,
                      cb, tb, low_out, last, mode, tau);
    }
}

// One synthesis level: the merge passes in reverse axis order, the last one
// writing dst (= base + scale * result on the final level).
template <int NF, int NT>
static void synthesis_level(fl_framelet* w, const BandPtrs& cb, const float* low, float* dst,
                            int step, const float* base, float scale, int final_, cudaStream_t s)
{
    using P = Pass<NF, NT>;
    const long long N = w->N;
    float* A = w->work;
    float* Bm = A + (long long)NF * N;
    BandPtrs ib, jb;
    for (int b = 0; b < kMaxBands; b++) ib.p[b] = jb.p[b] = nullptr;
    if (w->dim == 3) {
        P::merge(w->axes[2], pass_grid(w, NF * NF), s, cb, low, Bm, N, w->nx, w->ny, w->nz,
                 step, w->R, nullptr, 1.0f, 0);
        for (int b = 0; b < NF * NF; b++) ib.p[b] = Bm + (long long)b * N;
        P::merge(w->axes[1], pass_grid(w, NF), s, ib, nullptr, A, N, w->nx, w->ny, w->nz, step,
                 w->R, nullptr, 1.0f, 0);
        for (int b = 0; b < NF; b++) jb.p[b] = A + (long long)b * N;
        P::merge(w->axes[0], pass_grid(w, 1), s, jb, nullptr, dst, N, w->nx, w->ny, w->nz, step,
                 w->R, base, scale, final_);
    } else {
        P::merge(w->axes[1], pass_grid(w, NF), s, cb, low, A, N, w->nx, w->ny, w->nz, step,
                 w->R, nullptr, 1.0f, 0);
        for (int b = 0; b < NF; b++) jb.p[b] = A + (long long)b * N;
        P::merge(w->axes[0], pass_grid(w, 1), s, jb, nullptr, dst, N, w->nx, w->ny, w->nz, step,
                 w->R, base, scale, final_);
    }
}

// Analysis of all levels. mode 0: coef = W u. mode 1: Bregman update of v
// (coef argument) writing t = alpha - v_new into tcoef.
static int analysis(fl_framelet* w, const float* u, float* coef, float* tcoef, int mode,
                    float tau, cudaStream_t s)
{
    const long long N = w->N;
    float* low0 = w->work + (w->work_elems - 2 * N);
    float* low1 = low0 + N;
    const float* in = u;
    for (int l = 0; l < w->levels; l++) {
        const int step = 1 << l;
        const int last = (l == w->levels - 1) ? 1 : 0;
        float* low_out = last ? nullptr : ((l % 2 == 0) ? low0 : low1);
        BandPtrs cb = level_bands(w, coef, l), tb = level_bands(w, tcoef, l);
        if (w->kind == FL_FRAMELET_LINEAR)
            analysis_level<3, 3>(w, in, step, cb, tb, low_out, last, mode, tau, s);
        else if (w->kind == FL_FRAMELET_CUBIC)
            analysis_level<5, 5>(w, in, step, cb, tb, low_out, last, mode, tau, s);
        else
            analysis_level<2, 3>(w, in, step, cb, tb, low_out, last, mode, tau, s);
        int st = fl_check_launch("framelet analysis");
        if (st) return st;
        in = low_out;
    }
    return FL_OK;
}

// Synthesis: out = base + scale * W^T coef (base may be null, scale 1).
static int synthesis(fl_framelet* w, float* coef, float* out, const float* base, float scale,
                     cudaStream_t s)
{
    const long long N = w->N;
    float* low0 = w->work + (w->work_elems - 2 * N);
    float* low1 = low0 + N;
    const float* low = nullptr;
    for (int l = w->levels - 1; l >= 0; l--) {
        const int step = 1 << l;
        const int final_ = (l == 0) ? 1 : 0;
        float* dst = final_ ? out : ((l % 2 == 0) ? low0 : low1);
        BandPtrs cb = level_bands(w, coef, l);
        const float* bs = final_ ? base : nullptr;
        const float sc = final_ ? scale : 1.0f;
        if (w->kind == FL_FRAMELET_LINEAR)
            synthesis_level<3, 3>(w, cb, low, dst, step, bs, sc, final_, s);
        else if (w->kind == FL_FRAMELET_CUBIC)
            synthesis_level<5, 5>(w, cb, low, dst, step, bs, sc, final_, s);
        else
            synthesis_level<2, 3>(w, cb, low, dst, step, bs, sc, final_, s);
        int st = fl_check_launch("framelet synthesis");
        if (st) return st;
        low = dst;
    }
    return FL_OK;
}

extern "C" int fl_framelet_analysis(fl_framelet* w, const float* u, float* coef, void* stream)
{
    FL_RANGE("fl_framelet_analysis");
    if (!w || !u || !coef) return fl_set_error(FL_ERR_INVALID, "fl_framelet_analysis: null argument");
    int st = analysis(w, u, coef, nullptr, 0, 0.0f, (cudaStream_t)stream);
    return st ? st : fl_set_error(FL_OK, "");
}

extern "C" int fl_framelet_synthesis(fl_framelet* w, const float* coef, float* u, void* stream)
{
    FL_RANGE("fl_framelet_synthesis");
    if (!w || !u || !coef) return fl_set_error(FL_ERR_INVALID, "fl_framelet_synthesis: null argument");
    int st = synthesis(w, const_cast<float*>(coef), u, nullptr, 1.0f, (cudaStream_t)stream);
    return st ? st : fl_set_error(FL_OK, "");
}

extern "C" int fl_framelet_bregman(fl_framelet* w, const float* u, float* v, float* t,
                                   const float* Atf, float mu, float tau, float* b, void* stream)
{
    FL_RANGE("fl_framelet_bregman");
    if (!w || !u || !v || !t || !b)
        return fl_set_error(FL_ERR_INVALID, "fl_framelet_bregman: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    int st = analysis(w, u, v, t, 1, tau, s);
    if (st) return st;
    st = synthesis(w, t, b, Atf, mu, s);
    return st ? st : fl_set_error(FL_OK, "");
}

extern "C" int fl_framelet_shrink(fl_framelet* w, const float* coef, float* out, float tau,
                                  void* stream)
{
    if (!w || !coef || !out) return fl_set_error(FL_ERR_INVALID, "fl_framelet_shrink: null argument");
    const long long n = w->ncoef_bands * w->N;
    const long long low = w->level_base[w->levels - 1] * w->N;   // band 0 of the last level
    k_shrink<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(coef, out, n, low, low + w->N, tau);
    int st = fl_check_launch("framelet shrink");
    return st ? st : fl_set_error(FL_OK, "");
}
