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
    float vv[NF];                                          // v of every band, read before any store
#pragma unroll
    for (int f = 0; f < NF; f++)
        vv[f] = (mode == 0 || (NF * c + f == 0 && !last)) ? 0.0f : coef.p[NF * c + f][q];
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
            const float s = vv[f] + w;                     // v + W u
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

// ---------------------------------------------------------------------------
// z-streaming 3-D level kernels for the three-tap banks (linear, Haar). A
// block owns a column tile (warp = one row y, lane = x) and walks the slices
// z = r, r + s, r + 2s, ... of one residue class r mod s (s = 2^level), up to
// kSegZ output slices. The z taps of an output slice are the slices z - s, z,
// z + s of its own class, so each thread keeps the z-pass inputs of its
// sample in a three-slot register window and every slice is read once per
// block. Every value is the same fmaf chain as in the separable pass kernels
// above (taps in order, filters in order), so both forms give identical bits.
constexpr int kSX = 32, kSY = 8, kST = kSX * kSY;   // column tile, threads per block
constexpr int kSegZ = 32;                            // output slices of one class per block
constexpr int kMaxStreamStep = 8;                    // dilations the streaming kernels take

// slices of residue class r in [0, nz): r, r + s, ...
__host__ __device__ inline int class_len(int nz, int s, int r)
{
    return r < nz ? (nz - 1 - r) / s + 1 : 0;
}

// One analysis level: the y and x passes of each slice in shared memory, the
// z pass from the register window, fused with the coefficient write (mode 0)
// or the Bregman update (mode 1) exactly as k_split_last.
template <int NF, int S>
__global__ void __launch_bounds__(kST, 2)
k_ana_stream(const float* __restrict__ in, int nx, int ny, int nz, int nseg, Filters F,
             BandPtrs coef, BandPtrs tout, float* __restrict__ low, int last, int mode, float tau)
{
    constexpr int RX = kSX + 2 * S, RY = kSY + 2 * S;   // in-plane region (halo S)
    constexpr int XR = RX - 32;                        // lanes holding a second column
    constexpr int LR = (RY + kSY - 1) / kSY;           // region rows per warp
    constexpr int NC = NF * NF;                        // channels into the z pass
    __shared__ float s_in[2][RY][RX];
    __shared__ float s_p1[2][NF][kSY][RX];
    const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int x0 = blockIdx.x * kSX, y0 = blockIdx.y * kSY;
    const int seg = blockIdx.z % nseg, r = blockIdx.z / nseg;
    const int nfirst = seg * kSegZ, nend = min(nfirst + kSegZ, class_len(nz, S, r));
    if (nfirst >= nend) return;                        // uniform per block
    const int xa = wrapi(x0 - S + lane, nx);
    const int xb = lane < XR ? wrapi(x0 - S + 32 + lane, nx) : 0;
    int rows[LR];
#pragma unroll
    for (int m = 0; m < LR; m++) rows[m] = wrapi(y0 - S + wy + kSY * m, ny);
    const int x = x0 + lane, y = y0 + wy;
    const bool ok = x < nx && y < ny;
    float pa[LR], pb[LR];                              // the next slice's region, in flight
    auto fetch = [&](int n) {
        const long long zo = (long long)wrapi(r + S * n, nz) * ny;
#pragma unroll
        for (int m = 0; m < LR; m++)
            if (wy + kSY * m < RY) {
                const float* row = in + (zo + rows[m]) * nx;
                pa[m] = __ldg(row + xa);
                pb[m] = lane < XR ? __ldg(row + xb) : 0.0f;
            }
    };
    float win[3][NC];
    fetch(nfirst - 1);
    for (int n = nfirst - 1, it = 0; n <= nend; n++, it++) {
        const int b = it & 1;
#pragma unroll
        for (int m = 0; m < LR; m++)
            if (wy + kSY * m < RY) {
                s_in[b][wy + kSY * m][lane] = pa[m];
                if (lane < XR) s_in[b][wy + kSY * m][32 + lane] = pb[m];
            }
        if (n < nend) fetch(n + 1);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < NF; i++) {                 // y pass (D_i)
            float s0 = 0.0f;
#pragma unroll
            for (int t = 0; t < 3; t++) s0 = fmaf(F.f[i][t], s_in[b][wy + t * S][lane], s0);
            s_p1[b][i][wy][lane] = s0;
            if (lane < XR) {
                float s1 = 0.0f;
#pragma unroll
                for (int t = 0; t < 3; t++) s1 = fmaf(F.f[i][t], s_in[b][wy + t * S][32 + lane], s1);
                s_p1[b][i][wy][32 + lane] = s1;
            }
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < NC; c++) { win[0][c] = win[1][c]; win[1][c] = win[2][c]; }
#pragma unroll
        for (int i = 0; i < NF; i++)                   // x pass (D_j) into the newest slot
#pragma unroll
            for (int j = 0; j < NF; j++) {
                float s0 = 0.0f;
#pragma unroll
                for (int t = 0; t < 3; t++) s0 = fmaf(F.f[j][t], s_p1[b][i][wy][lane + t * S], s0);
                win[2][NF * i + j] = s0;
            }
        if (n < nfirst + 1 || !ok) continue;           // window filling, or outside the volume
        const int z = r + S * (n - 1);                 // slots: z - S, z, z + S
        const long long q = ((long long)z * ny + y) * nx + x;
        // every v of this sample is read before the first store (the band
        // pointers may alias as far as the compiler knows), so the loads are
        // in flight together
        float vv[NC * NF];
#pragma unroll
        for (int band = 0; band < NC * NF; band++)
            vv[band] = (mode == 0 || (band == 0 && !last)) ? 0.0f : coef.p[band][q];
#pragma unroll
        for (int c = 0; c < NC; c++)
#pragma unroll
            for (int k = 0; k < NF; k++) {             // z pass (D_k)
                const int band = NF * c + k;
                float w = 0.0f;
#pragma unroll
                for (int t = 0; t < 3; t++) w = fmaf(F.f[k][t], win[t][c], w);
                if (band == 0 && !last) {
                    if (low) low[q] = w;
                    continue;
                }
                if (mode == 0) {
                    coef.p[band][q] = w;
                } else {
                    const float sv = vv[band] + w;         // v + W u
                    float a = sv;                          // alpha
                    if (!(band == 0 && last)) {
                        const float mg = fabsf(sv) - tau;
                        a = mg > 0.0f ? copysignf(mg, sv) : 0.0f;
                    }
                    const float vn = sv - a;               // v + W u - alpha
                    coef.p[band][q] = vn;
                    tout.p[band][q] = a - vn;              // alpha - v_new
                }
            }
    }
}

// The z and x merges of one synthesis level (k_merge along z into NF^2
// arrays, then along x into the NF arrays A_i), band 0 taken from `low` when
// non-null. A warp covers one row y: its lanes hold the columns from S before
// its kSX - 2S outputs to S after them, and the x taps come from the
// neighbouring lanes. blockIdx.z = seg + nseg (i + NF r).
template <int NF, int S>
__global__ void __launch_bounds__(kST)
k_syn_zx(BandPtrs bands, const float* __restrict__ low, float* __restrict__ A, long long N,
         int nx, int ny, int nz, int nseg, Filters R)
{
    constexpr int OX = kSX - 2 * S, NB = NF * NF;      // outputs per warp, bands per thread
    const int lane = threadIdx.x & 31;
    const int y = blockIdx.y * kSY + (threadIdx.x >> 5);
    const int seg = blockIdx.z % nseg, ir = blockIdx.z / nseg, i = ir % NF, r = ir / NF;
    const int nfirst = seg * kSegZ, nend = min(nfirst + kSegZ, class_len(nz, S, r));
    if (nfirst >= nend || y >= ny) return;             // whole warps (no block barrier here)
    const int xl = blockIdx.x * OX - S + lane;         // this lane's column, unwrapped
    const long long col = (long long)y * nx + wrapi(xl, nx);
    const bool out_ok = lane >= S && lane < kSX - S && xl < nx;
    const long long plane = (long long)ny * nx;
    auto src = [&](int b) -> const float* {            // b = NF j + k: band NF (NF i + j) + k
        const int band = NF * NF * i + b;
        return (band == 0 && low) ? low : bands.p[band];
    };
    float win[3][NB], nxt[NB];
    auto fetch = [&](int n, float (&d)[NB]) {
        const long long o = (long long)wrapi(r + S * n, nz) * plane + col;
#pragma unroll
        for (int b = 0; b < NB; b++) d[b] = __ldg(src(b) + o);
    };
    fetch(nfirst - 1, win[1]);
    fetch(nfirst, win[2]);
    fetch(nfirst + 1, nxt);
    for (int n = nfirst + 1; n <= nend; n++) {
#pragma unroll
        for (int b = 0; b < NB; b++) { win[0][b] = win[1][b]; win[1][b] = win[2][b]; win[2][b] = nxt[b]; }
        if (n < nend) fetch(n + 1, nxt);
        float a = 0.0f;                                // output slice r + S (n - 1)
#pragma unroll
        for (int j = 0; j < NF; j++) {
            float bm = 0.0f;                           // z merge (R_k) of channel NF i + j
#pragma unroll
            for (int k = 0; k < NF; k++)
#pragma unroll
                for (int t = 0; t < 3; t++) bm = fmaf(R.f[k][t], win[t][NF * j + k], bm);
#pragma unroll
            for (int t = 0; t < 3; t++)                // x merge (R_j)
                a = fmaf(R.f[j][t], __shfl_sync(0xffffffffu, bm, lane + (t - 1) * S), a);
        }
        if (out_ok) A[i * N + (long long)(r + S * (n - 1)) * plane + (long long)y * nx + xl] = a;
    }
}

// The y merge of one synthesis level (k_merge along y into the output, final
// = base + scale * result), streaming along y: a thread owns one column
// (x, z) and walks the rows of one residue class mod S, the three y taps of
// each output row held in a register window per input array.
constexpr int kSegY = 32;                            // output rows of one class per thread

template <int NF, int S>
__global__ void __launch_bounds__(128)
k_merge_y_stream(const float* __restrict__ A, long long N, float* __restrict__ out, int nx,
                 int ny, int nz, int nseg, Filters R, const float* __restrict__ base,
                 float scale, int final_)
{
    const int x = blockIdx.x * 128 + threadIdx.x, z = blockIdx.y;
    const int seg = blockIdx.z % nseg, r = blockIdx.z / nseg;
    const int nfirst = seg * kSegY, nend = min(nfirst + kSegY, class_len(ny, S, r));
    if (x >= nx || nfirst >= nend) return;
    const long long zo = (long long)z * ny * nx + x;
    float win[3][NF], nxt[NF];
    auto fetch = [&](int n, float (&d)[NF]) {
        const long long o = zo + (long long)wrapi(r + S * n, ny) * nx;
#pragma unroll
        for (int i = 0; i < NF; i++) d[i] = __ldg(A + i * N + o);
    };
    fetch(nfirst - 1, win[1]);
    fetch(nfirst, win[2]);
    fetch(nfirst + 1, nxt);
    for (int n = nfirst + 1; n <= nend; n++) {
#pragma unroll
        for (int i = 0; i < NF; i++) { win[0][i] = win[1][i]; win[1][i] = win[2][i]; win[2][i] = nxt[i]; }
        if (n < nend) fetch(n + 1, nxt);
        float sum = 0.0f;
#pragma unroll
        for (int i = 0; i < NF; i++)
#pragma unroll
            for (int t = 0; t < 3; t++) sum = fmaf(R.f[i][t], win[t][i], sum);
        const long long q = zo + (long long)(r + S * (n - 1)) * nx;
        if (final_) sum = (base ? __ldg(base + q) : 0.0f) + scale * sum;
        out[q] = sum;
    }
}

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
    int fused;                      // 3-D levels through the z-streaming kernels
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
    w->kind = kind; w->N = (long long)nx * ny * nz; w->fused = 1;
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

// z-streaming form of a 3-D level (three-tap banks, dilation up to
// kMaxStreamStep): analysis in one kernel; synthesis as the z + x merges in
// one kernel and the y merge (with the final base + scale) streaming along y.
static bool stream_ok(const fl_framelet* w, int step)
{
    return w->fused && w->dim == 3 && w->D.nt == 3 && step <= kMaxStreamStep;
}

static int stream_nseg(const fl_framelet* w, int step)
{
    return fl_div_up(class_len(w->nz, step, 0), kSegZ);
}

template <int NF, int S>
static void ana_stream(fl_framelet* w, const float* in, const BandPtrs& cb, const BandPtrs& tb,
                       float* low_out, int last, int mode, float tau, cudaStream_t s)
{
    const int nseg = stream_nseg(w, S);
    const dim3 grid(fl_div_up(w->nx, kSX), fl_div_up(w->ny, kSY), (unsigned)(nseg * S));
    k_ana_stream<NF, S><<<grid, kST, 0, s>>>(in, w->nx, w->ny, w->nz, nseg, w->D, cb, tb,
                                             low_out, last, mode, tau);
}

template <int NF, int S>
static void syn_stream(fl_framelet* w, const BandPtrs& cb, const float* low, float* dst,
                       const float* base, float scale, int final_, cudaStream_t s)
{
    const int nseg = stream_nseg(w, S);
    const long long N = w->N;
    float* A = w->work;                                // NF arrays
    const dim3 grid(fl_div_up(w->nx, kSX - 2 * S), fl_div_up(w->ny, kSY),
                    (unsigned)(nseg * NF * S));
    k_syn_zx<NF, S><<<grid, kST, 0, s>>>(cb, low, A, N, w->nx, w->ny, w->nz, nseg, w->R);
    const int nsegy = fl_div_up(class_len(w->ny, S, 0), kSegY);
    const dim3 gy(fl_div_up(w->nx, 128), w->nz, (unsigned)(nsegy * S));
    k_merge_y_stream<NF, S><<<gy, 128, 0, s>>>(A, N, dst, w->nx, w->ny, w->nz, nsegy, w->R, base,
                                               scale, final_);
}

template <int NF>
static void stream_level(fl_framelet* w, int step, bool analysis_pass, const float* in,
                         const BandPtrs& cb, const BandPtrs& tb, float* low_out, int last,
                         int mode, float tau, const float* low, float* dst, const float* base,
                         float scale, int final_, cudaStream_t s)
{
    switch (step) {
#define FL_STREAM_CASE(SS)                                                                   \
    case SS:                                                                                 \
        if (analysis_pass) ana_stream<NF, SS>(w, in, cb, tb, low_out, last, mode, tau, s);   \
        else syn_stream<NF, SS>(w, cb, low, dst, base, scale, final_, s);                    \
        break;
        FL_STREAM_CASE(1)
        FL_STREAM_CASE(2)
        FL_STREAM_CASE(4)
        FL_STREAM_CASE(8)
#undef FL_STREAM_CASE
    }
}

template <int NF, int NT>
static void run_analysis_level(fl_framelet* w, const float* in, int step, const BandPtrs& cb,
                               const BandPtrs& tb, float* low_out, int last, int mode, float tau,
                               cudaStream_t s)
{
    if constexpr (NT == 3)
        if (stream_ok(w, step)) {
            stream_level<NF>(w, step, true, in, cb, tb, low_out, last, mode, tau, nullptr,
                             nullptr, nullptr, 1.0f, 0, s);
            return;
        }
    analysis_level<NF, NT>(w, in, step, cb, tb, low_out, last, mode, tau, s);
}

template <int NF, int NT>
static void run_synthesis_level(fl_framelet* w, const BandPtrs& cb, const float* low, float* dst,
                                int step, const float* base, float scale, int final_,
                                cudaStream_t s)
{
    if constexpr (NT == 3)
        if (stream_ok(w, step)) {
            stream_level<NF>(w, step, false, nullptr, cb, cb, nullptr, 0, 0, 0.0f, low, dst,
                             base, scale, final_, s);
            return;
        }
    synthesis_level<NF, NT>(w, cb, low, dst, step, base, scale, final_, s);
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
            run_analysis_level<3, 3>(w, in, step, cb, tb, low_out, last, mode, tau, s);
        else if (w->kind == FL_FRAMELET_CUBIC)
            run_analysis_level<5, 5>(w, in, step, cb, tb, low_out, last, mode, tau, s);
        else
            run_analysis_level<2, 3>(w, in, step, cb, tb, low_out, last, mode, tau, s);
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
            run_synthesis_level<3, 3>(w, cb, low, dst, step, bs, sc, final_, s);
        else if (w->kind == FL_FRAMELET_CUBIC)
            run_synthesis_level<5, 5>(w, cb, low, dst, step, bs, sc, final_, s);
        else
            run_synthesis_level<2, 3>(w, cb, low, dst, step, bs, sc, final_, s);
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

extern "C" int fl_framelet_option(fl_framelet* w, int option, int value)
{
    if (!w) return fl_set_error(FL_ERR_INVALID, "fl_framelet_option: null framelet");
    if (option != FL_FRAMELET_OPT_FUSED)
        return fl_set_error(FL_ERR_INVALID, "fl_framelet_option: unknown option %d", option);
    w->fused = value ? 1 : 0;
    return fl_set_error(FL_OK, "");
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
