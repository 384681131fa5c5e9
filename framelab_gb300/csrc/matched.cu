// matched.cu -- matched Siddon projector pair (FL_MODEL_MATCHED).
//
// Matrix. For ray r and voxel V = (ix, iy, iz) the entry is
//     A[r,V] = c_r * w_rV,   c_r = scale * |D - S|,
//     w_rV   = fl( min_a U_a(V) - max_a L_a(V) )
// when positive, where L_a / U_a are the crossings of the planes at which the
// ray enters / leaves V's slab on axis a, evaluated in the frame of the
// segment of the ray's dominant axis that holds V (fl_plan.h,
// matched_dev.cuh). This is the exact Siddon intersection length with FP32
// arithmetic on small, anchored crossing parameters.
//
// Forward: one thread per ray walks each segment's sub-box, stepping the
// smallest next crossing (an incremental Siddon walk); the segment it
// accumulates inside V is exactly w_rV above.
//
// Adjoint: one thread per voxel column gathers over the rays whose detector
// window covers the column and evaluates the same w_rV from the same table
// entries in the same frame -- the exact transpose, with no atomics.
#include <algorithm>

#include <type_traits>

#include "fl_trace.h"
#include "fl_common.cuh"
#include "fl_plan.h"
#include "matched_dev.cuh"

namespace {

// ---------------------------------------------------------------------------
// Forward kernels. Block (32, 4): 32 adjacent detector columns x 4 rows of one
// view, so a warp's rays are neighbours and their gathers share cache lines.
// ---------------------------------------------------------------------------
// MIRROR (scans symmetric about the source plane, fl_plan::zmirror): X is
// z-folded; the block walks only the rows ib < nb/2 and also produces each
// ray's mirrored companion, row nb-1-ib, from the same walk. yfold selects
// the folded sinogram layout (pairs of rows ib and nb-1-ib) for the output.
template <typename TX, typename TY, bool MIRROR>
__global__ void __launch_bounds__(128, 8)
k_fwd_cone(const TX* __restrict__ X, TY* __restrict__ y, const ColEntry* __restrict__ col,
           const float* __restrict__ colr, const RowEntry* __restrict__ row,
           const int* __restrict__ vframe, int nx, int ny, int nz, int na, int nb,
           long long nper, float scale, int cr_power, const int* __restrict__ skip,
           const float* __restrict__ xscale, int yfold)
{
    if (skip && *skip) return;
    // grid y = view, grid z = band of detector rows: the blocks that run
    // together cover all views of one row band, whose rays share a z-slab of
    // the volume, so the gathers stay in L2
    int ia = blockIdx.x * blockDim.x + threadIdx.x;
    int iv = blockIdx.y;
    int ib = blockIdx.z * blockDim.y + threadIdx.y;
    if (ia >= na || ib >= (MIRROR ? nb / 2 : nb)) return;
    const ColEntry* ce = col + (long long)iv * na + ia;
    const RowEntry* re = row + (long long)iv * nb + ib;
    const TX* x = X + (long long)vframe[iv] * nper;
    float accm = 0.0f;
    float acc = walk<TX, true, false, MIRROR>(x, ce, &re->z, nx, ny, nz, nullptr,
                                              &accm, nper);
    float cr = ray_cr(scale, colr[(long long)iv * na + ia], __ldg(&re->dz2));
    if (xscale) { acc *= *xscale; accm *= *xscale; }
    float out = cr * acc;
    if (cr_power == 2) out = cr * out;
    if (MIRROR) {
        float om = cr * accm;
        if (cr_power == 2) om = cr * om;
        if (yfold) {
            Store<TY>::st2(y + 2 * (((long long)iv * (nb / 2) + ib) * na + ia), out, om);
        } else {
            Store<TY>::st(y + ((long long)iv * nb + ib) * na + ia, out);
            Store<TY>::st(y + ((long long)iv * nb + (nb - 1 - ib)) * na + ia, om);
        }
    } else {
        Store<TY>::st(y + ((long long)iv * nb + ib) * na + ia, out);
    }
}

// Half-turn form (fl_plan::rot, on a z-mirror plan): the block walks rows
// ib < nb/2 of views iv < nv/2 only; each walk also yields the rays of view
// iv + nv/2 at the same column and rows (the turned ray, over the turned
// voxels), all four with the walked ray's c_r. yfold writes the
// backprojection's input layout for these plans: per (iv < nv/2, ib < nb/2,
// ia) the 4 values (views iv, iv + nv/2; rows ib, nb-1-ib) side by side
// (k_weight_packed<TY, 2>).
template <typename TX, typename TY>
__global__ void __launch_bounds__(128, 8)
k_fwd_quad(const TX* __restrict__ X, TY* __restrict__ y, const ColEntry* __restrict__ col,
           const float* __restrict__ colr, const RowEntry* __restrict__ row, int nx, int ny,
           int nz, int na, int nb, int nv, long long nper, float scale, int cr_power,
           const int* __restrict__ skip, const float* __restrict__ xscale, int yfold)
{
    if (skip && *skip) return;
    const int ia = blockIdx.x * blockDim.x + threadIdx.x;
    const int iv = blockIdx.y;                      // < nv / 2
    const int ib = blockIdx.z * blockDim.y + threadIdx.y;
    const int nbh = nb / 2, hv = nv / 2;
    if (ia >= na || ib >= nbh) return;
    const ColEntry* ce = col + (long long)iv * na + ia;
    const RowEntry* re = row + (long long)iv * nb + ib;
    float2 a, r;
    walk_quad<TX>(X, ce, &re->z, nx, ny, nz, &a, &r, nper);
    float cr = ray_cr(scale, colr[(long long)iv * na + ia], __ldg(&re->dz2));
    if (xscale) {
        const float xs = *xscale;
        a.x *= xs; a.y *= xs; r.x *= xs; r.y *= xs;
    }
    float o[4] = {cr * a.x, cr * a.y, cr * r.x, cr * r.y};
    if (cr_power == 2)
        for (int k = 0; k < 4; k++) o[k] = cr * o[k];
    if (yfold) {                        // the 4 values of the pair of views side by side
        const long long u = 4 * (((long long)iv * nbh + ib) * na + ia);
        Store<TY>::st2(y + u, o[0], o[1]);
        Store<TY>::st2(y + u + 2, o[2], o[3]);
    } else {
        Store<TY>::st(y + ((long long)iv * nb + ib) * na + ia, o[0]);
        Store<TY>::st(y + ((long long)iv * nb + (nb - 1 - ib)) * na + ia, o[1]);
        Store<TY>::st(y + ((long long)(iv + hv) * nb + ib) * na + ia, o[2]);
        Store<TY>::st(y + ((long long)(iv + hv) * nb + (nb - 1 - ib)) * na + ia, o[3]);
    }
}

// Quarter-turn form (fl_plan::rot4): the block walks rows ib < nb/2 of views
// iv < nv/4; each walk yields the rays of views iv + j nv/4 (j = 0..3) at the
// same column and rows, all eight with the walked ray's c_r. yfold writes the
// backprojection's input layout for these plans: per (iv < nv/4, ib < nb/2,
// ia) the 8 values (view iv + j nv/4, rows ib / nb-1-ib) side by side
// (k_weight_packed<TY, 4>).
template <typename TX, typename TY>
__global__ void __launch_bounds__(128, 8)
k_fwd_oct(const TX* __restrict__ X, TY* __restrict__ y, const ColEntry* __restrict__ col,
          const float* __restrict__ colr, const RowEntry* __restrict__ row, int n, int nz,
          int na, int nb, int nv, long long nper, float scale, int cr_power,
          const int* __restrict__ skip, const float* __restrict__ xscale, int yfold)
{
    if (skip && *skip) return;
    const int ia = blockIdx.x * blockDim.x + threadIdx.x;
    const int iv = blockIdx.y;                      // < nv / 4
    const int ib = blockIdx.z * blockDim.y + threadIdx.y;
    const int nbh = nb / 2, qv = nv / 4;
    if (ia >= na || ib >= nbh) return;
    const ColEntry* ce = col + (long long)iv * na + ia;
    const RowEntry* re = row + (long long)iv * nb + ib;
    float2 a[4];
    walk_oct<TX>(X, ce, &re->z, n, nz, a, nper);
    float cr = ray_cr(scale, colr[(long long)iv * na + ia], __ldg(&re->dz2));
    const float xs = xscale ? *xscale : 1.0f;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        float o0 = a[j].x, o1 = a[j].y;
        if (xscale) { o0 *= xs; o1 *= xs; }
        o0 = cr * o0; o1 = cr * o1;
        if (cr_power == 2) { o0 = cr * o0; o1 = cr * o1; }
        const long long vj = iv + (long long)j * qv;
        if (yfold) {                    // the 8 values of the orbit side by side
            Store<TY>::st2(y + 8 * (((long long)iv * nbh + ib) * na + ia) + 2 * j, o0, o1);
        } else {
            Store<TY>::st(y + (vj * nb + ib) * na + ia, o0);
            Store<TY>::st(y + (vj * nb + (nb - 1 - ib)) * na + ia, o1);
        }
    }
}

// Reflection forms (fl_plan::refl; NR = 4: quarter turns, square grid; NR =
// 2: half turn): the block walks rows ib < nb/2 of the slots s (refl_slot:
// the walked views 0 .. ov); each walk yields the rays of its 4 NR images
// (refl_image, rows ib and nb-1-ib), all with the walked ray's c_r. yfold
// writes the backprojection's input layout for these plans (two planes,
// ReflGeom; k_weight_packed_refl).
template <typename TX, typename TY, int NR>
__global__ void __launch_bounds__(128, NR == 4 ? 6 : 8)
k_fwd_refl(const TX* __restrict__ X, TY* __restrict__ y, const ColEntry* __restrict__ col,
           const float* __restrict__ colr, const RowEntry* __restrict__ row, int nx, int ny,
           int nz, int na, int nb, int nv, long long nper, float scale, int cr_power,
           const int* __restrict__ skip, const float* __restrict__ xscale, int yfold)
{
    if (skip && *skip) return;
    const ReflGeom g = refl_geom(NR, nv, na, nb);
    const int ia = blockIdx.x * blockDim.x + threadIdx.x;
    const int sl = blockIdx.y;                      // < g.slots
    const int ib = blockIdx.z * blockDim.y + threadIdx.y;
    if (ia >= na || ib >= g.nbh) return;
    int v, vt, a, stride;
    long long off;
    if (!refl_slot(g, sl, ia, v, vt, a, off, stride)) return;
    const ColEntry* ce = col + (long long)vt * na + a;
    const RowEntry* re = row + (long long)vt * nb + ib;
    float2 acc[2 * NR];
    walk_refl<TX, NR>(X, ce, &re->z, nx, ny, nz, acc, nper);
    const float cr = ray_cr(scale, colr[(long long)vt * na + a], __ldg(&re->dz2));
    const float xs = xscale ? *xscale : 1.0f;
#pragma unroll
    for (int k = 0; k < 2 * NR; k++) {
        float o0 = acc[k].x, o1 = acc[k].y;
        if (xscale) { o0 *= xs; o1 *= xs; }
        o0 = cr * o0; o1 = cr * o1;
        if (cr_power == 2) { o0 = cr * o0; o1 = cr * o1; }
        if (yfold) {                    // the orbit's two planes of 2 NR values
            Store<TY>::st2(y + (k < NR ? 0 : g.plane) + off +
                               (long long)g.vpr * ((long long)ib * stride + ia) + 2 * (k % NR),
                           o0, o1);
        } else {
            long long vk; int ak;
            refl_image<NR>(k, v, a, na, nv, vk, ak);
            Store<TY>::st(y + (vk * nb + ib) * na + ak, o0);
            Store<TY>::st(y + (vk * nb + (nb - 1 - ib)) * na + ak, o1);
        }
    }
}

template <typename TX, typename TY>
__global__ void __launch_bounds__(128, 8)
k_fwd_fan(const TX* __restrict__ X, const TX* __restrict__ XT, TY* __restrict__ y,
          const ColEntry* __restrict__ col, const float* __restrict__ colr,
          const int* __restrict__ vframe, int nx, int ny, int na, int nv, long long nper,
          float scale, int cr_power, const int* __restrict__ skip,
          const float* __restrict__ xscale)
{
    if (skip && *skip) return;
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (long long)na * nv) return;
    int iv = (int)(r / na);
    const TX* x = X + (long long)vframe[iv] * nper;
    const TX* xt = XT + (long long)vframe[iv] * nper;
    float a1[1];
    walk_fan<TX, 1>(x, xt, &col[r].x, &col[r].y, nx, ny, a1, nper);
    float acc = a1[0];
    float cr = ray_cr(scale, colr[r], 0.0f);
    if (xscale) acc *= *xscale;
    float out = cr * acc;
    if (cr_power == 2) out = cr * out;
    Store<TY>::st(y + r, out);
}

// Fan forward of a turn plan (G = 2 or 4, one frame): blocks of kFanBlock
// threads, L parts per ray (fan_turn_forward_block, fl_plan_fan_lanes).
template <typename TX, typename TY, int G>
__global__ void __launch_bounds__(kFanBlock, 3)
k_fwd_fan_turn(const TX* __restrict__ X, const TX* __restrict__ XT, TY* __restrict__ y,
               const ColEntry* __restrict__ col, const float* __restrict__ colr, int nx, int ny,
               int na, int nv, float scale, int cr_power, const int* __restrict__ skip,
               const float* __restrict__ xscale, int ypack, int L)
{
    if (skip && *skip) return;                 // uniform (one flag for the launch)
    fan_turn_forward_block<TX, TY, G>(X, XT, y, col, colr, nx, ny, na, nv, scale, cr_power,
                                      xscale, ypack, (long long)blockIdx.x * (kFanBlock / L), L);
}

// Fan reflection forms (NR = 1, 2 or 4, one frame): forward blocks of
// kFanBlock threads, L parts per walked ray (fan_refl_forward_block).
template <typename TX, typename TY, int NR>
__global__ void __launch_bounds__(kFanBlock, 3)
k_fwd_fan_refl(const TX* __restrict__ X, const TX* __restrict__ XT, TY* __restrict__ y,
               const ColEntry* __restrict__ col,
               const float* __restrict__ colr, int nx, int ny, int na, int nv, float scale,
               int cr_power, const int* __restrict__ skip, const float* __restrict__ xscale,
               int ypack, int L)
{
    if (skip && *skip) return;                 // uniform (one flag for the launch)
    fan_refl_forward_block<TX, TY, NR>(X, XT, y, col, colr, nx, ny, na, nv, scale, cr_power, xscale,
                                       ypack, (long long)blockIdx.x * (kFanBlock / L), L);
}

// Fan reflection backprojection: blocks of kFanX PB x PB pixel blocks of one
// block row x kTurnGroups view groups (fan_refl_adjoint_block).
template <typename TX, int NR, int PB, int NG>
__global__ void __launch_bounds__(kFanX * NG)
k_adj_fan_refl(TX* __restrict__ X, const float* __restrict__ ywp,
               const ColEntry* __restrict__ col, const ViewEntry* __restrict__ view, DetGrid G,
               int nx, int ny, int na, int nv, const int* __restrict__ skip)
{
    if (skip && *skip) return;
    __shared__ float smem[NG * 2 * NR * PB * PB * kFanX];
    fan_refl_adjoint_block<TX, NR, PB, NG>(X, ywp, col, view, G, nx, ny, na, nv,
                                           blockIdx.x * kFanX, blockIdx.y, smem);
}

// Transposed copy of fan images (all frames): xt[f nper + x ny + y] =
// x[f nper + y nx + x], through a 32 x 32 tile in shared memory.
template <typename T>
__global__ void __launch_bounds__(256)
k_transpose_fan(const T* __restrict__ x, T* __restrict__ xt, int nx, int ny, long long nper)
{
    __shared__ T tile[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    const T* src = x + (long long)blockIdx.z * nper;
    T* dst = xt + (long long)blockIdx.z * nper;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int yy = by + k, xx = bx + threadIdx.x;
        if (yy < ny && xx < nx) tile[k][threadIdx.x] = src[(long long)yy * nx + xx];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int xx = bx + k, yy = by + threadIdx.x;
        if (xx < nx && yy < ny) dst[(long long)xx * ny + yy] = tile[threadIdx.x][k];
    }
}

__global__ void __launch_bounds__(128)
k_count(int32_t* __restrict__ cnt, const ColEntry* __restrict__ col,
        const RowEntry* __restrict__ row, int nx, int ny, int nz, int na, int nb, int nv,
        int three)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long nr = (long long)na * nb * nv;
    if (r >= nr) return;
    int ia = (int)(r % na);
    long long q = r / na;
    int ib = (int)(q % nb);
    int iv = (int)(q / nb);
    const ColEntry* ce = col + (long long)iv * na + ia;
    int c = 0;
    if (three) {
        const RowEntry* re = row + (long long)iv * nb + ib;
        walk<float, true, true>(nullptr, ce, &re->z, nx, ny, nz, &c);
    } else {
        walk<float, false, true>(nullptr, ce, &ce->y, nx, ny, 1, &c);
    }
    cnt[r] = c;
}

// Folded yw for a z-mirror plan: the pair (c_r y[ib], c_r y[nb-1-ib]) of rows
// ib < nb/2, both with the walked row's c_r (equal to the mirror's: its d_z is
// the exact negation).
// pv: view iv takes c_r of view iv % pv, the ray it is defined by (pv = nv:
// turn plans pack their input with k_weight_packed instead).
template <typename TY>
__global__ void k_weight_fold(float* __restrict__ yw, const TY* __restrict__ y,
                              const float* __restrict__ colr, const RowEntry* __restrict__ row,
                              int na, int nb, long long npairs, float scale, int pv)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= npairs) return;
    const int nbh = nb / 2;
    int ia = (int)(r % na);
    long long q = r / na;
    int ib = (int)(q % nbh);
    int iv = (int)(q / nbh);
    const int ivc = iv % pv;
    float cr = ray_cr(scale, colr[(long long)ivc * na + ia], row[(long long)ivc * nb + ib].dz2);
    float a = Store<TY>::ld_plain(y + ((long long)iv * nb + ib) * na + ia);
    float b = Store<TY>::ld_plain(y + ((long long)iv * nb + (nb - 1 - ib)) * na + ia);
    Store<float>::st2(yw + 2 * r, cr * a, cr * b);
}

// Packed yw of a half- (G = 2) or quarter-turn (G = 4) plan: for
// r = (iv < nv/G, ib < nb/2, ia) the 2 G values c_r y of views iv + j nv/G
// (j < G), rows ib and nb-1-ib, with c_r of view iv (the ray they are all
// defined by).
template <typename TY, int G>
__global__ void k_weight_packed(float* __restrict__ yw, const TY* __restrict__ y,
                                const float* __restrict__ colr, const RowEntry* __restrict__ row,
                                int na, int nb, int nv, long long npack, float scale)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= npack) return;
    const int nbh = nb / 2, pv = nv / G;
    const int ia = (int)(r % na);
    const long long q = r / na;
    const int ib = (int)(q % nbh);
    const int iv = (int)(q / nbh);
    const float cr = ray_cr(scale, colr[(long long)iv * na + ia], row[(long long)iv * nb + ib].dz2);
#pragma unroll
    for (int j = 0; j < G; j++) {
        const long long vj = iv + (long long)j * pv;
        const float a = Store<TY>::ld_plain(y + (vj * nb + ib) * na + ia);
        const float b = Store<TY>::ld_plain(y + (vj * nb + (nb - 1 - ib)) * na + ia);
        Store<float>::st2(yw + 2 * G * r + 2 * j, cr * a, cr * b);
    }
}

// Packed yw of a reflection form: for each walked ray (refl_slot) and row ib
// < nb/2 the 4 NR values c_r y of its images (refl_image, rows ib and
// nb-1-ib), with c_r of the walked ray, in the two planes of ReflGeom.
template <typename TY, int NR>
__global__ void k_weight_packed_refl(float* __restrict__ yw, const TY* __restrict__ y,
                                     const float* __restrict__ colr,
                                     const RowEntry* __restrict__ row, int na, int nb, int nv,
                                     long long npack, float scale)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= npack) return;                         // npack = slots * nb/2 * na
    const ReflGeom g = refl_geom(NR, nv, na, nb);
    const int ia = (int)(r % na);
    const long long q = r / na;
    const int ib = (int)(q % g.nbh);
    const int sl = (int)(q / g.nbh);
    int v, vt, a, stride;
    long long off;
    if (!refl_slot(g, sl, ia, v, vt, a, off, stride)) return;
    const float cr = ray_cr(scale, colr[(long long)vt * na + a], row[(long long)vt * nb + ib].dz2);
    const long long at = off + (long long)g.vpr * ((long long)ib * stride + ia);
#pragma unroll
    for (int k = 0; k < 2 * NR; k++) {
        long long vk; int ak;
        refl_image<NR>(k, v, a, na, nv, vk, ak);
        const float p0 = Store<TY>::ld_plain(y + (vk * nb + ib) * na + ak);
        const float p1 = Store<TY>::ld_plain(y + (vk * nb + (nb - 1 - ib)) * na + ak);
        Store<float>::st2(yw + (k < NR ? 0 : g.plane) + at + 2 * (k % NR), cr * p0, cr * p1);
    }
}

// Packed yw of a fan turn plan (G = 2 or 4): for r = (iv < nv/G, ia) the G
// values c_r y of views iv + j nv/G at column ia, with c_r of view iv.
template <typename TY, int G>
__global__ void k_weight_fan_packed(float* __restrict__ yw, const TY* __restrict__ y,
                                    const float* __restrict__ colr, int na, int nv,
                                    long long npack, float scale)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= npack) return;
    const int gv = nv / G;
    const int iv = (int)(r / na), ia = (int)(r - (long long)iv * na);
    const float cr = ray_cr(scale, colr[r], 0.0f);
#pragma unroll
    for (int j = 0; j < G; j++)
        yw[G * r + j] = cr * Store<TY>::ld_plain(y + ((long long)iv + (long long)j * gv) * na + ia);
}

// Packed yw of a fan reflection form (NR = 1, 2, 4): for each walked ray
// (refl_slot of FanReflGeom) the 2 NR values c_r y of its images
// (refl_image), with c_r of the walked ray.
template <typename TY, int NR>
__global__ void k_weight_fan_refl(float* __restrict__ yw, const TY* __restrict__ y,
                                  const float* __restrict__ colr, int na, int nv,
                                  long long nslot, float scale)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nslot) return;                         // nslot = slots * na
    const FanReflGeom g = fan_refl_geom(NR, nv, na);
    const int sl = (int)(r / na), ia = (int)(r - (long long)sl * na);
    int v, vt, a, stride;
    long long off;
    if (!refl_slot(g, sl, ia, v, vt, a, off, stride)) return;
    const float cr = ray_cr(scale, colr[(long long)vt * na + a], 0.0f);
#pragma unroll
    for (int k = 0; k < 2 * NR; k++) {
        long long vk; int ak;
        refl_image<NR>(k, v, a, na, nv, vk, ak);
        yw[off + (long long)(2 * NR) * ia + k] = cr * Store<TY>::ld_plain(y + vk * na + ak);
    }
}

// z-fold / unfold of volumes (all frames): pair r = (iz < nz/2, iy, ix) of a
// frame holds voxel (ix, iy, iz) and its mirror (ix, iy, nz-1-iz).
template <typename T>
__global__ void k_fold(const T* __restrict__ src, T* __restrict__ dst, long long nxy, int nz,
                       long long npairs_frame, long long npairs, int unfold)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < npairs;
         i += (long long)gridDim.x * blockDim.x) {
        const long long f = i / npairs_frame, r = i % npairs_frame;
        const long long iz = r / nxy, q = r % nxy;
        const long long base = f * 2 * npairs_frame;
        const long long lo = base + iz * nxy + q, hi = base + (nz - 1 - iz) * nxy + q;
        if (unfold) {
            const T a = src[base + 2 * r], b = src[base + 2 * r + 1];
            dst[lo] = a; dst[hi] = b;
        } else {
            const T a = src[lo], b = src[hi];
            dst[base + 2 * r] = a; dst[base + 2 * r + 1] = b;
        }
    }
}

// Fold / unfold of a half- or quarter-turn plan's volume (one frame,
// nx x ny x nz, nx and ny multiples of 4): the tiled pair r (fl_plan.h) holds
// voxel (x, y, z) and its mirror (x, y, nz-1-z).
template <typename T>
__global__ void k_fold_tiled(const T* __restrict__ src, T* __restrict__ dst, int nx, int ny,
                             int nz, long long npairs, int unfold)
{
    const long long nn = (long long)nx * ny;
    const int nx4 = nx >> 2;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < npairs;
         r += (long long)gridDim.x * blockDim.x) {
        const long long z = r / nn;
        const int rem = (int)(r - z * nn), tile = rem >> 4, w = rem & 15;
        const int y = (tile / nx4) * 4 + (w >> 2), x = (tile % nx4) * 4 + (w & 3);
        const long long lo = z * nn + (long long)y * nx + x;
        const long long hi = (nz - 1 - z) * nn + (long long)y * nx + x;
        if (unfold) {
            const T a = src[2 * r], b = src[2 * r + 1];
            dst[lo] = a; dst[hi] = b;
        } else {
            const T a = src[lo], b = src[hi];
            dst[2 * r] = a; dst[2 * r + 1] = b;
        }
    }
}

// yw = c_r * y  (the adjoint gathers pre-weighted sinogram values)
template <typename TY>
__global__ void k_weight(float* __restrict__ yw, const TY* __restrict__ y,
                         const float* __restrict__ colr, const RowEntry* __restrict__ row,
                         int na, int nb, long long nrays, float scale, int three)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrays) return;
    int ia = (int)(r % na);
    long long q = r / na;
    int ib = (int)(q % nb);
    int iv = (int)(q / nb);
    float dz2 = three ? row[(long long)iv * nb + ib].dz2 : 0.0f;
    float cr = ray_cr(scale, colr[(long long)iv * na + ia], dz2);
    yw[r] = cr * Store<TY>::ld_plain(y + r);
}


// ---------------------------------------------------------------------------
// Fan adjoint: one thread per (pixel, frame).
// ---------------------------------------------------------------------------
// Fan adjoint of one P x P pixel block of one frame per thread. Small images
// (GROUPED, P = 1): blocks of kFanX x kFanGroups threads, thread (x, g)
// gathers view group g and group 0 writes the combined sums, so that four
// times as many threads share the views. Large images (P = 2): blocks of 128
// threads, each gathering all groups itself. Both give the same bits.

template <typename TX, int P, bool GROUPED>
__global__ void __launch_bounds__(128)
k_adj_fan(TX* __restrict__ X, const float* __restrict__ yw, const ColEntry* __restrict__ col,
          const ViewEntry* __restrict__ view, const int* __restrict__ idY,
          const int* __restrict__ Nv, int tmp_size, DetGrid G, int nx, int ny, int na,
          const int* __restrict__ skip)
{
    if (skip && *skip) return;                 // uniform (one flag for the launch)
    const int ix0 = P * (blockIdx.x * blockDim.x + threadIdx.x);
    const int iy0 = P * blockIdx.y;
    const int it = blockIdx.z;
    float acc[P][P];
    if (GROUPED) {
#pragma unroll
        for (int j = 0; j < P; j++)
#pragma unroll
            for (int i = 0; i < P; i++) acc[j][i] = 0.0f;
        if (ix0 < nx)
            fan_block_gather<P, P>(acc, yw, col, view, idY + it * tmp_size, Nv[it], G, ix0, iy0,
                                   nx, ny, na, threadIdx.y);
        if (!fan_combine_groups<P, kFanX>(acc) || ix0 >= nx) return;
    } else {
        if (ix0 >= nx) return;
        fan_block_gather_all<P, P>(acc, yw, col, view, idY + it * tmp_size, Nv[it], G, ix0, iy0,
                                   nx, ny, na);
    }
    TX* xf = X + (long long)it * nx * ny;
#pragma unroll
    for (int j = 0; j < P; j++)
#pragma unroll
        for (int i = 0; i < P; i++)
            if (iy0 + j < ny && ix0 + i < nx)
                Store<TX>::st(xf + (long long)(iy0 + j) * nx + ix0 + i, acc[j][i]);
}

// Fan adjoint of a turn plan (G = 2 or 4, one frame): blocks of kFanX P x P
// blocks of primary pixels x kTurnGroups view groups (fan_turn_adjoint_block;
// the bits do not depend on P).
template <typename TX, int G, int P, int NG>
__global__ void __launch_bounds__(kFanX * NG)
k_adj_fan_turn(TX* __restrict__ X, const float* __restrict__ ywp,
               const ColEntry* __restrict__ col, const ViewEntry* __restrict__ view, DetGrid D,
               int nx, int ny, int na, int nv, const int* __restrict__ skip)
{
    if (skip && *skip) return;                 // uniform (one flag for the launch)
    fan_turn_adjoint_block<TX, G, P, NG>(X, ywp, col, view, D, nx, ny, na, nv,
                                         blockIdx.x * kFanX * P, blockIdx.y * P);
}

// ---------------------------------------------------------------------------
// Cone adjoint: one thread per voxel column (ix, iy) and a run of TZ voxels in
// z (block 32 x 4 columns). Per view, the thread finds the detector columns
// whose rays can cross its column (projection of the column's four corners),
// and per such column the xy crossing interval [l, h] of the ray family. For
// each voxel k of the run it then visits only the detector rows whose ray is
// inside that voxel's z range somewhere in [l, h], and adds w_rV * (c_r y_r)
// with w_rV evaluated exactly as in the forward walk. The TZ accumulators are
// registers (k is a compile-time index).
// ---------------------------------------------------------------------------
// The backprojection input (pre-weighted sinogram) is FP32, or FP16 in the
// mixed CGLS form. ld_in<TW, N> reads N consecutive values of one orbit from
// an address aligned to N elements, as one vector load, and widens them.
template <typename TW, int N>
__device__ __forceinline__ void ld_in(const TW* __restrict__ p, float (&v)[N]);

template <>
__device__ __forceinline__ void ld_in<float, 1>(const float* __restrict__ p, float (&v)[1])
{
    v[0] = __ldg(p);
}
template <>
__device__ __forceinline__ void ld_in<float, 2>(const float* __restrict__ p, float (&v)[2])
{
    const float2 u = __ldg(reinterpret_cast<const float2*>(p));
    v[0] = u.x; v[1] = u.y;
}
template <>
__device__ __forceinline__ void ld_in<float, 4>(const float* __restrict__ p, float (&v)[4])
{
    const float4 u = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = u.x; v[1] = u.y; v[2] = u.z; v[3] = u.w;
}
template <>
__device__ __forceinline__ void ld_in<float, 8>(const float* __restrict__ p, float (&v)[8])
{
    // one 32-byte load (sm_100 and later; orbits are 32-byte aligned)
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]),
          "=f"(v[7])
        : "l"(p));
}
template <>
__device__ __forceinline__ void ld_in<__half, 1>(const __half* __restrict__ p, float (&v)[1])
{
    v[0] = __half2float(__ldg(p));
}
template <>
__device__ __forceinline__ void ld_in<__half, 2>(const __half* __restrict__ p, float (&v)[2])
{
    const float2 a = __half22float2(__ldg(reinterpret_cast<const __half2*>(p)));
    v[0] = a.x; v[1] = a.y;
}
template <>
__device__ __forceinline__ void ld_in<__half, 4>(const __half* __restrict__ p, float (&v)[4])
{
    const uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
template <>
__device__ __forceinline__ void ld_in<__half, 8>(const __half* __restrict__ p, float (&v)[8])
{
    const uint4 u = __ldg(reinterpret_cast<const uint4*>(p));
    const unsigned w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&w[k]));
        v[2 * k] = a.x; v[2 * k + 1] = a.y;
    }
}

// Candidate rays of one detector column for the TZ voxels of a run. MODE +1:
// the run lies above the source plane, so every ray that reaches it rises
// (A_z increasing in k); MODE -1: below, every such ray falls; MODE 0: the run
// straddles the source plane (general min/max). The other orientation's rays
// get w <= 0 from the specialised formula, as they miss the run.
template <int MODE, int TZ, typename TW>
__device__ __forceinline__ void adj_rows(float (&acc)[TZ], int nk, int z0, float l, float h,
                                         float e1, float e2, float s1, float s2,
                                         const AxisEntry* __restrict__ rv, float bh, float be,
                                         const TW* __restrict__ ycol, int na, int nb)
{
    float mn = fminf(e1, e2), mx = fmaxf(e1, e2);   // row span at plane k
#pragma unroll
    for (int k = 0; k < TZ; k++) {
        if (k >= nk) break;
        e1 += s1; e2 += s2;
        const float mn1 = fminf(e1, e2), mx1 = fmaxf(e1, e2);   // plane k + 1
        const int blo = max(__float2int_ru(fminf(mn, mn1) - 0.02f), 0);
        const int bhi = min(__float2int_rd(fmaxf(mx, mx1) + 0.02f), nb - 1);
        mn = mn1; mx = mx1;
        const float fk0 = (float)(z0 + k), fk1 = (float)(z0 + k + 1);
        for (int ib = blo; ib <= bhi; ib++) {
            if (!FL_IN(ib, nb)) continue;
            const AxisEntry re = rv[ib];                 // (inv_z, off_z) of row ib
            float yv1[1];
            ld_in<TW, 1>(ycol + (long long)ib * na, yv1);
            const float yval = yv1[0];
            const float2 azp = row_planes(re, fk0, fk1, bh, be);
            const float az0 = azp.x, az1 = azp.y;
            float l2, h2;
            if (MODE > 0)      { l2 = fmaxf(l, az0); h2 = fminf(h, az1); }
            else if (MODE < 0) { l2 = fmaxf(l, az1); h2 = fminf(h, az0); }
            else { l2 = fmaxf(l, fminf(az0, az1)); h2 = fminf(h, fmaxf(az0, az1)); }
            // w <= 0 (the ray misses voxel k) adds exactly 0 for finite y
            acc[k] = fmaf(fmaxf(h2 - l2, 0.0f), yval, acc[k]);
        }
    }
}

// z-mirror form: rows limited to the walked half (nb here is nb/2); ycol
// points into the folded sinogram (pairs of rows ib and nb-1-ib, row stride
// 2*na); acc[k] holds the voxel k and its mirror, both updated by one paired
// FMA (per lane the same rounding as fmaf). MODE -1 (every lower run except
// the one at the source plane): the rays descend and the row grid rises
// (dv > 0 for any z-mirror plan), so e1 <= e2 at every plane and both grow
// with k; voxel k's rows are then [e1(k), e2(k + 1)] without per-plane
// min / max. MODE 0: the general window. (MODE +1 does not occur: every run
// of the lower half lies below the source.)
template <int MODE, int TZ, typename TW>
__device__ __forceinline__ void adj_rows_pair(float2 (&acc)[TZ], int nk, int z0, float l,
                                              float h, float e1, float e2, float s1, float s2,
                                              const AxisEntry* __restrict__ rv, float bh, float be,
                                              const TW* __restrict__ ycol, int na, int nb)
{
    float mn = fminf(e1, e2), mx = fmaxf(e1, e2);
    float lo_e = e1 - 0.02f, hi_e = e2 + s2 + 0.02f;
#pragma unroll
    for (int k = 0; k < TZ; k++) {
        if (k >= nk) break;
        int blo, bhi;
        if (MODE < 0) {
            blo = max(__float2int_ru(lo_e), 0);
            bhi = min(__float2int_rd(hi_e), nb - 1);
            lo_e += s1; hi_e += s2;
        } else {
            e1 += s1; e2 += s2;
            const float mn1 = fminf(e1, e2), mx1 = fmaxf(e1, e2);
            blo = max(__float2int_ru(fminf(mn, mn1) - 0.02f), 0);
            bhi = min(__float2int_rd(fmaxf(mx, mx1) + 0.02f), nb - 1);
            mn = mn1; mx = mx1;
        }
        const float fk0 = (float)(z0 + k), fk1 = (float)(z0 + k + 1);
        for (int ib = blo; ib <= bhi; ib++) {
            if (!FL_IN(ib, nb)) continue;
            const AxisEntry re = rv[ib];
            float tv[2];
            ld_in<TW, 2>(ycol + 2 * (long long)ib * na, tv);
            const float2 t = make_float2(tv[0], tv[1]);
            const float2 az = row_planes(re, fk0, fk1, bh, be);
            float l2, h2;
            if (MODE < 0) { l2 = fmaxf(l, az.y); h2 = fminf(h, az.x); }
            else { l2 = fmaxf(l, fminf(az.x, az.y)); h2 = fminf(h, fmaxf(az.x, az.y)); }
            const float w = fmaxf(h2 - l2, 0.0f);
            acc[k] = __ffma2_rn(make_float2(w, w), t, acc[k]);
        }
    }
}

// Half-turn form of adj_rows_pair: every weight also multiplies the row pair
// of view v + nv/2 into the turned voxels' sums accr; y4 holds both row pairs
// side by side (4 floats per row and column, 16-byte aligned).
template <int MODE, int TZ, typename TW>
__device__ __forceinline__ void adj_rows_quad(float2 (&acc)[TZ], float2 (&accr)[TZ], int nk,
                                              int z0, float l, float h, float e1, float e2,
                                              float s1, float s2, const AxisEntry* __restrict__ rv, float bh, float be,
                                              const TW* __restrict__ y4, int na, int nb)
{
    float mn = fminf(e1, e2), mx = fmaxf(e1, e2);
    float lo_e = e1 - 0.02f, hi_e = e2 + s2 + 0.02f;
#pragma unroll
    for (int k = 0; k < TZ; k++) {
        if (k >= nk) break;
        int blo, bhi;
        if (MODE < 0) {
            blo = max(__float2int_ru(lo_e), 0);
            bhi = min(__float2int_rd(hi_e), nb - 1);
            lo_e += s1; hi_e += s2;
        } else {
            e1 += s1; e2 += s2;
            const float mn1 = fminf(e1, e2), mx1 = fmaxf(e1, e2);
            blo = max(__float2int_ru(fminf(mn, mn1) - 0.02f), 0);
            bhi = min(__float2int_rd(fmaxf(mx, mx1) + 0.02f), nb - 1);
            mn = mn1; mx = mx1;
        }
        const float fk0 = (float)(z0 + k), fk1 = (float)(z0 + k + 1);
        for (int ib = blo; ib <= bhi; ib++) {
            if (!FL_IN(ib, nb)) continue;
            const AxisEntry re = rv[ib];
            float u[4];
            ld_in<TW, 4>(y4 + 4 * (long long)ib * na, u);
            const float2 t = make_float2(u[0], u[1]), tr = make_float2(u[2], u[3]);
            const float2 az = row_planes(re, fk0, fk1, bh, be);
            float l2, h2;
            if (MODE < 0) { l2 = fmaxf(l, az.y); h2 = fminf(h, az.x); }
            else { l2 = fmaxf(l, fminf(az.x, az.y)); h2 = fminf(h, fmaxf(az.x, az.y)); }
            const float w = fmaxf(h2 - l2, 0.0f);
            acc[k] = __ffma2_rn(make_float2(w, w), t, acc[k]);
            accr[k] = __ffma2_rn(make_float2(w, w), tr, accr[k]);
        }
    }
}

// Half-turn + z-mirror backprojection (fl_plan::rot): one thread per voxel
// column V = (ix, iy < ny/2) and its turned column T = (nx-1-ix, ny-1-iy),
// with a run of TZ voxels of the lower half and their mirrors; one frame. The
// thread visits the views iv < nv/2 only. In view iv it evaluates the weights
// of both columns: a weight of V multiplies the row pair of view iv into V
// and the row pair of view iv + nv/2 into T (A[(iv + nv/2, r), T] =
// A[(iv, r), V]); a weight of T, the other way round. yw is the packed
// sinogram of k_weight_packed / k_fwd_quad (4 values per (iv < nv/2,
// ib < nb/2, ia)); X the tiled folded volume (xfold) or the standard one.
template <typename TX, int TZ, typename TW>
__global__ void __launch_bounds__(128, 8)
k_adj_quad(TX* __restrict__ X, const TW* __restrict__ yw, const ColEntry* __restrict__ col,
           const AxisEntry* __restrict__ rowz, const ViewEntry* __restrict__ view, DetGrid G,
           int nx, int ny, int nz, int na, int nb, int nv, float dz, int zruns,
           const int* __restrict__ skip, int xfold)
{
    if (skip && *skip) return;
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;     // < ny / 2
    const int z0 = blockIdx.z * TZ;
    const int nzw = nz / 2, nbw = nb / 2, hv = nv / 2;
    const int nk = min(TZ, nzw - z0);
    if (ix >= nx || iy >= ny / 2) return;
    const int tx = nx - 1 - ix, ty = ny - 1 - iy;             // the turned column
    float2 accV[TZ], accT[TZ];
#pragma unroll
    for (int k = 0; k < TZ; k++) { accV[k] = make_float2(0.0f, 0.0f); accT[k] = accV[k]; }
    const float inv_dv = 1.0f / G.dv;
    const long long vstride = (long long)nbw * na * 4;        // packed floats per view pair
    for (int iv = 0; iv < hv; iv++) {
        const ViewEntry ve = view[iv];
        const ColEntry* cv = col + (long long)iv * na;
        const AxisEntry* rv = rowz + (long long)iv * nb;
        const TW* yv = yw + (long long)iv * vstride;
        const float zr0 = (float)(z0 - nz / 2) * dz - ve.sz;
        const float zr1 = (float)(z0 + nk - nz / 2) * dz - ve.sz;
        const float tol = 1e-3f * dz;
        const int mode = (zr1 <= -tol) ? -1 : 0;               // lower half: never above
        // column (cx, cy) in view iv: its weights go to `own` with view iv and
        // to `other` with view iv + nv/2
        auto column = [&](int cx, int cy, float2 (&own)[TZ], float2 (&other)[TZ]) {
            int alo, ahi; float dmin, dmax;
            column_window(G, ve.c, ve.s, (float)(cx - nx / 2), (float)(cy - ny / 2), 1.0f, 1.0f,
                          na, alo, ahi, dmin, dmax);
            for (int ia = alo; ia <= ahi; ia++) {
                if (!FL_IN(ia, na)) continue;
                const ColEntry ce = cv[ia];
                float bh, be, l, h;
                if (!cone_column(ce, cx, cy, nx, ny, bh, be, l, h)) continue;
                // absolute parameters of the column's ends (row windows only)
                const float r1 = __fdividef(1.0f, __fadd_rn(bh, l) + ve.ac);
                const float r2 = __fdividef(1.0f, __fadd_rn(bh, h) + ve.ac);
                const float s1 = dz * r1 * inv_dv, s2 = dz * r2 * inv_dv;
                const float e1 = (zr0 * r1 - G.v0) * inv_dv, e2 = (zr0 * r2 - G.v0) * inv_dv;
                if (mode < 0)
                    adj_rows_quad<-1, TZ, TW>(own, other, nk, z0, l, h, e1, e2, s1, s2, rv, bh, be,
                                          yv + 4 * ia, na, nbw);
                else
                    adj_rows_quad<0, TZ, TW>(own, other, nk, z0, l, h, e1, e2, s1, s2, rv, bh, be,
                                         yv + 4 * ia, na, nbw);
            }
        };
        // both columns in one rolled loop (one copy of the row code); the two
        // sets swap after each column and are back in order after the second
#pragma unroll 1
        for (int k = 0; k < 2; k++) {
            column(k ? tx : ix, k ? ty : iy, accV, accT);
#pragma unroll
            for (int z = 0; z < TZ; z++) {
                const float2 t = accV[z];
                accV[z] = accT[z]; accT[z] = t;
            }
        }
    }
    const long long nxy = (long long)nx * ny;
    const long long cV = (long long)iy * nx + ix, cT = (long long)ty * nx + tx;
#pragma unroll
    for (int k = 0; k < TZ; k++)
        if (k < nk) {
            const long long zl = (long long)(z0 + k) * nxy, zh = (long long)(nz - 1 - z0 - k) * nxy;
            if (xfold) {                      // the tiled folded volume
                const int tV = tiled_pair(ix, iy, (int)zl, nx >> 2);
                const int tT = tiled_pair(tx, ty, (int)zl, nx >> 2);
                Store<TX>::st2(X + 2 * (long long)tV, accV[k].x, accV[k].y);
                Store<TX>::st2(X + 2 * (long long)tT, accT[k].x, accT[k].y);
            } else {
                Store<TX>::st(X + zl + cV, accV[k].x);
                Store<TX>::st(X + zh + cV, accV[k].y);
                Store<TX>::st(X + zl + cT, accT[k].x);
                Store<TX>::st(X + zh + cT, accT[k].y);
            }
        }
}

// Quarter-turn form of adj_rows_pair: every weight multiplies the row pairs of
// views v + j nv/4 into the sums a0..a3; y8 holds them side by side (8 floats
// per row and column, 32-byte aligned).
template <int MODE, int TZ, typename TW>
__device__ __forceinline__ void adj_rows_oct(float2 (&a0)[TZ], float2 (&a1)[TZ],
                                             float2 (&a2)[TZ], float2 (&a3)[TZ], int nk, int z0,
                                             float l, float h, float e1, float e2, float s1,
                                             float s2, const AxisEntry* __restrict__ rv, float bh, float be,
                                             const TW* __restrict__ y8, int na, int nb)
{
    float mn = fminf(e1, e2), mx = fmaxf(e1, e2);
    float lo_e = e1 - 0.02f, hi_e = e2 + s2 + 0.02f;
#pragma unroll
    for (int k = 0; k < TZ; k++) {
        if (k >= nk) break;
        int blo, bhi;
        if (MODE < 0) {
            blo = max(__float2int_ru(lo_e), 0);
            bhi = min(__float2int_rd(hi_e), nb - 1);
            lo_e += s1; hi_e += s2;
        } else {
            e1 += s1; e2 += s2;
            const float mn1 = fminf(e1, e2), mx1 = fmaxf(e1, e2);
            blo = max(__float2int_ru(fminf(mn, mn1) - 0.02f), 0);
            bhi = min(__float2int_rd(fmaxf(mx, mx1) + 0.02f), nb - 1);
            mn = mn1; mx = mx1;
        }
        const float fk0 = (float)(z0 + k), fk1 = (float)(z0 + k + 1);
        for (int ib = blo; ib <= bhi; ib++) {
            if (!FL_IN(ib, nb)) continue;
            const AxisEntry re = rv[ib];
            // the orbit's 8 values in one vector load (32 bytes FP32, 16 bytes FP16)
            float o8[8];
            ld_in<TW, 8>(y8 + 8 * (long long)ib * na, o8);
            const float2 t0 = make_float2(o8[0], o8[1]), t1 = make_float2(o8[2], o8[3]);
            const float2 t2 = make_float2(o8[4], o8[5]), t3 = make_float2(o8[6], o8[7]);
            const float2 az = row_planes(re, fk0, fk1, bh, be);
            float l2, h2;
            if (MODE < 0) { l2 = fmaxf(l, az.y); h2 = fminf(h, az.x); }
            else { l2 = fmaxf(l, fminf(az.x, az.y)); h2 = fminf(h, fmaxf(az.x, az.y)); }
            const float2 w2 = make_float2(fmaxf(h2 - l2, 0.0f), fmaxf(h2 - l2, 0.0f));
            a0[k] = __ffma2_rn(w2, t0, a0[k]);
            a1[k] = __ffma2_rn(w2, t1, a1[k]);
            a2[k] = __ffma2_rn(w2, t2, a2[k]);
            a3[k] = __ffma2_rn(w2, t3, a3[k]);
        }
    }
}

// Quarter-turn + z-mirror backprojection (fl_plan::rot4, nx == ny == n): one
// thread per voxel column V0 = (x, y) of the quadrant x, y < n/2 and its
// turns V_j = R^j V0, with a run of TZ voxels of the lower half and their
// mirrors; one frame. It visits the views iv < nv/4. In view iv a weight of
// column V_k multiplies the row pairs of view iv + j nv/4 into V_{k+j mod 4}
// (A[(iv + j nv/4, r), R^j V] = A[(iv, r), V]). yw is the packed sinogram of
// k_weight_packed / k_fwd_oct (8 values per (iv < nv/4, ib < nb/2, ia)); X the
// tiled folded volume (xfold) or the standard one.
template <typename TX, int TZ, typename TW>
__global__ void __launch_bounds__(128, TZ == 2 ? 8 : 6)
k_adj_oct(TX* __restrict__ X, const TW* __restrict__ yw, const ColEntry* __restrict__ col,
          const AxisEntry* __restrict__ rowz, const ViewEntry* __restrict__ view, DetGrid G, int n,
          int nz, int na, int nb, int nv, float dz, const int* __restrict__ skip, int xfold)
{
    if (skip && *skip) return;
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;    // < n / 2
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;    // < n / 2
    const int z0 = blockIdx.z * TZ;
    const int nzw = nz / 2, nbw = nb / 2, qv = nv / 4, h = n / 2;
    const int nk = min(TZ, nzw - z0);
    if (ix >= h || iy >= h) return;
    const int cx[4] = {ix, n - 1 - iy, n - 1 - ix, iy};
    const int cy[4] = {iy, ix, n - 1 - iy, n - 1 - ix};
    float2 A0[TZ], A1[TZ], A2[TZ], A3[TZ];
#pragma unroll
    for (int k = 0; k < TZ; k++) {
        A0[k] = make_float2(0.0f, 0.0f); A1[k] = A0[k]; A2[k] = A0[k]; A3[k] = A0[k];
    }
    const float inv_dv = 1.0f / G.dv;
    const long long vstride = (long long)nbw * na * 8;        // packed floats per view
    for (int iv = 0; iv < qv; iv++) {
        const ViewEntry ve = view[iv];
        const ColEntry* cv = col + (long long)iv * na;
        const AxisEntry* rv = rowz + (long long)iv * nb;
        const TW* yv = yw + (long long)iv * vstride;
        const float zr0 = (float)(z0 - nz / 2) * dz - ve.sz;
        const float zr1 = (float)(z0 + nk - nz / 2) * dz - ve.sz;
        const float tol = 1e-3f * dz;
        const int mode = (zr1 <= -tol) ? -1 : 0;               // lower half: never above
        // column (px, py) in view iv: its weights go to b0 with view iv,
        // b1 with iv + nv/4, b2 with iv + nv/2, b3 with iv + 3 nv/4
        auto column = [&](int px_, int py_, float2 (&b0)[TZ], float2 (&b1)[TZ],
                          float2 (&b2)[TZ], float2 (&b3)[TZ]) {
            int alo, ahi; float dmin, dmax;
            column_window(G, ve.c, ve.s, (float)(px_ - h), (float)(py_ - h), 1.0f, 1.0f, na, alo,
                          ahi, dmin, dmax);
            for (int ia = alo; ia <= ahi; ia++) {
                if (!FL_IN(ia, na)) continue;
                const ColEntry ce = cv[ia];
                float bh, be, l, hh;
                if (!cone_column(ce, px_, py_, n, n, bh, be, l, hh)) continue;
                // absolute parameters of the column's ends (row windows only)
                const float r1 = __fdividef(1.0f, __fadd_rn(bh, l) + ve.ac);
                const float r2 = __fdividef(1.0f, __fadd_rn(bh, hh) + ve.ac);
                const float s1 = dz * r1 * inv_dv, s2 = dz * r2 * inv_dv;
                const float e1 = (zr0 * r1 - G.v0) * inv_dv, e2 = (zr0 * r2 - G.v0) * inv_dv;
                const TW* y8 = yv + 8 * ia;
                if (mode < 0)
                    adj_rows_oct<-1, TZ, TW>(b0, b1, b2, b3, nk, z0, l, hh, e1, e2, s1, s2, rv, bh, be, y8,
                                         na, nbw);
                else
                    adj_rows_oct<0, TZ, TW>(b0, b1, b2, b3, nk, z0, l, hh, e1, e2, s1, s2, rv, bh, be, y8,
                                        na, nbw);
            }
        };
        // the four turns in one rolled loop (one copy of the row code: the
        // unrolled form overflowed the instruction cache): turn k's weights go
        // to A_{k+j} with view iv + j nv/4, so the sets rotate one place after
        // each turn and are back in order after the fourth
#pragma unroll 1
        for (int k = 0; k < 4; k++) {
            column(k == 0 ? cx[0] : k == 1 ? cx[1] : k == 2 ? cx[2] : cx[3],
                   k == 0 ? cy[0] : k == 1 ? cy[1] : k == 2 ? cy[2] : cy[3], A0, A1, A2, A3);
#pragma unroll
            for (int z = 0; z < TZ; z++) {
                const float2 t = A0[z];
                A0[z] = A1[z]; A1[z] = A2[z]; A2[z] = A3[z]; A3[z] = t;
            }
        }
    }
    const long long nn = (long long)n * n;
#pragma unroll
    for (int k = 0; k < TZ; k++)
        if (k < nk) {
            const long long zl = (long long)(z0 + k) * nn, zh = (long long)(nz - 1 - z0 - k) * nn;
            const float2* accs[4] = {&A0[k], &A1[k], &A2[k], &A3[k]};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const long long c = (long long)cy[j] * n + cx[j];
                if (xfold) {                  // the tiled folded volume
                    const long long t = tiled_pair(cx[j], cy[j], (int)zl, n >> 2);
                    Store<TX>::st2(X + 2 * t, accs[j]->x, accs[j]->y);
                } else {
                    Store<TX>::st(X + zl + c, accs[j]->x);
                    Store<TX>::st(X + zh + c, accs[j]->y);
                }
            }
        }
}

// Reflection forms of adj_rows_oct: every weight multiplies the row pairs of
// the walked ray's 2 NR images into the sums P[j] (turn images) and Q[j]
// (reflected images); yt / yr hold them side by side (2 NR values per row and
// column in each plane, rows rs columns apart), so each is one vector load
// whose lanes read neighbouring columns' orbits. RU rows per iteration: RU =
// 2 issues the loads of two rows before either's arithmetic (more loads in
// flight per thread); RU = 0 loads each row of the run once for all its
// voxels; the rows are added in order either way.
template <int MODE, int TZ, int RU, typename TW, int NR>
__device__ __forceinline__ void adj_rows_refl(float2 (&P)[NR][TZ], float2 (&Q)[NR][TZ], int nk,
                                              int z0, float l, float h, float e1, float e2,
                                              float s1, float s2,
                                              const AxisEntry* __restrict__ rv, float bh,
                                              float be, const TW* __restrict__ yt,
                                              const TW* __restrict__ yr, int rs, int nb)
{
    float mn = fminf(e1, e2), mx = fmaxf(e1, e2);
    float lo_e = e1 - 0.02f, hi_e = e2 + s2 + 0.02f;
    if constexpr (RU == 0) {
        // the run's rows once: each row in the union of the voxels' windows
        // is loaded once and adds to every voxel whose window holds it (the
        // same terms in the same order as one pass per voxel)
        int blo[TZ], bhi[TZ];
        int ulo = nb, uhi = -1;
#pragma unroll
        for (int k = 0; k < TZ; k++) {
            if (MODE < 0) {
                blo[k] = max(__float2int_ru(lo_e), 0);
                bhi[k] = min(__float2int_rd(hi_e), nb - 1);
                lo_e += s1; hi_e += s2;
            } else {
                e1 += s1; e2 += s2;
                const float mn1 = fminf(e1, e2), mx1 = fmaxf(e1, e2);
                blo[k] = max(__float2int_ru(fminf(mn, mn1) - 0.02f), 0);
                bhi[k] = min(__float2int_rd(fmaxf(mx, mx1) + 0.02f), nb - 1);
                mn = mn1; mx = mx1;
            }
            if (k >= nk) { blo[k] = nb; bhi[k] = -1; }
            ulo = min(ulo, blo[k]); uhi = max(uhi, bhi[k]);
        }
        for (int ib = ulo; ib <= uhi; ib++) {
            if (!FL_IN(ib, nb)) continue;
            const AxisEntry re = rv[ib];
            float o[4 * NR];
            ld_in<TW, 2 * NR>(yt + 2 * NR * (long long)ib * rs,
                              *reinterpret_cast<float(*)[2 * NR]>(o));
            ld_in<TW, 2 * NR>(yr + 2 * NR * (long long)ib * rs,
                              *reinterpret_cast<float(*)[2 * NR]>(o + 2 * NR));
            const float cb = __fsub_rn(re.c, be);
            float az[TZ + 1];
#pragma unroll
            for (int k = 0; k <= TZ; k++)
                az[k] = xrel(re, __fsub_rn((float)(z0 + k), re.kq), bh, cb);
#pragma unroll
            for (int k = 0; k < TZ; k++) {
                if (ib < blo[k] || ib > bhi[k]) continue;
                float l2, h2;
                if (MODE < 0) { l2 = fmaxf(l, az[k + 1]); h2 = fminf(h, az[k]); }
                else {
                    l2 = fmaxf(l, fminf(az[k], az[k + 1]));
                    h2 = fminf(h, fmaxf(az[k], az[k + 1]));
                }
                const float w = fmaxf(h2 - l2, 0.0f);
                const float2 w2 = make_float2(w, w);
#pragma unroll
                for (int j = 0; j < NR; j++) {
                    P[j][k] = __ffma2_rn(w2, make_float2(o[2 * j], o[2 * j + 1]), P[j][k]);
                    Q[j][k] = __ffma2_rn(w2, make_float2(o[2 * NR + 2 * j], o[2 * NR + 2 * j + 1]),
                                         Q[j][k]);
                }
            }
        }
        return;
    }
    constexpr int RN = RU > 0 ? RU : 1;          // rows per iteration below
#pragma unroll
    for (int k = 0; k < TZ; k++) {
        if (k >= nk) break;
        int blo, bhi;
        if (MODE < 0) {
            blo = max(__float2int_ru(lo_e), 0);
            bhi = min(__float2int_rd(hi_e), nb - 1);
            lo_e += s1; hi_e += s2;
        } else {
            e1 += s1; e2 += s2;
            const float mn1 = fminf(e1, e2), mx1 = fmaxf(e1, e2);
            blo = max(__float2int_ru(fminf(mn, mn1) - 0.02f), 0);
            bhi = min(__float2int_rd(fmaxf(mx, mx1) + 0.02f), nb - 1);
            mn = mn1; mx = mx1;
        }
        const float fk0 = (float)(z0 + k), fk1 = (float)(z0 + k + 1);
        for (int ib = blo; ib <= bhi; ib += RN) {
            AxisEntry re[RN];
            float o[RN][4 * NR];
            bool on[RN];
#pragma unroll
            for (int u = 0; u < RN; u++) {
                on[u] = ib + u <= bhi && FL_IN(ib + u, nb);
                const long long r = on[u] ? ib + u : min(max(ib, 0), nb - 1);   // one that exists
                re[u] = rv[r];
                ld_in<TW, 2 * NR>(yt + 2 * NR * r * rs, *reinterpret_cast<float(*)[2 * NR]>(o[u]));
                ld_in<TW, 2 * NR>(yr + 2 * NR * r * rs,
                                  *reinterpret_cast<float(*)[2 * NR]>(o[u] + 2 * NR));
            }
#pragma unroll
            for (int u = 0; u < RN; u++) {
                const float2 az = row_planes(re[u], fk0, fk1, bh, be);
                float l2, h2;
                if (MODE < 0) { l2 = fmaxf(l, az.y); h2 = fminf(h, az.x); }
                else { l2 = fmaxf(l, fminf(az.x, az.y)); h2 = fminf(h, fmaxf(az.x, az.y)); }
                if (!on[u]) continue;
                const float w = fmaxf(h2 - l2, 0.0f);
                const float2 w2 = make_float2(w, w);
#pragma unroll
                for (int j = 0; j < NR; j++) {
                    P[j][k] = __ffma2_rn(w2, make_float2(o[u][2 * j], o[u][2 * j + 1]), P[j][k]);
                    Q[j][k] = __ffma2_rn(
                        w2, make_float2(o[u][2 * NR + 2 * j], o[u][2 * NR + 2 * j + 1]), Q[j][k]);
                }
            }
        }
    }
}

// Reflection + z-mirror backprojections (fl_plan::refl). NR = 4 (quarter
// turns, nx == ny == n): one thread per voxel column V0 = (x, y) of the octant
// x <= y < n/2; NR = 2 (half turn): of the quadrant x < nx/2, y < ny/2. With
// S = R^(4/NR) the thread owns the images C_k = S^k V0 and D_k = S^k M V0 (k
// < NR; for NR = 4 and x == y, D_k = C_{k+3} and only the C_k are visited),
// a run of TZ voxels of the lower half and their mirrors; one frame. It
// visits the walked views w = 0 .. ov (refl_view). In view w a weight of
// column C_k multiplies turn slot j (view w + j nv/NR) into C_{k+j} and
// reflected slot j (view j nv/NR - w, column na-1-a) into D_{j-k}; a weight of
// D_k, turn slot j into D_{k+j} and reflected slot j into C_{j-k}. One weight
// thus feeds 4 NR (voxel, ray) pairs. yw is the packed input of
// k_weight_packed_refl / k_fwd_refl (two planes); X the tiled folded volume
// (xfold) or the standard one.
// View chunks: the walked views w0 .. w1 only. A launch that is not the
// first continues the sums it finds in X (FP32, either layout) and one that
// is not the last leaves them there, so a sequence of launches over
// consecutive chunks adds every term in the order one launch would: the bits
// are the same. On the diagonal (NR = 4, x == y) P and Q are carried apart
// between chunks, P in X and Q in dq (dq[((x * dqz + z) * NR + j)] for the
// voxel pair at height z < nz/2), and combined by the last.
template <typename TX, int TZ, int RU, typename TW, int NR>
__global__ void __launch_bounds__(128, TZ == 1 ? (RU == 2 ? 6 : 8) : (RU == 1 ? 6 : 5))
k_adj_refl(TX* __restrict__ X, const TW* __restrict__ yw, const ColEntry* __restrict__ col,
           const AxisEntry* __restrict__ rowz, const ViewEntry* __restrict__ view, DetGrid G,
           int nx, int ny, int nz, int na, int nb, int nv, float dz,
           const int* __restrict__ skip, int xfold, int w0, int w1, int first, int last,
           float2* __restrict__ dq, int dqz)
{
    if (skip && *skip) return;
    const ReflGeom g = refl_geom(NR, nv, na, nb);
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;    // < nx / 2
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;    // < ny / 2
    const int z0 = blockIdx.z * TZ;
    const int nzw = nz / 2, hx = nx / 2, hy = ny / 2;
    const int nk = min(TZ, nzw - z0);
    if (ix >= hx || iy >= hy || (NR == 4 && ix > iy)) return;
    const bool diag = NR == 4 && ix == iy;
    // P: the sums the turn slots feed, Q: the reflected slots' (rotated one
    // place per column, in opposite directions; exchanged between the C and
    // the D columns)
    float2 P[NR][TZ], Q[NR][TZ];
#pragma unroll
    for (int j = 0; j < NR; j++)
#pragma unroll
        for (int k = 0; k < TZ; k++) { P[j][k] = make_float2(0.0f, 0.0f); Q[j][k] = P[j][k]; }
    const float inv_dv = 1.0f / G.dv;
    const int nsteps = diag ? NR : 2 * NR;
    // C_j = S^j V0 and D_j = S^j M V0 of the thread's column (the stores
    // below; the loads of a chunk after the first)
    const long long nxy = (long long)nx * ny;
    int cx[NR], cy[NR], dxs[NR], dys[NR];
    if (NR == 4) {
        cx[0] = ix; cx[1 % NR] = nx - 1 - iy; cx[2 % NR] = nx - 1 - ix; cx[3 % NR] = iy;
        cy[0] = iy; cy[1 % NR] = ix; cy[2 % NR] = ny - 1 - iy; cy[3 % NR] = ny - 1 - ix;
        dxs[0] = ix; dxs[1 % NR] = iy; dxs[2 % NR] = nx - 1 - ix; dxs[3 % NR] = nx - 1 - iy;
        dys[0] = ny - 1 - iy; dys[1 % NR] = ix; dys[2 % NR] = iy; dys[3 % NR] = ny - 1 - ix;
    } else {
        cx[0] = ix; cx[1 % NR] = nx - 1 - ix; cy[0] = iy; cy[1 % NR] = ny - 1 - iy;
        dxs[0] = ix; dxs[1 % NR] = nx - 1 - ix; dys[0] = ny - 1 - iy; dys[1 % NR] = iy;
    }
    if (!first) {                                    // continue the chunk before
#pragma unroll
        for (int k = 0; k < TZ; k++)
            if (k < nk) {
                const int zl = (z0 + k) * (int)nxy;
#pragma unroll
                for (int j = 0; j < 2 * NR; j++) {
                    if (diag && j >= NR) {
                        Q[j - NR][k] = dq[((long long)ix * dqz + z0 + k) * NR + (j - NR)];
                        continue;
                    }
                    const int qx = j < NR ? cx[j] : dxs[j - NR], qy = j < NR ? cy[j] : dys[j - NR];
                    const float* Xf = (const float*)X;
                    float2 a;
                    if (xfold) {
                        a = Store<float>::ld2(Xf + 2 * tiled_pair(qx, qy, zl, nx >> 2));
                    } else {
                        const long long c = (long long)qy * nx + qx;
                        a = make_float2(Xf[zl + c], Xf[(long long)(nz - 1 - z0 - k) * nxy + c]);
                    }
                    if (j < NR) P[j][k] = a; else Q[j - NR][k] = a;
                }
            }
    }
    for (int w = w0; w <= min(w1, g.ov); w++) {
        int vt, rs, alim;
        long long base;
        refl_view(g, w, vt, base, rs, alim);
        const ViewEntry ve = view[vt];
        const ColEntry* cv = col + (long long)vt * na;
        const AxisEntry* rv = rowz + (long long)vt * nb;
        const TW* yv = yw + base;
        const float zr0 = (float)(z0 - nz / 2) * dz - ve.sz;
        const float zr1 = (float)(z0 + nk - nz / 2) * dz - ve.sz;
        const float tol = 1e-3f * dz;
        const int mode = (zr1 <= -tol) ? -1 : 0;               // lower half: never above
        int px = ix, py = iy;                                  // C_0
#pragma unroll 1
        for (int k = 0; k < nsteps; k++) {
            if (k == NR) {                                     // the D columns: D_0 = M V0
                px = ix; py = ny - 1 - iy;
#pragma unroll
                for (int j = 0; j < NR; j++)
#pragma unroll
                    for (int z = 0; z < TZ; z++) {
                        const float2 t = P[j][z];
                        P[j][z] = Q[j][z]; Q[j][z] = t;
                    }
            }
            int alo, ahi; float dmin, dmax;
            column_window(G, ve.c, ve.s, (float)(px - hx), (float)(py - hy), 1.0f, 1.0f, na, alo,
                          ahi, dmin, dmax);
            ahi = min(ahi, alim - 1);
            for (int ia = alo; ia <= ahi; ia++) {
                if (!FL_IN(ia, na)) continue;
                const ColEntry ce = cv[ia];
                float bh, be, l, hh;
                if (!cone_column(ce, px, py, nx, ny, bh, be, l, hh)) continue;
                // absolute parameters of the column's ends (row windows only)
                const float r1 = __fdividef(1.0f, __fadd_rn(bh, l) + ve.ac);
                const float r2 = __fdividef(1.0f, __fadd_rn(bh, hh) + ve.ac);
                const float s1 = dz * r1 * inv_dv, s2 = dz * r2 * inv_dv;
                const float e1 = (zr0 * r1 - G.v0) * inv_dv, e2 = (zr0 * r2 - G.v0) * inv_dv;
                const TW* yt = yv + g.vpr * ia;
                if (mode < 0)
                    adj_rows_refl<-1, TZ, RU, TW, NR>(P, Q, nk, z0, l, hh, e1, e2, s1, s2, rv, bh,
                                                      be, yt, yt + g.plane, rs, g.nbh);
                else
                    adj_rows_refl<0, TZ, RU, TW, NR>(P, Q, nk, z0, l, hh, e1, e2, s1, s2, rv, bh,
                                                     be, yt, yt + g.plane, rs, g.nbh);
            }
            // next column S (px, py); P rotates back one place, Q forward one
            if (NR == 4) {
                const int t = px;
                px = nx - 1 - py; py = t;
            } else {
                px = nx - 1 - px; py = ny - 1 - py;
            }
#pragma unroll
            for (int z = 0; z < TZ; z++) {
                const float2 a = P[0][z];
#pragma unroll
                for (int j = 0; j + 1 < NR; j++) P[j][z] = P[j + 1][z];
                P[NR - 1][z] = a;
                const float2 b = Q[NR - 1][z];
#pragma unroll
                for (int j = NR - 1; j > 0; j--) Q[j][z] = Q[j - 1][z];
                Q[0][z] = b;
            }
        }
        if (!diag) {                                           // C sums back into P
#pragma unroll
            for (int j = 0; j < NR; j++)
#pragma unroll
                for (int z = 0; z < TZ; z++) {
                    const float2 t = P[j][z];
                    P[j][z] = Q[j][z]; Q[j][z] = t;
                }
        }
    }
    // C_j = S^j V0 holds P[j] (and, on the diagonal of NR = 4, Q[j + 1], the
    // sums of D_{j+1} = C_j; before the last chunk they stay apart, Q in dq);
    // D_j = S^j M V0 holds Q[j]
#pragma unroll
    for (int k = 0; k < TZ; k++)
        if (k < nk) {
            const long long zl = (long long)(z0 + k) * nxy, zh = (long long)(nz - 1 - z0 - k) * nxy;
#pragma unroll
            for (int j = 0; j < 2 * NR; j++) {
                if (diag && j >= NR) {
                    if (!last) dq[((long long)ix * dqz + z0 + k) * NR + (j - NR)] = Q[j - NR][k];
                    continue;
                }
                float2 a;
                int qx, qy;
                if (j < NR) {
                    a = P[j][k];
                    if (diag && last) {
                        const float2 b = Q[(j + 1) % NR][k];
                        a.x += b.x; a.y += b.y;
                    }
                    qx = cx[j]; qy = cy[j];
                } else {
                    a = Q[j - NR][k]; qx = dxs[j - NR]; qy = dys[j - NR];
                }
                if (xfold) {                  // the tiled folded volume
                    const long long t = tiled_pair(qx, qy, (int)zl, nx >> 2);
                    Store<TX>::st2(X + 2 * t, a.x, a.y);
                } else {
                    const long long c = (long long)qy * nx + qx;
                    Store<TX>::st(X + zl + c, a.x);
                    Store<TX>::st(X + zh + c, a.y);
                }
            }
        }
}

// MIRROR: yw is the folded sinogram; the runs cover the lower half z < nz/2
// only (the walked rows' rays never reach the upper half) and each thread also
// produces the mirrored run, into the folded volume when xfold is set.
template <typename TX, int TZ, bool MIRROR, typename TW>
__global__ void __launch_bounds__(128, 8)
k_adj_cone(TX* __restrict__ X, const TW* __restrict__ yw, const ColEntry* __restrict__ col,
           const AxisEntry* __restrict__ rowz, const ViewEntry* __restrict__ view,
           const int* __restrict__ idY, const int* __restrict__ Nv, int tmp_size, DetGrid G,
           int nx, int ny, int nz, int na, int nb, float dz, int zruns,
           const int* __restrict__ skip, int xfold)
{
    if (skip && *skip) return;
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    const int zr = blockIdx.z % zruns, it = blockIdx.z / zruns;
    const int z0 = zr * TZ;
    const int nzw = MIRROR ? nz / 2 : nz;      // voxels gathered directly
    const int nbw = MIRROR ? nb / 2 : nb;      // rows evaluated
    const int nk = min(TZ, nzw - z0);          // voxels of this run inside that range
    if (ix >= nx || iy >= ny) return;
    float acc[TZ];                 // general form
    float2 acc2[TZ];               // mirror form: (voxel, mirrored voxel)
#pragma unroll
    for (int k = 0; k < TZ; k++) { acc[k] = 0.0f; acc2[k] = make_float2(0.0f, 0.0f); }
    const float x0 = (float)(ix - nx / 2), y0 = (float)(iy - ny / 2);
    const float inv_dv = 1.0f / G.dv;
    const int nvf = Nv[it];
    for (int j = 0; j < nvf; j++) {
        const int iv = idY[it * tmp_size + j];
        const ViewEntry ve = view[iv];
        int alo, ahi; float dmin, dmax;
        column_window(G, ve.c, ve.s, x0, y0, 1.0f, 1.0f, na, alo, ahi, dmin, dmax);
        const ColEntry* cv = col + (long long)iv * na;
        const AxisEntry* rv = rowz + (long long)iv * nb;
        const TW* yv = yw + (long long)iv * nb * na;      // folded: nb/2 rows of pairs
        // run planes relative to the source: lowest and highest
        const float zr0 = (float)(z0 - nz / 2) * dz - ve.sz;
        const float zr1 = (float)(z0 + nk - nz / 2) * dz - ve.sz;
        // uniform per block; a run within rounding distance of the source plane
        // takes the general path
        const float tol = 1e-3f * dz;
        const int mode = (zr0 >= tol) ? 1 : ((zr1 <= -tol) ? -1 : 0);
        for (int ia = alo; ia <= ahi; ia++) {
            if (!FL_IN(ia, na)) continue;
            const ColEntry ce = cv[ia];
            float bh, be, l, h;
            if (!cone_column(ce, ix, iy, nx, ny, bh, be, l, h)) continue;
            // A ray of row ib is at z = sz + (A + ac) * d_ib, d_ib ~ v0 + ib * dv. It is
            // inside voxel k somewhere in [l, h] iff d_ib lies between the plane
            // heights over (A + ac) at the two ends: in detector-row units the
            // rows [e(k), e(k+1)], stepping by dz/(A + ac)/dv per plane.
            const float r1 = __fdividef(1.0f, __fadd_rn(bh, l) + ve.ac);
            const float r2 = __fdividef(1.0f, __fadd_rn(bh, h) + ve.ac);
            const float s1 = dz * r1 * inv_dv, s2 = dz * r2 * inv_dv;
            const float e1 = (zr0 * r1 - G.v0) * inv_dv, e2 = (zr0 * r2 - G.v0) * inv_dv;
            if (MIRROR) {
                const TW* ycol = yv + 2 * ia;
                if (mode < 0)
                    adj_rows_pair<-1, TZ, TW>(acc2, nk, z0, l, h, e1, e2, s1, s2, rv, bh, be, ycol, na, nbw);
                else
                    adj_rows_pair<0, TZ, TW>(acc2, nk, z0, l, h, e1, e2, s1, s2, rv, bh, be, ycol, na, nbw);
            } else {
                const TW* ycol = yv + ia;
                if (mode > 0)
                    adj_rows<1, TZ, TW>(acc, nk, z0, l, h, e1, e2, s1, s2, rv, bh, be, ycol, na, nbw);
                else if (mode < 0)
                    adj_rows<-1, TZ, TW>(acc, nk, z0, l, h, e1, e2, s1, s2, rv, bh, be, ycol, na, nbw);
                else
                    adj_rows<0, TZ, TW>(acc, nk, z0, l, h, e1, e2, s1, s2, rv, bh, be, ycol, na, nbw);
            }
        }
    }
    const long long frame = (long long)it * nx * ny * nz, col_ = (long long)iy * nx + ix;
#pragma unroll
    for (int k = 0; k < TZ; k++)
        if (k < nk) {
            if (MIRROR && xfold) {
                Store<TX>::st2(X + frame + 2 * ((long long)(z0 + k) * nx * ny + col_),
                               acc2[k].x, acc2[k].y);
            } else if (MIRROR) {
                Store<TX>::st(X + frame + (long long)(z0 + k) * nx * ny + col_, acc2[k].x);
                Store<TX>::st(X + frame + (long long)(nz - 1 - z0 - k) * nx * ny + col_,
                              acc2[k].y);
            } else {
                Store<TX>::st(X + frame + (long long)(z0 + k) * nx * ny + col_, acc[k]);
            }
        }
}

DetGrid det_grid(const fl_plan* p)
{
    DetGrid G;
    G.kind = p->det_kind; G.u0 = p->u0; G.du = p->du; G.g0 = p->g0; G.dg = p->dg;
    G.v0 = p->v0; G.dv = p->dv; G.SO = p->s.SO; G.SD = p->SD;
    G.rdu = p->du != 0.0f ? 1.0f / p->du : 0.0f;
    G.rdg = p->dg != 0.0f ? 1.0f / p->dg : 0.0f;
    return G;
}

}  // namespace

// Tunables of fan plans (fl_plan.h).
int fl_plan_fan_lanes(const fl_plan* p)
{
    if (p->fan_lanes) return p->fan_lanes;
    const int G = fl_plan_turns(p);
    if (G <= 1 || p->s.ndim != 2) return 1;
    if (const int NR = fl_plan_refl(p))           // walked rays: slots x columns
        return fan_turn_lanes((long long)p->s.na * fan_refl_geom(NR, p->s.nv, p->s.na).slots);
    return fan_turn_lanes((long long)p->s.na * (p->s.nv / G));
}

int fl_plan_adj_chunks(const fl_plan* p, bool f32_out)
{
    if (!f32_out || p->adj_chunks < 2) return 1;
    if (fl_plan_refl(p) == 4 && !p->d_dq) return 1;        // no room for the diagonal's sums
    return p->adj_chunks;
}

int fl_plan_fan_groups(const fl_plan* p)
{
    // the quarter-turn reflection backprojection with 2 x 2 blocks keeps 8
    // (16 would need 64 KB of shared memory per thread block)
    const int NR = p->s.ndim == 2 ? fl_plan_refl(p) : 0;
    if (NR == 4 && fan_refl_pblock(NR, p->s.nx, p->s.ny) == 2) return kTurnGroups;
    return p->fan_groups ? p->fan_groups : kTurnGroups;
}

int fl_plan_fan_block(const fl_plan* p)
{
    if (p->fan_block) return p->fan_block;
    const fl_scan& s = p->s;
    const int T = fl_plan_turns(p);
    long long blocks2;
    if (T > 1) {
        const int hx = T == 2 ? s.nx : s.nx / 2, hy = s.ny / 2;
        blocks2 = (long long)fl_div_up(hx, 2 * kFanX) * fl_div_up(hy, 2);
    } else {
        blocks2 = (long long)fl_div_up(s.nx, 2 * 128) * ((s.ny + 1) / 2) * s.nt;
    }
    return blocks2 >= 4LL * 152 ? 2 : 1;
}

namespace {

// The fan forward's transposed copy of its input (walk_fan), in the plan's
// buffer (allocated with the plan: nothing is allocated here, so a forward
// can be captured in a CUDA graph): by TMA where it applies, else by a
// shared-memory tile transpose.
template <typename TX>
const TX* fan_transposed(fl_plan* p, const void* x, cudaStream_t st)
{
    const fl_scan& s = p->s;
    const int dt = std::is_same<TX, float>::value    ? FL_F32
                   : std::is_same<TX, __half>::value ? FL_F16
                                                     : FL_BF16;
    if (fl_fan_transpose_tma(p, x, dt, st)) return (const TX*)p->d_xt;   // fan_tma.cu
    const dim3 grid(fl_div_up(s.nx, 32), fl_div_up(s.ny, 32), s.nt);
    k_transpose_fan<TX><<<grid, dim3(32, 8), 0, st>>>((const TX*)x, (TX*)p->d_xt, s.nx, s.ny,
                                                      p->n_vox_frame);
    return (const TX*)p->d_xt;
}

template <typename TX, typename TY>
void launch_fwd(fl_plan* p, const void* x, void* y, int cr_power, const int* skip,
                const float* xscale, int yfold, cudaStream_t st)
{
    const fl_scan& s = p->s;
    const dim3 fb = p->fwd_bx ? dim3(p->fwd_bx, p->fwd_by) : dim3(8, 16);
    if (s.ndim == 3 && fl_plan_refl(p)) {
        const int NR = fl_plan_refl(p);
        const ReflGeom g = refl_geom(NR, s.nv, s.na, s.nb);
        dim3 grid(fl_div_up(s.na, fb.x), g.slots, fl_div_up(s.nb / 2, fb.y));
#define FL_FWD_REFL(NR_)                                                                     \
    k_fwd_refl<TX, TY, NR_><<<grid, fb, 0, st>>>(                                            \
        (const TX*)x, (TY*)y, p->d_col, p->d_colr, p->d_row, s.nx, s.ny, s.nz, s.na, s.nb, s.nv, \
        p->n_vox_frame, s.scale, cr_power, skip, xscale, yfold)
        if (NR == 4) FL_FWD_REFL(4);
        else FL_FWD_REFL(2);
#undef FL_FWD_REFL
    } else if (s.ndim == 3 && p->zmirror && p->rot && p->rot4) {
        dim3 grid(fl_div_up(s.na, fb.x), s.nv / 4, fl_div_up(s.nb / 2, fb.y));
        k_fwd_oct<TX, TY><<<grid, fb, 0, st>>>(
            (const TX*)x, (TY*)y, p->d_col, p->d_colr, p->d_row, s.nx, s.nz, s.na, s.nb, s.nv,
            p->n_vox_frame, s.scale, cr_power, skip, xscale, yfold);
    } else if (s.ndim == 3 && p->zmirror && p->rot) {
        dim3 grid(fl_div_up(s.na, fb.x), s.nv / 2, fl_div_up(s.nb / 2, fb.y));
        k_fwd_quad<TX, TY><<<grid, fb, 0, st>>>(
            (const TX*)x, (TY*)y, p->d_col, p->d_colr, p->d_row, s.nx, s.ny, s.nz, s.na, s.nb,
            s.nv, p->n_vox_frame, s.scale, cr_power, skip, xscale, yfold);
    } else if (s.ndim == 3 && p->zmirror) {
        dim3 grid(fl_div_up(s.na, fb.x), s.nv, fl_div_up(s.nb / 2, fb.y));
        k_fwd_cone<TX, TY, true><<<grid, fb, 0, st>>>(
            (const TX*)x, (TY*)y, p->d_col, p->d_colr, p->d_row, p->d_view_frame, s.nx, s.ny,
            s.nz, s.na, s.nb, p->n_vox_frame, s.scale, cr_power, skip, xscale, yfold);
    } else if (s.ndim == 3) {
        dim3 grid(fl_div_up(s.na, fb.x), s.nv, fl_div_up(s.nb, fb.y));
        k_fwd_cone<TX, TY, false><<<grid, fb, 0, st>>>(
            (const TX*)x, (TY*)y, p->d_col, p->d_colr, p->d_row, p->d_view_frame, s.nx, s.ny,
            s.nz, s.na, s.nb, p->n_vox_frame, s.scale, cr_power, skip, xscale, 0);
    } else if (fl_plan_refl(p)) {
        const TX* xt = fan_transposed<TX>(p, x, st);
        const int NR = fl_plan_refl(p);
        const long long nr = (long long)s.na * fan_refl_geom(NR, s.nv, s.na).slots;
        const int lanes = fl_plan_fan_lanes(p);
        const unsigned g = fl_div_up(nr, kFanBlock / lanes);
#define FL_FAN_REFL(NN)                                                                      \
    k_fwd_fan_refl<TX, TY, NN><<<g, kFanBlock, 0, st>>>(                                     \
        (const TX*)x, xt, (TY*)y, p->d_col, p->d_colr, s.nx, s.ny, s.na, s.nv, s.scale,         \
        cr_power, skip, xscale, yfold, lanes)
        if (NR == 4) FL_FAN_REFL(4);
        else if (NR == 2) FL_FAN_REFL(2);
        else FL_FAN_REFL(1);
#undef FL_FAN_REFL
    } else if (fl_plan_turns(p) > 1) {
        const TX* xt = fan_transposed<TX>(p, x, st);
        const int G = fl_plan_turns(p);
        const long long nr = (long long)s.na * (s.nv / G);
        const int lanes = fl_plan_fan_lanes(p);
        const unsigned g = fl_div_up(nr, kFanBlock / lanes);
#define FL_FAN_TURN(GG)                                                                      \
    k_fwd_fan_turn<TX, TY, GG><<<g, kFanBlock, 0, st>>>(                                     \
        (const TX*)x, xt, (TY*)y, p->d_col, p->d_colr, s.nx, s.ny, s.na, s.nv, s.scale,         \
        cr_power, skip, xscale, yfold, lanes)
        if (G == 4) FL_FAN_TURN(4);
        else FL_FAN_TURN(2);
#undef FL_FAN_TURN
    } else {
        long long nr = (long long)s.na * s.nv;
        const TX* xt = fan_transposed<TX>(p, x, st);
        k_fwd_fan<TX, TY><<<fl_div_up(nr, 128), 128, 0, st>>>(
            (const TX*)x, xt, (TY*)y, p->d_col, p->d_colr, p->d_view_frame, s.nx, s.ny, s.na,
            s.nv, p->n_vox_frame, s.scale, cr_power, skip, xscale);
    }
}

template <typename TX>
void launch_fwd_y(fl_plan* p, const void* x, void* y, int yt, int cr_power, const int* skip,
                  const float* xscale, int yfold, cudaStream_t st)
{
    if (yt == FL_F32) launch_fwd<TX, float>(p, x, y, cr_power, skip, xscale, yfold, st);
    else if (yt == FL_F16) launch_fwd<TX, __half>(p, x, y, cr_power, skip, xscale, yfold, st);
    else launch_fwd<TX, __nv_bfloat16>(p, x, y, cr_power, skip, xscale, yfold, st);
}

// The cone backprojections, input TW (FP32, or FP16 in the mixed CGLS form).
template <typename TX, typename TW>
void launch_adj_cone(fl_plan* p, const TW* yw, void* x, const int* skip, int xfold,
                     cudaStream_t st)
{
    const fl_scan& s = p->s;
    DetGrid G = det_grid(p);
    {
        constexpr int TZ = 8;
        const int nzw = p->zmirror ? s.nz / 2 : s.nz;
        int zruns = (nzw + TZ - 1) / TZ;
        if (fl_plan_refl(p)) {
            // runs of 2 voxels or of 1; one or two rows per iteration, or (runs
            // of 2) one pass over the run's rows: fl_plan_autotune
            const int NR = fl_plan_refl(p);
            const int run = p->adj_run == 1 ? 1 : 2;
            const int ru = p->adj_rows == 2 ? 2 : (p->adj_rows == 3 && run == 2 ? 0 : 1);
            zruns = (nzw + run - 1) / run;
            const dim3 ab = p->adj_bx ? dim3(p->adj_bx, p->adj_by) : dim3(8, 16);
            dim3 grid(fl_div_up(s.nx / 2, ab.x), fl_div_up(s.ny / 2, ab.y), (unsigned)zruns);
            // view chunks (fl_plan_adj_chunks): launches over consecutive
            // walked views, so the blocks resident together read the same
            // views' rows from L2; FP32 output only
            const int nch = fl_plan_adj_chunks(p, std::is_same<TX, float>::value);
            const int wper = (refl_geom(NR, s.nv, s.na, s.nb).ov + nch) / nch;
#define FL_ADJ_REFL(TZ_, RU_, NR_)                                                             \
    for (int c = 0; c < nch; c++)                                                             \
        k_adj_refl<TX, TZ_, RU_, TW, NR_><<<grid, ab, 0, st>>>(                                 \
            (TX*)x, yw, p->d_col, p->d_rowz, p->d_view, G, s.nx, s.ny, s.nz, s.na, s.nb, s.nv,   \
            s.dz, skip, xfold, c * wper, c * wper + wper - 1, c == 0, c == nch - 1, p->d_dq,    \
            s.nz / 2)
#define FL_ADJ_REFL_NR(NR_)                                                                    \
    do {                                                                                       \
        if (run == 1 && ru == 1) FL_ADJ_REFL(1, 1, NR_);                                      \
        else if (run == 1) FL_ADJ_REFL(1, 2, NR_);                                            \
        else if (ru == 1) FL_ADJ_REFL(2, 1, NR_);                                             \
        else if (ru == 2) FL_ADJ_REFL(2, 2, NR_);                                             \
        else FL_ADJ_REFL(2, 0, NR_);                                                          \
    } while (0)
            if (NR == 4) FL_ADJ_REFL_NR(4);
            else FL_ADJ_REFL_NR(2);
#undef FL_ADJ_REFL_NR
#undef FL_ADJ_REFL
        } else if (p->zmirror && p->rot && p->rot4) {
            // runs of 2: the four columns' 16 accumulators keep 8 blocks per SM
            constexpr int TO = 2;
            zruns = (nzw + TO - 1) / TO;
            const dim3 ab = p->adj_bx ? dim3(p->adj_bx, p->adj_by) : dim3(8, 16);
            dim3 grid(fl_div_up(s.nx / 2, ab.x), fl_div_up(s.ny / 2, ab.y), (unsigned)zruns);
            k_adj_oct<TX, TO, TW><<<grid, ab, 0, st>>>(
                (TX*)x, yw, p->d_col, p->d_rowz, p->d_view, G, s.nx, s.nz, s.na, s.nb, s.nv,
                s.dz, skip, xfold);
        } else if (p->zmirror && p->rot) {
            // runs of 4: the two columns' 16 accumulators keep 8 blocks per SM
            constexpr int TQ = 4;
            zruns = (nzw + TQ - 1) / TQ;
            const dim3 ab = p->adj_bx ? dim3(p->adj_bx, p->adj_by) : dim3(16, 8);
            dim3 grid(fl_div_up(s.nx, ab.x), fl_div_up(s.ny / 2, ab.y), (unsigned)zruns);
            k_adj_quad<TX, TQ, TW><<<grid, ab, 0, st>>>(
                (TX*)x, yw, p->d_col, p->d_rowz, p->d_view, G, s.nx, s.ny, s.nz, s.na, s.nb, s.nv,
                s.dz, zruns, skip, xfold);
        } else if (p->zmirror) {
            const dim3 ab = p->adj_bx ? dim3(p->adj_bx, p->adj_by) : dim3(16, 8);
            dim3 grid(fl_div_up(s.nx, ab.x), fl_div_up(s.ny, ab.y), (unsigned)zruns * s.nt);
            k_adj_cone<TX, TZ, true, TW><<<grid, ab, 0, st>>>(
                (TX*)x, yw, p->d_col, p->d_rowz, p->d_view, p->d_idY, p->d_Nv, p->tmp_size, G,
                s.nx, s.ny, s.nz, s.na, s.nb, s.dz, zruns, skip, xfold);
        } else {
            const dim3 ab = p->adj_bx ? dim3(p->adj_bx, p->adj_by) : dim3(32, 4);
            dim3 grid(fl_div_up(s.nx, ab.x), fl_div_up(s.ny, ab.y), (unsigned)zruns * s.nt);
            k_adj_cone<TX, TZ, false, TW><<<grid, ab, 0, st>>>(
                (TX*)x, yw, p->d_col, p->d_rowz, p->d_view, p->d_idY, p->d_Nv, p->tmp_size, G,
                s.nx, s.ny, s.nz, s.na, s.nb, s.dz, zruns, skip, 0);
        }
    }
}

template <typename TX>
void launch_adj(fl_plan* p, const float* yw, void* x, const int* skip, int xfold,
                cudaStream_t st)
{
    const fl_scan& s = p->s;
    DetGrid G = det_grid(p);
    if (s.ndim == 3) {
        launch_adj_cone<TX, float>(p, yw, x, skip, xfold, st);
    } else if (fl_plan_refl(p)) {
        // one PB x PB block of primary pixels per thread (fan_refl_pblock); the
        // octant's blocks right of the diagonal have no primary block and return
        const int NR = fl_plan_refl(p);
        const int PB = fan_refl_pblock(NR, s.nx, s.ny);
        const int hxb = (NR == 1 ? s.nx : s.nx / 2) / PB, hyb = (s.ny / 2) / PB;
        const int NG = fl_plan_fan_groups(p);
        const dim3 blk(kFanX, NG), g1(fl_div_up(hxb, kFanX), hyb);
#define FL_ADJ_FAN_REFL(NN, PP, GG)                                                          \
    k_adj_fan_refl<TX, NN, PP, GG><<<g1, blk, 0, st>>>((TX*)x, yw, p->d_col, p->d_view, G,   \
                                                       s.nx, s.ny, s.na, s.nv, skip)
#define FL_ADJ_FAN_REFL_G(NN, PP)                                                            \
    do {                                                                                     \
        if (NG == 16) FL_ADJ_FAN_REFL(NN, PP, 16);                                           \
        else FL_ADJ_FAN_REFL(NN, PP, kTurnGroups);                                           \
    } while (0)
        if (NR == 4 && PB == 2) FL_ADJ_FAN_REFL(4, 2, kTurnGroups);   // fl_plan_fan_groups
        else if (NR == 4) FL_ADJ_FAN_REFL_G(4, 1);
        else if (NR == 2 && PB == 2) FL_ADJ_FAN_REFL_G(2, 2);
        else if (NR == 2) FL_ADJ_FAN_REFL_G(2, 1);
        else if (PB == 2) FL_ADJ_FAN_REFL_G(1, 2);
        else FL_ADJ_FAN_REFL_G(1, 1);
#undef FL_ADJ_FAN_REFL_G
#undef FL_ADJ_FAN_REFL
    } else if (fl_plan_turns(p) > 1) {
        // 2 x 2 primary blocks once there are at least 4 waves of them, else
        // one primary pixel per thread (the same bits)
        const int T = fl_plan_turns(p);
        const int hx = T == 2 ? s.nx : s.nx / 2, hy = s.ny / 2;
        const int NG = fl_plan_fan_groups(p);
        const dim3 blk(kFanX, NG);
        const dim3 g2(fl_div_up(hx, 2 * kFanX), fl_div_up(hy, 2)), g1(fl_div_up(hx, kFanX), hy);
        const bool two = fl_plan_fan_block(p) == 2;
#define FL_ADJ_FAN_TURN(TT, PP, GG)                                                          \
    k_adj_fan_turn<TX, TT, PP, GG><<<PP == 2 ? g2 : g1, blk, 0, st>>>(                       \
        (TX*)x, yw, p->d_col, p->d_view, G, s.nx, s.ny, s.na, s.nv, skip)
#define FL_ADJ_FAN_TURN_G(TT, PP)                                                            \
    do {                                                                                     \
        if (NG == 16) FL_ADJ_FAN_TURN(TT, PP, 16);                                           \
        else FL_ADJ_FAN_TURN(TT, PP, kTurnGroups);                                           \
    } while (0)
        if (T == 4 && two) FL_ADJ_FAN_TURN_G(4, 2);
        else if (T == 4) FL_ADJ_FAN_TURN_G(4, 1);
        else if (two) FL_ADJ_FAN_TURN_G(2, 2);
        else FL_ADJ_FAN_TURN_G(2, 1);
#undef FL_ADJ_FAN_TURN_G
#undef FL_ADJ_FAN_TURN
    } else {
        // 2 x 2 pixel blocks, one thread each, once there are at least 4 waves
        // of 128-thread blocks; else one pixel per view group
        if (fl_plan_fan_block(p) == 2) {
            dim3 grid(fl_div_up(s.nx, 2 * 128), (s.ny + 1) / 2, s.nt);
            k_adj_fan<TX, 2, false><<<grid, 128, 0, st>>>((TX*)x, yw, p->d_col, p->d_view,
                                                           p->d_idY, p->d_Nv, p->tmp_size, G,
                                                           s.nx, s.ny, s.na, skip);
        } else {
            dim3 grid(fl_div_up(s.nx, kFanX), s.ny, s.nt);
            k_adj_fan<TX, 1, true><<<grid, dim3(kFanX, kFanGroups), 0, st>>>(
                (TX*)x, yw, p->d_col, p->d_view, p->d_idY, p->d_Nv, p->tmp_size, G, s.nx, s.ny,
                s.na, skip);
        }
    }
}

template <typename T>
void launch_fold(fl_plan* p, const void* src, void* dst, int unfold, cudaStream_t st)
{
    const fl_scan& s = p->s;
    const long long nxy = (long long)s.nx * s.ny;
    const long long npf = nxy * (s.nz / 2), np = npf * s.nt;
    unsigned g = (unsigned)std::min<long long>((np + 255) / 256, 16LL * 152);
    if (p->rot)                 // half- or quarter-turn plan: tiled (one frame)
        k_fold_tiled<T><<<g, 256, 0, st>>>((const T*)src, (T*)dst, s.nx, s.ny, s.nz, npf,
                                           unfold);
    else
        k_fold<T><<<g, 256, 0, st>>>((const T*)src, (T*)dst, nxy, s.nz, npf, np, unfold);
}

size_t dtype_bytes(int t) { return t == FL_F32 ? 4 : 2; }

template <int G>
void launch_weight_packed(fl_plan* p, const void* y, int yt, float* yw, cudaStream_t st)
{
    const fl_scan& s = p->s;
    const long long npk = (long long)(s.nv / G) * (s.nb / 2) * s.na;
    const unsigned g = fl_div_up(npk, 256);
    if (yt == FL_F32)
        k_weight_packed<float, G><<<g, 256, 0, st>>>(yw, (const float*)y, p->d_colr, p->d_row,
                                                     s.na, s.nb, s.nv, npk, s.scale);
    else if (yt == FL_F16)
        k_weight_packed<__half, G><<<g, 256, 0, st>>>(yw, (const __half*)y, p->d_colr, p->d_row,
                                                      s.na, s.nb, s.nv, npk, s.scale);
    else
        k_weight_packed<__nv_bfloat16, G><<<g, 256, 0, st>>>(yw, (const __nv_bfloat16*)y,
                                                             p->d_colr, p->d_row, s.na, s.nb,
                                                             s.nv, npk, s.scale);
}

template <int NR>
void launch_weight_packed_refl(fl_plan* p, const void* y, int yt, float* yw, cudaStream_t st)
{
    const fl_scan& s = p->s;
    const ReflGeom gm = refl_geom(NR, s.nv, s.na, s.nb);
    const long long npk = (long long)gm.slots * gm.nbh * s.na;
    const unsigned g = fl_div_up(npk, 256);
    if (yt == FL_F32)
        k_weight_packed_refl<float, NR><<<g, 256, 0, st>>>(yw, (const float*)y, p->d_colr,
                                                           p->d_row, s.na, s.nb, s.nv, npk,
                                                           s.scale);
    else if (yt == FL_F16)
        k_weight_packed_refl<__half, NR><<<g, 256, 0, st>>>(yw, (const __half*)y, p->d_colr,
                                                            p->d_row, s.na, s.nb, s.nv, npk,
                                                            s.scale);
    else
        k_weight_packed_refl<__nv_bfloat16, NR><<<g, 256, 0, st>>>(
            yw, (const __nv_bfloat16*)y, p->d_colr, p->d_row, s.na, s.nb, s.nv, npk, s.scale);
}

template <int G>
void launch_weight_fan_packed(fl_plan* p, const void* y, int yt, float* yw, cudaStream_t st)
{
    const fl_scan& s = p->s;
    const long long npk = (long long)s.na * (s.nv / G);
    const unsigned g = fl_div_up(npk, 256);
    if (yt == FL_F32)
        k_weight_fan_packed<float, G><<<g, 256, 0, st>>>(yw, (const float*)y, p->d_colr, s.na,
                                                         s.nv, npk, s.scale);
    else if (yt == FL_F16)
        k_weight_fan_packed<__half, G><<<g, 256, 0, st>>>(yw, (const __half*)y, p->d_colr, s.na,
                                                          s.nv, npk, s.scale);
    else
        k_weight_fan_packed<__nv_bfloat16, G><<<g, 256, 0, st>>>(
            yw, (const __nv_bfloat16*)y, p->d_colr, s.na, s.nv, npk, s.scale);
}

template <int NR>
void launch_weight_fan_refl(fl_plan* p, const void* y, int yt, float* yw, cudaStream_t st)
{
    const fl_scan& s = p->s;
    const long long ns = (long long)s.na * fan_refl_geom(NR, s.nv, s.na).slots;
    const unsigned g = fl_div_up(ns, 256);
    if (yt == FL_F32)
        k_weight_fan_refl<float, NR><<<g, 256, 0, st>>>(yw, (const float*)y, p->d_colr, s.na,
                                                        s.nv, ns, s.scale);
    else if (yt == FL_F16)
        k_weight_fan_refl<__half, NR><<<g, 256, 0, st>>>(yw, (const __half*)y, p->d_colr, s.na,
                                                         s.nv, ns, s.scale);
    else
        k_weight_fan_refl<__nv_bfloat16, NR><<<g, 256, 0, st>>>(
            yw, (const __nv_bfloat16*)y, p->d_colr, s.na, s.nv, ns, s.scale);
}

}  // namespace

int fl_matched_fold(fl_plan* p, const void* src, void* dst, int dtype, int unfold,
                    cudaStream_t st)
{
    if (!p->zmirror) return fl_set_error(FL_ERR_INVALID, "fold: plan has no z-mirror layout");
    if (dtype == FL_F32) launch_fold<float>(p, src, dst, unfold, st);
    else if (dtype == FL_F16) launch_fold<__half>(p, src, dst, unfold, st);
    else launch_fold<__nv_bfloat16>(p, src, dst, unfold, st);
    return fl_check_launch(unfold ? "z-unfold" : "z-fold");
}

int fl_matched_forward(fl_plan* p, const void* x, int xt, void* y, int yt, int cr_power,
                       const int* skip, const float* xscale, int layout, cudaStream_t st)
{
    int yfold = 0;
    if (p->s.ndim == 3 && p->zmirror) {
        if (!(layout & FL_LAY_X_FOLDED)) {
            void* w;
            int e = fl_plan_vwork(p, (size_t)p->n_vox * dtype_bytes(xt), &w);
            if (e) return e;
            if ((e = fl_matched_fold(p, x, w, xt, 0, st))) return e;
            x = w;
        }
        yfold = (layout & FL_LAY_Y_ADJ) ? 1 : 0;
    } else if (p->s.ndim == 2 && fl_plan_turns(p) > 1) {
        yfold = (layout & FL_LAY_Y_ADJ) ? 1 : 0;      // the packed fan layout
    }
    if (xt == FL_F32) launch_fwd_y<float>(p, x, y, yt, cr_power, skip, xscale, yfold, st);
    else if (xt == FL_F16) launch_fwd_y<__half>(p, x, y, yt, cr_power, skip, xscale, yfold, st);
    else launch_fwd_y<__nv_bfloat16>(p, x, y, yt, cr_power, skip, xscale, yfold, st);
    return fl_check_launch("matched forward");
}

int fl_matched_weight(fl_plan* p, const void* y, int yt, float* yw, cudaStream_t st)
{
    const fl_scan& s = p->s;
    long long nr = p->n_rays;
    int three = s.ndim == 3;
    if (three && fl_plan_refl(p)) {
        if (fl_plan_refl(p) == 4) launch_weight_packed_refl<4>(p, y, yt, yw, st);
        else launch_weight_packed_refl<2>(p, y, yt, yw, st);
        return fl_check_launch("matched adjoint weighting");
    }
    if (three && p->zmirror && p->rot) {
        if (p->rot4) launch_weight_packed<4>(p, y, yt, yw, st);
        else launch_weight_packed<2>(p, y, yt, yw, st);
        return fl_check_launch("matched adjoint weighting");
    }
    if (!three && fl_plan_refl(p)) {
        if (fl_plan_refl(p) == 4) launch_weight_fan_refl<4>(p, y, yt, yw, st);
        else if (fl_plan_refl(p) == 2) launch_weight_fan_refl<2>(p, y, yt, yw, st);
        else launch_weight_fan_refl<1>(p, y, yt, yw, st);
        return fl_check_launch("matched adjoint weighting");
    }
    if (!three && fl_plan_turns(p) > 1) {
        if (fl_plan_turns(p) == 4) launch_weight_fan_packed<4>(p, y, yt, yw, st);
        else launch_weight_fan_packed<2>(p, y, yt, yw, st);
        return fl_check_launch("matched adjoint weighting");
    }
    if (three && p->zmirror) {
        long long np = (long long)s.nv * (s.nb / 2) * s.na;
        unsigned g = fl_div_up(np, 256);
        const int hv = s.nv;            // view period: every view has its own rays here
        if (yt == FL_F32)
            k_weight_fold<float><<<g, 256, 0, st>>>(yw, (const float*)y, p->d_colr, p->d_row,
                                                    s.na, s.nb, np, s.scale, hv);
        else if (yt == FL_F16)
            k_weight_fold<__half><<<g, 256, 0, st>>>(yw, (const __half*)y, p->d_colr, p->d_row,
                                                     s.na, s.nb, np, s.scale, hv);
        else
            k_weight_fold<__nv_bfloat16><<<g, 256, 0, st>>>(yw, (const __nv_bfloat16*)y,
                                                            p->d_colr, p->d_row, s.na, s.nb, np,
                                                            s.scale, hv);
        return fl_check_launch("matched adjoint weighting");
    }
    unsigned g = fl_div_up(nr, 256);
    if (yt == FL_F32)
        k_weight<float><<<g, 256, 0, st>>>(yw, (const float*)y, p->d_colr, p->d_row, s.na,
                                           s.nb, nr, s.scale, three);
    else if (yt == FL_F16)
        k_weight<__half><<<g, 256, 0, st>>>(yw, (const __half*)y, p->d_colr, p->d_row, s.na,
                                            s.nb, nr, s.scale, three);
    else
        k_weight<__nv_bfloat16><<<g, 256, 0, st>>>(yw, (const __nv_bfloat16*)y, p->d_colr,
                                                   p->d_row, s.na, s.nb, nr, s.scale, three);
    return fl_check_launch("matched adjoint weighting");
}

int fl_matched_adjoint_w(fl_plan* p, const float* yw, void* x, int xt, const int* skip,
                         int layout, cudaStream_t st)
{
    const int xfold = (p->zmirror && (layout & FL_LAY_X_FOLDED)) ? 1 : 0;
    if (xt == FL_F32) launch_adj<float>(p, yw, x, skip, xfold, st);
    else if (xt == FL_F16) launch_adj<__half>(p, yw, x, skip, xfold, st);
    else launch_adj<__nv_bfloat16>(p, yw, x, skip, xfold, st);
    return fl_check_launch("matched adjoint");
}

int fl_matched_adjoint_wt(fl_plan* p, const void* yw, int wt, void* x, int xt, const int* skip,
                          int layout, cudaStream_t st)
{
    if (wt == FL_F32) return fl_matched_adjoint_w(p, (const float*)yw, x, xt, skip, layout, st);
    if (wt != FL_F16 || p->s.ndim != 3)
        return fl_set_error(FL_ERR_UNSUPPORTED,
                            "matched adjoint: FP16 input is for cone plans only");
    const int xfold = (p->zmirror && (layout & FL_LAY_X_FOLDED)) ? 1 : 0;
    const __half* w = (const __half*)yw;
    if (xt == FL_F32) launch_adj_cone<float, __half>(p, w, x, skip, xfold, st);
    else if (xt == FL_F16) launch_adj_cone<__half, __half>(p, w, x, skip, xfold, st);
    else launch_adj_cone<__nv_bfloat16, __half>(p, w, x, skip, xfold, st);
    return fl_check_launch("matched adjoint (FP16 input)");
}

// Launch-shape autotuner of the matched projector kernels: each candidate
// below is timed (CUDA events, one launch after one untimed) on the plan's own
// geometry, with the plan's scratch as input and output, and the fastest kept
// for the forward and for the backprojection.
// * Cone plans: the 128-thread block shapes of both kernels, and for the
//   reflection backprojection runs of 1 or 2 voxels per thread with 1 or 2
//   rows per iteration or one pass over a run's rows. A thread's result does
//   not depend on these, so neither do the projections.
// * Fan plans: the parts per walked ray of the turn forward (1, 4, 16: the
//   order of a ray's additions, within FP32 rounding) and the pixel block of
//   the backprojections (1 or 2: the same bits).
extern "C" int fl_plan_autotune(fl_plan* p, void* stream, int32_t* shapes)
{
    FL_RANGE("fl_plan_autotune");
    if (!p) return fl_set_error(FL_ERR_INVALID, "fl_plan_autotune: null plan");
    int st = fl_matched_ready(p);
    if (st) return st;
    const bool cone = p->s.ndim == 3;
    if (p->det_kind < 0 || (cone && p->det_kind == 1)) {   // no matched backprojection
        if (shapes) shapes[0] = shapes[1] = shapes[2] = shapes[3] = 0;
        return fl_set_error(FL_OK, "");
    }
    cudaStream_t s = (cudaStream_t)stream;
    float* y = nullptr;
    void* x = nullptr;
    if ((st = fl_plan_work(p, &y))) return st;
    if ((st = fl_plan_vwork(p, (size_t)p->n_vox * sizeof(float), &x))) return st;
    FL_CUDA(cudaMemsetAsync(y, 0, (size_t)p->n_rays * sizeof(float), s));
    FL_CUDA(cudaMemsetAsync(x, 0, (size_t)p->n_vox * sizeof(float), s));
    const int lay = p->zmirror ? FL_LAY_X_FOLDED : 0;
    cudaEvent_t e0, e1;
    FL_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fl_set_error(FL_ERR_CUDA, "fl_plan_autotune: cudaEventCreate failed");
    }
    auto timed = [&](bool fwd, float& ms) -> int {
        for (int rep = 0; rep < 2; rep++) {
            if (rep == 1 && cudaEventRecord(e0, s) != cudaSuccess) return FL_ERR_CUDA;
            int e = fwd ? fl_matched_forward(p, x, FL_F32, y, FL_F32, 2, nullptr, nullptr,
                                             lay | FL_LAY_Y_ADJ, s)
                        : fl_matched_adjoint_w(p, y, x, FL_F32, nullptr, lay, s);
            if (e) return e;
        }
        if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
            return fl_set_error(FL_ERR_CUDA, "fl_plan_autotune: timing failed");
        return FL_OK;
    };
    if (cone) {
        static const int cand[4][2] = {{8, 16}, {16, 8}, {32, 4}, {4, 32}};
        // the reflection backprojection also tries voxel runs of 2 and 1 per
        // thread with one or two rows per iteration, and runs of 2 in one pass
        // over their rows (variant r: run, rows)
        static const int var[5][2] = {{2, 1}, {1, 1}, {2, 2}, {1, 2}, {2, 3}};
        const int nvar = fl_plan_refl(p) ? 5 : 1;
        for (int pass = 0; pass < 2 && !st; pass++) {
            const bool fwd = pass == 0;
            float best = 3.0e38f;
            int bi = 0, br = 0;
            for (int c = 0; c < 4 && !st; c++)
                for (int r = 0; r < (fwd ? 1 : nvar) && !st; r++) {
                    if (fwd) { p->fwd_bx = cand[c][0]; p->fwd_by = cand[c][1]; }
                    else {
                        p->adj_bx = cand[c][0]; p->adj_by = cand[c][1];
                        p->adj_run = var[r][0]; p->adj_rows = var[r][1];
                    }
                    float ms = 0.0f;
                    st = timed(fwd, ms);
                    if (!st && ms < best) { best = ms; bi = c; br = r; }
                }
            if (fwd) { p->fwd_bx = cand[bi][0]; p->fwd_by = cand[bi][1]; }
            else {
                p->adj_bx = cand[bi][0]; p->adj_by = cand[bi][1];
                p->adj_run = var[br][0]; p->adj_rows = var[br][1];
            }
        }
        // then the view chunks of the reflection backprojection (FP32 output)
        if (!st && fl_plan_refl(p) && p->zmirror) {
            static const int chunks[4] = {1, 4, 8, 16};
            float best = 3.0e38f;
            int bi = 0;
            for (int c = 0; c < 4 && !st; c++) {
                p->adj_chunks = chunks[c];
                float ms = 0.0f;
                st = timed(false, ms);
                if (!st && ms < best) { best = ms; bi = c; }
            }
            p->adj_chunks = chunks[bi];
        }
        if (st)
            p->fwd_bx = p->fwd_by = p->adj_bx = p->adj_by = p->adj_run = p->adj_rows =
                p->adj_chunks = 0;
    } else {
        static const int parts[3] = {1, 4, 16};
        const bool turn = fl_plan_turns(p) > 1;
        for (int pass = 0; pass < 2 && !st; pass++) {
            const bool fwd = pass == 0;
            if (fwd && !turn) continue;            // the general forward has no parts
            float best = 3.0e38f;
            int bi = 0;
            // backprojection: pixel block 1 or 2 x view groups 8 or 16 (turn
            // and reflection forms; the general one has its own groups)
            const int nc = fwd ? 3 : (turn ? 4 : 2);
            for (int c = 0; c < nc && !st; c++) {
                if (fwd) p->fan_lanes = parts[c];
                else { p->fan_block = c % 2 + 1; p->fan_groups = c < 2 ? kTurnGroups : 16; }
                float ms = 0.0f;
                st = timed(fwd, ms);
                if (!st && ms < best) { best = ms; bi = c; }
            }
            if (fwd) p->fan_lanes = parts[bi];
            else { p->fan_block = bi % 2 + 1; p->fan_groups = bi < 2 ? kTurnGroups : 16; }
        }
        if (st) p->fan_lanes = p->fan_block = p->fan_groups = 0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;                    // the built-in shapes are kept after a failure
    if (shapes) {
        if (cone) {
            shapes[0] = p->fwd_bx; shapes[1] = p->fwd_by;
            shapes[2] = p->adj_bx; shapes[3] = p->adj_by;
        } else {
            shapes[0] = fl_plan_fan_lanes(p); shapes[1] = 0;
            shapes[2] = fl_plan_fan_block(p); shapes[3] = fl_plan_fan_groups(p);
        }
    }
    return fl_set_error(FL_OK, "");
}

int fl_matched_count(fl_plan* p, int32_t* counts, cudaStream_t st)
{
    const fl_scan& s = p->s;
    long long nr = p->n_rays;
    k_count<<<fl_div_up(nr, 128), 128, 0, st>>>(counts, p->d_col, p->d_row, s.nx, s.ny, s.nz,
                                                s.na, s.nb, s.nv, s.ndim == 3);
    return fl_check_launch("intersection count");
}

// ---------------------------------------------------------------------------
// Bounds-checked builds: violations counted by the matched and batched kernels
// ---------------------------------------------------------------------------
FL_OOB_ACCESSOR(fl_oob_matched)
extern "C" unsigned long long fl_oob_batch(int reset);

extern "C" int fl_debug_bounds(int64_t* violations, int reset)
{
    if (!violations) return fl_set_error(FL_ERR_INVALID, "fl_debug_bounds: null argument");
#ifdef FL_BOUNDS_CHECK
    FL_CUDA(cudaDeviceSynchronize());
    *violations = (int64_t)(fl_oob_matched(reset) + fl_oob_batch(reset));
    return fl_set_error(FL_OK, "");
#else
    *violations = 0;
    return fl_set_error(FL_ERR_UNSUPPORTED, "library built without FL_BOUNDS_CHECK");
#endif
}
