// matched_dev.cuh -- device building blocks of the matched Siddon model shared
// by the single-scan kernels (matched.cu) and the batched fan kernels
// (batch.cu): the incremental ray walk, the per-ray weight c_r, and the
// detector-column window of an xy box used by the gathers.
#pragma once
#include "fl_common.cuh"
#include "fl_plan.h"

namespace {

template <typename T>
__device__ __forceinline__ float ldv(const T* p) { return Store<T>::ld(p); }

// ---------------------------------------------------------------------------
// Crossings in a segment frame (the model is described in fl_plan.h).
// ---------------------------------------------------------------------------
constexpr int kSegCone = 7;    // 3-D rays: segments of 128 planes of the dominant axis
constexpr int kSegFan = 4;     // fan rays: segments of 16 planes

// Crossing of the plane with m = k - kq relative to the anchor bh + be,
// cb = c - be: the expression both projectors evaluate.
__device__ __forceinline__ float xrel(const AxisEntry& a, float m, float bh, float cb)
{
    return __fadd_rn(__fmaf_rn(m, a.ih, -bh), __fmaf_rn(m, a.il, cb));
}

// Both planes of a pair at once (m2 = (k0 - kq, k1 - kq)); per lane the same
// roundings as xrel.
__device__ __forceinline__ float2 xrel2(const AxisEntry& a, float2 m2, float bh, float cb)
{
    return __fadd2_rn(__ffma2_rn(m2, make_float2(a.ih, a.ih), make_float2(-bh, -bh)),
                      __ffma2_rn(m2, make_float2(a.il, a.il), make_float2(cb, cb)));
}

// Absolute crossing of plane k, hi part only: for estimates (which segments a
// ray meets, first guesses of its voxels) and detector windows, never a weight.
__device__ __forceinline__ float xabs(const AxisEntry& a, float k)
{
    return __fmul_rn(__fsub_rn(k, a.kq), a.ih);
}

// A ray's dominant xy axis, which its segments are cut along: the one with
// the smaller |ih| (the larger direction component).
__device__ __forceinline__ bool x_dominant(const AxisEntry& X, const AxisEntry& Y)
{
    return fabsf(X.ih) <= fabsf(Y.ih);
}

// Anchor of segment s of a ray (dominant axis D of nD planes): the crossing of
// the segment's middle plane (clamped to the volume) as bh + be, be holding
// the rounding of bh exactly and the table's low parts.
template <int SH>
__device__ __forceinline__ void make_anchor(const AxisEntry& D, int s, int nD, float& bh,
                                            float& be)
{
    const float m = __fsub_rn((float)min((s << SH) + (1 << (SH - 1)), nD), D.kq);
    bh = __fmul_rn(m, D.ih);
    be = __fadd_rn(__fmaf_rn(m, D.il, __fmaf_rn(m, D.ih, -bh)), D.c);
}

// First guess of the slab of an axis holding the absolute parameter a.
__device__ __forceinline__ int slab_guess(const AxisEntry& ax, float a, int n)
{
    float k = floorf(__fadd_rn(ax.kq, __fdividef(a, ax.ih)));
    k = fminf(fmaxf(k, 0.0f), (float)(n - 1));      // NaN -> 0
    return (int)k;
}

// Slab j in [lo, hi) of an axis holding the parameter v of a frame: a
// positive axis (ih > 0) t(j) <= v < t(j+1), a negative one t(j+1) <= v <
// t(j), found from the guess j (clamped into the range). Each loop moves one
// way and is bounded by the range.
__device__ __forceinline__ int slab_at(const AxisEntry& a, bool pos, int j, int lo, int hi,
                                       float v, float bh, float cb)
{
    j = min(max(j, lo), hi - 1);
    if (pos) {
        while (j + 1 < hi && xrel(a, __fsub_rn((float)(j + 1), a.kq), bh, cb) <= v) j++;
        while (j > lo && xrel(a, __fsub_rn((float)j, a.kq), bh, cb) > v) j--;
    } else {
        while (j > lo && xrel(a, __fsub_rn((float)j, a.kq), bh, cb) <= v) j--;
        while (j + 1 < hi && xrel(a, __fsub_rn((float)(j + 1), a.kq), bh, cb) > v) j++;
    }
    return j;
}

// Which segments of its dominant axis a ray can cross: from the box's entry
// and exit parameters (absolute hi parts), with one plane of margin on each
// side (a segment it does not cross is found empty in its own frame). Returns
// false for a ray that misses the box by more than the estimate's rounding.
template <int SH>
__device__ __forceinline__ bool seg_range(const AxisEntry& D, int nD, float a_in, float a_out,
                                          int& s1, int& s2)
{
    const float tol = 4e-7f * fmaxf(fabsf(a_in), fabsf(a_out)) + 1e-30f;
    if (!(a_in < a_out + tol)) return false;
    const float k1 = __fadd_rn(D.kq, __fdividef(a_in, D.ih));
    const float k2 = __fadd_rn(D.kq, __fdividef(a_out, D.ih));
    const float lo = fmaxf(floorf(fminf(k1, k2)) - 1.0f, 0.0f);          // NaN -> 0
    const float hi = fminf(floorf(fmaxf(k1, k2)) + 1.0f, (float)(nD - 1));
    if (!(lo <= hi)) return false;
    s1 = (int)lo >> SH;
    s2 = (int)hi >> SH;
    return true;
}

// ---------------------------------------------------------------------------
// The forward walk. A ray's matrix entries are, per segment s of its
// dominant axis, the weights
//   w_rV = fl(min_a U_a(V) - max_a L_a(V))    (entry c_r w_rV when positive)
// of the voxels V whose dominant index lies in the segment, with L_a / U_a
// the crossings (in segment s's frame) of the planes where the ray enters /
// leaves V's slab on axis a. Segments are independent: the walk visits them
// in the ray's order and walks each one's sub-box (the segment's dominant
// slabs times the other axes' full ranges) from its entry v_in, stepping the
// axes whose next crossing is the smallest (all tied axes at once). Every
// visited voxel's segment is then exactly its w_rV: it starts at the latest
// crossing behind the voxel and ends at the earliest ahead, and the voxels it
// skips have w_rV <= 0. The backprojection evaluates the same expression per
// (voxel, ray) in the voxel's own segment.
//
// The axis entries are read from global memory (kq and c again at every
// segment start, so they hold no registers during the steps).
// Body (the gathers of one kernel form):
//   at(jx, jy, jz)        load the value(s) of voxel (jx, jy, jz)
//   take(seg, more, jx, jy, jz)
//                         if more, load the value(s) of the new current voxel
//                         (jx, jy, jz); then add seg times the value(s) of
//                         the voxel just left
// Termination: each step advances at least one axis inside a finite
// sub-box; the step budget is a second, independent bound.
// ---------------------------------------------------------------------------
// One dominant axis (XD: x, else y), the segments [s1, s2] in the ray's order.
template <bool THREE, bool XD, typename Body>
__device__ __forceinline__ void seg_walk_dom(const ColEntry* __restrict__ ce,
                                             const AxisEntry* __restrict__ pZ, int nx, int ny,
                                             int nzr, int s1, int s2, int jx, int jy, int jz,
                                             Body& body)
{
    constexpr int SH = THREE ? kSegCone : kSegFan;
    const float ihx = __ldg(&ce->x.ih), ilx = __ldg(&ce->x.il);
    const float ihy = __ldg(&ce->y.ih), ily = __ldg(&ce->y.il);
    const float ihz = THREE ? __ldg(&pZ->ih) : 1.0f, ilz = THREE ? __ldg(&pZ->il) : 0.0f;
    const bool px = ihx > 0.0f, py = ihy > 0.0f, pz = ihz > 0.0f;
    const bool pd = XD ? px : py;
    const int nD = XD ? nx : ny;
    const int nseg = s2 - s1;
    for (int q = 0; q <= nseg; q++) {
        const int s = pd ? s1 + q : s2 - q;
        const AxisEntry X{__ldg(&ce->x.kq), ihx, ilx, __ldg(&ce->x.c)};
        const AxisEntry Y{__ldg(&ce->y.kq), ihy, ily, __ldg(&ce->y.c)};
        const AxisEntry Z{THREE ? __ldg(&pZ->kq) : 0.0f, ihz, ilz, THREE ? __ldg(&pZ->c) : 0.0f};
        float bh, be;
        make_anchor<SH>(XD ? X : Y, s, nD, bh, be);
        const float cbx = __fsub_rn(X.c, be), cby = __fsub_rn(Y.c, be);
        const float cbz = THREE ? __fsub_rn(Z.c, be) : 0.0f;
        const int dlo = s << SH, dhi = min((s + 1) << SH, nD);
        // the sub-box's entry and exit in this frame
        const float tx0 = xrel(X, __fsub_rn((float)(XD ? dlo : 0), X.kq), bh, cbx);
        const float tx1 = xrel(X, __fsub_rn((float)(XD ? dhi : nx), X.kq), bh, cbx);
        const float ty0 = xrel(Y, __fsub_rn((float)(XD ? 0 : dlo), Y.kq), bh, cby);
        const float ty1 = xrel(Y, __fsub_rn((float)(XD ? ny : dhi), Y.kq), bh, cby);
        float v_in = fmaxf(fminf(tx0, tx1), fminf(ty0, ty1));
        float v_out = fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1));
        if (THREE) {
            const float tz0 = xrel(Z, __fsub_rn(0.0f, Z.kq), bh, cbz);
            const float tz1 = xrel(Z, __fsub_rn((float)nzr, Z.kq), bh, cbz);
            v_in = fmaxf(v_in, fminf(tz0, tz1));
            v_out = fminf(v_out, fmaxf(tz0, tz1));
        }
        if (!(v_in < v_out)) continue;
        jx = slab_at(X, px, jx, XD ? dlo : 0, XD ? dhi : nx, v_in, bh, cbx);
        jy = slab_at(Y, py, jy, XD ? 0 : dlo, XD ? ny : dhi, v_in, bh, cby);
        if (THREE) jz = slab_at(Z, pz, jz, 0, nzr, v_in, bh, cbz);
        float mx = __fsub_rn((float)(px ? jx + 1 : jx), X.kq);
        float my = __fsub_rn((float)(py ? jy + 1 : jy), Y.kq);
        float mz = THREE ? __fsub_rn((float)(pz ? jz + 1 : jz), Z.kq) : 0.0f;
        float Ux = xrel(X, mx, bh, cbx), Uy = xrel(Y, my, bh, cby);
        float Uz = THREE ? xrel(Z, mz, bh, cbz) : 3.0e38f;
        body.at(jx, jy, jz);
        float cur = v_in;
        // The voxel being left is the sub-box's last exactly when the next
        // crossing reaches the sub-box's exit: every voxel inside has its
        // next crossings at or before the exit planes', and the exit plane's
        // crossing is computed from the same m as v_out.
        const int budget = (dhi - dlo) + (XD ? ny : nx) + (THREE ? nzr : 0) + 2;
#pragma unroll 2
        for (int it = 0; it < budget; it++) {
            const float nxt = THREE ? fminf(fminf(Ux, Uy), Uz) : fminf(Ux, Uy);
            const float seg = __fsub_rn(nxt, cur);
            const bool more = nxt < v_out;             // false at the exit (and for NaN)
            if (Ux == nxt) {
                jx += px ? 1 : -1;
                mx = __fadd_rn(mx, px ? 1.0f : -1.0f); Ux = xrel(X, mx, bh, cbx);
            }
            if (Uy == nxt) {
                jy += py ? 1 : -1;
                my = __fadd_rn(my, py ? 1.0f : -1.0f); Uy = xrel(Y, my, bh, cby);
            }
            if (THREE && Uz == nxt) {
                jz += pz ? 1 : -1;
                mz = __fadd_rn(mz, pz ? 1.0f : -1.0f); Uz = xrel(Z, mz, bh, cbz);
            }
            body.take(seg, more, jx, jy, jz);
            if (!more) break;
            cur = nxt;
        }
    }
}

// The walk of ray (ce, pZ) through an nx x ny (x nzr) box: finds the segments
// it can cross and its first slabs, then walks them along its dominant axis.
template <bool THREE, typename Body>
__device__ __forceinline__ void seg_walk(const ColEntry* __restrict__ ce,
                                         const AxisEntry* __restrict__ pZ, int nx, int ny,
                                         int nzr, Body& body)
{
    constexpr int SH = THREE ? kSegCone : kSegFan;
    const AxisEntry X = ce->x, Y = ce->y;
    float a_in = fmaxf(fminf(xabs(X, 0.0f), xabs(X, (float)nx)),
                       fminf(xabs(Y, 0.0f), xabs(Y, (float)ny)));
    float a_out = fminf(fmaxf(xabs(X, 0.0f), xabs(X, (float)nx)),
                        fmaxf(xabs(Y, 0.0f), xabs(Y, (float)ny)));
    int jz = 0;
    if (THREE) {
        const AxisEntry Z = *pZ;
        const float z0 = xabs(Z, 0.0f), z1 = xabs(Z, (float)nzr);
        a_in = fmaxf(a_in, fminf(z0, z1));
        a_out = fminf(a_out, fmaxf(z0, z1));
        jz = slab_guess(Z, a_in, nzr);
    }
    const bool xd = x_dominant(X, Y);
    int s1 = 0, s2 = -1;
    const bool hit = seg_range<SH>(xd ? X : Y, xd ? nx : ny, a_in, a_out, s1, s2);
    // Warp alignment: when the warp's rays share their dominant axis and its
    // direction (all but the warps at a 45-degree switch), every lane walks
    // the warp's whole range of segments, so that all lanes work on the same
    // segment at the same time instead of drifting a segment apart (a lane's
    // first segment depends on where its ray enters). A segment a ray does
    // not cross is empty in its own frame and costs the lane only the test.
    const unsigned am = __activemask();
    const bool pd = xd ? X.ih > 0.0f : Y.ih > 0.0f;
    const int key = (xd ? 2 : 0) | (pd ? 1 : 0);
    const int lo = __reduce_min_sync(am, hit ? s1 : 0x7fffffff);
    const int hi = __reduce_max_sync(am, hit ? s2 : -1);
    if (!hit) return;
    if (__match_any_sync(am, key) == am) { s1 = lo; s2 = hi; }
    const int jx = slab_guess(X, a_in, nx), jy = slab_guess(Y, a_in, ny);
    if (xd) seg_walk_dom<THREE, true>(ce, pZ, nx, ny, nzr, s1, s2, jx, jy, jz, body);
    else seg_walk_dom<THREE, false>(ce, pZ, nx, ny, nzr, s1, s2, jx, jy, jz, body);
}

// Body of the general forward and the count: the standard volume, or with
// MIRROR the z-folded one (pairs of voxel (ix, iy, iz) and its mirror (ix,
// iy, nz-1-iz) at pair index (iz*ny + iy)*nx + ix; acc gets the voxel's sum,
// accm the mirror's -- the companion ray of a scan symmetric about the
// source plane). COUNT: counts the voxels with w > 0, no loads. xlen:
// elements available at x (checked builds verify every gather index).
template <typename TX, bool COUNT, bool MIRROR>
struct GenBody {
    const TX* __restrict__ x;
    long long xlen;
    int nx, ny;
    int cnt = 0;
    float acc = 0.0f, xv = 0.0f;
    float2 acc2 = make_float2(0.0f, 0.0f), xv2 = make_float2(0.0f, 0.0f);
    __device__ __forceinline__ void load(int jx, int jy, int jz, float& s, float2& s2) const
    {
        if (COUNT) return;
        const int v = (jz * ny + jy) * nx + jx;      // < 2^31 (checked at plan creation)
        if (MIRROR) {
            s2 = make_float2(0.0f, 0.0f);
            if (FL_IN(2 * (long long)v + 1, xlen)) s2 = Store<TX>::ld2(x + 2 * (long long)v);
        } else {
            s = 0.0f;
            if (FL_IN(v, xlen)) s = ldv(x + v);
        }
    }
    __device__ __forceinline__ void at(int jx, int jy, int jz) { load(jx, jy, jz, xv, xv2); }
    __device__ __forceinline__ void take(float seg, bool more, int jx, int jy, int jz)
    {
        float xn = 0.0f;
        float2 xn2 = make_float2(0.0f, 0.0f);
        if (more) load(jx, jy, jz, xn, xn2);
        if (COUNT) cnt += seg > 0.0f;
        else if (MIRROR) acc2 = __ffma2_rn(make_float2(seg, seg), xv2, acc2);
        else acc = fmaf(seg, xv, acc);
        xv = xn;
        xv2 = xn2;
    }
};

// The general walk (2-D with THREE = false; z-folded volume with MIRROR: the
// ray must descend from the source plane, so it stays in iz < nz/2).
// Returns sum over voxels of w * x; *nseg counts segments with w > 0.
template <typename TX, bool THREE, bool COUNT, bool MIRROR = false>
__device__ __forceinline__ float walk(const TX* __restrict__ x, const ColEntry* ce,
                                      const AxisEntry* pZ, int nx, int ny, int nz, int* nseg,
                                      float* accm = nullptr, long long xlen = 0)
{
    GenBody<TX, COUNT, MIRROR> b{x, xlen, nx, ny};
    if (!(MIRROR && !(__ldg(&pZ->ih) < 0.0f)))      // the folded walk takes descending rays
        seg_walk<THREE>(ce, pZ, nx, ny, THREE ? (MIRROR ? nz / 2 : nz) : 1, b);
    if (COUNT) *nseg = b.cnt;
    if (MIRROR) { *accm = b.acc2.y; return b.acc2.x; }
    return b.acc;
}

// Folded pair index of voxel (x, y, z) in the 4 x 4 tiled volume of a
// half- or quarter-turn plan (fl_plan.h); zb = z * nx * ny, nx4 = nx / 4.
// The voxel turned by pi, (nx-1-x, ny-1-y, z), is at 2 zb + nx ny - 1 minus it.
__device__ __forceinline__ int tiled_pair(int x, int y, int zb, int nx4)
{
    return zb + (((y >> 2) * nx4 + (x >> 2)) << 4) + ((y & 3) << 2) + (x & 3);
}

// The z-mirror walk of a descending ray with the half-turn partner (plan
// flag rot): besides the folded pair of voxel (ix, iy, iz) it gathers the
// pair of voxel (nx-1-ix, ny-1-iy, iz), which the turned ray of view v + nv/2
// crosses with the same segment. x is the tiled folded volume (nx, ny
// multiples of 4). acc gets the (voxel, mirror) sums, accr the turned pair's.
template <typename TX>
struct QuadBody {
    const TX* __restrict__ x;
    long long xlen;
    int nxy, nx4;
    float2 acc = make_float2(0.0f, 0.0f), accr = make_float2(0.0f, 0.0f);
    float2 xv = make_float2(0.0f, 0.0f), xr = make_float2(0.0f, 0.0f);
    __device__ __forceinline__ void load(int jx, int jy, int jz, float2& a, float2& r) const
    {
        const int zb = jz * nxy;                     // < 2^31 (checked at plan creation)
        const int t = tiled_pair(jx, jy, zb, nx4), tr = 2 * zb + nxy - 1 - t;
        a = make_float2(0.0f, 0.0f); r = a;
        if (FL_IN(2 * (long long)t + 1, xlen)) a = Store<TX>::ld2(x + 2 * (long long)t);
        if (FL_IN(2 * (long long)tr + 1, xlen)) r = Store<TX>::ld2(x + 2 * (long long)tr);
    }
    __device__ __forceinline__ void at(int jx, int jy, int jz) { load(jx, jy, jz, xv, xr); }
    __device__ __forceinline__ void take(float seg, bool more, int jx, int jy, int jz)
    {
        float2 xn = make_float2(0.0f, 0.0f), xnr = xn;
        if (more) load(jx, jy, jz, xn, xnr);
        acc = __ffma2_rn(make_float2(seg, seg), xv, acc);
        accr = __ffma2_rn(make_float2(seg, seg), xr, accr);
        xv = xn;
        xr = xnr;
    }
};

template <typename TX>
__device__ __forceinline__ void walk_quad(const TX* __restrict__ x, const ColEntry* ce,
                                          const AxisEntry* pZ, int nx, int ny, int nz,
                                          float2* acc, float2* accr, long long xlen)
{
    QuadBody<TX> b{x, xlen, nx * ny, nx >> 2};
    if (__ldg(&pZ->ih) < 0.0f) seg_walk<true>(ce, pZ, nx, ny, nz / 2, b);
    *acc = b.acc;
    *accr = b.accr;
}

// The z-mirror walk with all four quarter turns (plan flag rot4, nx == ny ==
// n, a multiple of 4): per step it gathers the folded pairs of voxel (ix, iy)
// and of its turns R^j (ix, iy), R (x, y) = (n-1-y, x), which the ray of view
// v + j nv/4 at the same column and row crosses with the same segment. x is
// the tiled folded volume. acc[j] gets the (voxel, mirror) sums of turn j.
template <typename TX>
struct OctBody {
    const TX* __restrict__ x;
    long long xlen;
    int n, nn, n4;
    float2 acc[4], xv[4];
    __device__ __forceinline__ void load(int jx, int jy, int jz, float2 (&o)[4]) const
    {
        const int zb = jz * nn;
        int q[4];                                    // turns 2, 3 are turns 0, 1 by pi
        q[0] = tiled_pair(jx, jy, zb, n4);
        q[1] = tiled_pair(n - 1 - jy, jx, zb, n4);
        q[2] = 2 * zb + nn - 1 - q[0];
        q[3] = 2 * zb + nn - 1 - q[1];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            o[j] = make_float2(0.0f, 0.0f);
            if (FL_IN(2 * (long long)q[j] + 1, xlen)) o[j] = Store<TX>::ld2(x + 2 * (long long)q[j]);
        }
    }
    __device__ __forceinline__ void at(int jx, int jy, int jz) { load(jx, jy, jz, xv); }
    __device__ __forceinline__ void take(float seg, bool more, int jx, int jy, int jz)
    {
        float2 xn[4];
#pragma unroll
        for (int j = 0; j < 4; j++) xn[j] = make_float2(0.0f, 0.0f);
        if (more) load(jx, jy, jz, xn);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            acc[j] = __ffma2_rn(make_float2(seg, seg), xv[j], acc[j]);
            xv[j] = xn[j];
        }
    }
};

template <typename TX>
__device__ __forceinline__ void walk_oct(const TX* __restrict__ x, const ColEntry* ce,
                                         const AxisEntry* pZ, int n, int nz, float2 (&acc)[4],
                                         long long xlen)
{
    OctBody<TX> b;
    b.x = x; b.xlen = xlen; b.n = n; b.nn = n * n; b.n4 = n >> 2;
#pragma unroll
    for (int j = 0; j < 4; j++) { b.acc[j] = make_float2(0.0f, 0.0f); b.xv[j] = b.acc[j]; }
    if (__ldg(&pZ->ih) < 0.0f) seg_walk<true>(ce, pZ, n, n, nz / 2, b);
#pragma unroll
    for (int j = 0; j < 4; j++) acc[j] = b.acc[j];
}

// The z-mirror walk of a reflection form (fl_plan.h): NR = 4, the quarter
// turns and the reflection (square grid); NR = 2, the half turn and the
// reflection. Per step the folded pairs of the voxel's 2 NR images g_k =
// R^(4k/NR) (k < NR) and R^(4(k-NR)/NR) M (k >= NR), with M (x, y) = (x,
// ny-1-y), R (x, y) = (n-1-y, x), R^2 (x, y) = (nx-1-x, ny-1-y); R M (x, y) =
// (y, x). acc[k] gets the (voxel, mirror) sums of image k, the sums of the ray
// g_k takes the walked ray to.
template <typename TX, int NR>
struct ReflBody {
    const TX* __restrict__ x;
    long long xlen;
    int nx, ny, nxy, nx4;
    float2 acc[2 * NR], xv[2 * NR];
    __device__ __forceinline__ void load(int jx, int jy, int jz, float2 (&o)[2 * NR]) const
    {
        const int zb = jz * nxy, pi2 = 2 * zb + nxy - 1;  // q -> pi2 - q: the turn by pi
        int q[2 * NR];
        if (NR == 4) {
            q[0] = tiled_pair(jx, jy, zb, nx4);
            q[1] = tiled_pair(nx - 1 - jy, jx, zb, nx4);
            q[4] = tiled_pair(jx, ny - 1 - jy, zb, nx4);
            q[5] = tiled_pair(jy, jx, zb, nx4);
            q[2] = pi2 - q[0];
            q[3] = pi2 - q[1];
            q[6] = pi2 - q[4];
            q[7] = pi2 - q[5];
        } else {
            q[0] = tiled_pair(jx, jy, zb, nx4);
            q[2] = tiled_pair(jx, ny - 1 - jy, zb, nx4);
            q[1] = pi2 - q[0];
            q[3] = pi2 - q[2];
        }
#pragma unroll
        for (int j = 0; j < 2 * NR; j++) {
            o[j] = make_float2(0.0f, 0.0f);
            if (FL_IN(2 * (long long)q[j] + 1, xlen)) o[j] = Store<TX>::ld2(x + 2 * (long long)q[j]);
        }
    }
    __device__ __forceinline__ void at(int jx, int jy, int jz) { load(jx, jy, jz, xv); }
    __device__ __forceinline__ void take(float seg, bool more, int jx, int jy, int jz)
    {
        float2 xn[2 * NR];
#pragma unroll
        for (int j = 0; j < 2 * NR; j++) xn[j] = make_float2(0.0f, 0.0f);
        if (more) load(jx, jy, jz, xn);
#pragma unroll
        for (int j = 0; j < 2 * NR; j++) {
            acc[j] = __ffma2_rn(make_float2(seg, seg), xv[j], acc[j]);
            xv[j] = xn[j];
        }
    }
};

template <typename TX, int NR>
__device__ __forceinline__ void walk_refl(const TX* __restrict__ x, const ColEntry* ce,
                                          const AxisEntry* pZ, int nx, int ny, int nz,
                                          float2 (&acc)[2 * NR], long long xlen)
{
    ReflBody<TX, NR> b;
    b.x = x; b.xlen = xlen; b.nx = nx; b.ny = ny; b.nxy = nx * ny; b.nx4 = nx >> 2;
#pragma unroll
    for (int j = 0; j < 2 * NR; j++) { b.acc[j] = make_float2(0.0f, 0.0f); b.xv[j] = b.acc[j]; }
    if (__ldg(&pZ->ih) < 0.0f) seg_walk<true>(ce, pZ, nx, ny, nz / 2, b);
#pragma unroll
    for (int j = 0; j < 2 * NR; j++) acc[j] = b.acc[j];
}

// Views and input layout of a reflection form (fl_plan.h). The walked views
// are w = 0 .. ov (ov = nv/8 for NR = 4, floor(nv/4) for NR = 2). View 0 walks
// its columns a < na/2; so does view ov when it is its own mirror image ("end":
// NR = 4, or NR = 2 with nv a multiple of 4), walked from table row endrow
// (nv: the exact angle pi/4; nv + 1: the exact angle pi/2). The backprojection
// input has two planes of nv nb na / 2 values (the turn images, the reflected
// images), vpr = 2 NR values per walked ray and plane (NR images x two rows).
// Per plane: with an end view, slots s < ov of nb/2 rows x na columns, slot 0
// holding view 0 at columns < na/2 and view ov at columns >= na/2, slot s
// view s; without one, slot s < ov holds view s + 1 and a half slot at the end
// (rows of na/2 columns) view 0.
struct ReflGeom {
    int nv, na, nbh, ov, end, endrow, vpr, slots;   // slots: forward grid (whole and half)
    long long slot, plane;                          // values per slot / per plane
};

__host__ __device__ inline ReflGeom refl_geom(int NR, int nv, int na, int nb)
{
    ReflGeom g;
    g.nv = nv; g.na = na; g.nbh = nb / 2;
    g.ov = NR == 4 ? nv / 8 : nv / 4;
    g.end = NR == 4 || nv % 4 == 0;
    g.endrow = NR == 4 ? nv : nv + 1;
    g.vpr = 2 * NR;
    g.slots = g.end ? g.ov : g.ov + 1;
    g.slot = (long long)g.nbh * na * g.vpr;
    g.plane = (long long)nv * nb * na / 2;
    return g;
}

// Fan reflection forms (fl_plan::refl on a fan plan, NR = 1, 2 or 4): with
// M (x, y) = (x, ny-1-y), S = the identity (NR = 1), the half turn R^2 (NR =
// 2) or the quarter turn R (NR = 4) and q = nv/NR, the walked views v = 0 ..
// ov (ov = floor(q/2)) define
//   A[(v + j q, a), S^j p] = A[(j q - v, na-1-a), S^j M p] = A[(v, a), p].
// View 0, and view ov where q is even (then its own mirror image), walk their
// columns a < na/2 only; view ov is walked from table row nv (NR = 4: the
// exact angle pi/4) or nv + 1 (NR = 2: the exact angle pi/2). NR = 1 takes
// odd view counts (no end view). The packed input holds the 2 NR values of a
// walked ray's orbit side by side (the turn images', then the reflected
// images'), in slots of na columns laid out as the cone's (refl_slot /
// refl_view with one row): nv * na values in all.
struct FanReflGeom {
    int nv, na, ov, end, endrow, vpr, slots;
    long long slot;                                 // values per slot
};

__host__ __device__ inline FanReflGeom fan_refl_geom(int NR, int nv, int na)
{
    FanReflGeom g;
    g.nv = nv; g.na = na;
    const int q = nv / NR;
    g.ov = q / 2;
    g.end = q % 2 == 0;
    g.endrow = NR == 4 ? nv : nv + 1;
    g.vpr = 2 * NR;
    g.slots = g.end ? g.ov : g.ov + 1;
    g.slot = (long long)na * g.vpr;
    return g;
}

// Forward slot (s, column ia) of a reflection form: the walked view v, its
// table row vt and column a, and where its values go in each plane (offset
// off + vpr (ib stride + ia) + 2 k for row ib, image k mod NR). False for the
// unused half of the last slot. (Geo: ReflGeom, or FanReflGeom with one row.)
template <typename Geo>
__device__ __forceinline__ bool refl_slot(const Geo& g, int s, int ia, int& v, int& vt,
                                          int& a, long long& off, int& stride)
{
    const int h = g.na / 2;
    a = ia; stride = g.na;
    if (g.end) {
        off = s * g.slot;
        v = vt = s;
        if (s == 0 && ia >= h) { v = g.ov; vt = g.endrow; a = ia - h; }
        return true;
    }
    if (s == g.ov) {
        if (ia >= h) return false;
        v = vt = 0; off = g.ov * g.slot; stride = h;
        return true;
    }
    v = vt = s + 1; off = s * g.slot;
    return true;
}

// View and column of the ray that image k of a walked ray (v, a) is, on a
// reflection form (NR = 4, 2 or 1): k < NR the turn S^k (view v + k nv/NR,
// column a), k >= NR the reflection S^(k-NR) M (view (k-NR) nv/NR - v,
// column na-1-a).
template <int NR>
__device__ __forceinline__ void refl_image(int k, int v, int a, int na, int nv, long long& vk,
                                           int& ak)
{
    const int sv = nv / NR;
    if (k < NR) { vk = v + (long long)k * sv; ak = a; }
    else { vk = ((long long)(k - NR) * sv - v + nv) % nv; ak = na - 1 - a; }
}

// Backprojection view w of a reflection form: table row, the plane offset of
// its values (column ia, row ib at base + vpr (ib stride + ia)), and the
// number of its walked columns.
template <typename Geo>
__device__ __forceinline__ void refl_view(const Geo& g, int w, int& vt, long long& base,
                                          int& stride, int& alim)
{
    const int h = g.na / 2;
    stride = g.na; alim = g.na; vt = w;
    if (g.end) {
        base = w * g.slot;
        if (w == 0) alim = h;
        else if (w == g.ov) { vt = g.endrow; base = (long long)g.vpr * h; alim = h; }
        return;
    }
    if (w == 0) { base = g.ov * g.slot; stride = h; alim = h; }
    else base = (w - 1) * g.slot;
}
// The fan walk in batches of kFanBatch steps: the crossings of a batch are
// found first (they do not depend on the image), then its gathers are issued
// together and the segments added in walk order -- the same sums as the
// general walk, bit for bit, waiting for the gathers once per batch.
// G = 1: the ray's own pixels (acc[0]). G = 2 or 4 (a turn plan, one frame):
// per step also the turns R^j (ix, iy) of the pixel -- G = 2: R (x, y) =
// (nx-1-x, ny-1-y); G = 4 (nx == ny == n): R (x, y) = (n-1-y, x) -- which
// the ray of view v + j nv/G at the same column crosses with the same
// segment; acc[j] gets turn j's sum.
// L > 1: the ray's segments (in walk order) are dealt to L parts, part k
// taking those with index q in [k S / L, (k+1) S / L) of the S it can cross;
// this call walks part `lane`. Segments are independent, so every matrix
// entry lies whole in one part and is the walk's own; only the order of the
// additions changes (the caller adds the parts in lane order).
// RF (a fan reflection form, G = NR = 1, 2 or 4): per step also the images
// S^j M (ix, iy) of the pixel, M (x, y) = (x, ny-1-y), into acc[G + j].
constexpr int kFanBatch = 4;

// xt: the same image transposed, xt[x ny + y] = x[y nx + x]. A warp's rays
// at one step lie along the detector, across the direction they travel: for
// an image ray that travels mostly along x they sit in one column of pixels,
// consecutive in xt, so its gathers read xt; the others read x. The values,
// and so the sums, are the same either way.
// walk_fan_parts: the same walk with the parts count L a run-time value.
template <typename TX, int G, bool RF>
__device__ __forceinline__ void walk_fan_parts(const TX* __restrict__ x,
                                               const TX* __restrict__ xt, const AxisEntry* pX,
                                               const AxisEntry* pY, int nx, int ny,
                                               float (&acc)[RF ? 2 * G : G], long long xlen,
                                               int lane, int L);

template <typename TX, int G, int L = 1, bool RF = false>
__device__ __forceinline__ void walk_fan(const TX* __restrict__ x, const TX* __restrict__ xt,
                                         const AxisEntry* pX, const AxisEntry* pY, int nx,
                                         int ny, float (&acc)[RF ? 2 * G : G], long long xlen,
                                         int lane = 0)
{
    walk_fan_parts<TX, G, RF>(x, xt, pX, pY, nx, ny, acc, xlen, lane, L);
}

template <typename TX, int G, bool RF>
__device__ __forceinline__ void walk_fan_parts(const TX* __restrict__ x,
                                               const TX* __restrict__ xt, const AxisEntry* pX,
                                               const AxisEntry* pY, int nx, int ny,
                                               float (&acc)[RF ? 2 * G : G], long long xlen,
                                               int lane, int L)
{
    const AxisEntry X = *pX, Y = *pY;
    static_assert(G == 1 || G == 2 || G == 4, "one, two or four turns");
    constexpr int SH = kSegFan;
    constexpr int NI = RF ? 2 * G : G;             // images per step
    // steps batched per gather round (eight images: two, within the registers)
    constexpr int NB = NI > 4 ? 2 : kFanBatch;
#pragma unroll
    for (int j = 0; j < NI; j++) acc[j] = 0.0f;
    const float a_in = fmaxf(fminf(xabs(X, 0.0f), xabs(X, (float)nx)),
                             fminf(xabs(Y, 0.0f), xabs(Y, (float)ny)));
    const float a_out = fminf(fmaxf(xabs(X, 0.0f), xabs(X, (float)nx)),
                              fmaxf(xabs(Y, 0.0f), xabs(Y, (float)ny)));
    const bool xd = x_dominant(X, Y);
    const AxisEntry D = xd ? X : Y;
    const int nD = xd ? nx : ny;
    int s1, s2;
    if (!seg_range<SH>(D, nD, a_in, a_out, s1, s2)) return;
    const bool px = X.ih > 0.0f, py = Y.ih > 0.0f, pd = xd ? px : py;
    const int S = s2 - s1 + 1;
    const int q0 = L > 1 ? (lane * S) / L : 0, q1 = L > 1 ? ((lane + 1) * S) / L : S;
    if (q0 >= q1) return;
    // first guesses at the entry of this part's first segment
    float ag = a_in;
    if (L > 1 && q0 > 0) {
        const int s = pd ? s1 + q0 : s2 - q0;
        ag = fmaxf(a_in, xabs(D, (float)(pd ? (s << SH) : min((s + 1) << SH, nD))));
    }
    int jx = slab_guess(X, ag, nx), jy = slab_guess(Y, ag, ny);
    const int nxy = nx * ny;                       // < 2^31 (checked at plan creation)
    // The array the walked ray's own direction reads (xt when it travels
    // mostly along x, else x) is E, the other O. Two running indices a, b
    // address every image: in E, a the pixel and b its mirror image M p
    // (x-dominant: x ny + y and x ny + ny-1-y in xt; else y nx + x and
    // (ny-1-y) nx + x in x). With G = 4 the odd images (quarter turns) travel
    // across, and read O, where b is the quarter turn C_1 and a the image
    // D_1 = R M p (x n + n-1-y and x n + y in x, or (n-1-y) n + x and y n + x
    // in xt). The turns by pi are nxy - 1 minus these, in either array.
    const TX* E = xd ? xt : x;
    const TX* O = xd ? x : xt;
    const int sx = xd ? ny : 1, sy = xd ? 1 : nx;   // a's steps in x and y
    const int dax = px ? sx : -sx, day = py ? sy : -sy;
    const float stx = px ? 1.0f : -1.0f, sty = py ? 1.0f : -1.0f;
    float sacc[NI];
#pragma unroll
    for (int j = 0; j < NI; j++) sacc[j] = 0.0f;
    for (int q = q0; q < q1; q++) {
        const int s = pd ? s1 + q : s2 - q;
        float bh, be;
        make_anchor<SH>(D, s, nD, bh, be);
        const float cbx = __fsub_rn(X.c, be), cby = __fsub_rn(Y.c, be);
        const int dlo = s << SH, dhi = min((s + 1) << SH, nD);
        const int lox = xd ? dlo : 0, hix = xd ? dhi : nx;
        const int loy = xd ? 0 : dlo, hiy = xd ? ny : dhi;
        const float tx0 = xrel(X, __fsub_rn((float)lox, X.kq), bh, cbx);
        const float tx1 = xrel(X, __fsub_rn((float)hix, X.kq), bh, cbx);
        const float ty0 = xrel(Y, __fsub_rn((float)loy, Y.kq), bh, cby);
        const float ty1 = xrel(Y, __fsub_rn((float)hiy, Y.kq), bh, cby);
        const float v_in = fmaxf(fminf(tx0, tx1), fminf(ty0, ty1));
        const float v_out = fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1));
        if (!(v_in < v_out)) continue;
        jx = slab_at(X, px, jx, lox, hix, v_in, bh, cbx);
        jy = slab_at(Y, py, jy, loy, hiy, v_in, bh, cby);
        float mx = __fsub_rn((float)(px ? jx + 1 : jx), X.kq);
        float my = __fsub_rn((float)(py ? jy + 1 : jy), Y.kq);
        float Ux = xrel(X, mx, bh, cbx), Uy = xrel(Y, my, bh, cby);
        int a = xd ? jx * ny + jy : jy * nx + jx;
        int b = xd ? jx * ny + (ny - 1 - jy) : (ny - 1 - jy) * nx + jx;
        float cur = v_in;
        bool in = true;
        const int budget = (hix - lox) + (hiy - loy) + 2;
        for (int it = 0; it < budget && in; it += NB) {
            float seg[NB];
            int ia[NB], ib[NB];
            bool live[NB];
#pragma unroll
            for (int u = 0; u < NB; u++) {
                const float nxt = fminf(Ux, Uy);
                live[u] = in;
                seg[u] = __fsub_rn(nxt, cur);
                ia[u] = a; ib[u] = b;
                if (in) {
                    // the last voxel of the sub-box: its next crossing is the exit
                    const bool more = nxt < v_out;
                    if (Ux == nxt) {
                        jx += px ? 1 : -1;
                        mx = __fadd_rn(mx, stx); Ux = xrel(X, mx, bh, cbx);
                        a += dax; b += dax;
                    }
                    if (Uy == nxt) {
                        jy += py ? 1 : -1;
                        my = __fadd_rn(my, sty); Uy = xrel(Y, my, bh, cby);
                        a += day; b -= day;
                    }
                    cur = nxt;
                    in = more;
                }
            }
            float vv[NB][NI];
#pragma unroll
            for (int u = 0; u < NB; u++) {
                // images C_0 .. C_{G-1}, then (RF) D_0 .. D_{G-1}
                const int A = ia[u], B = ib[u], A2 = nxy - 1 - A, B2 = nxy - 1 - B;
                const int q4[8] = {A, B, A2, B2, B, A, B2, A2};       // G = 4: odd ones in O
                const int q2[4] = {A, A2, B, B2};                      // G = 2
                const int q1[2] = {A, B};                              // G = 1
#pragma unroll
                for (int j = 0; j < NI; j++) {
                    const int q = G == 4 ? q4[j] : (G == 2 ? q2[j] : q1[j]);
                    const TX* arr = (G == 4 && (j & 1)) ? O : E;
                    vv[u][j] = 0.0f;
                    if (live[u] && FL_IN(q, xlen)) vv[u][j] = ldv(arr + q);
                }
            }
#pragma unroll
            for (int u = 0; u < NB; u++)
#pragma unroll
                for (int j = 0; j < NI; j++)
                    if (live[u]) sacc[j] = fmaf(seg[u], vv[u][j], sacc[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < NI; j++) acc[j] = sacc[j];
}

// The xy part of a cone ray's crossings with the voxel column (cx, cy): the
// frame of the column's segment (anchor bh + be) and the column's entry l and
// exit h in it, the crossings the forward walk computes for the column's
// planes. Returns false when the ray misses the column (l >= h).
__device__ __forceinline__ bool cone_column(const ColEntry& ce, int cx, int cy, int nx, int ny,
                                            float& bh, float& be, float& l, float& h)
{
    const bool xd = x_dominant(ce.x, ce.y);
    make_anchor<kSegCone>(xd ? ce.x : ce.y, (xd ? cx : cy) >> kSegCone, xd ? nx : ny, bh, be);
    const float mx = __fsub_rn((float)cx, ce.x.kq), my = __fsub_rn((float)cy, ce.y.kq);
    const float2 tx = xrel2(ce.x, make_float2(mx, __fadd_rn(mx, 1.0f)), bh,
                            __fsub_rn(ce.x.c, be));
    const float2 ty = xrel2(ce.y, make_float2(my, __fadd_rn(my, 1.0f)), bh,
                            __fsub_rn(ce.y.c, be));
    l = fmaxf(fminf(tx.x, tx.y), fminf(ty.x, ty.y));
    h = fminf(fmaxf(tx.x, tx.y), fmaxf(ty.x, ty.y));
    return l < h;
}

// Crossings of z planes k0 and k1 of row re in the frame bh + be.
__device__ __forceinline__ float2 row_planes(const AxisEntry& re, float k0, float k1, float bh,
                                             float be)
{
    return xrel2(re, make_float2(__fsub_rn(k0, re.kq), __fsub_rn(k1, re.kq)), bh,
                 __fsub_rn(re.c, be));
}

__device__ __forceinline__ float ray_cr(float scale, float dxy2, float dz2)
{
    return fmul(scale, fsqrt(fadd(dxy2, dz2)));
}

// ---------------------------------------------------------------------------
// Adjoint helpers: detector column window of an axis-aligned xy box.
// ---------------------------------------------------------------------------
struct DetGrid {
    int kind;          // 0 flat uniform, 1 equiangular
    float u0, du, g0, dg, v0, dv, SO, SD;
    float rdu, rdg;    // 1/du, 1/dg (column windows only: they carry 0.02 columns of slack)
};

// Column range [lo, hi] of rays that can cross the xy square [x0,x0+1]x[y0,y0+1]
// in a view with cos/sin (c, s); also returns the depth range SO + t.
__device__ __forceinline__ void column_window(const DetGrid& G, float c, float s, float x0,
                                              float y0, float wx, float wy, int na, int& lo,
                                              int& hi, float& dmin, float& dmax)
{
    float umin = 3.0e38f, umax = -3.0e38f;
    dmin = 3.0e38f; dmax = -3.0e38f;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float px = x0 + ((k & 1) ? wx : 0.0f);
        float py = y0 + ((k & 2) ? wy : 0.0f);
        float depth = G.SO + (c * px + s * py);        // distance from source along the axis
        float lat = -s * px + c * py;
        float u = (G.kind == 0) ? G.SD * __fdividef(lat, depth) : atan2f(lat, depth);
        umin = fminf(umin, u); umax = fmaxf(umax, u);
        dmin = fminf(dmin, depth); dmax = fmaxf(dmax, depth);
    }
    float f0, f1;
    if (G.kind == 0) { f0 = (umin - G.u0) * G.rdu; f1 = (umax - G.u0) * G.rdu; }
    else             { f0 = (umin - G.g0) * G.rdg; f1 = (umax - G.g0) * G.rdg; }
    if (f0 > f1) { float t = f0; f0 = f1; f1 = t; }
    // the rays of columns whose detector position lies in the shadow [f0, f1];
    // 0.02 column of slack covers the float evaluation and the tolerance
    // fl_plan_create allows between y_det and the uniform grid
    f0 = fmaxf(ceilf(f0 - 0.02f), 0.0f);
    f1 = fminf(floorf(f1 + 0.02f), (float)(na - 1));
    lo = (int)f0; hi = (int)f1;                   // empty when lo > hi
}

// Fan adjoint of a PX x PY block of pixels with lower corner (ix0, iy0): for
// the views views[g], views[g + kFanGroups], ... (view group g of nvf views)
// and every ray whose column window covers the block, w_rV * yw_r is added to
// each pixel the ray crosses, w_rV evaluated from the same crossing table as
// the forward walk. A group's sum runs over its views in order and the
// columns in increasing order, and only rays with w > 0 add to it, so each
// pixel's result does not depend on the block shape: the block's window
// contains every pixel's own window (the corners' column shadow with 0.02
// columns of slack is far wider than the FP32 error of w). The groups' sums
// are then added in the order g = 0, 1, ... (fan_combine_groups).
constexpr int kFanGroups = 4;

// The crossings of the planes ix0 .. ix0 + PX (x) and iy0 .. iy0 + PY (y) of
// fan ray ce, relative to the anchor of the segment holding the block (the
// block lies in one segment of either axis: PX, PY <= 2 and ix0, iy0
// multiples of them). These are the crossings the forward walk computes for
// the same planes in the same segment.
template <int PX, int PY>
__device__ __forceinline__ void fan_block_crossings(const ColEntry& ce, int ix0, int iy0, int nx,
                                                    int ny, float (&ax)[PX + 1],
                                                    float (&ay)[PY + 1])
{
    const bool xd = x_dominant(ce.x, ce.y);
    float bh, be;
    make_anchor<kSegFan>(xd ? ce.x : ce.y, (xd ? ix0 : iy0) >> kSegFan, xd ? nx : ny, bh, be);
    const float cbx = __fsub_rn(ce.x.c, be), cby = __fsub_rn(ce.y.c, be);
    const float mx = __fsub_rn((float)ix0, ce.x.kq), my = __fsub_rn((float)iy0, ce.y.kq);
#pragma unroll
    for (int i = 0; i <= PX; i++) ax[i] = xrel(ce.x, __fadd_rn(mx, (float)i), bh, cbx);
#pragma unroll
    for (int j = 0; j <= PY; j++) ay[j] = xrel(ce.y, __fadd_rn(my, (float)j), bh, cby);
}

// One view of the fan gather: adds w_rV * yw_r for every ray of view iv whose
// column window covers the block with lower corner (ix0, iy0).
template <int PX, int PY>
__device__ __forceinline__ void fan_view_gather(float (&acc)[PY][PX], const float* __restrict__ yw,
                                                const ColEntry* __restrict__ col,
                                                const ViewEntry& ve, int iv, const DetGrid& G,
                                                int ix0, int iy0, int nx, int ny, int na)
{
    int lo, hi; float dmin, dmax;
    column_window(G, ve.c, ve.s, (float)(ix0 - nx / 2), (float)(iy0 - ny / 2), (float)PX,
                  (float)PY, na, lo, hi, dmin, dmax);
    const ColEntry* cv = col + (long long)iv * na;
    const float* yv = yw + (long long)iv * na;
    for (int ia = lo; ia <= hi; ia++) {
        if (!FL_IN(ia, na)) continue;
        const ColEntry ce = cv[ia];
        const float yval = __ldg(yv + ia);
        float ax[PX + 1], ay[PY + 1];
        fan_block_crossings<PX, PY>(ce, ix0, iy0, nx, ny, ax, ay);
#pragma unroll
        for (int j = 0; j < PY; j++)
#pragma unroll
            for (int i = 0; i < PX; i++) {
                const float l = fmaxf(fminf(ax[i], ax[i + 1]), fminf(ay[j], ay[j + 1]));
                const float h = fminf(fmaxf(ax[i], ax[i + 1]), fmaxf(ay[j], ay[j + 1]));
                const float w = h - l;
                if (w > 0.0f) acc[j][i] = fmaf(w, yval, acc[j][i]);
            }
    }
}

// View group g alone (one thread per group; fan_combine_groups adds them).
template <int PX, int PY>
__device__ __forceinline__ void fan_block_gather(float (&acc)[PY][PX],
                                                 const float* __restrict__ yw,
                                                 const ColEntry* __restrict__ col,
                                                 const ViewEntry* __restrict__ view,
                                                 const int* __restrict__ views, int nvf,
                                                 const DetGrid& G, int ix0, int iy0, int nx,
                                                 int ny, int na, int g)
{
#pragma unroll
    for (int j = 0; j < PY; j++)
#pragma unroll
        for (int i = 0; i < PX; i++) acc[j][i] = 0.0f;
    for (int jv = g; jv < nvf; jv += kFanGroups) {
        const int iv = views[jv];
        fan_view_gather<PX, PY>(acc, yw, col, view[iv], iv, G, ix0, iy0, nx, ny, na);
    }
}

// Every view group in one thread: the views in order, each into its group's
// own sums (register sets rotated once per view), then
// ((S_0 + S_1) + S_2) + S_3 -- the same bits as one thread per group and
// fan_combine_groups, without the extra threads (for launches that fill the
// GPU anyway).
template <int PX, int PY>
__device__ __forceinline__ void fan_block_gather_all(float (&acc)[PY][PX],
                                                     const float* __restrict__ yw,
                                                     const ColEntry* __restrict__ col,
                                                     const ViewEntry* __restrict__ view,
                                                     const int* __restrict__ views, int nvf,
                                                     const DetGrid& G, int ix0, int iy0, int nx,
                                                     int ny, int na)
{
    // part[0] always holds the group of the next view: after each view the
    // groups rotate one place, and after the loop back into group order
    float part[kFanGroups][PY][PX];
#pragma unroll
    for (int g = 0; g < kFanGroups; g++)
#pragma unroll
        for (int j = 0; j < PY; j++)
#pragma unroll
            for (int i = 0; i < PX; i++) part[g][j][i] = 0.0f;
    auto rotate = [&]() {
#pragma unroll
        for (int j = 0; j < PY; j++)
#pragma unroll
            for (int i = 0; i < PX; i++) {
                const float t = part[0][j][i];
#pragma unroll
                for (int g = 0; g < kFanGroups - 1; g++) part[g][j][i] = part[g + 1][j][i];
                part[kFanGroups - 1][j][i] = t;
            }
    };
    for (int jv = 0; jv < nvf; jv++) {
        const int iv = views[jv];
        fan_view_gather<PX, PY>(part[0], yw, col, view[iv], iv, G, ix0, iy0, nx, ny, na);
        rotate();
    }
    for (int k = (kFanGroups - nvf % kFanGroups) % kFanGroups; k > 0; k--) rotate();
#pragma unroll
    for (int j = 0; j < PY; j++)
#pragma unroll
        for (int i = 0; i < PX; i++) {
            float s = part[0][j][i];
#pragma unroll
            for (int g = 1; g < kFanGroups; g++) s += part[g][j][i];
            acc[j][i] = s;
        }
}

// Pixel p0 = (ix, iy) of a fan turn plan and its turns p_k = R^k p0
// (walk_fan's R).
template <int G>
__device__ __forceinline__ void fan_turn_pixels(int ix, int iy, int nx, int ny, int (&px)[G],
                                                int (&py)[G])
{
    px[0] = ix; py[0] = iy;
    if (G == 2) {
        px[1] = nx - 1 - ix; py[1] = ny - 1 - iy;
    } else {
        px[1] = nx - 1 - iy; py[1] = ix;
        px[2] = nx - 1 - ix; py[2] = nx - 1 - iy;
        px[3] = iy;          py[3] = nx - 1 - ix;
    }
}

// View groups of the fan turn and reflection backprojections: 8 in batches
// and by default; a plan may take 16 (FL_TUNE_FAN_GROUPS), which changes the
// order of a pixel's additions.
constexpr int kTurnGroups = 8;

// Turn k of a P x P block of primary pixels with lower corner (ix0, iy0):
// R^k maps the block onto the P x P block with lower corner (X0, Y0) (the
// turns of walk_fan's R), and primary pixel (ix0 + i, iy0 + j) onto that
// block's pixel (X0 + a, Y0 + b). turn_local gives (i, j) for (a, b).
template <int G, int P>
__device__ __forceinline__ void turn_corner(int k, int ix0, int iy0, int nx, int ny, int& X0,
                                            int& Y0)
{
    if (k == 0) { X0 = ix0; Y0 = iy0; }
    else if (G == 2 || k == 2) { X0 = nx - ix0 - P; Y0 = ny - iy0 - P; }
    else if (k == 1) { X0 = nx - iy0 - P; Y0 = ix0; }
    else { X0 = iy0; Y0 = nx - ix0 - P; }
}

template <int G, int P>
__host__ __device__ constexpr int turn_local_i(int k, int a, int b)
{
    return k == 0 ? a : (G == 2 || k == 2) ? P - 1 - a : k == 1 ? b : P - 1 - b;
}

template <int G, int P>
__host__ __device__ constexpr int turn_local_j(int k, int a, int b)
{
    return k == 0 ? b : (G == 2 || k == 2) ? P - 1 - b : k == 1 ? P - 1 - a : a;
}

// Fan adjoint of a turn plan (G = 2 or 4, one frame): the P x P block of
// primary pixels at (ix0, iy0) and its turns, over the views iv = g, g + NG,
// ... < nv/G of view group g. In view iv the weight of a turned pixel R^k p
// and ray (iv, ia), from the same crossing table as the walk, multiplies the
// value of ray (iv + j nv/G, ia) into R^{k+j mod G} p: A[(iv + j nv/G, a),
// R^j p] = A[(iv, a), p]. acc[m][j][i] collects turn m of primary pixel
// (ix0 + i, iy0 + j). ywp is the packed sinogram (G values per
// (iv < nv/G, ia)). A pixel's sum runs over the group's views in order, per
// view over k = 0, 1, ... and the columns in increasing order; only rays
// with w > 0 add to it. The turned block's column window contains each of
// its pixels' own windows (0.02 columns of slack against the FP32 error of
// w), so the sums do not depend on P.
template <int G, int P>
__device__ __forceinline__ void fan_turn_gather(float (&acc)[G][P][P],
                                                const float* __restrict__ ywp,
                                                const ColEntry* __restrict__ col,
                                                const ViewEntry* __restrict__ view,
                                                const DetGrid& D, int ix0, int iy0, int nx,
                                                int ny, int na, int nv, int g, int NG)
{
    int X0[G], Y0[G];
#pragma unroll
    for (int k = 0; k < G; k++) turn_corner<G, P>(k, ix0, iy0, nx, ny, X0[k], Y0[k]);
    const int gv = nv / G;
    for (int iv = g; iv < gv; iv += NG) {
        const ViewEntry ve = view[iv];
        const ColEntry* cv = col + (long long)iv * na;
        const float* yv = ywp + (long long)G * iv * na;
#pragma unroll
        for (int k = 0; k < G; k++) {
            int lo, hi; float dmin, dmax;
            column_window(D, ve.c, ve.s, (float)(X0[k] - nx / 2), (float)(Y0[k] - ny / 2),
                          (float)P, (float)P, na, lo, hi, dmin, dmax);
            for (int ia = lo; ia <= hi; ia++) {
                if (!FL_IN(ia, na)) continue;
                const ColEntry ce = cv[ia];
                float ax[P + 1], ay[P + 1];
                fan_block_crossings<P, P>(ce, X0[k], Y0[k], nx, ny, ax, ay);
                float t[G];
                if constexpr (G == 4) {
                    const float4 u = __ldg(reinterpret_cast<const float4*>(yv + 4 * ia));
                    t[0] = u.x; t[1] = u.y; t[2] = u.z; t[3] = u.w;
                } else {
                    const float2 u = __ldg(reinterpret_cast<const float2*>(yv + 2 * ia));
                    t[0] = u.x; t[1] = u.y;
                }
#pragma unroll
                for (int b = 0; b < P; b++)
#pragma unroll
                    for (int a = 0; a < P; a++) {
                        const float l = fmaxf(fminf(ax[a], ax[a + 1]), fminf(ay[b], ay[b + 1]));
                        const float h = fminf(fmaxf(ax[a], ax[a + 1]), fmaxf(ay[b], ay[b + 1]));
                        const float w = h - l;
                        if (!(w > 0.0f)) continue;
                        const int i = turn_local_i<G, P>(k, a, b), j = turn_local_j<G, P>(k, a, b);
#pragma unroll
                        for (int m = 0; m < G; m++)
                            acc[(k + m) % G][j][i] = fmaf(w, t[m], acc[(k + m) % G][j][i]);
                    }
            }
        }
    }
}

// Pixels per block row of the grouped fan backprojections.
constexpr int kFanX = 32;
// Parts per ray of the fan turn forward: kFanLanes for scans with fewer
// than kFanSplitWalks walks (nv/G views x na columns), else 1. A function of
// the scan alone, so a plan and a batch holding it choose alike.
constexpr int kFanLanes = 16;
constexpr long long kFanSplitWalks = 1LL << 16;
constexpr int kFanBlock = 256;       // threads per block of the fan turn forward

__host__ __device__ inline int fan_turn_lanes(long long walks)
{
    return walks < kFanSplitWalks ? kFanLanes : 1;
}

// One block of kFanBlock threads of the fan turn forward (G = 2 or 4, one
// frame; XT the transposed image, walk_fan): L (1, 4 or 16, uniform in the
// launch) threads per ray (iv < nv/G, ia), each walking one part of it
// (walk_fan), their sums added in part order; the walk also yields the rays
// of views iv + j nv/G at the same column, all with the walked ray's c_r.
// The block holds the rays r0, r0 + 1, ... : with L parts, kFanBlock / L
// rays, part k in warp(s) k, so a warp's gathers follow neighbouring rays.
// Small fan launches have few rays: the parts give the GPU L times the
// threads, each with that fraction of the walk. ypack writes the
// adjoint-input layout of these plans: the G values of ray (iv, ia)'s orbit
// side by side at G (iv na + ia) + j. Every thread of the block must call it
// (it synchronises the block).
template <typename TX, typename TY, int G>
__device__ __forceinline__ void fan_turn_forward_block(const TX* __restrict__ X,
                                                       const TX* __restrict__ XT,
                                                       TY* __restrict__ y,
                                                       const ColEntry* __restrict__ col,
                                                       const float* __restrict__ colr, int nx,
                                                       int ny, int na, int nv, float scale,
                                                       int cr_power,
                                                       const float* __restrict__ xscale,
                                                       int ypack, long long r0, int L)
{
    const int nry = kFanBlock / L;             // rays per block
    const int gv = nv / G;
    const int tx = threadIdx.x % nry, lane = threadIdx.x / nry;
    const long long r = r0 + tx;
    const bool ray = r < (long long)na * gv;
    float acc[G];
#pragma unroll
    for (int j = 0; j < G; j++) acc[j] = 0.0f;
    if (ray)
        walk_fan_parts<TX, G, false>(X, XT, &col[r].x, &col[r].y, nx, ny, acc,
                                     (long long)nx * ny, lane, L);
    if (L > 1) {
        // part k of ray tx is thread k nry + tx: the first nry threads add them in order
        __shared__ float part[G][kFanBlock];
#pragma unroll
        for (int j = 0; j < G; j++) part[j][threadIdx.x] = acc[j];
        __syncthreads();
        if (lane != 0) return;
#pragma unroll
        for (int j = 0; j < G; j++) {
            float sum = part[j][tx];
            for (int k = 1; k < L; k++) sum += part[j][k * nry + tx];
            acc[j] = sum;
        }
    }
    if (!ray) return;
    const int iv = (int)(r / na), ia = (int)(r - (long long)iv * na);
    const float cr = ray_cr(scale, colr[r], 0.0f);
    float o[G];
#pragma unroll
    for (int j = 0; j < G; j++) {
        float a = acc[j];
        if (xscale) a *= *xscale;
        o[j] = cr * a;
        if (cr_power == 2) o[j] = cr * o[j];
    }
    if (ypack) {
#pragma unroll
        for (int j = 0; j < G; j += 2) Store<TY>::st2(y + G * r + j, o[j], o[j + 1]);
    } else {
#pragma unroll
        for (int j = 0; j < G; j++)
            Store<TY>::st(y + ((long long)iv + (long long)j * gv) * na + ia, o[j]);
    }
}

// One block of the fan turn backprojection (G = 2 or 4, one frame): thread
// (x, g) of a block of kFanX x kTurnGroups threads takes the P x P block of
// primary pixels at (ix0 + P x, iy0) -- G = 2: rows y < ny/2; G = 4: x, y <
// n/2 -- with its turns, over view group g of the views iv < nv/G
// (fan_turn_gather). The groups' sums meet in shared memory and are added in
// the order g = 0, 1, ...; group 0 stores the pixels. Every thread of the
// block must call it (it synchronises the block).
template <typename TX, int G, int P, int NG = kTurnGroups>
__device__ __forceinline__ void fan_turn_adjoint_block(TX* __restrict__ X,
                                                       const float* __restrict__ ywp,
                                                       const ColEntry* __restrict__ col,
                                                       const ViewEntry* __restrict__ view,
                                                       const DetGrid& D, int nx, int ny, int na,
                                                       int nv, int ix0, int iy0)
{
    const int hx = G == 2 ? nx : nx / 2, hy = ny / 2;
    const int tx = threadIdx.x, g = threadIdx.y, bx = ix0 + P * tx;
    float acc[G][P][P];
#pragma unroll
    for (int m = 0; m < G; m++)
#pragma unroll
        for (int j = 0; j < P; j++)
#pragma unroll
            for (int i = 0; i < P; i++) acc[m][j][i] = 0.0f;
    if (bx < hx)
        fan_turn_gather<G, P>(acc, ywp, col, view, D, bx, iy0, nx, ny, na, nv, g, NG);
    __shared__ float part[NG][G * P * P][kFanX];
#pragma unroll
    for (int m = 0; m < G; m++)
#pragma unroll
        for (int j = 0; j < P; j++)
#pragma unroll
            for (int i = 0; i < P; i++) part[g][(m * P + j) * P + i][tx] = acc[m][j][i];
    __syncthreads();
    if (g != 0) return;
#pragma unroll
    for (int j = 0; j < P; j++)
#pragma unroll
        for (int i = 0; i < P; i++) {
            if (bx + i >= hx || iy0 + j >= hy) continue;      // not a primary pixel
            int px[G], py[G];
            fan_turn_pixels<G>(bx + i, iy0 + j, nx, ny, px, py);
#pragma unroll
            for (int m = 0; m < G; m++) {
                float sum = part[0][(m * P + j) * P + i][tx];
#pragma unroll
                for (int k = 1; k < NG; k++) sum += part[k][(m * P + j) * P + i][tx];
                Store<TX>::st(X + (long long)py[m] * nx + px[m], sum);
            }
        }
}

// One block of kFanBlock threads of a fan reflection form's forward (NR = 1,
// 2 or 4; FanReflGeom; XT the transposed image, walk_fan): L (1, 4 or 16, uniform in the launch) threads per
// walked ray r = (slot, column) of the r0, r0 + 1, ... (kFanBlock / L
// rays), each walking one part of it (walk_fan with the reflected images),
// their sums added in part order. The walk yields the rays of the 2 NR images
// (refl_image) of the walked ray, all with its c_r. ypack writes the packed
// input of the backprojection (the 2 NR values at off + 2 NR ia of
// refl_slot). Every thread of the block must call it (it synchronises the
// block).
template <typename TX, typename TY, int NR>
__device__ __forceinline__ void fan_refl_forward_block(const TX* __restrict__ X,
                                                       const TX* __restrict__ XT,
                                                       TY* __restrict__ y,
                                                       const ColEntry* __restrict__ col,
                                                       const float* __restrict__ colr, int nx,
                                                       int ny, int na, int nv, float scale,
                                                       int cr_power,
                                                       const float* __restrict__ xscale,
                                                       int ypack, long long r0, int L)
{
    constexpr int NI = 2 * NR;
    const int nry = kFanBlock / L;             // rays per block
    const FanReflGeom g = fan_refl_geom(NR, nv, na);
    const int tx = threadIdx.x % nry, lane = threadIdx.x / nry;
    const long long r = r0 + tx;
    int v = 0, vt = 0, a = 0, stride = 0;
    long long off = 0;
    const int sl = (int)(r / na), ia = (int)(r - (long long)sl * na);
    const bool ray = r < (long long)g.slots * na && refl_slot(g, sl, ia, v, vt, a, off, stride);
    float acc[NI];
#pragma unroll
    for (int j = 0; j < NI; j++) acc[j] = 0.0f;
    const long long rr = (long long)vt * na + a;      // the walked ray's table entry
    if (ray) walk_fan_parts<TX, NR, true>(X, XT, &col[rr].x, &col[rr].y, nx, ny, acc,
                                          (long long)nx * ny, lane, L);
    if (L > 1) {
        // part k of ray tx is thread k nry + tx: the first nry threads add them in order
        __shared__ float part[NI][kFanBlock];
#pragma unroll
        for (int j = 0; j < NI; j++) part[j][threadIdx.x] = acc[j];
        __syncthreads();
        if (lane != 0) return;
#pragma unroll
        for (int j = 0; j < NI; j++) {
            float sum = part[j][tx];
            for (int k = 1; k < L; k++) sum += part[j][k * nry + tx];
            acc[j] = sum;
        }
    }
    if (!ray) return;
    const float cr = ray_cr(scale, colr[rr], 0.0f);
    float o[NI];
#pragma unroll
    for (int j = 0; j < NI; j++) {
        float t = acc[j];
        if (xscale) t *= *xscale;
        o[j] = cr * t;
        if (cr_power == 2) o[j] = cr * o[j];
    }
    if (ypack) {
#pragma unroll
        for (int j = 0; j < NI; j += 2) Store<TY>::st2(y + off + (long long)NI * ia + j, o[j], o[j + 1]);
    } else {
#pragma unroll
        for (int k = 0; k < NI; k++) {
            long long vk; int ak;
            refl_image<NR>(k, v, a, na, nv, vk, ak);
            Store<TY>::st(y + vk * na + ak, o[k]);
        }
    }
}

// Primary pixels of a fan reflection form (NR = 4: the octant x <= y < n/2;
// 2: the quadrant x < nx/2, y < ny/2; 1: the rows y < ny/2) and their images
// C_k = S^k p, D_k = S^k M p (k < NR), as (x, y).
template <int NR>
__host__ __device__ inline bool fan_refl_primary(int ix, int iy, int nx, int ny)
{
    if (NR == 4) return ix <= iy && iy < ny / 2;
    if (NR == 2) return ix < nx / 2 && iy < ny / 2;
    return ix < nx && iy < ny / 2;
}

template <int NR>
__device__ __forceinline__ void fan_refl_images(int ix, int iy, int nx, int ny, int (&cx)[NR],
                                                int (&cy)[NR], int (&dx)[NR], int (&dy)[NR])
{
    if (NR == 4) {
        cx[0] = ix; cx[1 % NR] = nx - 1 - iy; cx[2 % NR] = nx - 1 - ix; cx[3 % NR] = iy;
        cy[0] = iy; cy[1 % NR] = ix; cy[2 % NR] = ny - 1 - iy; cy[3 % NR] = ny - 1 - ix;
        dx[0] = ix; dx[1 % NR] = iy; dx[2 % NR] = nx - 1 - ix; dx[3 % NR] = nx - 1 - iy;
        dy[0] = ny - 1 - iy; dy[1 % NR] = ix; dy[2 % NR] = iy; dy[3 % NR] = ny - 1 - ix;
    } else if (NR == 2) {
        cx[0] = ix; cx[1 % NR] = nx - 1 - ix; cy[0] = iy; cy[1 % NR] = ny - 1 - iy;
        dx[0] = ix; dx[1 % NR] = nx - 1 - ix; dy[0] = ny - 1 - iy; dy[1 % NR] = iy;
    } else {
        cx[0] = ix; cy[0] = iy; dx[0] = ix; dy[0] = ny - 1 - iy;
    }
}

// Pixel block of a fan reflection backprojection: PB x PB (1, or 2 where the
// primary domain tiles into 2 x 2 blocks: NR = 4, n a multiple of 4; NR = 2,
// nx and ny multiples of 4; NR = 1, nx even and ny a multiple of 4). A
// function of the geometry alone, so a plan and a batch holding it choose
// alike.
__host__ __device__ inline int fan_refl_pblock(int NR, int nx, int ny)
{
    if (NR == 4) return nx % 4 == 0 ? 2 : 1;
    if (NR == 2) return (nx % 4 == 0 && ny % 4 == 0) ? 2 : 1;
    return (nx % 2 == 0 && ny % 4 == 0) ? 2 : 1;
}

// Fan reflection backprojection of the primary PB x PB block with lower corner
// (X0, Y0) over the walked views w = g, g + NG, ... <= ov (FanReflGeom). The
// thread visits the block's images C_0 .. C_{NR-1} (S^k of the block) and
// D_0 .. D_{NR-1} (S^k M of it) in one rolled loop. In view w a weight of a
// pixel of C_k (from the same crossing table as the walk) multiplies turn
// slot j (view w + j q) into C_{k+j} and reflected slot j (view j q - w,
// column na-1-a) into D_{j-k}; a weight of a pixel of D_k, turn slot j into
// D_{k+j} and reflected slot j into C_{j-k}. P holds the turn slots' sums, Q
// the reflected ones', rotated one place per block image in opposite
// directions and exchanged between the C and the D images; their pixel index
// follows the image block's own pixel order (re-indexed by S and M at each
// step), so at the end P[j][b][a] is C_j's sum and Q[j][b][a] D_j's for the
// primary pixel (X0 + a, Y0 + b). On the diagonal blocks of NR = 4 (X0 ==
// Y0) D_k = C_{k+3} T with T the transpose within the block: only the C_k
// are visited, and C_j of pixel p sums P[j][p] + Q[(j+1) % NR][T p]. Per
// pixel the sums run over the group's views in order, per view over the
// images in order and the columns in increasing order; only rays with w > 0
// add (the block's column window contains each pixel's own).
template <int NR, int PB>
__device__ __forceinline__ void fan_refl_gather(float (&P)[NR][PB][PB], float (&Q)[NR][PB][PB],
                                                const float* __restrict__ ywp,
                                                const ColEntry* __restrict__ col,
                                                const ViewEntry* __restrict__ view,
                                                const DetGrid& D, int X0, int Y0, int nx, int ny,
                                                int na, int nv, int g, int NG)
{
    const FanReflGeom geo = fan_refl_geom(NR, nv, na);
    const bool diag = NR == 4 && X0 == Y0;
    const int nsteps = diag ? NR : 2 * NR;
    // re-index the pixel dimension of P and Q: T[b][a] <- T[f(b, a)]
    auto turn_px = [&](float (&A)[NR][PB][PB]) {          // the block turned by S
        if (PB == 1 || NR == 1) return;
#pragma unroll
        for (int j = 0; j < NR; j++) {
            float o[PB][PB];
#pragma unroll
            for (int b = 0; b < PB; b++)
#pragma unroll
                for (int a = 0; a < PB; a++) o[b][a] = A[j][b][a];
#pragma unroll
            for (int b = 0; b < PB; b++)
#pragma unroll
                for (int a = 0; a < PB; a++)
                    // R: new (a, b) holds old (b, PB-1-a); R^2: old (PB-1-a, PB-1-b)
                    A[j][b][a] = NR == 4 ? o[PB - 1 - a][b] : o[PB - 1 - b][PB - 1 - a];
        }
    };
    auto mirror_px = [&](float (&A)[NR][PB][PB]) {        // M: (a, b) <- (a, PB-1-b)
        if (PB == 1) return;
#pragma unroll
        for (int j = 0; j < NR; j++)
#pragma unroll
            for (int a = 0; a < PB; a++) {
                const float t = A[j][0][a]; A[j][0][a] = A[j][PB - 1][a]; A[j][PB - 1][a] = t;
            }
    };
    for (int w = g; w <= geo.ov; w += NG) {
        int vt, rs, alim;
        long long base;
        refl_view(geo, w, vt, base, rs, alim);
        const ViewEntry ve = view[vt];
        const ColEntry* cv = col + (long long)vt * na;
        const float* yv = ywp + base;
        int bx = X0, by = Y0;                          // C_0
#pragma unroll 1
        for (int k = 0; k < nsteps; k++) {
            if (k == NR) {                             // the D images: D_0 = M block
                bx = X0; by = ny - Y0 - PB;
#pragma unroll
                for (int j = 0; j < NR; j++)
#pragma unroll
                    for (int b = 0; b < PB; b++)
#pragma unroll
                        for (int a = 0; a < PB; a++) {
                            const float t = P[j][b][a]; P[j][b][a] = Q[j][b][a]; Q[j][b][a] = t;
                        }
                mirror_px(P);
                mirror_px(Q);
            }
            int lo, hi; float dmin, dmax;
            column_window(D, ve.c, ve.s, (float)(bx - nx / 2), (float)(by - ny / 2), (float)PB,
                          (float)PB, na, lo, hi, dmin, dmax);
            hi = min(hi, alim - 1);
            for (int ia = lo; ia <= hi; ia++) {
                if (!FL_IN(ia, na)) continue;
                const ColEntry ce = cv[ia];
                float ax[PB + 1], ay[PB + 1];
                fan_block_crossings<PB, PB>(ce, bx, by, nx, ny, ax, ay);
                float t[2 * NR];
                const float* yo = yv + (long long)(2 * NR) * ia;
                if constexpr (NR == 4) {
                    const float4 u0 = __ldg(reinterpret_cast<const float4*>(yo));
                    const float4 u1 = __ldg(reinterpret_cast<const float4*>(yo) + 1);
                    t[0] = u0.x; t[1] = u0.y; t[2] = u0.z; t[3] = u0.w;
                    t[4] = u1.x; t[5] = u1.y; t[6] = u1.z; t[7] = u1.w;
                } else if constexpr (NR == 2) {
                    const float4 u = __ldg(reinterpret_cast<const float4*>(yo));
                    t[0] = u.x; t[1] = u.y; t[2] = u.z; t[3] = u.w;
                } else {
                    const float2 u = __ldg(reinterpret_cast<const float2*>(yo));
                    t[0] = u.x; t[1] = u.y;
                }
#pragma unroll
                for (int b = 0; b < PB; b++)
#pragma unroll
                    for (int a = 0; a < PB; a++) {
                        const float l = fmaxf(fminf(ax[a], ax[a + 1]), fminf(ay[b], ay[b + 1]));
                        const float h = fminf(fmaxf(ax[a], ax[a + 1]), fmaxf(ay[b], ay[b + 1]));
                        const float wt = h - l;
                        if (!(wt > 0.0f)) continue;
#pragma unroll
                        for (int j = 0; j < NR; j++) {
                            P[j][b][a] = fmaf(wt, t[j], P[j][b][a]);
                            Q[j][b][a] = fmaf(wt, t[NR + j], Q[j][b][a]);
                        }
                    }
            }
            // next image S (block); P rotates back one place, Q forward one;
            // the pixel index follows the turned block
            if (NR == 4) {
                const int tt = bx;
                bx = nx - by - PB; by = tt;
            } else if (NR == 2) {
                bx = nx - bx - PB; by = ny - by - PB;
            }
            if (NR > 1) {
#pragma unroll
                for (int b = 0; b < PB; b++)
#pragma unroll
                    for (int a = 0; a < PB; a++) {
                        const float a0 = P[0][b][a];
#pragma unroll
                        for (int j = 0; j + 1 < NR; j++) P[j][b][a] = P[j + 1][b][a];
                        P[NR - 1][b][a] = a0;
                        const float b0 = Q[NR - 1][b][a];
#pragma unroll
                        for (int j = NR - 1; j > 0; j--) Q[j][b][a] = Q[j - 1][b][a];
                        Q[0][b][a] = b0;
                    }
                turn_px(P);
                turn_px(Q);
            }
        }
        if (!diag) {                                   // back to the C order
            mirror_px(P);
            mirror_px(Q);
#pragma unroll
            for (int j = 0; j < NR; j++)
#pragma unroll
                for (int b = 0; b < PB; b++)
#pragma unroll
                    for (int a = 0; a < PB; a++) {
                        const float t = P[j][b][a]; P[j][b][a] = Q[j][b][a]; Q[j][b][a] = t;
                    }
        }
    }
}

// Shared floats fan_refl_adjoint_block needs (the largest form: NR = 4,
// 2 x 2 blocks).
constexpr int kFanReflShared = kTurnGroups * 2 * 4 * 4 * kFanX;

// One block of a fan reflection backprojection: thread (x, g) of a block of
// kFanX x kTurnGroups threads takes the PB x PB block of primary pixels with
// lower corner (PB (bx0 + x), PB by) where it is a primary block (in block
// units: x < the domain's width; NR = 4: x <= by) over view group g of the
// walked views (fan_refl_gather). The groups' sums meet in shared memory
// (smem: NG 2 NR PB^2 kFanX floats) and are added in the order g = 0, 1, ...;
// group 0 stores the images. Every thread of the block must call it (it
// synchronises the block).
template <typename TX, int NR, int PB, int NG = kTurnGroups>
__device__ __forceinline__ void fan_refl_adjoint_block(TX* __restrict__ X,
                                                       const float* __restrict__ ywp,
                                                       const ColEntry* __restrict__ col,
                                                       const ViewEntry* __restrict__ view,
                                                       const DetGrid& D, int nx, int ny, int na,
                                                       int nv, int bx0, int by, float* smem)
{
    constexpr int NV = NR * PB * PB;
    const int tx = threadIdx.x, g = threadIdx.y, bx = bx0 + tx;
    const int hxb = (NR == 1 ? nx : nx / 2) / PB, hyb = (ny / 2) / PB;
    const bool prim = bx < hxb && by < hyb && (NR != 4 || bx <= by);
    const int X0 = PB * bx, Y0 = PB * by;
    float P[NR][PB][PB], Q[NR][PB][PB];
#pragma unroll
    for (int j = 0; j < NR; j++)
#pragma unroll
        for (int b = 0; b < PB; b++)
#pragma unroll
            for (int a = 0; a < PB; a++) { P[j][b][a] = 0.0f; Q[j][b][a] = 0.0f; }
    if (prim)
        fan_refl_gather<NR, PB>(P, Q, ywp, col, view, D, X0, Y0, nx, ny, na, nv, g, NG);
    float(*part)[2 * NV][kFanX] = reinterpret_cast<float(*)[2 * NV][kFanX]>(smem);
#pragma unroll
    for (int j = 0; j < NR; j++)
#pragma unroll
        for (int b = 0; b < PB; b++)
#pragma unroll
            for (int a = 0; a < PB; a++) {
                part[g][(j * PB + b) * PB + a][tx] = P[j][b][a];
                part[g][NV + (j * PB + b) * PB + a][tx] = Q[j][b][a];
            }
    __syncthreads();
    if (g != 0 || !prim) return;
    auto sum = [&](int k) {
        float t = part[0][k][tx];
#pragma unroll
        for (int m = 1; m < NG; m++) t += part[m][k][tx];
        return t;
    };
    const bool diag = NR == 4 && X0 == Y0;
#pragma unroll
    for (int b = 0; b < PB; b++)
#pragma unroll
        for (int a = 0; a < PB; a++) {
            int cx[NR], cy[NR], dx[NR], dy[NR];
            fan_refl_images<NR>(X0 + a, Y0 + b, nx, ny, cx, cy, dx, dy);
#pragma unroll
            for (int j = 0; j < NR; j++) {
                float c = sum((j * PB + b) * PB + a);
                if (diag) c += sum(NV + (((j + 1) % NR) * PB + a) * PB + b);   // Q[j+1][T p]
                Store<TX>::st(X + (long long)cy[j] * nx + cx[j], c);
                if (!diag) Store<TX>::st(X + (long long)dy[j] * nx + dx[j], sum(NV + (j * PB + b) * PB + a));
            }
        }
}

// The kFanGroups view groups of a pixel block are the threads (x, g) of a
// block of NX x kFanGroups threads; their sums meet in shared memory and
// group 0 returns true holding ((S_0 + S_1) + S_2) + S_3. Every thread of the
// block must call it (it synchronises the block).
template <int P, int NX>
__device__ __forceinline__ bool fan_combine_groups(float (&acc)[P][P])
{
    __shared__ float part[kFanGroups][P * P][NX];
    const int tx = threadIdx.x, g = threadIdx.y;
#pragma unroll
    for (int j = 0; j < P; j++)
#pragma unroll
        for (int i = 0; i < P; i++) part[g][j * P + i][tx] = acc[j][i];
    __syncthreads();
    if (g != 0) return false;
#pragma unroll
    for (int j = 0; j < P; j++)
#pragma unroll
        for (int i = 0; i < P; i++) {
            float s = part[0][j * P + i][tx];
#pragma unroll
            for (int k = 1; k < kFanGroups; k++) s += part[k][j * P + i][tx];
            acc[j][i] = s;
        }
    return true;
}

}  // namespace
