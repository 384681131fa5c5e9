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

// Slab index of the ray at parameter a on one axis, consistent with the FP32
// crossings: inv > 0 -> A(j) <= a < A(j+1); inv < 0 -> A(j+1) <= a < A(j).
__device__ __forceinline__ int start_slab(float a, float inv, float off, int n)
{
    float t = floorf(__fdividef(a - off, inv));
    t = fminf(fmaxf(t, 0.0f), (float)(n - 1));   // NaN -> 0
    int j = (int)t;
    if (inv > 0.0f) {
        while (j < n - 1 && fmaf((float)(j + 1), inv, off) <= a) j++;
        while (j > 0 && fmaf((float)j, inv, off) > a) j--;
    } else {
        while (j > 0 && fmaf((float)j, inv, off) <= a) j--;
        while (j < n - 1 && fmaf((float)(j + 1), inv, off) > a) j++;
    }
    return j;
}

// Walk one ray through an nx*ny*nz volume (nz == 1 with no z axis for 2-D).
// Returns sum over voxels of w * x; *nseg counts segments with w > 0.
// Termination: every step advances at least one axis to a strictly larger
// crossing (consecutive FP32 crossings of one axis are thousands of ulps
// apart for any table fl_plan_create accepts), and the loop leaves as soon as
// the crossing reaches the exit (or is NaN); the step budget nx+ny+nz+4 is a
// second, independent bound.
// MIRROR: x is the z-folded volume (pairs of voxel (ix, iy, iz < nz/2) and its
// mirror (ix, iy, nz-1-iz), fl_plan.h); the ray must descend from the source
// plane, so it stays in iz < nz/2. Every step gathers the pair: the voxel's
// value goes to the return value and the mirror's, with the same segment
// length, to *accm -- the companion ray of a scan symmetric about the source
// plane (fl_plan::zmirror).
// xlen: elements available at x (checked builds verify every gather index).
template <typename TX, bool THREE, bool COUNT, bool MIRROR = false>
__device__ __forceinline__ float walk(const TX* __restrict__ x, float inv_x, float off_x,
                                      float inv_y, float off_y, float inv_z, float off_z,
                                      int nx, int ny, int nz, int* nseg, float* accm = nullptr,
                                      long long xlen = 0)
{
    float ax0 = fmaf(0.0f, inv_x, off_x), ax1 = fmaf((float)nx, inv_x, off_x);
    float ay0 = fmaf(0.0f, inv_y, off_y), ay1 = fmaf((float)ny, inv_y, off_y);
    float a_in = fmaxf(fminf(ax0, ax1), fminf(ay0, ay1));
    float a_out = fminf(fmaxf(ax0, ax1), fmaxf(ay0, ay1));
    if (THREE) {
        float az0 = fmaf(0.0f, inv_z, off_z), az1 = fmaf((float)nz, inv_z, off_z);
        a_in = fmaxf(a_in, fminf(az0, az1));
        a_out = fminf(a_out, fmaxf(az0, az1));
    }
    if (!(a_in < a_out)) {
        if (COUNT) *nseg = 0;
        if (MIRROR) *accm = 0.0f;
        return 0.0f;
    }
    if (MIRROR && !(inv_z < 0.0f)) {               // not a descending ray: no walk
        *accm = 0.0f;
        return 0.0f;
    }
    const int jx = start_slab(a_in, inv_x, off_x, nx);
    const int jy = start_slab(a_in, inv_y, off_y, ny);
    int jz = THREE ? start_slab(a_in, inv_z, off_z, nz) : 0;
    // a descending ray enters below the source plane and only steps down, so
    // the folded index below stays inside the nz/2 stored slices
    if (MIRROR) jz = min(jz, nz / 2 - 1);
    int v = (jz * ny + jy) * nx + jx;              // < 2^31 (checked at plan creation)
    const bool px = inv_x > 0.0f, py = inv_y > 0.0f, pz = inv_z > 0.0f;
    float pax = (float)(px ? jx + 1 : jx);
    float pay = (float)(py ? jy + 1 : jy);
    float paz = (float)(pz ? jz + 1 : jz);
    const float stx = px ? 1.0f : -1.0f, sty = py ? 1.0f : -1.0f, stz = pz ? 1.0f : -1.0f;
    const int dvx = px ? 1 : -1, dvy = py ? nx : -nx, dvz = pz ? nx * ny : -(nx * ny);
    float nAx = fmaf(pax, inv_x, off_x);
    float nAy = fmaf(pay, inv_y, off_y);
    float nAz = THREE ? fmaf(paz, inv_z, off_z) : 3.0e38f;
    float cur = a_in, acc = 0.0f;
    float2 acc2 = make_float2(0.0f, 0.0f);   // MIRROR: (voxel, mirror) sums, paired FMA
    int cnt = 0;
    // the gather of the next voxel is issued as soon as its index is known and
    // consumed one step later, so its latency overlaps the next step's compares
    float xv = 0.0f;
    float2 xv2 = make_float2(0.0f, 0.0f);
    if (MIRROR) { if (FL_IN(2 * (long long)v + 1, xlen)) xv2 = Store<TX>::ld2(x + 2 * (long long)v); }
    else if (!COUNT) { if (FL_IN(v, xlen)) xv = ldv(x + v); }
    const int budget = nx + ny + (THREE ? nz : 0) + 4;
    for (int it = 0; it < budget; it += 4) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float nxt = THREE ? fminf(fminf(nAx, nAy), nAz) : fminf(nAx, nAy);
            const float seg = nxt - cur;
            const bool cont = nxt < a_out;          // false at the exit (and for NaN)
            float xn = 0.0f;
            float2 xn2 = make_float2(0.0f, 0.0f);
            if (cont) {
                if (nAx == nxt) { pax += stx; v += dvx; nAx = fmaf(pax, inv_x, off_x); }
                if (nAy == nxt) { pay += sty; v += dvy; nAy = fmaf(pay, inv_y, off_y); }
                if (THREE && nAz == nxt) { paz += stz; v += dvz; nAz = fmaf(paz, inv_z, off_z); }
                // v is inside the (folded) volume here
                if (MIRROR) { if (FL_IN(2 * (long long)v + 1, xlen)) xn2 = Store<TX>::ld2(x + 2 * (long long)v); }
                else if (!COUNT) { if (FL_IN(v, xlen)) xn = ldv(x + v); }
            }
            if (COUNT) cnt += (seg > 0.0f);
            else if (MIRROR) acc2 = __ffma2_rn(make_float2(seg, seg), xv2, acc2);
            else acc = fmaf(seg, xv, acc);
            if (!cont) goto done;
            xv = xn;
            xv2 = xn2;
            cur = nxt;
        }
    }
done:
    if (COUNT) *nseg = cnt;
    if (MIRROR) { *accm = acc2.y; return acc2.x; }
    return acc;
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
// multiples of 4). *acc gets the (voxel, mirror) sums, *accr the turned
// pair's. Termination as in walk().
template <typename TX>
__device__ __forceinline__ void walk_quad(const TX* __restrict__ x, float inv_x, float off_x,
                                          float inv_y, float off_y, float inv_z, float off_z,
                                          int nx, int ny, int nz, float2* acc, float2* accr,
                                          long long xlen)
{
    *acc = make_float2(0.0f, 0.0f);
    *accr = make_float2(0.0f, 0.0f);
    float ax0 = fmaf(0.0f, inv_x, off_x), ax1 = fmaf((float)nx, inv_x, off_x);
    float ay0 = fmaf(0.0f, inv_y, off_y), ay1 = fmaf((float)ny, inv_y, off_y);
    float a_in = fmaxf(fminf(ax0, ax1), fminf(ay0, ay1));
    float a_out = fminf(fmaxf(ax0, ax1), fmaxf(ay0, ay1));
    float az0 = fmaf(0.0f, inv_z, off_z), az1 = fmaf((float)nz, inv_z, off_z);
    a_in = fmaxf(a_in, fminf(az0, az1));
    a_out = fminf(a_out, fmaxf(az0, az1));
    if (!(a_in < a_out) || !(inv_z < 0.0f)) return;
    const int jx = start_slab(a_in, inv_x, off_x, nx);
    const int jy = start_slab(a_in, inv_y, off_y, ny);
    const int jz = min(start_slab(a_in, inv_z, off_z, nz), nz / 2 - 1);
    const int nxy = nx * ny, nx4 = nx >> 2;
    int cx = jx, cy = jy, zb = jz * nxy;           // < 2^31 (checked at plan creation)
    int v = tiled_pair(cx, cy, zb, nx4), vr = 2 * zb + nxy - 1 - v;
    const bool px = inv_x > 0.0f, py = inv_y > 0.0f;
    float pax = (float)(px ? jx + 1 : jx);
    float pay = (float)(py ? jy + 1 : jy);
    float paz = (float)jz;                         // descending: next plane is jz
    const float stx = px ? 1.0f : -1.0f, sty = py ? 1.0f : -1.0f;
    const int dx = px ? 1 : -1, dy = py ? 1 : -1;
    float nAx = fmaf(pax, inv_x, off_x);
    float nAy = fmaf(pay, inv_y, off_y);
    float nAz = fmaf(paz, inv_z, off_z);
    float cur = a_in;
    float2 s2 = make_float2(0.0f, 0.0f), r2 = make_float2(0.0f, 0.0f);
    float2 xv2 = make_float2(0.0f, 0.0f), xr2 = make_float2(0.0f, 0.0f);
    if (FL_IN(2 * (long long)v + 1, xlen)) xv2 = Store<TX>::ld2(x + 2 * (long long)v);
    if (FL_IN(2 * (long long)vr + 1, xlen)) xr2 = Store<TX>::ld2(x + 2 * (long long)vr);
    const int budget = nx + ny + nz + 4;
    for (int it = 0; it < budget; it += 4) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float nxt = fminf(fminf(nAx, nAy), nAz);
            const float seg = nxt - cur;
            const bool cont = nxt < a_out;         // false at the exit (and for NaN)
            float2 xn2 = make_float2(0.0f, 0.0f), xnr2 = make_float2(0.0f, 0.0f);
            if (cont) {
                if (nAx == nxt) { pax += stx; cx += dx; nAx = fmaf(pax, inv_x, off_x); }
                if (nAy == nxt) { pay += sty; cy += dy; nAy = fmaf(pay, inv_y, off_y); }
                if (nAz == nxt) { paz -= 1.0f; zb -= nxy; nAz = fmaf(paz, inv_z, off_z); }
                v = tiled_pair(cx, cy, zb, nx4);
                vr = 2 * zb + nxy - 1 - v;
                if (FL_IN(2 * (long long)v + 1, xlen)) xn2 = Store<TX>::ld2(x + 2 * (long long)v);
                if (FL_IN(2 * (long long)vr + 1, xlen)) xnr2 = Store<TX>::ld2(x + 2 * (long long)vr);
            }
            s2 = __ffma2_rn(make_float2(seg, seg), xv2, s2);
            r2 = __ffma2_rn(make_float2(seg, seg), xr2, r2);
            if (!cont) goto done;
            xv2 = xn2;
            xr2 = xnr2;
            cur = nxt;
        }
    }
done:
    *acc = s2;
    *accr = r2;
}


// The z-mirror walk with all four quarter turns (plan flag rot4, nx == ny ==
// n, a multiple of 4): per step it gathers the folded pairs of voxel (ix, iy)
// and of its turns R^j (ix, iy), R (x, y) = (n-1-y, x), which the ray of view
// v + j nv/4 at the same column and row crosses with the same segment. x is
// the tiled folded volume. acc[j] gets the (voxel, mirror) sums of turn j.
// Termination as in walk().
template <typename TX>
__device__ __forceinline__ void walk_oct(const TX* __restrict__ x, float inv_x, float off_x,
                                         float inv_y, float off_y, float inv_z, float off_z,
                                         int n, int nz, float2 (&acc)[4], long long xlen)
{
#pragma unroll
    for (int j = 0; j < 4; j++) acc[j] = make_float2(0.0f, 0.0f);
    float ax0 = fmaf(0.0f, inv_x, off_x), ax1 = fmaf((float)n, inv_x, off_x);
    float ay0 = fmaf(0.0f, inv_y, off_y), ay1 = fmaf((float)n, inv_y, off_y);
    float a_in = fmaxf(fminf(ax0, ax1), fminf(ay0, ay1));
    float a_out = fminf(fmaxf(ax0, ax1), fmaxf(ay0, ay1));
    float az0 = fmaf(0.0f, inv_z, off_z), az1 = fmaf((float)nz, inv_z, off_z);
    a_in = fmaxf(a_in, fminf(az0, az1));
    a_out = fminf(a_out, fmaxf(az0, az1));
    if (!(a_in < a_out) || !(inv_z < 0.0f)) return;
    const int jx = start_slab(a_in, inv_x, off_x, n);
    const int jy = start_slab(a_in, inv_y, off_y, n);
    const int jz = min(start_slab(a_in, inv_z, off_z, nz), nz / 2 - 1);
    const int nn = n * n, n4 = n >> 2;
    int cx = jx, cy = jy, zb = jz * nn;            // voxel of turn 0; z base of all turns
    int q[4];                                      // folded pair index of each turn
    auto turns = [&]() {                           // turns 2, 3 are turns 0, 1 by pi
        q[0] = tiled_pair(cx, cy, zb, n4);
        q[1] = tiled_pair(n - 1 - cy, cx, zb, n4);
        q[2] = 2 * zb + nn - 1 - q[0];
        q[3] = 2 * zb + nn - 1 - q[1];
    };
    turns();
    const bool px = inv_x > 0.0f, py = inv_y > 0.0f;
    float pax = (float)(px ? jx + 1 : jx);
    float pay = (float)(py ? jy + 1 : jy);
    float paz = (float)jz;                         // descending: next plane is jz
    const float stx = px ? 1.0f : -1.0f, sty = py ? 1.0f : -1.0f;
    const int dx = px ? 1 : -1, dy = py ? 1 : -1;
    float nAx = fmaf(pax, inv_x, off_x);
    float nAy = fmaf(pay, inv_y, off_y);
    float nAz = fmaf(paz, inv_z, off_z);
    float cur = a_in;
    float2 xv[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        xv[j] = make_float2(0.0f, 0.0f);
        if (FL_IN(2 * (long long)q[j] + 1, xlen)) xv[j] = Store<TX>::ld2(x + 2 * (long long)q[j]);
    }
    float2 s[4];
#pragma unroll
    for (int j = 0; j < 4; j++) s[j] = make_float2(0.0f, 0.0f);
    const int budget = 2 * n + nz + 4;
    for (int it = 0; it < budget; it += 2) {
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const float nxt = fminf(fminf(nAx, nAy), nAz);
            const float seg = nxt - cur;
            const bool cont = nxt < a_out;         // false at the exit (and for NaN)
            float2 xn[4];
#pragma unroll
            for (int j = 0; j < 4; j++) xn[j] = make_float2(0.0f, 0.0f);
            if (cont) {
                if (nAx == nxt) { pax += stx; nAx = fmaf(pax, inv_x, off_x); cx += dx; }
                if (nAy == nxt) { pay += sty; nAy = fmaf(pay, inv_y, off_y); cy += dy; }
                if (nAz == nxt) { paz -= 1.0f; nAz = fmaf(paz, inv_z, off_z); zb -= nn; }
                turns();
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (FL_IN(2 * (long long)q[j] + 1, xlen)) xn[j] = Store<TX>::ld2(x + 2 * (long long)q[j]);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) s[j] = __ffma2_rn(make_float2(seg, seg), xv[j], s[j]);
            if (!cont) goto done;
#pragma unroll
            for (int j = 0; j < 4; j++) xv[j] = xn[j];
            cur = nxt;
        }
    }
done:
#pragma unroll
    for (int j = 0; j < 4; j++) acc[j] = s[j];
}

// The fan walk in batches of kFanBatch steps: the crossings of a batch are
// found first (they do not depend on the image), then its gathers are issued
// together and the segments added in walk order. The sums are the same as
// walk()'s, bit for bit, but a batch waits for its gathers once instead of
// once per step.
// G = 1: the ray's own pixels (acc[0]). G = 2 or 4 (a turn plan, one frame):
// per step also the turns R^j (ix, iy) of the pixel -- G = 2: R (x, y) =
// (nx-1-x, ny-1-y); G = 4 (nx == ny == n): R (x, y) = (n-1-y, x) -- which
// the ray of view v + j nv/G at the same column crosses with the same
// segment; acc[j] gets turn j's sum.
// L > 1: the ray is cut into L parts and this call walks part `lane`. Part k
// runs from crossing c_k to crossing c_{k+1}, where c_k (0 < k < L) is the
// first crossing after a_in + k (a_out - a_in) / L (c_0 = a_in, c_L =
// a_out). Every lane computes the cuts from the same expressions, and a cut
// is a crossing of the ray's own table, so each segment -- each matrix
// entry -- lies whole in one part and is the walk's own; only the order of
// the additions changes (the caller adds the parts in lane order).
// Termination as in walk().
constexpr int kFanBatch = 4;

template <typename TX, int G, int L = 1>
__device__ __forceinline__ void walk_fan(const TX* __restrict__ x, float inv_x, float off_x,
                                         float inv_y, float off_y, int nx, int ny,
                                         float (&acc)[G], long long xlen, int lane = 0)
{
    static_assert(G == 1 || G == 2 || G == 4, "one, two or four turns");
#pragma unroll
    for (int j = 0; j < G; j++) acc[j] = 0.0f;
    float ax0 = fmaf(0.0f, inv_x, off_x), ax1 = fmaf((float)nx, inv_x, off_x);
    float ay0 = fmaf(0.0f, inv_y, off_y), ay1 = fmaf((float)ny, inv_y, off_y);
    const float a_in = fmaxf(fminf(ax0, ax1), fminf(ay0, ay1));
    const float a_out = fminf(fmaxf(ax0, ax1), fmaxf(ay0, ay1));
    if (!(a_in < a_out)) return;
    const bool px = inv_x > 0.0f, py = inv_y > 0.0f;
    // the crossing that ends the slab pair (jx, jy)
    auto next_x = [&](int j) { return fmaf((float)(px ? j + 1 : j), inv_x, off_x); };
    auto next_y = [&](int j) { return fmaf((float)(py ? j + 1 : j), inv_y, off_y); };
    float cur = a_in, end = a_out;
    int jx, jy;
    if (L > 1 && lane > 0) {
        const float t = fmaf((float)lane, (a_out - a_in) * (1.0f / L), a_in);
        jx = start_slab(t, inv_x, off_x, nx);
        jy = start_slab(t, inv_y, off_y, ny);
        const float cx = next_x(jx), cy = next_y(jy), c = fminf(cx, cy);
        if (!(c < a_out)) return;                  // the cut falls at the exit: nothing left
        if (cx == c) jx += px ? 1 : -1;
        if (cy == c) jy += py ? 1 : -1;
        cur = c;
    } else {
        jx = start_slab(a_in, inv_x, off_x, nx);
        jy = start_slab(a_in, inv_y, off_y, ny);
    }
    if (L > 1 && lane + 1 < L) {
        const float t = fmaf((float)(lane + 1), (a_out - a_in) * (1.0f / L), a_in);
        const int ex = start_slab(t, inv_x, off_x, nx), ey = start_slab(t, inv_y, off_y, ny);
        end = fminf(fminf(next_x(ex), next_y(ey)), a_out);
        if (!(cur < end)) return;                  // an empty part
    }
    const int nxy = nx * ny;                       // < 2^31 (checked at plan creation)
    // q0: the pixel; q1 (G = 4): its quarter turn x * n + n-1-y; the turns by
    // pi of both are nxy - 1 minus them
    int q0 = jy * nx + jx, q1 = jx * nx + (nx - 1 - jy);
    float pax = (float)(px ? jx + 1 : jx);
    float pay = (float)(py ? jy + 1 : jy);
    const float stx = px ? 1.0f : -1.0f, sty = py ? 1.0f : -1.0f;
    const int dq0x = px ? 1 : -1, dq0y = py ? nx : -nx;
    const int dq1x = px ? nx : -nx, dq1y = py ? -1 : 1;
    float nAx = fmaf(pax, inv_x, off_x);
    float nAy = fmaf(pay, inv_y, off_y);
    float s[G];
#pragma unroll
    for (int j = 0; j < G; j++) s[j] = 0.0f;
    bool in = true;                                // the walk is at a pixel of the part
    const int budget = nx + ny + 4;
    for (int it = 0; it < budget && in; it += kFanBatch) {
        float seg[kFanBatch];
        int i0[kFanBatch], i1[kFanBatch];
        bool live[kFanBatch];
#pragma unroll
        for (int u = 0; u < kFanBatch; u++) {
            const float nxt = fminf(nAx, nAy);
            const bool cont = nxt < end;           // false at the part's end (and for NaN)
            live[u] = in;
            seg[u] = nxt - cur;
            i0[u] = q0; i1[u] = q1;
            if (in && cont) {
                if (nAx == nxt) { pax += stx; nAx = fmaf(pax, inv_x, off_x); q0 += dq0x; q1 += dq1x; }
                if (nAy == nxt) { pay += sty; nAy = fmaf(pay, inv_y, off_y); q0 += dq0y; q1 += dq1y; }
                cur = nxt;
            }
            in = in && cont;
        }
        float v[kFanBatch][G];
#pragma unroll
        for (int u = 0; u < kFanBatch; u++) {
            const int q[4] = {i0[u], G == 4 ? i1[u] : nxy - 1 - i0[u], nxy - 1 - i0[u],
                              nxy - 1 - i1[u]};
#pragma unroll
            for (int j = 0; j < G; j++) {
                v[u][j] = 0.0f;
                if (live[u] && FL_IN(q[j], xlen)) v[u][j] = ldv(x + q[j]);
            }
        }
#pragma unroll
        for (int u = 0; u < kFanBatch; u++)
#pragma unroll
            for (int j = 0; j < G; j++)
                if (live[u]) s[j] = fmaf(seg[u], v[u][j], s[j]);
    }
#pragma unroll
    for (int j = 0; j < G; j++) acc[j] = s[j];
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

// One view of the fan gather: adds w_rV * yw_r for every ray of view iv whose
// column window covers the block.
template <int PX, int PY>
__device__ __forceinline__ void fan_view_gather(float (&acc)[PY][PX], const float* __restrict__ yw,
                                                const ColEntry* __restrict__ col,
                                                const ViewEntry& ve, int iv, const DetGrid& G,
                                                float x0, float y0, const float (&fx)[PX + 1],
                                                const float (&fy)[PY + 1], int na)
{
    int lo, hi; float dmin, dmax;
    column_window(G, ve.c, ve.s, x0, y0, (float)PX, (float)PY, na, lo, hi, dmin, dmax);
    const ColEntry* cv = col + (long long)iv * na;
    const float* yv = yw + (long long)iv * na;
    for (int ia = lo; ia <= hi; ia++) {
        if (!FL_IN(ia, na)) continue;
        const ColEntry ce = cv[ia];
        const float yval = __ldg(yv + ia);
        float ax[PX + 1], ay[PY + 1];
#pragma unroll
        for (int i = 0; i <= PX; i++) ax[i] = fmaf(fx[i], ce.inv_x, ce.off_x);
#pragma unroll
        for (int j = 0; j <= PY; j++) ay[j] = fmaf(fy[j], ce.inv_y, ce.off_y);
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
    const float x0 = (float)(ix0 - nx / 2), y0 = (float)(iy0 - ny / 2);
    float fx[PX + 1], fy[PY + 1];
#pragma unroll
    for (int i = 0; i <= PX; i++) fx[i] = (float)(ix0 + i);
#pragma unroll
    for (int j = 0; j <= PY; j++) fy[j] = (float)(iy0 + j);
#pragma unroll
    for (int j = 0; j < PY; j++)
#pragma unroll
        for (int i = 0; i < PX; i++) acc[j][i] = 0.0f;
    for (int jv = g; jv < nvf; jv += kFanGroups) {
        const int iv = views[jv];
        fan_view_gather<PX, PY>(acc, yw, col, view[iv], iv, G, x0, y0, fx, fy, na);
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
    const float x0 = (float)(ix0 - nx / 2), y0 = (float)(iy0 - ny / 2);
    float fx[PX + 1], fy[PY + 1];
#pragma unroll
    for (int i = 0; i <= PX; i++) fx[i] = (float)(ix0 + i);
#pragma unroll
    for (int j = 0; j <= PY; j++) fy[j] = (float)(iy0 + j);
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
        fan_view_gather<PX, PY>(part[0], yw, col, view[iv], iv, G, x0, y0, fx, fy, na);
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

// View groups of the fan turn adjoint (k_adj_fan_turn).
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
            float fx[P + 1], fy[P + 1];
#pragma unroll
            for (int q = 0; q <= P; q++) { fx[q] = (float)(X0[k] + q); fy[q] = (float)(Y0[k] + q); }
            for (int ia = lo; ia <= hi; ia++) {
                if (!FL_IN(ia, na)) continue;
                const ColEntry ce = cv[ia];
                float ax[P + 1], ay[P + 1];
#pragma unroll
                for (int q = 0; q <= P; q++) {
                    ax[q] = fmaf(fx[q], ce.inv_x, ce.off_x);
                    ay[q] = fmaf(fy[q], ce.inv_y, ce.off_y);
                }
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
constexpr int kFanLanes = 8;
constexpr long long kFanSplitWalks = 1LL << 16;
constexpr int kFanBlock = 256;       // threads per block of the fan turn forward

__host__ __device__ inline int fan_turn_lanes(long long walks)
{
    return walks < kFanSplitWalks ? kFanLanes : 1;
}

// One block of kFanBlock threads of the fan turn forward (G = 2 or 4, one
// frame): L threads per ray (iv < nv/G, ia), each walking one part of it
// (walk_fan), their sums added in part order; the walk also yields the rays
// of views iv + j nv/G at the same column, all with the walked ray's c_r.
// The block holds the rays r0, r0 + 1, ... : with L parts, kFanBlock / L
// rays, part k in warp(s) k, so a warp's gathers follow neighbouring rays.
// Small fan launches have few rays: the parts give the GPU L times the
// threads, each with that fraction of the walk. ypack writes the
// adjoint-input layout of these plans: the G values of ray (iv, ia)'s orbit
// side by side at G (iv na + ia) + j. Every thread of the block must call it
// (it synchronises the block).
template <typename TX, typename TY, int G, int L>
__device__ __forceinline__ void fan_turn_forward_block(const TX* __restrict__ X,
                                                       TY* __restrict__ y,
                                                       const ColEntry* __restrict__ col,
                                                       const float* __restrict__ colr, int nx,
                                                       int ny, int na, int nv, float scale,
                                                       int cr_power,
                                                       const float* __restrict__ xscale,
                                                       int ypack, long long r0)
{
    constexpr int NR = kFanBlock / L;          // rays per block
    const int gv = nv / G;
    const int tx = threadIdx.x % NR, lane = threadIdx.x / NR;
    const long long r = r0 + tx;
    const bool ray = r < (long long)na * gv;
    float acc[G];
#pragma unroll
    for (int j = 0; j < G; j++) acc[j] = 0.0f;
    if (ray) {
        const ColEntry ce = col[r];
        walk_fan<TX, G, L>(X, ce.inv_x, ce.off_x, ce.inv_y, ce.off_y, nx, ny, acc,
                           (long long)nx * ny, lane);
    }
    if constexpr (L > 1) {
        // part k of ray tx is thread k NR + tx: the first NR threads add them in order
        __shared__ float part[L][G][NR];
#pragma unroll
        for (int j = 0; j < G; j++) part[lane][j][tx] = acc[j];
        __syncthreads();
        if (lane != 0) return;
#pragma unroll
        for (int j = 0; j < G; j++) {
            float sum = part[0][j][tx];
#pragma unroll
            for (int k = 1; k < L; k++) sum += part[k][j][tx];
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
template <typename TX, int G, int P>
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
        fan_turn_gather<G, P>(acc, ywp, col, view, D, bx, iy0, nx, ny, na, nv, g, kTurnGroups);
    __shared__ float part[kTurnGroups][G * P * P][kFanX];
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
                for (int k = 1; k < kTurnGroups; k++) sum += part[k][(m * P + j) * P + i][tx];
                Store<TX>::st(X + (long long)py[m] * nx + px[m], sum);
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
