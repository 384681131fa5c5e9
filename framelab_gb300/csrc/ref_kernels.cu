// ref_kernels.cu -- GPU kernels that reproduce the reference's CPU projectors
// bit for bit (FL_MODEL_SIDDON_REF forward, FL_MODEL_CHORD_REF adjoint).
//
// Every float operation is the one the reference performs, in its order,
// through the pinned intrinsics of fl_common.cuh (no FMA contraction).
// Work that cannot change the result is skipped: the Siddon merge starts a
// few planes before the ray enters the image and stops a few planes after it
// leaves (decided in FP64 with a 2-voxel safety band), since segments
// outside the image add nothing in the reference either.
#include "fl_common.cuh"
#include "fl_plan.h"

namespace {

// ---------------------------------------------------------------------------
// Siddon merge (version 0). One axis of plane crossings; see oracle.c for the
// argument that a plain sorted merge equals the reference's sort_alpha() merge
// (sort_alpha.cpp:15-60) for the sum it feeds.
// ---------------------------------------------------------------------------
struct MergeAxis {
    int i;        // current plane index
    int left;     // planes still to emit (including i)
    int di;       // +1 / -1
    float p1, d;  // source coordinate, direction component
    float pitch;  // plane spacing: 1 for x/y, dz0 for z
    bool zaxis;
    float head;
};

__device__ __forceinline__ float merge_alpha(const MergeAxis& a, int i)
{
    if (a.zaxis) return fdiv(fsub(fmul((float)i, a.pitch), a.p1), a.d);  // Ax_cone_mf_cpu_siddon.cpp:69
    return fdiv(fsub((float)i, a.p1), a.d);                               // Ax_fan_mf_cpu_siddon.cpp:44
}

// Box-clip one axis of the ray (p1 -> p1+d) against planes [lo, hi] in FP64;
// returns false when the ray misses the slab entirely.
__device__ __forceinline__ bool clip_axis(double p1, double d, double lo, double hi,
                                          double& amin, double& amax)
{
    if (d == 0.0) return p1 >= lo && p1 <= hi;
    double t0 = (lo - p1) / d, t1 = (hi - p1) / d;
    if (t0 > t1) { double t = t0; t0 = t1; t1 = t; }
    amin = fmax(amin, t0);
    amax = fmin(amax, t1);
    return true;
}

// Plane index range [first..last] (in traversal order) covering alpha in
// [A0, A1] plus one plane on either side and one more for rounding.
__device__ __forceinline__ void init_axis(MergeAxis& a, float p1, float p2, int n, bool zaxis,
                                          float dz0, double A0, double A1)
{
    int n2 = n / 2;
    a.p1 = p1; a.d = fsub(p2, p1); a.zaxis = zaxis; a.pitch = zaxis ? dz0 : 1.0f;
    a.left = 0;
    if (p1 == p2) return;
    double pitch = zaxis ? (double)dz0 : 1.0;
    double c0 = ((double)p1 + A0 * (double)a.d) / pitch;
    double c1 = ((double)p1 + A1 * (double)a.d) / pitch;
    int first, last;
    if (p1 < p2) {
        a.di = 1;
        first = max(-n2, (int)floor(c0) - 2);
        last = min(n2, (int)ceil(c1) + 2);
        a.left = last - first + 1;
    } else {
        a.di = -1;
        first = min(n2, (int)ceil(c0) + 2);
        last = max(-n2, (int)floor(c1) - 2);
        a.left = first - last + 1;
    }
    if (a.left < 0) a.left = 0;
    a.i = first;
    if (a.left > 0) a.head = merge_alpha(a, a.i);
}

template <int NA>
__device__ __forceinline__ int pick_min(const MergeAxis (&ax)[NA])
{
    int best = -1;
#pragma unroll
    for (int k = 0; k < NA; k++)
        if (ax[k].left > 0 && (best < 0 || ax[k].head < ax[best].head)) best = k;
    return best;
}

template <int NA>
__device__ __forceinline__ float pop(MergeAxis (&ax)[NA], int k)
{
    float v = ax[k].head;
    // select by constant index so the array stays in registers
#pragma unroll
    for (int j = 0; j < NA; j++) {
        if (j == k) {
            ax[j].left -= 1;
            ax[j].i += ax[j].di;
            if (ax[j].left > 0) ax[j].head = merge_alpha(ax[j], ax[j].i);
        }
    }
    return v;
}

// Fan-beam Siddon, restating Ax_fan_mf_cpu_siddon.cpp:19-93. One thread per ray.
__global__ void __launch_bounds__(128)
k_ref_fan_siddon(const float* __restrict__ X, float* __restrict__ y,
                 const float* __restrict__ cphi_v, const float* __restrict__ sphi_v,
                 const float* __restrict__ ydet, const int* __restrict__ vframe, float SO,
                 float OD, float scale, int nx, int ny, int nd, long long nper)
{
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    int iv = blockIdx.y;
    if (id >= nd) return;
    const float* x = X + (long long)vframe[iv] * nper;
    float c = cphi_v[iv], s = sphi_v[iv];
    float x1 = fmul(c, -SO), y1 = fmul(s, -SO);
    float u = ydet[id];
    float x2 = fsub(fmul(c, OD), fmul(s, u));
    float y2 = fadd(fmul(s, OD), fmul(c, u));
    float dx = fsub(x2, x1), dy = fsub(y2, y1);
    float total = fsqrt(fadd(fmul(dx, dx), fmul(dy, dy)));
    int nx2 = nx / 2, ny2 = ny / 2;

    double A0 = -1e300, A1 = 1e300;
    bool hit = clip_axis(x1, dx, -nx2 - 2.0, nx - nx2 + 2.0, A0, A1) &&
               clip_axis(y1, dy, -ny2 - 2.0, ny - ny2 + 2.0, A0, A1);
    float acc = 0.0f;
    if (hit && A0 < A1) {
        MergeAxis ax[2];
        init_axis(ax[0], x1, x2, nx, false, 1.0f, A0, A1);
        init_axis(ax[1], y1, y2, ny, false, 1.0f, A0, A1);
        int k = pick_min(ax);
        if (k >= 0) {
            float prev = pop(ax, k);
            while ((k = pick_min(ax)) >= 0) {
                float next = pop(ax, k);
                float ac = fmul(0.5f, fadd(prev, next));
                int tx = (int)floorf(fadd(fadd(x1, fmul(ac, dx)), (float)nx2));
                if (tx >= 0 && tx < nx) {
                    int ty = (int)floorf(fadd(fadd(y1, fmul(ac, dy)), (float)ny2));
                    if (ty >= 0 && ty < ny) {
                        float seg = fmul(fsub(next, prev), total);
                        acc = fadd(acc, fmul(seg, __ldg(x + ty * nx + tx)));
                    }
                }
                prev = next;
            }
        }
    }
    y[(long long)iv * nd + id] = fmul(acc, scale);
}

// Cone-beam Siddon, restating Ax_cone_mf_cpu_siddon.cpp:19-134.
__global__ void __launch_bounds__(128)
k_ref_cone_siddon(const float* __restrict__ X, float* __restrict__ y,
                  const float* __restrict__ cphi_v, const float* __restrict__ sphi_v,
                  const float* __restrict__ sdz, const float* __restrict__ ydet,
                  const float* __restrict__ zdet, const int* __restrict__ vframe, float SO,
                  float OD, float scale, int nx, int ny, int nz, float dz0, int na, int nb,
                  long long nper)
{
    int ia = blockIdx.x * blockDim.x + threadIdx.x;
    int ib = blockIdx.y;
    int iv = blockIdx.z;
    if (ia >= na) return;
    const float* x = X + (long long)vframe[iv] * nper;
    float c = cphi_v[iv], s = sphi_v[iv];
    float x1 = fmul(c, -SO), y1 = fmul(s, -SO), z1 = sdz[iv];
    float u = ydet[ia];
    float x2 = fsub(fmul(c, OD), fmul(s, u));
    float y2 = fadd(fmul(s, OD), fmul(c, u));
    float z2 = fadd(zdet[ib], sdz[iv]);
    float dx = fsub(x2, x1), dy = fsub(y2, y1), dz = fsub(z2, z1);
    float total = fsqrt(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)));
    int nx2 = nx / 2, ny2 = ny / 2, nz2 = nz / 2;

    double A0 = -1e300, A1 = 1e300;
    bool hit = clip_axis(x1, dx, -nx2 - 2.0, nx - nx2 + 2.0, A0, A1) &&
               clip_axis(y1, dy, -ny2 - 2.0, ny - ny2 + 2.0, A0, A1) &&
               clip_axis(z1, dz, (-nz2 - 2.0) * (double)dz0, (nz - nz2 + 2.0) * (double)dz0,
                         A0, A1);
    float acc = 0.0f;
    if (hit && A0 < A1) {
        MergeAxis ax[3];
        init_axis(ax[0], x1, x2, nx, false, 1.0f, A0, A1);
        init_axis(ax[1], y1, y2, ny, false, 1.0f, A0, A1);
        init_axis(ax[2], z1, z2, nz, true, dz0, A0, A1);
        int k = pick_min(ax);
        if (k >= 0) {
            float prev = pop(ax, k);
            while ((k = pick_min(ax)) >= 0) {
                float next = pop(ax, k);
                float ac = fmul(0.5f, fadd(prev, next));
                int tx = (int)floorf(fadd(fadd(x1, fmul(ac, dx)), (float)nx2));
                if (tx >= 0 && tx < nx) {
                    int ty = (int)floorf(fadd(fadd(y1, fmul(ac, dy)), (float)ny2));
                    if (ty >= 0 && ty < ny) {
                        int tz = (int)floorf(fadd(fdiv(fadd(z1, fmul(ac, dz)), dz0), (float)nz2));
                        if (tz >= 0 && tz < nz) {
                            float seg = fmul(fsub(next, prev), total);
                            acc = fadd(acc, fmul(seg, __ldg(x + ((long long)tz * ny + ty) * nx + tx)));
                        }
                    }
                }
                prev = next;
            }
        }
    }
    y[((long long)iv * nb + ib) * na + ia] = fmul(acc, scale);
}

// ---------------------------------------------------------------------------
// Chord-length backprojectors (version 1).
// ---------------------------------------------------------------------------

// find_l (find_l.cpp:18-45): chord of the line a*x+b*y=c through the unit
// pixel centred at (x, y).
__device__ __forceinline__ float chord_unit_pixel(float a, float b, float c, float x, float y)
{
    float aa = fabs_ref(a), bb = fabs_ref(b);
    float ha = fdiv(aa, 2.0f), hb = fdiv(bb, 2.0f);
    float reach = fadd(ha, hb);
    float d = fabs_ref(fsub(fsub(c, fmul(a, x)), fmul(b, y)));
    if (!(d < reach)) return 0.0f;
    float flat = fabs_ref(fsub(ha, hb));
    float full = (ha < hb) ? fdiv(1.0f, bb) : fdiv(1.0f, aa);
    return (d <= flat) ? full : fdiv(fsub(reach, d), fmul(aa, bb));
}

// 2-D helper of find_l_3d.cpp:19-92 (a line through a w x h rectangle).
__device__ float chord_rect(float px, float py, float qx, float qy, float w, float h, float x,
                            float y)
{
    float a = fsub(qx, px), b = fsub(qy, py);
    float hw = fdiv(w, 2.0f), hh = fdiv(h, 2.0f);
    if (a == 0.0f) return (fabs_ref(fsub(px, x)) <= hw) ? h : 0.0f;
    if (b == 0.0f) return (fabs_ref(fsub(py, y)) <= hh) ? w : 0.0f;
    float rx = fsub(px, x), ry = fsub(py, y);
    float hx0 = 0, hy0 = 0, hx1 = 0, hy1 = 0;
    int nh = 0;
    bool xfirst = fabs_ref(a) > fabs_ref(b);
#pragma unroll
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1 && nh >= 2) break;
        bool xfam = (pass == 0) ? xfirst : !xfirst;
        float s, t, uu;
        if (xfam) { s = fdiv(b, a); t = fadd(fmul(s, -rx), ry); uu = fmul(s, hw); }
        else      { s = fdiv(a, b); t = fadd(fmul(s, -ry), rx); uu = fmul(s, hh); }
#pragma unroll
        for (int side = 0; side < 2; side++) {
            if (pass == 1 && side == 1 && nh >= 2) break;
            float v = side ? fadd(t, uu) : fsub(t, uu);
            bool ok = xfam ? (fabs_ref(v) <= hh) : (fabs_ref(v) <= hw);
            if (ok) {
                float px_ = xfam ? (side ? hw : -hw) : v;
                float py_ = xfam ? v : (side ? hh : -hh);
                if (nh == 0) { hx0 = px_; hy0 = py_; } else { hx1 = px_; hy1 = py_; }
                nh++;
            }
        }
    }
    if (nh != 2) return 0.0f;
    float ex = fsub(hx1, hx0), ey = fsub(hy1, hy0);
    return fsqrt(fadd(fmul(ex, ex), fmul(ey, ey)));
}

// find_l_3d (find_l_3d.cpp:94-182): chord of the line P->Q through the box of
// size (w,h,t) centred at (x,y,z); faces of the dominant xy axis first, then
// the other xy axis, then z; the first two hits give the chord.
__device__ float chord_box(float px, float py, float pz, float qx, float qy, float qz, float w,
                           float h, float t, float x, float y, float z)
{
    float a = fsub(qx, px), b = fsub(qy, py), c = fsub(qz, pz);
    float hw = fdiv(w, 2.0f), hh = fdiv(h, 2.0f), ht = fdiv(t, 2.0f);
    if (a == 0.0f) return chord_rect(py, pz, qy, qz, h, t, y, z);
    if (b == 0.0f) return chord_rect(px, pz, qx, qz, w, t, x, z);
    float rx = fsub(px, x), ry = fsub(py, y), rz = fsub(pz, z);
    float P0[3] = {0, 0, 0}, P1[3] = {0, 0, 0};
    int nh = 0;
    int f0 = (fabs_ref(a) > fabs_ref(b)) ? 0 : 1;
#pragma unroll
    for (int pass = 0; pass < 3; pass++) {
        if (pass > 0 && nh >= 2) break;
        int fam = (pass == 0) ? f0 : (pass == 1 ? 1 - f0 : 2);
        float u0, u1, v0, v1, lim0, lim1;
        if (fam == 0) {
            float s = fdiv(b, a); u0 = fadd(fmul(s, -rx), ry); u1 = fmul(s, hw);
            s = fdiv(c, a);       v0 = fadd(fmul(s, -rx), rz); v1 = fmul(s, hw);
            lim0 = hh; lim1 = ht;
        } else if (fam == 1) {
            float s = fdiv(a, b); u0 = fadd(fmul(s, -ry), rx); u1 = fmul(s, hh);
            s = fdiv(c, b);       v0 = fadd(fmul(s, -ry), rz); v1 = fmul(s, hh);
            lim0 = hw; lim1 = ht;
        } else {
            float s = fdiv(a, c); u0 = fadd(fmul(s, -rz), rx); u1 = fmul(s, ht);
            s = fdiv(b, c);       v0 = fadd(fmul(s, -rz), ry); v1 = fmul(s, ht);
            lim0 = hw; lim1 = hh;
        }
#pragma unroll
        for (int side = 0; side < 2; side++) {
            if (pass > 0 && side == 1 && nh >= 2) break;
            float uu = side ? fadd(u0, u1) : fsub(u0, u1);
            float vv = side ? fadd(v0, v1) : fsub(v0, v1);
            if (fabs_ref(uu) <= lim0 && fabs_ref(vv) <= lim1) {
                float q0, q1, q2;
                if (fam == 0)      { q0 = side ? hw : -hw; q1 = uu; q2 = vv; }
                else if (fam == 1) { q0 = uu; q1 = side ? hh : -hh; q2 = vv; }
                else               { q0 = uu; q1 = vv; q2 = side ? ht : -ht; }
                if (nh == 0) { P0[0] = q0; P0[1] = q1; P0[2] = q2; }
                else         { P1[0] = q0; P1[1] = q1; P1[2] = q2; }
                nh++;
            }
        }
    }
    if (nh != 2) return 0.0f;
    float ex = fsub(P1[0], P0[0]), ey = fsub(P1[1], P0[1]), ez = fsub(P1[2], P0[2]);
    return fsqrt(fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez)));
}

// chord_box for a unit cube (w = h = t = 1) when the in-plane direction
// (a, b) has no zero component, with the x- and y-face families' in-plane
// crossings u0x, u1x (the b / a family) and u0y, u1y (the a / b family)
// computed by the caller once per detector column. Every value is the same
// float expression chord_box evaluates, so the result has the same bits.
__device__ float chord_box_col(float a, float b, float c, float u0x, float u1x, float u0y,
                               float u1y, float rx, float ry, float rz)
{
    const float hw = 0.5f, hh = 0.5f, ht = 0.5f;          // fdiv(1, 2), exact
    float P0[3] = {0, 0, 0}, P1[3] = {0, 0, 0};
    int nh = 0;
    int f0 = (fabs_ref(a) > fabs_ref(b)) ? 0 : 1;
#pragma unroll
    for (int pass = 0; pass < 3; pass++) {
        if (pass > 0 && nh >= 2) break;
        int fam = (pass == 0) ? f0 : (pass == 1 ? 1 - f0 : 2);
        float u0, u1, v0, v1, lim0, lim1;
        if (fam == 0) {
            u0 = u0x; u1 = u1x;
            float s = fdiv(c, a); v0 = fadd(fmul(s, -rx), rz); v1 = fmul(s, hw);
            lim0 = hh; lim1 = ht;
        } else if (fam == 1) {
            u0 = u0y; u1 = u1y;
            float s = fdiv(c, b); v0 = fadd(fmul(s, -ry), rz); v1 = fmul(s, hh);
            lim0 = hw; lim1 = ht;
        } else {
            float s = fdiv(a, c); u0 = fadd(fmul(s, -rz), rx); u1 = fmul(s, ht);
            s = fdiv(b, c);       v0 = fadd(fmul(s, -rz), ry); v1 = fmul(s, ht);
            lim0 = hw; lim1 = hh;
        }
#pragma unroll
        for (int side = 0; side < 2; side++) {
            if (pass > 0 && side == 1 && nh >= 2) break;
            float uu = side ? fadd(u0, u1) : fsub(u0, u1);
            float vv = side ? fadd(v0, v1) : fsub(v0, v1);
            if (fabs_ref(uu) <= lim0 && fabs_ref(vv) <= lim1) {
                float q0, q1, q2;
                if (fam == 0)      { q0 = side ? hw : -hw; q1 = uu; q2 = vv; }
                else if (fam == 1) { q0 = uu; q1 = side ? hh : -hh; q2 = vv; }
                else               { q0 = uu; q1 = vv; q2 = side ? ht : -ht; }
                if (nh == 0) { P0[0] = q0; P0[1] = q1; P0[2] = q2; }
                else         { P1[0] = q0; P1[1] = q1; P1[2] = q2; }
                nh++;
            }
        }
    }
    if (nh != 2) return 0.0f;
    float ex = fsub(P1[0], P0[0]), ey = fsub(P1[1], P0[1]), ez = fsub(P1[2], P0[2]);
    return fsqrt(fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez)));
}

// Fan-beam chord backprojection, restating Atx_fan_mf_cpu_new.cpp:21-63.
// One thread per (pixel, frame).
__global__ void __launch_bounds__(128)
k_ref_fan_chord_adj(float* __restrict__ x, const float* __restrict__ Y,
                    const float* __restrict__ cos_phi, const float* __restrict__ sin_phi,
                    const float* __restrict__ cos_det, const float* __restrict__ sin_det,
                    const int* __restrict__ idY, const int* __restrict__ Nv, int tmp_size,
                    float SO, float OD, float scale, float dy_det, float y_os, int nx, int ny,
                    int nd, int nt)
{
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y;
    int it = blockIdx.z;
    if (ix >= nx) return;
    int nd2 = nd / 2, nx2 = nx / 2, ny2 = ny / 2;
    float SD = fadd(SO, OD);
    // (float)(i + 0.5 - n2) is exact for any realistic size
    float yc = (float)(iy - ny2) + 0.5f;
    float xc = (float)(ix - nx2) + 0.5f;
    float acc = 0.0f;
    int nvf = Nv[it];
    for (int j = 0; j < nvf; j++) {
        int iv = idY[it * tmp_size + j];
        const float* yv = Y + (long long)iv * nd;
        float c = cos_phi[iv], s = sin_phi[iv];
        float xr = fadd(fmul(c, xc), fmul(s, yc));
        float yr = fadd(fmul(-s, xc), fmul(c, yc));
        float g = fdiv(SD, fmul(fadd(xr, SO), dy_det));
        int hi = (int)floorf(fadd(fsub(fmul(fadd(yr, 1.0f), g), y_os), (float)nd2));
        int lo = (int)floorf(fadd(fsub(fmul(fsub(yr, 1.0f), g), y_os), (float)nd2));
        lo = max(lo, 0);
        hi = min(hi, nd - 1);
        for (int id = lo; id <= hi; id++) {
            float sd = __ldg(sin_det + id), cd = __ldg(cos_det + id);
            float Px = -fadd(fmul(sd, c), fmul(cd, s));
            float Py = fsub(fmul(cd, c), fmul(sd, s));
            float Pd = fmul(SO, sd);
            float l = chord_unit_pixel(Px, Py, Pd, xc, yc);
            if (l > 0.0f) acc = fadd(acc, fmul(l, __ldg(yv + id)));
        }
    }
    x[(long long)it * nx * ny + (long long)iy * nx + ix] = fmul(acc, scale);
}

// Cone-beam chord backprojection, restating Atx_cone_mf_cpu_new.cpp:23-85
// (unit-cube chord, z window half-width sqrt(1 + dz^2/2)). Per view, the
// detector columns of a voxel's window (up to kChordCols of them) get their
// row-independent find_l_3d terms once, in shared memory (one slot per
// thread), and every row of the window reuses them; wider windows take the
// plain per-(column, row) evaluation. The sums run in the reference's order.
constexpr int kChordCols = 8;

__global__ void __launch_bounds__(128)
k_ref_cone_chord_adj(float* __restrict__ x, const float* __restrict__ Y,
                     const float* __restrict__ cos_phi, const float* __restrict__ sin_phi,
                     const float* __restrict__ sdz, const float* __restrict__ ydet,
                     const float* __restrict__ zdet, const int* __restrict__ idY,
                     const int* __restrict__ Nv, int tmp_size, float SO, float OD, float scale,
                     float dy_det, float y_os, float dz_det, float dz, int nx, int ny, int nz,
                     int na, int nb)
{
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y;
    int izt = blockIdx.z;            // iz + nz * it
    int iz = izt % nz, it = izt / nz;
    // the window columns' row-independent terms, one slot per thread
    __shared__ float cols[6][kChordCols][128];
    const int t = threadIdx.x;
    if (ix >= nx) return;
    float SD = fadd(SO, OD);
    int na2 = na / 2, nb2 = nb / 2, nx2 = nx / 2, ny2 = ny / 2, nz2 = nz / 2;
    long long nd = (long long)na * nb;
    float dwin = fsqrt(fadd(1.0f, fdiv(fmul(dz, dz), 2.0f)));
    float zc = fmul((float)(iz - nz2) + 0.5f, dz);
    float yc = (float)(iy - ny2) + 0.5f;
    float xc = (float)(ix - nx2) + 0.5f;
    float acc = 0.0f;
    int nvf = Nv[it];
    for (int j = 0; j < nvf; j++) {
        int iv = idY[it * tmp_size + j];
        const float* yv = Y + (long long)iv * nd;
        float c = cos_phi[iv], s = sin_phi[iv];
        float xr = fadd(fmul(c, xc), fmul(s, yc));
        float yr = fadd(fmul(-s, xc), fmul(c, yc));
        float g = fdiv(SD, fmul(fadd(xr, SO), dy_det));
        int amax = (int)floorf(fadd(fsub(fmul(fadd(yr, 1.0f), g), y_os), (float)na2));
        int amin = (int)floorf(fadd(fsub(fmul(fsub(yr, 1.0f), g), y_os), (float)na2));
        g = fdiv(SD, fmul(fadd(xr, SO), dz_det));
        int bmax = (int)floorf(fadd(fmul(fadd(zc, dwin), g), (float)nb2));
        int bmin = (int)floorf(fadd(fmul(fsub(zc, dwin), g), (float)nb2));
        amin = max(amin, 0); amax = min(amax, na - 1);
        bmin = max(bmin, 0); bmax = min(bmax, nb - 1);
        float x1 = fmul(c, -SO), y1 = fmul(s, -SO), z1 = sdz[iv];
        float cOD = fmul(c, OD), sOD = fmul(s, OD);
        const int W = amax - amin + 1;
        if (W >= 1 && W <= kChordCols) {
            // chord_box's offsets of the source from the voxel centre
            const float rx = fsub(x1, xc), ry = fsub(y1, yc), rz = fsub(z1, zc);
            for (int k = 0; k < W; k++) {
                const float u = __ldg(ydet + amin + k);
                const float x2 = fsub(cOD, fmul(s, u)), y2 = fadd(sOD, fmul(c, u));
                const float a = fsub(x2, x1), b = fsub(y2, y1);
                float u0x = 0.0f, u1x = 0.0f, u0y = 0.0f, u1y = 0.0f;
                if (a != 0.0f && b != 0.0f) {
                    float q = fdiv(b, a);
                    u0x = fadd(fmul(q, -rx), ry); u1x = fmul(q, 0.5f);
                    q = fdiv(a, b);
                    u0y = fadd(fmul(q, -ry), rx); u1y = fmul(q, 0.5f);
                }
                cols[0][k][t] = x2; cols[1][k][t] = y2;
                cols[2][k][t] = u0x; cols[3][k][t] = u1x;
                cols[4][k][t] = u0y; cols[5][k][t] = u1y;
            }
            for (int ib = bmin; ib <= bmax; ib++) {
                const float z2 = fadd(__ldg(zdet + ib), z1);
                const float cz = fsub(z2, z1);
                const float* yr_ = yv + (long long)ib * na + amin;
                for (int k = 0; k < W; k++) {
                    const float x2 = cols[0][k][t], y2 = cols[1][k][t];
                    const float a = fsub(x2, x1), b = fsub(y2, y1);
                    const float l =
                        (a == 0.0f || b == 0.0f)
                            ? chord_box(x1, y1, z1, x2, y2, z2, 1.0f, 1.0f, 1.0f, xc, yc, zc)
                            : chord_box_col(a, b, cz, cols[2][k][t], cols[3][k][t],
                                            cols[4][k][t], cols[5][k][t], rx, ry, rz);
                    acc = fadd(acc, fmul(l, __ldg(yr_ + k)));
                }
            }
            continue;
        }
        for (int ib = bmin; ib <= bmax; ib++) {
            float z2 = fadd(__ldg(zdet + ib), z1);
            for (int ia = amin; ia <= amax; ia++) {
                float u = __ldg(ydet + ia);
                float x2 = fsub(cOD, fmul(s, u));
                float y2 = fadd(sOD, fmul(c, u));
                float l = chord_box(x1, y1, z1, x2, y2, z2, 1.0f, 1.0f, 1.0f, xc, yc, zc);
                acc = fadd(acc, fmul(l, __ldg(yv + (long long)ib * na + ia)));
            }
        }
    }
    x[(long long)it * nx * ny * nz + ((long long)iz * ny + iy) * nx + ix] = fmul(acc, scale);
}

// ---------------------------------------------------------------------------
// Dominant-axis forward (version 1): Ax_cone_mf_cpu_new.cpp:23-235 and
// Ax_fan_mf_cpu_new.cpp:18-122. Per slab of the dominant axis the ray touches
// at most two cells along the other in-plane axis and two along z; the case
// analysis (11, 12, 21, 22) and every float operation follow the reference.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float gao_slab(float acc, float p1, float p2, float q1, float q2,
                                          float l, int ns, int nz, const float* __restrict__ x,
                                          long long ss, long long zs, long long base)
{
    const int c1 = (int)floorf(p1), c2 = (int)floorf(p2);
    const int k1 = (int)floorf(q1), k2 = (int)floorf(q2);
#define VOX(c, k) __ldg(x + base + (long long)(k) * zs + (long long)(c) * ss)
    if (c2 == c1) {
        if (c1 >= 0 && c1 <= ns - 1) {
            if (k2 == k1) {
                if (k1 >= 0 && k1 <= nz - 1) acc = fadd(acc, fmul(l, VOX(c1, k1)));
            } else if (k1 >= -1 && k1 <= nz - 1) {
                const float rz = fdiv(fsub((float)k2, q1), fsub(q2, q1));
                if (k1 > -1) acc = fadd(acc, fmul(fmul(rz, l), VOX(c1, k1)));
                if (k2 < nz) acc = fadd(acc, fmul(fmul(fsub(1.0f, rz), l), VOX(c1, k2)));
            }
        }
    } else if (c1 >= -1 && c1 <= ns - 1) {
        const float d = fsub(p2, p1);
        if (k2 == k1) {
            if (k1 >= 0 && k1 <= nz - 1) {
                const float rs = fdiv(fsub((float)c2, p1), d);
                if (c1 > -1) acc = fadd(acc, fmul(fmul(rs, l), VOX(c1, k1)));
                if (c2 < ns) acc = fadd(acc, fmul(fmul(fsub(1.0f, rs), l), VOX(c2, k1)));
            }
        } else if (k1 >= -1 && k1 <= nz - 1) {
            const float rs = fdiv(fsub((float)c2, p1), d);
            const float rz = fdiv(fsub((float)k2, q1), fsub(q2, q1));
            if (rs > rz) {
                if (c1 > -1 && k1 > -1) acc = fadd(acc, fmul(fmul(rz, l), VOX(c1, k1)));
                if (c1 > -1 && k2 < nz) acc = fadd(acc, fmul(fmul(fsub(rs, rz), l), VOX(c1, k2)));
                if (c2 < ns && k2 < nz) acc = fadd(acc, fmul(fmul(fsub(1.0f, rs), l), VOX(c2, k2)));
            } else {
                if (c1 > -1 && k1 > -1) acc = fadd(acc, fmul(fmul(rs, l), VOX(c1, k1)));
                if (c2 < ns && k1 > -1) acc = fadd(acc, fmul(fmul(fsub(rz, rs), l), VOX(c2, k1)));
                if (c2 < ns && k2 < nz) acc = fadd(acc, fmul(fmul(fsub(1.0f, rz), l), VOX(c2, k2)));
            }
        }
    }
#undef VOX
    return acc;
}

__global__ void __launch_bounds__(128)
k_ref_cone_gao(const float* __restrict__ X, float* __restrict__ y, float* __restrict__ ynorm,
               const float* __restrict__ cphi_v, const float* __restrict__ sphi_v,
               const float* __restrict__ sdz, const float* __restrict__ ydet,
               const float* __restrict__ zdet, const int* __restrict__ vframe, float SO,
               float OD, float scale, int nx, int ny, int nz, float dz, int na, int nb,
               long long nper)
{
    const int ia = blockIdx.x * blockDim.x + threadIdx.x;
    const int ib = blockIdx.y, iv = blockIdx.z;
    if (ia >= na) return;
    const float* x = X + (long long)vframe[iv] * nper;
    const int nx2 = nx / 2, ny2 = ny / 2, nz2 = nz / 2;
    const float c = cphi_v[iv], s = sphi_v[iv];
    const float x1 = fmul(c, -SO), y1 = fmul(s, -SO), z1 = sdz[iv];
    const float u = ydet[ia];
    const float x2 = fsub(fmul(c, OD), fmul(s, u));
    const float y2 = fadd(fmul(s, OD), fmul(c, u));
    const float z2 = fadd(zdet[ib], sdz[iv]);
    // norm3 (Ax_cone_mf_cpu_new.cpp:19-20): double sqrt of float differences, returned as float
    const double ex = (double)fsub(x1, x2), ey = (double)fsub(y1, y2), ez = (double)fsub(z1, z2);
    const float norm = fmul(__double2float_rn(__dsqrt_rn(
                                __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez)))),
                            scale);
    const float tmp = fadd(fmul(fsub(x1, x2), fsub(x1, x2)), fmul(fsub(y1, y2), fsub(y1, y2)));
    const float zz = fmul(fsub(z1, z2), fsub(z1, z2));
    const long long zs = (long long)nx * ny;
    float acc = 0.0f;
    const bool xdom = fabs_ref(fsub(x1, x2)) > fabs_ref(fsub(y1, y2));
    // primary axis a (walked), secondary in-plane axis b
    const float pa = xdom ? x1 : y1, pb = xdom ? y1 : x1;
    const float s1 = xdom ? fdiv(fsub(y2, y1), fsub(x2, x1)) : fdiv(fsub(x2, x1), fsub(y2, y1));
    const float s2 = xdom ? fdiv(fsub(z2, z1), fsub(x2, x1)) : fdiv(fsub(z2, z1), fsub(y2, y1));
    const int np = xdom ? nx : ny, np2 = xdom ? nx2 : ny2;
    const int ns = xdom ? ny : nx, ns2 = xdom ? ny2 : nx2;
    const long long ss = xdom ? nx : 1;
    for (int ip = 0; ip < np; ip++) {
        const float a1 = (float)(ip - np2), a2 = fadd(a1, 1.0f);
        const float lo = (s1 >= 0.0f) ? a1 : a2, hi = (s1 >= 0.0f) ? a2 : a1;
        const float p1 = fadd(fadd(pb, fmul(s1, fsub(lo, pa))), (float)ns2);
        const float p2 = fadd(fadd(pb, fmul(s1, fsub(hi, pa))), (float)ns2);
        const float zlo = (s2 >= 0.0f) ? a1 : a2, zhi = (s2 >= 0.0f) ? a2 : a1;
        const float q1 = fadd(fdiv(fadd(z1, fmul(s2, fsub(zlo, pa))), dz), (float)nz2);
        const float q2 = fadd(fdiv(fadd(z1, fmul(s2, fsub(zhi, pa))), dz), (float)nz2);
        const float d = fsub(p2, p1);
        const float l = fsqrt(fdiv(fmul(fadd(fmul(d, d), 1.0f), fadd(tmp, zz)), tmp));
        acc = gao_slab(acc, p1, p2, q1, q2, l, ns, nz, x, ss, zs, xdom ? ip : (long long)ip * nx);
    }
    const long long r = ((long long)iv * nb + ib) * na + ia;
    const float out = fmul(acc, scale);
    y[r] = out;
    if (ynorm) ynorm[r] = fdiv(out, norm);
}

__global__ void __launch_bounds__(128)
k_ref_fan_gao(const float* __restrict__ X, float* __restrict__ y,
              const float* __restrict__ cphi_v, const float* __restrict__ sphi_v,
              const float* __restrict__ ydet, const int* __restrict__ vframe, float SO, float OD,
              float scale, int nx, int ny, int nd, long long nper)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    const int iv = blockIdx.y;
    if (id >= nd) return;
    const float* x = X + (long long)vframe[iv] * nper;
    const int nx2 = nx / 2, ny2 = ny / 2;
    const float c = cphi_v[iv], s = sphi_v[iv];
    const float x1 = fmul(c, -SO), y1 = fmul(s, -SO);
    const float u = ydet[id];
    const float x2 = fsub(fmul(c, OD), fmul(s, u));
    const float y2 = fadd(fmul(s, OD), fmul(c, u));
    const bool xdom = fabs_ref(fsub(x1, x2)) > fabs_ref(fsub(y1, y2));
    const float sl = xdom ? fdiv(fsub(y2, y1), fsub(x2, x1)) : fdiv(fsub(x2, x1), fsub(y2, y1));
    const float pa = xdom ? x1 : y1, pb = xdom ? y1 : x1;
    const int np = xdom ? nx : ny, np2 = xdom ? nx2 : ny2;
    const int ns = xdom ? ny : nx, ns2 = xdom ? ny2 : nx2;
    float acc = 0.0f;
    for (int ip = 0; ip < np; ip++) {
        const float a1 = (float)(ip - np2), a2 = fadd(a1, 1.0f);
        const float lo = (sl >= 0.0f) ? a1 : a2, hi = (sl >= 0.0f) ? a2 : a1;
        const float p1 = fadd(fadd(pb, fmul(sl, fsub(lo, pa))), (float)ns2);
        const float p2 = fadd(fadd(pb, fmul(sl, fsub(hi, pa))), (float)ns2);
        const int c1 = (int)floorf(p1), c2 = (int)floorf(p2);
#define PIX(cc) __ldg(xdom ? x + (long long)(cc) * nx + ip : x + (long long)ip * nx + (cc))
        const float d = fsub(p2, p1);
        const float l = fsqrt(fadd(fmul(d, d), 1.0f));
        if (c2 == c1) {
            if (c1 >= 0 && c1 <= ns - 1) acc = fadd(acc, fmul(l, PIX(c1)));
        } else if (c2 > 0 && c2 < ns) {
            // the reference reads x outside the image when the two crossings round
            // more than a pixel apart (c1 < 0, Ax_fan_mf_cpu_new.cpp:60-63): skipped
            if (c1 >= 0) acc = fadd(acc, fmul(fmul(fdiv(fsub((float)c2, p1), d), l), PIX(c1)));
            acc = fadd(acc, fmul(fmul(fdiv(fsub(p2, (float)c2), d), l), PIX(c2)));
        } else {
            if (c2 == 0) acc = fadd(acc, fmul(fmul(fdiv(fsub(p2, (float)c2), d), l), PIX(c2)));
            // the reference tests c2 == ny on both branches (Ax_fan_mf_cpu_new.cpp:70,111)
            if (c2 == ny && c1 >= 0 && c1 < ns)
                acc = fadd(acc, fmul(fmul(fdiv(fsub((float)c2, p1), d), l), PIX(c1)));
        }
#undef PIX
    }
    y[(long long)iv * nd + id] = fmul(acc, scale);
}

// ---------------------------------------------------------------------------
// Finite-size beam fan pair (version 2): Ax_fan_mf_cpu_new_fb.cpp:19-123,
// Atx_fan_mf_cpu_new_fb.cpp:20-66, find_area.cpp:18-70.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float edge_area(float a, float b, float c, float x, float y, int& sgn)
{
    const float aa = fabs_ref(a), bb = fabs_ref(b);
    const float hx = fdiv(aa, 2.0f), hy = fdiv(bb, 2.0f);
    const float reach = fadd(hx, hy);
    const float off = fsub(fsub(c, fmul(a, x)), fmul(b, y));
    const float d = fabs_ref(off);
    sgn = off > 0.0f ? 1 : -1;
    if (!(d < reach)) return 0.5f;
    const float flat = fabs_ref(fsub(hx, hy));
    const float inv = (hx < hy) ? fdiv(1.0f, bb) : fdiv(1.0f, aa);
    if (d <= flat) return fmul(d, inv);
    const float r = fsub(reach, d);
    return fsub(0.5f, fdiv(fmul(fmul(0.5f, r), r), fmul(aa, bb)));
}

__device__ __forceinline__ float beam_area(float a1, float b1, float c1, float a2, float b2,
                                           float c2, float x, float y)
{
    int s1, s2;
    const float A1 = edge_area(a1, b1, c1, x, y, s1);
    const float A2 = edge_area(a2, b2, c2, x, y, s2);
    return fabs_ref(fsub(A1, fmul((float)(s1 * s2), A2)));
}

// edges: per (view, bin, edge e) the beam-edge line (Px, Py, Pd), evaluated on
// the host with the float libm calls the reference makes.
__global__ void __launch_bounds__(128)
k_ref_fan_fb(const float* __restrict__ X, float* __restrict__ y,
             const float* __restrict__ cphi_v, const float* __restrict__ sphi_v,
             const float* __restrict__ ydet, const float* __restrict__ edges,
             const int* __restrict__ vframe, float SO, float OD, float scale, float dy_det,
             int nx, int ny, int nd, long long nper)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    const int iv = blockIdx.y;
    if (id >= nd) return;
    const float* x = X + (long long)vframe[iv] * nper;
    const int nx2 = nx / 2, ny2 = ny / 2;
    const float c = cphi_v[iv], s = sphi_v[iv];
    const float x1 = fmul(c, -SO), y1 = fmul(s, -SO);
    const float hd = fdiv(dy_det, 2.0f);
    const float u0 = fsub(ydet[id], hd), u1 = fadd(ydet[id], hd);
    const float x20 = fsub(fmul(c, OD), fmul(s, u0)), y20 = fadd(fmul(s, OD), fmul(c, u0));
    const float x21 = fsub(fmul(c, OD), fmul(s, u1)), y21 = fadd(fmul(s, OD), fmul(c, u1));
    const float* E = edges + ((long long)iv * nd + id) * 6;
    const float Px0 = E[0], Py0 = E[1], Pd0 = E[2], Px1 = E[3], Py1 = E[4], Pd1 = E[5];
    const bool xdom = fabs_ref(fsub(x1, fdiv(fadd(x20, x21), 2.0f))) >
                      fabs_ref(fsub(y1, fdiv(fadd(y20, y21), 2.0f)));
    const float p1 = xdom ? x1 : y1, q1 = xdom ? y1 : x1;
    const float pe0 = xdom ? x20 : y20, pe1 = xdom ? x21 : y21;
    const float qe0 = xdom ? y20 : x20, qe1 = xdom ? y21 : x21;
    const int np = xdom ? nx : ny, nq = xdom ? ny : nx;
    const int np2 = xdom ? nx2 : ny2, nq2 = xdom ? ny2 : nx2;
    const bool degen = !(pe0 != p1 && pe1 != p1);
    float s0 = 0.0f, s1 = 0.0f;
    if (!degen) { s0 = fdiv(fsub(qe0, q1), fsub(pe0, p1)); s1 = fdiv(fsub(qe1, q1), fsub(pe1, p1)); }
    float acc = 0.0f;
    for (int ip = 0; ip < np; ip++) {
        const float pc = (float)(ip - np2) + 0.5f;
        const float a1 = (float)(ip - np2), a2 = fadd(a1, 1.0f);
        int qmin, qmax;
        if (degen) {
            if (fabs_ref(fsub(p1, pc)) <= 0.5f) { qmin = 0; qmax = nq - 1; }
            else { qmin = 1; qmax = 0; }
        } else {
            const int c0 = (int)floorf(fadd(fadd(q1, fmul(s0, fsub(a1, p1))), (float)nq2));
            const int c1 = (int)floorf(fadd(fadd(q1, fmul(s0, fsub(a2, p1))), (float)nq2));
            const int c2 = (int)floorf(fadd(fadd(q1, fmul(s1, fsub(a1, p1))), (float)nq2));
            const int c3 = (int)floorf(fadd(fadd(q1, fmul(s1, fsub(a2, p1))), (float)nq2));
            qmin = nq - 1; qmax = 0;
            // only in-range crossings move the bounds (Ax_fan_mf_cpu_new_fb.cpp:62-67)
            const int cc[4] = {c0, c1, c2, c3};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (cc[k] < qmin && cc[k] >= 0) qmin = cc[k];
                if (cc[k] > qmax && cc[k] <= nq - 1) qmax = cc[k];
            }
        }
        for (int iq = qmin; iq <= qmax; iq++) {
            const float qc = (float)(iq - nq2) + 0.5f;
            const float l = beam_area(Px0, Py0, Pd0, Px1, Py1, Pd1, xdom ? pc : qc, xdom ? qc : pc);
            if (l > 0.0f)
                acc = fadd(acc, fmul(l, __ldg(xdom ? x + (long long)iq * nx + ip
                                                  : x + (long long)ip * nx + iq)));
        }
    }
    y[(long long)iv * nd + id] = fmul(acc, scale);
}

__global__ void __launch_bounds__(128)
k_ref_fan_fb_adj(float* __restrict__ x, const float* __restrict__ Y,
                 const float* __restrict__ cos_phi, const float* __restrict__ sin_phi,
                 const float* __restrict__ cos_e, const float* __restrict__ sin_e,
                 const int* __restrict__ idY, const int* __restrict__ Nv, int tmp_size,
                 float SO, float OD, float scale, float dy_det, int nx, int ny, int nd, int nt)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y, it = blockIdx.z;
    if (ix >= nx) return;
    const int nd2 = nd / 2, nx2 = nx / 2, ny2 = ny / 2;
    const float SD = fadd(SO, OD);
    const float yc = (float)(iy - ny2) + 0.5f, xc = (float)(ix - nx2) + 0.5f;
    float acc = 0.0f;
    const int nvf = Nv[it];
    for (int j = 0; j < nvf; j++) {
        const int iv = idY[it * tmp_size + j];
        const float* yv = Y + (long long)iv * nd;
        const float c = cos_phi[iv], s = sin_phi[iv];
        const float xr = fadd(fmul(c, xc), fmul(s, yc));
        const float yr = fadd(fmul(-s, xc), fmul(c, yc));
        const float g = fdiv(SD, fmul(fadd(xr, SO), dy_det));
        int hi = (int)floorf(fadd(fmul(fadd(yr, 1.0f), g), (float)nd2));
        int lo = (int)floorf(fadd(fmul(fsub(yr, 1.0f), g), (float)nd2));
        lo = max(lo, 0);
        hi = min(hi, nd - 1);
        for (int id = lo; id <= hi; id++) {
            const float sd0 = __ldg(sin_e + id), cd0 = __ldg(cos_e + id);
            const float sd1 = __ldg(sin_e + id + 1), cd1 = __ldg(cos_e + id + 1);
            const float Px0 = -fadd(fmul(sd0, c), fmul(cd0, s));
            const float Py0 = fsub(fmul(cd0, c), fmul(sd0, s));
            const float Pd0 = fmul(SO, sd0);
            const float Px1 = -fadd(fmul(sd1, c), fmul(cd1, s));
            const float Py1 = fsub(fmul(cd1, c), fmul(sd1, s));
            const float Pd1 = fmul(SO, sd1);
            const float l = beam_area(Px0, Py0, Pd0, Px1, Py1, Pd1, xc, yc);
            if (l > 0.0f) acc = fadd(acc, fmul(l, __ldg(yv + id)));
        }
    }
    x[(long long)it * nx * ny + (long long)iy * nx + ix] = fmul(acc, scale);
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers (device pointers, stream-ordered)
// ---------------------------------------------------------------------------
int fl_ref_forward(fl_plan* p, const float* x, float* y, cudaStream_t st)
{
    const fl_scan& s = p->s;
    if (s.nx % 2 || s.ny % 2 || (s.ndim == 3 && s.nz % 2))
        return fl_set_error(FL_ERR_UNSUPPORTED,
                            "Siddon (version 0) needs even nx, ny, nz: the reference's plane "
                            "lists are one entry short for odd sizes");
    long long nper = (long long)s.nx * s.ny * s.nz;
    if (s.ndim == 2) {
        dim3 grid(fl_div_up(s.na, 128), s.nv);
        k_ref_fan_siddon<<<grid, 128, 0, st>>>(x, y, p->d_cphi_f, p->d_sphi_f, p->d_y_det,
                                               p->d_view_frame, s.SO, s.OD, s.scale, s.nx,
                                               s.ny, s.na, nper);
    } else {
        dim3 grid(fl_div_up(s.na, 128), s.nb, s.nv);
        k_ref_cone_siddon<<<grid, 128, 0, st>>>(x, y, p->d_cphi_f, p->d_sphi_f, p->d_sd_z,
                                                p->d_y_det, p->d_z_det, p->d_view_frame, s.SO,
                                                s.OD, s.scale, s.nx, s.ny, s.nz, s.dz, s.na,
                                                s.nb, nper);
    }
    return fl_check_launch("reference Siddon forward");
}

int fl_ref_adjoint(fl_plan* p, const float* y, float* x, cudaStream_t st)
{
    const fl_scan& s = p->s;
    if (s.ndim == 2) {
        dim3 grid(fl_div_up(s.nx, 128), s.ny, s.nt);
        k_ref_fan_chord_adj<<<grid, 128, 0, st>>>(
            x, y, p->d_cos_phi, p->d_sin_phi, p->d_cos_det, p->d_sin_det, p->d_idY, p->d_Nv,
            p->tmp_size, s.SO, s.OD, s.scale, s.dy_det, s.y_os, s.nx, s.ny, s.na, s.nt);
    } else {
        if ((long long)s.nz * s.nt > 65535)
            return fl_set_error(FL_ERR_UNSUPPORTED, "reference backprojector: nz * nt > 65535");
        dim3 grid(fl_div_up(s.nx, 128), s.ny, (unsigned)s.nz * s.nt);
        k_ref_cone_chord_adj<<<grid, 128, 0, st>>>(
            x, y, p->d_cos_phi, p->d_sin_phi, p->d_sd_z, p->d_y_det, p->d_z_det, p->d_idY,
            p->d_Nv, p->tmp_size, s.SO, s.OD, s.scale, s.dy_det, s.y_os, s.dz_det, s.dz, s.nx,
            s.ny, s.nz, s.na, s.nb);
    }
    return fl_check_launch("reference chord backprojection");
}

int fl_ref_gao_forward(fl_plan* p, const float* x, float* y, float* ynorm, cudaStream_t st)
{
    const fl_scan& s = p->s;
    long long nper = (long long)s.nx * s.ny * s.nz;
    if (s.ndim == 2) {
        dim3 grid(fl_div_up(s.na, 128), s.nv);
        k_ref_fan_gao<<<grid, 128, 0, st>>>(x, y, p->d_cphi_f, p->d_sphi_f, p->d_y_det,
                                            p->d_view_frame, s.SO, s.OD, s.scale, s.nx, s.ny,
                                            s.na, nper);
        if (ynorm) return fl_set_error(FL_ERR_UNSUPPORTED, "yNorm is a cone-beam output");
    } else {
        dim3 grid(fl_div_up(s.na, 128), s.nb, s.nv);
        k_ref_cone_gao<<<grid, 128, 0, st>>>(x, y, ynorm, p->d_cphi_f, p->d_sphi_f, p->d_sd_z,
                                             p->d_y_det, p->d_z_det, p->d_view_frame, s.SO, s.OD,
                                             s.scale, s.nx, s.ny, s.nz, s.dz, s.na, s.nb, nper);
    }
    return fl_check_launch("reference dominant-axis forward");
}

int fl_ref_fb_forward(fl_plan* p, const float* x, float* y, cudaStream_t st)
{
    const fl_scan& s = p->s;
    if (s.ndim != 2) return fl_set_error(FL_ERR_UNSUPPORTED, "finite-beam model is fan-beam only");
    if (!p->d_fb_edges) return fl_set_error(FL_ERR_INVALID, "finite-beam model needs dy_det > 0");
    dim3 grid(fl_div_up(s.na, 128), s.nv);
    k_ref_fan_fb<<<grid, 128, 0, st>>>(x, y, p->d_cphi_f, p->d_sphi_f, p->d_y_det, p->d_fb_edges,
                                       p->d_view_frame, s.SO, s.OD, s.scale, s.dy_det, s.nx,
                                       s.ny, s.na, (long long)s.nx * s.ny);
    return fl_check_launch("reference finite-beam forward");
}

int fl_ref_fb_adjoint(fl_plan* p, const float* y, float* x, cudaStream_t st)
{
    const fl_scan& s = p->s;
    if (s.ndim != 2) return fl_set_error(FL_ERR_UNSUPPORTED, "finite-beam model is fan-beam only");
    dim3 grid(fl_div_up(s.nx, 128), s.ny, s.nt);
    k_ref_fan_fb_adj<<<grid, 128, 0, st>>>(x, y, p->d_cos_phi, p->d_sin_phi, p->d_cos_det2,
                                           p->d_sin_det2, p->d_idY, p->d_Nv, p->tmp_size, s.SO,
                                           s.OD, s.scale, s.dy_det, s.nx, s.ny, s.na, s.nt);
    return fl_check_launch("reference finite-beam backprojection");
}
