/*
 * oracle.c -- CPU restatement of FrameLab's reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker the GPU library is
 * compared against; nothing in the product library links, loads or calls it.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * Two families of functions:
 *
 *  (1) *_f32: restatements of the reference's own single-precision CPU
 *      kernels, written so that every float operation (operands, order,
 *      rounding) is the one the reference performs. Compiled with
 *      -ffp-contract=off they reproduce the reference bit for bit; that claim
 *      is pinned by tests/test_oracle_pin.py against the reference sources
 *      compiled unmodified into oracle/_ref (Makefile in this directory) and
 *      by the committed fixtures in tests/golden/.
 *
 *  (2) *_f64: exact-arithmetic (FP64) Siddon model of the same geometry:
 *      exact ray/voxel intersection lengths, its transpose, and the count of
 *      voxels each ray crosses. This is the "FP64 oracle" every error figure
 *      is quoted against.
 *
 * Conventions (reference's own, matlab/mex/src/Ax_cone_mf_cpu_siddon.cpp):
 *   volume index  iz*ny*nx + iy*nx + ix  (x fastest), voxel xy pitch 1,
 *   x/y planes at integers -n/2 .. n/2, z planes at (k - nz/2)*dz;
 *   sinogram index iv*na*nb + ib*na + ia (detector column fastest);
 *   source  (-SO cos phi, -SO sin phi, sd_z[iv]),
 *   detector (OD cos phi - y_det sin phi, OD sin phi + y_det cos phi,
 *             z_det[ib] + sd_z[iv]);  outputs multiplied by `scale`.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* (1a) Siddon forward, FP32, reference arithmetic                            */
/* ------------------------------------------------------------------------- */

/*
 * One axis of plane crossings, generated lazily in ascending alpha order.
 * The reference fills arrays alpha_x[] etc. with (i - p1)/d for
 * i = -n/2..n/2 (ascending when p1 < p2, descending i when p1 > p2) and merges
 * them with sort_alpha() (sort_alpha.cpp:15-60), dropping a value of one list
 * that equals the current head of the other. Here the lists are produced on
 * the fly and merged by always taking the smallest head; a value that the
 * reference de-duplicates becomes a zero-length segment whose contribution is
 * 0*x = +0, so the running sum is bit-identical for finite volumes.
 */
typedef struct {
    int active;     /* p1 != p2 : the ray crosses this family of planes */
    int i, iend;    /* current and one-past-last plane index (stepping by di) */
    int di;         /* +1 when p1 < p2, -1 when p1 > p2 */
    int zaxis;      /* 1: alpha = (i*dz0 - p1)/d ; 0: alpha = (i - p1)/d */
    float p1, d, dz0;
    float head;     /* alpha of plane i */
} orc_axis;

static float orc_axis_alpha(const orc_axis *a, int i)
{
    if (a->zaxis) {
        float zi = (float)i * a->dz0;            /* Ax_cone_mf_cpu_siddon.cpp:69 */
        return (zi - a->p1) / a->d;
    }
    return ((float)i - a->p1) / a->d;            /* Ax_fan_mf_cpu_siddon.cpp:44 */
}

static void orc_axis_init(orc_axis *a, float p1, float p2, int n, int zaxis, float dz0)
{
    int n2 = n / 2;
    a->zaxis = zaxis; a->dz0 = dz0; a->p1 = p1; a->d = p2 - p1;
    a->active = (p1 != p2);
    if (!a->active) return;
    if (p1 < p2) { a->i = -n2; a->iend = n2 + 1; a->di = 1; }
    else         { a->i = n2;  a->iend = -n2 - 1; a->di = -1; }
    a->head = orc_axis_alpha(a, a->i);
}

static int orc_axis_more(const orc_axis *a) { return a->active && a->i != a->iend; }

static void orc_axis_pop(orc_axis *a)
{
    a->i += a->di;
    if (a->i != a->iend) a->head = orc_axis_alpha(a, a->i);
}

/* index of the axis holding the smallest head, or -1 when all are exhausted */
static int orc_pick(orc_axis *ax, int naxes)
{
    int best = -1;
    for (int k = 0; k < naxes; k++)
        if (orc_axis_more(&ax[k]) && (best < 0 || ax[k].head < ax[best].head)) best = k;
    return best;
}

/*
 * Fan-beam Siddon projection of views [v0, v1).
 * Restates Ax_fan_mf_cpu_siddon (Ax_fan_mf_cpu_siddon.cpp:19-93).
 */
void orc_fan_siddon_f32(const float *X, float *y, float SO, float OD, float scale,
                        int nx, int ny, int v0, int v1, const float *sd_phi, int nd,
                        const float *y_det, const int *id_X)
{
    int nx2 = nx / 2, ny2 = ny / 2;
    long n = (long)nx * ny;
    for (int iv = v0; iv < v1; iv++) {
        const float *x = X + (long)id_X[iv] * n;
        /* C++ <math.h> resolves cos(float) to the float overload (cosf) */
        float cphi = cosf(sd_phi[iv]), sphi = sinf(sd_phi[iv]);
        float x1 = cphi * (-SO), y1 = sphi * (-SO);
        for (int id = 0; id < nd; id++) {
            float x2 = cphi * OD - sphi * y_det[id];
            float y2 = sphi * OD + cphi * y_det[id];
            float dx = x2 - x1, dy = y2 - y1;
            orc_axis ax[2];
            orc_axis_init(&ax[0], x1, x2, nx, 0, 1.0f);
            orc_axis_init(&ax[1], y1, y2, ny, 0, 1.0f);
            float total = (float)sqrt(dx * dx + dy * dy);
            float acc = 0.0f;
            int k = orc_pick(ax, 2);
            if (k >= 0) {
                float prev = ax[k].head;
                orc_axis_pop(&ax[k]);
                while ((k = orc_pick(ax, 2)) >= 0) {
                    float next = ax[k].head;
                    orc_axis_pop(&ax[k]);
                    float ac = 0.5f * (prev + next);
                    int tx = (int)floorf(x1 + ac * dx + (float)nx2);
                    if (tx >= 0 && tx < nx) {
                        int ty = (int)floorf(y1 + ac * dy + (float)ny2);
                        if (ty >= 0 && ty < ny) {
                            float seg = (next - prev) * total;
                            acc += seg * x[ty * nx + tx];
                        }
                    }
                    prev = next;
                }
            }
            y[(long)iv * nd + id] = acc * scale;
        }
    }
}

/*
 * One ray of the cone-beam Siddon projection: source angle trig (cphi, sphi),
 * source z `sz`, detector point (ydet, zdet). The float operations and their
 * order are those of Ax_cone_mf_cpu_siddon.cpp:35-131 for that ray.
 */
static float orc_cone_siddon_ray(const float *x, float SO, float OD, float scale, int nx,
                                 int ny, int nz, float cphi, float sphi, float sz, float ydet,
                                 float zdet, float dz0)
{
    int nx2 = nx / 2, ny2 = ny / 2, nz2 = nz / 2;
    float x1 = cphi * (-SO), y1 = sphi * (-SO), z1 = sz;
    float x2 = cphi * OD - sphi * ydet;
    float y2 = sphi * OD + cphi * ydet;
    float z2 = zdet + sz;
    float dx = x2 - x1, dy = y2 - y1, dz = z2 - z1;
    orc_axis ax[3];
    orc_axis_init(&ax[0], x1, x2, nx, 0, 1.0f);
    orc_axis_init(&ax[1], y1, y2, ny, 0, 1.0f);
    orc_axis_init(&ax[2], z1, z2, nz, 1, dz0);
    float total = (float)sqrt(dx * dx + dy * dy + dz * dz);
    float acc = 0.0f;
    int k = orc_pick(ax, 3);
    if (k >= 0) {
        float prev = ax[k].head;
        orc_axis_pop(&ax[k]);
        while ((k = orc_pick(ax, 3)) >= 0) {
            float next = ax[k].head;
            orc_axis_pop(&ax[k]);
            float ac = (prev + next) / 2;
            int tx = (int)floorf(x1 + ac * dx + (float)nx2);
            if (tx >= 0 && tx < nx) {
                int ty = (int)floorf(y1 + ac * dy + (float)ny2);
                if (ty >= 0 && ty < ny) {
                    int tz = (int)floorf((z1 + ac * dz) / dz0 + (float)nz2);
                    if (tz >= 0 && tz < nz) {
                        float seg = (next - prev) * total;
                        acc += seg * x[((long)tz * ny + ty) * nx + tx];
                    }
                }
            }
            prev = next;
        }
    }
    return acc * scale;
}

/*
 * Cone-beam Siddon projection of views [v0, v1).
 * Restates Ax_cone_mf_cpu_siddon (Ax_cone_mf_cpu_siddon.cpp:19-134).
 */
void orc_cone_siddon_f32(const float *X, float *y, float SO, float OD, float scale,
                         int nx, int ny, int nz, int v0, int v1, const float *sd_phi,
                         const float *sd_z, int na, int nb, const float *y_det,
                         const float *z_det, const int *id_X, float dz0)
{
    long n = (long)nx * ny * nz, nd = (long)na * nb;
    for (int iv = v0; iv < v1; iv++) {
        const float *x = X + (long)id_X[iv] * n;
        /* C++ <math.h> resolves cos(float) to the float overload (cosf) */
        float cphi = cosf(sd_phi[iv]), sphi = sinf(sd_phi[iv]);
        for (int ib = 0; ib < nb; ib++)
            for (int ia = 0; ia < na; ia++)
                y[(long)iv * nd + (long)ib * na + ia] =
                    orc_cone_siddon_ray(x, SO, OD, scale, nx, ny, nz, cphi, sphi, sd_z[iv],
                                        y_det[ia], z_det[ib], dz0);
    }
}

/*
 * The same projection for a list of rays (ray id iv*na*nb + ib*na + ia);
 * y[k] is ray rays[k]. Each value is the one orc_cone_siddon_f32 writes.
 */
void orc_cone_siddon_rays(const float *X, float *y, float SO, float OD, float scale, int nx,
                          int ny, int nz, const float *sd_phi, const float *sd_z, int na,
                          int nb, const float *y_det, const float *z_det, const int *id_X,
                          float dz0, const int64_t *rays, long nr)
{
    long n = (long)nx * ny * nz, nd = (long)na * nb;
    for (long k = 0; k < nr; k++) {
        int iv = (int)(rays[k] / nd);
        long r = rays[k] - (long)iv * nd;
        int ib = (int)(r / na), ia = (int)(r - (long)ib * na);
        float cphi = cosf(sd_phi[iv]), sphi = sinf(sd_phi[iv]);
        y[k] = orc_cone_siddon_ray(X + (long)id_X[iv] * n, SO, OD, scale, nx, ny, nz, cphi,
                                   sphi, sd_z[iv], y_det[ia], z_det[ib], dz0);
    }
}

/* ------------------------------------------------------------------------- */
/* (1b) Chord-length backprojectors, FP32, reference arithmetic               */
/* ------------------------------------------------------------------------- */

static float orc_absf(float v) { return v > 0 ? v : -v; }

/*
 * Chord of the line a*x + b*y = c through the unit pixel centred at (x, y).
 * Restates find_l (find_l.cpp:18-45): the distance of the centre to the line
 * decides between the full chord 1/max(|a|,|b|) and the corner-clipped one.
 */
float orc_chord_unit_pixel(float a, float b, float c, float x, float y)
{
    float aa = orc_absf(a), bb = orc_absf(b);
    float ha = aa / 2, hb = bb / 2;
    float reach = ha + hb;
    float off = c - a * x - b * y;
    float d = orc_absf(off);
    if (!(d < reach)) return 0.0f;
    float flat = orc_absf(ha - hb);
    float full = (ha < hb) ? (float)1.0 / bb : (float)1.0 / aa;
    return (d <= flat) ? full : (reach - d) / (aa * bb);
}

/*
 * Chord of the segment line through a (w x h) rectangle centred at (x, y).
 * Restates the 2-D helper of find_l_3d.cpp:19-92: faces perpendicular to the
 * dominant direction are tried first; the first two hits define the chord.
 */
static float orc_chord_rect(float px, float py, float qx, float qy, float w, float h,
                            float x, float y)
{
    float a = qx - px, b = qy - py;
    float hw = w / 2, hh = h / 2;
    if (a == 0) return (orc_absf(px - x) <= hw) ? h : 0.0f;
    if (b == 0) return (orc_absf(py - y) <= hh) ? w : 0.0f;
    float rx = px - x, ry = py - y;
    float hx[2], hy[2];
    int nh = 0;
    /* families: 0 = faces x = -+hw, 1 = faces y = -+hh */
    int first = (orc_absf(a) > orc_absf(b)) ? 0 : 1;
    for (int pass = 0; pass < 2; pass++) {
        int fam = (pass == 0) ? first : 1 - first;
        if (pass == 1 && nh >= 2) break;
        for (int side = 0; side < 2; side++) {
            if (pass == 1 && side == 1 && nh >= 2) break;
            if (fam == 0) {
                float s = b / a, t = s * (-rx) + ry, u = s * hw;
                float yy = side ? t + u : t - u;
                if (orc_absf(yy) <= hh) { hx[nh] = side ? hw : -hw; hy[nh] = yy; nh++; }
            } else {
                float s = a / b, t = s * (-ry) + rx, u = s * hh;
                float xx = side ? t + u : t - u;
                if (orc_absf(xx) <= hw) { hy[nh] = side ? hh : -hh; hx[nh] = xx; nh++; }
            }
        }
    }
    if (nh != 2) return 0.0f;
    float ex = hx[1] - hx[0], ey = hy[1] - hy[0];
    return (float)sqrt(ex * ex + ey * ey);
}

/*
 * Chord of the line through P=(px,py,pz) and Q=(qx,qy,qz) with the box of
 * size (w,h,t) centred at (x,y,z). Restates find_l_3d (find_l_3d.cpp:94-182):
 * the two face families perpendicular to x and y are tried in order of the
 * dominant xy direction, the z faces last; the first two hits give the chord.
 */
float orc_chord_box(float px, float py, float pz, float qx, float qy, float qz,
                    float w, float h, float t, float x, float y, float z)
{
    float a = qx - px, b = qy - py, c = qz - pz;
    float hw = w / 2, hh = h / 2, ht = t / 2;
    if (a == 0) return orc_chord_rect(py, pz, qy, qz, h, t, y, z);
    if (b == 0) return orc_chord_rect(px, pz, qx, qz, w, t, x, z);
    float rx = px - x, ry = py - y, rz = pz - z;
    float hx[2], hy[2], hz[2];
    int nh = 0;
    /* families: 0 = x faces, 1 = y faces, 2 = z faces */
    int order[3];
    if (orc_absf(a) > orc_absf(b)) { order[0] = 0; order[1] = 1; }
    else                           { order[0] = 1; order[1] = 0; }
    order[2] = 2;
    for (int pass = 0; pass < 3; pass++) {
        if (pass > 0 && nh >= 2) break;
        int fam = order[pass];
        float u0, v0, u1, v1;   /* the two in-face coordinates, centre and half-span */
        float lim0, lim1;
        if (fam == 0) {
            float s = b / a; u0 = s * (-rx) + ry; u1 = s * hw;
            s = c / a;       v0 = s * (-rx) + rz; v1 = s * hw;
            lim0 = hh; lim1 = ht;
        } else if (fam == 1) {
            float s = a / b; u0 = s * (-ry) + rx; u1 = s * hh;
            s = c / b;       v0 = s * (-ry) + rz; v1 = s * hh;
            lim0 = hw; lim1 = ht;
        } else {
            float s = a / c; u0 = s * (-rz) + rx; u1 = s * ht;
            s = b / c;       v0 = s * (-rz) + ry; v1 = s * ht;
            lim0 = hw; lim1 = hh;
        }
        for (int side = 0; side < 2; side++) {
            if (pass > 0 && side == 1 && nh >= 2) break;
            float uu = side ? u0 + u1 : u0 - u1;
            float vv = side ? v0 + v1 : v0 - v1;
            if (orc_absf(uu) <= lim0 && orc_absf(vv) <= lim1) {
                if (fam == 0)      { hx[nh] = side ? hw : -hw; hy[nh] = uu; hz[nh] = vv; }
                else if (fam == 1) { hx[nh] = uu; hy[nh] = side ? hh : -hh; hz[nh] = vv; }
                else               { hx[nh] = uu; hy[nh] = vv; hz[nh] = side ? ht : -ht; }
                nh++;
            }
        }
    }
    if (nh != 2) return 0.0f;
    float ex = hx[1] - hx[0], ey = hy[1] - hy[0], ez = hz[1] - hz[0];
    return (float)sqrt(ex * ex + ey * ey + ez * ez);
}

/*
 * Fan-beam backprojection for image rows [iy0, iy1).
 * Restates Atx_fan_mf_cpu_new (Atx_fan_mf_cpu_new.cpp:21-63).
 */
void orc_fan_adj_f32(float *x, const float *Y, float SO, float OD, float scale, int nx,
                     int ny, int nd, float dy_det, float y_os, int nt, const int *id_Y,
                     const int *Nv, int tmp_size, const float *cos_phi,
                     const float *sin_phi, const float *cos_det, const float *sin_det,
                     int iy0, int iy1)
{
    int nd2 = nd / 2, nx2 = nx / 2, ny2 = ny / 2;
    float SD = SO + OD;
    long n = (long)nx * ny;
    for (int iy = iy0; iy < iy1; iy++) {
        float yc = (float)(iy + 0.5 - ny2);
        for (int ix = 0; ix < nx; ix++) {
            float xc = (float)(ix + 0.5 - nx2);
            for (int it = 0; it < nt; it++) {
                float acc = 0.0f;
                for (int j = 0; j < Nv[it]; j++) {
                    int iv = id_Y[it * tmp_size + j];
                    const float *yv = Y + (long)iv * nd;
                    float c = cos_phi[iv], s = sin_phi[iv];
                    float xr = c * xc + s * yc;
                    float yr = -s * xc + c * yc;
                    float g = SD / ((xr + SO) * dy_det);
                    int hi = (int)floor((yr + 1) * g - y_os + nd2);
                    int lo = (int)floor((yr - 1) * g - y_os + nd2);
                    if (lo < 0) lo = 0;
                    if (hi > nd - 1) hi = nd - 1;
                    for (int id = lo; id <= hi; id++) {
                        float Px = -(sin_det[id] * c + cos_det[id] * s);
                        float Py = cos_det[id] * c - sin_det[id] * s;
                        float Pd = SO * sin_det[id];
                        float l = orc_chord_unit_pixel(Px, Py, Pd, xc, yc);
                        if (l > 0) acc += l * yv[id];
                    }
                }
                x[it * n + (long)iy * nx + ix] = acc * scale;
            }
        }
    }
}

/*
 * One voxel (ix, iy, iz) of frame `it` of the cone-beam chord backprojection:
 * the float operations and their order are those of
 * Atx_cone_mf_cpu_new.cpp:38-81 for that voxel, including its unit-cube chord
 * (it passes voxel size 1,1,1 whatever dz is) and its z window half-width
 * sqrt(1 + dz^2/2).
 */
static float orc_cone_adj_voxel(const float *Y, float SO, float OD, float scale, int nx,
                                int ny, int nz, const float *sd_z, const float *y_det,
                                const float *z_det, float dy_det, float y_os, float dz_det,
                                float dz, const int *id_Y, const int *Nv, int tmp_size,
                                const float *cos_phi, const float *sin_phi, int na, int nb,
                                int ix, int iy, int iz, int it)
{
    float SD = SO + OD;
    int na2 = na / 2, nb2 = nb / 2, nx2 = nx / 2, ny2 = ny / 2, nz2 = nz / 2;
    long nd = (long)na * nb;
    float d = (float)sqrt(1 + dz * dz / 2);
    float zc = (float)(iz + 0.5 - nz2) * dz;
    float yc = (float)(iy + 0.5 - ny2);
    float xc = (float)(ix + 0.5 - nx2);
    float acc = 0.0f;
    for (int j = 0; j < Nv[it]; j++) {
        int iv = id_Y[it * tmp_size + j];
        const float *yv = Y + (long)iv * nd;
        float c = cos_phi[iv], s = sin_phi[iv];
        float xr = c * xc + s * yc;
        float yr = -s * xc + c * yc;
        float g = SD / ((xr + SO) * dy_det);
        int amax = (int)floor((yr + 1) * g - y_os + na2);
        int amin = (int)floor((yr - 1) * g - y_os + na2);
        g = SD / ((xr + SO) * dz_det);
        int bmax = (int)floor((zc + d) * g + nb2);
        int bmin = (int)floor((zc - d) * g + nb2);
        if (amin < 0) amin = 0;
        if (amax > na - 1) amax = na - 1;
        if (bmin < 0) bmin = 0;
        if (bmax > nb - 1) bmax = nb - 1;
        for (int ib = bmin; ib <= bmax; ib++) {
            for (int ia = amin; ia <= amax; ia++) {
                float x1 = c * (-SO), y1 = s * (-SO), z1 = sd_z[iv];
                float x2 = c * OD - s * y_det[ia];
                float y2 = s * OD + c * y_det[ia];
                float z2 = z_det[ib] + sd_z[iv];
                float l = orc_chord_box(x1, y1, z1, x2, y2, z2, 1.0f, 1.0f, 1.0f, xc, yc, zc);
                acc += l * yv[(long)ib * na + ia];
            }
        }
    }
    return acc * scale;
}

/*
 * Cone-beam backprojection for volume slices [iz0, iz1).
 * Restates Atx_cone_mf_cpu_new (Atx_cone_mf_cpu_new.cpp:23-85).
 */
void orc_cone_adj_f32(float *x, const float *Y, float SO, float OD, float scale, int nx,
                      int ny, int nz, const float *sd_z, const float *y_det,
                      const float *z_det, float dy_det, float y_os, float dz_det, float dz,
                      int nt, const int *id_Y, const int *Nv, int tmp_size,
                      const float *cos_phi, const float *sin_phi, int na, int nb, int iz0,
                      int iz1)
{
    long n = (long)nx * ny * nz;
    for (int iz = iz0; iz < iz1; iz++)
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++)
                for (int it = 0; it < nt; it++)
                    x[it * n + ((long)iz * ny + iy) * nx + ix] = orc_cone_adj_voxel(
                        Y, SO, OD, scale, nx, ny, nz, sd_z, y_det, z_det, dy_det, y_os, dz_det,
                        dz, id_Y, Nv, tmp_size, cos_phi, sin_phi, na, nb, ix, iy, iz, it);
}

/*
 * The same backprojection for a list of voxels of frame 0 (index
 * iz*ny*nx + iy*nx + ix); x[k] is voxel vox[k]. Each value is the one
 * orc_cone_adj_f32 writes.
 */
void orc_cone_adj_vox(float *x, const float *Y, float SO, float OD, float scale, int nx,
                      int ny, int nz, const float *sd_z, const float *y_det,
                      const float *z_det, float dy_det, float y_os, float dz_det, float dz,
                      const int *id_Y, const int *Nv, int tmp_size, const float *cos_phi,
                      const float *sin_phi, int na, int nb, const int64_t *vox, long nvx)
{
    for (long k = 0; k < nvx; k++) {
        long v = vox[k];
        int iz = (int)(v / ((long)nx * ny));
        long r = v - (long)iz * nx * ny;
        int iy = (int)(r / nx), ix = (int)(r - (long)iy * nx);
        x[k] = orc_cone_adj_voxel(Y, SO, OD, scale, nx, ny, nz, sd_z, y_det, z_det, dy_det,
                                  y_os, dz_det, dz, id_Y, Nv, tmp_size, cos_phi, sin_phi, na,
                                  nb, ix, iy, iz, 0);
    }
}

/* ------------------------------------------------------------------------- */
/* (2) Exact (FP64) Siddon model                                              */
/* ------------------------------------------------------------------------- */

/*
 * Geometry of one ray in FP64 from the FP32 parameters: source S, detector D.
 * The detector column positions y_det are points on the flat panel
 * (Ax_cone_mf_cpu_siddon.cpp:38-45); an equiangular detector is described by
 * the flat-panel points SD*tan(gamma) of its bins, which define the same rays.
 */
typedef struct {
    int nx, ny, nz;
    double dz;          /* z voxel pitch in xy units */
} orc_grid;

/*
 * Calls visit(ctx, voxel_index, length_in_voxel_units) for every voxel the
 * segment S->D crosses with positive length, in order along the ray.
 * Planes: x = k - nx/2 (k = 0..nx), y likewise, z = (k - nz/2)*dz.
 * Returns the number of voxels visited.
 */
typedef void (*orc_visit_fn)(void *ctx, long vox, double len);

static long orc_exact_walk(const orc_grid *g, const double S[3], const double D[3],
                           orc_visit_fn visit, void *ctx)
{
    int n[3] = {g->nx, g->ny, g->nz};
    double pitch[3] = {1.0, 1.0, g->dz};
    double lo[3], d[3], amin = 0.0, amax = 1.0;
    for (int a = 0; a < 3; a++) {
        lo[a] = -(n[a] / 2) * pitch[a];
        d[a] = D[a] - S[a];
        double hi = lo[a] + n[a] * pitch[a];
        if (d[a] == 0.0) {
            if (S[a] < lo[a] || S[a] >= hi) return 0;
        } else {
            double t0 = (lo[a] - S[a]) / d[a], t1 = (hi - S[a]) / d[a];
            if (t0 > t1) { double tt = t0; t0 = t1; t1 = tt; }
            if (t0 > amin) amin = t0;
            if (t1 < amax) amax = t1;
        }
    }
    if (!(amin < amax)) return 0;
    double len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    /* voxel containing the midpoint of the first step; then step plane by plane */
    int idx[3], step[3];
    double next[3];
    double am = amin;
    for (int a = 0; a < 3; a++) {
        double p = S[a] + (am + 1e-12 * (amax - amin)) * d[a];
        int k = (int)floor((p - lo[a]) / pitch[a]);
        if (k < 0) k = 0;
        if (k >= n[a]) k = n[a] - 1;
        idx[a] = k;
        if (d[a] > 0) {
            step[a] = 1; next[a] = (lo[a] + (k + 1) * pitch[a] - S[a]) / d[a];
        } else if (d[a] < 0) {
            step[a] = -1; next[a] = (lo[a] + k * pitch[a] - S[a]) / d[a];
        } else {
            step[a] = 0; next[a] = INFINITY;
        }
    }
    long count = 0;
    double acur = amin;
    while (acur < amax) {
        int a = 0;
        if (next[1] < next[a]) a = 1;
        if (next[2] < next[a]) a = 2;
        double anext = next[a] < amax ? next[a] : amax;
        double seg = (anext - acur) * len;
        if (seg > 0) {
            long vox = ((long)idx[2] * g->ny + idx[1]) * g->nx + idx[0];
            if (visit) visit(ctx, vox, seg);
            count++;
        }
        acur = anext;
        if (acur >= amax) break;
        idx[a] += step[a];
        if (idx[a] < 0 || idx[a] >= n[a]) break;
        /* next crossing recomputed from the plane index (no drift) */
        int k1 = idx[a] + (step[a] > 0 ? 1 : 0);
        next[a] = (lo[a] + k1 * pitch[a] - S[a]) / d[a];
    }
    return count;
}

typedef struct { const double *x; double acc; } orc_fwd_ctx;
static void orc_fwd_visit(void *c, long vox, double len)
{
    orc_fwd_ctx *f = (orc_fwd_ctx *)c;
    f->acc += len * f->x[vox];
}

typedef struct { double *x; double w; } orc_adj_ctx;
static void orc_adj_visit(void *c, long vox, double len)
{
    orc_adj_ctx *f = (orc_adj_ctx *)c;
    f->x[vox] += len * f->w;
}

static void orc_ray_points(double SO, double OD, double phi, double sz, double ydet,
                           double zdet, double S[3], double D[3])
{
    double c = cos(phi), s = sin(phi);
    S[0] = -SO * c; S[1] = -SO * s; S[2] = sz;
    D[0] = OD * c - ydet * s; D[1] = OD * s + ydet * c; D[2] = zdet + sz;
}

/*
 * Exact cone (nz >= 1; a fan is nz = 1, nb = 1, z_det = {0}, dz = 1) forward
 * projection of views [v0, v1): y = scale * sum(len * x).
 */
void orc_exact_forward_f64(const double *X, double *y, double SO, double OD, double scale,
                           int nx, int ny, int nz, double dz, int v0, int v1,
                           const double *phi, const float *sd_z, int na, int nb,
                           const float *y_det, const float *z_det)
{
    orc_grid g = {nx, ny, nz, dz};
    long nd = (long)na * nb;
    for (int iv = v0; iv < v1; iv++) {
        double sz = sd_z ? (double)sd_z[iv] : 0.0;
        for (int ib = 0; ib < nb; ib++) {
            for (int ia = 0; ia < na; ia++) {
                double S[3], D[3];
                orc_ray_points(SO, OD, phi[iv], sz, (double)y_det[ia],
                               z_det ? (double)z_det[ib] : 0.0, S, D);
                orc_fwd_ctx f = {X, 0.0};
                orc_exact_walk(&g, S, D, orc_fwd_visit, &f);
                y[(long)iv * nd + (long)ib * na + ia] = scale * f.acc;
            }
        }
    }
}

/* Exact transpose: X += scale * sum over rays of views [v0, v1) (len * y). */
void orc_exact_adjoint_f64(double *X, const double *y, double SO, double OD, double scale,
                           int nx, int ny, int nz, double dz, int v0, int v1,
                           const double *phi, const float *sd_z, int na, int nb,
                           const float *y_det, const float *z_det)
{
    orc_grid g = {nx, ny, nz, dz};
    long nd = (long)na * nb;
    for (int iv = v0; iv < v1; iv++) {
        double sz = sd_z ? (double)sd_z[iv] : 0.0;
        for (int ib = 0; ib < nb; ib++) {
            for (int ia = 0; ia < na; ia++) {
                double S[3], D[3];
                orc_ray_points(SO, OD, phi[iv], sz, (double)y_det[ia],
                               z_det ? (double)z_det[ib] : 0.0, S, D);
                orc_adj_ctx f = {X, scale * y[(long)iv * nd + (long)ib * na + ia]};
                orc_exact_walk(&g, S, D, orc_adj_visit, &f);
            }
        }
    }
}

/* Number of voxels crossed with positive length, per ray of views [v0, v1). */
void orc_exact_count(int64_t *cnt, double SO, double OD, int nx, int ny, int nz, double dz,
                     int v0, int v1, const double *phi, const float *sd_z, int na, int nb,
                     const float *y_det, const float *z_det)
{
    orc_grid g = {nx, ny, nz, dz};
    long nd = (long)na * nb;
    for (int iv = v0; iv < v1; iv++) {
        double sz = sd_z ? (double)sd_z[iv] : 0.0;
        for (int ib = 0; ib < nb; ib++) {
            for (int ia = 0; ia < na; ia++) {
                double S[3], D[3];
                orc_ray_points(SO, OD, phi[iv], sz, (double)y_det[ia],
                               z_det ? (double)z_det[ib] : 0.0, S, D);
                cnt[(long)(iv - v0) * nd + (long)ib * na + ia] =
                    orc_exact_walk(&g, S, D, NULL, NULL);
            }
        }
    }
}

/* Exact forward for a list of rays (ray id iv*na*nb + ib*na + ia): y[k] is
 * ray rays[k], as orc_exact_forward_f64 computes it. */
void orc_exact_forward_rays(const double *X, double *y, double SO, double OD, double scale,
                            int nx, int ny, int nz, double dz, const double *phi,
                            const float *sd_z, int na, int nb, const float *y_det,
                            const float *z_det, const int64_t *rays, long nr)
{
    orc_grid g = {nx, ny, nz, dz};
    long nd = (long)na * nb;
    for (long k = 0; k < nr; k++) {
        int iv = (int)(rays[k] / nd);
        long r = rays[k] - (long)iv * nd;
        int ib = (int)(r / na), ia = (int)(r - (long)ib * na);
        double S[3], D[3];
        orc_ray_points(SO, OD, phi[iv], sd_z ? (double)sd_z[iv] : 0.0,
                       (double)y_det[ia], z_det ? (double)z_det[ib] : 0.0, S, D);
        orc_fwd_ctx f = {X, 0.0};
        orc_exact_walk(&g, S, D, orc_fwd_visit, &f);
        y[k] = scale * f.acc;
    }
}

/* Length of the segment S->D inside the box [lo, hi] (FP64 slab method). */
static double orc_box_chord(const double S[3], const double D[3], const double lo[3],
                            const double hi[3])
{
    double t0 = 0.0, t1 = 1.0, len2 = 0.0;
    for (int a = 0; a < 3; a++) {
        double d = D[a] - S[a];
        len2 += d * d;
        if (d == 0.0) {
            if (S[a] < lo[a] || S[a] >= hi[a]) return 0.0;
            continue;
        }
        double u = (lo[a] - S[a]) / d, v = (hi[a] - S[a]) / d;
        if (u > v) { double t = u; u = v; v = t; }
        if (u > t0) t0 = u;
        if (v < t1) t1 = v;
    }
    return t1 > t0 ? (t1 - t0) * sqrt(len2) : 0.0;
}

/* Indices [*i0, *i1] of a monotonic grid g[0..n) whose values lie in [lo, hi],
 * widened by one index on each side (the whole grid when it is not monotonic). */
static void orc_grid_range(const float *g, int n, double lo, double hi, int *i0, int *i1)
{
    int asc = 1, desc = 1;
    if (n > 1) { asc = g[n - 1] >= g[0]; desc = !asc; }
    for (int k = 1; k < n && (asc || desc); k++) {
        if (g[k] < g[k - 1]) asc = 0;
        if (g[k] > g[k - 1]) desc = 0;
    }
    if (!asc && !desc) { *i0 = 0; *i1 = n - 1; return; }
    /* first index whose value is >= lo (ascending) / <= hi (descending) */
    int a = 0, b = n;
    while (a < b) {
        int m = (a + b) / 2;
        int before = asc ? (double)g[m] < lo : (double)g[m] > hi;
        if (before) a = m + 1; else b = m;
    }
    int first = a;
    a = 0; b = n;
    while (a < b) {
        int m = (a + b) / 2;
        int inside_or_before = asc ? (double)g[m] <= hi : (double)g[m] >= lo;
        if (inside_or_before) a = m + 1; else b = m;
    }
    int last = a - 1;
    *i0 = first - 1 < 0 ? 0 : first - 1;
    *i1 = last + 1 > n - 1 ? n - 1 : last + 1;
}

/*
 * Exact transpose for a list of voxels of one frame (index iz*ny*nx + iy*nx +
 * ix) of an FP32 sinogram y: x[k] = scale * sum over the rays of views
 * [v0, v1) of len * y, in FP64, with len the FP64
 * chord of each ray through voxel vox[k]. Per view, only the detector cells
 * inside the projection of the voxel's eight corners (plus one cell on each
 * side) are visited; every other ray misses the voxel. A fan is nz = 1,
 * nb = 1, z_det = {0}, dz = 1.
 */
void orc_exact_adjoint_vox(double *x, const float *y, double SO, double OD, double scale,
                           int nx, int ny, int nz, double dz, int v0, int v1,
                           const double *phi, const float *sd_z, int na, int nb,
                           const float *y_det, const float *z_det, const int64_t *vox,
                           long nvx)
{
    long nd = (long)na * nb;
    double SD = SO + OD;
    for (long k = 0; k < nvx; k++) {
        long v = vox[k];
        int iz = (int)(v / ((long)nx * ny));
        long r = v - (long)iz * nx * ny;
        int iy = (int)(r / nx), ix = (int)(r - (long)iy * nx);
        double lo[3] = {(double)(ix - nx / 2), (double)(iy - ny / 2), (iz - nz / 2) * dz};
        double hi[3] = {lo[0] + 1.0, lo[1] + 1.0, lo[2] + dz};
        double acc = 0.0;
        for (int iv = v0; iv < v1; iv++) {
            double c = cos(phi[iv]), s = sin(phi[iv]);
            double sz = sd_z ? (double)sd_z[iv] : 0.0;
            double umin = INFINITY, umax = -INFINITY, wmin = INFINITY, wmax = -INFINITY;
            for (int q = 0; q < 8; q++) {
                double px = (q & 1) ? hi[0] : lo[0], py = (q & 2) ? hi[1] : lo[1];
                double pz = (q & 4) ? hi[2] : lo[2];
                double depth = SO + c * px + s * py, lat = -s * px + c * py;
                double u = SD * lat / depth, w = SD * (pz - sz) / depth;
                if (u < umin) umin = u;
                if (u > umax) umax = u;
                if (w < wmin) wmin = w;
                if (w > wmax) wmax = w;
            }
            int a0, a1, b0 = 0, b1 = 0;
            orc_grid_range(y_det, na, umin, umax, &a0, &a1);
            if (z_det) orc_grid_range(z_det, nb, wmin, wmax, &b0, &b1);
            for (int ib = b0; ib <= b1; ib++)
                for (int ia = a0; ia <= a1; ia++) {
                    double S[3], D[3];
                    orc_ray_points(SO, OD, phi[iv], sz, (double)y_det[ia],
                                   z_det ? (double)z_det[ib] : 0.0, S, D);
                    double l = orc_box_chord(S, D, lo, hi);
                    if (l > 0.0) acc += l * (double)y[(long)iv * nd + (long)ib * na + ia];
                }
        }
        x[k] = scale * acc;
    }
}

/* ------------------------------------------------------------------------- */
/* (1c) Dominant-axis forward projector (version 1), FP32, reference arithmetic */
/* ------------------------------------------------------------------------- */

/*
 * One slab of the dominant-axis walk: the ray crosses the slab between
 * secondary coordinates [p1, p2] (grid units, p1 <= p2) and, in 3-D, z
 * coordinates [q1, q2]; it touches at most two voxels along each secondary
 * axis. Restates the case analysis of Ax_cone_mf_cpu_new.cpp:77-155 (cases
 * 11, 12, 21, 22); `vox(s, z)` maps secondary and z cell to a voxel pointer.
 */
typedef struct { const float *x; long sstride, zstride, base; } orc_gao_vox;

static float orc_gao_slab(float acc, float p1, float p2, float q1, float q2, float l, int ns,
                          int nz, const orc_gao_vox *V)
{
    int c1 = (int)floor(p1), c2 = (int)floor(p2);
    int k1 = (int)floor(q1), k2 = (int)floor(q2);
#define VOX(s, z) (V->x[V->base + (long)(z) * V->zstride + (long)(s) * V->sstride])
    if (c2 == c1) {
        if (c1 >= 0 && c1 <= ns - 1) {
            if (k2 == k1) {
                if (k1 >= 0 && k1 <= nz - 1) acc += l * VOX(c1, k1);
            } else if (k1 >= -1 && k1 <= nz - 1) {
                float rz = (k2 - q1) / (q2 - q1);
                if (k1 > -1) acc += rz * l * VOX(c1, k1);
                if (k2 < nz) acc += (1 - rz) * l * VOX(c1, k2);
            }
        }
    } else if (c1 >= -1 && c1 <= ns - 1) {
        float d = p2 - p1;
        if (k2 == k1) {
            if (k1 >= 0 && k1 <= nz - 1) {
                float rs = (c2 - p1) / d;
                if (c1 > -1) acc += rs * l * VOX(c1, k1);
                if (c2 < ns) acc += (1 - rs) * l * VOX(c2, k1);
            }
        } else if (k1 >= -1 && k1 <= nz - 1) {
            float rs = (c2 - p1) / d, rz = (k2 - q1) / (q2 - q1);
            if (rs > rz) {
                if (c1 > -1 && k1 > -1) acc += rz * l * VOX(c1, k1);
                if (c1 > -1 && k2 < nz) acc += (rs - rz) * l * VOX(c1, k2);
                if (c2 < ns && k2 < nz) acc += (1 - rs) * l * VOX(c2, k2);
            } else {
                if (c1 > -1 && k1 > -1) acc += rs * l * VOX(c1, k1);
                if (c2 < ns && k1 > -1) acc += (rz - rs) * l * VOX(c2, k1);
                if (c2 < ns && k2 < nz) acc += (1 - rz) * l * VOX(c2, k2);
            }
        }
    }
#undef VOX
    return acc;
}

/*
 * Cone-beam dominant-axis projection with its normalised twin, views [v0, v1).
 * Restates Ax_cone_mf_cpu_new (Ax_cone_mf_cpu_new.cpp:23-235) and its norm3
 * helper (:19-20: a double sqrt, since pow(float, int) promotes, returned as
 * float).
 */
void orc_cone_gao_f32(const float *X, float *y, float *yNorm, float SO, float OD, float scale,
                      int nx, int ny, int nz, int v0, int v1, const float *sd_phi,
                      const float *sd_z, int na, int nb, const float *y_det, const float *z_det,
                      const int *id_X, float dz)
{
    int nx2 = nx / 2, ny2 = ny / 2, nz2 = nz / 2;
    long n = (long)nx * ny * nz, nd = (long)na * nb;
    for (int iv = v0; iv < v1; iv++) {
        float cphi = cosf(sd_phi[iv]), sphi = sinf(sd_phi[iv]);
        float x1 = cphi * (-SO), y1 = sphi * (-SO), z1 = sd_z[iv];
        for (int ib = 0; ib < nb; ib++) {
            for (int ia = 0; ia < na; ia++) {
                float x2 = cphi * OD - sphi * y_det[ia];
                float y2 = sphi * OD + cphi * y_det[ia];
                float z2 = z_det[ib] + sd_z[iv];
                /* norm3 returns float: sqrt in double (pow(float, int) promotes), rounded
                   to float on return, then scaled in float */
                double ex = (double)(x1 - x2), ey = (double)(y1 - y2), ez = (double)(z1 - z2);
                float norm = (float)sqrt(ex * ex + ey * ey + ez * ez) * scale;
                float tmp = (x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2);
                float zz = (z1 - z2) * (z1 - z2);
                float acc = 0.0f;
                orc_gao_vox V;
                V.x = X + (long)id_X[iv] * n;
                V.zstride = (long)nx * ny;
                if (orc_absf(x1 - x2) > orc_absf(y1 - y2)) {
                    float s1 = (y2 - y1) / (x2 - x1), s2 = (z2 - z1) / (x2 - x1);
                    V.sstride = nx;
                    for (int ix = 0; ix < nx; ix++) {
                        float a1 = (float)(ix - nx2), a2 = a1 + 1;
                        float p1, p2, q1, q2;
                        if (s1 >= 0) { p1 = y1 + s1 * (a1 - x1) + ny2; p2 = y1 + s1 * (a2 - x1) + ny2; }
                        else         { p1 = y1 + s1 * (a2 - x1) + ny2; p2 = y1 + s1 * (a1 - x1) + ny2; }
                        if (s2 >= 0) { q1 = (z1 + s2 * (a1 - x1)) / dz + nz2; q2 = (z1 + s2 * (a2 - x1)) / dz + nz2; }
                        else         { q1 = (z1 + s2 * (a2 - x1)) / dz + nz2; q2 = (z1 + s2 * (a1 - x1)) / dz + nz2; }
                        float d = p2 - p1;
                        float l = sqrtf((d * d + 1) * (tmp + zz) / tmp);
                        V.base = ix;
                        acc = orc_gao_slab(acc, p1, p2, q1, q2, l, ny, nz, &V);
                    }
                } else {
                    float s1 = (x2 - x1) / (y2 - y1), s2 = (z2 - z1) / (y2 - y1);
                    V.sstride = 1;
                    for (int iy = 0; iy < ny; iy++) {
                        float a1 = (float)(iy - ny2), a2 = a1 + 1;
                        float p1, p2, q1, q2;
                        if (s1 >= 0) { p1 = x1 + s1 * (a1 - y1) + nx2; p2 = x1 + s1 * (a2 - y1) + nx2; }
                        else         { p1 = x1 + s1 * (a2 - y1) + nx2; p2 = x1 + s1 * (a1 - y1) + nx2; }
                        if (s2 >= 0) { q1 = (z1 + s2 * (a1 - y1)) / dz + nz2; q2 = (z1 + s2 * (a2 - y1)) / dz + nz2; }
                        else         { q1 = (z1 + s2 * (a2 - y1)) / dz + nz2; q2 = (z1 + s2 * (a1 - y1)) / dz + nz2; }
                        float d = p2 - p1;
                        float l = sqrtf((d * d + 1) * (tmp + zz) / tmp);
                        V.base = (long)iy * nx;
                        acc = orc_gao_slab(acc, p1, p2, q1, q2, l, nx, nz, &V);
                    }
                }
                acc = acc * scale;
                y[(long)iv * nd + (long)ib * na + ia] = acc;
                yNorm[(long)iv * nd + (long)ib * na + ia] = acc / norm;
            }
        }
    }
}

/*
 * Fan-beam dominant-axis projection, views [v0, v1). Restates
 * Ax_fan_mf_cpu_new (Ax_fan_mf_cpu_new.cpp:18-122), including its y-dominant
 * edge test against ny where nx is meant (:111; equal for square images).
 */
void orc_fan_gao_f32(const float *X, float *y, float SO, float OD, float scale, int nx, int ny,
                     int v0, int v1, const float *sd_phi, int nd, const float *y_det,
                     const int *id_X)
{
    int nx2 = nx / 2, ny2 = ny / 2;
    long n = (long)nx * ny;
    for (int iv = v0; iv < v1; iv++) {
        const float *x = X + (long)id_X[iv] * n;
        float cphi = cosf(sd_phi[iv]), sphi = sinf(sd_phi[iv]);
        float x1 = cphi * (-SO), y1 = sphi * (-SO);
        for (int id = 0; id < nd; id++) {
            float x2 = cphi * OD - sphi * y_det[id];
            float y2 = sphi * OD + cphi * y_det[id];
            float acc = 0.0f;
            int xdom = orc_absf(x1 - x2) > orc_absf(y1 - y2);
            float s = xdom ? (y2 - y1) / (x2 - x1) : (x2 - x1) / (y2 - y1);
            float pa = xdom ? x1 : y1, pb = xdom ? y1 : x1;   /* primary, secondary start */
            int np = xdom ? nx : ny, ns = xdom ? ny : nx;
            int np2 = xdom ? nx2 : ny2, ns2 = xdom ? ny2 : nx2;
            int nedge = ny;                                     /* the reference's `c2==ny` */
            for (int ip = 0; ip < np; ip++) {
                float a1 = (float)(ip - np2), a2 = a1 + 1;
                float p1, p2;
                if (s >= 0) { p1 = pb + s * (a1 - pa) + ns2; p2 = pb + s * (a2 - pa) + ns2; }
                else        { p1 = pb + s * (a2 - pa) + ns2; p2 = pb + s * (a1 - pa) + ns2; }
                int c1 = (int)floor(p1), c2 = (int)floor(p2);
#define PIX(c) (xdom ? x[(long)(c) * nx + ip] : x[(long)ip * nx + (c)])
                if (c2 == c1) {
                    if (c1 >= 0 && c1 <= ns - 1) {
                        float d = p2 - p1, l = sqrtf(d * d + 1);
                        acc += l * PIX(c1);
                    }
                } else if (c2 > 0 && c2 < ns) {
                    float d = p2 - p1, l = sqrtf(d * d + 1);
                    /* c1 < 0 (crossings rounded more than a pixel apart): the
                       reference reads outside the image here; the term is skipped */
                    if (c1 >= 0) acc += ((c2 - p1) / d) * l * PIX(c1);
                    acc += ((p2 - c2) / d) * l * PIX(c2);
                } else {
                    if (c2 == 0) {
                        float d = p2 - p1, l = sqrtf(d * d + 1);
                        acc += ((p2 - c2) / d) * l * PIX(c2);
                    }
                    if (c2 == (xdom ? ny : nedge) && c1 >= 0 && c1 < ns) {
                        float d = p2 - p1, l = sqrtf(d * d + 1);
                        acc += ((c2 - p1) / d) * l * PIX(c1);
                    }
                }
#undef PIX
            }
            y[(long)iv * nd + id] = acc * scale;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* (1d) Finite-size beam fan projector pair (version 2), FP32 reference arithmetic */
/* ------------------------------------------------------------------------- */

/* Area of the unit pixel at (x, y) on one side of the line a*x + b*y = c,
   measured from the line (half-plane split), as find_area.cpp:18-70 computes
   it for each beam edge; returns the area and the side (+1 / -1). */
static float orc_edge_area(float a, float b, float c, float x, float y, int *sgn)
{
    float aa = orc_absf(a), bb = orc_absf(b);
    float hx = aa / 2, hy = bb / 2;
    float reach = hx + hy;
    float off = c - a * x - b * y;
    float d = orc_absf(off);
    *sgn = off > 0 ? 1 : -1;
    if (!(d < reach)) return (float)0.5;
    float flat = orc_absf(hx - hy);
    float inv = (hx < hy) ? (float)1.0 / bb : (float)1.0 / aa;
    if (d <= flat) return d * inv;
    return (float)0.5 - (float)0.5 * (reach - d) * (reach - d) / (aa * bb);
}

/* find_area (find_area.cpp:18-70): pixel area between two beam edges. */
float orc_beam_area(float a1, float b1, float c1, float a2, float b2, float c2, float x,
                    float y)
{
    int s1, s2;
    float A1 = orc_edge_area(a1, b1, c1, x, y, &s1);
    float A2 = orc_edge_area(a2, b2, c2, x, y, &s2);
    float t = A1 - (float)(s1 * s2) * A2;
    return orc_absf(t);
}

/*
 * Finite-beam fan projection of views [v0, v1). Restates Ax_fan_mf_cpu_new_fb
 * (Ax_fan_mf_cpu_new_fb.cpp:19-123), including its candidate-row bounds that
 * keep only in-range crossings (a beam half outside the image may skip rows)
 * and its float trigonometry of the edge angles. Where a beam edge is exactly
 * parallel to the walked axis and the pixel centre is farther than 0.5 the
 * reference reads bounds it never set; that degenerate case is empty here.
 */
void orc_fan_fb_f32(const float *X, float *y, float SO, float OD, float scale, int nx, int ny,
                    int v0, int v1, const float *sd_phi, int nd, const float *y_det,
                    const int *id_X, float dy_det)
{
    int nx2 = nx / 2, ny2 = ny / 2;
    long n = (long)nx * ny;
    float SD = SO + OD;
    for (int iv = v0; iv < v1; iv++) {
        const float *x = X + (long)id_X[iv] * n;
        float cphi = cosf(sd_phi[iv]), sphi = sinf(sd_phi[iv]);
        float x1 = cphi * (-SO), y1 = sphi * (-SO);
        for (int id = 0; id < nd; id++) {
            float x2[2], y2[2], Px[2], Py[2], Pd[2];
            for (int e = 0; e < 2; e++) {
                float u = e ? y_det[id] + dy_det / 2 : y_det[id] - dy_det / 2;
                x2[e] = cphi * OD - sphi * u;
                y2[e] = sphi * OD + cphi * u;
                float ang = atan2f(u, SD);
                Px[e] = -sinf(ang + sd_phi[iv]);
                Py[e] = cosf(ang + sd_phi[iv]);
                Pd[e] = SO * sinf(ang);
            }
            float acc = 0.0f;
            int xdom = orc_absf(x1 - (x2[0] + x2[1]) / 2) > orc_absf(y1 - (y2[0] + y2[1]) / 2);
            float p1 = xdom ? x1 : y1, q1 = xdom ? y1 : x1;        /* walked, other */
            float pe0 = xdom ? x2[0] : y2[0], pe1 = xdom ? x2[1] : y2[1];
            float qe0 = xdom ? y2[0] : x2[0], qe1 = xdom ? y2[1] : x2[1];
            int np = xdom ? nx : ny, nq = xdom ? ny : nx;
            int np2 = xdom ? nx2 : ny2, nq2 = xdom ? ny2 : nx2;
            int degen = !(pe0 != p1 && pe1 != p1);
            float s0 = 0, s1 = 0;
            if (!degen) { s0 = (qe0 - q1) / (pe0 - p1); s1 = (qe1 - q1) / (pe1 - p1); }
            for (int ip = 0; ip < np; ip++) {
                float pc = (float)(ip + 0.5 - np2);
                float a1 = (float)(ip - np2), a2 = a1 + 1;
                int qmin, qmax;
                if (degen) {
                    if (orc_absf(p1 - pc) <= 0.5) { qmin = 0; qmax = nq - 1; }
                    else { qmin = 1; qmax = 0; }
                } else {
                    int c[4];
                    c[0] = (int)floor(q1 + s0 * (a1 - p1) + nq2);
                    c[1] = (int)floor(q1 + s0 * (a2 - p1) + nq2);
                    c[2] = (int)floor(q1 + s1 * (a1 - p1) + nq2);
                    c[3] = (int)floor(q1 + s1 * (a2 - p1) + nq2);
                    qmin = nq - 1; qmax = 0;
                    for (int k = 0; k < 4; k++) {
                        if (c[k] < qmin && c[k] >= 0) qmin = c[k];
                        if (c[k] > qmax && c[k] <= nq - 1) qmax = c[k];
                    }
                }
                for (int iq = qmin; iq <= qmax; iq++) {
                    float qc = (float)(iq + 0.5 - nq2);
                    float xc = xdom ? pc : qc, yc = xdom ? qc : pc;
                    float l = orc_beam_area(Px[0], Py[0], Pd[0], Px[1], Py[1], Pd[1], xc, yc);
                    if (l > 0) acc += l * (xdom ? x[(long)iq * nx + ip] : x[(long)ip * nx + iq]);
                }
            }
            y[(long)iv * nd + id] = acc * scale;
        }
    }
}

/*
 * Finite-beam fan backprojection for image rows [iy0, iy1). Restates
 * Atx_fan_mf_cpu_new_fb (Atx_fan_mf_cpu_new_fb.cpp:20-66); cos_det/sin_det hold
 * the nd + 1 bin-edge angles (the gateway's cos_det2/sin_det2).
 */
void orc_fan_fb_adj_f32(float *x, const float *Y, float SO, float OD, float scale, int nx,
                        int ny, int nd, float dy_det, int nt, const int *id_Y, const int *Nv,
                        int tmp_size, const float *cos_phi, const float *sin_phi,
                        const float *cos_det, const float *sin_det, int iy0, int iy1)
{
    int nd2 = nd / 2, nx2 = nx / 2, ny2 = ny / 2;
    float SD = SO + OD;
    long n = (long)nx * ny;
    for (int iy = iy0; iy < iy1; iy++) {
        float yc = (float)(iy + 0.5 - ny2);
        for (int ix = 0; ix < nx; ix++) {
            float xc = (float)(ix + 0.5 - nx2);
            for (int it = 0; it < nt; it++) {
                float acc = 0.0f;
                for (int j = 0; j < Nv[it]; j++) {
                    int iv = id_Y[it * tmp_size + j];
                    const float *yv = Y + (long)iv * nd;
                    float c = cos_phi[iv], s = sin_phi[iv];
                    float xr = c * xc + s * yc;
                    float yr = -s * xc + c * yc;
                    float g = SD / ((xr + SO) * dy_det);
                    int hi = (int)floor((yr + 1) * g + nd2);
                    int lo = (int)floor((yr - 1) * g + nd2);
                    if (lo < 0) lo = 0;
                    if (hi > nd - 1) hi = nd - 1;
                    for (int id = lo; id <= hi; id++) {
                        float Px0 = -(sin_det[id] * c + cos_det[id] * s);
                        float Py0 = cos_det[id] * c - sin_det[id] * s;
                        float Pd0 = SO * sin_det[id];
                        float Px1 = -(sin_det[id + 1] * c + cos_det[id + 1] * s);
                        float Py1 = cos_det[id + 1] * c - sin_det[id + 1] * s;
                        float Pd1 = SO * sin_det[id + 1];
                        float l = orc_beam_area(Px0, Py0, Pd0, Px1, Py1, Pd1, xc, yc);
                        if (l > 0) acc += l * yv[id];
                    }
                }
                x[it * n + (long)iy * nx + ix] = acc * scale;
            }
        }
    }
}
