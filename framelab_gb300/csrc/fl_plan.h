// fl_plan.h -- internal layout of an fl_plan (geometry uploaded to HBM).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "framelab_gb300.h"

// Per-ray parameters of the matched Siddon model, one AxisEntry per axis.
// The ray crosses plane k of an axis (x, y: planes at k - n/2; z: planes at
// (k - nz/2)*dz) at A(k) = alpha(k) - alpha_c(view), the source->detector
// parameter measured from the isocentre crossing, with
//     A(k) = (k - kq) * (ih + il) + c,
// where kq is a quantised plane coordinate of the ray's isocentre crossing
// (its quantum makes k - kq exact in FP32 for every plane the kernels use),
// ih + il the FP64 pitch/d rounded to a pair of floats and c the rest of
// the quantisation. Built in FP64 on the host, rounded once per field.
//
// The kernels never use an A(k) on its own: a ray's path is cut into
// segments of 2^SH planes of its dominant xy axis (the one with the
// smaller |ih|), and within segment s every crossing is taken relative to
// the anchor B_s = A_D(kA) of the dominant axis D at the segment's middle
// plane kA, held as bh + be (make_anchor, matched_dev.cuh):
//     t(k) = fma(m, ih, -bh) + fma(m, il, c - be),   m = k - kq.
// t is a small number (a few voxels of path), so the difference of two
// crossings -- the weight -- carries FP32 rounding of t, not of A: the
// weight's relative error stays near 1e-7 whatever the size of the volume.
// The forward walk and the backprojection gather evaluate this same
// expression from the same table entries, so both see identical crossings.
// 16- and 32-byte aligned, so each entry is read with vector loads
struct alignas(16) AxisEntry {
    float kq, ih, il, c;
};
struct alignas(32) ColEntry {   // per (view, detector column): x and y axes
    AxisEntry x, y;
};
struct alignas(32) RowEntry {   // per (view, detector row): z axis (cone only)
    AxisEntry z;
    float dz2;        // fl(d_z^2), for c_r
    float pad[3];
};
struct ViewEntry {  // per view, for the adjoint's detector windows
    float c, s;       // cos/sin of the source angle
    float sz;         // source z
    float ac;         // alpha_c: A = alpha - ac
};

struct fl_plan {
    fl_scan s;                 // scalar fields; array pointers below are device copies
    int tmp_size;
    int64_t n_vox_frame, n_vox, n_rays;
    // reference geometry (device)
    float *d_sd_phi, *d_sd_z, *d_y_det, *d_z_det;
    float *d_cos_phi, *d_sin_phi, *d_cos_det, *d_sin_det;
    float *d_cphi_f, *d_sphi_f;    // cosf/sinf(sd_phi): the reference Siddon's own trig
    float *d_cos_det2, *d_sin_det2; // [na+1] bin-edge trig (finite-beam backprojector)
    float *d_fb_edges;             // [nv*na*6] finite-beam edge lines (Px, Py, Pd) x 2
    int32_t *d_view_frame, *d_idY, *d_Nv;
    // matched-model tables (device); rows nv and nv + 1 (two extra views) hold
    // view nv/8 at the exact angle pi/4 and view nv/4 at the exact angle pi/2
    // for the reflection forms
    ColEntry *d_col;           // [(nv+2)*na]
    float *d_colr;             // [(nv+2)*na] fl(d_x^2 + d_y^2)
    RowEntry *d_row;           // [(nv+2)*nb]
    AxisEntry *d_rowz;         // [(nv+2)*nb] z axes: the backprojector's 16-byte copy
    ViewEntry *d_view;         // [nv+2]
    // detector grid for the adjoint windows (matched model)
    int det_kind;              // 0 flat uniform, 1 equiangular (fan), -1 irregular
    float u0, du, g0, dg;      // flat: u = u0 + ia*du ; arc: gamma = g0 + ia*dg
    float v0, dv;              // rows: v = v0 + ib*dv
    float SD;
    // z-mirror symmetry: with the source in the volume's central plane for
    // every view (sd_z = 0), an even nz, an even nb and z_det exactly
    // antisymmetric (z_det[nb-1-ib] == -z_det[ib], z_det[0] < 0), the ray of
    // row nb-1-ib is the mirror image of the ray of row ib. The matched model
    // then defines A[(v, a, nb-1-b), (x, y, nz-1-z)] = A[(v, a, b), (x, y, z)]
    // for b < nb/2, so one walk / one weight serves both rays.
    int zmirror_ok;            // the geometry allows it
    int zmirror;               // in use (FL_OPT_Z_MIRROR)
    // half-turn symmetry on top of the z mirror: one frame, an even number of
    // views with view v + nv/2 opposite view v (sources and detector turned by
    // pi about the z axis), nx and ny multiples of 4. The matched model then defines
    // A[(v + nv/2, a, b), (nx-1-x, ny-1-y, z)] = A[(v, a, b), (x, y, z)] for
    // v < nv/2 (with c_r of view v), so one walk / one weight serves four
    // rays: rows b and nb-1-b of views v and v + nv/2.
    int rot_ok;                // the geometry allows it
    int rot;                   // in use (FL_OPT_ROT_MIRROR; only with zmirror)
    // quarter turn on top of the half turn: nx == ny, nv a multiple of 4 and
    // view v + nv/4 view v turned by pi/2. The matched model then defines
    // A[(v + j nv/4, a, b), R^j (x, y, z)] = A[(v, a, b), (x, y, z)] for
    // v < nv/4, j = 1..3, R (x, y) = (n-1-y, x), so one walk / one weight
    // serves eight rays (views v + j nv/4, rows b and nb-1-b).
    int rot4_ok;
    int rot4;                  // in use (FL_OPT_QUARTER_TURN; only with rot and zmirror)
    // reflection on top of the half or the quarter turn (cone plans): view nv
    // - v the mirror image of view v about the x axis (to within 1e-6), view 0
    // at angle 0 and a detector symmetric about its centre (y_det[na-1-a] ==
    // -y_det[a] exactly, na even). With M (x, y) = (x, ny-1-y) and S = R (the
    // quarter turn, NR = 4 rotations; nv a multiple of 8) or S = R^2 (the half
    // turn, NR = 2), the matched model defines, for the walked views v = 0 ..
    // ov (ov = nv/8, or floor(nv/4)),
    //   A[(v + j nv/NR, a, b), S^j V] = A[(j nv/NR - v, na-1-a, b), S^j M V]
    //     = A[(v, a, b), V],
    // so one walk / one weight serves 4 NR rays (the symmetries of the square,
    // or of the rectangle, times the z mirror). View 0, and view ov where it
    // is its own mirror image (NR = 4; NR = 2 with nv a multiple of 4), walk
    // their columns a < na/2 only, the other half being their mirror images;
    // view ov is then walked from table row nv (NR = 4: the exact diagonal
    // angle pi/4) or nv + 1 (NR = 2: the exact angle pi/2), so the scan the
    // plan projects has every view at an angle of its orbit.
    int refl4_ok, refl2_ok;    // the geometry allows it with the quarter / half turn
    int refl;                  // wanted (FL_OPT_REFLECT); used where the turn in use allows
    // fan plans take both turns without a mirror: the half turn with ny even,
    // the quarter turn with nx == ny even (A[(v + j nv/G, a), R^j (x, y)] =
    // A[(v, a), (x, y)], one walk / one weight serving G rays), and the
    // reflection with either (one walk / weight serving 2 G rays; the quarter
    // turns with nv a multiple of 8) or alone for odd view counts (two rays:
    // S = identity, walked views 0 .. (nv-1)/2; FanReflGeom in matched_dev.cuh)
    int refl1_ok;              // fan: the reflection alone (odd nv)
    // Every turn form needs one frame whose view list is 0, 1, ..., nv-1.
    int views_natural;
    // launch shapes (threads in x and y, x * y = 128) of the cone projector
    // kernels; 0 keeps each kernel's built-in shape (set by fl_plan_autotune;
    // every thread's result is independent of the shape)
    int fwd_bx, fwd_by, adj_bx, adj_by;
    // voxels per thread of the reflection backprojection (1 or 2; 0 = 2) and
    // its row loop: 1 or 2 rows per iteration, 3 one pass over the run's rows
    // (runs of 2; 0 = 1)
    int adj_run, adj_rows;
    // launches over consecutive view chunks of the reflection backprojection
    // (FP32 output; 0 or 1: one launch), and the diagonal columns'
    // second sums between them ((nx/2) (nz/2) 4 float2, allocated with
    // quarter-turn reflection plans)
    int adj_chunks;
    float2 *d_dq;
    // fan plans: parts per walked ray of the turn forward (1, 4 or 16; 0 =
    // the scan's default, fl_plan_fan_lanes) and pixels per thread side of
    // the backprojections (1 or 2; 0 = 2 once there are 4 waves of blocks)
    int fan_lanes, fan_block;
    // fan plans: view groups of the turn and reflection backprojections (8
    // or 16; 0 = 8)
    int fan_groups;
    // scale of an FP16 backprojection input (the mixed CGLS form): the largest
    // power of two with y16_scale * c_r^2 <= 1 for every ray, so c_r^2 * (a
    // ray's sum of w p) stays within FP16's range whenever |p| does
    float y16_scale;
    // reusable scratch: sinogram-sized f32 for the pre-weighted adjoint input,
    // volume-sized for the z-folded copy of a forward input
    float *d_work;
    size_t work_elems;
    void *d_vwork;
    size_t vwork_bytes;
    // fan plans: the forward's transposed copy of its input (n_vox elements
    // of up to 4 bytes; allocated with the plan), made by TMA where possible
    // (fan_tma.cu; FL_TUNE_FAN_TMA, default on) with its timeout flag
    void *d_xt;
    int fan_tma_ok;
    int *d_tma_err;
    int tma_stall;   // FL_DEBUG_TMA_STALL (tests): polls of a wait nothing ends
};

// The matched kernel form a plan uses (its options within what its geometry
// allows). A cone plan's turn forms also need the z mirror.
enum {
    FL_FORM_GENERAL = 0,      // general kernels (fan: no turn; cone: no mirror)
    FL_FORM_MIRROR,           // cone: z mirror
    FL_FORM_HALF,             // half turn (cone: with the z mirror)
    FL_FORM_QUARTER,          // quarter turns (cone: with the z mirror)
    FL_FORM_HALF_REFL,        // half turn and reflection (cone: with the z mirror)
    FL_FORM_QUARTER_REFL,     // quarter turns and reflection (cone: with the z mirror)
    FL_FORM_REFL              // fan: the reflection alone (odd nv)
};

inline int fl_plan_form(const fl_plan* p)
{
    if (p->s.ndim == 3 && !p->zmirror) return FL_FORM_GENERAL;
    if (!p->rot) {
        if (p->s.ndim == 3) return FL_FORM_MIRROR;
        return (p->refl && p->refl1_ok) ? FL_FORM_REFL : FL_FORM_GENERAL;
    }
    if (p->rot4) return (p->refl && p->refl4_ok) ? FL_FORM_QUARTER_REFL : FL_FORM_QUARTER;
    return (p->refl && p->refl2_ok) ? FL_FORM_HALF_REFL : FL_FORM_HALF;
}

// Views one walk or weight of the matched kernels in use serves: 8 (quarter
// turns and the reflection), 4 (quarter turns, or the half turn and the
// reflection), 2 (half turn, or the reflection alone) or 1.
inline int fl_plan_turns(const fl_plan* p)
{
    switch (fl_plan_form(p)) {
    case FL_FORM_QUARTER_REFL: return 8;
    case FL_FORM_QUARTER: case FL_FORM_HALF_REFL: return 4;
    case FL_FORM_HALF: case FL_FORM_REFL: return 2;
    default: return 1;
    }
}

// Rotations of a reflection form (4, 2, or 1 for the fan's reflection
// alone), or 0.
inline int fl_plan_refl(const fl_plan* p)
{
    switch (fl_plan_form(p)) {
    case FL_FORM_QUARTER_REFL: return 4;
    case FL_FORM_HALF_REFL: return 2;
    case FL_FORM_REFL: return 1;
    default: return 0;
    }
}

// Layouts of the matched launchers' operands. For a z-mirror plan the
// z-folded volume stores, per frame, the pairs (voxel (ix, iy, iz),
// voxel (ix, iy, nz-1-iz)) for iz < nz/2 at pair index (iz*ny + iy)*nx + ix;
// the adjoint input (pre-weighted sinogram) is always folded the same way:
// pairs (row ib, row nb-1-ib) for ib < nb/2 at pair index (iv*nb/2 + ib)*na + ia,
// except on a half- (G = 2) or quarter-turn (G = 4) plan, where the 2 G values
// of views iv + j nv/G (j < G), rows ib and nb-1-ib, lie side by side at
// 2 G ((iv*nb/2 + ib)*na + ia) + 2 j for iv < nv/G. A reflection form packs
// the 4 NR values of a walked ray's orbit in two planes of nv*nb*na/2 values
// (the turn images' rows, then the reflected images'; ReflGeom in
// matched_dev.cuh), exactly nv*nb*na values in all. A fan plan with turns
// (G = 2 or 4) packs the G values of views iv + j nv/G side by side at
// G (iv*na + ia) + j.
// A half- or quarter-turn plan's folded volume is tiled in xy: the pair of
// voxel (x, y, z < nz/2) is at z*nx*ny + 16*((y/4)*(nx/4) + x/4) + 4*(y%4) +
// x%4, so one 128-byte line holds a 4 x 4 patch of pairs (the gathers of a
// warp's neighbouring rays share lines whatever the ray direction).
// For other plans both layouts are the standard ones.
enum {
    FL_LAY_X_FOLDED = 1,   // the volume operand is z-folded
    FL_LAY_Y_ADJ = 2       // the forward writes the adjoint-input layout
};

// Parts per walked ray of a fan turn plan's forward: the plan's setting
// (FL_TUNE_FAN_PARTS), else 16 for scans of fewer than 65,536 walks and 1
// above (a batch takes its slices' values when it is built).
int fl_plan_fan_lanes(const fl_plan* p);
// Pixels per thread side of a fan plan's backprojection (1 or 2): the plan's
// setting (FL_TUNE_FAN_BLOCK), else 2 once the 2 x 2 blocks make four waves
// of thread blocks on 152 SMs.
int fl_plan_fan_block(const fl_plan* p);
// View groups of a fan plan's turn and reflection backprojections (8 or 16):
// the plan's setting (FL_TUNE_FAN_GROUPS), else 8.
int fl_plan_fan_groups(const fl_plan* p);
// View chunks of a cone plan's reflection backprojection: the plan's setting
// (FL_TUNE_ADJ_CHUNKS) where the output is FP32, else 1.
int fl_plan_adj_chunks(const fl_plan* p, bool f32_out);

// The fan forward's transposed copy of x by TMA (fan_tma.cu): false, with
// nothing launched, where the plan, the input address or the row sizes do
// not allow it.
bool fl_fan_transpose_tma(fl_plan* p, const void* x, int dtype, cudaStream_t st);
bool fl_tma_available();
// FL_ERR_TIMEOUT (and the flag cleared) if a TMA tile load of one of the
// plan's forwards gave up its bounded wait since the last check; reads the
// flag after synchronising the stream. FL_OK for plans without the flag.
int fl_plan_take_timeouts(fl_plan* p, cudaStream_t s);

// internal launchers
int fl_ref_forward(fl_plan* p, const float* x, float* y, cudaStream_t st);
int fl_ref_adjoint(fl_plan* p, const float* y, float* x, cudaStream_t st);
int fl_ref_gao_forward(fl_plan* p, const float* x, float* y, float* ynorm, cudaStream_t st);
int fl_ref_fb_forward(fl_plan* p, const float* x, float* y, cudaStream_t st);
int fl_ref_fb_adjoint(fl_plan* p, const float* y, float* x, cudaStream_t st);
// skip: optional device flag; when *skip != 0 the kernels return at once
// (lets a captured CGLS iteration become a no-op after convergence).
// xscale: optional device factor applied to the gathered sum (scaled storage).
int fl_matched_forward(fl_plan* p, const void* x, int xt, void* y, int yt, int cr_power,
                       const int* skip, const float* xscale, int layout, cudaStream_t st);
// yw (adjoint-input layout) = c_r * y (standard layout)
int fl_matched_weight(fl_plan* p, const void* y, int yt, float* yw, cudaStream_t st);
int fl_matched_adjoint_w(fl_plan* p, const float* yw, void* x, int xt, const int* skip,
                         int layout, cudaStream_t st);
// the same with the input in FP32 or (cone plans) FP16, wt = FL_F32 / FL_F16
int fl_matched_adjoint_wt(fl_plan* p, const void* yw, int wt, void* x, int xt, const int* skip,
                          int layout, cudaStream_t st);
// volume (all frames) to the z-folded layout, or back with unfold = 1
int fl_matched_fold(fl_plan* p, const void* src, void* dst, int dtype, int unfold,
                    cudaStream_t st);
int fl_plan_work(fl_plan* p, float** w);
int fl_plan_vwork(fl_plan* p, size_t bytes, void** w);
int fl_matched_ready(fl_plan* p);
int fl_matched_count(fl_plan* p, int32_t* counts, cudaStream_t st);
