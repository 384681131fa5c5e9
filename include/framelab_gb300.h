/*
 * framelab_gb300.h -- C ABI of libframelab_gb300.so
 *
 * GB300-native (sm_103a) implementation of FrameLab's CT reconstruction hot
 * path: Siddon fan/cone projectors, their backprojectors, the undecimated
 * piecewise-linear framelet with soft-shrinkage, and the CGLS / split-Bregman
 * vector algebra.
 *
 * Two layers:
 *  (1) Drop-ins. The reference's own extern "C" entry points, same names and
 *      argument lists, host pointers in and out (the mex gateways and the
 *      MATLAB classes call these unchanged). They return void like the
 *      reference; the outcome is readable with fl_last_status()/fl_last_error().
 *  (2) The device API. Plans (uploaded geometry + precomputed tables), device
 *      pointers, a caller-supplied CUDA stream (passed as void*), int status.
 *
 * No function aborts the process. Every CUDA error is turned into a status.
 * Volumes are x-fastest (iz*ny*nx + iy*nx + ix); sinograms are detector
 * column fastest (iv*na*nb + ib*na + ia). All lengths are in xy-voxel units
 * (xy pitch = 1); outputs are multiplied by `scale`, the physical xy pitch.
 */
#ifndef FRAMELAB_GB300_H
#define FRAMELAB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status                                                                    */
/* ------------------------------------------------------------------------ */
enum {
    FL_OK = 0,
    FL_ERR_INVALID = 1,      /* bad argument or geometry */
    FL_ERR_UNSUPPORTED = 2,  /* valid but not implemented for this case */
    FL_ERR_CUDA = 3,         /* a CUDA runtime call or a kernel failed */
    FL_ERR_ALLOC = 4,        /* device or host allocation failed */
    FL_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
    FL_ERR_NUMERIC = 6       /* a solve met NaN / Inf (in its inputs or the operator) */
};

/* Status of the last call made on this host thread, and its message. */
int fl_last_status(void);
const char *fl_last_error(void);
const char *fl_version(void);

/* ------------------------------------------------------------------------ */
/* (1) Drop-ins for the reference's GPU entry points                         */
/* ------------------------------------------------------------------------ */

/* Fan-beam Siddon projection (version 0), bit-exact with the reference's
 * Ax_fan_mf_cpu_siddon. Replaces Ax_fan_mf_gpu_siddon
 * (matlab/mex/src/Ax_fan_mf.h:3, Ax_fan_mf_gpu_siddon.cu:106-129).
 * y[iv*nd+id]; X holds nt frames, view iv reads frame id_X[iv]. */
void Ax_fan_mf_gpu_siddon(float *X, float *y, float SO, float OD, float scale, int nx, int ny,
                          int nv, float *sd_phi, int nd, float *y_det, int *id_X, int nt);

/* Fan-beam chord-length backprojection (version 1), bit-exact with the
 * reference's Atx_fan_mf_cpu_new. Replaces Atx_fan_mf_gpu_new
 * (matlab/mex/src/Atx_fan_mf.h:4, Atx_fan_mf_gpu_new.cu:77-106). */
void Atx_fan_mf_gpu_new(float *x, float *Y, float SO, float OD, float scale, int nx, int ny,
                        float *sd_phi, int nd, float *y_det, float dy_det, float y_os, int nt,
                        int *id_Y, int *Nv, int tmp_size, int nv, float *cos_phi,
                        float *sin_phi, float *cos_det, float *sin_det);

/* Fan-beam finite-size-beam projection (version 2), bit-exact with the
 * reference's Ax_fan_mf_cpu_new_fb (pixel area between the bin's two edge
 * rays). Replaces Ax_fan_mf_gpu_new_fb (matlab/mex/src/Ax_fan_mf.h:13,
 * Ax_fan_mf_gpu_new_fb.cu:138-164). */
void Ax_fan_mf_gpu_new_fb(float *X, float *y, float SO, float OD, float scale, int nx, int ny,
                          int nv, float *sd_phi, int nd, float *y_det, int *id_X, int nt,
                          float dy_det);

/* Fan-beam finite-size-beam backprojection (version 2), bit-exact with the
 * reference's Atx_fan_mf_cpu_new_fb; cos_det/sin_det are the nd + 1 bin-edge
 * arrays the gateway reads from cos_det2/sin_det2. Replaces
 * Atx_fan_mf_gpu_new_fb (matlab/mex/src/Atx_fan_mf.h:13, Atx_fan_mf_gpu_new_fb.cu:81-111). */
void Atx_fan_mf_gpu_new_fb(float *x, float *Y, float SO, float OD, float scale, int nx, int ny,
                           float *sd_phi, int nd, float *y_det, float dy_det, int nt, int *id_Y,
                           int *Nv, int tmp_size, int nv, float *cos_phi, float *sin_phi,
                           float *cos_det, float *sin_det);

/* Cone-beam Siddon projection (version 0), bit-exact with the reference's
 * CPU kernel Ax_cone_mf_cpu_siddon (the reference's own GPU version of this
 * entry point divides by the wrong z step). Replaces Ax_cone_mf_gpu_siddon
 * (matlab/mex/src/Ax_cone_mf.h:10, Ax_cone_mf_gpu_siddon.cu:149-188).
 * Frame it owns views id_Y[it*tmp_size + j], j < Nv[it]. nv_block is
 * accepted and ignored (the reference used it to dodge the display watchdog). */
void Ax_cone_mf_gpu_siddon(float *X, float *y, float *sd_phi, float *sd_z, float *y_det,
                           float *z_det, int *id_Y, int *Nv, float SO, float OD, float scale,
                           float dz, int nx, int ny, int nz, int nt, int na, int nb, int nv,
                           int tmp_size, int nv_block);

/* Fan-beam dominant-axis projection (version 1, the classes' default),
 * bit-exact with the reference's Ax_fan_mf_cpu_new. Replaces
 * Ax_fan_mf_gpu_new (matlab/mex/src/Ax_fan_mf.h:7, Ax_fan_mf_gpu_new.cu:138-164). */
void Ax_fan_mf_gpu_new(float *X, float *y, float SO, float OD, float scale, int nx, int ny,
                       int nv, float *sd_phi, int nd, float *y_det, int *id_X, int nt);

/* Cone-beam dominant-axis projection (version 1, the classes' default) and
 * its normalised twin yNorm = y / (|src - det| scale), bit-exact with the
 * reference's CPU kernel Ax_cone_mf_cpu_new (its GPU version handles
 * partially covered border voxels differently). Replaces Ax_cone_mf_gpu_new
 * (matlab/mex/src/Ax_cone_mf.h:3, Ax_cone_mf_gpu_new.cu:469-521). */
void Ax_cone_mf_gpu_new(float *X, float *y, float *yNorm, float *sd_phi, float *sd_z,
                        float *y_det, float *z_det, int *id_Y, int *Nv, float SO, float OD,
                        float scale, float dz, int nx, int ny, int nz, int nt, int na, int nb,
                        int nv, int tmp_size, int nv_block);

/* Cone-beam chord-length backprojection (version 1), bit-exact with the
 * reference's Atx_cone_mf_cpu_new. Replaces Atx_cone_mf_gpu_new
 * (matlab/mex/src/Atx_cone_mf.h:4, Atx_cone_mf_gpu_new.cu:114-162). */
void Atx_cone_mf_gpu_new(float *X, float *y, float *cos_phi, float *sin_phi, float *sd_z,
                         float *y_det, float *z_det, int *id_Y, int *Nv, float SO, float OD,
                         float scale, float dy_det, float y_os, float dz_det, float dz, int nx,
                         int ny, int nz, int nt, int na, int nb, int nv, int tmp_size,
                         int nv_block);

/* ------------------------------------------------------------------------ */
/* (2) Device API                                                            */
/* ------------------------------------------------------------------------ */

/* Scan description. Host pointers; copied at plan creation. Field meanings
 * follow the reference's `para` struct (ConeBeamScanner/setPara.m:5-82,
 * FanBeamScanner/setPara.m:4-55). */
typedef struct fl_scan {
    int32_t ndim;            /* 2: fan beam, 3: cone beam */
    int32_t nx, ny, nz;      /* voxels; nz = 1 for a fan */
    int32_t nt;              /* volume frames (>= 1) */
    int32_t nv;              /* views */
    int32_t na, nb;          /* detector columns; rows (1 for a fan) */
    float SO, OD;            /* source-isocentre, isocentre-detector distance */
    float scale;             /* physical xy voxel pitch */
    float dz;                /* z voxel pitch / xy pitch (cone) */
    float dy_det, dz_det;    /* detector pitches (chord backprojector window) */
    float y_os;              /* detector column offset in pixels (window) */
    const float *sd_phi;     /* [nv] source angles; NULL = atan2(sin_phi, cos_phi) */
    const float *sd_z;       /* [nv] source z, NULL = all 0 (circular) */
    const float *y_det;      /* [na] column positions on the flat panel */
    const float *z_det;      /* [nb] row positions (cone), NULL for a fan */
    const float *cos_phi;    /* [nv] chord backprojector trig, NULL = computed */
    const float *sin_phi;    /* [nv] */
    const float *cos_det;    /* [na] fan chord backprojector, NULL = computed */
    const float *sin_det;    /* [na] */
    const int32_t *view_frame; /* [nv] frame read by each view (id_X), NULL = 0 */
    const int32_t *id_Y;     /* [tmp_size*nt] views of frame it at it*tmp_size + j,
                                j < Nv[it], in accumulation order; NULL = derived
                                from view_frame in increasing view order */
    const int32_t *Nv;       /* [nt] */
    int32_t tmp_size;
    const float *cos_det2;   /* [na+1] fan bin-edge trig (finite beam), NULL = computed */
    const float *sin_det2;   /* [na+1] */
} fl_scan;

typedef struct fl_plan fl_plan;

/* Projection models */
enum {
    FL_MODEL_SIDDON_REF = 0, /* version 0: bit-exact reference Siddon forward */
    FL_MODEL_CHORD_REF = 1,  /* version 1 adjoint: bit-exact reference chord backprojector */
    FL_MODEL_GAO_REF = 2,    /* version 1 forward: bit-exact reference dominant-axis projector */
    FL_MODEL_FB_REF = 3,     /* version 2 fan pair: bit-exact reference finite-size beam */
    FL_MODEL_MATCHED = 16    /* matched Siddon pair; adjoint is the exact transpose */
};

/* Storage dtypes of volumes / sinograms (arithmetic is always f32) */
enum { FL_F32 = 0, FL_F16 = 1, FL_BF16 = 2 };

int fl_plan_create(const fl_scan *scan, fl_plan **plan);
void fl_plan_destroy(fl_plan *plan);
/* Number of voxels (all frames) and rays of the plan. */
int fl_plan_sizes(const fl_plan *plan, int64_t *n_vox, int64_t *n_rays);

/* Plan options.
 * FL_OPT_Z_MIRROR: on by default for a cone scan that is symmetric about the
 *   source plane (every sd_z = 0, nz and nb even, dz > 0, z_det[nb-1-ib] ==
 *   -z_det[ib] exactly and z_det[ib] < 0 for ib < nb/2). The matched pair then
 *   walks / weighs only the rows ib < nb/2 and gives row nb-1-ib the mirrored
 *   values, with voxel pairs (iz, nz-1-iz) and row pairs stored side by side
 *   internally, so both kernels do about half the work; the matrix stays
 *   exactly transposed.
 *   Setting 0 selects the general kernels; 1 re-enables it where allowed.
 * FL_OPT_ROT_MIRROR: on top of FL_OPT_Z_MIRROR, on by default for a scan of
 *   one frame with an even number of views where view v + nv/2 is view v
 *   turned by pi about the z axis (cos and sin of the angles opposite to
 *   within 1e-6) and nx, ny multiples of 4. The matched pair then walks /
 *   weighs only views v < nv/2: ray (v + nv/2, a, b) is defined as ray
 *   (v, a, b) turned by pi, crossing voxel (nx-1-x, ny-1-y, z) where ray
 *   (v, a, b) crosses (x, y, z), with the same length and c_r. One walk or
 *   weight serves four rays; the matrix stays exactly transposed and differs
 *   from the general kernels' by the FP32 rounding of the turned views' own
 *   tables.
 *   Queries report 0 while FL_OPT_Z_MIRROR is off. Fan-beam plans take the
 *   half turn without a mirror (one frame, ny even, the same view test):
 *   ray (v + nv/2, a) crosses pixel (nx-1-x, ny-1-y) where ray (v, a) crosses
 *   (x, y), one walk or weight serving two rays.
 * FL_OPT_QUARTER_TURN: on top of FL_OPT_ROT_MIRROR, on by default when
 *   nx == ny, nv is a multiple of 4 and view v + nv/4 is view v turned by
 *   pi/2 (to within 1e-6). Ray (v + j nv/4, a, b) is then defined as ray
 *   (v, a, b) turned by j pi/2, crossing voxel R^j (x, y, z) with
 *   R (x, y, z) = (n-1-y, x, z): one walk or weight serves eight rays (four
 *   on a fan plan, R (x, y) = (n-1-y, x), nx == ny even). Queries report 0
 *   while either option below it is off.
 *   A ray that runs exactly along a pixel boundary (the central ray of an
 *   odd detector at a view angle of exactly 0) has no unique discretisation:
 *   on the turn forms its turned copies take the walked view's choice, which
 *   can differ from the general kernels' at O(1) for that ray alone. */
/* FL_OPT_REFLECT: on by default for cone plans, and taken by fan plans when
 *   set (a single small fan scan has too few walked rays and pixel blocks to
 *   fill the GPU with it: 256^2, 360 views, 6107 against 6851 CGLS it/s;
 *   batches of many slices gain: 64 uneven slices, 61.9 against 51.9 it/s),
 *   where view 0 is at angle 0, view nv - v is
 *   the mirror image of view v about the x axis (to within 1e-6) and the
 *   detector is symmetric about its centre (y_det[na-1-a] == -y_det[a], na
 *   even), on top of the quarter turns (with nv a multiple of 8) or of the
 *   half turn; fan plans of one frame with an odd view count and ny even
 *   also take it alone. With M (x, y) = (x, ny-1-y), S the quarter turn R,
 *   the half turn R^2 or (alone) the identity, NR = 4, 2, 1 its order and q =
 *   nv/NR, ray (j q - v, na-1-a, b) is defined as ray (v, a, b) reflected by
 *   M and turned by S^j, for the walked views v = 0 .. floor(q/2). View 0,
 *   and view q/2 where q is even (then its own mirror image), walk their
 *   columns a < na/2, the other half being their mirror images; view q/2 is
 *   walked at the exact angle pi/NR (cone: the quarter or half turn; fan:
 *   the same). One walk or weight serves sixteen (cone, quarter turns),
 *   eight (cone, half turn; fan, quarter turns), four (fan, half turn) or two
 *   (fan, alone) rays. Queries report 0 while an option it rides on is off. */
enum { FL_OPT_Z_MIRROR = 1, FL_OPT_ROT_MIRROR = 2, FL_OPT_QUARTER_TURN = 3,
       FL_OPT_REFLECT = 4 };
int fl_plan_option(fl_plan *plan, int option, int value);
int fl_plan_query(const fl_plan *plan, int option, int *value);
/* Launch-shape autotuner for a plan's matched projector kernels: times each
 * candidate on the plan's own geometry, one launch each on `stream` after one
 * untimed, and keeps the fastest for the forward and for the backprojection.
 * Cone plans: the 128-thread block shapes (8x16, 16x8, 32x4, 4x32) of both
 * kernels and, on reflection plans, the backprojection's voxel run and row
 * loop (FL_TUNE_ADJ_RUN / _ROWS). Fan plans: the parts per walked ray of the
 * turn and reflection forwards (FL_TUNE_FAN_PARTS: 1, 4, 16), the pixel block
 * of the backprojections (FL_TUNE_FAN_BLOCK: 1 or 2) and the view groups of
 * the turn and reflection backprojections (FL_TUNE_FAN_GROUPS: 8 or 16). Only
 * the fan parts and groups change any bit of a result (the order of a ray's
 * or a pixel's additions, not the matrix). Synchronises `stream`; uses the
 * plan's scratch buffers. shapes (optional, [4]): the chosen forward x, y and
 * backprojection x, y of a cone plan; for a fan plan the parts count, 0, the
 * pixel block and the view groups. */
int fl_plan_autotune(fl_plan *plan, void *stream, int32_t *shapes);
/* FL_TUNE_ADJ_RUN: voxels per thread of the reflection backprojection (1 or
 * 2); FL_TUNE_ADJ_ROWS: its row loop, 1 or 2 detector rows per iteration, or
 * 3: one pass over a run's rows, each row loaded once for all the run's
 * voxels (runs of 2; with runs of 1 it is 1). fl_plan_autotune times the
 * pairs and keeps the fastest; fl_plan_option sets them (other values are
 * refused), fl_plan_query reads them. The results do not depend on them. */
enum { FL_TUNE_ADJ_RUN = 16, FL_TUNE_ADJ_ROWS = 17 };
/* Fan plans. FL_TUNE_FAN_PARTS: threads per walked ray of the half- or
 * quarter-turn forward (1, 4 or 16), each walking a run of the ray's segments,
 * their sums added in order; by default 16 for scans of fewer than 65,536
 * walks (nv/G views x na columns), else 1. It sets the order of a ray's
 * additions: the forward's bits (within FP32 rounding), not its matrix. A batch
 * takes each turn slice's count when it is created, so batched and single-plan
 * results stay equal bit for bit. FL_TUNE_FAN_BLOCK: pixels per thread side of
 * the fan backprojections, 1 (one pixel, view groups over threads) or 2 (a 2x2
 * block); by default 2 once there are four waves of blocks. The results do not
 * depend on it. fl_plan_option sets them (other values are refused),
 * fl_plan_query reads the values in effect. */
enum { FL_TUNE_FAN_PARTS = 18, FL_TUNE_FAN_BLOCK = 19 };
/* FL_TUNE_FAN_GROUPS: view groups of a fan plan's turn and reflection
 * backprojections, 8 (the default) or 16: each thread block's threads split a
 * pixel block's views into that many interleaved groups, added in order at
 * the end. It sets the order of a pixel's additions (its bits within FP32
 * rounding); batches take 8, so batched and single-plan results are equal bit
 * for bit with 8. The quarter-turn reflection form with 2 x 2 pixel blocks
 * always takes 8 (fl_plan_query reports the value in effect).
 * fl_plan_autotune times both on turn and reflection plans. */
enum { FL_TUNE_FAN_GROUPS = 20 };
/* FL_TUNE_ADJ_CHUNKS: the reflection backprojection of a cone plan runs as
 * this many launches over consecutive chunks of its walked views (1 .. 64;
 * default 1), each continuing the sums the one before left in the output, so
 * the blocks resident together read the same views' detector rows and L2
 * serves them (512^3, 720 views: 16 chunks, 264 -> 256 ms per CGLS iteration).
 * The sums are added in the same order: the results do not depend on it. It
 * applies where the backprojection writes FP32 (FP16 / BF16 outputs take one
 * launch). fl_plan_autotune times 1, 4, 8, 16. */
enum { FL_TUNE_ADJ_CHUNKS = 21 };
/* FL_TUNE_FAN_TMA: a fan plan's forward makes the transposed copy of its
 * input that its walks read with the tensor memory accelerator (tiled
 * cp.async.bulk.tensor loads and stores of 32 x 32 tiles through shared
 * memory; 1, the default) or with plain loads and stores (0). The copy, and
 * so every result, is the same either way. TMA needs the input on a 16-byte
 * boundary and image rows of a multiple of 16 bytes (nx, ny multiples of 4 in
 * FP32, 8 in FP16 / BF16); elsewhere the plain copy runs.
 * FL_DEBUG_TMA_TIMEOUTS (query only): 1 if a TMA tile of this plan did not
 * arrive within its bounded wait since the last query (the copy was then
 * incomplete); the query clears it. */
enum { FL_TUNE_FAN_TMA = 22, FL_DEBUG_TMA_TIMEOUTS = 23 };
/* FL_DEBUG_TMA_STALL (tests only; 0, the default, is off): the plan's TMA
 * copy issues no load and each block waits N polls on a barrier phase that
 * nothing completes, then records the timeout and returns, with no copy in
 * flight. fl_cgls_solve (and so fl_cgls_solve_host and the split-Bregman
 * solves) then return FL_ERR_TIMEOUT, and clear the flag, when a forward of
 * the solve timed out. N in 0 .. 2^20. */
enum { FL_DEBUG_TMA_STALL = 24 };

/* y = A x on `stream`. x: n_vox elements, y: n_rays elements, device memory.
 * The matched model works in buffers the plan owns: a z-mirror cone plan
 * folds x into its volume scratch, a fan plan writes the transposed copy of
 * x its walks read (allocated with the plan). Matched forwards and
 * backprojections of one plan are therefore ordered on one stream: calls of
 * one plan that overlap on the GPU (different streams) race; different
 * plans do not share buffers. */
int fl_forward(fl_plan *plan, int model, const void *x, int x_dtype, void *y, int y_dtype,
               void *stream);
/* x = A^T y on `stream`. For FL_MODEL_MATCHED this is the exact transpose of
 * fl_forward's matrix (it weights y into the plan's sinogram scratch first);
 * FL_MODEL_CHORD_REF is the reference's backprojector. */
int fl_adjoint(fl_plan *plan, int model, const void *y, int y_dtype, void *x, int x_dtype,
               void *stream);
/* Version-1 forward with the cone-beam normalised output (ynorm may be NULL;
 * fan beams have no ynorm). Replaces the [y, yNorm] of Ax_cone_mf. */
int fl_forward_gao(fl_plan *plan, const float *x, float *y, float *ynorm, void *stream);

/* Number of voxels each ray crosses with positive length (matched model). */
int fl_count_intersections(fl_plan *plan, int32_t *counts, void *stream);

/* No counterpart in the reference. The matched-model backprojection of
 * fl_adjoint without any device allocation, for callers that cannot call
 * cudaMalloc when they backproject: work being captured into a CUDA graph, a
 * host application whose own pool allocator owns the GPU's memory, a loop
 * that must not block on the allocator. The sinogram pre-weighting scratch
 * that fl_adjoint allocates in the plan is instead a fixed array of
 * FL_ADJOINT_NOALLOC_MAX_RAYS floats (8 MiB) inside the library; plans with
 * more rays are refused with FL_ERR_INVALID. The first call on each device
 * looks up that array's device address, and with CUDA's lazy module loading
 * that is when the 8 MiB are placed on the device: make that first call
 * before any stream capture and before a pool allocator takes the GPU's
 * memory. Later calls allocate nothing; the array stays until the process
 * exits. The stream must belong to the current device (another device's
 * stream is refused). All calls share the array: calls that can overlap on
 * the GPU race and must be serialised. */
#define FL_ADJOINT_NOALLOC_MAX_RAYS (1 << 21)
int fl_adjoint_noalloc(fl_plan *plan, const void *y, int y_dtype, void *x, int x_dtype,
                       void *stream);

/* ------------------------------------------------------------------------ */
/* Vector algebra and CGLS (solveCGLS.m:6-31, ObjectData.m:96-125)           */
/* ------------------------------------------------------------------------ */

/* *out (device double) = sum a[i]*b[i], accumulated in FP64. Replaces
 * ObjectData.objdot (ObjectData.m:118-121). Uses a per-device scratch buffer
 * allocated on first use; calls that overlap on the GPU (different streams)
 * must not share a device. */
int fl_dot(const float *a, const float *b, int64_t n, double *out, void *stream);

/* y = a*x + b*y on n device floats (x may be NULL: y = b*y). The object
 * algebra of ObjectData / CTData / FrameletExpansion (plus, minus, mtimes). */
int fl_axpby(float *y, const float *x, float a, float b, int64_t n, void *stream);

/* q = (A^T A + lam I) x for the matched model, FP32 (the operator
 * A_loc of solveCGLS.m:7). x, q: n_vox device floats. */
int fl_normal_apply(fl_plan *plan, const float *x, float *q, float lam, void *stream);

typedef struct fl_cgls fl_cgls;
/* PLAIN: FP32, one kernel per vector operation, scalars on the host.
 * GRAPH: FP32, fused updates with device-side scalars, CUDA-graph replay.
 * MIXED: GRAPH plus an FP16 copy of the search direction for the projector
 *        and an FP32 residual refresh every `refresh` iterations. */
enum { FL_CGLS_PLAIN = 0, FL_CGLS_MIXED = 1, FL_CGLS_GRAPH = 2 };
enum { FL_CGLS_ZERO_START = 1 };   /* u0 == 0: skip the initial A_loc(u0) */

/* CGLS workspace bound to a plan (matched model). Allocates r, p, q, a
 * sinogram temporary (and an FP16 copy of p in FL_CGLS_MIXED). */
int fl_cgls_create(fl_plan *plan, int mode, fl_cgls **cg);
void fl_cgls_destroy(fl_cgls *cg);

/* Solve (A^T A + lam I) u = b by CGLS (Optimizers.CGLS/solveCGLS): u holds
 * u0 on entry and the result on return; at most `iters` iterations, stop once
 * gamma = <r,r> < tol. FL_CGLS_MIXED recomputes the FP32 residual every
 * `refresh` iterations (0 = never). gamma_history (host, optional, >= iters
 * doubles) receives gamma after each iteration; *iters_done the count.
 * Returns when the result is in u (the call synchronises with `stream`). */
int fl_cgls_solve(fl_cgls *cg, const float *b, float *u, float lam, int iters, double tol,
                  int refresh, int flags, double *gamma_history, int *iters_done,
                  void *stream);

/* ------------------------------------------------------------------------ */
/* Framelets and split Bregman (FrameletSystem, softThreshold,               */
/* solveSplitBregman.m:15-41)                                                */
/* ------------------------------------------------------------------------ */
typedef struct fl_framelet fl_framelet;
enum { FL_FRAMELET_HAAR = 0, FL_FRAMELET_LINEAR = 1, FL_FRAMELET_CUBIC = 3 };

/* Undecimated tensor-product framelet on nx*ny*nz volumes (nz == 1: the 2-D
 * transform), `levels` levels, filter bank `kind` (GenerateFrameletFilter.m).
 * Replaces FrameletSystem(dim, type, level) (FrameletSystem.m:12-29). */
int fl_framelet_create(int nx, int ny, int nz, int levels, int kind, fl_framelet **fw);
void fl_framelet_destroy(fl_framelet *fw);
/* Floats in a coefficient set: every band of every level except the low band
 * of levels below the last (which the synthesis never reads). */
int64_t fl_framelet_ncoef(const fl_framelet *fw);
/* FL_FRAMELET_OPT_FUSED (default 1): each 3-D level of the three-tap banks
 * (linear, Haar) with dilation up to 8 streams along z: the analysis (with
 * the Bregman update) is one kernel, the synthesis two; 0 selects the
 * separable pass per axis. Both forms give identical results. */
enum { FL_FRAMELET_OPT_FUSED = 1 };
int fl_framelet_option(fl_framelet *fw, int option, int value);
/* coef = W u (forwardTransform, FraDecMultiLevel3D.m) */
int fl_framelet_analysis(fl_framelet *fw, const float *u, float *coef, void *stream);
/* u = W^T coef (adjointTransform, FraRecMultiLevel3D.m) */
int fl_framelet_synthesis(fl_framelet *fw, const float *coef, float *u, void *stream);
/* One split-Bregman coefficient step (solveSplitBregman.m:30-38) in two
 * passes: alpha = shrink(v + W u, tau) (low band of the last level not
 * shrunk); v += W u - alpha; t = alpha - v; b = Atf + mu * W^T t.
 * v and t are coefficient sets; Atf may be NULL (taken as 0). */
int fl_framelet_bregman(fl_framelet *fw, const float *u, float *v, float *t, const float *Atf,
                        float mu, float tau, float *b, void *stream);

/* Split Bregman for min 1/2|Au - f|^2 + lam |W u|_1 (SplitBregman.m,
 * solveSplitBregman.m): `outer` iterations of { CGLS on (A^T A + mu I) u = b
 * warm-started from u, `cg_iters` iterations; framelet step }. f: sinogram,
 * u: initial guess in, result out (device). `mode` selects the CGLS form.
 * history (host, optional, >= outer doubles): |u_k - u_{k-1}| / |u_k| (FP64). */
int fl_sb_solve(fl_plan *plan, const float *f, float *u, float lam, float mu, int outer,
                int cg_iters, double cg_tol, int levels, int kind, int mode, double *history,
                void *stream);

/* Persistent form of fl_sb_solve: the framelet, the CGLS workspace and the
 * coefficient sets of one plan (about 2 * 53 volumes for a 2-level linear
 * framelet) are allocated once and reused by every fl_sb_run. */
typedef struct fl_sb fl_sb;
int fl_sb_create(fl_plan *plan, int levels, int kind, int mode, fl_sb **sb);
int fl_sb_run(fl_sb *sb, const float *f, float *u, float lam, float mu, int outer,
              int cg_iters, double cg_tol, double *history, void *stream);
void fl_sb_destroy(fl_sb *sb);

/* The same solve with host buffers (the mex-style boundary): b and u0 are
 * copied to the device (u0 skipped with FL_CGLS_ZERO_START), the result is
 * copied back into u. Device copies are kept in the workspace for reuse.
 * Exception, same results: with a z-mirror plan in the graph or mixed form,
 * b and u pinned (cudaHostAlloc) or registered (cudaHostRegister), the
 * solve's fold reads b (and u0) and its unfold writes u in host memory
 * directly, with no staging copies. Returns once u holds the result. */
int fl_cgls_solve_host(fl_cgls *cg, const float *b_host, float *u_host, float lam, int iters,
                       double tol, int refresh, int flags, double *gamma_history,
                       int *iters_done, void *stream);

/* ---- batched uneven fan-beam slices ------------------------------------
 * A batch projects and solves many independent single-frame fan-beam scans of
 * different sizes at once (matched model): images and sinograms of all slices
 * are concatenated in plan order (offsets from fl_batch_layout) and every
 * operator is one launch over all slices of a kind: general slices, slices
 * whose plans use a turn alone (FL_OPT_ROT_MIRROR / FL_OPT_QUARTER_TURN) and
 * slices whose plans use a reflection form (FL_OPT_REFLECT) run those
 * plans' kernels, as parallel branches of the stream. Each
 * slice's forward/adjoint result is bit-identical to its own plan's, with the
 * plan's options as they were at fl_batch_create. The plans must outlive the
 * batch.
 * Replaces looping the reference's per-slice Ax_fan_mf / Atx_fan_mf calls
 * (FanBeamScanner/apply.m:11-20, applyAdjoint.m:21-29) and solveCGLS.m:6-31
 * over the slices. */
typedef struct fl_batch fl_batch;
int fl_batch_create(fl_plan *const *plans, int32_t n_plans, fl_batch **out);
void fl_batch_destroy(fl_batch *b);
/* vox_offsets / ray_offsets: [n_plans + 1] each (either may be NULL) */
int fl_batch_layout(const fl_batch *b, int64_t *vox_offsets, int64_t *ray_offsets);
int fl_batch_forward(fl_batch *b, const float *x, float *y, void *stream);
int fl_batch_adjoint(fl_batch *b, const float *y, float *x, void *stream);
/* CGLS per slice on (A_i^T A_i + lam I) u_i = rhs_i, all slices in lockstep,
 * each stopping on its own once gamma_i < tol (or <p, q> = 0). u: initial
 * guess in (ignored with FL_CGLS_ZERO_START), result out (device).
 * gamma_history (host, optional): [n_plans * iters], row i = slice i's gamma
 * after each iteration (0 after it stopped); iters_done (host, optional):
 * [n_plans]. One iteration is a replayed CUDA graph of 3 launches plus a
 * forward and a backprojection for each kind of slice present (general,
 * turn, reflection; the kinds run as parallel branches) and a transposed
 * copy of the direction the forwards read. */
int fl_batch_cgls(fl_batch *b, const float *rhs, float *u, float lam, int32_t iters, double tol,
                  int32_t flags, double *gamma_history, int32_t *iters_done, void *stream);
/* Launch tuner of a batch: times the parts per walked ray of its half- and
 * quarter-turn slices (1, 4, 16; FL_TUNE_FAN_PARTS) on the batch's own
 * forward, one launch each on `stream` after one untimed, and keeps the
 * fastest for every turn slice (a small scan needs parts to fill the GPU
 * alone, not always beside other slices). The count sets the order of a
 * ray's additions, so the batch's forward then equals its slice plans' with
 * that count set. Synchronises `stream`; clobbers the batch's CGLS scratch
 * (not the solution). parts (optional): the count chosen, 0 when the batch
 * has no turn slice. Replaces nothing in the reference (its slices run one
 * by one). */
int fl_batch_autotune(fl_batch *b, void *stream, int32_t *parts);

/* Bounds-checked builds only (compiled with -DFL_BOUNDS_CHECK, the
 * "checked" build variant): *violations = the number of gathers of the
 * matched and batched kernels whose index fell outside its array since the
 * last reset (each such access was skipped); reset = 1 clears the count.
 * Normal builds return FL_ERR_UNSUPPORTED with *violations = 0. */
int fl_debug_bounds(int64_t *violations, int reset);

/* Failure injection for tests: the nth next device allocation of the library
 * (1 = the next one) fails as an out-of-memory would, once; 0 disarms it.
 * Every entry point then returns FL_ERR_ALLOC and releases what it held. */
void fl_debug_fail_alloc(int64_t nth);

#ifdef __cplusplus
}
#endif
#endif /* FRAMELAB_GB300_H */
