// fl_runtime.cpp -- host runtime: status, plans (geometry -> HBM tables),
// projector dispatch and the reference-signature drop-ins.
#include <atomic>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "fl_trace.h"
#include "fl_plan.h"
#include "framelab_gb300.h"

// ---------------------------------------------------------------------------
// Status (per host thread)
// ---------------------------------------------------------------------------
static thread_local int g_status = FL_OK;
static thread_local char g_msg[512] = "";

int fl_set_error(int code, const char* fmt, ...)
{
    g_status = code;
    if (code == FL_OK) { g_msg[0] = 0; return FL_OK; }
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, ap);
    va_end(ap);
    return code;
}

int fl_check_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return FL_OK;
    cudaGetLastError();   // clear a non-sticky error so the next call starts clean
    return fl_set_error(e == cudaErrorMemoryAllocation ? FL_ERR_ALLOC : FL_ERR_CUDA,
                        "%s: %s", what, cudaGetErrorString(e));
}

int fl_check_launch(const char* what) { return fl_check_cuda(cudaGetLastError(), what); }

// Allocation failure injection: g_fail_countdown = n > 0 makes the n-th next
// fl_malloc fail as an out-of-memory would (one shot).
static std::atomic<long long> g_fail_countdown{0};

extern "C" void fl_debug_fail_alloc(int64_t nth) { g_fail_countdown.store(nth > 0 ? nth : 0); }

cudaError_t fl_malloc(void** p, size_t bytes)
{
    long long c = g_fail_countdown.load();
    while (c > 0) {
        if (g_fail_countdown.compare_exchange_weak(c, c - 1)) {
            if (c == 1) {
                *p = nullptr;
                return cudaErrorMemoryAllocation;
            }
            break;
        }
    }
    return cudaMalloc(p, bytes);
}

extern "C" int fl_last_status(void) { return g_status; }
extern "C" const char* fl_last_error(void) { return g_msg; }
extern "C" const char* fl_version(void) { return "framelab_gb300 1.0 (sm_103a)"; }

// ---------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------
template <typename T>
static int upload(T** dst, const T* src, size_t n)
{
    *dst = nullptr;
    if (n == 0) return FL_OK;
    int st = fl_check_cuda(fl_malloc((void**)dst, n * sizeof(T)), "fl_malloc(plan)");
    if (st) return st;
    return fl_check_cuda(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice),
                         "cudaMemcpy(plan)");
}

static void free_plan_arrays(fl_plan* p)
{
    void* ptrs[] = {p->d_sd_phi, p->d_sd_z,   p->d_y_det,      p->d_z_det, p->d_cos_phi,
                    p->d_sin_phi, p->d_cos_det, p->d_sin_det,   p->d_cphi_f, p->d_sphi_f,
                    p->d_view_frame, p->d_idY, p->d_Nv,        p->d_col,   p->d_colr,
                    p->d_row,    p->d_rowz,   p->d_view,       p->d_work,
                    p->d_cos_det2, p->d_sin_det2, p->d_fb_edges, p->d_vwork, p->d_xt,
                    p->d_dq, p->d_tma_err};
    for (void* q : ptrs)
        if (q) cudaFree(q);
}

// Nudge a direction component away from zero so 1/d stays finite; the ray
// moves by at most 1e-9 of its length, identically for forward and adjoint.
static double nudge(double d, double len)
{
    double eps = 1e-9 * len;
    if (std::fabs(d) < eps) return d < 0 ? -eps : eps;
    return d;
}

// One axis of a ray (fl_plan.h): crossings A(k) = (k - K) * inv for plane
// index k in [0, n], with K the plane coordinate of the ray's isocentre
// crossing. K is quantised to kq, a multiple of a power of two chosen so that
// every k - kq the kernels form (k in [-1, n + 1]) has at most 24 significant
// bits, i.e. is exact in FP32; c carries the quantisation remainder.
static AxisEntry axis_entry(double K, double inv, int n)
{
    double span = std::fmax(std::fabs(K + 1.0), std::fabs((double)n + 1.0 - K)) + 2.0;
    int e = 0;
    std::frexp(span, &e);                        // span < 2^e
    double q = std::ldexp(1.0, e - 23);          // |k - kq| / q < 2^23 + ...
    double kq = std::nearbyint(K / q) * q;
    AxisEntry a;
    a.kq = (float)kq;                            // exact: 24 significant bits at most
    a.ih = (float)inv;
    a.il = (float)(inv - (double)a.ih);
    a.c = (float)((kq - K) * inv);
    return a;
}

// Finite, and kq within 2^22 planes (its quantum is then at most 1, so every
// k - kq of an integer k is exact).
static bool axis_finite(const AxisEntry& a)
{
    return std::isfinite(a.kq) && std::isfinite(a.ih) && std::isfinite(a.il) &&
           std::isfinite(a.c) && a.ih != 0.0f && std::fabs(a.kq) < 4194304.0f;
}

static int build_tables(fl_plan* p, const std::vector<float>& phi, const float* sd_z,
                        const float* y_det, const float* z_det)
{
    const fl_scan& s = p->s;
    const double SO = s.SO, OD = s.OD, SD = SO + OD;
    const double ac = SO / SD;   // alpha at the isocentre plane: A = alpha - ac
    const int nx2 = s.nx / 2, ny2 = s.ny / 2, nz2 = s.nz / 2;
    // views 0 .. nv-1, then row nv: view nv/8 at the exact diagonal angle
    // pi/4, row nv + 1: view nv/4 at the exact angle pi/2 (the reflection
    // forms walk them there; copies of view 0 where nv/8 or nv/4 is no view)
    const int nvt = s.nv + 2;
    std::vector<ColEntry> col((size_t)nvt * s.na);
    std::vector<float> colr((size_t)nvt * s.na);
    std::vector<RowEntry> row((size_t)nvt * s.nb);
    std::vector<ViewEntry> view(nvt);
    const bool diag = s.nv % 8 == 0, side = s.nv % 4 == 0;
    for (int iv = 0; iv < nvt; iv++) {
        int src = iv;
        if (iv == s.nv) src = diag ? s.nv / 8 : 0;
        if (iv == s.nv + 1) src = side ? s.nv / 4 : 0;
        double c = std::cos((double)phi[src]), sn = std::sin((double)phi[src]);
        if (iv == s.nv && diag) c = sn = std::sqrt(0.5);
        if (iv == s.nv + 1 && side) { c = 0.0; sn = 1.0; }
        double Sx = -SO * c, Sy = -SO * sn, Sz = sd_z ? (double)sd_z[src] : 0.0;
        view[iv] = ViewEntry{(float)c, (float)sn, (float)Sz, (float)ac};
        for (int ia = 0; ia < s.na; ia++) {
            double u = y_det[ia];
            double dx = (OD * c - u * sn) - Sx, dy = (OD * sn + u * c) - Sy;
            double len = std::sqrt(dx * dx + dy * dy);
            dx = nudge(dx, len); dy = nudge(dy, len);
            // the ray's isocentre crossing P = S + ac d, in plane coordinates
            ColEntry e;
            e.x = axis_entry(nx2 + (Sx + ac * dx), 1.0 / dx, s.nx);
            e.y = axis_entry(ny2 + (Sy + ac * dy), 1.0 / dy, s.ny);
            col[(size_t)iv * s.na + ia] = e;
            colr[(size_t)iv * s.na + ia] = (float)(dx * dx + dy * dy);
        }
        for (int ib = 0; ib < s.nb; ib++) {
            RowEntry r{};
            r.z = AxisEntry{0.0f, 1.0f, 0.0f, 0.0f};
            if (s.ndim == 3) {
                double dzr = nudge((double)z_det[ib], SD);   // detector z - source z
                double pitch = s.dz;
                r.z = axis_entry(nz2 + (Sz + ac * dzr) / pitch, pitch / dzr, s.nz);
                r.dz2 = (float)(dzr * dzr);
            }
            row[(size_t)iv * s.nb + ib] = r;
        }
    }
    // FP16 backprojection input scale: 2^-ceil(log2(max c_r^2))
    {
        double cr2max = 0.0, sc = (double)s.scale * (double)s.scale;
        for (int iv = 0; iv < s.nv; iv++) {      // c_r^2 = scale^2 (|d_xy|^2 + d_z^2)
            double mxy = 0.0, mz = 0.0;
            for (int ia = 0; ia < s.na; ia++)
                mxy = std::fmax(mxy, (double)colr[(size_t)iv * s.na + ia]);
            for (int ib = 0; ib < s.nb; ib++)
                mz = std::fmax(mz, (double)row[(size_t)iv * s.nb + ib].dz2);
            cr2max = std::fmax(cr2max, sc * (mxy + mz));
        }
        int e = 0;
        std::frexp(cr2max > 0.0 ? cr2max : 1.0, &e);        // cr2max < 2^e
        p->y16_scale = (float)std::ldexp(1.0, -e);
    }
    // every crossing parameter the kernels read must be finite
    for (const ColEntry& e : col)
        if (!axis_finite(e.x) || !axis_finite(e.y))
            return fl_set_error(FL_ERR_INVALID, "geometry gives a non-finite ray parameter");
    for (const RowEntry& r : row)
        if (!axis_finite(r.z))
            return fl_set_error(FL_ERR_INVALID, "geometry gives a non-finite ray parameter");
    int st;
    if ((st = upload(&p->d_col, col.data(), col.size()))) return st;
    if ((st = upload(&p->d_colr, colr.data(), colr.size()))) return st;
    if ((st = upload(&p->d_row, row.data(), row.size()))) return st;
    std::vector<AxisEntry> rowz(row.size());
    for (size_t i = 0; i < row.size(); i++) rowz[i] = row[i].z;
    if ((st = upload(&p->d_rowz, rowz.data(), rowz.size()))) return st;
    if ((st = upload(&p->d_view, view.data(), view.size()))) return st;

    // detector grids for the adjoint windows
    p->SD = (float)SD;
    p->det_kind = -1;
    if (s.na == 1) {
        p->det_kind = 0; p->u0 = y_det[0]; p->du = 1.0f;
    } else {
        double u0 = y_det[0], du = ((double)y_det[s.na - 1] - u0) / (s.na - 1);
        double g0 = std::atan2((double)y_det[0], SD);
        double dg = (std::atan2((double)y_det[s.na - 1], SD) - g0) / (s.na - 1);
        double eflat = 0, earc = 0;
        for (int ia = 0; ia < s.na; ia++) {
            eflat = std::fmax(eflat, std::fabs(y_det[ia] - (u0 + ia * du)));
            earc = std::fmax(earc, std::fabs(std::atan2((double)y_det[ia], SD) - (g0 + ia * dg)));
        }
        if (du != 0 && eflat <= 0.005 * std::fabs(du)) {
            p->det_kind = 0; p->u0 = (float)u0; p->du = (float)du;
        } else if (dg != 0 && earc <= 0.005 * std::fabs(dg)) {
            p->det_kind = 1; p->g0 = (float)g0; p->dg = (float)dg;
        }
    }
    p->v0 = 0.0f; p->dv = 1.0f;
    if (s.ndim == 3) {
        p->v0 = z_det[0];
        if (s.nb > 1) {
            double dv = ((double)z_det[s.nb - 1] - z_det[0]) / (s.nb - 1);
            double e = 0;
            for (int ib = 0; ib < s.nb; ib++)
                e = std::fmax(e, std::fabs(z_det[ib] - (z_det[0] + ib * dv)));
            if (dv == 0 || e > 0.005 * std::fabs(dv)) p->det_kind = -2;   // irregular rows
            else p->dv = (float)dv;
        }
    }
    // z-mirror symmetry (fl_plan.h): exact comparisons, so only a geometry that
    // is symmetric in its FP32 inputs qualifies
    // (every walked row must descend -- z_det < 0 for ib < nb/2 -- so its ray
    // stays below the source plane: the z-folded volume holds only that half)
    p->zmirror_ok = 0;
    if (s.ndim == 3 && s.nz % 2 == 0 && s.nb % 2 == 0 && s.dz > 0.0f) {
        bool ok = true;
        for (int iv = 0; iv < s.nv && ok; iv++)
            if (sd_z && sd_z[iv] != 0.0f) ok = false;
        for (int ib = 0; ib < s.nb && ok; ib++)
            if (z_det[s.nb - 1 - ib] != -z_det[ib]) ok = false;
        for (int ib = 0; ib < s.nb / 2 && ok; ib++)
            if (!(z_det[ib] < 0.0f)) ok = false;
        p->zmirror_ok = ok ? 1 : 0;
    }
    p->zmirror = p->zmirror_ok;
    // half-turn symmetry (fl_plan.h): view v + nv/2 is view v turned by pi to
    // within 1e-6 in cos and sin (FP32 angles such as 2 pi k / nv are never
    // exactly opposite), one frame, nx and ny multiples of 4 (the folded volume
    // is tiled in 4 x 4 columns)
    // fan plans: no mirror, ny even (the rows y < ny/2 are the primary half)
    p->rot_ok = 0;
    const bool cone_turn = s.ndim == 3 && p->zmirror_ok && s.nx % 4 == 0 && s.ny % 4 == 0;
    // fan turn plans: even nx and ny, so a turned 2 x 2 pixel block starts at
    // even coordinates and lies in one segment of the matched model's frames
    const bool fan_turn = s.ndim == 2 && s.ny % 2 == 0 && s.nx % 2 == 0;
    if ((cone_turn || fan_turn) && s.nt == 1 && p->views_natural && s.nv % 2 == 0) {
        bool ok = true;
        const int h = s.nv / 2;
        for (int iv = 0; iv < h && ok; iv++) {
            const double c0 = std::cos((double)phi[iv]), s0 = std::sin((double)phi[iv]);
            const double c1 = std::cos((double)phi[iv + h]), s1 = std::sin((double)phi[iv + h]);
            if (std::fabs(c0 + c1) > 1e-6 || std::fabs(s0 + s1) > 1e-6) ok = false;
        }
        p->rot_ok = ok ? 1 : 0;
    }
    p->rot = p->rot_ok;
    // quarter turn (fl_plan.h): view v + nv/4 is view v turned by pi/2 to
    // within 1e-6 (cos -> -sin, sin -> cos), square xy grid
    p->rot4_ok = 0;
    if (p->rot_ok && s.nv % 4 == 0 && s.nx == s.ny && s.nx % (s.ndim == 3 ? 4 : 2) == 0) {
        bool ok = true;
        const int q = s.nv / 4;
        for (int iv = 0; iv < q && ok; iv++) {
            const double c0 = std::cos((double)phi[iv]), s0 = std::sin((double)phi[iv]);
            const double c1 = std::cos((double)phi[iv + q]), s1 = std::sin((double)phi[iv + q]);
            if (std::fabs(c1 + s0) > 1e-6 || std::fabs(s1 - c0) > 1e-6) ok = false;
        }
        p->rot4_ok = ok ? 1 : 0;
    }
    p->rot4 = p->rot4_ok;
    // reflection (fl_plan.h): plans with the half turn (and, for the
    // quarter-turn form, the quarter turn and nv a multiple of 8), or fan
    // plans of one frame, natural view order, an odd view count and ny even
    // (the reflection alone), with view nv - v the mirror image of view v
    // about the x axis to within 1e-6 (cos equal, sin opposite), view 0 at
    // angle 0 and an exactly symmetric detector of even width; fan plans also
    // need the uniform detector of their backprojection
    p->refl2_ok = p->refl4_ok = p->refl1_ok = 0;
    const bool fan_alone = s.ndim == 2 && s.nt == 1 && p->views_natural && s.nv % 2 == 1 &&
                           s.ny % 2 == 0;
    if ((p->rot_ok || fan_alone) && s.na % 2 == 0 && (s.ndim == 3 || p->det_kind >= 0)) {
        bool ok = true;
        for (int ia = 0; ia < s.na / 2 && ok; ia++)
            if (y_det[s.na - 1 - ia] != -y_det[ia]) ok = false;
        for (int iv = 1; iv < s.nv && ok; iv++) {
            const double c0 = std::cos((double)phi[iv]), s0 = std::sin((double)phi[iv]);
            const int m = s.nv - iv;
            const double c1 = std::cos((double)phi[m]), s1 = std::sin((double)phi[m]);
            if (std::fabs(c0 - c1) > 1e-6 || std::fabs(s0 + s1) > 1e-6) ok = false;
        }
        if (phi[0] != 0.0f) ok = false;             // view 0 is its own mirror image
        p->refl2_ok = (ok && p->rot_ok) ? 1 : 0;
        p->refl4_ok = (ok && p->rot4_ok && diag) ? 1 : 0;
        p->refl1_ok = (ok && fan_alone) ? 1 : 0;
    }
    // cone plans take the reflection by default; fan plans when asked: the
    // octant of a single fan image of a few hundred pixels has too few pixel
    // blocks to fill the GPU with it, while a batch of many slices gains
    p->refl = s.ndim == 3 ? 1 : 0;
    return FL_OK;
}

extern "C" int fl_plan_option(fl_plan* p, int option, int value)
{
    if (!p) return fl_set_error(FL_ERR_INVALID, "fl_plan_option: null plan");
    if (option == FL_OPT_Z_MIRROR) {
        p->zmirror = (value && p->zmirror_ok) ? 1 : 0;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_OPT_ROT_MIRROR) {
        p->rot = (value && p->rot_ok) ? 1 : 0;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_OPT_QUARTER_TURN) {
        p->rot4 = (value && p->rot4_ok) ? 1 : 0;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_OPT_REFLECT) {
        p->refl = value ? 1 : 0;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_ADJ_RUN || option == FL_TUNE_ADJ_ROWS) {
        const int top = option == FL_TUNE_ADJ_RUN ? 2 : 3;
        if (value < 1 || value > top)
            return fl_set_error(FL_ERR_INVALID, "fl_plan_option: %d is not in 1..%d", value, top);
        (option == FL_TUNE_ADJ_RUN ? p->adj_run : p->adj_rows) = value;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_FAN_PARTS) {
        if (value != 1 && value != 4 && value != 16)
            return fl_set_error(FL_ERR_INVALID, "fl_plan_option: %d parts (1, 4 or 16)", value);
        p->fan_lanes = value;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_FAN_BLOCK) {
        if (value != 1 && value != 2)
            return fl_set_error(FL_ERR_INVALID, "fl_plan_option: pixel block %d (1 or 2)", value);
        p->fan_block = value;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_DEBUG_TMA_STALL) {
        if (value < 0 || value > (1 << 20))
            return fl_set_error(FL_ERR_INVALID, "fl_plan_option: %d polls (0 .. 2^20)", value);
        p->tma_stall = value;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_FAN_TMA) {
        if (value != 0 && value != 1)
            return fl_set_error(FL_ERR_INVALID, "fl_plan_option: %d (0 or 1)", value);
        p->fan_tma_ok = p->s.ndim == 2 && value && fl_tma_available() ? 1 : 0;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_ADJ_CHUNKS) {
        if (value < 1 || value > 64)
            return fl_set_error(FL_ERR_INVALID, "fl_plan_option: %d view chunks (1 .. 64)", value);
        p->adj_chunks = value;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_FAN_GROUPS) {
        if (value != 8 && value != 16)
            return fl_set_error(FL_ERR_INVALID, "fl_plan_option: %d view groups (8 or 16)", value);
        p->fan_groups = value;
        return fl_set_error(FL_OK, "");
    }
    return fl_set_error(FL_ERR_INVALID, "fl_plan_option: unknown option %d", option);
}

extern "C" int fl_plan_query(const fl_plan* p, int option, int* value)
{
    if (!p || !value) return fl_set_error(FL_ERR_INVALID, "fl_plan_query: null argument");
    if (option == FL_OPT_Z_MIRROR) {
        *value = p->zmirror;
        return fl_set_error(FL_OK, "");
    }
    const int form = fl_plan_form(p);
    if (option == FL_OPT_ROT_MIRROR) {
        *value = (form >= FL_FORM_HALF && form != FL_FORM_REFL) ? 1 : 0;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_OPT_QUARTER_TURN) {
        *value = (form == FL_FORM_QUARTER || form == FL_FORM_QUARTER_REFL) ? 1 : 0;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_OPT_REFLECT) {
        *value = fl_plan_refl(p) ? 1 : 0;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_ADJ_RUN) {
        *value = p->adj_run == 1 ? 1 : 2;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_ADJ_ROWS) {
        *value = p->adj_rows ? p->adj_rows : 1;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_FAN_PARTS) {
        *value = fl_plan_fan_lanes(p);
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_FAN_BLOCK) {
        *value = fl_plan_fan_block(p);
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_FAN_GROUPS) {
        *value = fl_plan_fan_groups(p);
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_ADJ_CHUNKS) {
        *value = fl_plan_refl(p) && p->s.ndim == 3 ? fl_plan_adj_chunks(p, true) : 1;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_TUNE_FAN_TMA) {
        *value = p->fan_tma_ok;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_DEBUG_TMA_TIMEOUTS) {          // and clears the flag
        const int st = fl_plan_take_timeouts(const_cast<fl_plan*>(p), nullptr);
        *value = st == FL_ERR_TIMEOUT;
        if (st && st != FL_ERR_TIMEOUT) return st;
        return fl_set_error(FL_OK, "");
    }
    if (option == FL_DEBUG_TMA_STALL) {
        *value = p->tma_stall;
        return fl_set_error(FL_OK, "");
    }
    return fl_set_error(FL_ERR_INVALID, "fl_plan_query: unknown option %d", option);
}

int fl_plan_take_timeouts(fl_plan* p, cudaStream_t s)
{
    if (!p || !p->d_tma_err) return FL_OK;
    int v = 0;
    int st = fl_check_cuda(cudaMemcpyAsync(&v, p->d_tma_err, sizeof v, cudaMemcpyDeviceToHost, s),
                           "cudaMemcpyAsync");
    if (!st) st = fl_check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (st || !v) return st;
    st = fl_check_cuda(cudaMemsetAsync(p->d_tma_err, 0, sizeof v, s), "cudaMemsetAsync");
    if (!st) st = fl_check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (st) return st;
    return fl_set_error(FL_ERR_TIMEOUT,
                        "a TMA tile load of the fan forward's transposed copy did not arrive "
                        "within its bounded wait: the projections since the last check are "
                        "incomplete");
}

extern "C" int fl_plan_create(const fl_scan* scan, fl_plan** out)
{
    FL_RANGE("fl_plan_create");
    if (!scan || !out) return fl_set_error(FL_ERR_INVALID, "fl_plan_create: null argument");
    *out = nullptr;
    fl_scan s = *scan;
    if (s.ndim != 2 && s.ndim != 3)
        return fl_set_error(FL_ERR_INVALID, "ndim must be 2 (fan) or 3 (cone)");
    if (s.ndim == 2) { s.nz = 1; s.nb = 1; s.dz = 1.0f; }
    if (s.nt < 1) s.nt = 1;
    if (s.nx < 1 || s.ny < 1 || s.nz < 1 || s.nv < 1 || s.na < 1 || s.nb < 1)
        return fl_set_error(FL_ERR_INVALID, "sizes must be positive");
    if ((int64_t)s.nx * s.ny * s.nz >= (int64_t)1 << 31)
        return fl_set_error(FL_ERR_UNSUPPORTED, "a frame must hold fewer than 2^31 voxels");
    // views, detector rows and image rows index grid dimensions y / z
    if (s.nv > 65535 || s.nb > 65535 || s.ny > 65535 || s.nt > 65535)
        return fl_set_error(FL_ERR_UNSUPPORTED,
                            "at most 65535 views, detector rows, image rows and frames per plan");
    if (!(s.SO > 0) || !(s.OD > -s.SO) || !(s.scale > 0) || !(s.dz > 0))
        return fl_set_error(FL_ERR_INVALID, "SO, SO+OD, scale and dz must be positive");
    if ((!s.sd_phi && !(s.cos_phi && s.sin_phi)) || !s.y_det || (s.ndim == 3 && !s.z_det))
        return fl_set_error(FL_ERR_INVALID, "geometry arrays missing");

    fl_plan* p = new (std::nothrow) fl_plan;
    if (!p) return fl_set_error(FL_ERR_ALLOC, "fl_plan_create: out of host memory");
    std::memset((void*)p, 0, sizeof *p);
    p->s = s;
    p->n_vox_frame = (int64_t)s.nx * s.ny * s.nz;
    p->n_vox = p->n_vox_frame * s.nt;
    p->n_rays = (int64_t)s.nv * s.na * s.nb;
    const int nv = s.nv, na = s.na, nb = s.nb, nt = s.nt;

    std::vector<float> phi(nv), cphi(nv), sphi(nv), cf(nv), sf(nv), sdz(nv, 0.0f);
    for (int iv = 0; iv < nv; iv++) {
        phi[iv] = s.sd_phi ? s.sd_phi[iv] : (float)std::atan2((double)s.sin_phi[iv], (double)s.cos_phi[iv]);
        // the reference Siddon evaluates cos/sin of a float (C++ float overloads)
        cf[iv] = std::cos(phi[iv]);
        sf[iv] = std::sin(phi[iv]);
        cphi[iv] = s.cos_phi ? s.cos_phi[iv] : (float)std::cos((double)phi[iv]);
        sphi[iv] = s.sin_phi ? s.sin_phi[iv] : (float)std::sin((double)phi[iv]);
        if (s.sd_z) sdz[iv] = s.sd_z[iv];
    }
    std::vector<float> cdet(na), sdet(na);
    for (int ia = 0; ia < na; ia++) {
        if (s.cos_det && s.sin_det) { cdet[ia] = s.cos_det[ia]; sdet[ia] = s.sin_det[ia]; }
        else {
            float ang = (float)std::atan2((double)s.y_det[ia], (double)(s.SO + s.OD));
            cdet[ia] = (float)std::cos((double)ang);
            sdet[ia] = (float)std::sin((double)ang);
        }
    }
    // finite-beam bin edges: backprojector trig (cos_det2/sin_det2, given or as
    // setPara-style singles) and the forward's edge lines with the float libm
    // calls of Ax_fan_mf_cpu_new_fb.cpp:36-46
    std::vector<float> cdet2(na + 1), sdet2(na + 1), fbe;
    if (s.ndim == 2) {
        for (int e = 0; e <= na; e++) {
            if (s.cos_det2 && s.sin_det2) { cdet2[e] = s.cos_det2[e]; sdet2[e] = s.sin_det2[e]; }
            else {
                float u = (e < na) ? s.y_det[e] - s.dy_det / 2 : s.y_det[na - 1] + s.dy_det / 2;
                float ang = (float)std::atan2((double)u, (double)(s.SO + s.OD));
                cdet2[e] = (float)std::cos((double)ang);
                sdet2[e] = (float)std::sin((double)ang);
            }
        }
        if (s.dy_det > 0) {
            fbe.resize((size_t)nv * na * 6);
            const float SD = s.SO + s.OD;
            for (int iv = 0; iv < nv; iv++)
                for (int ia = 0; ia < na; ia++)
                    for (int e = 0; e < 2; e++) {
                        float u = e ? s.y_det[ia] + s.dy_det / 2 : s.y_det[ia] - s.dy_det / 2;
                        float ang = std::atan2(u, SD);
                        float* E = &fbe[((size_t)iv * na + ia) * 6 + 3 * e];
                        E[0] = -std::sin(ang + phi[iv]);
                        E[1] = std::cos(ang + phi[iv]);
                        E[2] = s.SO * std::sin(ang);
                    }
        }
    }
    std::vector<int32_t> vframe(nv, 0);
    for (int iv = 0; iv < nv; iv++) {
        vframe[iv] = s.view_frame ? s.view_frame[iv] : 0;
        if (vframe[iv] < 0 || vframe[iv] >= nt) {
            delete p;
            return fl_set_error(FL_ERR_INVALID, "view %d reads frame %d (nt = %d)", iv, vframe[iv], nt);
        }
    }
    std::vector<int32_t> idY, Nvv(nt, 0);
    int tmp = 0;
    if (s.id_Y && s.Nv) {
        tmp = s.tmp_size;
        for (int it = 0; it < nt; it++) {
            Nvv[it] = s.Nv[it];
            if (Nvv[it] < 0 || Nvv[it] > tmp) {
                delete p;
                return fl_set_error(FL_ERR_INVALID, "Nv[%d] = %d outside [0, tmp_size]", it, Nvv[it]);
            }
        }
        idY.assign(s.id_Y, s.id_Y + (size_t)tmp * nt);
        for (int it = 0; it < nt; it++)
            for (int j = 0; j < Nvv[it]; j++) {
                int iv = idY[(size_t)it * tmp + j];
                if (iv < 0 || iv >= nv) {
                    delete p;
                    return fl_set_error(FL_ERR_INVALID, "id_Y entry %d out of range", iv);
                }
            }
    } else {
        for (int iv = 0; iv < nv; iv++) Nvv[vframe[iv]]++;
        for (int it = 0; it < nt; it++) tmp = tmp > Nvv[it] ? tmp : Nvv[it];
        idY.assign((size_t)tmp * nt, 0);
        std::vector<int> fill(nt, 0);
        for (int iv = 0; iv < nv; iv++) idY[(size_t)vframe[iv] * tmp + fill[vframe[iv]]++] = iv;
    }
    if (tmp < 1) tmp = 1, idY.resize((size_t)nt, 0);
    p->tmp_size = tmp;
    p->views_natural = nt == 1 && Nvv[0] == nv;
    for (int j = 0; j < Nvv[0] && p->views_natural; j++)
        if (idY[j] != j) p->views_natural = 0;

    int st = FL_OK;
    if (!st) st = upload(&p->d_sd_phi, phi.data(), nv);
    if (!st) st = upload(&p->d_sd_z, sdz.data(), nv);
    if (!st) st = upload(&p->d_y_det, s.y_det, na);
    if (!st && s.ndim == 3) st = upload(&p->d_z_det, s.z_det, nb);
    if (!st) st = upload(&p->d_cos_phi, cphi.data(), nv);
    if (!st) st = upload(&p->d_sin_phi, sphi.data(), nv);
    if (!st) st = upload(&p->d_cphi_f, cf.data(), nv);
    if (!st) st = upload(&p->d_sphi_f, sf.data(), nv);
    if (!st) st = upload(&p->d_cos_det, cdet.data(), na);
    if (!st) st = upload(&p->d_sin_det, sdet.data(), na);
    if (!st) st = upload(&p->d_view_frame, vframe.data(), nv);
    if (!st && s.ndim == 2) st = upload(&p->d_cos_det2, cdet2.data(), na + 1);
    if (!st && s.ndim == 2) st = upload(&p->d_sin_det2, sdet2.data(), na + 1);
    if (!st && !fbe.empty()) st = upload(&p->d_fb_edges, fbe.data(), fbe.size());
    if (!st) st = upload(&p->d_idY, idY.data(), idY.size());
    if (!st) st = upload(&p->d_Nv, Nvv.data(), nt);
    if (!st) st = build_tables(p, phi, s.sd_z ? sdz.data() : nullptr, s.y_det, s.z_det);
    // host copies of the arrays are not kept: clear the caller's pointers
    p->s.sd_phi = p->s.sd_z = p->s.y_det = p->s.z_det = nullptr;
    p->s.cos_phi = p->s.sin_phi = p->s.cos_det = p->s.sin_det = nullptr;
    p->s.view_frame = p->s.id_Y = p->s.Nv = nullptr;
    p->s.cos_det2 = p->s.sin_det2 = nullptr;
    // fan plans: the forward's transposed copy of its input (matched.cu)
    if (!st && s.ndim == 2)
        st = fl_check_cuda(fl_malloc(&p->d_xt, (size_t)p->n_vox * sizeof(float)),
                           "fl_malloc(plan)");
    if (!st && s.ndim == 2) {
        st = fl_check_cuda(fl_malloc((void**)&p->d_tma_err, sizeof(int)), "fl_malloc(plan)");
        if (!st) st = fl_check_cuda(cudaMemset(p->d_tma_err, 0, sizeof(int)), "cudaMemset(plan)");
        p->fan_tma_ok = fl_tma_available() ? 1 : 0;
    }
    // quarter-turn reflection plans: the diagonal columns' second sums
    // between view chunks of the backprojection (matched.cu)
    if (!st && s.ndim == 3 && p->refl4_ok)
        st = fl_check_cuda(fl_malloc((void**)&p->d_dq, (size_t)(s.nx / 2) * (s.nz / 2) * 4 *
                                                           sizeof(float2)),
                           "fl_malloc(plan)");
    if (st) {
        free_plan_arrays(p);
        delete p;
        return st;
    }
    *out = p;
    return fl_set_error(FL_OK, "");
}

extern "C" void fl_plan_destroy(fl_plan* p)
{
    if (!p) return;
    free_plan_arrays(p);
    delete p;
}

extern "C" int fl_plan_sizes(const fl_plan* p, int64_t* n_vox, int64_t* n_rays)
{
    if (!p) return fl_set_error(FL_ERR_INVALID, "null plan");
    if (n_vox) *n_vox = p->n_vox;
    if (n_rays) *n_rays = p->n_rays;
    return FL_OK;
}

static int check_dtype(int t)
{
    if (t != FL_F32 && t != FL_F16 && t != FL_BF16)
        return fl_set_error(FL_ERR_INVALID, "unknown dtype %d", t);
    return FL_OK;
}

int fl_matched_ready(fl_plan* p)
{
    const fl_scan& s = p->s;
    double r = std::sqrt(0.25 * s.nx * s.nx + 0.25 * s.ny * s.ny) + 1.0;
    if (!(s.SO > r))
        return fl_set_error(FL_ERR_UNSUPPORTED,
                            "matched model needs the source outside the volume (SO > %.1f)", r);
    return FL_OK;
}

extern "C" int fl_forward(fl_plan* p, int model, const void* x, int xt, void* y, int yt,
                          void* stream)
{
    FL_RANGE("fl_forward");
    if (!p || !x || !y) return fl_set_error(FL_ERR_INVALID, "fl_forward: null argument");
    int st;
    if ((st = check_dtype(xt)) || (st = check_dtype(yt))) return st;
    cudaStream_t sm = (cudaStream_t)stream;
    if (model == FL_MODEL_SIDDON_REF) {
        if (xt != FL_F32 || yt != FL_F32)
            return fl_set_error(FL_ERR_UNSUPPORTED, "reference Siddon is FP32 only");
        return fl_ref_forward(p, (const float*)x, (float*)y, sm);
    }
    if (model == FL_MODEL_MATCHED) {
        if ((st = fl_matched_ready(p))) return st;
        return fl_matched_forward(p, x, xt, y, yt, 1, nullptr, nullptr, 0, sm);
    }
    if (model == FL_MODEL_GAO_REF) {
        if (xt != FL_F32 || yt != FL_F32)
            return fl_set_error(FL_ERR_UNSUPPORTED, "reference dominant-axis forward is FP32 only");
        return fl_ref_gao_forward(p, (const float*)x, (float*)y, nullptr, sm);
    }
    if (model == FL_MODEL_FB_REF) {
        if (xt != FL_F32 || yt != FL_F32)
            return fl_set_error(FL_ERR_UNSUPPORTED, "reference finite-beam model is FP32 only");
        return fl_ref_fb_forward(p, (const float*)x, (float*)y, sm);
    }
    return fl_set_error(FL_ERR_UNSUPPORTED, "fl_forward: model %d not available", model);
}

// scratch for the pre-weighted adjoint input, owned by the plan
int fl_plan_vwork(fl_plan* p, size_t bytes, void** w)
{
    if (p->vwork_bytes < bytes) {
        if (p->d_vwork) cudaFree(p->d_vwork);
        p->d_vwork = nullptr;
        p->vwork_bytes = 0;
        int st = fl_check_cuda(fl_malloc(&p->d_vwork, bytes), "fl_malloc(volume scratch)");
        if (st) return st;
        p->vwork_bytes = bytes;
    }
    *w = p->d_vwork;
    return FL_OK;
}

int fl_plan_work(fl_plan* p, float** w)
{
    size_t need = (size_t)p->n_rays;
    if (p->work_elems < need) {
        if (p->d_work) cudaFree(p->d_work);
        p->d_work = nullptr;
        p->work_elems = 0;
        int st = fl_check_cuda(fl_malloc((void**)&p->d_work, need * sizeof(float)),
                               "fl_malloc(adjoint scratch)");
        if (st) return st;
        p->work_elems = need;
    }
    *w = p->d_work;
    return FL_OK;
}

extern "C" int fl_adjoint(fl_plan* p, int model, const void* y, int yt, void* x, int xt,
                          void* stream)
{
    FL_RANGE("fl_adjoint");
    if (!p || !x || !y) return fl_set_error(FL_ERR_INVALID, "fl_adjoint: null argument");
    int st;
    if ((st = check_dtype(xt)) || (st = check_dtype(yt))) return st;
    cudaStream_t sm = (cudaStream_t)stream;
    if (model == FL_MODEL_CHORD_REF) {
        if (xt != FL_F32 || yt != FL_F32)
            return fl_set_error(FL_ERR_UNSUPPORTED, "reference backprojector is FP32 only");
        return fl_ref_adjoint(p, (const float*)y, (float*)x, sm);
    }
    if (model == FL_MODEL_FB_REF) {
        if (xt != FL_F32 || yt != FL_F32)
            return fl_set_error(FL_ERR_UNSUPPORTED, "reference finite-beam model is FP32 only");
        return fl_ref_fb_adjoint(p, (const float*)y, (float*)x, sm);
    }
    if (model == FL_MODEL_MATCHED) {
        if ((st = fl_matched_ready(p))) return st;
        if (p->det_kind < 0)
            return fl_set_error(FL_ERR_UNSUPPORTED,
                                "matched adjoint needs a uniform flat or equiangular detector");
        if (p->det_kind == 1 && p->s.ndim == 3)
            return fl_set_error(FL_ERR_UNSUPPORTED, "equiangular detector is fan-beam only");
        float* w;
        if ((st = fl_plan_work(p, &w))) return st;
        if ((st = fl_matched_weight(p, y, yt, w, sm))) return st;
        return fl_matched_adjoint_w(p, w, x, xt, nullptr, 0, sm);
    }
    return fl_set_error(FL_ERR_UNSUPPORTED, "fl_adjoint: model %d not available", model);
}

extern "C" int fl_forward_gao(fl_plan* p, const float* x, float* y, float* ynorm, void* stream)
{
    FL_RANGE("fl_forward_gao");
    if (!p || !x || !y) return fl_set_error(FL_ERR_INVALID, "fl_forward_gao: null argument");
    return fl_ref_gao_forward(p, x, y, ynorm, (cudaStream_t)stream);
}

extern "C" int fl_count_intersections(fl_plan* p, int32_t* counts, void* stream)
{
    FL_RANGE("fl_count_intersections");
    if (!p || !counts) return fl_set_error(FL_ERR_INVALID, "null argument");
    int st = fl_matched_ready(p);
    if (st) return st;
    return fl_matched_count(p, counts, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// Drop-ins: host pointers in/out, one synchronous call, like the reference.
// ---------------------------------------------------------------------------
namespace {
struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    int alloc(size_t bytes) { return fl_check_cuda(fl_malloc(&p, bytes ? bytes : 4), "cudaMalloc"); }
};
struct PlanGuard {
    fl_plan* p = nullptr;
    ~PlanGuard() { fl_plan_destroy(p); }
};

// frames from (id_Y, Nv, tmp_size): view -> frame
std::vector<int32_t> frames_of(const int* id_Y, const int* Nv, int nt, int tmp, int nv, int* bad)
{
    std::vector<int32_t> f(nv, 0);
    *bad = 0;
    for (int it = 0; it < nt; it++)
        for (int j = 0; j < Nv[it]; j++) {
            int iv = id_Y[(size_t)it * tmp + j];
            if (iv < 0 || iv >= nv) { *bad = 1; continue; }
            f[iv] = it;
        }
    return f;
}

int run_forward_host(const fl_scan& s, int model, const float* X, float* y)
{
    PlanGuard g;
    int st = fl_plan_create(&s, &g.p);
    if (st) return st;
    DevBuf dx, dy;
    size_t nvox = (size_t)g.p->n_vox, nray = (size_t)g.p->n_rays;
    if ((st = dx.alloc(nvox * 4)) || (st = dy.alloc(nray * 4))) return st;
    if ((st = fl_check_cuda(cudaMemcpy(dx.p, X, nvox * 4, cudaMemcpyHostToDevice), "H2D"))) return st;
    if ((st = fl_forward(g.p, model, dx.p, FL_F32, dy.p, FL_F32, nullptr))) return st;
    if ((st = fl_check_cuda(cudaMemcpy(y, dy.p, nray * 4, cudaMemcpyDeviceToHost), "D2H"))) return st;
    return fl_set_error(FL_OK, "");
}

int run_gao_host(const fl_scan& s, const float* X, float* y, float* ynorm)
{
    PlanGuard g;
    int st = fl_plan_create(&s, &g.p);
    if (st) return st;
    DevBuf dx, dy, dn;
    size_t nvox = (size_t)g.p->n_vox, nray = (size_t)g.p->n_rays;
    if ((st = dx.alloc(nvox * 4)) || (st = dy.alloc(nray * 4))) return st;
    if (ynorm && (st = dn.alloc(nray * 4))) return st;
    if ((st = fl_check_cuda(cudaMemcpy(dx.p, X, nvox * 4, cudaMemcpyHostToDevice), "H2D"))) return st;
    if ((st = fl_ref_gao_forward(g.p, (const float*)dx.p, (float*)dy.p, (float*)dn.p, nullptr))) return st;
    if ((st = fl_check_cuda(cudaMemcpy(y, dy.p, nray * 4, cudaMemcpyDeviceToHost), "D2H"))) return st;
    if (ynorm && (st = fl_check_cuda(cudaMemcpy(ynorm, dn.p, nray * 4, cudaMemcpyDeviceToHost), "D2H")))
        return st;
    return fl_set_error(FL_OK, "");
}

int run_adjoint_host(const fl_scan& s, int model, const float* Y, float* x)
{
    PlanGuard g;
    int st = fl_plan_create(&s, &g.p);
    if (st) return st;
    DevBuf dx, dy;
    size_t nvox = (size_t)g.p->n_vox, nray = (size_t)g.p->n_rays;
    if ((st = dx.alloc(nvox * 4)) || (st = dy.alloc(nray * 4))) return st;
    if ((st = fl_check_cuda(cudaMemcpy(dy.p, Y, nray * 4, cudaMemcpyHostToDevice), "H2D"))) return st;
    if ((st = fl_adjoint(g.p, model, dy.p, FL_F32, dx.p, FL_F32, nullptr))) return st;
    if ((st = fl_check_cuda(cudaMemcpy(x, dx.p, nvox * 4, cudaMemcpyDeviceToHost), "D2H"))) return st;
    return fl_set_error(FL_OK, "");
}
}  // namespace

extern "C" void Ax_fan_mf_gpu_siddon(float* X, float* y, float SO, float OD, float scale, int nx,
                                     int ny, int nv, float* sd_phi, int nd, float* y_det,
                                     int* id_X, int nt)
{
    FL_RANGE("Ax_fan_mf_gpu_siddon");
    fl_scan s;
    std::memset(&s, 0, sizeof s);
    s.ndim = 2; s.nx = nx; s.ny = ny; s.nz = 1; s.nt = nt; s.nv = nv; s.na = nd; s.nb = 1;
    s.SO = SO; s.OD = OD; s.scale = scale; s.dz = 1.0f;
    s.sd_phi = sd_phi; s.y_det = y_det; s.view_frame = id_X;
    run_forward_host(s, FL_MODEL_SIDDON_REF, X, y);
}

extern "C" void Atx_fan_mf_gpu_new(float* x, float* Y, float SO, float OD, float scale, int nx,
                                   int ny, float* sd_phi, int nd, float* y_det, float dy_det,
                                   float y_os, int nt, int* id_Y, int* Nv, int tmp_size, int nv,
                                   float* cos_phi, float* sin_phi, float* cos_det,
                                   float* sin_det)
{
    FL_RANGE("Atx_fan_mf_gpu_new");
    fl_scan s;
    std::memset(&s, 0, sizeof s);
    s.ndim = 2; s.nx = nx; s.ny = ny; s.nz = 1; s.nt = nt; s.nv = nv; s.na = nd; s.nb = 1;
    s.SO = SO; s.OD = OD; s.scale = scale; s.dz = 1.0f; s.dy_det = dy_det; s.y_os = y_os;
    s.sd_phi = sd_phi; s.y_det = y_det; s.cos_phi = cos_phi; s.sin_phi = sin_phi;
    s.cos_det = cos_det; s.sin_det = sin_det;
    s.id_Y = id_Y; s.Nv = Nv; s.tmp_size = tmp_size;
    int bad;
    std::vector<int32_t> vf = frames_of(id_Y, Nv, nt, tmp_size, nv, &bad);
    if (bad) { fl_set_error(FL_ERR_INVALID, "id_Y entry out of range"); return; }
    s.view_frame = vf.data();
    run_adjoint_host(s, FL_MODEL_CHORD_REF, Y, x);
}

extern "C" void Ax_cone_mf_gpu_siddon(float* X, float* y, float* sd_phi, float* sd_z,
                                      float* y_det, float* z_det, int* id_Y, int* Nv, float SO,
                                      float OD, float scale, float dz, int nx, int ny, int nz,
                                      int nt, int na, int nb, int nv, int tmp_size, int nv_block)
{
    FL_RANGE("Ax_cone_mf_gpu_siddon");
    (void)nv_block;
    fl_scan s;
    std::memset(&s, 0, sizeof s);
    s.ndim = 3; s.nx = nx; s.ny = ny; s.nz = nz; s.nt = nt; s.nv = nv; s.na = na; s.nb = nb;
    s.SO = SO; s.OD = OD; s.scale = scale; s.dz = dz;
    s.sd_phi = sd_phi; s.sd_z = sd_z; s.y_det = y_det; s.z_det = z_det;
    int bad;
    std::vector<int32_t> vf = frames_of(id_Y, Nv, nt, tmp_size, nv, &bad);
    if (bad) { fl_set_error(FL_ERR_INVALID, "id_Y entry out of range"); return; }
    s.view_frame = vf.data();
    s.id_Y = id_Y; s.Nv = Nv; s.tmp_size = tmp_size;
    run_forward_host(s, FL_MODEL_SIDDON_REF, X, y);
}

extern "C" void Atx_cone_mf_gpu_new(float* X, float* y, float* cos_phi, float* sin_phi,
                                    float* sd_z, float* y_det, float* z_det, int* id_Y, int* Nv,
                                    float SO, float OD, float scale, float dy_det, float y_os,
                                    float dz_det, float dz, int nx, int ny, int nz, int nt,
                                    int na, int nb, int nv, int tmp_size, int nv_block)
{
    FL_RANGE("Atx_cone_mf_gpu_new");
    (void)nv_block;
    fl_scan s;
    std::memset(&s, 0, sizeof s);
    s.ndim = 3; s.nx = nx; s.ny = ny; s.nz = nz; s.nt = nt; s.nv = nv; s.na = na; s.nb = nb;
    s.SO = SO; s.OD = OD; s.scale = scale; s.dz = dz;
    s.dy_det = dy_det; s.y_os = y_os; s.dz_det = dz_det;
    s.cos_phi = cos_phi; s.sin_phi = sin_phi; s.sd_z = sd_z; s.y_det = y_det; s.z_det = z_det;
    int bad;
    std::vector<int32_t> vf = frames_of(id_Y, Nv, nt, tmp_size, nv, &bad);
    if (bad) { fl_set_error(FL_ERR_INVALID, "id_Y entry out of range"); return; }
    s.view_frame = vf.data();
    s.id_Y = id_Y; s.Nv = Nv; s.tmp_size = tmp_size;
    run_adjoint_host(s, FL_MODEL_CHORD_REF, y, X);
}

extern "C" void Ax_fan_mf_gpu_new(float* X, float* y, float SO, float OD, float scale, int nx,
                                  int ny, int nv, float* sd_phi, int nd, float* y_det,
                                  int* id_X, int nt)
{
    FL_RANGE("Ax_fan_mf_gpu_new");
    fl_scan s;
    std::memset(&s, 0, sizeof s);
    s.ndim = 2; s.nx = nx; s.ny = ny; s.nz = 1; s.nt = nt; s.nv = nv; s.na = nd; s.nb = 1;
    s.SO = SO; s.OD = OD; s.scale = scale; s.dz = 1.0f;
    s.sd_phi = sd_phi; s.y_det = y_det; s.view_frame = id_X;
    run_gao_host(s, X, y, nullptr);
}

extern "C" void Ax_cone_mf_gpu_new(float* X, float* y, float* yNorm, float* sd_phi, float* sd_z,
                                   float* y_det, float* z_det, int* id_Y, int* Nv, float SO,
                                   float OD, float scale, float dz, int nx, int ny, int nz,
                                   int nt, int na, int nb, int nv, int tmp_size, int nv_block)
{
    FL_RANGE("Ax_cone_mf_gpu_new");
    (void)nv_block;
    fl_scan s;
    std::memset(&s, 0, sizeof s);
    s.ndim = 3; s.nx = nx; s.ny = ny; s.nz = nz; s.nt = nt; s.nv = nv; s.na = na; s.nb = nb;
    s.SO = SO; s.OD = OD; s.scale = scale; s.dz = dz;
    s.sd_phi = sd_phi; s.sd_z = sd_z; s.y_det = y_det; s.z_det = z_det;
    int bad;
    std::vector<int32_t> vf = frames_of(id_Y, Nv, nt, tmp_size, nv, &bad);
    if (bad) { fl_set_error(FL_ERR_INVALID, "id_Y entry out of range"); return; }
    s.view_frame = vf.data();
    s.id_Y = id_Y; s.Nv = Nv; s.tmp_size = tmp_size;
    run_gao_host(s, X, y, yNorm);
}

extern "C" void Ax_fan_mf_gpu_new_fb(float* X, float* y, float SO, float OD, float scale, int nx,
                                     int ny, int nv, float* sd_phi, int nd, float* y_det,
                                     int* id_X, int nt, float dy_det)
{
    FL_RANGE("Ax_fan_mf_gpu_new_fb");
    fl_scan s;
    std::memset(&s, 0, sizeof s);
    s.ndim = 2; s.nx = nx; s.ny = ny; s.nz = 1; s.nt = nt; s.nv = nv; s.na = nd; s.nb = 1;
    s.SO = SO; s.OD = OD; s.scale = scale; s.dz = 1.0f; s.dy_det = dy_det;
    s.sd_phi = sd_phi; s.y_det = y_det; s.view_frame = id_X;
    run_forward_host(s, FL_MODEL_FB_REF, X, y);
}

extern "C" void Atx_fan_mf_gpu_new_fb(float* x, float* Y, float SO, float OD, float scale, int nx,
                                      int ny, float* sd_phi, int nd, float* y_det, float dy_det,
                                      int nt, int* id_Y, int* Nv, int tmp_size, int nv,
                                      float* cos_phi, float* sin_phi, float* cos_det,
                                      float* sin_det)
{
    FL_RANGE("Atx_fan_mf_gpu_new_fb");
    fl_scan s;
    std::memset(&s, 0, sizeof s);
    s.ndim = 2; s.nx = nx; s.ny = ny; s.nz = 1; s.nt = nt; s.nv = nv; s.na = nd; s.nb = 1;
    s.SO = SO; s.OD = OD; s.scale = scale; s.dz = 1.0f; s.dy_det = dy_det;
    s.sd_phi = sd_phi; s.y_det = y_det; s.cos_phi = cos_phi; s.sin_phi = sin_phi;
    s.cos_det2 = cos_det; s.sin_det2 = sin_det;
    s.id_Y = id_Y; s.Nv = Nv; s.tmp_size = tmp_size;
    int bad;
    std::vector<int32_t> vf = frames_of(id_Y, Nv, nt, tmp_size, nv, &bad);
    if (bad) { fl_set_error(FL_ERR_INVALID, "id_Y entry out of range"); return; }
    s.view_frame = vf.data();
    run_adjoint_host(s, FL_MODEL_FB_REF, Y, x);
}
