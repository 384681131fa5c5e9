// fl_common.cuh -- shared helpers for the FrameLab-GB300 kernels.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "framelab_gb300.h"

// ---------------------------------------------------------------------------
// Pinned single-precision arithmetic.
//
// nvcc contracts a*b+c into one FMA by default; the reference's CPU kernels
// round every product and sum separately (x86-64 build, no FMA). Kernels
// that must reproduce the reference bit for bit use these explicit
// round-to-nearest intrinsics, which the compiler never fuses or reorders.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }
// |a| exactly as `a>0?a:-(a)` (equal to fabsf for every non-NaN input)
__device__ __forceinline__ float fabs_ref(float a) { return fabsf(a); }

// ---------------------------------------------------------------------------
// Storage types. Volumes and sinograms may be stored as f32, f16 or bf16;
// arithmetic is always f32.
// ---------------------------------------------------------------------------
template <typename T> struct Store;
// ld2/st2: the two adjacent elements p[0], p[1] (p 2-element aligned) as one
// access -- a voxel and its mirror in the z-folded layout (fl_plan.h).
template <> struct Store<float> {
    static __device__ __forceinline__ float ld(const float* p) { return __ldg(p); }
    static __device__ __forceinline__ float ld_plain(const float* p) { return *p; }
    static __device__ __forceinline__ void st(float* p, float v) { *p = v; }
    static __device__ __forceinline__ float2 ld2(const float* p)
    {
        return __ldg(reinterpret_cast<const float2*>(p));
    }
    static __device__ __forceinline__ void st2(float* p, float a, float b)
    {
        *reinterpret_cast<float2*>(p) = make_float2(a, b);
    }
};
template <> struct Store<__half> {
    static __device__ __forceinline__ float ld(const __half* p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ float ld_plain(const __half* p) { return __half2float(*p); }
    static __device__ __forceinline__ void st(__half* p, float v) { *p = __float2half_rn(v); }
    static __device__ __forceinline__ float2 ld2(const __half* p)
    {
        return __half22float2(__ldg(reinterpret_cast<const __half2*>(p)));
    }
    static __device__ __forceinline__ void st2(__half* p, float a, float b)
    {
        *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a, b);
    }
};
template <> struct Store<__nv_bfloat16> {
    static __device__ __forceinline__ float ld(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }
    static __device__ __forceinline__ float ld_plain(const __nv_bfloat16* p) { return __bfloat162float(*p); }
    static __device__ __forceinline__ void st(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }
    static __device__ __forceinline__ float2 ld2(const __nv_bfloat16* p)
    {
        return __bfloat1622float2(__ldg(reinterpret_cast<const __nv_bfloat162*>(p)));
    }
    static __device__ __forceinline__ void st2(__nv_bfloat16* p, float a, float b)
    {
        *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(a, b);
    }
};

// ---------------------------------------------------------------------------
// Bounds-checked builds (-DFL_BOUNDS_CHECK). FL_IN(i, n) is true when
// 0 <= i < n; otherwise it counts a violation in this translation unit's
// counter and the caller skips the access. In normal builds it is the
// constant true and costs nothing. FL_OOB_ACCESSOR(name) defines the host
// function that reads (and optionally clears) the counter.
// ---------------------------------------------------------------------------
#if defined(FL_BOUNDS_CHECK) && defined(__CUDACC__)
static __device__ unsigned long long fl_oob_count;
__device__ __forceinline__ bool fl_in(long long i, long long n)
{
    if (i >= 0 && i < n) return true;
    atomicAdd(&fl_oob_count, 1ULL);
    return false;
}
#define FL_IN(i, n) fl_in((long long)(i), (long long)(n))
#define FL_OOB_ACCESSOR(name)                                                         \
    extern "C" unsigned long long name(int reset)                                     \
    {                                                                                 \
        unsigned long long v = 0, z = 0;                                              \
        cudaMemcpyFromSymbol(&v, fl_oob_count, sizeof v);                             \
        if (reset) cudaMemcpyToSymbol(fl_oob_count, &z, sizeof z);                    \
        return v;                                                                     \
    }
#else
#define FL_IN(i, n) true
#define FL_OOB_ACCESSOR(name) \
    extern "C" unsigned long long name(int) { return 0; }
#endif

// ---------------------------------------------------------------------------
// Host-side status handling (fl_runtime.cpp).
// ---------------------------------------------------------------------------
int fl_set_error(int code, const char* fmt, ...);
// Every device allocation of the library goes through fl_malloc, so a test can
// make the n-th one fail (fl_debug_fail_alloc) and check the error paths.
cudaError_t fl_malloc(void** p, size_t bytes);
int fl_check_cuda(cudaError_t e, const char* what);
int fl_check_launch(const char* what);
#define FL_CUDA(call)                                                     \
    do {                                                                  \
        int _st = fl_check_cuda((call), #call);                           \
        if (_st != FL_OK) return _st;                                     \
    } while (0)

static inline unsigned fl_div_up(long long a, long long b) { return (unsigned)((a + b - 1) / b); }
