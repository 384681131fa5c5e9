// noalloc.cu -- matched backprojection that allocates no device memory.
//
// fl_adjoint (FL_MODEL_MATCHED) first writes the sinogram multiplied by each
// ray's length factor into a scratch buffer, then gathers from it. It takes
// that buffer from the plan and allocates it with cudaMalloc on first use.
// Some callers cannot allocate at that point: code being captured into a CUDA
// graph (cudaMalloc is not allowed while a stream is capturing), a host
// application that hands the GPU's memory to its own pool allocator and
// forbids others from calling cudaMalloc (a MATLAB session managing gpuArray
// memory, for example), or a real-time loop that must not block on the
// allocator. fl_adjoint_noalloc runs the same two kernels with the scratch in
// a fixed array compiled into this library instead.
//
// The array holds FL_ADJOINT_NOALLOC_MAX_RAYS floats (8 MiB) per GPU, until the
// process exits. With CUDA's default lazy module loading it is placed on a GPU
// when the first call on that GPU looks up its address: that first call takes
// the 8 MiB, so it belongs before the caller's pool allocator takes the GPU's
// memory and before any stream capture. Later calls allocate nothing. All
// calls share the array, so calls whose work can overlap on the GPU
// (different streams, or different host threads) race on it and must be
// serialised by the caller. Nothing in it has to start at zero: the weighting
// kernel writes every element the gather reads, and each call overwrites what
// the previous call left there. The stream must belong to the current device
// (the array's address is the current device's); a stream of another device
// is refused.
#include <mutex>

#include "fl_trace.h"
#include "fl_common.cuh"
#include "fl_plan.h"

static __device__ __align__(256) float g_adjoint_scratch[FL_ADJOINT_NOALLOC_MAX_RAYS];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
float* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_adjoint_scratch on the current device. In host code the
// symbol itself is only a host-side stand-in, never a device address; the
// address is looked up once per device, with that device current.
int scratch_for_current_device(float** out)
{
    int dev = 0;
    FL_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fl_set_error(FL_ERR_UNSUPPORTED, "fl_adjoint_noalloc: device %d", dev);
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        FL_CUDA(cudaGetSymbolAddress(&p, g_adjoint_scratch));
        g_scratch_ptr[dev] = static_cast<float*>(p);
    }
    *out = g_scratch_ptr[dev];
    return FL_OK;
}
}  // namespace

extern "C" int fl_adjoint_noalloc(fl_plan* p, const void* y, int yt, void* x, int xt,
                                  void* stream)
{
    FL_RANGE("fl_adjoint_noalloc");
    if (!p || !x || !y) return fl_set_error(FL_ERR_INVALID, "fl_adjoint_noalloc: null argument");
    if ((xt != FL_F32 && xt != FL_F16 && xt != FL_BF16) ||
        (yt != FL_F32 && yt != FL_F16 && yt != FL_BF16))
        return fl_set_error(FL_ERR_INVALID, "fl_adjoint_noalloc: unknown dtype");
    if (p->n_rays > (int64_t)FL_ADJOINT_NOALLOC_MAX_RAYS)
        return fl_set_error(FL_ERR_INVALID,
                            "fl_adjoint_noalloc: %lld rays exceed the fixed scratch of %d rays; "
                            "use fl_adjoint for this plan",
                            (long long)p->n_rays, FL_ADJOINT_NOALLOC_MAX_RAYS);
    int st = fl_matched_ready(p);
    if (st) return st;
    if (p->det_kind < 0 || (p->det_kind == 1 && p->s.ndim == 3))
        return fl_set_error(FL_ERR_UNSUPPORTED,
                            "matched adjoint needs a uniform flat or (fan) equiangular detector");
    cudaStream_t s = (cudaStream_t)stream;
    if (s) {
        int dev = 0, sdev = 0;
        FL_CUDA(cudaGetDevice(&dev));
        FL_CUDA(cudaStreamGetDevice(s, &sdev));
        if (sdev != dev)
            return fl_set_error(FL_ERR_INVALID,
                                "fl_adjoint_noalloc: the stream belongs to device %d, the "
                                "current device is %d", sdev, dev);
    }
    float* w = nullptr;
    if ((st = scratch_for_current_device(&w))) return st;
    if ((st = fl_matched_weight(p, y, yt, w, s))) return st;
    if ((st = fl_matched_adjoint_w(p, w, x, xt, nullptr, 0, s))) return st;
    return fl_set_error(FL_OK, "");
}
