// fan_tma.cu -- the fan forward's transposed copy of its input (walk_fan in
// matched_dev.cuh reads each image from the array whose fast axis runs along
// that image's detector) moved by the tensor memory accelerator.
//
// A block owns one 32 x 32 tile of one frame: one thread issues a tiled TMA
// load of the tile (cp.async.bulk.tensor, completion counted on an mbarrier),
// the block transposes it in shared memory, and one thread issues the tiled
// TMA store of the transposed tile into the plan's buffer. Edge tiles are
// clipped by the tensor unit (loads fill zeros out of range, stores write the
// part in range). Both tensor maps are encoded per call on the host, so they
// carry the caller's input address (a CUDA graph captures them by value).
// Conditions (else the SIMT transpose of matched.cu runs): the driver's
// tensor-map encoder is available, the input starts on a 16-byte boundary,
// and the rows of both arrays are multiples of 16 bytes (nx and ny multiples
// of 4 in FP32, of 8 in FP16 / BF16). Tile origins are multiples of 32
// elements, so every innermost coordinate is 16-byte aligned.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "fl_common.cuh"
#include "fl_plan.h"

namespace {

constexpr int kTile = 32;
// rows of threads per block: 4 (128 threads, 8 KB of tiles) lets 16 blocks,
// so 16 tile loads of 4 KB (FP32), be in flight per SM
constexpr int kRows = 4;
// mbarrier polls before a block gives up on its tile (a 4 KB load takes
// microseconds; this is seconds): it then records the timeout and returns
constexpr int kTmaPolls = 1 << 24;
// stall > 0 (FL_DEBUG_TMA_STALL, tests only): no load is issued and the block
// waits, for stall polls, on a phase that nothing completes, so the timeout
// path runs with no copy in flight.

template <typename T>
__global__ void __launch_bounds__(kTile * kRows)
k_transpose_tma(const __grid_constant__ CUtensorMap src, const __grid_constant__ CUtensorMap dst,
                int* __restrict__ err, int stall)
{
    __shared__ alignas(128) T tin[kTile * kTile];
    __shared__ alignas(128) T tout[kTile * kTile];
    __shared__ alignas(8) unsigned long long bar;
    const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile, f = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTile + tx;
    const unsigned sbar = (unsigned)__cvta_generic_to_shared(&bar);
    const unsigned sin = (unsigned)__cvta_generic_to_shared(tin);
    const unsigned sout = (unsigned)__cvta_generic_to_shared(tout);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (!stall) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                         ::"r"(sbar), "r"((unsigned)(kTile * kTile * sizeof(T)))
                         : "memory");
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
                " [%0], [%1, {%2, %3, %4}], [%5];"
                ::"r"(sin), "l"(&src), "r"(x0), "r"(y0), "r"(f), "r"(sbar)
                : "memory");
        }
    }
    __syncthreads();                       // the barrier is set up before anyone waits
    unsigned done = 0;
    const int polls = stall ? stall : kTmaPolls;
    for (int i = 0; i < polls && !done; i++)
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;"
            " selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(sbar)
            : "memory");
    if (!__syncthreads_and(done)) {        // a block-wide vote: the tile never arrived
        if (tid == 0 && err) atomicExch(err, 1);
        return;
    }
    // tin[y][x] (x fastest) -> tout[x][y] (y fastest). Both tiles stay dense
    // (the TMA boxes), so the order is skewed instead of padded: at step k,
    // thread tx moves element (y = (k + tx) mod 32, x = tx), and the 32 lanes
    // of a warp address 32 different banks on both sides (FP32).
#pragma unroll
    for (int k = ty; k < kTile; k += kRows) {
        const int c = (k + tx) & (kTile - 1);
        tout[tx * kTile + c] = tin[c * kTile + tx];
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // visible to the TMA unit
    __syncthreads();
    if (tid == 0) {
        asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group"
                     " [%0, {%1, %2, %3}], [%4];"
                     ::"l"(&dst), "r"(y0), "r"(x0), "r"(f), "r"(sout)
                     : "memory");
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");   // tout read out
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

// 3-D map of rows of n0 elements, n1 rows per frame, n2 frames; 32 x 32 boxes
bool encode(CUtensorMap* m, CUtensorMapDataType t, int es, void* base, int n0, int n1, int n2)
{
    const cuuint64_t dims[3] = {(cuuint64_t)n0, (cuuint64_t)n1, (cuuint64_t)n2};
    const cuuint64_t strides[2] = {(cuuint64_t)n0 * es, (cuuint64_t)n0 * n1 * es};
    const cuuint32_t box[3] = {kTile, kTile, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return encoder()(m, t, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// Whether the driver's tensor-map encoder is available; fan plans ask at
// creation, so the first forward (possibly under stream capture) makes no
// driver entry-point query.
bool fl_tma_available() { return encoder() != nullptr; }

// The transposed copy of a fan forward's input x (all frames) into p->d_xt by
// TMA. Returns false, having launched nothing, where the conditions above do
// not hold; the caller then runs the SIMT transpose.
bool fl_fan_transpose_tma(fl_plan* p, const void* x, int dtype, cudaStream_t st)
{
    const fl_scan& s = p->s;
    const int es = dtype == FL_F32 ? 4 : 2;
    if (!p->fan_tma_ok || !p->d_xt || !encoder()) return false;
    if ((reinterpret_cast<uintptr_t>(x) & 15) || (s.nx * es) % 16 || (s.ny * es) % 16)
        return false;
    const CUtensorMapDataType t = dtype == FL_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                  : dtype == FL_F16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                    : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    alignas(64) CUtensorMap src, dst;
    if (!encode(&src, t, es, const_cast<void*>(x), s.nx, s.ny, s.nt) ||
        !encode(&dst, t, es, p->d_xt, s.ny, s.nx, s.nt))
        return false;
    const dim3 grid(fl_div_up(s.nx, kTile), fl_div_up(s.ny, kTile), s.nt), blk(kTile, kRows);
    int* e = p->d_tma_err;
    const int z = p->tma_stall;
    if (dtype == FL_F32) k_transpose_tma<float><<<grid, blk, 0, st>>>(src, dst, e, z);
    else if (dtype == FL_F16) k_transpose_tma<__half><<<grid, blk, 0, st>>>(src, dst, e, z);
    else k_transpose_tma<__nv_bfloat16><<<grid, blk, 0, st>>>(src, dst, e, z);
    return true;
}
