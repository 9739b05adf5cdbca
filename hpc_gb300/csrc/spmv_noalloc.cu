// spmv_noalloc.cu -- y = A x and x.y without any device allocation.
//
// Who this is for: code that may not allocate device memory at the point of
// the call. Examples are a framework whose caching allocator owns all of the
// device memory, a caller that must not synchronise the device (cudaMalloc and
// cudaFree can), and a host thread that only owns buffers handed to it. Such a
// caller cannot create an xJPCG handle, because a handle allocates its
// buffers. This entry point needs no handle. The caller passes the CSR matrix
// and the vectors in device memory it already owns. The only other memory the
// kernel uses (the per-CTA partial sums of x.y and the ticket counter of the
// last-CTA reduction) lives in one file-scope __device__ array.
//
// The kernel is the library's fused SpMV + dot step (the kCgDot mode of
// spmv_kernels.cu: y = A x and a deterministic x.y, reduced per CTA and then
// summed in CTA order by the last CTA to finish). It reads the caller's arrays
// with plain loads and never reads past rowPtr[n] or nnz, because the caller's
// arrays carry none of the padding the handle's copies have.
//
// Limits and contract (also stated in include/xjpcg_gb300.h):
//   - one CTA per tile of kRows rows, one partial per CTA: n <= kMaxRows
//     (kMaxTiles * kRows = 524288 rows).  Larger n is rejected with
//     XJPCG_STATUS_INVALID_VALUE before anything is launched.
//   - the scratch array (kScratchBytes = 131328 bytes: a 256-byte header with
//     the ticket counter, then 16384 doubles of partial sums) is a __device__ global
//     of this library, so every GPU that loads the library holds it until
//     the process exits.
//   - every call shares the array; calls whose kernels overlap on the GPU
//     (different streams, no ordering) race on it.  Calls on one stream are
//     ordered and safe.
//   - the first call in a CUDA context (normally: the first call on a device,
//     in its primary context) looks the array's device address up with
//     cudaGetSymbolAddress, with that context current, and caches it for that
//     context; make that first call before any stream capture.  A context
//     created later (cudaDeviceReset, cuCtxCreate) gets its own lookup.  No
//     call allocates, frees or calls an allocating library routine.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/xjpcg_gb300.h"
#include "xjpcg_device.cuh"

namespace xjpcg {
namespace {

constexpr int kThreads = 256;
constexpr int kLanes = 8;                      // lanes per row
constexpr int kRows = kThreads / kLanes;       // rows per CTA
constexpr int kMaxTiles = 16384;               // partial sums the scratch holds
constexpr uint32_t kMaxRows = (uint32_t)kMaxTiles * kRows;

struct alignas(256) NoAllocScratch {
    uint32_t ticket;          // last-CTA counter; cleared before every launch
    uint32_t pad[63];
    double partials[kMaxTiles];
};
constexpr size_t kScratchBytes = sizeof(NoAllocScratch);
static_assert(kScratchBytes == 131328, "scratch size is part of the documented contract");

static __device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

__global__ void __launch_bounds__(kThreads) spmv_dot_noalloc_kernel(uint32_t n, const int* __restrict__ rowptr,
                                                                    const int* __restrict__ col,
                                                                    const double* __restrict__ val,
                                                                    const double* __restrict__ x,
                                                                    double* __restrict__ y, NoAllocScratch* scr,
                                                                    double* __restrict__ dot) {
    const int lane = threadIdx.x % kLanes;
    const uint32_t row = blockIdx.x * kRows + threadIdx.x / kLanes;
    const bool live = row < n;
    double acc = 0.0;
    if (live) {
        const int s = rowptr[row], e = rowptr[row + 1];
        for (int k = s + lane; k < e; k += kLanes) acc = fma(val[k], __ldg(&x[col[k]]), acc);
    }
#pragma unroll
    for (int o = kLanes / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    double d = 0.0;
    if (live && lane == 0) {
        y[row] = acc;
        d = x[row] * acc;
    }
    double v[1] = {d};
    block_sum<kThreads, 1, double>(v);
    double fin[1];
    if (grid_sum_last<kThreads, 1>(v, scr->partials, &scr->ticket, fin) && threadIdx.x == 0) *dot = fin[0];
}

// The array's device address depends on the CUDA context the library's
// module is loaded in: the device's primary context, a context the caller
// created with cuCtxCreate, or a primary context re-created after
// cudaDeviceReset.  The address is therefore cached per context, keyed by the
// driver's unique context id (cuCtxGetId), and looked up with
// cudaGetSymbolAddress once for each new context, with that context current.
// The driver functions are reached through cudaGetDriverEntryPointByVersion,
// so the library does not link libcuda itself.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

struct ScratchSlot {
    unsigned long long ctxId;
    NoAllocScratch* addr;
};
constexpr int kSlots = 64;

std::mutex g_setupMutex;
ScratchSlot g_slots[kSlots] = {};
int g_slotsUsed = 0, g_slotNext = 0;
CtxGetCurrentFn g_ctxGetCurrent = nullptr;
CtxGetIdFn g_ctxGetId = nullptr;

// Address of the scratch array in the current context (nullptr on failure).
// Called with g_setupMutex held.
NoAllocScratch* scratch_for_current_context() {
    if (g_ctxGetCurrent == nullptr || g_ctxGetId == nullptr) {
        void* f0 = nullptr;
        void* f1 = nullptr;
        cudaDriverEntryPointQueryResult q0, q1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || f0 == nullptr || f1 == nullptr)
            return nullptr;
        g_ctxGetCurrent = reinterpret_cast<CtxGetCurrentFn>(f0);
        g_ctxGetId = reinterpret_cast<CtxGetIdFn>(f1);
    }
    CUcontext ctx = nullptr;
    void* first = nullptr;
    if (g_ctxGetCurrent(&ctx) != CUDA_SUCCESS) return nullptr;
    if (ctx == nullptr) {
        // No context is current on this thread yet: the lookup itself makes
        // the current device's primary context current.
        if (cudaGetSymbolAddress(&first, g_noallocScratch) != cudaSuccess || first == nullptr) return nullptr;
        if (g_ctxGetCurrent(&ctx) != CUDA_SUCCESS || ctx == nullptr) return nullptr;
    }
    unsigned long long id = 0;
    if (g_ctxGetId(ctx, &id) != CUDA_SUCCESS) return nullptr;
    for (int i = 0; i < g_slotsUsed; ++i)
        if (g_slots[i].ctxId == id) return g_slots[i].addr;
    void* p = first;
    if (p == nullptr && (cudaGetSymbolAddress(&p, g_noallocScratch) != cudaSuccess || p == nullptr)) return nullptr;
    // A new context: take a free slot, else replace the oldest entry.
    const int slot = g_slotsUsed < kSlots ? g_slotsUsed++ : (g_slotNext++ % kSlots);
    g_slots[slot].ctxId = id;
    g_slots[slot].addr = static_cast<NoAllocScratch*>(p);
    return g_slots[slot].addr;
}

}  // namespace
}  // namespace xjpcg

extern "C" XJPCG_Status_t xJPCG_gbSpmvDotNoAlloc(uint32_t n, const int32_t* d_rowPtr, const int32_t* d_colIdx,
                                                 const double* d_values, const double* d_x, double* d_y,
                                                 double* d_dot, void* stream) {
    using namespace xjpcg;
    if (n == 0 || d_rowPtr == nullptr || d_colIdx == nullptr || d_values == nullptr || d_x == nullptr ||
        d_y == nullptr || d_dot == nullptr)
        return XJPCG_STATUS_INVALID_VALUE;
    if (n > kMaxRows) return XJPCG_STATUS_INVALID_VALUE;  // scratch holds kMaxTiles partial sums
    NoAllocScratch* scr = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setupMutex);
        scr = scratch_for_current_context();
    }
    if (scr == nullptr) {
        cudaGetLastError();
        return XJPCG_STATUS_INTERNAL_ERROR;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The kernel's last CTA leaves the ticket at 0, so after a completed call
    // it is already clear.  It is cleared here all the same: the array keeps
    // whatever the previous call left, and a previous call that raced with
    // another one (overlapping kernels on two streams, which the contract
    // rules out but cannot prevent) can leave the ticket off by some CTAs,
    // which would make this call's reduction finish early or never.  The
    // clear costs one 4-byte memset on the stream and allocates nothing.
    if (cudaMemsetAsync(&scr->ticket, 0, sizeof(uint32_t), st) != cudaSuccess) {
        cudaGetLastError();
        return XJPCG_STATUS_INTERNAL_ERROR;
    }
    const unsigned grid = (n + kRows - 1) / kRows;
    spmv_dot_noalloc_kernel<<<grid, kThreads, 0, st>>>(n, d_rowPtr, d_colIdx, d_values, d_x, d_y, scr, d_dot);
    if (cudaGetLastError() != cudaSuccess) return XJPCG_STATUS_INTERNAL_ERROR;
    return XJPCG_STATUS_SUCCESS;
}
