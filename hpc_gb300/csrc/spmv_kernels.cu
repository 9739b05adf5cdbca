// spmv_kernels.cu -- CSR SpMV for sm_103a.
//
// A persistent, warp-specialized kernel family, templated on the value type,
// the consumer threads per CTA (NC), the lanes per row (G), the nnz chunk size
// (C) and the pipeline depth (S).  Rows are cut into tiles of R = NC/G
// consecutive rows; CTA b walks tiles b, b+gridDim.x, ...  A tile's nnz range
// [rowptr[r0], rowptr[r0+R]) is streamed through shared memory in chunks of at
// most C entries ("jobs").
//
//   warp 0 (producer)   one lane reads the tile bounds from global memory and,
//                       per job, issues three cp.async.bulk copies (TMA bulk
//                       copies of 1-D ranges): the tile's row-pointer slice,
//                       the chunk's values and its column indices, completing
//                       on the stage's "full" mbarrier.  The matrix is read
//                       with an L2 evict-first policy so the gathered vector
//                       stays resident in L2.  Before reusing a stage the lane
//                       waits on its "empty" mbarrier.
//   warps 1.. (consumers)
//                       G lanes per row stride over the row's entries of the
//                       chunk (two independent FP64 accumulators per lane),
//                       gather x through the read-only path, and release the
//                       stage with one arrive per warp.  Partial sums stay in
//                       registers across the chunks of a tile, so rows of any
//                       length are handled; the G partials are combined with
//                       a fixed shuffle tree when the tile ends.
//
// Consumers read nothing from global memory but x (and p / b for the fused
// epilogues), so the only latency they see is the gather's.  Every wait is
// bounded in time; on a timeout the CTA records kStatusWaitTimeout, drains its
// copies in flight and leaves, and the solver loop stops.
//
// Modes (runtime, uniform across the grid):
//   kPlain     y = A x
//   kCgDot     y = A p, then p.y reduced over the grid; the last CTA writes
//              pAp and alpha = rz / pAp into the solver state.  This is the
//              reference's SpMV chain plus krnl_storeApk (pcg/hw/src/
//              krnl_storeApk.cpp:63-73) in one launch.
//   kResidual  y = b - A x and ||y||^2 reduced into state->rrTrue (true
//              residual of the mixed-precision refinement loop).
//   kCgPart    y = A p, and each CTA's partial p.y in partials[blockIdx.x]
//              (sliced kernel only): the fused vector kernel adds them.
#include <algorithm>
#include <cstdio>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

enum SpmvMode : int { kPlain = 0, kCgDot = 1, kResidual = 2, kCgPart = 3 };

template <typename VT>
struct AccOf {
    typedef double type;
};
template <>
struct AccOf<float> {
    typedef float type;
};

constexpr uint64_t kWaitBudgetNs = 2000000000ull;  // 2 s per wait, far above any chunk

template <typename VT, int NC, int G, int C, int S>
struct SpmvShape {
    static constexpr int NT = NC + 32;  // + producer warp
    static constexpr int R = NC / G;    // rows per tile
    static constexpr int RP = R + 4;    // row-pointer slice, padded to 16 bytes
    static constexpr int CP = C + 4;    // chunk capacity widened to 4-entry alignment
    static constexpr size_t kValOff = 0;
    static constexpr size_t kColOff = kValOff + sizeof(VT) * (size_t)S * CP;
    static constexpr size_t kRpOff = kColOff + sizeof(int) * (size_t)S * CP;
    static constexpr size_t kSmem = kRpOff + sizeof(int) * (size_t)S * RP;
    static_assert(NC % 32 == 0 && 32 % G == 0 && R % 4 == 0, "bad shape");
    static_assert((CP * sizeof(VT)) % 16 == 0 && (CP * 4) % 16 == 0 && (RP * 4) % 16 == 0, "stage alignment");
};

template <typename VT, int NC, int G, int C, int S>
__global__ void __launch_bounds__(NC + 32) spmv_ws_kernel(int n, int ntiles, const int* __restrict__ rowptr,
                                                          const int* __restrict__ col, const VT* __restrict__ val,
                                                          const VT* __restrict__ x, VT* __restrict__ y,
                                                          const VT* __restrict__ b, CgState* state,
                                                          double* partials, int mode, const uint32_t* doneFlag) {
    typedef SpmvShape<VT, NC, G, C, S> Sh;
    typedef typename AccOf<VT>::type AccT;
    constexpr int R = Sh::R;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    VT* sval = reinterpret_cast<VT*>(smem_raw + Sh::kValOff);
    int* scol = reinterpret_cast<int*>(smem_raw + Sh::kColOff);
    int* srp = reinterpret_cast<int*>(smem_raw + Sh::kRpOff);
    __shared__ __align__(8) uint64_t fullBar[S];
    __shared__ __align__(8) uint64_t emptyBar[S];
    __shared__ volatile int abortFlag;

    if (doneFlag && *(volatile const uint32_t*)doneFlag) return;

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        abortFlag = 0;
#pragma unroll
        for (int s = 0; s < S; ++s) {
            mbar_init(&fullBar[s], 1);
            mbar_init(&emptyBar[s], NC / 32);
        }
        mbar_fence_init();
    }
    __syncthreads();

    AccT dacc = AccT(0);
    int pjob = 0;  // jobs the producer issued
    if (warp == 0) {
        // ------------------------------ producer ------------------------------
        if (lane == 0) {
            const uint64_t pol = l2_policy_evict_first();
            int& job = pjob;
            for (int t = blockIdx.x; t < ntiles && !abortFlag; t += gridDim.x) {
                const int r0 = t * R, r1 = min(r0 + R, n);
                const int ts = __ldg(&rowptr[r0]), te = __ldg(&rowptr[r1]);
                const int nch = max(1, (te - ts + C - 1) / C);
                for (int c = 0; c < nch; ++c, ++job) {
                    const int st = job % S;
                    if (!mbar_wait_bounded(&emptyBar[st], ((uint32_t)(job / S) & 1u) ^ 1u, kWaitBudgetNs)) {
                        abortFlag = 1;
                        break;
                    }
                    const int cs = ts + c * C, ce = min(cs + C, te);
                    const int a0 = cs & ~3, a1 = (ce + 3) & ~3;
                    const uint32_t cnt = ce > cs ? (uint32_t)(a1 - a0) : 0u;
                    mbar_arrive_expect_tx(&fullBar[st], (uint32_t)Sh::RP * 4u + cnt * (uint32_t)(sizeof(VT) + 4));
                    bulk_g2s(srp + st * Sh::RP, rowptr + r0, (uint32_t)Sh::RP * 4u, &fullBar[st], pol);
                    if (cnt) {
                        bulk_g2s(sval + st * Sh::CP, val + a0, cnt * (uint32_t)sizeof(VT), &fullBar[st], pol);
                        bulk_g2s(scol + st * Sh::CP, col + a0, cnt * 4u, &fullBar[st], pol);
                    }
                }
            }
        }
        __syncwarp();
    } else {
        // ------------------------------ consumers -----------------------------
        const int ctid = tid - 32;
        const int lg = ctid % G;
        const int grp = ctid / G;
        int job = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            const int r0 = t * R, r1 = min(r0 + R, n);
            const int row = r0 + grp;
            const bool live = row < r1;
            AccT pRow = AccT(0);
            if (mode == kCgDot && lg == 0 && live) pRow = (AccT)__ldg(&x[row]);
            if (mode == kResidual && lg == 0 && live) pRow = (AccT)__ldg(&b[row]);
            AccT a0 = AccT(0), a1 = AccT(0);
            int nch = 1;
            for (int c = 0; c < nch; ++c, ++job) {
                const int st = job % S;
                if (!mbar_wait_bounded(&fullBar[st], (uint32_t)(job / S) & 1u, kWaitBudgetNs)) abortFlag = 1;
                if (abortFlag) break;
                const int* rp = srp + st * Sh::RP;
                const int ts = rp[0], te = rp[r1 - r0];
                nch = max(1, (te - ts + C - 1) / C);
                const int cs = ts + c * C, ce = min(cs + C, te);
                const int base = st * Sh::CP - (cs & ~3);
                int lo = cs, hi = cs;
                if (live) {
                    lo = max(rp[grp], cs);
                    hi = min(rp[grp + 1], ce);
                }
                int e = lo + lg;
#pragma unroll 2
                for (; e + G < hi; e += 2 * G) {
                    const VT v0 = sval[base + e], v1 = sval[base + e + G];
                    const int c0 = scol[base + e], c1 = scol[base + e + G];
                    a0 = fma((AccT)v0, (AccT)__ldg(&x[c0]), a0);
                    a1 = fma((AccT)v1, (AccT)__ldg(&x[c1]), a1);
                }
                if (e < hi) a0 = fma((AccT)sval[base + e], (AccT)__ldg(&x[scol[base + e]]), a0);
                __syncwarp();
                if (lane == 0) mbar_arrive(&emptyBar[st]);
            }
            if (abortFlag) break;
            AccT acc = a0 + a1;
            if (G > 1) {
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            }
            if (lg == 0 && live) {
                if (mode == kResidual) {
                    const AccT rv = pRow - acc;
                    y[row] = (VT)rv;
                    dacc = fma(rv, rv, dacc);
                } else {
                    y[row] = (VT)acc;
                    if (mode == kCgDot) dacc = fma(pRow, acc, dacc);
                }
            }
        }
    }
    __syncthreads();
    if (abortFlag) {
        if (tid == 0) {
            // Drain: whichever side gave up, the last S jobs may still be in
            // flight (each wait bounded; a completed one returns at once).
            for (int j = max(0, pjob - S); j < pjob; ++j)
                mbar_wait_bounded(&fullBar[j % S], (uint32_t)(j / S) & 1u, kWaitBudgetNs);
            atomicOr(&state->status, kStatusWaitTimeout);
            *(volatile uint32_t*)&state->done = 1u;  // later kernels of the loop stand down
        }
        return;
    }
    if (mode == kPlain) return;
    AccT v[1] = {dacc};
    block_sum<Sh::NT, 1, AccT>(v);
    double tot[1] = {(double)v[0]}, fin[1];
    if (grid_sum_last<Sh::NT, 1>(tot, partials, &state->counters[0], fin)) {
        if (threadIdx.x == 0) {
            if (mode == kCgDot) {
                state->pAp = fin[0];
                state->alpha = state->rz / fin[0];
            } else {
                state->rrTrue = fin[0];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host side: configuration table and launcher.
// ---------------------------------------------------------------------------
namespace {

template <typename VT, int NC, int G, int C, int S>
struct SpmvInst {
    typedef SpmvShape<VT, NC, G, C, S> Sh;
    static cudaError_t setup() {
        return cudaFuncSetAttribute(spmv_ws_kernel<VT, NC, G, C, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)Sh::kSmem);
    }
    static int blocksPerSm() {
        int nb = 0;
        if (setup() != cudaSuccess) return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_ws_kernel<VT, NC, G, C, S>, Sh::NT, Sh::kSmem) !=
            cudaSuccess)
            return 0;
        return nb;
    }
    static cudaError_t launch(int grid, cudaStream_t st, int n, const int* rp, const int* ci, const VT* v, const VT* x,
                              VT* y, const VT* b, CgState* state, double* partials, int mode,
                              const uint32_t* doneFlag) {
        const int ntiles = (n + Sh::R - 1) / Sh::R;
        spmv_ws_kernel<VT, NC, G, C, S>
            <<<grid, Sh::NT, Sh::kSmem, st>>>(n, ntiles, rp, ci, v, x, y, b, state, partials, mode, doneFlag);
        return cudaGetLastError();
    }
    static int tiles(int n) { return (n + Sh::R - 1) / Sh::R; }
};

template <typename VT>
struct Row {
    int lanes, consumers, chunk, stages;
    int (*blocksPerSm)();
    cudaError_t (*launch)(int, cudaStream_t, int, const int*, const int*, const VT*, const VT*, VT*, const VT*,
                          CgState*, double*, int, const uint32_t*);
    int (*tiles)(int);
};

#define XJ_ROW(VT, NC, G, C, S) \
    {G, NC, C, S, &SpmvInst<VT, NC, G, C, S>::blocksPerSm, &SpmvInst<VT, NC, G, C, S>::launch, \
     &SpmvInst<VT, NC, G, C, S>::tiles}
#define XJ_TABLE(VT)                                                                                     \
    XJ_ROW(VT, 128, 1, 4096, 2), XJ_ROW(VT, 128, 2, 2048, 3), XJ_ROW(VT, 256, 2, 4096, 2),             \
        XJ_ROW(VT, 256, 4, 2048, 4), XJ_ROW(VT, 128, 4, 1024, 4), XJ_ROW(VT, 256, 8, 2048, 4),          \
        XJ_ROW(VT, 256, 16, 2048, 4), XJ_ROW(VT, 256, 32, 2048, 4)

const Row<double> kRowsF64[] = {XJ_TABLE(double)};
const Row<float> kRowsF32[] = {XJ_TABLE(float)};
constexpr int kNumCfg = sizeof(kRowsF64) / sizeof(kRowsF64[0]);

template <typename VT>
const Row<VT>* rows();
template <>
const Row<double>* rows<double>() {
    return kRowsF64;
}
template <>
const Row<float>* rows<float>() {
    return kRowsF32;
}

}  // namespace

int spmv_num_configs() { return kNumCfg; }
int spmv_config_lanes(int cfg) { return kRowsF64[cfg].lanes; }
void spmv_config_shape(int cfg, int* lanes, int* consumers, int* chunk, int* stages) {
    *lanes = kRowsF64[cfg].lanes;
    *consumers = kRowsF64[cfg].consumers;
    *chunk = kRowsF64[cfg].chunk;
    *stages = kRowsF64[cfg].stages;
}

template <typename VT>
int spmv_grid(int cfg, int n, int numSms) {
    const Row<VT>& r = rows<VT>()[cfg];
    int bps = r.blocksPerSm();
    if (bps <= 0) return 0;
    int tiles = r.tiles(n);
    return std::max(1, std::min(tiles, bps * numSms));
}

template <typename VT>
cudaError_t spmv_launch(int cfg, int grid, cudaStream_t st, int n, const int* rp, const int* ci, const VT* v,
                        const VT* x, VT* y, const VT* b, CgState* state, double* partials, int mode,
                        const uint32_t* doneFlag) {
    if (n <= 0) return cudaSuccess;
    return rows<VT>()[cfg].launch(grid, st, n, rp, ci, v, x, y, b, state, partials, mode, doneFlag);
}

template int spmv_grid<double>(int, int, int);
template int spmv_grid<float>(int, int, int);
template cudaError_t spmv_launch<double>(int, int, cudaStream_t, int, const int*, const int*, const double*,
                                         const double*, double*, const double*, CgState*, double*, int,
                                         const uint32_t*);
template cudaError_t spmv_launch<float>(int, int, cudaStream_t, int, const int*, const int*, const float*,
                                        const float*, float*, const float*, CgState*, double*, int,
                                        const uint32_t*);

}  // namespace xjpcg

// ===========================================================================
// Sliced layout (SELL-32): rows in slices of 32, each slice padded to its
// longest row and stored column-major (entry j of the slice's 32 rows is
// contiguous).  One lane per row, no shared memory and no reduction: every
// warp-wide load of values or columns is one contiguous 256-byte (values) or
// 128-byte (columns) segment, occupancy is limited only by registers, and the
// FP64 pipe sees exactly one DFMA per stored entry.  On this part FP64 issue
// (about two DFMA per clock per SM) is as scarce as HBM bandwidth, so the
// autotuner picks this layout for matrices with near-uniform row lengths
// (stencils) and the staged CSR kernels above for irregular ones.  Padding
// entries hold value 0 and the row's own index as column.
//
// Narrow columns: when every stored column lies within 32767 of its row
// (banded matrices, e.g. any 27-point grid up to 180 x 180 planes), the
// column array is also kept as int16 offsets col - row, cutting the streamed
// bytes per entry from 12 to 10 (fp64) and from 8 to 6 (fp32).  Rows past n
// in the last slice read x[n - 1] with value 0.
// ===========================================================================
namespace xjpcg {

constexpr int kSellThreads = 256;

__global__ void sell_slice_len_kernel(int n, const int* __restrict__ rowptr, int* __restrict__ sliceLen) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    const int nslices = (n + 31) / 32;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warpsPerGrid) {
        const int row = s * 32 + lane;
        int len = row < n ? rowptr[row + 1] - rowptr[row] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) len = max(len, __shfl_xor_sync(0xffffffffu, len, o));
        if (lane == 0) sliceLen[s] = len * 32;
    }
}

// Sets *tooWide when some stored column lies more than 32767 below or 32767
// above its row, so the int16 offset copy cannot hold it.
__global__ void sell_width_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                  int* __restrict__ tooWide) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        const int rs = rowptr[row], re = rowptr[row + 1];
        bool wide = false;
        for (int j = rs; j < re; ++j) {
            const int d = col[j] - row;
            wide |= d > 32767 || d < -32767;
        }
        if (wide) atomicOr(tooWide, 1);
    }
}

__global__ void sell_fill_narrow_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                        const int* __restrict__ sliceOff, int16_t* __restrict__ scol16) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    const int nslices = (n + 31) / 32;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warpsPerGrid) {
        const int off = sliceOff[s];
        const int len = (sliceOff[s + 1] - off) / 32;
        const int row = s * 32 + lane;
        const int rs = row < n ? rowptr[row] : 0;
        const int rl = row < n ? rowptr[row + 1] - rs : 0;
        for (int j = 0; j < len; ++j) scol16[off + j * 32 + lane] = (int16_t)(j < rl ? col[rs + j] - row : 0);
    }
}

template <typename VT>
__global__ void sell_fill_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                 const double* __restrict__ val, const int* __restrict__ sliceOff,
                                 int* __restrict__ scol, VT* __restrict__ sval) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    const int nslices = (n + 31) / 32;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warpsPerGrid) {
        const int off = sliceOff[s];
        const int len = (sliceOff[s + 1] - off) / 32;
        const int row = s * 32 + lane;
        const int rs = row < n ? rowptr[row] : 0;
        const int rl = row < n ? rowptr[row + 1] - rs : 0;
        for (int j = 0; j < len; ++j) {
            const int dst = off + j * 32 + lane;
            if (j < rl) {
                if (scol) scol[dst] = col[rs + j];
                sval[dst] = (VT)val[rs + j];
            } else {
                if (scol) scol[dst] = row < n ? row : 0;
                sval[dst] = VT(0);
            }
        }
    }
}

// Streams one stored column (evict-first) and returns the absolute column.
template <typename CT>
__device__ __forceinline__ int sell_column(const CT* p, int base);
template <>
__device__ __forceinline__ int sell_column<int>(const int* p, int) {
    return __ldcs(p);
}
template <>
__device__ __forceinline__ int sell_column<int16_t>(const int16_t* p, int base) {
    return base + (int)__ldcs(reinterpret_cast<const short*>(p));
}

// Resident CTAs per SM the register budget is set for: 6 (40 registers).
// An FP32 build capped at 32 registers (8 CTAs) measured slower.
template <typename VT, int U>
struct SellMinBlocks {
    static constexpr int value = 6;
};

// CT = int: absolute columns; CT = int16_t: offsets from the row.
template <typename VT, int U, typename CT>
__global__ void __launch_bounds__(kSellThreads, SellMinBlocks<VT, U>::value) spmv_sell_kernel(int n, int nslices, const int* __restrict__ sliceOff,
                                                                 const CT* __restrict__ scol,
                                                                 const VT* __restrict__ sval, const VT* __restrict__ x,
                                                                 VT* __restrict__ y, const VT* __restrict__ b,
                                                                 CgState* state, double* partials, int mode,
                                                                 const uint32_t* doneFlag) {
    typedef typename AccOf<VT>::type AccT;
    if (doneFlag && *(volatile const uint32_t*)doneFlag) return;
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    AccT dacc = AccT(0);
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warpsPerGrid) {
        const int off = __ldg(&sliceOff[s]);
        const int len = (__ldg(&sliceOff[s + 1]) - off) >> 5;
        const int row = s * 32 + lane;
        const int base = min(row, n - 1);
        const VT* vp = sval + off + lane;
        const CT* cp = scol + off + lane;
        AccT acc = AccT(0);
        int j = 0;
        for (; j + U <= len; j += U) {
            VT v[U];
            int c[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                v[u] = __ldcs(vp + (j + u) * 32);
                c[u] = sell_column<CT>(cp + (j + u) * 32, base);
            }
            AccT xv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) xv[u] = (AccT)__ldg(&x[c[u]]);
#pragma unroll
            for (int u = 0; u < U; ++u) acc = fma((AccT)v[u], xv[u], acc);
        }
        for (; j < len; ++j)
            acc = fma((AccT)__ldcs(vp + j * 32), (AccT)__ldg(&x[sell_column<CT>(cp + j * 32, base)]), acc);
        if (row < n) {
            if (mode == kResidual) {
                const AccT rv = (AccT)b[row] - acc;
                y[row] = (VT)rv;
                dacc = fma(rv, rv, dacc);
            } else {
                y[row] = (VT)acc;
                if (mode == kCgDot || mode == kCgPart) dacc = fma((AccT)x[row], acc, dacc);
            }
        }
    }
    if (mode == kPlain) return;
    AccT v[1] = {dacc};
    block_sum<kSellThreads, 1, AccT>(v);
    double tot[1] = {(double)v[0]}, fin[1];
    if (mode == kCgPart) {
        if (threadIdx.x == 0) partials[blockIdx.x] = tot[0];
        return;
    }
    if (grid_sum_last<kSellThreads, 1>(tot, partials, &state->counters[0], fin)) {
        if (threadIdx.x == 0) {
            if (mode == kCgDot) {
                state->pAp = fin[0];
                state->alpha = state->rz / fin[0];
            } else {
                state->rrTrue = fin[0];
            }
        }
    }
}

namespace {
template <typename VT, int U, typename CT>
int sell_bps() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_sell_kernel<VT, U, CT>, kSellThreads, 0) !=
        cudaSuccess)
        return 0;
    return nb;
}

template <typename VT, typename CT>
void sell_kernel_launch(int u, int grid, cudaStream_t st, int n, int nslices, const int* sliceOff, const CT* scol,
                        const VT* sval, const VT* x, VT* y, const VT* b, CgState* state, double* partials, int mode,
                        const uint32_t* doneFlag) {
    if (u == 16)
        spmv_sell_kernel<VT, 16, CT><<<grid, kSellThreads, 0, st>>>(n, nslices, sliceOff, scol, sval, x, y, b, state,
                                                                   partials, mode, doneFlag);
    else if (u == 4)
        spmv_sell_kernel<VT, 4, CT><<<grid, kSellThreads, 0, st>>>(n, nslices, sliceOff, scol, sval, x, y, b, state,
                                                                  partials, mode, doneFlag);
    else if (u == 8)
        spmv_sell_kernel<VT, 8, CT><<<grid, kSellThreads, 0, st>>>(n, nslices, sliceOff, scol, sval, x, y, b, state,
                                                                  partials, mode, doneFlag);
    else
        spmv_sell_kernel<VT, 2, CT><<<grid, kSellThreads, 0, st>>>(n, nslices, sliceOff, scol, sval, x, y, b, state,
                                                                  partials, mode, doneFlag);
}
}  // namespace

// Sliced configurations: 0-2 absolute int32 columns with unroll 4, 8, 2;
// 3-5 int16 column offsets with unroll 4, 8, 16.
int sell_num_configs() { return 6; }
int sell_config_unroll(int cfg) {
    static const int u[6] = {4, 8, 2, 4, 8, 16};
    return u[cfg];
}
bool sell_config_narrow(int cfg) { return cfg >= 3; }

cudaError_t sell_build(cudaStream_t st, int n, const int* rowptr, const int* col, const double* val, int* sliceOff,
                       int* blockSums, int64_t* total) {
    const int nslices = (n + 31) / 32;
    int grid = (int)std::min<int64_t>(((int64_t)nslices * 32 + 255) / 256, device_sm_count() * 64);
    sell_slice_len_kernel<<<grid, 256, 0, st>>>(n, rowptr, sliceOff);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(sliceOff + nslices, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    e = scan_exclusive(st, sliceOff, sliceOff, nslices + 1, blockSums);
    if (e != cudaSuccess) return e;
    int t = 0;
    e = cudaMemcpyAsync(&t, sliceOff + nslices, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    *total = t;
    return e;
}

cudaError_t sell_narrow_fits(cudaStream_t st, int n, const int* rowptr, const int* col, int* flag, bool* fits) {
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)n + 255) / 256, device_sm_count() * 16));
    sell_width_kernel<<<grid, 256, 0, st>>>(n, rowptr, col, flag);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int h = 1;
    e = cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    *fits = h == 0;
    return e;
}

cudaError_t sell_fill_narrow(cudaStream_t st, int n, const int* rowptr, const int* col, const int* sliceOff,
                             int16_t* scol16) {
    const int nslices = (n + 31) / 32;
    int grid = (int)std::min<int64_t>(((int64_t)nslices * 32 + 255) / 256, device_sm_count() * 64);
    sell_fill_narrow_kernel<<<grid, 256, 0, st>>>(n, rowptr, col, sliceOff, scol16);
    return cudaGetLastError();
}

template <typename VT>
cudaError_t sell_fill(cudaStream_t st, int n, const int* rowptr, const int* col, const double* val,
                      const int* sliceOff, int* scol, VT* sval) {
    const int nslices = (n + 31) / 32;
    int grid = (int)std::min<int64_t>(((int64_t)nslices * 32 + 255) / 256, device_sm_count() * 64);
    sell_fill_kernel<VT><<<grid, 256, 0, st>>>(n, rowptr, col, val, sliceOff, scol, sval);
    return cudaGetLastError();
}

template <typename VT>
int sell_grid(int cfg, int n, int numSms) {
    const int u = sell_config_unroll(cfg);
    int bps;
    if (sell_config_narrow(cfg))
        bps = u == 4 ? sell_bps<VT, 4, int16_t>() : (u == 8 ? sell_bps<VT, 8, int16_t>() : sell_bps<VT, 16, int16_t>());
    else
        bps = u == 4 ? sell_bps<VT, 4, int>() : (u == 8 ? sell_bps<VT, 8, int>() : sell_bps<VT, 2, int>());
    if (bps <= 0) return 0;
    const int nslices = (n + 31) / 32;
    const int need = (nslices + kSellThreads / 32 - 1) / (kSellThreads / 32);
    return std::max(1, std::min(need, bps * numSms));
}

template <typename VT>
cudaError_t spmv_sell_launch(int cfg, int grid, cudaStream_t st, int n, const int* sliceOff, const int* scol,
                             const int16_t* scol16, const VT* sval, const VT* x, VT* y, const VT* b, CgState* state,
                             double* partials, int mode, const uint32_t* doneFlag) {
    if (n <= 0) return cudaSuccess;
    const int nslices = (n + 31) / 32;
    const int u = sell_config_unroll(cfg);
    if (sell_config_narrow(cfg)) {
        if (scol16 == nullptr) return cudaErrorInvalidValue;
        sell_kernel_launch<VT, int16_t>(u, grid, st, n, nslices, sliceOff, scol16, sval, x, y, b, state, partials,
                                        mode, doneFlag);
    } else {
        if (u == 16) return cudaErrorInvalidValue;  // no int32-column unroll-16 configuration
        sell_kernel_launch<VT, int>(u, grid, st, n, nslices, sliceOff, scol, sval, x, y, b, state, partials, mode,
                                    doneFlag);
    }
    return cudaGetLastError();
}

template cudaError_t sell_fill<double>(cudaStream_t, int, const int*, const int*, const double*, const int*, int*,
                                       double*);
template cudaError_t sell_fill<float>(cudaStream_t, int, const int*, const int*, const double*, const int*, int*,
                                      float*);
template int sell_grid<double>(int, int, int);
template int sell_grid<float>(int, int, int);
template cudaError_t spmv_sell_launch<double>(int, int, cudaStream_t, int, const int*, const int*,
                                              const int16_t*, const double*, const double*, double*, const double*,
                                              CgState*, double*, int, const uint32_t*);
template cudaError_t spmv_sell_launch<float>(int, int, cudaStream_t, int, const int*, const int*, const int16_t*,
                                             const float*, const float*, float*, const float*, CgState*, double*,
                                             int, const uint32_t*);

}  // namespace xjpcg
