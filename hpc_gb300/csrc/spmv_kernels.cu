// spmv_kernels.cu -- CSR SpMV for sm_103a.
//
// One persistent kernel family, templated on the value type, the threads per
// CTA (NT), the lanes per row (G), the nnz chunk size (C) and the pipeline
// depth (S).  Rows are cut into tiles of R = NT/G consecutive rows; a CTA walks
// its tiles (blockIdx.x, +gridDim.x, ...) and streams each tile's nnz range
// [rowptr[r0], rowptr[r0+R]) through shared memory in chunks of C values and C
// column indices.  Chunks are moved by cp.async.bulk (TMA bulk copies, no
// tensor map needed for 1-D ranges) that complete on per-stage mbarriers, with
// an L2 evict-first policy so the streamed matrix does not push the gathered
// vector out of L2.  Thread 0 keeps S chunks in flight ahead of the consumers.
// A row's G lanes stride over its entries in each chunk and keep their partial
// sum in registers across chunks, so rows of any length are handled; the G
// partials are combined with a fixed shuffle tree at the end of the tile.
//
// Modes (runtime, uniform across the grid):
//   kPlain     y = A x
//   kCgDot     y = A p, then p.y reduced over the grid; the last CTA writes
//              pAp and alpha = rz / pAp into the solver state.  This is the
//              reference's SpMV chain plus krnl_storeApk (pcg/hw/src/
//              krnl_storeApk.cpp:63-73) fused into one launch.
//   kResidual  y = b - A x and ||y||^2 reduced into state->rrTrue (true
//              residual of the mixed-precision refinement loop).
#include <algorithm>
#include <cstdio>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

enum SpmvMode : int { kPlain = 0, kCgDot = 1, kResidual = 2 };

template <typename VT>
struct AccOf {
    typedef double type;
};
template <>
struct AccOf<float> {
    typedef float type;
};

constexpr uint64_t kWaitBudgetNs = 2000000000ull;  // 2 s per wait, far above any chunk

template <typename VT, int NT, int G, int C, int S>
__global__ void __launch_bounds__(NT) spmv_staged_kernel(int n, int ntiles, const int* __restrict__ rowptr,
                                                         const int* __restrict__ col, const VT* __restrict__ val,
                                                         const VT* __restrict__ x, VT* __restrict__ y,
                                                         const VT* __restrict__ b, CgState* state,
                                                         double* partials, int mode, const uint32_t* doneFlag) {
    typedef typename AccOf<VT>::type AccT;
    constexpr int R = NT / G;
    constexpr int CP = C + 4;  // stage capacity: a chunk widened to 4-element alignment
    static_assert(NT % 32 == 0 && 32 % G == 0, "bad shape");
    static_assert((CP * sizeof(VT)) % 16 == 0 && (CP * 4) % 16 == 0, "stage alignment");

    extern __shared__ __align__(128) unsigned char smem_raw[];
    VT* sval = reinterpret_cast<VT*>(smem_raw);
    int* scol = reinterpret_cast<int*>(smem_raw + sizeof(VT) * S * CP);
    __shared__ __align__(8) uint64_t fullBar[S];
    __shared__ int abortFlag;

    if (doneFlag && *(volatile const uint32_t*)doneFlag) return;

    const int tid = threadIdx.x;
    const int lane = tid % G;
    const int grp = tid / G;

    // ---- producer state (thread 0 only) ----
    int pTile = (int)blockIdx.x - (int)gridDim.x, pChunk = 0, pNch = 0, pTs = 0, pTe = 0;
    bool pHas = true;
    uint64_t pol = 0;
    auto pAdvance = [&]() -> bool {
        ++pChunk;
        while (pChunk >= pNch) {
            pTile += gridDim.x;
            if (pTile >= ntiles) return false;
            const int r0 = pTile * R, r1 = min(r0 + R, n);
            pTs = rowptr[r0];
            pTe = rowptr[r1];
            pNch = (pTe - pTs + C - 1) / C;
            pChunk = 0;
        }
        return true;
    };
    auto pIssue = [&](int job) {
        const int cs = pTs + pChunk * C;
        const int ce = min(cs + C, pTe);
        const int a0 = cs & ~3, a1 = (ce + 3) & ~3;
        const uint32_t cnt = (uint32_t)(a1 - a0);
        const int st = job % S;
        mbar_arrive_expect_tx(&fullBar[st], cnt * (uint32_t)(sizeof(VT) + 4));
        bulk_g2s(sval + st * CP, val + a0, cnt * (uint32_t)sizeof(VT), &fullBar[st], pol);
        bulk_g2s(scol + st * CP, col + a0, cnt * 4u, &fullBar[st], pol);
    };

    if (tid == 0) {
        abortFlag = 0;
#pragma unroll
        for (int s = 0; s < S; ++s) mbar_init(&fullBar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    int issued = 0;
    if (tid == 0) {
        pol = l2_policy_evict_first();
        for (int s = 0; s < S; ++s) {
            pHas = pAdvance();
            if (!pHas) break;
            pIssue(s);
            ++issued;
        }
    }

    AccT dacc = AccT(0);
    int job = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int r0 = t * R, r1 = min(r0 + R, n);
        const int ts = rowptr[r0], te = rowptr[r1];
        const int row = r0 + grp;
        int rs = 0, re = 0;
        if (row < r1) {
            rs = rowptr[row];
            re = rowptr[row + 1];
        }
        AccT acc = AccT(0);
        const int nch = (te - ts + C - 1) / C;
        for (int c = 0; c < nch; ++c, ++job) {
            const int st = job % S;
            const uint32_t parity = (uint32_t)(job / S) & 1u;
            if (!mbar_wait_bounded(&fullBar[st], parity, kWaitBudgetNs)) abortFlag = 1;
            const int cs = ts + c * C;
            const int ce = min(cs + C, te);
            const int base = st * CP - (cs & ~3);
            const int lo = max(rs, cs), hi = min(re, ce);
#pragma unroll 4
            for (int e = lo + lane; e < hi; e += G) {
                const VT v = sval[base + e];
                const int cidx = scol[base + e];
                acc = fma((AccT)v, (AccT)__ldg(&x[cidx]), acc);
            }
            __syncthreads();
            if (abortFlag) break;
            if (tid == 0 && pHas) {
                pHas = pAdvance();
                if (pHas) {
                    pIssue(job + S);
                    ++issued;
                }
            }
        }
        if (abortFlag) break;
        if (G > 1) {
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        }
        if (lane == 0 && row < r1) {
            if (mode == kResidual) {
                const AccT rv = (AccT)b[row] - acc;
                y[row] = (VT)rv;
                dacc = fma(rv, rv, dacc);
            } else {
                y[row] = (VT)acc;
                if (mode == kCgDot) dacc = fma((AccT)x[row], acc, dacc);
            }
        }
    }

    if (abortFlag) {
        // Drain copies still in flight so no bulk write lands after exit.
        if (tid == 0) {
            for (int j = job; j < issued; ++j) mbar_wait_bounded(&fullBar[j % S], (uint32_t)(j / S) & 1u, kWaitBudgetNs);
            atomicOr(&state->status, kStatusWaitTimeout);
            *(volatile uint32_t*)&state->done = 1u;  // later kernels of the loop stand down
        }
        return;
    }

    if (mode == kPlain) return;
    AccT v[1] = {dacc};
    block_sum<NT, 1, AccT>(v);
    double tot[1] = {(double)v[0]}, fin[1];
    if (grid_sum_last<1>(tot, partials, &state->counters[0], fin)) {
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

template <typename VT, int NT, int G, int C, int S>
struct SpmvInst {
    static constexpr size_t smem() { return (size_t)S * (C + 4) * (sizeof(VT) + 4); }
    static cudaError_t setup() {
        return cudaFuncSetAttribute(spmv_staged_kernel<VT, NT, G, C, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem());
    }
    static int blocksPerSm() {
        int nb = 0;
        if (setup() != cudaSuccess) return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_staged_kernel<VT, NT, G, C, S>, NT, smem()) !=
            cudaSuccess)
            return 0;
        return nb;
    }
    static cudaError_t launch(int grid, cudaStream_t st, int n, const int* rp, const int* ci, const VT* v, const VT* x,
                              VT* y, const VT* b, CgState* state, double* partials, int mode, const uint32_t* doneFlag) {
        const int ntiles = (n + NT / G - 1) / (NT / G);
        spmv_staged_kernel<VT, NT, G, C, S>
            <<<grid, NT, smem(), st>>>(n, ntiles, rp, ci, v, x, y, b, state, partials, mode, doneFlag);
        return cudaGetLastError();
    }
    static int tiles(int n) { return (n + NT / G - 1) / (NT / G); }
};

template <typename VT>
struct Table;

#define XJPCG_SPMV_ROWS(VT)                                                                              \
    {1, &SpmvInst<VT, 256, 1, 2048, 4>::blocksPerSm, &SpmvInst<VT, 256, 1, 2048, 4>::launch,          \
     &SpmvInst<VT, 256, 1, 2048, 4>::tiles},                                                             \
        {2, &SpmvInst<VT, 256, 2, 2048, 4>::blocksPerSm, &SpmvInst<VT, 256, 2, 2048, 4>::launch,      \
         &SpmvInst<VT, 256, 2, 2048, 4>::tiles},                                                         \
        {4, &SpmvInst<VT, 256, 4, 2048, 4>::blocksPerSm, &SpmvInst<VT, 256, 4, 2048, 4>::launch,      \
         &SpmvInst<VT, 256, 4, 2048, 4>::tiles},                                                         \
        {8, &SpmvInst<VT, 256, 8, 2048, 4>::blocksPerSm, &SpmvInst<VT, 256, 8, 2048, 4>::launch,      \
         &SpmvInst<VT, 256, 8, 2048, 4>::tiles},                                                         \
        {16, &SpmvInst<VT, 256, 16, 2048, 4>::blocksPerSm, &SpmvInst<VT, 256, 16, 2048, 4>::launch,   \
         &SpmvInst<VT, 256, 16, 2048, 4>::tiles},                                                        \
    {                                                                                                    \
        32, &SpmvInst<VT, 256, 32, 2048, 4>::blocksPerSm, &SpmvInst<VT, 256, 32, 2048, 4>::launch,     \
            &SpmvInst<VT, 256, 32, 2048, 4>::tiles                                                       \
    }

template <typename VT>
struct Row {
    int lanes;
    int (*blocksPerSm)();
    cudaError_t (*launch)(int, cudaStream_t, int, const int*, const int*, const VT*, const VT*, VT*, const VT*,
                          CgState*, double*, int, const uint32_t*);
    int (*tiles)(int);
};

const Row<double> kRowsF64[] = {XJPCG_SPMV_ROWS(double)};
const Row<float> kRowsF32[] = {XJPCG_SPMV_ROWS(float)};

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

int spmv_num_configs() { return 6; }
int spmv_config_lanes(int cfg) { return kRowsF64[cfg].lanes; }

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
                        const VT* x, VT* y, const VT* b, CgState* state, double* partials, int mode, const uint32_t* doneFlag) {
    if (n <= 0) return cudaSuccess;
    return rows<VT>()[cfg].launch(grid, st, n, rp, ci, v, x, y, b, state, partials, mode, doneFlag);
}

template int spmv_grid<double>(int, int, int);
template int spmv_grid<float>(int, int, int);
template cudaError_t spmv_launch<double>(int, int, cudaStream_t, int, const int*, const int*, const double*,
                                         const double*, double*, const double*, CgState*, double*, int, const uint32_t*);
template cudaError_t spmv_launch<float>(int, int, cudaStream_t, int, const int*, const int*, const float*,
                                        const float*, float*, const float*, CgState*, double*, int, const uint32_t*);

}  // namespace xjpcg
