// spmv_sellsort.cu -- sliced SpMV with rows sorted by length, for irregular
// (power-law) matrices.
//
// The plain sliced layout pads every 32-row slice to its longest row, which
// for rows of very different lengths (lengths 4 .. 4000 in one slice) wastes
// most of the bandwidth; the tuner then rejects it.  Here the rows are first
// reordered by length, longest first (SELL-C-sigma with sigma = n, C = 32), so
// the 32 rows of a slice have nearly the same length and padding vanishes.
// Rows longer than kLongRow are taken out and handled by a whole warp each
// (lanes stride along the row, then a fixed shuffle tree), so a 4000-entry
// row costs one warp 4000/32 steps instead of one lane 4000 steps.
//
// The reorder is a stable counting sort by length (ties by row index): one
// warp per 1024-row tile builds per-tile histograms, a scan gives every
// (length, tile) its start, and the warp scatters its rows in row order
// with __match_any_sync ranks.  The layout is therefore deterministic, and so
// is every sum: each row is summed over its own entries in CSR order.  The
// permutation only decides which lane computes which row; y is written back
// at the original row index.
//
// Work items, in warp-stride order: the long rows (one warp each), then the
// slices (one lane per row).  kCgDot / kResidual reduce through the same
// last-block-done grid sum as the other SpMV kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

namespace {
constexpr int kLongRow = 256;              // rows longer than this get a warp
constexpr int kBins = kLongRow + 2;        // 0 = long rows, 1 + (kLongRow - len) for the rest
constexpr int kTileRows = 1024;            // rows per histogram tile
constexpr int kSortThreads = 256;          // SpMV CTA size

template <typename VT>
struct SortAcc {
    typedef double type;
};
template <>
struct SortAcc<float> {
    typedef float type;
};

__device__ __forceinline__ int sort_bin(int len) { return len > kLongRow ? 0 : 1 + (kLongRow - len); }

int grid_of(int64_t work, int threads) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((work + threads - 1) / threads, device_sm_count() * 32));
}
}  // namespace

// One warp per tile: histogram of the tile's bins, written bin-major
// (hist[bin * nTiles + tile]) so one exclusive scan orders (bin, tile).
__global__ void ss_hist_kernel(int n, int nTiles, const int* __restrict__ rowptr, int* __restrict__ hist) {
    __shared__ int cnt[kBins];
    const int lane = threadIdx.x;
    for (int b = lane; b < kBins; b += 32) cnt[b] = 0;
    __syncwarp();
    const int tile = blockIdx.x;
    for (int k = 0; k < kTileRows; k += 32) {
        const int r = tile * kTileRows + k + lane;
        const bool valid = r < n;
        const int bin = valid ? sort_bin(rowptr[r + 1] - rowptr[r]) : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, bin);
        if (valid && lane == __ffs(peers) - 1) cnt[bin] += __popc(peers);
        __syncwarp();
    }
    for (int b = lane; b < kBins; b += 32) hist[b * nTiles + tile] = cnt[b];
}

// One warp per tile: stable scatter of the tile's rows to their sorted slots.
__global__ void ss_scatter_kernel(int n, int nTiles, const int* __restrict__ rowptr, const int* __restrict__ start,
                                  int* __restrict__ sorted) {
    __shared__ int next[kBins];
    const int lane = threadIdx.x;
    const int tile = blockIdx.x;
    for (int b = lane; b < kBins; b += 32) next[b] = start[b * nTiles + tile];
    __syncwarp();
    for (int k = 0; k < kTileRows; k += 32) {
        const int r = tile * kTileRows + k + lane;
        const bool valid = r < n;
        const int bin = valid ? sort_bin(rowptr[r + 1] - rowptr[r]) : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, bin);
        if (valid) sorted[next[bin] + __popc(peers & ((1u << lane) - 1u))] = r;
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) next[bin] += __popc(peers);
        __syncwarp();
    }
}

// Slice lengths (entries per lane, times 32) of the short rows.
__global__ void ss_slice_len_kernel(int n, int nLong, int nSlices, const int* __restrict__ rowptr,
                                    const int* __restrict__ sorted, int* __restrict__ sliceLen) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nSlices; s += gridDim.x * blockDim.x) {
        const int r = sorted[nLong + 32 * s];  // longest row of the slice
        sliceLen[s] = 32 * (rowptr[r + 1] - rowptr[r]);
    }
}

template <typename VT>
__global__ void ss_fill_kernel(int n, int nLong, int nSlices, const int* __restrict__ rowptr,
                               const int* __restrict__ col, const double* __restrict__ val,
                               const int* __restrict__ sorted, const int* __restrict__ sliceOff,
                               int* __restrict__ scol, VT* __restrict__ sval) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nSlices; s += warpsPerGrid) {
        const int off = sliceOff[s];
        const int len = (sliceOff[s + 1] - off) >> 5;
        const int pos = nLong + 32 * s + lane;
        const int r = pos < n ? sorted[pos] : -1;
        const int rs = r >= 0 ? rowptr[r] : 0;
        const int rl = r >= 0 ? rowptr[r + 1] - rs : 0;
        for (int j = 0; j < len; ++j) {
            const int dst = off + j * 32 + lane;
            if (j < rl) {
                if (scol) scol[dst] = col[rs + j];
                sval[dst] = (VT)val[rs + j];
            } else {
                if (scol) scol[dst] = r >= 0 ? r : 0;
                sval[dst] = VT(0);
            }
        }
    }
}

template <typename VT, int U>
__global__ void __launch_bounds__(kSortThreads) spmv_sellsort_kernel(
    int n, int nLong, int nSlices, const int* __restrict__ sorted, const int* __restrict__ sliceOff,
    const int* __restrict__ scol, const VT* __restrict__ sval, const int* __restrict__ rowptr,
    const int* __restrict__ col, const VT* __restrict__ val, const VT* __restrict__ x, VT* __restrict__ y,
    const VT* __restrict__ b, CgState* state, double* partials, int mode, const uint32_t* doneFlag) {
    typedef typename SortAcc<VT>::type AccT;
    if (doneFlag && *(volatile const uint32_t*)doneFlag) return;
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    const int items = nLong + nSlices;
    AccT dacc = AccT(0);
    for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < items; w += warpsPerGrid) {
        int row;
        AccT acc = AccT(0);
        if (w < nLong) {
            // long row: the warp strides along it
            row = sorted[w];
            const int j0 = rowptr[row], j1 = rowptr[row + 1];
            int j = j0 + lane;
            for (; j + 32 * (U - 1) < j1; j += 32 * U) {
                VT v[U];
                int c[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    v[u] = __ldcs(&val[j + 32 * u]);
                    c[u] = __ldcs(&col[j + 32 * u]);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) acc = fma((AccT)v[u], (AccT)__ldg(&x[c[u]]), acc);
            }
            for (; j < j1; j += 32) acc = fma((AccT)__ldcs(&val[j]), (AccT)__ldg(&x[__ldcs(&col[j])]), acc);
            acc = warp_sum(acc);
            if (lane != 0) continue;
        } else {
            // slice of 32 rows of nearly equal length: one lane per row
            const int s = w - nLong;
            const int pos = nLong + 32 * s + lane;
            row = pos < n ? sorted[pos] : -1;
            const int off = __ldg(&sliceOff[s]);
            const int len = (__ldg(&sliceOff[s + 1]) - off) >> 5;
            const VT* vp = sval + off + lane;
            const int* cp = scol + off + lane;
            int j = 0;
            for (; j + U <= len; j += U) {
                VT v[U];
                int c[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    v[u] = __ldcs(vp + (j + u) * 32);
                    c[u] = __ldcs(cp + (j + u) * 32);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) acc = fma((AccT)v[u], (AccT)__ldg(&x[c[u]]), acc);
            }
            for (; j < len; ++j) acc = fma((AccT)__ldcs(vp + j * 32), (AccT)__ldg(&x[__ldcs(cp + j * 32)]), acc);
            if (row < 0) continue;
        }
        if (mode == kSpmvResidual) {
            const AccT rv = (AccT)b[row] - acc;
            y[row] = (VT)rv;
            dacc = fma(rv, rv, dacc);
        } else {
            y[row] = (VT)acc;
            if (mode == kSpmvCgDot || mode == kSpmvCgPart) dacc = fma((AccT)x[row], acc, dacc);
        }
    }
    if (mode == kSpmvPlain) return;
    AccT v[1] = {dacc};
    block_sum<kSortThreads, 1, AccT>(v);
    double tot[1] = {(double)v[0]}, fin[1];
    if (mode == kSpmvCgPart) {
        if (threadIdx.x == 0) partials[blockIdx.x] = tot[0];
        return;
    }
    if (grid_sum_last<kSortThreads, 1>(tot, partials, &state->counters[0], fin)) {
        if (threadIdx.x == 0) {
            if (mode == kSpmvCgDot) {
                state->pAp = fin[0];
                state->alpha = state->rz / fin[0];
            } else {
                state->rrTrue = fin[0];
            }
        }
    }
}

// ---- host side ----
int sellsort_num_configs() { return 2; }
int sellsort_config_unroll(int cfg) { return cfg == 0 ? 4 : 8; }

int sellsort_tiles(int n) { return (n + kTileRows - 1) / kTileRows; }
int sellsort_bins() { return kBins; }

cudaError_t sellsort_order(cudaStream_t st, int n, const int* rowptr, int* hist, int* start, int* blockSums,
                           int* sorted, int* nLong) {
    const int nTiles = sellsort_tiles(n);
    ss_hist_kernel<<<nTiles, 32, 0, st>>>(n, nTiles, rowptr, hist);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = scan_exclusive(st, hist, start, kBins * nTiles, blockSums);
    if (e != cudaSuccess) return e;
    ss_scatter_kernel<<<nTiles, 32, 0, st>>>(n, nTiles, rowptr, start, sorted);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // long rows occupy bin 0, so bin 1 starts after them
    e = cudaMemcpyAsync(nLong, start + nTiles, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

cudaError_t sellsort_slices(cudaStream_t st, int n, int nLong, const int* rowptr, const int* sorted, int* sliceOff,
                            int* blockSums, int64_t* total) {
    const int nSlices = (n - nLong + 31) / 32;
    if (nSlices > 0) {
        ss_slice_len_kernel<<<grid_of(nSlices, 256), 256, 0, st>>>(n, nLong, nSlices, rowptr, sorted, sliceOff);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaMemsetAsync(sliceOff + nSlices, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    e = scan_exclusive(st, sliceOff, sliceOff, nSlices + 1, blockSums);
    if (e != cudaSuccess) return e;
    int t = 0;
    e = cudaMemcpyAsync(&t, sliceOff + nSlices, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    *total = t;
    return e;
}

template <typename VT>
cudaError_t sellsort_fill(cudaStream_t st, int n, int nLong, const int* rowptr, const int* col, const double* val,
                          const int* sorted, const int* sliceOff, int* scol, VT* sval) {
    const int nSlices = (n - nLong + 31) / 32;
    if (nSlices <= 0) return cudaSuccess;
    ss_fill_kernel<VT><<<grid_of((int64_t)nSlices * 32, 256), 256, 0, st>>>(n, nLong, nSlices, rowptr, col, val,
                                                                             sorted, sliceOff, scol, sval);
    return cudaGetLastError();
}

namespace {
template <typename VT, int U>
int ss_bps() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_sellsort_kernel<VT, U>, kSortThreads, 0) !=
        cudaSuccess)
        return 0;
    return nb;
}
}  // namespace

template <typename VT>
int sellsort_grid(int cfg, int n, int nLong, int numSms) {
    const int bps = sellsort_config_unroll(cfg) == 4 ? ss_bps<VT, 4>() : ss_bps<VT, 8>();
    if (bps <= 0) return 0;
    const int items = nLong + (n - nLong + 31) / 32;
    const int need = (items + kSortThreads / 32 - 1) / (kSortThreads / 32);
    return std::max(1, std::min(need, bps * numSms));
}

template <typename VT>
cudaError_t spmv_sellsort_launch(int cfg, int grid, cudaStream_t st, int n, int nLong, const int* sorted,
                                 const int* sliceOff, const int* scol, const VT* sval, const int* rowptr,
                                 const int* col, const VT* val, const VT* x, VT* y, const VT* b, CgState* state,
                                 double* partials, int mode, const uint32_t* doneFlag) {
    if (n <= 0) return cudaSuccess;
    const int nSlices = (n - nLong + 31) / 32;
    if (sellsort_config_unroll(cfg) == 4)
        spmv_sellsort_kernel<VT, 4><<<grid, kSortThreads, 0, st>>>(n, nLong, nSlices, sorted, sliceOff, scol, sval,
                                                                   rowptr, col, val, x, y, b, state, partials, mode,
                                                                   doneFlag);
    else
        spmv_sellsort_kernel<VT, 8><<<grid, kSortThreads, 0, st>>>(n, nLong, nSlices, sorted, sliceOff, scol, sval,
                                                                   rowptr, col, val, x, y, b, state, partials, mode,
                                                                   doneFlag);
    return cudaGetLastError();
}

template cudaError_t sellsort_fill<double>(cudaStream_t, int, int, const int*, const int*, const double*, const int*,
                                           const int*, int*, double*);
template cudaError_t sellsort_fill<float>(cudaStream_t, int, int, const int*, const int*, const double*, const int*,
                                          const int*, int*, float*);
template int sellsort_grid<double>(int, int, int, int);
template int sellsort_grid<float>(int, int, int, int);
template cudaError_t spmv_sellsort_launch<double>(int, int, cudaStream_t, int, int, const int*, const int*,
                                                  const int*, const double*, const int*, const int*, const double*,
                                                  const double*, double*, const double*, CgState*, double*, int,
                                                  const uint32_t*);
template cudaError_t spmv_sellsort_launch<float>(int, int, cudaStream_t, int, int, const int*, const int*, const int*,
                                                 const float*, const int*, const int*, const float*, const float*,
                                                 float*, const float*, CgState*, double*, int, const uint32_t*);

}  // namespace xjpcg
