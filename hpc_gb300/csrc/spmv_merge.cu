// spmv_merge.cu -- merge-path CSR SpMV for irregular (power-law) rows.
//
// The SpMV is a walk along the merge path of the row-end list
// (rowptr[1..n]) and the entry indices 0..nnz-1: each step either consumes an
// entry (acc += val * x[col]) or ends a row (emit acc).  The path has n + nnz
// steps; CTA t owns steps [t*TILE, (t+1)*TILE) and each of its threads ITEMS
// consecutive steps, so every thread does the same amount of work however
// the entries are spread over rows (a 4000-entry row costs the same as 4000
// rows of one entry).  The CTA stages its row ends and its entries into shared
// memory with coalesced loads (gathering x[col] for every entry while it does,
// so the gathers are all in flight at once), each thread finds its start by a binary search
// on the diagonal, walks its steps, and hands the partial sum of an unfinished
// row to its successor.  Rows that cross threads are finished in the CTA by
// adding the carries of the preceding threads in thread order; rows that
// cross CTAs leave a per-tile carry that a small fix-up kernel adds in tile
// order.  All sums have a fixed order, so results are bitwise reproducible.
//
// One DFMA per entry; a row split over k threads adds k - 1 DADDs.
//
// Modes: kPlain (y = A x) and kCgDot (y = A p, then p.y and alpha = rz / p.y
// into the solver state, the reference's krnl_storeApk step).  Rows whose value
// is completed by the fix-up contribute to p.y there.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

namespace {
constexpr int kMT = 256;     // threads per CTA
// Merge-path steps per thread.  Odd, so that the per-thread runs of staged
// values (read at stride ~kItems by consecutive threads) spread over the
// shared-memory banks instead of piling onto two of them.
constexpr int kItems = 7;
constexpr int kTile = kMT * kItems;

// Largest i in [lo, hi] with rowEnd(i-1) + i <= diag, i.e. the number of rows
// fully consumed before path step `diag`.  rowEnd(i) = rowptr[i + 1].
__device__ __forceinline__ int path_search(const int* rowptr, int diag, int lo, int hi) {
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;  // candidate row count
        // mid rows consumed needs rowptr[mid] entries before them: rowptr[mid] + mid <= diag
        if (__ldg(&rowptr[mid]) + mid <= diag)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}
}  // namespace

template <typename VT>
struct MergeAcc {
    typedef double type;
};
template <>
struct MergeAcc<float> {
    typedef float type;
};

template <typename VT>
__global__ void __launch_bounds__(kMT) spmv_merge_kernel(int n, int nnz, const int* __restrict__ rowptr,
                                                         const int* __restrict__ col, const VT* __restrict__ val,
                                                         const VT* __restrict__ x, VT* __restrict__ y,
                                                         const int* __restrict__ tileRow, int* __restrict__ carryRow,
                                                         typename MergeAcc<VT>::type* __restrict__ carryVal,
                                                         double* __restrict__ partials, CgState* state, int mode,
                                                         const uint32_t* doneFlag) {
    typedef typename MergeAcc<VT>::type AccT;
    __shared__ int sRowEnd[kTile + 1];      // rowptr[i0+1 ..] for the tile's rows
    __shared__ VT sVal[kTile];
    __shared__ VT sXg[kTile];  // x gathered at the entry's column while staging
    __shared__ int sCarryRow[kMT];
    __shared__ AccT sCarryVal[kMT];
    __shared__ int sBounds[4];

    if (doneFlag && *(volatile const uint32_t*)doneFlag) return;
    const int tid = threadIdx.x;
    const int total = n + nnz;
    const int d0 = blockIdx.x * kTile;
    const int d1 = min(d0 + kTile, total);
    if (tid == 0) {
        // tile start rows are computed once per matrix (merge_partition_kernel)
        const int i0 = tileRow[blockIdx.x];
        const int i1 = tileRow[blockIdx.x + 1];
        sBounds[0] = i0;
        sBounds[1] = d0 - i0;  // j0
        sBounds[2] = i1;
        sBounds[3] = d1 - i1;  // j1
    }
    __syncthreads();
    const int i0 = sBounds[0], j0 = sBounds[1], i1 = sBounds[2], j1 = sBounds[3];
    // Stage row ends of rows i0 .. min(i1, n-1) and the entries j0 .. j1 - 1.
    const int nrows = min(i1, n - 1) - i0 + 1;
    const int cnt = j1 - j0;
    // Unrolled so each thread has all its loads in flight at once; the
    // gathers of x are issued here, independent of each other, instead of one
    // per step inside the sequential walk below.
    int cidx[kItems];
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
        const int k = tid + u * kMT;
        cidx[u] = k < cnt ? __ldcs(&col[j0 + k]) : 0;
    }
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
        const int k = tid + u * kMT;
        if (k < cnt) {
            sXg[k] = __ldg(&x[cidx[u]]);
            sVal[k] = __ldcs(&val[j0 + k]);
        }
    }
#pragma unroll
    for (int u = 0; u <= kItems; ++u) {
        const int k = tid + u * kMT;
        if (k < nrows) sRowEnd[k] = __ldg(&rowptr[i0 + 1 + k]);
    }
    __syncthreads();

    // This thread's start on the path, searched inside the staged tile.
    const int dt = min(d0 + tid * kItems, d1);
    int lo = max(i0, dt - j1), hi = min(i1, dt - j0);
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int endPrev = mid > i0 ? sRowEnd[mid - 1 - i0] : j0;  // rowptr[mid] (>= j0 inside the tile)
        if (endPrev + mid <= dt)
            lo = mid;
        else
            hi = mid - 1;
    }
    int i = lo, j = dt - lo;
    const int de = min(dt + kItems, d1);
    AccT acc = AccT(0);
    int firstRow = -1;
    AccT firstVal = AccT(0);
    AccT dacc = AccT(0);
    // midRow: the thread's first row began before this thread's range.
    const int rowStartI = i < n ? (i > i0 ? sRowEnd[i - 1 - i0] : __ldg(&rowptr[i])) : nnz;
    const bool midRow = (i < n) && (j > rowStartI);
    for (int d = dt; d < de; ++d) {
        const int rend = i < n ? sRowEnd[i - i0] : nnz;
        if (j < rend) {
            acc = fma((AccT)sVal[j - j0], (AccT)sXg[j - j0], acc);
            ++j;
        } else {
            // row i ends here
            if (firstRow < 0 && midRow) {
                firstRow = i;
                firstVal = acc;
            } else {
                y[i] = (VT)acc;
                if (mode == kSpmvCgDot) dacc = fma((AccT)x[i], acc, dacc);
            }
            acc = AccT(0);
            ++i;
        }
    }
    sCarryRow[tid] = (i < n) ? i : -1;
    sCarryVal[tid] = acc;
    __syncthreads();
    // Finish the row this thread ended but did not start: add the carries of
    // the preceding threads of the same row, in thread order.
    if (firstRow >= 0) {
        int u = tid - 1;
        while (u >= 0 && sCarryRow[u] == firstRow) --u;
        AccT sum = AccT(0);
        for (int w = u + 1; w < tid; ++w) sum += sCarryVal[w];
        sum += firstVal;
        y[firstRow] = (VT)sum;
        // A row that also started in an earlier CTA is completed (and dotted)
        // by the fix-up; a row that started in this CTA is complete now.
        const bool fromEarlierTile = (u < 0) && (firstRow == i0) && (j0 > __ldg(&rowptr[i0]));
        if (mode == kSpmvCgDot && !fromEarlierTile) dacc = fma((AccT)x[firstRow], sum, dacc);
    }
    // Tile carry: the row still open at the end of the tile, summed over the
    // trailing threads that carry it, in thread order.
    // Only a row that the next tile enters mid-row (j1 > rowptr[i1]) carries;
    // the next tile then treats that row as started in an earlier tile.
    if (tid == kMT - 1) {
        const int r = sCarryRow[kMT - 1];
        const bool open = r >= 0 && d1 < total && i1 < n && j1 > __ldg(&rowptr[i1]);
        int u = kMT - 1;
        while (u > 0 && sCarryRow[u - 1] == r) --u;
        AccT sum = AccT(0);
        if (open)
            for (int w = u; w < kMT; ++w) sum += sCarryVal[w];
        carryRow[blockIdx.x] = open ? r : -1;
        carryVal[blockIdx.x] = sum;
    }
    if (mode == kSpmvCgDot) {
        AccT v[1] = {dacc};
        block_sum<kMT, 1, AccT>(v);
        if (tid == 0) partials[blockIdx.x] = (double)v[0];
    }
}

// Adds the tile carries to the rows they belong to (chains of tiles with the
// same open row are summed in tile order), then, in kCgDot mode, reduces the
// main kernel's CTA partials and the fix-up's own contributions in a fixed
// order and writes pAp and alpha.
template <typename VT>
__global__ void __launch_bounds__(kMT) spmv_merge_fixup_kernel(int ntiles, const int* __restrict__ carryRow,
                                                               const typename MergeAcc<VT>::type* __restrict__ carryVal,
                                                               const VT* __restrict__ x, VT* __restrict__ y,
                                                               double* __restrict__ partials, CgState* state, int mode,
                                                               const uint32_t* doneFlag) {
    typedef typename MergeAcc<VT>::type AccT;
    if (doneFlag && *(volatile const uint32_t*)doneFlag) return;
    AccT dacc = AccT(0);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
        const int r = carryRow[t];
        if (r < 0 || (t > 0 && carryRow[t - 1] == r)) continue;  // not the start of a chain
        AccT sum = AccT(0);
        for (int u = t; u < ntiles && carryRow[u] == r; ++u) sum += carryVal[u];
        const AccT yr = (AccT)y[r] + sum;
        y[r] = (VT)yr;
        if (mode == kSpmvCgDot) dacc = fma((AccT)x[r], yr, dacc);
    }
    if (mode != kSpmvCgDot) return;
    AccT v[1] = {dacc};
    block_sum<kMT, 1, AccT>(v);
    // partials[0 .. ntiles) hold the main kernel's CTA sums; the fix-up's
    // CTA sums go after them.
    double tot[1] = {(double)v[0]};
    __shared__ bool amLast;
    if (threadIdx.x == 0) {
        partials[ntiles + blockIdx.x] = tot[0];
        __threadfence();
        amLast = atomicAdd(&state->counters[4], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!amLast) return;
    __threadfence();
    __shared__ double fin;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const int count = ntiles + gridDim.x;
        double s = 0.0;
        for (int b = lane; b < count; b += 32) s += __ldcg(&partials[b]);
        s = warp_sum(s);
        if (lane == 0) {
            fin = s;
            state->counters[4] = 0u;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        state->pAp = fin;
        state->alpha = state->rz / fin;
    }
}

// Start row of every tile's path segment (ntiles + 1 entries); the matrix
// structure is fixed, so this runs once per matrix.
__global__ void merge_partition_kernel(int n, int nnz, int ntiles, const int* __restrict__ rowptr,
                                       int* __restrict__ tileRow) {
    const int total = n + nnz;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t <= ntiles; t += gridDim.x * blockDim.x) {
        const int d = min(t * kTile, total);
        tileRow[t] = path_search(rowptr, d, max(0, d - nnz), min(d, n));
    }
}

cudaError_t merge_partition(cudaStream_t st, int n, int nnz, const int* rowptr, int* tileRow) {
    const int ntiles = (int)(((int64_t)n + nnz + kTile - 1) / kTile);
    const int grid = std::max(1, std::min((ntiles + 256) / 256, device_sm_count() * 8));
    merge_partition_kernel<<<grid, 256, 0, st>>>(n, nnz, ntiles, rowptr, tileRow);
    return cudaGetLastError();
}

int merge_tiles(int n, int64_t nnz) { return (int)((n + nnz + kTile - 1) / kTile); }
int merge_items_per_thread() { return kItems; }
int merge_fixup_grid(int ntiles) { return std::max(1, std::min((ntiles + kMT - 1) / kMT, device_sm_count() * 4)); }

template <typename VT>
cudaError_t spmv_merge_launch(cudaStream_t st, int n, int nnz, const int* rowptr, const int* col, const VT* val,
                              const VT* x, VT* y, const int* tileRow, int* carryRow, void* carryVal, double* partials,
                              CgState* state, int mode, const uint32_t* doneFlag) {
    if (n <= 0) return cudaSuccess;
    typedef typename MergeAcc<VT>::type AccT;
    const int ntiles = merge_tiles(n, nnz);
    spmv_merge_kernel<VT><<<ntiles, kMT, 0, st>>>(n, nnz, rowptr, col, val, x, y, tileRow, carryRow,
                                                   static_cast<AccT*>(carryVal), partials, state, mode, doneFlag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    spmv_merge_fixup_kernel<VT><<<merge_fixup_grid(ntiles), kMT, 0, st>>>(
        ntiles, carryRow, static_cast<const AccT*>(carryVal), x, y, partials, state, mode, doneFlag);
    return cudaGetLastError();
}

template cudaError_t spmv_merge_launch<double>(cudaStream_t, int, int, const int*, const int*, const double*,
                                               const double*, double*, const int*, int*, void*, double*, CgState*,
                                               int, const uint32_t*);
template cudaError_t spmv_merge_launch<float>(cudaStream_t, int, int, const int*, const int*, const float*,
                                              const float*, float*, const int*, int*, void*, double*, CgState*, int,
                                              const uint32_t*);

}  // namespace xjpcg

namespace xjpcg {
// y = b - y (y holds A x from a plain SpMV) and ||y||^2 into state->rrTrue:
// the true-residual step of the refinement loop for the merge-path layout.
template <typename VT>
__global__ void __launch_bounds__(kMT) residual_finish_kernel(int n, const VT* __restrict__ b, VT* __restrict__ y,
                                                              double* partials, CgState* state,
                                                              const uint32_t* doneFlag) {
    if (doneFlag && *(volatile const uint32_t*)doneFlag) return;
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double r = (double)b[i] - (double)y[i];
        y[i] = (VT)r;
        acc = fma(r, r, acc);
    }
    double v[1] = {acc};
    block_sum<kMT, 1, double>(v);
    double fin[1];
    if (grid_sum_last<kMT, 1>(v, partials, &state->counters[0], fin) && threadIdx.x == 0) state->rrTrue = fin[0];
}

template <typename VT>
cudaError_t residual_finish_launch(cudaStream_t st, int n, const VT* b, VT* y, double* partials, CgState* state,
                                   const uint32_t* doneFlag) {
    const int grid = std::max(1, std::min((n + kMT - 1) / kMT, device_sm_count() * 8));
    residual_finish_kernel<VT><<<grid, kMT, 0, st>>>(n, b, y, partials, state, doneFlag);
    return cudaGetLastError();
}
template cudaError_t residual_finish_launch<double>(cudaStream_t, int, const double*, double*, double*, CgState*,
                                                    const uint32_t*);
}  // namespace xjpcg
