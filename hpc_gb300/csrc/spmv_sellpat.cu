// spmv_sellpat.cu -- sliced SpMV with column offsets shared by a slice.
//
// In a matrix from a structured grid, the 32 consecutive rows of a slice
// usually hold the same column offsets (col - row): the stencil.  Storing
// those offsets once per slice instead of once per entry removes the index
// stream altogether: 4 B per FP32 entry instead of 6, 8 B per FP64 entry
// instead of 10.  The gather address row + offset is then the same offset
// for every lane, so a warp's gather reads 32 consecutive x values.
//
// Per slice, the offsets of its 32 rows are merged (ascending, duplicates kept
// with their largest multiplicity) into the slice pattern.  A row that lacks
// one of the pattern's offsets (a boundary row of the grid) gets an explicit
// zero there.  Because the pattern is ascending and a row's own entries are
// ascending by column, every row is still summed in its CSR order, with
// fma(0, x, acc) = acc for the zeros: the results equal the plain sliced
// kernel's bit for bit.  A slice is stored this way ("shared") when its
// pattern adds at most 25 % zeros and every row + offset of every lane lies
// in [0, n); otherwise ("general") it keeps per-entry int32 columns.  A
// pattern equal to the previous slice's is not stored again.
//
// Run-aware gathers (the RUNS form).  A stencil's offsets come in runs of
// consecutive values (o, o + 1, o + 2 for the three x-neighbours of a
// 27-point stencil).  For offset o + 1, lane l needs x[row0 + l + o + 1],
// which lane l + 1 already gathered for offset o: the warp passes it down
// with one shuffle, and only lane 31 loads its value.  A run of three then
// costs one 32-wide gather and two one-lane loads instead of three 32-wide
// gathers, which cuts the L2 sectors the x gathers read by about half.  The
// values and the order of the FMAs are unchanged, so the sums are the same
// bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

namespace {
constexpr int kPatThreads = 256;
constexpr int kEnd = 0x7fffffff;  // exhausted lane in the merge

template <typename VT>
struct PatAcc {
    typedef double type;
};
template <>
struct PatAcc<float> {
    typedef float type;
};

int grid_of(int64_t work, int threads) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((work + threads - 1) / threads, device_sm_count() * 32));
}

__device__ __forceinline__ int warp_min(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_sum_int(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
}  // namespace

// One warp per slice: stored values of the slice (32 x pattern length for a
// shared slice, 32 x longest row for a general one), pattern length (0 = a
// general slice) and general-slice columns.
__global__ void sp_plan_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                               int* __restrict__ lenOut, int* __restrict__ patLen, int* __restrict__ genLen) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    const int nslices = (n + 31) / 32;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warpsPerGrid) {
        const int row = s * 32 + lane;
        const bool real = row < n;
        const int j0 = real ? rowptr[row] : 0, j1 = real ? rowptr[row + 1] : 0;
        const int maxLen = warp_max(j1 - j0);
        const int sumLen = warp_sum_int(j1 - j0);
        const bool full = warp_max(real ? 0 : 1) == 0;  // no phantom rows
        // Merge of the rows' offsets, stopped once the pattern would pad more
        // than 25 % (32 L > 1.25 sumLen).  Every step advances at least one
        // lane, so the loop is also bounded by the slice's entries.
        const int lMax = (int)((5ll * sumLen) / 128);
        int j = j0, L = 0;
        bool inRange = true, tooLong = false;
        while (true) {
            const int head = j < j1 ? col[j] - row : kEnd;
            const int m = warp_min(head);
            if (m == kEnd) break;
            if (++L > lMax) {
                tooLong = true;
                break;
            }
            if (head == m) ++j;
            // every lane gathers x[row + m]: it must exist
            const long long c = (long long)row + m;
            inRange = inRange && c >= 0 && c < n;
        }
        const bool allIn = warp_min(inRange ? 1 : 0) == 1;
        const bool shared = full && allIn && !tooLong && L > 0;
        if (lane == 0) {
            lenOut[s] = 32 * (shared ? L : maxLen);
            patLen[s] = shared ? L : 0;
            genLen[s] = shared ? 0 : 32 * maxLen;
        }
    }
}

// Pattern dedupe against the previous slice (same length and same offsets).
__global__ void sp_dedupe_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                 const int* __restrict__ patLen, int* __restrict__ patNew) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    const int nslices = (n + 31) / 32;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warpsPerGrid) {
        const int L = patLen[s];
        if (L == 0) {
            if (lane == 0) patNew[s] = 0;
            continue;
        }
        bool same = s > 0 && patLen[s - 1] == L;
        if (same) {
            // rebuild both patterns in lockstep and compare
            const int rowA = (s - 1) * 32 + lane, rowB = s * 32 + lane;
            int ja = rowptr[rowA], ja1 = rowptr[rowA + 1];
            int jb = rowptr[rowB], jb1 = rowptr[rowB + 1];
            for (int k = 0; k < L && same; ++k) {
                const int ha = ja < ja1 ? col[ja] - rowA : kEnd;
                const int hb = jb < jb1 ? col[jb] - rowB : kEnd;
                const int ma = warp_min(ha), mb = warp_min(hb);
                same = ma == mb;
                if (ha == ma) ++ja;
                if (hb == mb) ++jb;
            }
        }
        if (lane == 0) patNew[s] = same ? 0 : 1;
    }
}

// Values (and per-entry columns of general slices, and the stored patterns).
template <typename VT>
__global__ void sp_fill_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                               const double* __restrict__ val, const int* __restrict__ sliceOff,
                               const int* __restrict__ patLen, const int* __restrict__ patNew,
                               const int* __restrict__ patIdx, const int* __restrict__ patOff,
                               const int* __restrict__ genOff, VT* __restrict__ sval, int* __restrict__ pat,
                               int* __restrict__ gcol, int writeIndex) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    const int nslices = (n + 31) / 32;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warpsPerGrid) {
        const int off = sliceOff[s];
        const int len = (sliceOff[s + 1] - off) >> 5;
        const int row = s * 32 + lane;
        const bool real = row < n;
        const int j0 = real ? rowptr[row] : 0, j1 = real ? rowptr[row + 1] : 0;
        const int L = patLen[s];
        if (L > 0) {
            int* p = pat + patOff[patIdx[s]];
            const bool store = writeIndex && patNew[s];
            int j = j0;
            for (int k = 0; k < L; ++k) {
                const int head = j < j1 ? col[j] - row : kEnd;
                const int m = warp_min(head);
                VT v = VT(0);
                if (head == m) {
                    v = (VT)val[j];
                    ++j;
                }
                sval[off + k * 32 + lane] = v;
                if (store && lane == 0) p[k] = m;
            }
        } else {
            const int g = genOff[s];
            for (int k = 0; k < len; ++k) {
                const bool has = j0 + k < j1;
                sval[off + k * 32 + lane] = has ? (VT)val[j0 + k] : VT(0);
                if (writeIndex) gcol[g + k * 32 + lane] = has ? col[j0 + k] : (real ? row : 0);
            }
        }
    }
}


template <typename VT, int U, bool RUNS>
__global__ void __launch_bounds__(kPatThreads, 6) spmv_sellpat_kernel(
    int n, int nslices, const int* __restrict__ sliceOff, const int* __restrict__ patLen,
    const int* __restrict__ patIdx, const int* __restrict__ patOff, const int* __restrict__ genOff,
    const int* __restrict__ pat, const int* __restrict__ gcol, const VT* __restrict__ sval,
    const VT* __restrict__ x, VT* __restrict__ y, const VT* __restrict__ b, CgState* state, double* partials,
    int mode, const uint32_t* doneFlag) {
    typedef typename PatAcc<VT>::type AccT;
    if (doneFlag && *(volatile const uint32_t*)doneFlag) return;
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    AccT dacc = AccT(0);
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warpsPerGrid) {
        const int off = __ldg(&sliceOff[s]);
        const int len = (__ldg(&sliceOff[s + 1]) - off) >> 5;
        const int row = s * 32 + lane;
        const VT* vp = sval + off + lane;
        AccT acc = AccT(0);
        const int L = __ldg(&patLen[s]);
        if (L > 0) {
            // shared offsets: one warp-uniform offset per stored column
            const int* p = pat + __ldg(&patOff[__ldg(&patIdx[s])]);
            const VT* xr = x + row;
            int j = 0;
            if (RUNS) {
                // oPrev / xPrev: the previous stored column's offset (warp-
                // uniform) and this lane's x value for it.
                int oPrev = -0x7fffffff;
                VT xPrev = VT(0);
                for (; j + U <= len; j += U) {
                    VT v[U], xg[U];
                    int o[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        v[u] = ld_val(vp + (j + u) * 32);
                        o[u] = __ldg(p + j + u);
                    }
                    bool c[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        c[u] = o[u] == (u == 0 ? oPrev : o[u - 1]) + 1;
                        xg[u] = (!c[u] || lane == 31) ? __ldg(xr + o[u]) : VT(0);
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const VT down = __shfl_down_sync(0xffffffffu, xPrev, 1);
                        const VT xv = (c[u] && lane != 31) ? down : xg[u];
                        acc = fma((AccT)v[u], (AccT)xv, acc);
                        xPrev = xv;
                    }
                    oPrev = o[U - 1];
                }
                for (; j < len; ++j) {
                    const VT v = ld_val(vp + j * 32);
                    const int o = __ldg(p + j);
                    const bool c = o == oPrev + 1;
                    const VT xg = (!c || lane == 31) ? __ldg(xr + o) : VT(0);
                    const VT down = __shfl_down_sync(0xffffffffu, xPrev, 1);
                    const VT xv = (c && lane != 31) ? down : xg;
                    acc = fma((AccT)v, (AccT)xv, acc);
                    xPrev = xv;
                    oPrev = o;
                }
            } else {
                for (; j + U <= len; j += U) {
                    VT v[U];
                    int o[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        v[u] = ld_val(vp + (j + u) * 32);
                        o[u] = __ldg(p + j + u);
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) acc = fma((AccT)v[u], (AccT)__ldg(xr + o[u]), acc);
                }
                for (; j < len; ++j) acc = fma((AccT)ld_val(vp + j * 32), (AccT)__ldg(xr + __ldg(p + j)), acc);
            }
        } else {
            const int* cp = gcol + __ldg(&genOff[s]) + lane;
            int j = 0;
            for (; j + U <= len; j += U) {
                VT v[U];
                int c[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    v[u] = ld_val(vp + (j + u) * 32);
                    c[u] = __ldcs(cp + (j + u) * 32);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) acc = fma((AccT)v[u], (AccT)__ldg(&x[c[u]]), acc);
            }
            for (; j < len; ++j) acc = fma((AccT)ld_val(vp + j * 32), (AccT)__ldg(&x[__ldcs(cp + j * 32)]), acc);
        }
        if (row < n) {
            if (mode == kSpmvResidual) {
                const AccT rv = (AccT)b[row] - acc;
                y[row] = (VT)rv;
                dacc = fma(rv, rv, dacc);
            } else {
                y[row] = (VT)acc;
                if (mode == kSpmvCgDot || mode == kSpmvCgPart) dacc = fma((AccT)x[row], acc, dacc);
            }
        }
    }
    if (mode == kSpmvPlain) return;
    AccT v[1] = {dacc};
    block_sum<kPatThreads, 1, AccT>(v);
    double tot[1] = {(double)v[0]}, fin[1];
    if (mode == kSpmvCgPart) {
        if (threadIdx.x == 0) partials[blockIdx.x] = tot[0];
        return;
    }
    if (grid_sum_last<kPatThreads, 1>(tot, partials, &state->counters[0], fin)) {
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

// TMA-fed form (FP32).  Each warp walks its slices as the plain kernel does,
// but lane 0 prefetches the whole value block of the warp's next shared slice
// (32 rows x its stored columns, contiguous) into shared memory with one
// cp.async.bulk on an mbarrier while the warp computes the current slice from
// the other buffer.  A warp thus keeps a whole slice (3.5 KB for a 27-point
// stencil) in flight with no registers held for it.  Slices with per-entry
// columns, or more than kTmaCols stored columns, take the plain loads.  Every
// wait is bounded (2 s); on expiry the warp drains both of its copies (bounded),
// records kStatusWaitTimeout, marks the loop done and stops.  The FMAs run in
// the plain kernel's order, so the sums are the same bit for bit.
constexpr int kTmaCols = 32;
constexpr uint64_t kTmaWaitNs = 2000000000ull;

// Slice t is prefetched when it has shared offsets and fits a buffer.
__device__ __forceinline__ bool tma_fetchable(const int* __restrict__ sliceOff, const int* __restrict__ patLen, int t,
                                              int& off, int& len) {
    off = __ldg(&sliceOff[t]);
    len = (__ldg(&sliceOff[t + 1]) - off) >> 5;
    return __ldg(&patLen[t]) > 0 && len > 0 && len <= kTmaCols;
}

template <typename VT, int U>
__global__ void __launch_bounds__(kPatThreads, 3) spmv_sellpat_tma_kernel(
    int n, int nslices, const int* __restrict__ sliceOff, const int* __restrict__ patLen,
    const int* __restrict__ patIdx, const int* __restrict__ patOff, const int* __restrict__ genOff,
    const int* __restrict__ pat, const int* __restrict__ gcol, const VT* __restrict__ sval,
    const VT* __restrict__ x, VT* __restrict__ y, const VT* __restrict__ b, CgState* state, double* partials,
    int mode, const uint32_t* doneFlag) {
    typedef typename PatAcc<VT>::type AccT;
    extern __shared__ __align__(128) unsigned char tmaSmem[];
    __shared__ __align__(8) uint64_t bars[kPatThreads / 32][2];
    if (doneFlag && *(volatile const uint32_t*)doneFlag) return;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    VT* bufs = reinterpret_cast<VT*>(tmaSmem) + (size_t)wid * 2 * kTmaCols * 32;
    if (lane == 0) {
        mbar_init(&bars[wid][0], 1);
        mbar_init(&bars[wid][1], 1);
        mbar_fence_init();
    }
    __syncwarp();
    const uint64_t pol = l2_policy_evict_first();
    uint32_t phase0 = 0u, phase1 = 0u;  // parity of each buffer's next completion
    bool abort = false;
    AccT dacc = AccT(0);
    int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int off = 0, len = 0;
    bool fits = s < nslices && tma_fetchable(sliceOff, patLen, s, off, len);
    if (fits && lane == 0) {
        const uint32_t bytes = (uint32_t)(len * 32 * sizeof(VT));
        mbar_arrive_expect_tx(&bars[wid][0], bytes);
        bulk_g2s(bufs, sval + off, bytes, &bars[wid][0], pol);
    }
    for (int k = 0; s < nslices; s += warpsPerGrid, ++k) {
        const int cb = k & 1;
        VT* cur = bufs + cb * kTmaCols * 32;
        VT* nxt = bufs + (cb ^ 1) * kTmaCols * 32;
        const int sn = s + warpsPerGrid;
        int offn = 0, lenn = 0;
        const bool fitsn = sn < nslices && tma_fetchable(sliceOff, patLen, sn, offn, lenn);
        if (fitsn && lane == 0) {
            const uint32_t bytes = (uint32_t)(lenn * 32 * sizeof(VT));
            mbar_arrive_expect_tx(&bars[wid][cb ^ 1], bytes);
            bulk_g2s(nxt, sval + offn, bytes, &bars[wid][cb ^ 1], pol);
        }
        const int row = s * 32 + lane;
        AccT acc = AccT(0);
        if (fits) {
            const uint32_t ph = cb ? phase1 : phase0;
            const bool ok = mbar_wait_bounded(&bars[wid][cb], ph, kTmaWaitNs);
            if (cb)
                phase1 ^= 1u;
            else
                phase0 ^= 1u;
            if (__any_sync(0xffffffffu, !ok)) {
                abort = true;
                // drain both copies this warp may have in flight, the one it
                // gave up on and the prefetch (each wait bounded)
                mbar_wait_bounded(&bars[wid][cb], ph, kTmaWaitNs);
                if (fitsn) mbar_wait_bounded(&bars[wid][cb ^ 1], cb ? phase0 : phase1, kTmaWaitNs);
                break;
            }
            const int* p = pat + __ldg(&patOff[__ldg(&patIdx[s])]);
            const VT* xr = x + row;
            int j = 0;
            for (; j + U <= len; j += U) {
                VT v[U];
                int o[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    v[u] = cur[(j + u) * 32 + lane];
                    o[u] = __ldg(p + j + u);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) acc = fma((AccT)v[u], (AccT)__ldg(xr + o[u]), acc);
            }
            for (; j < len; ++j) acc = fma((AccT)cur[j * 32 + lane], (AccT)__ldg(xr + __ldg(p + j)), acc);
        } else {
            const int offp = __ldg(&sliceOff[s]);
            const int lenp = (__ldg(&sliceOff[s + 1]) - offp) >> 5;
            const VT* vp = sval + offp + lane;
            if (__ldg(&patLen[s]) > 0) {
                const int* p = pat + __ldg(&patOff[__ldg(&patIdx[s])]);
                const VT* xr = x + row;
                for (int j = 0; j < lenp; ++j) acc = fma((AccT)__ldcs(vp + j * 32), (AccT)__ldg(xr + __ldg(p + j)), acc);
            } else {
                const int* cp = gcol + __ldg(&genOff[s]) + lane;
                for (int j = 0; j < lenp; ++j)
                    acc = fma((AccT)__ldcs(vp + j * 32), (AccT)__ldg(&x[__ldcs(cp + j * 32)]), acc);
            }
        }
        if (row < n) {
            if (mode == kSpmvResidual) {
                const AccT rv = (AccT)b[row] - acc;
                y[row] = (VT)rv;
                dacc = fma(rv, rv, dacc);
            } else {
                y[row] = (VT)acc;
                if (mode == kSpmvCgDot || mode == kSpmvCgPart) dacc = fma((AccT)x[row], acc, dacc);
            }
        }
        __syncwarp();  // every lane is done with cur before it is refilled
        fits = fitsn;
        off = offn;
        len = lenn;
    }
    if (abort && lane == 0) {
        atomicOr(&state->status, kStatusWaitTimeout);
        *(volatile uint32_t*)&state->done = 1u;  // later kernels of the loop stand down
    }
    if (mode == kSpmvPlain) return;
    AccT v[1] = {dacc};
    block_sum<kPatThreads, 1, AccT>(v);
    double tot[1] = {(double)v[0]}, fin[1];
    if (mode == kSpmvCgPart) {
        if (threadIdx.x == 0) partials[blockIdx.x] = tot[0];
        return;
    }
    if (grid_sum_last<kPatThreads, 1>(tot, partials, &state->counters[0], fin)) {
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
// Unroll 4 and 8 (an unroll-16 build at 64 registers measured slower in
// both precisions), then, FP32 only, the TMA-fed unroll 4 and 8.
// 0, 1: plain loads, unroll 4 / 8; 2, 3: TMA-fed values (FP32 only), unroll
// 4 / 8; 4, 5: run-aware gathers, unroll 4 / 8.
int sellpat_num_configs() { return 6; }
int sellpat_config_unroll(int cfg) { return (cfg & 1) ? 8 : 4; }
int sellpat_config_tma(int cfg) { return (cfg == 2 || cfg == 3) ? 1 : 0; }
int sellpat_config_runs(int cfg) { return cfg >= 4 ? 1 : 0; }

// Plans the layout.  Per slice (nslices + 1 ints each): sliceOff (values),
// patLen, patNew, patIdx (before sellpat_index: the scan of patNew), genOff.
// totals = {stored values, general-slice columns, stored patterns}.
cudaError_t sellpat_plan(cudaStream_t st, int n, const int* rowptr, const int* col, int* sliceOff, int* patLen,
                         int* patNew, int* patIdx, int* genOff, int* blockSums, int64_t* totals) {
    const int nslices = (n + 31) / 32;
    const int grid = grid_of((int64_t)nslices * 32, 256);
    sp_plan_kernel<<<grid, 256, 0, st>>>(n, rowptr, col, sliceOff, patLen, genOff);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    sp_dedupe_kernel<<<grid, 256, 0, st>>>(n, rowptr, col, patLen, patNew);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    for (int* a : {sliceOff, genOff, patNew})
        if ((e = cudaMemsetAsync(a + nslices, 0, sizeof(int), st)) != cudaSuccess) return e;
    // pattern index per slice: exclusive scan of patNew gives the index of
    // each stored pattern; a reused pattern takes the index of the previous
    // stored one (scan value - 1 + patNew)
    if ((e = scan_exclusive(st, patNew, patIdx, nslices + 1, blockSums)) != cudaSuccess) return e;
    if ((e = scan_exclusive(st, sliceOff, sliceOff, nslices + 1, blockSums)) != cudaSuccess) return e;
    if ((e = scan_exclusive(st, genOff, genOff, nslices + 1, blockSums)) != cudaSuccess) return e;
    int h[3];
    if ((e = cudaMemcpyAsync(&h[0], sliceOff + nslices, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(&h[1], genOff + nslices, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(&h[2], patIdx + nslices, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    totals[0] = h[0];
    totals[1] = h[1];
    totals[2] = h[2];  // stored patterns
    return cudaSuccess;
}

// Per-slice pattern index fix-up and pattern offsets.
__global__ void sp_patidx_kernel(int nslices, const int* __restrict__ patLen, const int* __restrict__ patNew,
                                 int* __restrict__ patIdx, int* __restrict__ storedLen) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nslices; s += gridDim.x * blockDim.x) {
        if (patLen[s] == 0) continue;
        const int idx = patIdx[s] + patNew[s] - 1;  // stored pattern this slice uses
        patIdx[s] = idx;
        if (patNew[s]) storedLen[idx] = patLen[s];
    }
}

cudaError_t sellpat_index(cudaStream_t st, int n, const int* patLen, const int* patNew, int* patIdx, int nPatterns,
                          int* patOff, int* blockSums, int64_t* patTotal) {
    const int nslices = (n + 31) / 32;
    sp_patidx_kernel<<<grid_of(nslices, 256), 256, 0, st>>>(nslices, patLen, patNew, patIdx, patOff);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(patOff + nPatterns, 0, sizeof(int), st)) != cudaSuccess) return e;
    if ((e = scan_exclusive(st, patOff, patOff, nPatterns + 1, blockSums)) != cudaSuccess) return e;
    int t = 0;
    if ((e = cudaMemcpyAsync(&t, patOff + nPatterns, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
    e = cudaStreamSynchronize(st);
    *patTotal = t;
    return e;
}

template <typename VT>
cudaError_t sellpat_fill(cudaStream_t st, int n, const int* rowptr, const int* col, const double* val,
                         const int* sliceOff, const int* patLen, const int* patNew, const int* patIdx,
                         const int* patOff, const int* genOff, VT* sval, int* pat, int* gcol, bool writeIndex) {
    const int nslices = (n + 31) / 32;
    sp_fill_kernel<VT><<<grid_of((int64_t)nslices * 32, 256), 256, 0, st>>>(
        n, rowptr, col, val, sliceOff, patLen, patNew, patIdx, patOff, genOff, sval, pat, gcol, writeIndex ? 1 : 0);
    return cudaGetLastError();
}

namespace {
template <typename VT, int U, bool RUNS>
int sp_bps() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_sellpat_kernel<VT, U, RUNS>, kPatThreads, 0) !=
        cudaSuccess)
        return 0;
    return nb;
}

constexpr size_t kTmaSmem = (size_t)(kPatThreads / 32) * 2 * kTmaCols * 32 * sizeof(float);

template <int U>
int sp_tma_bps() {
    int nb = 0;
    if (cudaFuncSetAttribute(spmv_sellpat_tma_kernel<float, U>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kTmaSmem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_sellpat_tma_kernel<float, U>, kPatThreads,
                                                      kTmaSmem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return nb;
}

template <typename VT>
int sp_config_bps(int cfg) {
    if (cfg == 0) return sp_bps<VT, 4, false>();
    if (cfg == 1) return sp_bps<VT, 8, false>();
    if (cfg == 4) return sp_bps<VT, 4, true>();
    if (cfg == 5) return sp_bps<VT, 8, true>();
    if (!std::is_same<VT, float>::value) return 0;  // the TMA-fed forms are FP32 only
    if (cfg == 2) return sp_tma_bps<4>();
    if (cfg == 3) return sp_tma_bps<8>();
    return 0;
}

template <typename VT>
struct PatTma {
    template <typename... A>
    static cudaError_t launch(int, int, cudaStream_t, A...) {
        return cudaErrorInvalidValue;
    }
};
template <>
struct PatTma<float> {
    template <typename... A>
    static cudaError_t launch(int cfg, int grid, cudaStream_t st, A... args) {
        if (cfg == 2)
            spmv_sellpat_tma_kernel<float, 4><<<grid, kPatThreads, kTmaSmem, st>>>(args...);
        else
            spmv_sellpat_tma_kernel<float, 8><<<grid, kPatThreads, kTmaSmem, st>>>(args...);
        return cudaGetLastError();
    }
};
}  // namespace

template <typename VT>
int sellpat_grid(int cfg, int n, int numSms) {
    const int bps = sp_config_bps<VT>(cfg);
    if (bps <= 0) return 0;
    const int nslices = (n + 31) / 32;
    const int need = (nslices + kPatThreads / 32 - 1) / (kPatThreads / 32);
    return std::max(1, std::min(need, bps * numSms));
}

template <typename VT>
cudaError_t spmv_sellpat_launch(int cfg, int grid, cudaStream_t st, int n, const int* sliceOff, const int* patLen,
                                const int* patIdx, const int* patOff, const int* genOff, const int* pat,
                                const int* gcol, const VT* sval, const VT* x, VT* y, const VT* b, CgState* state,
                                double* partials, int mode, const uint32_t* doneFlag) {
    if (n <= 0) return cudaSuccess;
    const int nslices = (n + 31) / 32;
    if (sellpat_config_tma(cfg))
        return PatTma<VT>::launch(cfg, grid, st, n, nslices, sliceOff, patLen, patIdx, patOff, genOff, pat, gcol,
                                  sval, x, y, b, state, partials, mode, doneFlag);
#define XJ_SELLPAT(U, R)                                                                                        \
    spmv_sellpat_kernel<VT, U, R><<<grid, kPatThreads, 0, st>>>(n, nslices, sliceOff, patLen, patIdx, patOff, genOff, \
                                                                pat, gcol, sval, x, y, b, state, partials, mode,      \
                                                                doneFlag)
    const bool runs = sellpat_config_runs(cfg) != 0;
    if (sellpat_config_unroll(cfg) == 4) {
        if (runs)
            XJ_SELLPAT(4, true);
        else
            XJ_SELLPAT(4, false);
    } else {
        if (runs)
            XJ_SELLPAT(8, true);
        else
            XJ_SELLPAT(8, false);
    }
#undef XJ_SELLPAT
    return cudaGetLastError();
}

template cudaError_t sellpat_fill<double>(cudaStream_t, int, const int*, const int*, const double*, const int*,
                                          const int*, const int*, const int*, const int*, const int*, double*, int*,
                                          int*, bool);
template cudaError_t sellpat_fill<float>(cudaStream_t, int, const int*, const int*, const double*, const int*,
                                         const int*, const int*, const int*, const int*, const int*, float*, int*,
                                         int*, bool);
template int sellpat_grid<double>(int, int, int);
template int sellpat_grid<float>(int, int, int);
template cudaError_t spmv_sellpat_launch<double>(int, int, cudaStream_t, int, const int*, const int*, const int*,
                                                 const int*, const int*, const int*, const int*, const double*,
                                                 const double*, double*, const double*, CgState*, double*, int,
                                                 const uint32_t*);
template cudaError_t spmv_sellpat_launch<float>(int, int, cudaStream_t, int, const int*, const int*, const int*,
                                                const int*, const int*, const int*, const int*, const float*,
                                                const float*, float*, const float*, CgState*, double*, int,
                                                const uint32_t*);

}  // namespace xjpcg
