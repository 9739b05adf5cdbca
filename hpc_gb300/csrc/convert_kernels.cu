// convert_kernels.cu -- device-side format conversion.
//
// COO (C or Fortran base) -> CSR in the order the reference partitioner stores
// a matrix: rows ascending, and inside a row the entries ordered by column,
// equal columns (duplicates, which are kept) in input order.  That is the net
// order of SparseMatrix::sort_by_row (L2/sparse/include/sw/fp64/
// matrix_params.hpp:219-246) followed by the per-row-block sort_by_col and the
// per-partition sort_by_row of Signature::gen_pars / create_padPar
// (signature.hpp:135-169, 233-236).  The permutation perm[j] = input position
// of CSR slot j is kept, so a later values-only update (KEEP_NZ_LAYOUT) is a
// gather.
//
// Steps: one pass counts rows, checks bounds and detects input that is already
// in (row, col) order; an exclusive scan gives rowptr; unsorted input is
// scattered into row slots with 64-bit keys (col << 32 | position) and every
// row is sorted by key (warp bitonic for rows <= 32, CTA bitonic in shared
// memory for rows <= 4096, CTA bitonic in global scratch above that).  Sorting
// by the full key makes the result independent of the scatter's atomic order.
//
// Symmetric half-CSC -> full COO follows the reference's emission order
// (matrix_params.hpp:82-134 for indices, gen_signature.hpp:73-112 for values):
// for column j, entry k: (i, j) and, when i != j, (j, i), both with data[k].
#include <cstdio>
#include <vector>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

constexpr int kScanThreads = 1024;
constexpr int kScanPerThread = 4;
constexpr int kScanTile = kScanThreads * kScanPerThread;

int scan_block_count(int count) { return (count + kScanTile - 1) / kScanTile; }

__device__ __forceinline__ int block_exclusive_scan_int(int v, int* total) {
    __shared__ int wsum[kScanThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int w = lane < kScanThreads / 32 ? wsum[lane] : 0;
        int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < kScanThreads / 32) wsum[lane] = wi - w;
        if (lane == kScanThreads / 32 - 1) *total = wi;
    }
    __syncthreads();
    const int res = inc - v + wsum[wid];
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const int* __restrict__ in, int count,
                                                                   int* __restrict__ blockSums) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanPerThread;
    int s = 0;
#pragma unroll
    for (int i = 0; i < kScanPerThread; ++i)
        if (base + i < count) s += in[base + i];
    s = warp_sum(s);
    __shared__ int ws[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        int t = threadIdx.x < kScanThreads / 32 ? ws[threadIdx.x] : 0;
        t = warp_sum(t);
        if (threadIdx.x == 0) blockSums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_blocksums_kernel(int* blockSums, int nb) {
    __shared__ int total;
    int carry = 0;
    for (int base = 0; base < nb; base += kScanThreads) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? blockSums[i] : 0;
        const int ex = block_exclusive_scan_int(v, &total);
        if (i < nb) blockSums[i] = ex + carry;
        carry += total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const int* in, int* out, int count,
                                                                  const int* __restrict__ blockSums) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanPerThread;
    int v[kScanPerThread];
    int s = 0;
#pragma unroll
    for (int i = 0; i < kScanPerThread; ++i) {
        v[i] = base + i < count ? in[base + i] : 0;
        s += v[i];
    }
    __shared__ int total;
    int ex = block_exclusive_scan_int(s, &total) + blockSums[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanPerThread; ++i) {
        if (base + i < count) out[base + i] = ex;
        ex += v[i];
    }
}

cudaError_t scan_exclusive(cudaStream_t st, const int* in, int* out, int count, int* blockSums) {
    if (count <= 0) return cudaSuccess;
    const int nb = scan_block_count(count);
    scan_reduce_kernel<<<nb, kScanThreads, 0, st>>>(in, count, blockSums);
    scan_blocksums_kernel<<<1, kScanThreads, 0, st>>>(blockSums, nb);
    scan_apply_kernel<<<nb, kScanThreads, 0, st>>>(in, out, count, blockSums);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// COO -> CSR
// ---------------------------------------------------------------------------
// flags[0]: error bits, flags[1]: 1 if the input is out of (row, col) order,
// flags[2]: count of rows 32 < len <= 4096, flags[3]: count of longer rows.
__global__ void coo_count_kernel(int64_t nnz, const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
                                 uint32_t base, uint32_t n, int* __restrict__ counts, int* flags) {
    bool bad = false, unsorted = false;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t r = row[k] - base, c = col[k] - base;
        if (r >= n || c >= n) {
            bad = true;
            continue;
        }
        atomicAdd(&counts[r], 1);
        if (k + 1 < nnz) {
            const uint32_t r2 = row[k + 1] - base, c2 = col[k + 1] - base;
            if (r2 < r || (r2 == r && c2 < c)) unsorted = true;
        }
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&flags[0], (int)kStatusIndexError);
    if (__any_sync(0xffffffffu, unsorted) && (threadIdx.x & 31) == 0) atomicOr(&flags[1], 1);
}

__global__ void coo_identity_kernel(int64_t nnz, const uint32_t* __restrict__ col, uint32_t base,
                                    int* __restrict__ colOut, uint32_t* __restrict__ perm) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        colOut[k] = (int)(col[k] - base);
        perm[k] = (uint32_t)k;
    }
}

__global__ void coo_scatter_kernel(int64_t nnz, const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
                                   uint32_t base, const int* __restrict__ rowptr, int* __restrict__ fill,
                                   uint64_t* __restrict__ keys) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t r = row[k] - base, c = col[k] - base;
        const int pos = rowptr[r] + atomicAdd(&fill[r], 1);
        keys[pos] = ((uint64_t)c << 32) | (uint64_t)(uint32_t)k;
    }
}

// One warp per row: rows of length <= 32 are sorted in registers; longer rows
// are appended to the medium / long lists for the CTA sorters.
__global__ void row_sort_warp_kernel(int n, const int* __restrict__ rowptr, uint64_t* __restrict__ keys,
                                     int* medList, int* longList, int* flags) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warpsPerGrid) {
        const int s = rowptr[r], len = rowptr[r + 1] - s;
        if (len <= 1) continue;
        if (len > 32) {
            if (lane == 0) {
                if (len <= 4096)
                    medList[atomicAdd(&flags[2], 1)] = r;
                else
                    longList[atomicAdd(&flags[3], 1)] = r;
            }
            continue;
        }
        uint64_t v = lane < len ? keys[s + lane] : ~0ull;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                const uint64_t o = __shfl_xor_sync(0xffffffffu, v, j);
                const bool up = ((lane & k) == 0);
                const bool lower = ((lane & j) == 0);
                const bool takeMin = (lower == up);
                v = takeMin ? (o < v ? o : v) : (o > v ? o : v);
            }
        }
        if (lane < len) keys[s + lane] = v;
    }
}

constexpr int kMedCap = 4096;
constexpr int kSortThreads = 1024;

__device__ __forceinline__ void bitonic_shared(uint64_t* a, int P) {
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const uint64_t x = a[i], y = a[l];
                    const bool up = ((i & k) == 0);
                    if ((x > y) == up) {
                        a[i] = y;
                        a[l] = x;
                    }
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(kSortThreads) row_sort_medium_kernel(const int* __restrict__ rowptr,
                                                                       uint64_t* __restrict__ keys,
                                                                       const int* __restrict__ medList) {
    __shared__ uint64_t a[kMedCap];
    const int r = medList[blockIdx.x];
    const int s = rowptr[r], len = rowptr[r + 1] - s;
    int P = 64;
    while (P < len) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) a[i] = i < len ? keys[s + i] : ~0ull;
    __syncthreads();
    bitonic_shared(a, P);
    for (int i = threadIdx.x; i < len; i += blockDim.x) keys[s + i] = a[i];
}

__global__ void __launch_bounds__(kSortThreads) row_sort_long_kernel(int len, int P, uint64_t* __restrict__ seg,
                                                                     uint64_t* __restrict__ scratch) {
    for (int i = threadIdx.x; i < P; i += blockDim.x) scratch[i] = i < len ? seg[i] : ~0ull;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const uint64_t x = scratch[i], y = scratch[l];
                    const bool up = ((i & k) == 0);
                    if ((x > y) == up) {
                        scratch[i] = y;
                        scratch[l] = x;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < len; i += blockDim.x) seg[i] = scratch[i];
}

__global__ void keys_unpack_kernel(int64_t nnz, const uint64_t* __restrict__ keys, int* __restrict__ colOut,
                                   uint32_t* __restrict__ perm) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t v = keys[j];
        colOut[j] = (int)(v >> 32);
        perm[j] = (uint32_t)(v & 0xffffffffull);
    }
}

__global__ void gather_kernel(int64_t nnz, const uint32_t* __restrict__ perm, const double* __restrict__ src,
                              double* __restrict__ dst) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x)
        dst[j] = src[perm[j]];
}

__global__ void f64_to_f32_kernel(int64_t count, const double* __restrict__ src, float* __restrict__ dst) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x)
        dst[j] = (float)src[j];
}

static int grid_for(int64_t work, int threads) {
    int64_t g = (work + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > device_sm_count() * 32) g = device_sm_count() * 32;
    return (int)g;
}

// Order-independent 64-bit fingerprint of a CSR structure: the sum, modulo
// 2^64, of a mixing function (the splitmix64 finaliser) over (position,
// column) and (position, row pointer) pairs.  Two structures that differ in any
// entry get different sums except with probability about 2^-64.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__global__ void struct_hash_kernel(int n, int64_t nnz, const int* __restrict__ rowptr, const int* __restrict__ col,
                                   unsigned long long* out) {
    unsigned long long h = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t i = t; i < nnz; i += stride) h += mix64(((unsigned long long)i << 32) ^ (unsigned)col[i]);
    for (int64_t i = t; i <= n; i += stride)
        h += mix64((((unsigned long long)i << 32) ^ (unsigned)rowptr[i]) + 0x9e3779b97f4a7c15ull);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, h);
}

cudaError_t struct_hash(cudaStream_t st, int n, int64_t nnz, const int* rowptr, const int* col,
                        unsigned long long* scratch, uint64_t* hash) {
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    struct_hash_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(n, nnz, rowptr, col, scratch);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    unsigned long long h = 0;
    if ((e = cudaMemcpyAsync(&h, scratch, sizeof(h), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    *hash = h;
    return cudaSuccess;
}

cudaError_t gather_values(cudaStream_t st, int64_t nnz, const uint32_t* perm, const double* src, double* dst) {
    if (nnz <= 0) return cudaSuccess;
    gather_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, perm, src, dst);
    return cudaGetLastError();
}

cudaError_t convert_f64_to_f32(cudaStream_t st, int64_t count, const double* src, float* dst) {
    if (count <= 0) return cudaSuccess;
    f64_to_f32_kernel<<<grid_for(count, 256), 256, 0, st>>>(count, src, dst);
    return cudaGetLastError();
}

#define XJ_CHECK(x)                         \
    do {                                    \
        cudaError_t e_ = (x);               \
        if (e_ != cudaSuccess) return e_;   \
    } while (0)

cudaError_t coo_to_csr(cudaStream_t st, int n, int64_t nnz, const uint32_t* row, const uint32_t* col, int base,
                       int* rowptr, int* colOut, uint32_t* perm, ConvertScratch& s, int* hostErr) {
    *hostErr = 0;
    int* flags = s.flags;
    XJ_CHECK(cudaMemsetAsync(flags, 0, 4 * sizeof(int), st));
    XJ_CHECK(cudaMemsetAsync(s.counts, 0, sizeof(int) * ((size_t)n + 1), st));
    coo_count_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, row, col, (uint32_t)base, (uint32_t)n, s.counts, flags);
    XJ_CHECK(cudaGetLastError());
    XJ_CHECK(scan_exclusive(st, s.counts, rowptr, n + 1, s.blockSums));
    int hflags[4];
    XJ_CHECK(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, st));
    XJ_CHECK(cudaStreamSynchronize(st));
    if (hflags[0]) {
        *hostErr = hflags[0];
        return cudaSuccess;
    }
    if (!hflags[1]) {
        coo_identity_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, col, (uint32_t)base, colOut, perm);
        return cudaGetLastError();
    }
    XJ_CHECK(cudaMemsetAsync(s.fill, 0, sizeof(int) * (size_t)n, st));
    coo_scatter_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, row, col, (uint32_t)base, rowptr, s.fill, s.keys);
    XJ_CHECK(cudaGetLastError());
    // The fill[] array doubles as the medium-row list and counts[] as the long-row list.
    int* medList = s.fill;
    int* longList = s.counts;
    XJ_CHECK(cudaMemsetAsync(flags + 2, 0, 2 * sizeof(int), st));
    {
        int64_t threads = (int64_t)n * 32;
        row_sort_warp_kernel<<<grid_for(threads, 256), 256, 0, st>>>(n, rowptr, s.keys, medList, longList, flags);
        XJ_CHECK(cudaGetLastError());
    }
    XJ_CHECK(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, st));
    XJ_CHECK(cudaStreamSynchronize(st));
    if (hflags[2] > 0) {
        row_sort_medium_kernel<<<hflags[2], kSortThreads, 0, st>>>(rowptr, s.keys, medList);
        XJ_CHECK(cudaGetLastError());
    }
    if (hflags[3] > 0) {
        std::vector<int> longRows(hflags[3]);
        XJ_CHECK(cudaMemcpyAsync(longRows.data(), longList, sizeof(int) * hflags[3], cudaMemcpyDeviceToHost, st));
        std::vector<int> rp((size_t)n + 1);
        XJ_CHECK(cudaMemcpyAsync(rp.data(), rowptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToHost, st));
        XJ_CHECK(cudaStreamSynchronize(st));
        int maxP = 1;
        for (int r : longRows) {
            int len = rp[r + 1] - rp[r];
            int P = 1;
            while (P < len) P <<= 1;
            if (P > maxP) maxP = P;
        }
        uint64_t* scratch = nullptr;
        XJ_CHECK(cudaMallocAsync((void**)&scratch, sizeof(uint64_t) * (size_t)maxP, st));
        for (int r : longRows) {
            int len = rp[r + 1] - rp[r];
            int P = 1;
            while (P < len) P <<= 1;
            row_sort_long_kernel<<<1, kSortThreads, 0, st>>>(len, P, s.keys + rp[r], scratch);
        }
        XJ_CHECK(cudaGetLastError());
        XJ_CHECK(cudaFreeAsync(scratch, st));
    }
    keys_unpack_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, s.keys, colOut, perm);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Symmetric half-CSC expansion
// ---------------------------------------------------------------------------
__global__ void csc_flags_kernel(int n, int64_t nnzHalf, const int64_t* __restrict__ rowIdx,
                                 const int64_t* __restrict__ colPtr, int64_t base, int* __restrict__ cnt,
                                 int* flags) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int64_t s = colPtr[j] - base, e = colPtr[j + 1] - base;
        if (s < 0 || e < s || e > nnzHalf) {
            atomicOr(&flags[0], (int)kStatusIndexError);
            continue;
        }
        for (int64_t k = s; k < e; ++k) {
            const int64_t i = rowIdx[k] - base;
            if (i < 0 || i >= n) {
                atomicOr(&flags[0], (int)kStatusIndexError);
                cnt[k] = 0;
                continue;
            }
            cnt[k] = (i != j) ? 2 : 1;
        }
    }
}

__global__ void csc_emit_kernel(int n, const int64_t* __restrict__ rowIdx, const int64_t* __restrict__ colPtr,
                                int64_t base, const double* __restrict__ data, const int* __restrict__ pos,
                                uint32_t* __restrict__ rowOut, uint32_t* __restrict__ colOut,
                                double* __restrict__ valOut) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int64_t s = colPtr[j] - base, e = colPtr[j + 1] - base;
        for (int64_t k = s; k < e; ++k) {
            const uint32_t i = (uint32_t)(rowIdx[k] - base);
            const int p = pos[k];
            if (rowOut) {
                rowOut[p] = i;
                colOut[p] = (uint32_t)j;
            }
            if (valOut) valOut[p] = data[k];
            if (i != (uint32_t)j) {
                if (rowOut) {
                    rowOut[p + 1] = (uint32_t)j;
                    colOut[p + 1] = i;
                }
                if (valOut) valOut[p + 1] = data[k];
            }
        }
    }
}

cudaError_t cscsym_expand(cudaStream_t st, int n, int64_t nnzHalf, int64_t nnzFull, const int64_t* rowIdx,
                          const int64_t* colPtr, const double* data, int base, uint32_t* rowOut, uint32_t* colOut,
                          double* valOut, int64_t* /*posScratch*/, int* flagScratch, int* blockSums, int* hostErr) {
    // flagScratch holds nnzHalf + 1 ints of counts (scanned in place into
    // positions) followed by 4 ints of flags.
    *hostErr = 0;
    int* cnt = flagScratch;
    int* flags = flagScratch + nnzHalf + 1;
    XJ_CHECK(cudaMemsetAsync(flagScratch, 0, sizeof(int) * ((size_t)nnzHalf + 5), st));
    csc_flags_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, nnzHalf, rowIdx, colPtr, base, cnt, flags);
    XJ_CHECK(cudaGetLastError());
    XJ_CHECK(scan_exclusive(st, cnt, cnt, (int)nnzHalf + 1, blockSums));
    int h[5];
    XJ_CHECK(cudaMemcpyAsync(&h[0], cnt + nnzHalf, sizeof(int), cudaMemcpyDeviceToHost, st));
    XJ_CHECK(cudaMemcpyAsync(&h[1], flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
    XJ_CHECK(cudaStreamSynchronize(st));
    if (h[1]) {
        *hostErr = h[1];
        return cudaSuccess;
    }
    if ((int64_t)h[0] != nnzFull) {
        *hostErr = (int)kStatusCountError;
        return cudaSuccess;
    }
    csc_emit_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, rowIdx, colPtr, base, data, cnt, rowOut, colOut, valOut);
    return cudaGetLastError();
}

}  // namespace xjpcg
