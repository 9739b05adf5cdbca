// signature_kernels.cu -- loads the reference's partitioned ("signature")
// matrix buffers onto the GPU and turns them into the library's CSR.
//
// The reference's SpmvHost (L2/sparse/include/sw/fp64/spmvHost.hpp:26-103)
// feeds an FPGA SpMV with 16 channel buffers nnzVal_c, a partition table
// parParam and a row-block table rbParam, as written by the host partitioner
// (signature.hpp:361-426 gen_nnzStore, matrix_params.hpp:329-688).  A
// channel buffer is a 32-byte header followed, for every row block and every
// partition of it, by that channel's chunk: groups of 4 fp64 values (32 bytes),
// with a 16 x uint16 row-index block before every 128th group (one row index
// per 32 entries) and a 16 x uint16 column-block block before every 16th group
// (one 4-column block index per 4 entries).  Padding entries hold value 0.
//
// The host parses the two small tables and lists the chunks (channel, byte
// offset, groups, row base, column base); this kernel decodes every group in
// parallel into (row, col, value) in stored order; the entries with a
// non-zero value are compacted (padding dropped) and handed to the COO->CSR
// conversion.  A stored entry whose value is exactly 0 is dropped as well,
// which leaves every product A x unchanged.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

__global__ void sig_decode_kernel(int nchunks, const SigChunk* __restrict__ chunks, const unsigned char* __restrict__ buf,
                                  int64_t groups, uint32_t* __restrict__ row, uint32_t* __restrict__ col,
                                  double* __restrict__ val, int* __restrict__ keep) {
    for (int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; gid < groups;
         gid += (int64_t)gridDim.x * blockDim.x) {
        // chunk with groupStart <= gid < next groupStart
        int lo = 0, hi = nchunks - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (chunks[mid].groupStart <= gid)
                lo = mid;
            else
                hi = mid - 1;
        }
        const SigChunk ck = chunks[lo];
        const int64_t g = gid - ck.groupStart;
        const int64_t g0 = g & ~(int64_t)127, g1 = g & ~(int64_t)15;
        const int64_t rowOff = ck.byteStart + 32 * (g0 + g0 / 128 + g0 / 16);
        const int64_t colOff = ck.byteStart + 32 * (g1 + g1 / 128 + 1 + g1 / 16);
        const int64_t valOff = ck.byteStart + 32 * (g + g / 128 + g / 16 + 2);
        const uint16_t ri = reinterpret_cast<const uint16_t*>(buf + rowOff)[(g % 128) / 8];
        const uint16_t ci = reinterpret_cast<const uint16_t*>(buf + colOff)[g % 16];
        const double* v = reinterpret_cast<const double*>(buf + valOff);
        const uint32_t r = (uint32_t)ck.rowBase + ri;
        const uint32_t c0 = ((uint32_t)ck.colBase + ci) * 4u;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t o = 4 * gid + j;
            const double vj = v[j];
            row[o] = r;
            col[o] = c0 + (uint32_t)j;
            val[o] = vj;
            keep[o] = vj != 0.0 ? 1 : 0;
        }
    }
}

__global__ void sig_compact_kernel(int64_t count, const int* __restrict__ pos, const int* __restrict__ keep,
                                   const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
                                   const double* __restrict__ val, uint32_t* __restrict__ rowOut,
                                   uint32_t* __restrict__ colOut, double* __restrict__ valOut) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        if (!keep[k]) continue;
        const int p = pos[k];
        rowOut[p] = row[k];
        colOut[p] = col[k];
        valOut[p] = val[k];
    }
}

// ---------------------------------------------------------------------------
// SpMV in the reference FPGA's summation order.
//
// The reference's SpMV (L1/sparse/include/hw/xf_sparse/fp64) adds in a fixed
// order that its C source spells out:
//   multAddX  (spmv.hpp:136-157)  each group of 4 stored entries: the four
//             products v_j * x_j, each rounded, summed left to right from 0;
//   regAcc    (spmv.hpp:159-185)  each run of 8 such group sums (the 32
//             entries under one row index) summed left to right from 0;
//   rowMemAcc (spmv.hpp:452-476)  each row's run sums added to its row store,
//             which starts at 0, in the order the channel stream holds them
//             (its row block's partitions in order);
//   accY      (dataMovers.hpp:339-375)  the 16 channels' row values summed
//             from 0 in channel order; a row lives in one channel, the other
//             fifteen give +0, so y = 0 + (the row store).
// Multiplies and adds are issued separately with round-to-nearest (no fused
// multiply-add), so the GPU result is the C semantics of that source bit for
// bit.  One thread per row walks its runs (32 stored entries each) in stream
// order; the run lists are built once when the matrix is loaded.
__global__ void sig_run_rows_kernel(int64_t runs, const uint32_t* __restrict__ row, uint32_t* __restrict__ runRow,
                                    uint32_t* __restrict__ runIdx) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < runs; k += (int64_t)gridDim.x * blockDim.x) {
        runRow[k] = row[32 * k];
        runIdx[k] = (uint32_t)k;
    }
}

__global__ void sig_ordered_spmv_kernel(int rows, const int* __restrict__ runPtr, const int* __restrict__ runIdx,
                                        const double* __restrict__ val, const uint32_t* __restrict__ col,
                                        const double* __restrict__ x, double* __restrict__ y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x) {
        double store = 0.0;
        for (int k = runPtr[i]; k < runPtr[i + 1]; ++k) {
            const int64_t e0 = 32 * (int64_t)runIdx[k];
            double run = 0.0;
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                double grp = 0.0;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int64_t e = e0 + 4 * b + j;
                    grp = __dadd_rn(grp, __dmul_rn(val[e], x[col[e]]));
                }
                run = __dadd_rn(run, grp);
            }
            store = __dadd_rn(store, run);
        }
        y[i] = __dadd_rn(0.0, store);
    }
}

cudaError_t sig_run_rows(cudaStream_t st, int64_t runs, const uint32_t* row, uint32_t* runRow, uint32_t* runIdx) {
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((runs + 255) / 256, device_sm_count() * 16));
    sig_run_rows_kernel<<<grid, 256, 0, st>>>(runs, row, runRow, runIdx);
    return cudaGetLastError();
}

cudaError_t sig_ordered_spmv(cudaStream_t st, int rows, const int* runPtr, const int* runIdx, const double* val,
                             const uint32_t* col, const double* x, double* y) {
    const int grid = std::max(1, std::min((rows + 127) / 128, device_sm_count() * 16));
    sig_ordered_spmv_kernel<<<grid, 128, 0, st>>>(rows, runPtr, runIdx, val, col, x, y);
    return cudaGetLastError();
}

cudaError_t sig_decode(cudaStream_t st, int nchunks, const SigChunk* chunks, const unsigned char* buf, int64_t groups,
                       uint32_t* row, uint32_t* col, double* val, int* keep) {
    if (groups <= 0) return cudaSuccess;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((groups + 255) / 256, device_sm_count() * 32));
    sig_decode_kernel<<<grid, 256, 0, st>>>(nchunks, chunks, buf, groups, row, col, val, keep);
    return cudaGetLastError();
}

cudaError_t sig_compact(cudaStream_t st, int64_t count, const int* pos, const int* keep, const uint32_t* row,
                        const uint32_t* col, const double* val, uint32_t* rowOut, uint32_t* colOut, double* valOut) {
    if (count <= 0) return cudaSuccess;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, device_sm_count() * 32));
    sig_compact_kernel<<<grid, 256, 0, st>>>(count, pos, keep, row, col, val, rowOut, colOut, valOut);
    return cudaGetLastError();
}

// transY framing (dSpmv/hw/include/impl/transY.hpp:35-65): one 64-byte header
// word {startAddr, rows, 0...} followed by the rows' values packed eight per
// 64-byte word, the last word zero-filled.
__global__ void transy_frame_kernel(uint32_t startAddr, uint32_t rows, const double* __restrict__ y,
                                    unsigned char* __restrict__ frame) {
    const uint32_t words = rows == 0 ? 1u : (rows + 7) / 8;  // the HLS loop always emits a final word
    const uint32_t total = 16 + words * 16;                    // in uint32 units
    uint32_t* f = reinterpret_cast<uint32_t*>(frame);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        if (k < 16) {
            f[k] = k == 0 ? startAddr : (k == 1 ? rows : 0u);
        } else {
            const uint32_t e = (k - 16) / 2;  // value index
            uint32_t w = 0;
            if (e < rows) {
                const uint64_t bits = (uint64_t)__double_as_longlong(y[e]);
                w = (k & 1) ? (uint32_t)(bits >> 32) : (uint32_t)bits;
            }
            f[k] = w;
        }
    }
}

cudaError_t transy_frame(cudaStream_t st, uint32_t startAddr, uint32_t rows, const double* y, unsigned char* frame) {
    const uint32_t total = 16 + (rows == 0 ? 1u : (rows + 7) / 8) * 16;
    const int grid = (int)std::max<uint32_t>(1, std::min<uint32_t>((total + 255) / 256, device_sm_count() * 16));
    transy_frame_kernel<<<grid, 256, 0, st>>>(startAddr, rows, y, frame);
    return cudaGetLastError();
}

}  // namespace xjpcg
