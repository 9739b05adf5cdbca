// signature_export.cu -- writes the stored matrix in the reference's
// partitioned ("signature") format, byte for byte, on the device.
//
// The reference partitions a matrix on the host before every FPGA solve
// (Signature::gen_sig, L2/sparse/include/sw/fp64/signature.hpp:471-532, with
// parEntries 4, accLatency 8, 16 HBM channels, 4096 x 4096 partitions) and
// can store the result as rbParam.dat / parParam.dat / nnzVal_<c>.dat /
// info.dat (gen_signature.cpp:58-81).  This file produces the same bytes from
// the library's CSR, whose entry order (rows ascending, columns ascending,
// duplicates in input order) is the reference's stored order.
//
// Structure, in the reference's terms and how it is computed here:
//   row blocks     a block starts at the first row not yet covered and takes
//                  the rows below start + 4096 (gen_rbs :95-138).  Host scan
//                  of the row pointers (O(n), once per matrix).
//   partitions     per block, a partition starts at the first uncovered
//                  4-column group and takes the next 1024 groups
//                  (genPars4Rb :140-173).  A bitmap of the groups present in
//                  each block, then one warp per block jumps from start to
//                  start with ballots.
//   padded rows    per (partition, row) segment the entries are placed into
//                  aligned 4-column groups, a slot without its column being
//                  a padding entry; the segment is padded to a multiple of 32
//                  slots (pad_par :186-231).  A CSR row's entries are sorted
//                  by column, so a segment is a contiguous CSR range: one warp
//                  per partition finds them with two binary searches per row
//                  of its block, in row order, which is the padded order.
//                  One thread per segment then runs the placement twice: once
//                  to size it, once (after a scan) to write the slots.
//   channels       each padded partition is cut into 16 chunks of about a
//                  sixteenth, every cut moved to the end of its row
//                  (gen_chPars :250-316), one thread per partition.
//   buffers        rbParam / parParam records (matrix_params.hpp:329-576),
//                  then the channel streams (gen_nnzStore :361-426): per chunk
//                  a 256-bit word of 16 row indices every 512 slots, one of 16
//                  column-group indices every 64 slots, and the values 4 per
//                  word.  One thread per 4-slot group writes its words; index
//                  words that run past the chunk repeat the previous word's
//                  entries, as the reference's reused index arrays do.
// A values-only update (update_sig :427-465) reruns only the last kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "pcg_handle.hpp"
#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

namespace {
constexpr int kPar = 4;                     // parEntries: columns per group
constexpr int kRowSlots = 32;               // parEntries * accLatency: row padding unit
constexpr int kCh = 16;                     // HBM channels
constexpr int kMaxRows = 4096;              // rows of a row block
constexpr int kPartGroups = 4096 / kPar;    // column groups of a partition
constexpr int kRowWordSlots = 16 * kRowSlots;  // slots covered by one row-index word
constexpr int kColWordSlots = 16 * kPar;       // slots covered by one column-index word
constexpr uint32_t kPadSrc = 0xffffffffu;   // ZERO_VAL: a padding slot
constexpr int kRec = 256;                   // bytes per rbParam / parParam record

__device__ __forceinline__ int upper_index(const int* a, int cnt, int v) {
    // number of entries of the ascending a[0..cnt) that are <= v
    int lo = 0, hi = cnt;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] <= v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

int grid_of(int64_t work, int threads) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((work + threads - 1) / threads, device_sm_count() * 32));
}
}  // namespace

// Column extent of each row block's entries.
__global__ void sig_block_minmax_kernel(const int* __restrict__ blkEnt, const int* __restrict__ col,
                                        int* __restrict__ minCol, int* __restrict__ maxCol) {
    const int b = blockIdx.x;
    int lo = 0x7fffffff, hi = -1;
    for (int j = blkEnt[b] + threadIdx.x; j < blkEnt[b + 1]; j += blockDim.x) {
        const int c = col[j];
        lo = min(lo, c);
        hi = max(hi, c);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __shared__ int sLo[32], sHi[32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sLo[w] = lo;
        sHi[w] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            lo = min(lo, sLo[k]);
            hi = max(hi, sHi[k]);
        }
        minCol[b] = lo;
        maxCol[b] = hi;
    }
}

// Marks, per block, the 4-column groups that hold an entry (one warp per row).
__global__ void sig_mark_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col, int nb,
                                const int* __restrict__ blkRow0, const int* __restrict__ blkMinG,
                                const int64_t* __restrict__ bitOff, uint32_t* __restrict__ bitmap) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warpsPerGrid) {
        const int j0 = rowptr[r], j1 = rowptr[r + 1];
        if (j0 == j1) continue;
        const int b = upper_index(blkRow0, nb, r) - 1;
        uint32_t* bm = bitmap + bitOff[b];
        const int g0 = blkMinG[b];
        for (int j = j0 + lane; j < j1; j += 32) {
            const int g = (col[j] >> 2) - g0;
            atomicOr(&bm[g >> 5], 1u << (g & 31));
        }
    }
}

// One warp per block: partition starts (relative groups), each the first
// present group at or after the previous start + 1024.
__global__ void sig_chain_kernel(int nb, const int* __restrict__ blkMinG, const int* __restrict__ blkMaxG,
                                 const int64_t* __restrict__ bitOff, const uint32_t* __restrict__ bitmap,
                                 const int64_t* __restrict__ slotOff, int* __restrict__ starts,
                                 int* __restrict__ nPart) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    for (int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < nb; b += warpsPerGrid) {
        const int range = blkMaxG[b] - blkMinG[b] + 1;
        const int words = (range + 31) >> 5;
        const uint32_t* bm = bitmap + bitOff[b];
        int* out = starts + slotOff[b];
        int pos = 0, cnt = 0;  // group 0 (the block's minimum) is always present
        while (true) {
            if (lane == 0) out[cnt] = pos;
            ++cnt;
            const int next = pos + kPartGroups;
            if (next >= range) break;
            int found = -1;
            for (int w0 = next >> 5; w0 < words && found < 0; w0 += 32) {
                const int w = w0 + lane;
                uint32_t v = w < words ? bm[w] : 0u;
                if (w == (next >> 5)) v &= ~0u << (next & 31);
                const unsigned ball = __ballot_sync(0xffffffffu, v != 0u);
                if (ball) {
                    const int l = __ffs(ball) - 1;
                    const uint32_t vl = __shfl_sync(0xffffffffu, v, l);
                    found = ((w0 + l) << 5) + __ffs(vl) - 1;
                }
            }
            if (found < 0) break;
            pos = found;
        }
        if (lane == 0) nPart[b] = cnt;
    }
}

__global__ void sig_part_table_kernel(int nb, const int* __restrict__ nPart, const int* __restrict__ parBase,
                                      const int64_t* __restrict__ slotOff, const int* __restrict__ starts,
                                      const int* __restrict__ blkMinG, int* __restrict__ partG0,
                                      int* __restrict__ partBlock) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
        for (int k = 0; k < nPart[b]; ++k) {
            partG0[parBase[b] + k] = blkMinG[b] + starts[slotOff[b] + k];
            partBlock[parBase[b] + k] = b;
        }
}

// Segment = the entries of one row inside one partition: in the CSR the
// contiguous range of the row whose columns fall in the partition's 4096.
// One warp per partition walks its block's rows in order; pass 0 counts the
// non-empty segments, pass 1 (after a scan) writes them.
__global__ void sig_segments_kernel(int P, int pass, const int* __restrict__ partG0,
                                    const int* __restrict__ partBlock, const int* __restrict__ blkRow0,
                                    const int* __restrict__ blkM, const int* __restrict__ rowptr,
                                    const int* __restrict__ col, int* __restrict__ segCount,
                                    const int* __restrict__ segBase, int* __restrict__ segLo,
                                    int* __restrict__ segHi, int* __restrict__ segRow) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < P; p += warpsPerGrid) {
        const int b = partBlock[p];
        const int r0 = blkRow0[b], m = blkM[b];
        const int cLo = partG0[p] * kPar, cHi = cLo + kPartGroups * kPar;
        int base = pass ? segBase[p] : 0;
        for (int k0 = 0; k0 < m; k0 += 32) {
            const int r = r0 + k0 + lane;
            int lo = 0, hi = 0;
            if (k0 + lane < m) {
                // first entry with col >= cLo, first with col >= cHi
                int a = rowptr[r], e = rowptr[r + 1];
                while (a < e) {
                    const int mid = (a + e) >> 1;
                    if (col[mid] < cLo) a = mid + 1; else e = mid;
                }
                lo = a;
                e = rowptr[r + 1];
                while (a < e) {
                    const int mid = (a + e) >> 1;
                    if (col[mid] < cHi) a = mid + 1; else e = mid;
                }
                hi = a;
            }
            const unsigned ball = __ballot_sync(0xffffffffu, hi > lo);
            if (pass && hi > lo) {
                const int s = base + __popc(ball & ((1u << lane) - 1u));
                segLo[s] = lo;
                segHi[s] = hi;
                segRow[s] = r;
            }
            base += __popc(ball);
        }
        if (!pass && lane == 0) segCount[p] = base;
    }
}

// Slot placement of pad_par: a new 4-slot group starts at the first entry,
// when the entry's column group changes, or when its slot (column % 4) is not
// after the previous entry's slot (a duplicate, or a full group).
struct Placement {
    int gs = -kPar;   // first slot of the current group
    int curG = -1;    // its column group
    int nextMod = kPar;
    __device__ __forceinline__ bool place(int c) {
        const int g = c >> 2, m = c & 3;
        const bool fresh = (g != curG || m < nextMod);
        if (fresh) {
            gs += kPar;
            curG = g;
        }
        nextMod = m + 1;
        return fresh;
    }
    __device__ __forceinline__ int padded() const { return (gs & ~(kRowSlots - 1)) + kRowSlots; }
};

__global__ void sig_seg_len_kernel(int S, const int* __restrict__ segLo, const int* __restrict__ segHi,
                                   const int* __restrict__ col, int* __restrict__ segLen, int* __restrict__ segMinG,
                                   int* __restrict__ segMaxG, unsigned long long* __restrict__ total) {
    unsigned long long mine = 0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
        const int j0 = segLo[s], j1 = segHi[s];
        Placement pl;
        for (int j = j0; j < j1; ++j) pl.place(col[j]);
        const int L = pl.padded();
        segLen[s] = L;
        segMinG[s] = col[j0] >> 2;
        segMaxG[s] = pl.curG;
        mine += (unsigned long long)L;
    }
    if (mine) atomicAdd(total, mine);
}

__global__ void sig_part_range_kernel(int P, int nnzPad, const int* __restrict__ segBase,
                                      const int* __restrict__ segOff, int* __restrict__ ppad) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p <= P; p += gridDim.x * blockDim.x)
        ppad[p] = p == P ? nnzPad : segOff[segBase[p]];
}

// Second placement pass: source slot of every entry (kPadSrc in the padding
// slots), row and column group of every 4-slot group (trailing padding groups
// keep the last column group).  A group's four slots are assembled in
// registers and stored as one 16-byte word once the group is complete, so
// every slot is written once and none needs a fill beforehand (segments
// start on 32-slot boundaries, groups on 4-slot ones).
__global__ void sig_emit_kernel(int S, const int* __restrict__ segLo, const int* __restrict__ segHi,
                                const int* __restrict__ col, const int* __restrict__ segOff,
                                const int* __restrict__ segLen, const int* __restrict__ segRow,
                                uint32_t* __restrict__ slotSrc, int* __restrict__ grpRow, int* __restrict__ grpG) {
    const uint4 pad = make_uint4(kPadSrc, kPadSrc, kPadSrc, kPadSrc);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
        const int off = segOff[s], row = segRow[s];
        Placement pl;
        uint4 cur = pad;
        for (int j = segLo[s]; j < segHi[s]; ++j) {
            const int c = col[j];
            if (pl.place(c)) {
                if (pl.gs > 0) *reinterpret_cast<uint4*>(slotSrc + off + pl.gs - kPar) = cur;
                cur = pad;
                grpRow[(off + pl.gs) >> 2] = row;
                grpG[(off + pl.gs) >> 2] = pl.curG;
            }
            const uint32_t src = (uint32_t)j;
            const int m = c & 3;
            cur.x = m == 0 ? src : cur.x;
            cur.y = m == 1 ? src : cur.y;
            cur.z = m == 2 ? src : cur.z;
            cur.w = m == 3 ? src : cur.w;
        }
        if (pl.gs >= 0) *reinterpret_cast<uint4*>(slotSrc + off + pl.gs) = cur;
        for (int k = pl.gs + kPar; k < segLen[s]; k += kPar) {
            *reinterpret_cast<uint4*>(slotSrc + off + k) = pad;
            grpRow[(off + k) >> 2] = row;
            grpG[(off + k) >> 2] = pl.curG;
        }
    }
}

__device__ __forceinline__ int warp_min_i32(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_max_i32(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// One warp per partition: the 16 channel cuts, the chunks' extents, the
// partition's parParam record and the chunks' byte sizes.  Every lane places
// the cuts the same way (binary searches over the partition's segments, so
// control flow stays warp-uniform); the column-group extents of the partition
// and of each chunk are warp-strided min / max reductions over its segments;
// lane 0 writes.
__global__ void sig_chan_kernel(int P, const int* __restrict__ ppad, const int* __restrict__ segFirst,
                                const int* __restrict__ segOff, const int* __restrict__ segLen,
                                const int* __restrict__ segRow, const int* __restrict__ segMinG,
                                const int* __restrict__ segMaxG, int* __restrict__ chStart, int* __restrict__ chLen,
                                int* __restrict__ chMinG, int* __restrict__ chEndRow,
                                long long* __restrict__ chBytes, unsigned char* __restrict__ parParam) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < P; p += warpsPerGrid) {
        const int base = ppad[p], Np = ppad[p + 1] - base;
        const int s0 = segFirst[p], s1 = segFirst[p + 1];
        const int per = Np / kCh;
        uint32_t w[64];
        for (int k = 0; k < 64; ++k) w[k] = 0u;
        int pMinG = 0x7fffffff, pMaxG = -1;
        for (int s = s0 + lane; s < s1; s += 32) {
            pMinG = min(pMinG, segMinG[s]);
            pMaxG = max(pMaxG, segMaxG[s]);
        }
        pMinG = warp_min_i32(pMinG);
        pMaxG = warp_max_i32(pMaxG);
        int start = 0, sa = s0;
        uint16_t cbase[kCh], ccols[kCh];
        for (int c = 0; c < kCh; ++c) {
            int e = (c == kCh - 1 || start + per >= Np) ? Np : start + per;
            if (e > 0 && e < Np) {
                // the segment holding slot e; a cut inside a row moves to its end
                int lo = s0, hi = s1 - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (segOff[mid] - base <= e)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                if (segOff[lo] - base != e) e = segOff[lo] - base + segLen[lo];
            }
            const int len = e - start;
            // sb: the first segment at or after the cut (segment offsets ascend)
            int sb = sa, hiS = s1;
            while (sb < hiS) {
                const int mid = (sb + hiS) >> 1;
                if (segOff[mid] - base < e)
                    sb = mid + 1;
                else
                    hiS = mid;
            }
            int gMin = 0x7fffffff, gMax = -1;
            for (int s = sa + lane; s < sb; s += 32) {
                gMin = min(gMin, segMinG[s]);
                gMax = max(gMax, segMaxG[s]);
            }
            gMin = warp_min_i32(gMin);
            gMax = warp_max_i32(gMax);
            int endRow = 0;
            if (len > 0) {
                endRow = segRow[sb - 1] + 1;
            } else {
                gMin = 0;
                gMax = -1;
            }
            if (lane == 0) {
                const int idx = p * kCh + c;
                chStart[idx] = start;
                chLen[idx] = len;
                chMinG[idx] = gMin;
                chEndRow[idx] = endRow;
                const long long words = (len + kRowWordSlots - 1) / kRowWordSlots +
                                        (len + kColWordSlots - 1) / kColWordSlots + len / kPar;
                chBytes[(size_t)c * P + p] = 32ll * words;
            }
            w[c] = len > 0 ? (uint32_t)(kPar * (gMax - gMin + 1)) : 0u;  // chCols
            w[16 + c] = (uint32_t)len;                                  // chNnzs
            cbase[c] = (uint16_t)((len > 0 ? gMin : 0) - pMinG);         // chBaseAddr
            ccols[c] = (uint16_t)(len > 0 ? gMax - gMin + 1 : 0);        // chCols / parEntries
            start = e;
            sa = sb;
        }
        if (lane != 0) continue;
        w[32] = (uint32_t)pMinG;                                 // base column group
        w[33] = (uint32_t)(pMaxG - pMinG + 1);                   // column blocks
        w[34] = (uint32_t)(segRow[s1 - 1] - segRow[s0] + 1);     // rows
        w[35] = (uint32_t)Np;                                    // padded entries
        for (int c = 0; c < kCh; c += 2) {
            w[40 + c / 2] = (uint32_t)cbase[c] | ((uint32_t)cbase[c + 1] << 16);
            w[48 + c / 2] = (uint32_t)ccols[c] | ((uint32_t)ccols[c + 1] << 16);
        }
        uint4* dst = reinterpret_cast<uint4*>(parParam + 32 + (size_t)kRec * p);
        for (int k = 0; k < 16; ++k) dst[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
    }
}

__global__ void sig_rb_kernel(int nb, const int* __restrict__ blkRow0, const int* __restrict__ blkMinCol,
                              const int* __restrict__ blkNcol, const int* __restrict__ blkM,
                              const int* __restrict__ nPart, const int* __restrict__ parBase,
                              const int* __restrict__ chLen, const int* __restrict__ chEndRow,
                              unsigned char* __restrict__ rbParam) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        uint32_t w[64];
        for (int k = 0; k < 64; ++k) w[k] = 0u;
        const int r0 = blkRow0[b];
        uint32_t tot = 0;
        uint16_t rows[kCh];
        for (int c = 0; c < kCh; ++c) {
            int end = r0;
            uint32_t cnt = 0;
            for (int p = parBase[b]; p < parBase[b] + nPart[b]; ++p) {
                const int idx = p * kCh + c;
                if (chLen[idx] > 0 && end < chEndRow[idx]) end = chEndRow[idx];
                cnt += (uint32_t)chLen[idx];
            }
            rows[c] = (uint16_t)(end - r0);
            w[32 + c] = cnt;  // words 4-5: padded entries per channel
            tot += cnt;
        }
        w[0] = (uint32_t)r0;
        w[1] = (uint32_t)blkMinCol[b];
        w[2] = (uint32_t)blkNcol[b];
        w[3] = (uint32_t)nPart[b];
        w[8] = (uint32_t)blkM[b];
        w[9] = tot;
        // word 2: per-channel first-row offsets, always 0 (update_rbParams)
        for (int c = 0; c < kCh; c += 2) w[24 + c / 2] = (uint32_t)rows[c] | ((uint32_t)rows[c + 1] << 16);
        uint4* dst = reinterpret_cast<uint4*>(rbParam + 32 + (size_t)kRec * b);
        for (int k = 0; k < 16; ++k) dst[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
    }
}

// One CTA per channel: exclusive scan of the chunks' byte sizes over the
// partitions, and the channel header counts.
__global__ void __launch_bounds__(1024) sig_chan_scan_kernel(int P, const long long* __restrict__ chBytes,
                                                             const int* __restrict__ chLen,
                                                             long long* __restrict__ chOff,
                                                             long long* __restrict__ chanBytes,
                                                             uint32_t* __restrict__ chanHdr) {
    const int c = blockIdx.x;
    __shared__ long long sScan[1024];
    __shared__ unsigned long long sCnt[3];
    if (threadIdx.x < 3) sCnt[threadIdx.x] = 0ull;
    long long carry = 0;
    unsigned long long rowW = 0, colW = 0, valW = 0;
    for (int t0 = 0; t0 < P; t0 += 1024) {
        const int p = t0 + threadIdx.x;
        const long long v = p < P ? chBytes[(size_t)c * P + p] : 0ll;
        if (p < P) {
            const int len = chLen[p * kCh + c];
            rowW += (len + kRowWordSlots - 1) / kRowWordSlots;
            colW += (len + kColWordSlots - 1) / kColWordSlots;
            valW += len / kPar;
        }
        sScan[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const long long add = threadIdx.x >= (unsigned)o ? sScan[threadIdx.x - o] : 0ll;
            __syncthreads();
            sScan[threadIdx.x] += add;
            __syncthreads();
        }
        if (p < P) chOff[(size_t)c * P + p] = carry + sScan[threadIdx.x] - v;
        carry += sScan[1023];
        __syncthreads();
    }
    atomicAdd(&sCnt[0], rowW);
    atomicAdd(&sCnt[1], colW);
    atomicAdd(&sCnt[2], valW);
    __syncthreads();
    if (threadIdx.x == 0) {
        chanBytes[c] = 32ll + carry;
        chanHdr[4 * c + 0] = (uint32_t)(sCnt[0] + sCnt[1] + sCnt[2]);
        chanHdr[4 * c + 1] = (uint32_t)sCnt[0];
        chanHdr[4 * c + 2] = (uint32_t)sCnt[1];
        chanHdr[4 * c + 3] = (uint32_t)sCnt[2];
    }
}

// One warp per chunk (partition p, channel c; idx = p kCh + c), its lanes
// taking the chunk's 4-slot groups g = lane, lane + 32, ...: each group's
// value word and, at the chunk's index positions, the row-index and
// column-index words.  A warp reads its chunk's place in the channel stream
// once; no group searches for its partition or channel.
__global__ void sig_format_kernel(int P, const int* __restrict__ ppad, const int* __restrict__ chStart,
                                  const int* __restrict__ chLen, const int* __restrict__ chMinG,
                                  const int* __restrict__ partBlock, const int* __restrict__ blkRow0,
                                  const long long* __restrict__ chOff, const long long* __restrict__ chanBase,
                                  const uint32_t* __restrict__ chanHdr, const uint32_t* __restrict__ slotSrc,
                                  const int* __restrict__ grpRow, const int* __restrict__ grpG,
                                  const double* __restrict__ val, unsigned char* __restrict__ out) {
    if (blockIdx.x == 0 && threadIdx.x < kCh) {
        uint4* h = reinterpret_cast<uint4*>(out + chanBase[threadIdx.x]);
        const uint32_t* hd = chanHdr + 4 * threadIdx.x;
        h[0] = make_uint4(hd[0], hd[1], hd[2], hd[3]);
        h[1] = make_uint4(0u, 0u, 0u, 0u);
    }
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; idx < P * kCh; idx += warps) {
        const int len = chLen[idx];
        if (len <= 0) continue;
        const int p = idx / kCh, c = idx % kCh;
        const int abs0 = ppad[p] + chStart[idx];
        unsigned char* cb = out + chanBase[c] + 32 + chOff[(size_t)c * P + p];
        const int r0 = blkRow0[partBlock[p]];
        const int g0 = chMinG[idx];
        for (int i = lane * kPar; i < len; i += 32 * kPar) {
            const int slot = abs0 + i;
            const int g = i / kPar;
            double v[kPar];
#pragma unroll
            for (int k = 0; k < kPar; ++k) {
                const uint32_t src = slotSrc[slot + k];
                v[k] = src == kPadSrc ? 0.0 : val[src];
            }
            double2* vd = reinterpret_cast<double2*>(cb + 32ll * (g + g / 128 + g / 16 + 2));
            vd[0] = make_double2(v[0], v[1]);
            vd[1] = make_double2(v[2], v[3]);
            if (g % 128 == 0) {
                uint32_t w[8];
                for (int k = 0; k < 16; k += 2) {
                    uint32_t h2[2];
                    for (int t = 0; t < 2; ++t) {
                        const int pos = i + (k + t) * kRowSlots;
                        int r = 0;
                        if (pos < len)
                            r = grpRow[(abs0 + pos) >> 2] - r0;
                        else if (i >= kRowWordSlots)
                            r = grpRow[(abs0 + pos - kRowWordSlots) >> 2] - r0;
                        h2[t] = (uint32_t)(uint16_t)r;
                    }
                    w[k / 2] = h2[0] | (h2[1] << 16);
                }
                uint4* d = reinterpret_cast<uint4*>(cb + 32ll * (g + g / 128 + g / 16));
                d[0] = make_uint4(w[0], w[1], w[2], w[3]);
                d[1] = make_uint4(w[4], w[5], w[6], w[7]);
            }
            if (g % 16 == 0) {
                uint32_t w[8];
                for (int k = 0; k < 16; k += 2) {
                    uint32_t h2[2];
                    for (int t = 0; t < 2; ++t) {
                        const int pos = i + (k + t) * kPar;
                        int cg = 0;
                        if (pos < len)
                            cg = grpG[(abs0 + pos) >> 2] - g0;
                        else if (i >= kColWordSlots)
                            cg = grpG[(abs0 + pos - kColWordSlots) >> 2] - g0;
                        h2[t] = (uint32_t)(uint16_t)cg;
                    }
                    w[k / 2] = h2[0] | (h2[1] << 16);
                }
                uint4* d = reinterpret_cast<uint4*>(cb + 32ll * (g + g / 128 + 1 + g / 16));
                d[0] = make_uint4(w[0], w[1], w[2], w[3]);
                d[1] = make_uint4(w[4], w[5], w[6], w[7]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------
namespace {
void sig_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw InternalError(std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace
#define SIG_CHECK(x, what) sig_check((x), what)

void SigExport::grow(DevBuf& b, size_t bytes, const char* what) {
    uint64_t gen = 0;
    if (!b.ensure(bytes, &gen)) throw AllocFailed(std::string("device allocation failed for ") + what);
}

void SigExport::build(cudaStream_t st, uint32_t n, uint64_t nnz64, const int* rowptr, const int* col) {
    valid = false;
    if (nnz64 == 0 || nnz64 > 0x7fffffffull) throw InvalidValue("signature export needs 0 < nnz < 2^31.");
    const int nnz = (int)nnz64;
    m = n;
    this->n = n;
    this->nnz = (uint32_t)nnz;

    // Row blocks from the row pointers (host).
    std::vector<int> rp((size_t)n + 1);
    SIG_CHECK(cudaMemcpyAsync(rp.data(), rowptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToHost, st), "D2H");
    SIG_CHECK(cudaStreamSynchronize(st), "sync");
    std::vector<int> row0, ent, mrows;
    {
        uint32_t r = 0;
        while (r < n && rp[r + 1] == rp[r]) ++r;
        while (r < n) {
            const uint32_t lim = std::min<uint64_t>((uint64_t)r + kMaxRows, n);
            uint32_t last = lim - 1;
            while (rp[last + 1] == rp[last]) --last;  // row r is not empty
            row0.push_back((int)r);
            ent.push_back(rp[r]);
            mrows.push_back((int)(last - r + 1));
            r = lim;
            while (r < n && rp[r + 1] == rp[r]) ++r;
        }
        ent.push_back(rp[n]);
    }
    nb = (int)row0.size();
    grow(bBlkRow0, sizeof(int) * (nb + 1), "signature blocks");
    grow(bBlkEnt, sizeof(int) * (nb + 1), "signature blocks");
    grow(bBlkM, sizeof(int) * nb, "signature blocks");
    grow(bBlkMin, sizeof(int) * nb, "signature blocks");
    grow(bBlkMax, sizeof(int) * nb, "signature blocks");
    SIG_CHECK(cudaMemcpyAsync(bBlkRow0.p, row0.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, st), "H2D");
    SIG_CHECK(cudaMemcpyAsync(bBlkEnt.p, ent.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, st), "H2D");
    SIG_CHECK(cudaMemcpyAsync(bBlkM.p, mrows.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, st), "H2D");
    sig_block_minmax_kernel<<<nb, 256, 0, st>>>(bBlkEnt.as<int>(), col, bBlkMin.as<int>(), bBlkMax.as<int>());
    SIG_CHECK(cudaGetLastError(), "block extents");
    std::vector<int> bmin(nb), bmax(nb);
    SIG_CHECK(cudaMemcpyAsync(bmin.data(), bBlkMin.p, sizeof(int) * nb, cudaMemcpyDeviceToHost, st), "D2H");
    SIG_CHECK(cudaMemcpyAsync(bmax.data(), bBlkMax.p, sizeof(int) * nb, cudaMemcpyDeviceToHost, st), "D2H");
    SIG_CHECK(cudaStreamSynchronize(st), "sync");
    std::vector<int> minG(nb), maxG(nb), ncol(nb);
    std::vector<int64_t> bitOff(nb + 1), slotOff(nb + 1);
    bitOff[0] = slotOff[0] = 0;
    for (int b = 0; b < nb; ++b) {
        minG[b] = bmin[b] >> 2;
        maxG[b] = bmax[b] >> 2;
        ncol[b] = bmax[b] - bmin[b] + 1;
        const int range = maxG[b] - minG[b] + 1;
        bitOff[b + 1] = bitOff[b] + (range + 31) / 32;
        slotOff[b + 1] = slotOff[b] + range / kPartGroups + 1;
    }
    grow(bBlkMinG, sizeof(int) * nb, "signature blocks");
    grow(bBlkMaxG, sizeof(int) * nb, "signature blocks");
    grow(bBlkNcol, sizeof(int) * nb, "signature blocks");
    grow(bBitOff, sizeof(int64_t) * (nb + 1), "signature blocks");
    grow(bSlotOff, sizeof(int64_t) * (nb + 1), "signature blocks");
    grow(bBitmap, sizeof(uint32_t) * (size_t)std::max<int64_t>(bitOff[nb], 1), "signature group bitmap");
    grow(bStarts, sizeof(int) * (size_t)slotOff[nb], "signature partition starts");
    grow(bNPart, sizeof(int) * nb, "signature partition counts");
    grow(bParBase, sizeof(int) * (nb + 1), "signature partition counts");
    SIG_CHECK(cudaMemcpyAsync(bBlkMinG.p, minG.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, st), "H2D");
    SIG_CHECK(cudaMemcpyAsync(bBlkMaxG.p, maxG.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, st), "H2D");
    SIG_CHECK(cudaMemcpyAsync(bBlkNcol.p, ncol.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, st), "H2D");
    SIG_CHECK(cudaMemcpyAsync(bBitOff.p, bitOff.data(), sizeof(int64_t) * (nb + 1), cudaMemcpyHostToDevice, st), "H2D");
    SIG_CHECK(cudaMemcpyAsync(bSlotOff.p, slotOff.data(), sizeof(int64_t) * (nb + 1), cudaMemcpyHostToDevice, st),
              "H2D");
    SIG_CHECK(cudaMemsetAsync(bBitmap.p, 0, sizeof(uint32_t) * (size_t)std::max<int64_t>(bitOff[nb], 1), st),
              "memset");

    // Present groups, partitions.
    sig_mark_kernel<<<grid_of((int64_t)n * 32, 256), 256, 0, st>>>((int)n, rowptr, col, nb, bBlkRow0.as<int>(),
                                                                    bBlkMinG.as<int>(), bBitOff.as<int64_t>(),
                                                                    bBitmap.as<uint32_t>());
    sig_chain_kernel<<<grid_of((int64_t)nb * 32, 256), 256, 0, st>>>(nb, bBlkMinG.as<int>(), bBlkMaxG.as<int>(),
                                                                      bBitOff.as<int64_t>(), bBitmap.as<uint32_t>(),
                                                                      bSlotOff.as<int64_t>(), bStarts.as<int>(),
                                                                      bNPart.as<int>());
    SIG_CHECK(cudaGetLastError(), "partition starts");
    std::vector<int> np(nb), pb(nb + 1);
    SIG_CHECK(cudaMemcpyAsync(np.data(), bNPart.p, sizeof(int) * nb, cudaMemcpyDeviceToHost, st), "D2H");
    SIG_CHECK(cudaStreamSynchronize(st), "sync");
    pb[0] = 0;
    for (int b = 0; b < nb; ++b) pb[b + 1] = pb[b] + np[b];
    P = pb[nb];
    SIG_CHECK(cudaMemcpyAsync(bParBase.p, pb.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, st), "H2D");
    grow(bPartG0, sizeof(int) * P, "signature partitions");
    grow(bPartBlock, sizeof(int) * P, "signature partitions");
    sig_part_table_kernel<<<grid_of(nb, 128), 128, 0, st>>>(nb, bNPart.as<int>(), bParBase.as<int>(),
                                                            bSlotOff.as<int64_t>(), bStarts.as<int>(),
                                                            bBlkMinG.as<int>(), bPartG0.as<int>(),
                                                            bPartBlock.as<int>());

    // Segments, in partition order and row order within a partition.
    grow(bSegCount, sizeof(int) * ((size_t)P + 1), "signature segments");
    grow(bSegBase, sizeof(int) * ((size_t)P + 1), "signature segments");
    grow(bBlockSums, sizeof(int) * ((size_t)scan_block_count(std::max(P + 1, nnz + 1)) + 16), "scan scratch");
    const int segGrid = grid_of((int64_t)P * 32, 256);
    sig_segments_kernel<<<segGrid, 256, 0, st>>>(P, 0, bPartG0.as<int>(), bPartBlock.as<int>(), bBlkRow0.as<int>(),
                                                 bBlkM.as<int>(), rowptr, col, bSegCount.as<int>(), nullptr, nullptr,
                                                 nullptr, nullptr);
    SIG_CHECK(cudaMemsetAsync(bSegCount.as<int>() + P, 0, sizeof(int), st), "memset");
    SIG_CHECK(scan_exclusive(st, bSegCount.as<int>(), bSegBase.as<int>(), P + 1, bBlockSums.as<int>()), "segment scan");
    SIG_CHECK(cudaMemcpyAsync(&S, bSegBase.as<int>() + P, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H");
    SIG_CHECK(cudaStreamSynchronize(st), "sync");
    for (DevBuf* b : {&bSegLo, &bSegHi, &bSegRow, &bSegLen, &bSegMinG, &bSegMaxG, &bSegOff})
        grow(*b, sizeof(int) * ((size_t)S + 1), "signature segments");
    sig_segments_kernel<<<segGrid, 256, 0, st>>>(P, 1, bPartG0.as<int>(), bPartBlock.as<int>(), bBlkRow0.as<int>(),
                                                 bBlkM.as<int>(), rowptr, col, nullptr, bSegBase.as<int>(),
                                                 bSegLo.as<int>(), bSegHi.as<int>(), bSegRow.as<int>());
    grow(bTotal, sizeof(unsigned long long), "signature total");
    SIG_CHECK(cudaMemsetAsync(bTotal.p, 0, sizeof(unsigned long long), st), "memset");
    sig_seg_len_kernel<<<grid_of(S, 256), 256, 0, st>>>(S, bSegLo.as<int>(), bSegHi.as<int>(), col,
                                                         bSegLen.as<int>(), bSegMinG.as<int>(), bSegMaxG.as<int>(),
                                                         bTotal.as<unsigned long long>());
    SIG_CHECK(cudaGetLastError(), "segment lengths");
    unsigned long long total = 0;
    SIG_CHECK(cudaMemcpyAsync(&total, bTotal.p, sizeof(total), cudaMemcpyDeviceToHost, st), "D2H");
    SIG_CHECK(cudaStreamSynchronize(st), "sync");
    if (total > 0x7ffffff0ull) throw InvalidValue("the partitioned matrix would exceed 2^31 stored entries.");
    nnzPad = (uint32_t)total;
    SIG_CHECK(scan_exclusive(st, bSegLen.as<int>(), bSegOff.as<int>(), S, bBlockSums.as<int>()), "segment offsets");
    grow(bPpad, sizeof(int) * ((size_t)P + 1), "signature partitions");
    sig_part_range_kernel<<<grid_of(P + 1, 256), 256, 0, st>>>(P, (int)nnzPad, bSegBase.as<int>(), bSegOff.as<int>(),
                                                                bPpad.as<int>());
    // Slots and groups.
    const size_t groups = nnzPad / kPar;
    grow(bSlotSrc, sizeof(uint32_t) * (size_t)nnzPad, "signature slots");
    grow(bGrpRow, sizeof(int) * groups, "signature groups");
    grow(bGrpG, sizeof(int) * groups, "signature groups");
    // sig_emit_kernel writes every slot, padding included
    sig_emit_kernel<<<grid_of(S, 256), 256, 0, st>>>(S, bSegLo.as<int>(), bSegHi.as<int>(), col, bSegOff.as<int>(),
                                                      bSegLen.as<int>(), bSegRow.as<int>(), bSlotSrc.as<uint32_t>(),
                                                      bGrpRow.as<int>(), bGrpG.as<int>());
    SIG_CHECK(cudaGetLastError(), "segment slots");

    // Channels, parameter records, channel byte offsets.
    for (DevBuf* b : {&bChStart, &bChLen, &bChMinG, &bChEndRow})
        grow(*b, sizeof(int) * (size_t)P * kCh, "signature chunks");
    grow(bChBytes, sizeof(long long) * (size_t)P * kCh, "signature chunks");
    grow(bChOff, sizeof(long long) * (size_t)P * kCh, "signature chunks");
    rbBytes = 32 + (uint64_t)kRec * nb;
    parBytes = 32 + (uint64_t)kRec * P;
    grow(bRb, rbBytes, "rbParam");
    grow(bPar, parBytes, "parParam");
    {
        uint32_t hdr[8] = {n, (uint32_t)nb, 0, 0, 0, 0, 0, 0};
        SIG_CHECK(cudaMemcpyAsync(bRb.p, hdr, sizeof(hdr), cudaMemcpyHostToDevice, st), "H2D");
        uint32_t phdr[8] = {(uint32_t)P, 0, 0, 0, 0, 0, 0, 0};
        SIG_CHECK(cudaMemcpyAsync(bPar.p, phdr, sizeof(phdr), cudaMemcpyHostToDevice, st), "H2D");
    }
    sig_chan_kernel<<<grid_of((int64_t)P * 32, 256), 256, 0, st>>>(P, bPpad.as<int>(), bSegBase.as<int>(), bSegOff.as<int>(),
                                                    bSegLen.as<int>(), bSegRow.as<int>(), bSegMinG.as<int>(),
                                                    bSegMaxG.as<int>(), bChStart.as<int>(), bChLen.as<int>(),
                                                    bChMinG.as<int>(), bChEndRow.as<int>(),
                                                    bChBytes.as<long long>(), bPar.as<unsigned char>());
    sig_rb_kernel<<<grid_of(nb, 64), 64, 0, st>>>(nb, bBlkRow0.as<int>(), bBlkMin.as<int>(), bBlkNcol.as<int>(),
                                                   bBlkM.as<int>(), bNPart.as<int>(), bParBase.as<int>(),
                                                   bChLen.as<int>(), bChEndRow.as<int>(), bRb.as<unsigned char>());
    grow(bChanBytes, sizeof(long long) * kCh, "signature channels");
    grow(bChanBase, sizeof(long long) * kCh, "signature channels");
    grow(bChanHdr, sizeof(uint32_t) * 4 * kCh, "signature channels");
    sig_chan_scan_kernel<<<kCh, 1024, 0, st>>>(P, bChBytes.as<long long>(), bChLen.as<int>(), bChOff.as<long long>(),
                                              bChanBytes.as<long long>(), bChanHdr.as<uint32_t>());
    SIG_CHECK(cudaGetLastError(), "channel layout");
    long long cb[kCh];
    SIG_CHECK(cudaMemcpyAsync(cb, bChanBytes.p, sizeof(cb), cudaMemcpyDeviceToHost, st), "D2H");
    SIG_CHECK(cudaStreamSynchronize(st), "sync");
    long long base[kCh];
    long long acc = 0;
    for (int c = 0; c < kCh; ++c) {
        chanBytes[c] = (uint64_t)cb[c];
        base[c] = acc;
        chanBase[c] = (uint64_t)acc;
        acc += (cb[c] + 255) / 256 * 256;
    }
    SIG_CHECK(cudaMemcpyAsync(bChanBase.p, base, sizeof(base), cudaMemcpyHostToDevice, st), "H2D");
    grow(bOut, (size_t)std::max<long long>(acc, 256), "signature channel buffers");
    valid = true;
}

void SigExport::format(cudaStream_t st, const double* val) {
    sig_format_kernel<<<grid_of((int64_t)P * kCh * 32, 256), 256, 0, st>>>(
        P, bPpad.as<int>(), bChStart.as<int>(), bChLen.as<int>(), bChMinG.as<int>(), bPartBlock.as<int>(),
        bBlkRow0.as<int>(), bChOff.as<long long>(), bChanBase.as<long long>(), bChanHdr.as<uint32_t>(),
        bSlotSrc.as<uint32_t>(), bGrpRow.as<int>(), bGrpG.as<int>(), val, bOut.as<unsigned char>());
    SIG_CHECK(cudaGetLastError(), "signature values");
    SIG_CHECK(cudaStreamSynchronize(st), "sync");
}

void SigExport::copyOut(cudaStream_t st, void* rb, void* par, void* const* nnzVal) const {
    if (!valid) throw InvalidValue("no signature has been exported.");
    if (rb) SIG_CHECK(cudaMemcpyAsync(rb, bRb.p, rbBytes, cudaMemcpyDeviceToHost, st), "D2H rbParam");
    if (par) SIG_CHECK(cudaMemcpyAsync(par, bPar.p, parBytes, cudaMemcpyDeviceToHost, st), "D2H parParam");
    if (nnzVal)
        for (int c = 0; c < kCh; ++c)
            if (nnzVal[c])
                SIG_CHECK(cudaMemcpyAsync(nnzVal[c], bOut.as<unsigned char>() + chanBase[c], chanBytes[c],
                                          cudaMemcpyDeviceToHost, st),
                          "D2H nnzVal");
    SIG_CHECK(cudaStreamSynchronize(st), "sync");
}

}  // namespace xjpcg
