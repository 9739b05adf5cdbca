// batched_kernels.cu -- thousands of independent Jacobi-PCG solves in one
// persistent launch.
//
// Layout: the systems are concatenated.  sysRow[s] .. sysRow[s+1] are system
// s's rows in the global row numbering; rowptr holds global nnz offsets and
// col holds system-local column indices; b, diag, x and the work vectors are
// concatenated the same way.
//
// Each CTA takes the next system from an atomic queue (the host orders the
// queue by decreasing nnz so the long solves start first) and runs that
// system's whole solve: the direction vector p lives in shared memory, so the
// SpMV gathers never leave the SM, and the matrix, r, x, J and Ap stream from
// L2/HBM.  Every reduction is a fixed-order CTA reduction, so a system's result
// does not depend on which CTA solved it or when.  Each system stops on its own
// test (the per-system convergence mask): the xJPCG rule r.r < b.b tol^2 with
// at most maxIter + 1 iterations (pcg/hw/include/control.hpp:83,
// L1/hpc/include/hw/cgSolver/tasks.hpp:43-47), and its iteration count,
// residual and status are written to its result slot.
//
// Two precisions share the CG core:
//   fp64    the xJPCG iteration in FP64 (same arithmetic as cg_kernels.cu).
//   mixed   reliable updates: FP32 CG recurrences (values, vectors and
//           per-thread accumulation) with FP64 refreshes of the true residual
//           that fold the FP32 increment into the FP64 x; stop when
//           ||b - A x|| <= tol ||b|| (true residual).
// Lanes per row (G) and CTA size are template parameters chosen by the host
// tuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <type_traits>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

struct BatchArgs {
    int nsys;
    const int* sysRow;
    const int* order;
    const int* rowptr;
    const int* col;
    const double* val;
    const float* val32;
    const double* b;
    const double* diag;
    double* x;
    double* r;
    double* Ap;
    double* J;
    float* r32;
    float* d32;
    float* Ap32;
    float* J32;
    double* pGlobal;   // p when a system does not fit in shared memory
    float* p32Global;
    BatchResult* res;
    uint32_t* queue;
    uint32_t maxIterP1;
    double tol;
    double delta2;     // mixed: refresh when the FP32 r.r falls below delta2 * its running maximum
    int smemRows;      // p capacity in shared memory (rows)
    // per-system SELL-32 copy (sliced kernels): slice s of system i is global
    // slice sliceBase[i] + s; its 32 x width stored entries start at
    // sliceOff[global slice], slice-column-major, with 16-bit local columns
    const int* sliceBase;
    const int* sliceOff;
    const double* sval;
    const float* sval32;
    const uint16_t* scol;
    const int* patLen;  // per global slice: shared column offsets, or 0
    const int* patOff;  // kBatchPatMax per global slice
    const int2* meta;   // per global slice: {value offset, width | kSliceSysPat}
    const int* sysPat;  // per system: pattern length, then kBatchPatMax offsets
};

// One sliced row sum: lane l of the warp holds row 32 j + l of its system.
template <typename VT, typename AccT>
__device__ __forceinline__ AccT slice_dot(const int* __restrict__ sliceOff, int j, const VT* __restrict__ sval,
                                          const uint16_t* __restrict__ scol, const VT* P, int lane32) {
    const int off = sliceOff[j], w = (sliceOff[j + 1] - off) >> 5;
    const VT* vp = sval + off + lane32;
    const uint16_t* cp = scol + off + lane32;
    AccT acc = AccT(0);
    int k = 0;
    for (; k + 4 <= w; k += 4) {
        VT v[4];
        int c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            v[u] = __ldcs(vp + 32 * (k + u));
            c[u] = __ldcs(cp + 32 * (k + u));
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) acc = fma((AccT)v[u], (AccT)P[c[u]], acc);
    }
    for (; k < w; ++k) acc = fma((AccT)__ldcs(vp + 32 * k), (AccT)P[__ldcs(cp + 32 * k)], acc);
    return acc;
}

// Which kernels read shared column offsets (slice_dot2's first branch).  On
// 4,096 systems (same iterations, same bits either way): mixed 71.7 ms
// against 77.1 ms without; fp64 143.4 ms against 142.0 ms without, where the
// slice's pattern length is one more dependent load before the values.
constexpr bool kBatchPat64 = false;
constexpr bool kBatchPat32 = true;
// Slice pairs that both use their system's offsets (held in shared memory)
// gather without any dependent load but the slice record: fp64 138.1 ms
// against 142.0 ms with the columns, mixed 65.0 ms against 71.5 ms with the
// per-slice offsets; same bits.
constexpr bool kBatchSys64 = true;
constexpr bool kBatchSys32 = true;

// Slice pairs of equal width up to this many columns take all their columns
// in one batch (fp64 kernel; at 40 registers the mixed kernel spilled).  On
// 4,096 systems: 143.7 / 143.4 / 142.3 ms with none / up to 5 / up to 7.
constexpr int kBatchOne = 7;

// R remaining columns of two slices as one batch: all loads, then the
// gathers, then each slice's FMAs in column order.
template <int R, typename VT, typename AccT>
__device__ __forceinline__ void slice_tail2(const VT* vp0, const uint16_t* cp0, const VT* vp1,
                                            const uint16_t* cp1, int k0, int k1, const VT* P, AccT& a0, AccT& a1) {
    VT v0[R], v1[R];
    int c0[R], c1[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
        v0[u] = __ldcs(vp0 + 32 * (k0 + u));
        c0[u] = __ldcs(cp0 + 32 * (k0 + u));
        v1[u] = __ldcs(vp1 + 32 * (k1 + u));
        c1[u] = __ldcs(cp1 + 32 * (k1 + u));
    }
#pragma unroll
    for (int u = 0; u < R; ++u) a0 = fma((AccT)v0[u], (AccT)P[c0[u]], a0);
#pragma unroll
    for (int u = 0; u < R; ++u) a1 = fma((AccT)v1[u], (AccT)P[c1[u]], a1);
}

// Two slices that both use their system's offsets (sPat, in shared memory),
// R columns each: the gathers x[row + o] depend on nothing loaded from DRAM
// and go out beside the value loads.  FMAs in column order.
template <int R, typename VT, typename AccT>
__device__ __forceinline__ void slice_sys2(const VT* vp0, const VT* vp1, const int* sPat, const VT* x0,
                                           const VT* x1, AccT& a0, AccT& a1) {
    VT v0[R], v1[R], g0[R], g1[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
        v0[u] = __ldcs(vp0 + 32 * u);
        v1[u] = __ldcs(vp1 + 32 * u);
    }
#pragma unroll
    for (int u = 0; u < R; ++u) {
        const int o = sPat[u];
        g0[u] = x0[o];
        g1[u] = x1[o];
    }
#pragma unroll
    for (int u = 0; u < R; ++u) a0 = fma((AccT)v0[u], (AccT)g0[u], a0);
#pragma unroll
    for (int u = 0; u < R; ++u) a1 = fma((AccT)v1[u], (AccT)g1[u], a1);
}

// Two slices with shared column offsets, R columns each, as one batch: the
// offsets come from the slices' small tables (one cached line for the warp),
// so the gathers x[row + o] need no column load from DRAM and go out with the
// value loads.  FMAs in column order, as in slice_dot.
template <int R, typename VT, typename AccT>
__device__ __forceinline__ void slice_pat2(const VT* vp0, const VT* vp1, const int* __restrict__ po0,
                                           const int* __restrict__ po1, const VT* x0, const VT* x1, AccT& a0,
                                           AccT& a1) {
    VT v0[R], v1[R];
    int o0[R], o1[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
        v0[u] = __ldcs(vp0 + 32 * u);
        v1[u] = __ldcs(vp1 + 32 * u);
        o0[u] = __ldg(po0 + u);
        o1[u] = __ldg(po1 + u);
    }
#pragma unroll
    for (int u = 0; u < R; ++u) a0 = fma((AccT)v0[u], (AccT)x0[o0[u]], a0);
#pragma unroll
    for (int u = 0; u < R; ++u) a1 = fma((AccT)v1[u], (AccT)x1[o1[u]], a1);
}

// Two slices of one warp at once (j0 and j1), for twice the loads in flight:
// their batches of 4 columns are interleaved while both slices have one, then
// each slice finishes alone.  Each slice's FMAs run in its column order, as in
// slice_dot, so both sums are slice_dot's bit for bit.
template <typename VT, typename AccT, int ONE, bool PAT>
__device__ __forceinline__ void slice_dot2(const int* __restrict__ sliceOff, const int* __restrict__ patLen,
                                           const int* __restrict__ patOff, int j0, int j1,
                                           const VT* __restrict__ sval, const uint16_t* __restrict__ scol,
                                           const VT* P, int lane32, AccT& acc0, AccT& acc1) {
    if (PAT) {
        const int L0 = patLen[j0], L1 = patLen[j1];
        if (L0 > 0 && L0 == L1 && L0 <= 7) {
            const VT* vp0 = sval + sliceOff[j0] + lane32;
            const VT* vp1 = sval + sliceOff[j1] + lane32;
            const int* po0 = patOff + (size_t)j0 * kBatchPatMax;
            const int* po1 = patOff + (size_t)j1 * kBatchPatMax;
            const VT* x0 = P + 32 * j0 + lane32;
            const VT* x1 = P + 32 * j1 + lane32;
            AccT a0 = AccT(0), a1 = AccT(0);
            switch (L0) {
                case 1: slice_pat2<1>(vp0, vp1, po0, po1, x0, x1, a0, a1); break;
                case 2: slice_pat2<2>(vp0, vp1, po0, po1, x0, x1, a0, a1); break;
                case 3: slice_pat2<3>(vp0, vp1, po0, po1, x0, x1, a0, a1); break;
                case 4: slice_pat2<4>(vp0, vp1, po0, po1, x0, x1, a0, a1); break;
                case 5: slice_pat2<5>(vp0, vp1, po0, po1, x0, x1, a0, a1); break;
                case 6: slice_pat2<6>(vp0, vp1, po0, po1, x0, x1, a0, a1); break;
                default: slice_pat2<7>(vp0, vp1, po0, po1, x0, x1, a0, a1); break;
            }
            acc0 = a0;
            acc1 = a1;
            return;
        }
    }
    const int off0 = sliceOff[j0], w0 = (sliceOff[j0 + 1] - off0) >> 5;
    const int off1 = sliceOff[j1], w1 = (sliceOff[j1 + 1] - off1) >> 5;
    const VT* vp0 = sval + off0 + lane32;
    const VT* vp1 = sval + off1 + lane32;
    const uint16_t* cp0 = scol + off0 + lane32;
    const uint16_t* cp1 = scol + off1 + lane32;
    AccT a0 = AccT(0), a1 = AccT(0);
    if (ONE > 0 && w0 == w1 && w0 <= ONE) {
        // narrow slices (a 5-point stencil): every column in one batch
        switch (w0) {
            case 1: slice_tail2<1>(vp0, cp0, vp1, cp1, 0, 0, P, a0, a1); break;
            case 2: slice_tail2<2>(vp0, cp0, vp1, cp1, 0, 0, P, a0, a1); break;
            case 3: slice_tail2<3>(vp0, cp0, vp1, cp1, 0, 0, P, a0, a1); break;
            case 4: slice_tail2<4>(vp0, cp0, vp1, cp1, 0, 0, P, a0, a1); break;
            case 5: slice_tail2<5>(vp0, cp0, vp1, cp1, 0, 0, P, a0, a1); break;
            case 6: if (ONE >= 6) slice_tail2<6>(vp0, cp0, vp1, cp1, 0, 0, P, a0, a1); break;
            case 7: if (ONE >= 7) slice_tail2<7>(vp0, cp0, vp1, cp1, 0, 0, P, a0, a1); break;
            default: break;
        }
        acc0 = a0;
        acc1 = a1;
        return;
    }
    const int wm = w0 < w1 ? w0 : w1;
    int k = 0;
    for (; k + 4 <= wm; k += 4) {
        VT v0[4], v1[4];
        int c0[4], c1[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            v0[u] = __ldcs(vp0 + 32 * (k + u));
            c0[u] = __ldcs(cp0 + 32 * (k + u));
            v1[u] = __ldcs(vp1 + 32 * (k + u));
            c1[u] = __ldcs(cp1 + 32 * (k + u));
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) a0 = fma((AccT)v0[u], (AccT)P[c0[u]], a0);
#pragma unroll
        for (int u = 0; u < 4; ++u) a1 = fma((AccT)v1[u], (AccT)P[c1[u]], a1);
    }
    int k0 = k, k1 = k;
    for (; k0 + 4 <= w0; k0 += 4) {
        VT v[4];
        int c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            v[u] = __ldcs(vp0 + 32 * (k0 + u));
            c[u] = __ldcs(cp0 + 32 * (k0 + u));
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) a0 = fma((AccT)v[u], (AccT)P[c[u]], a0);
    }
    for (; k1 + 4 <= w1; k1 += 4) {
        VT v[4];
        int c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            v[u] = __ldcs(vp1 + 32 * (k1 + u));
            c[u] = __ldcs(cp1 + 32 * (k1 + u));
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) a1 = fma((AccT)v[u], (AccT)P[c[u]], a1);
    }
    // the last w mod 4 columns: one unrolled batch when both slices have the
    // same number left (the usual case: equal widths), else column by column
    if (w0 - k0 == w1 - k1) {
        switch (w0 - k0) {
            case 1: slice_tail2<1>(vp0, cp0, vp1, cp1, k0, k1, P, a0, a1); break;
            case 2: slice_tail2<2>(vp0, cp0, vp1, cp1, k0, k1, P, a0, a1); break;
            case 3: slice_tail2<3>(vp0, cp0, vp1, cp1, k0, k1, P, a0, a1); break;
            default: break;
        }
        acc0 = a0;
        acc1 = a1;
        return;
    }
    for (; k0 < w0 || k1 < w1; ++k0, ++k1) {
        const bool h0 = k0 < w0, h1 = k1 < w1;
        VT v0 = VT(0), v1 = VT(0);
        int c0 = 0, c1 = 0;
        if (h0) {
            v0 = __ldcs(vp0 + 32 * k0);
            c0 = __ldcs(cp0 + 32 * k0);
        }
        if (h1) {
            v1 = __ldcs(vp1 + 32 * k1);
            c1 = __ldcs(cp1 + 32 * k1);
        }
        if (h0) a0 = fma((AccT)v0, (AccT)P[c0], a0);
        if (h1) a1 = fma((AccT)v1, (AccT)P[c1], a1);
    }
    acc0 = a0;
    acc1 = a1;
}

// Elements per step of the update and p-update passes (loads first).  On
// 4,096 systems the fp64 batch took 156.2 / 149.8 / 148.0 ms with 1 / 2 / 4.
constexpr int kBatchUpd = 4;

// Two slices j0 and j1 = j0 + stride/32 of one warp: by their system's
// offsets when both records carry the flag (SYS), else slice_dot2.
template <typename VT, typename AccT, int ONE, bool PAT, bool SYS>
__device__ __forceinline__ void slice_pair(const int* __restrict__ sliceOff, const int* __restrict__ patLen,
                                           const int* __restrict__ patOff, const int2* __restrict__ meta,
                                           const int* sPat, int sysL, int j0, int j1, int stride,
                                           const VT* __restrict__ sval, const uint16_t* __restrict__ scol,
                                           const VT* P, int lane32, AccT& acc0, AccT& acc1) {
    if (SYS && sysL > 0) {
        const int2 m0 = meta[j0], m1 = meta[j1];
        if (m0.y & m1.y & kSliceSysPat) {
            const VT* vp0 = sval + m0.x + lane32;
            const VT* vp1 = sval + m1.x + lane32;
            const VT* x0 = P + 32 * j0 + lane32;
            const VT* x1 = x0 + stride;
            AccT a0 = AccT(0), a1 = AccT(0);
            switch (sysL) {
                case 1: slice_sys2<1>(vp0, vp1, sPat + 1, x0, x1, a0, a1); break;
                case 2: slice_sys2<2>(vp0, vp1, sPat + 1, x0, x1, a0, a1); break;
                case 3: slice_sys2<3>(vp0, vp1, sPat + 1, x0, x1, a0, a1); break;
                case 4: slice_sys2<4>(vp0, vp1, sPat + 1, x0, x1, a0, a1); break;
                case 5: slice_sys2<5>(vp0, vp1, sPat + 1, x0, x1, a0, a1); break;
                case 6: slice_sys2<6>(vp0, vp1, sPat + 1, x0, x1, a0, a1); break;
                case 7: slice_sys2<7>(vp0, vp1, sPat + 1, x0, x1, a0, a1); break;
                default: slice_sys2<8>(vp0, vp1, sPat + 1, x0, x1, a0, a1); break;
            }
            acc0 = a0;
            acc1 = a1;
            return;
        }
    }
    slice_dot2<VT, AccT, ONE, PAT>(sliceOff, patLen, patOff, j0, j1, sval, scol, P, lane32, acc0, acc1);
}

// CTA sum returned in every thread.  Doubles: the narrow block_allsum, in
// which warp 0 alone adds the threads' values in a fixed order
// (xjpcg_device.cuh), so few FP64 adds are spent.  The FP64 kernel pins its
// CTAs per SM in its launch bounds: left to the compiler, the narrow sum's
// lower register count moved it to four CTAs with spills, which measured
// slower than a shuffle tree (190 against 176 ms for 4,096 systems).  Floats (the mixed kernel's
// inner sums): a shuffle tree in every warp, which costs no FP64 work and
// keeps the serial chain of warp 0 off the critical path (111.5 ms against
// 122.5 ms with the narrow form).
template <int NT, int NV, typename T>
__device__ __forceinline__ void block_allreduce_tree(T (&v)[NV]) {
    __shared__ T red[NV][NT / 32];
    __shared__ T bc[NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = warp_sum(v[i]);
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) red[i][wid] = v[i];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            T s = lane < NT / 32 ? red[i][lane] : T(0);
            s = warp_sum(s);
            if (lane == 0) bc[i] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = bc[i];
    __syncthreads();
}

template <int NT, int NV, typename T>
__device__ __forceinline__ void block_allreduce(T (&v)[NV]) {
    if (std::is_same<T, float>::value)
        block_allreduce_tree<NT, NV, T>(v);
    else
        block_allsum<NT, NV, T>(v);
}

// block_allreduce of doubles plus one quotient of a total, q = num /
// total[QI] (OVER = true) or total[QI] / num (OVER = false), formed by warp 0
// alone, which holds the totals, and returned in every thread with them.
// It ends without a barrier: the caller separates two calls of the same
// instantiation by at least one __syncthreads (cg_core has three between
// them), so that no thread still reads tot or qS when warp 0 rewrites them.  A
// double divide costs several FMAs on the FP64 pipe, which issues 2 per clock
// per SM; with every thread of a 512-thread CTA dividing, alpha and beta alone
// cost about 10 k FP64 operations per system and iteration, whatever the
// system's size.  (The mixed kernel keeps per-thread divides: its FP64 pipe is
// otherwise idle, and the helper's registers made its sliced form spill.)
template <int NT, int NV, int QI, bool OVER>
__device__ __forceinline__ double block_allreduce_q(double (&v)[NV], double num) {
    // the narrow form of block_allsum: warp 0 adds every thread's value
    __shared__ double part[NV][NT];
    __shared__ double tot[NV];
    __shared__ double qS;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) part[i][threadIdx.x] = v[i];
    __syncthreads();
    if (wid == 0) {
        double t[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = part[i][lane];
#pragma unroll 8
            for (int w = 1; w < NT / 32; ++w) s += part[i][w * 32 + lane];
            t[i] = warp_sum(s);  // every lane of warp 0 holds the total
            if (lane == 0) tot[i] = t[i];
        }
        // warp 0 divides (32 divides per CTA instead of NT, no divergence)
        const double q = OVER ? num / t[QI] : t[QI] / num;
        if (lane == 0) qS = q;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = tot[i];
    return qS;
}

// CG on one system: A d = rhs, d0 = 0, Jacobi preconditioner J.  On entry r
// holds rhs; on exit d holds the solution increment.  VT is the precision of
// the vectors and matrix values; reductions leave the CTA in double.
// Stop: rr < tols (tols = rr0 * relTol^2) or k reaches maxK.  Returns k (the
// iterations run) and the last r.r / rr0 through the references.
template <typename VT, int NT, int G, bool SL>
__device__ uint32_t cg_core(int n, const int* __restrict__ rowptr, int e0, const int* __restrict__ col,
                            const VT* __restrict__ val, const int* __restrict__ sliceOff,
                            const int* __restrict__ patLen, const int* __restrict__ patOff,
                            const int2* __restrict__ meta, const int* sPat,
                            const VT* __restrict__ sval, const uint16_t* __restrict__ scol, VT* __restrict__ r,
                            VT* __restrict__ d, const VT* __restrict__ J, VT* __restrict__ Ap, VT* P, double relTol,
                            uint32_t maxK, double& rrLast, double& rr0Out, bool& breakdown) {
    typedef typename std::conditional<sizeof(VT) == 8, double, float>::type AccT;
    const int tid = threadIdx.x;
    AccT rzA = 0, rrA = 0;
    for (int i = tid; i < n; i += NT) {
        const VT ri = r[i];
        const VT zi = J[i] * ri;
        P[i] = zi;
        d[i] = VT(0);
        rrA = fma((AccT)ri, (AccT)ri, rrA);
        rzA = fma((AccT)ri, (AccT)zi, rzA);
    }
    double v2[2] = {(double)rrA, (double)rzA};
    block_allreduce<NT, 2, double>(v2);
    const double rr0 = v2[0];
    double rz = v2[1];
    const double tols = rr0 * relTol * relTol;
    rr0Out = rr0;
    rrLast = rr0;
    breakdown = false;
    uint32_t k = 0;
    const int lane = tid % G;
    for (;;) {
        // Ap = A p, p.Ap
        AccT pAp = 0;
        if (SL) {
            // warp w takes slices w, w + NT/32, ...: 32 rows, one per lane
            int j = tid >> 5;
            const int sysL = kBatchSys64 ? sPat[0] : 0;  // the system's pattern length, 0: none
            for (; 32 * (j + NT / 32) < n; j += 2 * (NT / 32)) {
                AccT acc0, acc1;
                slice_pair<VT, AccT, kBatchOne, kBatchPat64, kBatchSys64>(sliceOff, patLen, patOff, meta, sPat, sysL, j,
                                                                          j + NT / 32, NT, sval, scol, P, tid & 31,
                                                                          acc0, acc1);
                const int row0 = 32 * j + (tid & 31), row1 = row0 + NT;
                if (row0 < n) {
                    Ap[row0] = (VT)acc0;
                    pAp = fma((AccT)P[row0], acc0, pAp);
                }
                if (row1 < n) {
                    Ap[row1] = (VT)acc1;
                    pAp = fma((AccT)P[row1], acc1, pAp);
                }
            }
            for (; 32 * j < n; j += NT / 32) {
                const AccT acc = slice_dot<VT, AccT>(sliceOff, j, sval, scol, P, tid & 31);
                const int row = 32 * j + (tid & 31);
                if (row < n) {
                    Ap[row] = (VT)acc;
                    pAp = fma((AccT)P[row], acc, pAp);
                }
            }
        } else {
            // Row blocks are warp-uniform so the lane shuffles always see 32 lanes.
            for (int rb = (tid >> 5) * (32 / G); rb < n; rb += NT / G) {
                const int row = rb + (tid & 31) / G;
                AccT acc = 0;
                if (row < n) {
                    const int s = rowptr[row] - e0, e = rowptr[row + 1] - e0;
                    for (int q = s + lane; q < e; q += G) acc = fma((AccT)val[q], (AccT)P[col[q]], acc);
                }
                if (G > 1) {
#pragma unroll
                    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
                }
                if (lane == 0 && row < n) {
                    Ap[row] = (VT)acc;
                    pAp = fma((AccT)P[row], acc, pAp);
                }
            }
        }
        double v1[1] = {(double)pAp};
        const double alphaD = block_allreduce_q<NT, 1, 0, true>(v1, rz);  // rz / p.Ap
        const VT alpha = (VT)alphaD;
        AccT rrP = 0, rzP = 0;
        // kBatchUpd elements per step, all loads first: the vectors stream
        // from DRAM, and one element's loads alone leave the warp waiting on
        // them.  The sums still take the elements in the order i, i + NT, ...
        constexpr int UPD = kBatchUpd;
        int i = tid;
        for (; i + (UPD - 1) * NT < n; i += UPD * NT) {
            VT pv[UPD], dv[UPD], av[UPD], qv[UPD], jv[UPD];
#pragma unroll
            for (int u = 0; u < UPD; ++u) {
                pv[u] = P[i + u * NT];
                dv[u] = d[i + u * NT];
                av[u] = Ap[i + u * NT];
                qv[u] = r[i + u * NT];
                jv[u] = J[i + u * NT];
            }
#pragma unroll
            for (int u = 0; u < UPD; ++u) {
                const VT ri = fma(-alpha, av[u], qv[u]);
                const VT zi = ri * jv[u];
                d[i + u * NT] = fma(alpha, pv[u], dv[u]);
                r[i + u * NT] = ri;
                Ap[i + u * NT] = zi;  // Ap is spent: keep z = J r for the p update
                rrP = fma((AccT)ri, (AccT)ri, rrP);
                rzP = fma((AccT)ri, (AccT)zi, rzP);
            }
        }
        for (; i < n; i += NT) {
            const VT di = fma(alpha, P[i], d[i]);
            const VT ri = fma(-alpha, Ap[i], r[i]);
            const VT zi = ri * J[i];
            d[i] = di;
            r[i] = ri;
            Ap[i] = zi;
            rrP = fma((AccT)ri, (AccT)ri, rrP);
            rzP = fma((AccT)ri, (AccT)zi, rzP);
        }
        double w[2] = {(double)rrP, (double)rzP};
        const double beta = block_allreduce_q<NT, 2, 1, false>(w, rz);  // r.z / rz
        rz = w[1];
        rrLast = w[0];
        ++k;
        if (!isfinite(alphaD) || !isfinite(beta) || !isfinite(w[0])) {
            breakdown = true;
            break;
        }
        if (!(w[0] >= tols) || k >= maxK) break;  // !(rr >= tols) == (rr < tols) or NaN (caught above)
        const VT betaV = (VT)beta;
        int t = tid;
        for (; t + (UPD - 1) * NT < n; t += UPD * NT) {  // z + beta p, z = J r
            VT pv[UPD], zv[UPD];
#pragma unroll
            for (int u = 0; u < UPD; ++u) {
                pv[u] = P[t + u * NT];
                zv[u] = Ap[t + u * NT];
            }
#pragma unroll
            for (int u = 0; u < UPD; ++u) P[t + u * NT] = fma(betaV, pv[u], zv[u]);
        }
        for (; t < n; t += NT) P[t] = fma(betaV, P[t], Ap[t]);
        __syncthreads();
    }
    return k;
}

// Next system from the queue, or -1.
__device__ __forceinline__ int next_system(const BatchArgs& a) {
    __shared__ int s_t;
    if (threadIdx.x == 0) s_t = (int)atomicAdd(a.queue, 1u);
    __syncthreads();
    const int t = s_t;
    __syncthreads();
    return t < a.nsys ? a.order[t] : -1;
}

// Launch bounds of 1,024 threads per SM (two 512-thread CTAs, 64 registers):
// the interleaved slices and the 4-element passes keep their loads in
// registers.  Pinned at 1,536 threads (40 registers) the same code spilled and
// the 4,096-system batch took 155.5 ms against 148.0 ms.
template <int NT, int G, bool SL>
__global__ void __launch_bounds__(NT, (1024 / NT) > 0 ? 1024 / NT : 1) batched_fp64_kernel(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int sPat[kBatchPatMax + 1];
    double* pS = reinterpret_cast<double*>(smem);
    for (;;) {
        const int sys = next_system(a);
        if (sys < 0) break;
        const int r0 = a.sysRow[sys], n = a.sysRow[sys + 1] - r0;
        const int e0 = a.rowptr[r0];
        double* P = n <= a.smemRows ? pS : a.pGlobal + r0;
        // the system's shared column offsets (read after the barrier below)
        if (SL && kBatchSys64 && threadIdx.x <= kBatchPatMax)
            sPat[threadIdx.x] = a.sysPat[(size_t)sys * (kBatchPatMax + 1) + threadIdx.x];
        // GenCgVector::init (cgVector.hpp:101-114): r = b, J = 1/diag, x = 0
        double bbA = 0;
        for (int i = threadIdx.x; i < n; i += NT) {
            const double bi = a.b[r0 + i];
            a.r[r0 + i] = bi;
            a.J[r0 + i] = 1.0 / a.diag[r0 + i];
            bbA = fma(bi, bi, bbA);
        }
        __syncthreads();
        double rrLast, rr0;
        bool bd;
        const uint32_t k = cg_core<double, NT, G, SL>(
            n, a.rowptr + r0, e0, a.col + e0, a.val + e0, SL ? a.sliceOff + a.sliceBase[sys] : nullptr,
            SL ? a.patLen + a.sliceBase[sys] : nullptr,
            SL ? a.patOff + (size_t)a.sliceBase[sys] * kBatchPatMax : nullptr, SL ? a.meta + a.sliceBase[sys] : nullptr,
            sPat, a.sval, a.scol,
            a.r + r0, a.x + r0, a.J + r0, a.Ap + r0, P, a.tol, a.maxIterP1, rrLast, rr0, bd);
        if (threadIdx.x == 0) {
            BatchResult& o = a.res[sys];
            o.itersRun = k;
            o.iters = k < a.maxIterP1 ? k : a.maxIterP1 - 1u;
            o.outer = 0;
            o.res = sqrt(rrLast / rr0);  // rr0 = b.b: r starts as b
            o.status = bd ? 1u : 0u;
        }
        __syncthreads();
    }
}

// Mixed precision with reliable updates, per system (the batched form of
// mixed_kernels.cu): the CG recurrences run in FP32 (values, r, p, Ap, J and
// the increment d; per-thread and CTA sums in FP32) and keep their
// search direction.  When the FP32 residual norm has fallen by delta below its
// largest value since the last refresh, looks converged, or the budget is
// spent, the refresh folds d into the FP64 x, recomputes r = b - A x with the
// FP64 matrix and restarts the FP32 residual from it.  The system stops on the
// true FP64 residual: r.r <= b.b tol^2.
// Launch bounds of 1,536 threads per SM (three 512-thread CTAs, 40 registers,
// no spills): 80.9 ms on 4,096 systems, against 95.8 ms at two CTAs per SM.
template <int NT, int G, bool SL>
__global__ void __launch_bounds__(NT, (1536 / NT) > 0 ? 1536 / NT : 1) batched_mixed_kernel(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int sPat[kBatchPatMax + 1];
    float* pS = reinterpret_cast<float*>(smem);
    const int tid = threadIdx.x;
    const int lane = tid % G;
    for (;;) {
        const int sys = next_system(a);
        if (sys < 0) break;
        const int r0 = a.sysRow[sys], n = a.sysRow[sys + 1] - r0;
        const int e0 = a.rowptr[r0];
        float* P = n <= a.smemRows ? pS : a.p32Global + r0;
        // the system's shared column offsets (read after the barrier below)
        if (SL && kBatchSys32 && threadIdx.x <= kBatchPatMax)
            sPat[threadIdx.x] = a.sysPat[(size_t)sys * (kBatchPatMax + 1) + threadIdx.x];
        const int* rp = a.rowptr + r0;
        const int* cl = a.col + e0;
        const double* vl = a.val + e0;
        const float* vl32 = a.val32 + e0;
        float* r = a.r32 + r0;
        float* d = a.d32 + r0;
        float* J = a.J32 + r0;
        float* Ap = a.Ap32 + r0;
        double* x = a.x + r0;
        // x = 0, d = 0, J = 1/diag, r = b, p = J r
        double bbA = 0;
        float rzA = 0.f;
        for (int i = tid; i < n; i += NT) {
            const double bi = a.b[r0 + i];
            const float ji = (float)(1.0 / a.diag[r0 + i]);
            const float ri = (float)bi;
            x[i] = 0.0;
            d[i] = 0.f;
            J[i] = ji;
            r[i] = ri;
            P[i] = ji * ri;
            bbA = fma(bi, bi, bbA);
            rzA = fmaf(ri, ji * ri, rzA);
        }
        double v0[2] = {bbA, (double)rzA};
        block_allreduce<NT, 2, double>(v0);
        const double bb = v0[0];
        const double tols = bb * a.tol * a.tol;
        double rz = v0[1], rrMax = bb, rrTrue = bb;
        uint32_t k = 0, outer = 0;
        bool bd = false, stop = false;
        while (!stop) {
            // Ap = A p (FP32), p.Ap
            float pAp = 0.f;
            if (SL) {
                const int* so = a.sliceOff + a.sliceBase[sys];
                const int sysL = kBatchSys32 ? sPat[0] : 0;
                int j = tid >> 5;
                for (; 32 * (j + NT / 32) < n; j += 2 * (NT / 32)) {
                    float acc0, acc1;
                    slice_pair<float, float, 0, kBatchPat32, kBatchSys32>(
                        so, a.patLen + a.sliceBase[sys], a.patOff + (size_t)a.sliceBase[sys] * kBatchPatMax,
                        a.meta + a.sliceBase[sys], sPat, sysL, j, j + NT / 32, NT, a.sval32, a.scol, P, tid & 31, acc0,
                        acc1);
                    const int row0 = 32 * j + (tid & 31), row1 = row0 + NT;
                    if (row0 < n) {
                        Ap[row0] = acc0;
                        pAp = fmaf(P[row0], acc0, pAp);
                    }
                    if (row1 < n) {
                        Ap[row1] = acc1;
                        pAp = fmaf(P[row1], acc1, pAp);
                    }
                }
                for (; 32 * j < n; j += NT / 32) {
                    const float acc = slice_dot<float, float>(so, j, a.sval32, a.scol, P, tid & 31);
                    const int row = 32 * j + (tid & 31);
                    if (row < n) {
                        Ap[row] = acc;
                        pAp = fmaf(P[row], acc, pAp);
                    }
                }
            } else {
                for (int rb = (tid >> 5) * (32 / G); rb < n; rb += NT / G) {
                    const int row = rb + (tid & 31) / G;
                    float acc = 0.f;
                    if (row < n) {
                        const int s0 = rp[row] - e0, s1 = rp[row + 1] - e0;
                        for (int q = s0 + lane; q < s1; q += G) acc = fmaf(vl32[q], P[cl[q]], acc);
                    }
                    if (G > 1) {
#pragma unroll
                        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
                    }
                    if (lane == 0 && row < n) {
                        Ap[row] = acc;
                        pAp = fmaf(P[row], acc, pAp);
                    }
                }
            }
            float v1[1] = {pAp};
            block_allreduce<NT, 1, float>(v1);
            const double alphaD = rz / (double)v1[0];
            const float alpha = (float)alphaD;
            float rrP = 0.f, rzP = 0.f;
            constexpr int UPDM = kBatchUpd;
            int i = tid;
            for (; i + (UPDM - 1) * NT < n; i += UPDM * NT) {
                float pv[UPDM], dv[UPDM], av[UPDM], qv[UPDM], jv[UPDM];
#pragma unroll
                for (int u = 0; u < UPDM; ++u) {
                    pv[u] = P[i + u * NT];
                    dv[u] = d[i + u * NT];
                    av[u] = Ap[i + u * NT];
                    qv[u] = r[i + u * NT];
                    jv[u] = J[i + u * NT];
                }
#pragma unroll
                for (int u = 0; u < UPDM; ++u) {
                    const float ri = fmaf(-alpha, av[u], qv[u]);
                    const float zi = ri * jv[u];
                    d[i + u * NT] = fmaf(alpha, pv[u], dv[u]);
                    r[i + u * NT] = ri;
                    Ap[i + u * NT] = zi;
                    rrP = fmaf(ri, ri, rrP);
                    rzP = fmaf(ri, zi, rzP);
                }
            }
            for (; i < n; i += NT) {
                const float ri = fmaf(-alpha, Ap[i], r[i]);
                const float zi = ri * J[i];
                d[i] = fmaf(alpha, P[i], d[i]);
                r[i] = ri;
                Ap[i] = zi;  // Ap is spent: keep z = J r for the p update
                rrP = fmaf(ri, ri, rrP);
                rzP = fmaf(ri, zi, rzP);
            }
            float w[2] = {rrP, rzP};
            block_allreduce<NT, 2, float>(w);
            ++k;
            const double rrN = w[0], rzN = w[1];
            if (rrN > rrMax) rrMax = rrN;
            bd = !isfinite(alphaD) || !isfinite(rrN) || !isfinite(rzN);
            const bool refresh = bd || rrN < a.delta2 * rrMax || rrN < tols || k + 1u >= a.maxIterP1;
            double beta;
            if (!refresh) {
                beta = rzN / rz;
                rz = rzN;
            } else {
                // fold, FP64 true residual, FP32 restart from it
                for (int i = tid; i < n; i += NT) {
                    x[i] += (double)d[i];
                    d[i] = 0.f;
                }
                __syncthreads();
                double rrA = 0;
                for (int row = tid; row < n; row += NT) {
                    const int s0 = rp[row] - e0, s1 = rp[row + 1] - e0;
                    double acc = 0;
                    for (int q = s0; q < s1; ++q) acc = fma(vl[q], x[cl[q]], acc);
                    const double ri = a.b[r0 + row] - acc;
                    r[row] = (float)ri;
                    rrA = fma(ri, ri, rrA);
                }
                __syncthreads();
                float rzR = 0.f;
                for (int i = tid; i < n; i += NT) {
                    const float zi = r[i] * J[i];
                    Ap[i] = zi;
                    rzR = fmaf(r[i], zi, rzR);
                }
                double v3[2] = {rrA, (double)rzR};
                block_allreduce<NT, 2, double>(v3);
                ++outer;
                rrTrue = v3[0];
                rrMax = rrTrue;
                stop = !(rrTrue > tols) || k + 1u >= a.maxIterP1;
                if (bd || !isfinite(rrTrue) || !isfinite(v3[1])) {
                    bd = true;
                    stop = true;
                }
                beta = v3[1] / rz;
                rz = v3[1];
            }
            if (stop) break;
            const float betaF = (float)beta;
            int t = tid;
            for (; t + (UPDM - 1) * NT < n; t += UPDM * NT) {  // z + beta p
                float pv[UPDM], zv[UPDM];
#pragma unroll
                for (int u = 0; u < UPDM; ++u) {
                    pv[u] = P[t + u * NT];
                    zv[u] = Ap[t + u * NT];
                }
#pragma unroll
                for (int u = 0; u < UPDM; ++u) P[t + u * NT] = fmaf(betaF, pv[u], zv[u]);
            }
            for (; t < n; t += NT) P[t] = fmaf(betaF, P[t], Ap[t]);  // z + beta p
            __syncthreads();
        }
        if (tid == 0) {
            BatchResult& o = a.res[sys];
            o.itersRun = k;
            o.iters = k;
            o.outer = outer;
            o.res = sqrt(rrTrue / bb);
            o.status = bd ? 1u : 0u;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
namespace {
template <int NT, int G, bool SL>
struct BatchInst {
    static cudaError_t launch(bool mixed, int grid, size_t smem, cudaStream_t st, const BatchArgs& a) {
        if (SL && a.sliceOff == nullptr) return cudaErrorInvalidValue;  // no sliced copy
        if (mixed) {
            cudaError_t e = cudaFuncSetAttribute(batched_mixed_kernel<NT, G, SL>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            batched_mixed_kernel<NT, G, SL><<<grid, NT, smem, st>>>(a);
        } else {
            cudaError_t e = cudaFuncSetAttribute(batched_fp64_kernel<NT, G, SL>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            batched_fp64_kernel<NT, G, SL><<<grid, NT, smem, st>>>(a);
        }
        return cudaGetLastError();
    }
    static int blocksPerSm(bool mixed, size_t smem) {
        int nb = 0;
        cudaError_t e;
        if (mixed) {
            cudaFuncSetAttribute(batched_mixed_kernel<NT, G, SL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_mixed_kernel<NT, G, SL>, NT, smem);
        } else {
            cudaFuncSetAttribute(batched_fp64_kernel<NT, G, SL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_fp64_kernel<NT, G, SL>, NT, smem);
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return nb;
    }
};

struct BatchCfg {
    int threads, lanes;
    bool sliced;
    cudaError_t (*launch)(bool, int, size_t, cudaStream_t, const BatchArgs&);
    int (*bps)(bool, size_t);
};
#define XJ_BATCH_CFG(NTV, GV, SLV) \
    { NTV, GV, SLV, &BatchInst<NTV, GV, SLV>::launch, &BatchInst<NTV, GV, SLV>::blocksPerSm }
// CSR kernels (threads x lanes per row), then the sliced kernels (one lane per row)
const BatchCfg kBatchCfgs[] = {
    XJ_BATCH_CFG(256, 1, false), XJ_BATCH_CFG(256, 2, false), XJ_BATCH_CFG(512, 1, false),
    XJ_BATCH_CFG(512, 2, false), XJ_BATCH_CFG(128, 1, false), XJ_BATCH_CFG(1024, 1, false),
    XJ_BATCH_CFG(256, 1, true),  XJ_BATCH_CFG(512, 1, true),  XJ_BATCH_CFG(1024, 1, true),
};
#undef XJ_BATCH_CFG
}  // namespace

__global__ void batch_validate_kernel(int nsys, const int* __restrict__ sysRow, const int* __restrict__ rowptr,
                                      const int* __restrict__ col, int* flag) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nsys; s += warpsPerGrid) {
        const int r0 = sysRow[s], n = sysRow[s + 1] - r0;
        const int e0 = rowptr[r0], e1 = rowptr[r0 + n];
        bool bad = false;
        for (int e = e0 + lane; e < e1; e += 32) {
            const int c = col[e];
            bad |= (c < 0 || c >= n);
        }
        if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(flag, 1);
    }
}

cudaError_t batch_validate_columns(cudaStream_t st, int nsys, const int* sysRow, const int* rowptr, const int* col,
                                   int* flag) {
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    const int grid = std::max(1, std::min((nsys * 32 + 255) / 256, device_sm_count() * 16));
    batch_validate_kernel<<<grid, 256, 0, st>>>(nsys, sysRow, rowptr, col, flag);
    return cudaGetLastError();
}

int batch_num_configs() { return (int)(sizeof(kBatchCfgs) / sizeof(kBatchCfgs[0])); }
void batch_config_shape(int cfg, int* threads, int* lanes) {
    *threads = kBatchCfgs[cfg].threads;
    *lanes = kBatchCfgs[cfg].lanes;
}
bool batch_config_sliced(int cfg) { return kBatchCfgs[cfg].sliced; }

// ---- per-system SELL-32 copy ----
namespace {
__device__ __forceinline__ int warp_max_i(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ int warp_min_i(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// System of global slice g: the largest s with sliceBase[s] <= g.
__device__ __forceinline__ int system_of_slice(const int* __restrict__ sliceBase, int nsys, int g) {
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sliceBase[mid] <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}
}  // namespace

// One warp per slice: stored entries 32 x (the slice's longest row).
// One warp per slice: the stored width, and whether the slice's rows share
// their column offsets.  The shared form takes the union of the 32 rows'
// offsets (column - row), in ascending order, as the slice's columns: row i's
// entry with offset o sits at o's position and the other positions hold 0.
// It is used when every row of the slice exists, every row's columns ascend
// strictly, the union has at most kBatchPatMax offsets and row + o lies in
// the system for all 32 rows and every o -- then each row's FMAs take its
// entries in the same order as the plain form, with exact zeros between them
// (adding +-0 to a sum that starts at +0 leaves it unchanged), and every
// gather, padding included, stays inside the system.  len[g] = 32 x width;
// patLen[g] = the number of shared offsets, or 0.  The union is built by
// repeated warp minima over each row's next offset, at most kBatchPatMax + 1
// steps.
__global__ void bsell_width_kernel(int nsys, int nslices, const int* __restrict__ sysRow,
                                   const int* __restrict__ sliceBase, const int* __restrict__ rowptr,
                                   const int* __restrict__ col, int* __restrict__ len, int* __restrict__ patLen,
                                   int* __restrict__ patOff, bool patterns) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < nslices; g += warps) {
        const int s = system_of_slice(sliceBase, nsys, g);
        const int r0 = sysRow[s], n = sysRow[s + 1] - r0;
        const int first = (g - sliceBase[s]) * 32;
        const int lr = first + lane;
        const bool in = lr < n;
        const int j0 = in ? rowptr[r0 + lr] : 0, j1 = in ? rowptr[r0 + lr + 1] : 0;
        const int w = warp_max_i(j1 - j0);
        bool ok = patterns && __all_sync(0xffffffffu, in);
        int L = 0, q = j0, myOff = 0;
        int cur = q < j1 ? col[q] - lr : INT_MAX;
        while (ok) {
            const int m = warp_min_i(cur);
            if (m == INT_MAX) break;
            if (L == kBatchPatMax || first + m < 0 || first + 31 + m >= n) {
                ok = false;
                break;
            }
            if (lane == L) myOff = m;
            ++L;
            bool bad = false;
            if (cur == m) {
                ++q;
                const int nx = q < j1 ? col[q] - lr : INT_MAX;
                bad = nx <= m;  // not strictly ascending
                cur = nx;
            }
            ok = !__any_sync(0xffffffffu, bad);
        }
        if (!ok) L = 0;
        if (lane == 0) {
            len[g] = 32 * (L > 0 ? L : w);
            patLen[g] = L;
        }
        if (lane < kBatchPatMax) patOff[(size_t)g * kBatchPatMax + lane] = lane < L ? myOff : 0;
    }
}

// One warp per slice: values (and, when scol is given, local columns) in
// slice-column-major order.  Plain slices: each row's entries in order, then
// padding with value 0 and column 0.  Shared slices: each row's entries at
// their offsets' positions, value 0 elsewhere, and column row + offset at
// every position.
template <typename VT>
__global__ void bsell_fill_kernel(int nsys, int nslices, const int* __restrict__ sysRow,
                                  const int* __restrict__ sliceBase, const int* __restrict__ rowptr,
                                  const int* __restrict__ col, const double* __restrict__ val,
                                  const int* __restrict__ sliceOff, const int* __restrict__ patLen,
                                  const int* __restrict__ patOff, VT* __restrict__ sval, uint16_t* __restrict__ scol) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < nslices; g += warps) {
        const int s = system_of_slice(sliceBase, nsys, g);
        const int r0 = sysRow[s], n = sysRow[s + 1] - r0;
        const int lr = (g - sliceBase[s]) * 32 + lane;
        const int j0 = lr < n ? rowptr[r0 + lr] : 0, j1 = lr < n ? rowptr[r0 + lr + 1] : 0;
        const int off = sliceOff[g], w = (sliceOff[g + 1] - off) >> 5;
        const int L = patLen[g];
        if (L > 0) {
            int q = j0;
            for (int k = 0; k < L; ++k) {
                const int o = patOff[(size_t)g * kBatchPatMax + k];
                const bool has = q < j1 && col[q] - lr == o;
                sval[off + 32 * k + lane] = has ? (VT)val[q] : VT(0);
                if (scol) scol[off + 32 * k + lane] = (uint16_t)(lr + o);
                if (has) ++q;
            }
            continue;
        }
        for (int k = 0; k < w; ++k) {
            const bool has = j0 + k < j1;
            sval[off + 32 * k + lane] = has ? (VT)val[j0 + k] : VT(0);
            if (scol) scol[off + 32 * k + lane] = has ? (uint16_t)col[j0 + k] : (uint16_t)0;
        }
    }
}

// One thread per slice: the slice record {value offset, width | flag} the
// kernels read with one 8-byte load, where the flag marks a slice whose shared
// offsets are its system's pattern (that of the system's middle slice, the
// interior stencil in a stencil system), and per system that pattern:
// sysPat[s * (kBatchPatMax + 1)] = its length (0: none), then the offsets.
__global__ void bsell_meta_kernel(int nsys, int nslices, const int* __restrict__ sysRow,
                                  const int* __restrict__ sliceBase, const int* __restrict__ sliceOff,
                                  const int* __restrict__ patLen, const int* __restrict__ patOff,
                                  int2* __restrict__ meta, int* __restrict__ sysPat) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < nslices; g += gridDim.x * blockDim.x) {
        const int s = system_of_slice(sliceBase, nsys, g);
        const int nsl = sliceBase[s + 1] - sliceBase[s];
        const int mid = sliceBase[s] + nsl / 2;
        const int Lm = patLen[mid], L = patLen[g];
        bool same = Lm > 0 && L == Lm;
        for (int k = 0; same && k < L; ++k)
            same = patOff[(size_t)g * kBatchPatMax + k] == patOff[(size_t)mid * kBatchPatMax + k];
        const int off = sliceOff[g], w = (sliceOff[g + 1] - off) >> 5;
        meta[g] = make_int2(off, w | (same ? kSliceSysPat : 0));
        if (g == mid) {
            int* sp = sysPat + (size_t)s * (kBatchPatMax + 1);
            sp[0] = Lm;
            for (int k = 0; k < kBatchPatMax; ++k) sp[1 + k] = k < Lm ? patOff[(size_t)mid * kBatchPatMax + k] : 0;
        }
    }
}

cudaError_t batch_sell_meta(cudaStream_t st, int nsys, int nslices, const int* sysRow, const int* sliceBase,
                            const int* sliceOff, const int* patLen, const int* patOff, int2* meta, int* sysPat) {
    const int grid = std::max(1, std::min((nslices + 255) / 256, device_sm_count() * 16));
    bsell_meta_kernel<<<grid, 256, 0, st>>>(nsys, nslices, sysRow, sliceBase, sliceOff, patLen, patOff, meta, sysPat);
    return cudaGetLastError();
}

cudaError_t batch_sell_widths(cudaStream_t st, int nsys, int nslices, const int* sysRow, const int* sliceBase,
                              const int* rowptr, const int* col, int* sliceLen, int* sliceOff, int* blockSums,
                              int* patLen, int* patOff, bool patterns) {
    const int grid = std::max(1, std::min((nslices * 32 + 255) / 256, device_sm_count() * 32));
    bsell_width_kernel<<<grid, 256, 0, st>>>(nsys, nslices, sysRow, sliceBase, rowptr, col, sliceLen, patLen, patOff,
                                             patterns);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return scan_exclusive(st, sliceLen, sliceOff, nslices + 1, blockSums);
}

template <typename VT>
cudaError_t batch_sell_fill(cudaStream_t st, int nsys, int nslices, const int* sysRow, const int* sliceBase,
                            const int* rowptr, const int* col, const double* val, const int* sliceOff,
                            const int* patLen, const int* patOff, VT* sval, uint16_t* scol) {
    const int grid = std::max(1, std::min((nslices * 32 + 255) / 256, device_sm_count() * 32));
    bsell_fill_kernel<VT><<<grid, 256, 0, st>>>(nsys, nslices, sysRow, sliceBase, rowptr, col, val, sliceOff, patLen,
                                                patOff, sval, scol);
    return cudaGetLastError();
}
template cudaError_t batch_sell_fill<double>(cudaStream_t, int, int, const int*, const int*, const int*, const int*,
                                             const double*, const int*, const int*, const int*, double*, uint16_t*);
template cudaError_t batch_sell_fill<float>(cudaStream_t, int, int, const int*, const int*, const int*, const int*,
                                            const double*, const int*, const int*, const int*, float*, uint16_t*);

// smemRows: rows of p kept in shared memory; systems larger than that keep p
// in the global scratch vector (still correct, slower).
cudaError_t batch_launch(int cfg, bool mixed, int numSms, int smemRows, cudaStream_t st, const BatchLaunch& L,
                         int* gridOut) {
    BatchArgs a;
    a.nsys = L.nsys;
    a.sysRow = L.sysRow;
    a.order = L.order;
    a.rowptr = L.rowptr;
    a.col = L.col;
    a.val = L.val;
    a.val32 = L.val32;
    a.b = L.b;
    a.diag = L.diag;
    a.x = L.x;
    a.r = L.r;
    a.Ap = L.Ap;
    a.J = L.J;
    a.r32 = L.r32;
    a.d32 = L.d32;
    a.Ap32 = L.Ap32;
    a.J32 = L.J32;
    a.pGlobal = L.pGlobal;
    a.p32Global = L.p32Global;
    a.res = L.res;
    a.queue = L.queue;
    a.maxIterP1 = L.maxIterP1;
    a.tol = L.tol;
    a.delta2 = L.delta2;
    a.smemRows = smemRows;
    a.sliceBase = L.sliceBase;
    a.sliceOff = L.sliceOff;
    a.sval = L.sval;
    a.sval32 = L.sval32;
    a.scol = L.scol;
    a.patLen = L.patLen;
    a.patOff = L.patOff;
    a.meta = L.meta;
    a.sysPat = L.sysPat;
    const size_t smem = (size_t)smemRows * (mixed ? sizeof(float) : sizeof(double));
    const BatchCfg& c = kBatchCfgs[cfg];
    const int bps = c.bps(mixed, smem);
    if (bps <= 0) return cudaErrorInvalidConfiguration;
    const int grid = std::max(1, std::min(L.nsys, bps * numSms));
    if (gridOut) *gridOut = grid;
    return c.launch(mixed, grid, smem, st, a);
}

}  // namespace xjpcg
