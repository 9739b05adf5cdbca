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
//   mixed   FP64 iterative refinement around an FP32 inner CG: r = b - A x in
//           FP64, inner solve A d = r / ||r|| in FP32 (values, vectors and
//           per-thread accumulation) to a relative drop innerTol, x += ||r|| d
//           in FP64; stop when ||b - A x|| <= tol ||b|| (true residual).
// Lanes per row (G) and CTA size are template parameters chosen by the host
// tuner.
#include <cuda_runtime.h>

#include <algorithm>
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
    double innerTol;
    int smemRows;      // p capacity in shared memory (rows)
    int maxOuter;
};

template <int NT, int NV, typename T>
__device__ __forceinline__ void block_allreduce(T (&v)[NV]) {
    __shared__ T bc[NV];
    block_sum<NT, NV, T>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) bc[i] = v[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = bc[i];
    __syncthreads();
}

// CG on one system: A d = rhs, d0 = 0, Jacobi preconditioner J.  On entry r
// holds rhs; on exit d holds the solution increment.  VT is the precision of
// the vectors and matrix values; reductions leave the CTA in double.
// Stop: rr < tols (tols = rr0 * relTol^2) or k reaches maxK.  Returns k (the
// iterations run) and the last r.r / rr0 through the references.
template <typename VT, int NT, int G>
__device__ uint32_t cg_core(int n, const int* __restrict__ rowptr, int e0, const int* __restrict__ col,
                            const VT* __restrict__ val, VT* __restrict__ r, VT* __restrict__ d,
                            const VT* __restrict__ J, VT* __restrict__ Ap, VT* P, double relTol, uint32_t maxK,
                            double& rrLast, double& rr0Out, bool& breakdown) {
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
        double v1[1] = {(double)pAp};
        block_allreduce<NT, 1, double>(v1);
        const double alphaD = rz / v1[0];
        const VT alpha = (VT)alphaD;
        AccT rrP = 0, rzP = 0;
        for (int i = tid; i < n; i += NT) {
            const VT di = fma(alpha, P[i], d[i]);
            const VT ri = fma(-alpha, Ap[i], r[i]);
            const VT zi = ri * J[i];
            d[i] = di;
            r[i] = ri;
            rrP = fma((AccT)ri, (AccT)ri, rrP);
            rzP = fma((AccT)ri, (AccT)zi, rzP);
        }
        double w[2] = {(double)rrP, (double)rzP};
        block_allreduce<NT, 2, double>(w);
        const double beta = w[1] / rz;
        rz = w[1];
        rrLast = w[0];
        ++k;
        if (!isfinite(alphaD) || !isfinite(beta) || !isfinite(w[0])) {
            breakdown = true;
            break;
        }
        if (!(w[0] >= tols) || k >= maxK) break;  // !(rr >= tols) == (rr < tols) or NaN (caught above)
        const VT betaV = (VT)beta;
        for (int i = tid; i < n; i += NT) P[i] = fma(betaV, P[i], r[i] * J[i]);
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

template <int NT, int G>
__global__ void __launch_bounds__(NT) batched_fp64_kernel(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    double* pS = reinterpret_cast<double*>(smem);
    for (;;) {
        const int sys = next_system(a);
        if (sys < 0) break;
        const int r0 = a.sysRow[sys], n = a.sysRow[sys + 1] - r0;
        const int e0 = a.rowptr[r0];
        double* P = n <= a.smemRows ? pS : a.pGlobal + r0;
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
        const uint32_t k = cg_core<double, NT, G>(n, a.rowptr + r0, e0, a.col + e0, a.val + e0, a.r + r0, a.x + r0,
                                                  a.J + r0, a.Ap + r0, P, a.tol, a.maxIterP1, rrLast, rr0, bd);
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

template <int NT, int G>
__global__ void __launch_bounds__(NT) batched_mixed_kernel(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    float* pS = reinterpret_cast<float*>(smem);
    for (;;) {
        const int sys = next_system(a);
        if (sys < 0) break;
        const int r0 = a.sysRow[sys], n = a.sysRow[sys + 1] - r0;
        const int e0 = a.rowptr[r0];
        float* P = n <= a.smemRows ? pS : a.p32Global + r0;
        const int* rp = a.rowptr + r0;
        const int* cl = a.col + e0;
        const double* vl = a.val + e0;
        double bbA = 0;
        for (int i = threadIdx.x; i < n; i += NT) {
            const double bi = a.b[r0 + i];
            a.x[r0 + i] = 0.0;
            a.J32[r0 + i] = (float)(1.0 / a.diag[r0 + i]);
            bbA = fma(bi, bi, bbA);
        }
        double vb[1] = {bbA};
        block_allreduce<NT, 1, double>(vb);
        const double bb = vb[0];
        uint32_t inner = 0, outer = 0;
        bool bd = false;
        double rrTrue = bb;
        for (;;) {
            // true residual in FP64: r = b - A x
            double rrA = 0;
            for (int row = threadIdx.x; row < n; row += NT) {
                const int s = rp[row] - e0, e = rp[row + 1] - e0;
                double acc = 0;
                for (int q = s; q < e; ++q) acc = fma(vl[q], a.x[r0 + cl[q]], acc);
                const double ri = a.b[r0 + row] - acc;
                a.r[r0 + row] = ri;
                rrA = fma(ri, ri, rrA);
            }
            double vr[1] = {rrA};
            block_allreduce<NT, 1, double>(vr);
            rrTrue = vr[0];
            if (!isfinite(rrTrue)) {
                bd = true;
                break;
            }
            if (!(rrTrue > bb * a.tol * a.tol) || inner >= a.maxIterP1 - 1u || outer >= (uint32_t)a.maxOuter) break;
            const double sc = rrTrue > 0 ? 1.0 / sqrt(rrTrue) : 1.0;
            for (int i = threadIdx.x; i < n; i += NT) a.r32[r0 + i] = (float)(a.r[r0 + i] * sc);
            __syncthreads();
            double rrL, rr0;
            bool bdi;
            const uint32_t budget = a.maxIterP1 - 1u - inner;
            const uint32_t k = cg_core<float, NT, G>(n, rp, e0, cl, a.val32 + e0, a.r32 + r0, a.d32 + r0,
                                                     a.J32 + r0, a.Ap32 + r0, P, a.innerTol, budget, rrL, rr0, bdi);
            inner += k;
            ++outer;
            const double inv = 1.0 / sc;
            for (int i = threadIdx.x; i < n; i += NT) a.x[r0 + i] = fma((double)a.d32[r0 + i], inv, a.x[r0 + i]);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            BatchResult& o = a.res[sys];
            o.itersRun = inner;
            o.iters = inner;
            o.outer = outer;
            o.res = sqrt(rrTrue / bb);
            o.status = bd ? 1u : 0u;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
namespace {
template <int NT, int G>
struct BatchInst {
    static cudaError_t launch(bool mixed, int grid, size_t smem, cudaStream_t st, const BatchArgs& a) {
        if (mixed) {
            cudaError_t e = cudaFuncSetAttribute(batched_mixed_kernel<NT, G>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            batched_mixed_kernel<NT, G><<<grid, NT, smem, st>>>(a);
        } else {
            cudaError_t e = cudaFuncSetAttribute(batched_fp64_kernel<NT, G>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            batched_fp64_kernel<NT, G><<<grid, NT, smem, st>>>(a);
        }
        return cudaGetLastError();
    }
    static int blocksPerSm(bool mixed, size_t smem) {
        int nb = 0;
        cudaError_t e;
        if (mixed) {
            cudaFuncSetAttribute(batched_mixed_kernel<NT, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_mixed_kernel<NT, G>, NT, smem);
        } else {
            cudaFuncSetAttribute(batched_fp64_kernel<NT, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_fp64_kernel<NT, G>, NT, smem);
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
    cudaError_t (*launch)(bool, int, size_t, cudaStream_t, const BatchArgs&);
    int (*bps)(bool, size_t);
};
const BatchCfg kBatchCfgs[] = {
    {256, 1, &BatchInst<256, 1>::launch, &BatchInst<256, 1>::blocksPerSm},
    {256, 2, &BatchInst<256, 2>::launch, &BatchInst<256, 2>::blocksPerSm},
    {512, 1, &BatchInst<512, 1>::launch, &BatchInst<512, 1>::blocksPerSm},
    {512, 2, &BatchInst<512, 2>::launch, &BatchInst<512, 2>::blocksPerSm},
    {128, 1, &BatchInst<128, 1>::launch, &BatchInst<128, 1>::blocksPerSm},
    {1024, 1, &BatchInst<1024, 1>::launch, &BatchInst<1024, 1>::blocksPerSm},
};
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
    const int grid = std::max(1, std::min((nsys * 32 + 255) / 256, 152 * 16));
    batch_validate_kernel<<<grid, 256, 0, st>>>(nsys, sysRow, rowptr, col, flag);
    return cudaGetLastError();
}

int batch_num_configs() { return (int)(sizeof(kBatchCfgs) / sizeof(kBatchCfgs[0])); }
void batch_config_shape(int cfg, int* threads, int* lanes) {
    *threads = kBatchCfgs[cfg].threads;
    *lanes = kBatchCfgs[cfg].lanes;
}

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
    a.innerTol = L.innerTol;
    a.smemRows = smemRows;
    a.maxOuter = 64;
    const size_t smem = (size_t)smemRows * (mixed ? sizeof(float) : sizeof(double));
    const BatchCfg& c = kBatchCfgs[cfg];
    const int bps = c.bps(mixed, smem);
    if (bps <= 0) return cudaErrorInvalidConfiguration;
    const int grid = std::max(1, std::min(L.nsys, bps * numSms));
    if (gridOut) *gridOut = grid;
    return c.launch(mixed, grid, smem, st, a);
}

}  // namespace xjpcg
