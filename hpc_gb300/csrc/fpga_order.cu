// fpga_order.cu -- the JPCG loop in the reference FPGA's arithmetic order.
//
// xJPCG_gbSignatureSolve with summation order 1 runs the solve over a matrix
// loaded from the reference's partitioned buffers with every operation in
// the order the reference's C source writes it, so that iteration records
// and x come out bit for bit as a C execution of that source gives them:
//
//   init   pcg/sw/include/impl/cgVector.hpp:101-114: r = b, J = 1/diag,
//          z = J*r, p = z, x = 0 over the 4-padded length (diag padded with
//          1, b with 0); bb += b*b and rz += r*z summed in index order from 0.
//   SpMV   sig_ordered_spmv_kernel (signature_kernels.cu).
//   dots   xf::blas::DotHelper<double, 2> and nrm2s (L1/blas/include/hw/blas/
//          helpers/funcs/dotHelper.hpp, sum.hpp, padding.hpp; L1/hpc/include/
//          hw/cgSolver/nrm2s.hpp): the rounded products of each 4-entry group
//          summed as (p0 + p1) + (p2 + p3); the group sums zero-padded to a
//          multiple of 8; each 8 summed as a binary tree (the delayed adder's
//          shift register; IEEE addition commutes, so the tree over the
//          register's reversed contents equals this one); those block sums
//          added in order to a sum that starts at 0.
//   update x = alpha*p + x, r = (-alpha)*Ap + r (axpy.hpp:71), z = r*J;
//          p = beta*p + z (update_pk.hpp:33); alpha = rz/pAp, beta = rz'/rz.
// Every multiply, add and divide is a separate round-to-nearest operation
// (__dmul_rn, __dadd_rn, __ddiv_rn): no contraction into fused multiply-adds.
//
// This is a checking mode, not the fast path: the block sums of each dot are
// added by one thread in order (the reference's accumulation is sequential),
// and the init sums run the same way.  The host drives the loop in batches;
// every kernel that changes the solve returns at once when the loop is done.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"
#include "xjpcg_state.h"

namespace xjpcg {

namespace {

constexpr int kFoThreads = 256;

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ void fo_record(CgState* s, uint32_t k, double rr, double rz, double alpha, double beta) {
    if (s->records == nullptr || s->recCap < 2) return;
    const uint32_t slot = (k + 1u < s->recCap) ? k + 1u : 1u + (k % (s->recCap - 1u));
    IterRecord rec;
    rec.id = 0;
    rec.iter = k;
    rec.vecSize = s->vecSize;
    rec.maxIter = s->maxIterP1;
    rec.tols = s->tols;
    rec.res = rr;
    rec.rz = rz;
    rec.alpha = alpha;
    rec.beta = beta;
    rec.clock = globaltimer_ns();
    s->records[slot] = rec;
}

__global__ void __launch_bounds__(kFoThreads) fo_init_kernel(int n, int n4, const double* __restrict__ b,
                                                             const double* __restrict__ diag, double* __restrict__ x,
                                                             double* __restrict__ r, double* __restrict__ p,
                                                             double* __restrict__ J, double* __restrict__ z) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const double bi = i < n ? b[i] : 0.0;
        const double di = i < n ? diag[i] : 1.0;
        const double ji = __ddiv_rn(1.0, di);
        const double zi = mul(ji, bi);
        r[i] = bi;
        J[i] = ji;
        z[i] = zi;
        p[i] = zi;
        x[i] = 0.0;
    }
}

// bb and rz of the init in index order, then the command slot and state.
__global__ void fo_init_sums_kernel(int n4, const double* __restrict__ r, const double* __restrict__ z, CgState* s) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double bb = 0.0, rz = 0.0;
    for (int i = 0; i < n4; ++i) {
        const double ri = r[i];
        bb = add(bb, mul(ri, ri));
        rz = add(rz, mul(ri, z[i]));
    }
    s->bb = bb;
    s->rz = rz;
    s->rr = bb;
    s->tols = mul(mul(bb, s->tol), s->tol);  // cgVector.hpp:153: p_dot * p_tol * p_tol
    s->k = 0;
    s->done = 0;
    s->status &= ~(kStatusBreakdown | kStatusWaitTimeout);
    s->vecSize = (uint32_t)n4;
    if (s->records && s->recCap > 0) {
        IterRecord rec = {};
        rec.maxIter = s->maxIterP1;
        rec.vecSize = (uint32_t)n4;
        rec.tols = s->tols;
        rec.res = bb;
        rec.rz = rz;
        rec.clock = globaltimer_ns();
        s->records[0] = rec;
    }
}

// One thread per block of 32 entries (8 groups of 4): the 8-group tree of
// the 4-entry trees of a[i]*b[i] (and of c[i]*d[i] when c is not null).
// Groups past the end are the zero padding.
__global__ void __launch_bounds__(kFoThreads) fo_block_dot_kernel(int n4, const double* __restrict__ a,
                                                                  const double* __restrict__ b,
                                                                  const double* __restrict__ c,
                                                                  const double* __restrict__ d,
                                                                  double* __restrict__ t1, double* __restrict__ t2,
                                                                  const CgState* s) {
    if (*(const volatile uint32_t*)&s->done) return;
    const int groups = n4 / 4;
    const int blocks = (groups + 7) / 8;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < blocks; j += gridDim.x * blockDim.x) {
        double g1[8], g2[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int grp = 8 * j + q;
            g1[q] = 0.0;
            g2[q] = 0.0;
            if (grp < groups) {
                const int e = 4 * grp;
                g1[q] = add(add(mul(a[e], b[e]), mul(a[e + 1], b[e + 1])),
                            add(mul(a[e + 2], b[e + 2]), mul(a[e + 3], b[e + 3])));
                if (c != nullptr)
                    g2[q] = add(add(mul(c[e], d[e]), mul(c[e + 1], d[e + 1])),
                                add(mul(c[e + 2], d[e + 2]), mul(c[e + 3], d[e + 3])));
            }
        }
        t1[j] = add(add(add(g1[0], g1[1]), add(g1[2], g1[3])), add(add(g1[4], g1[5]), add(g1[6], g1[7])));
        if (c != nullptr)
            t2[j] = add(add(add(g2[0], g2[1]), add(g2[2], g2[3])), add(add(g2[4], g2[5]), add(g2[6], g2[7])));
    }
}

// The block sums added in order from 0 by one thread; then alpha
// (krnl_storeApk.cpp:70) from p.Ap.
__global__ void fo_alpha_kernel(int blocks, const double* __restrict__ t, CgState* s) {
    if (blockIdx.x != 0 || threadIdx.x != 0 || s->done) return;
    double pAp = 0.0;
    for (int j = 0; j < blocks; ++j) pAp = add(pAp, t[j]);
    s->pAp = pAp;
    s->alpha = __ddiv_rn(s->rz, pAp);
}

// x = alpha*p + x, r = (-alpha)*Ap + r, z = r*J, z written over Ap.
__global__ void __launch_bounds__(kFoThreads) fo_update_kernel(int n4, double* __restrict__ x,
                                                               const double* __restrict__ p, double* __restrict__ r,
                                                               double* __restrict__ Apz, const double* __restrict__ J,
                                                               const CgState* s) {
    if (*(const volatile uint32_t*)&s->done) return;
    const double alpha = s->alpha, nalpha = -s->alpha;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        x[i] = add(mul(alpha, p[i]), x[i]);
        const double ri = add(mul(nalpha, Apz[i]), r[i]);
        r[i] = ri;
        Apz[i] = mul(ri, J[i]);
    }
}

// rr and rz' from their block sums (in order from 0), beta, the record and
// the stop rule of control.hpp:83.
__global__ void fo_beta_kernel(int blocks, const double* __restrict__ t1, const double* __restrict__ t2, CgState* s) {
    if (blockIdx.x != 0 || threadIdx.x != 0 || s->done) return;
    double rr = 0.0, rzN = 0.0;
    for (int j = 0; j < blocks; ++j) {
        rr = add(rr, t1[j]);
        rzN = add(rzN, t2[j]);
    }
    const double alpha = s->alpha;
    const double beta = __ddiv_rn(rzN, s->rz);
    s->rr = rr;
    s->rz = rzN;
    s->beta = beta;
    uint32_t k = s->k;
    fo_record(s, k, rr, rzN, alpha, beta);
    bool cont = !(rr < s->tols);
    ++k;
    cont = cont && (k < s->maxIterP1);
    if (!isfinite(alpha) || !isfinite(beta) || !isfinite(rr)) {
        s->status |= kStatusBreakdown;
        cont = false;
    }
    s->k = k;
    s->pupdateDue = 1u;
    s->done = cont ? 0u : 1u;
}

// p = beta*p + z, once per iteration (also on the iteration that stopped
// the loop, as update_pk runs there too; it changes no output).
__global__ void __launch_bounds__(kFoThreads) fo_pupdate_kernel(int n4, double* __restrict__ p,
                                                                const double* __restrict__ z, CgState* s) {
    if (!*(const volatile uint32_t*)&s->pupdateDue) return;
    const double beta = s->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x)
        p[i] = add(mul(beta, p[i]), z[i]);
}

__global__ void fo_pupdate_clear_kernel(CgState* s) {
    if (blockIdx.x == 0 && threadIdx.x == 0) s->pupdateDue = 0u;
}

int fo_grid(int work) {
    return std::max(1, std::min((work + kFoThreads - 1) / kFoThreads, device_sm_count() * 8));
}

}  // namespace

int fo_blocks(int n4) { return (n4 / 4 + 7) / 8; }

cudaError_t fo_init(cudaStream_t st, int n, int n4, const double* b, const double* diag, double* x, double* r,
                    double* p, double* J, double* z, CgState* s) {
    fo_init_kernel<<<fo_grid(n4), kFoThreads, 0, st>>>(n, n4, b, diag, x, r, p, J, z);
    fo_init_sums_kernel<<<1, 1, 0, st>>>(n4, r, z, s);
    fo_pupdate_clear_kernel<<<1, 1, 0, st>>>(s);
    return cudaGetLastError();
}

// One iteration after the SpMV: p.Ap and alpha, the x/r/z update, r.r and
// r.z, beta and the stop test, the p update.  t holds 2 * fo_blocks(n4).
cudaError_t fo_iteration_tail(cudaStream_t st, int n4, double* x, double* p, double* r, double* Apz, const double* J,
                              double* t, CgState* s) {
    const int blocks = fo_blocks(n4);
    fo_block_dot_kernel<<<fo_grid(blocks), kFoThreads, 0, st>>>(n4, p, Apz, nullptr, nullptr, t, nullptr, s);
    fo_alpha_kernel<<<1, 1, 0, st>>>(blocks, t, s);
    fo_update_kernel<<<fo_grid(n4), kFoThreads, 0, st>>>(n4, x, p, r, Apz, J, s);
    fo_block_dot_kernel<<<fo_grid(blocks), kFoThreads, 0, st>>>(n4, r, r, r, Apz, t, t + blocks, s);
    fo_beta_kernel<<<1, 1, 0, st>>>(blocks, t, t + blocks, s);
    fo_pupdate_kernel<<<fo_grid(n4), kFoThreads, 0, st>>>(n4, p, Apz, s);
    fo_pupdate_clear_kernel<<<1, 1, 0, st>>>(s);
    return cudaGetLastError();
}

}  // namespace xjpcg
