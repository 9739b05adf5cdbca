// mixed_kernels.cu -- mixed-precision Jacobi-PCG: FP32 inner CG inside an
// FP64 iterative-refinement loop.
//
// The whole solve is one CUDA graph with two nested conditional WHILE nodes:
//
//   ir_init                      x = 0 (fp64), J32 = 1/diag, b.b
//   WHILE outer:
//     SpMV fp64, kResidual       r = b - A x, ||r||^2          (FP64)
//     ir_check                   stop if ||r|| <= tol ||b||; s = 1/||r||
//     ir_inner_init              r32 = s r, p32 = J32 r32, d32 = 0, r.z
//     WHILE inner:
//       SpMV fp32, kCgDot        Ap = A p, p.Ap, alpha          (FP32 data)
//       cg32_update              r -= alpha Ap, r.r, r.z, beta
//       cg32_pupdate             d += alpha p, p = J r + beta p
//     ir_update                  x += d / s                     (FP64)
//
// FP64 is kept for the true residual, the outer x update and the alpha/beta
// scalars; the inner vectors, matrix values and per-thread accumulations are
// FP32 (the CTA partials are combined in FP64).  The inner loop is the same
// three-launch iteration as the fp64 solver (cg_kernels.cu) with its own
// state; it stops when its recursive r.r drops by innerTol^2 or the shared
// iteration budget is spent.
#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

constexpr int kMxThreads = 256;

__global__ void __launch_bounds__(kMxThreads) ir_init_kernel(int n, int n4, const double* __restrict__ b,
                                                             const double* __restrict__ diag, double* __restrict__ x,
                                                             float* __restrict__ J32, CgState* st, double* partials) {
    double bb = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const double bi = i < n ? b[i] : 0.0;
        const double di = i < n ? diag[i] : 1.0;
        x[i] = 0.0;
        J32[i] = (float)(1.0 / di);
        bb = fma(bi, bi, bb);
    }
    double v[1] = {bb};
    block_sum<kMxThreads, 1, double>(v);
    double fin[1];
    if (grid_sum_last<1>(v, partials, &st->counters[1], fin) && threadIdx.x == 0) {
        st->bb = fin[0];
        st->tols = fin[0] * st->tol * st->tol;
        st->done = 0;
        st->outer = 0;
        st->innerK = 0;
        st->k = 0;
        st->status &= ~(kStatusBreakdown | kStatusWaitTimeout);
        st->vecSize = (uint32_t)n4;
    }
}

// One warp.  Decides whether another refinement sweep runs.
__global__ void ir_check_kernel(CgState* st, CgState* in, uint64_t outerHandle, uint32_t maxOuter) {
    if (threadIdx.x != 0) return;
    const double rr = st->rrTrue;
    bool cont = !(rr <= st->tols);
    if (!isfinite(rr)) {
        st->status |= kStatusBreakdown;
        cont = false;
    }
    if (st->innerK >= st->maxIterP1 - 1u || st->outer >= maxOuter) cont = false;
    if ((st->status | in->status) & kStatusWaitTimeout) {
        st->status |= kStatusWaitTimeout;
        cont = false;
    }
    st->rr = rr;
    st->scale = rr > 0.0 ? 1.0 / sqrt(rr) : 1.0;
    st->done = cont ? 0u : 1u;
    in->done = 1u;
    if (st->useCond) cudaGraphSetConditional((cudaGraphConditionalHandle)outerHandle, cont ? 1u : 0u);
}

__global__ void __launch_bounds__(kMxThreads) ir_inner_init_kernel(int n4, const double* __restrict__ r64,
                                                                   const float* __restrict__ J32,
                                                                   float* __restrict__ r32, float* __restrict__ p32,
                                                                   float* __restrict__ d32, CgState* st, CgState* in,
                                                                   double* partials, uint64_t innerHandle,
                                                                   double innerTol) {
    if (*(volatile uint32_t*)&st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0 && st->useCond)
            cudaGraphSetConditional((cudaGraphConditionalHandle)innerHandle, 0u);
        return;
    }
    const double s = st->scale;
    float rr = 0.f, rz = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const float ri = (float)(r64[i] * s);
        const float zi = J32[i] * ri;
        r32[i] = ri;
        p32[i] = zi;
        d32[i] = 0.f;
        rr = fmaf(ri, ri, rr);
        rz = fmaf(ri, zi, rz);
    }
    float v[2] = {rr, rz};
    block_sum<kMxThreads, 2, float>(v);
    double tot[2] = {(double)v[0], (double)v[1]}, fin[2];
    if (grid_sum_last<2>(tot, partials, &in->counters[1], fin) && threadIdx.x == 0) {
        in->rr = fin[0];
        in->rz = fin[1];
        in->tols = fin[0] * innerTol * innerTol;
        in->k = 0;
        in->xTag = 0;
        const uint32_t used = st->innerK;
        const uint32_t budget = st->maxIterP1 - 1u;  // user maxIter
        in->maxIterP1 = budget > used ? budget - used : 1u;
        in->done = 0;
        if (st->useCond) cudaGraphSetConditional((cudaGraphConditionalHandle)innerHandle, 1u);
    }
}

__global__ void __launch_bounds__(kMxThreads) cg32_update_kernel(int n4, float* __restrict__ r,
                                                                 const float* __restrict__ Ap,
                                                                 const float* __restrict__ J, CgState* in,
                                                                 double* partials, uint64_t innerHandle, int useCond) {
    if (*(volatile uint32_t*)&in->done) {
        // Only reachable after the fp32 SpMV gave up on a wait: close the loop.
        if (blockIdx.x == 0 && threadIdx.x == 0 && useCond)
            cudaGraphSetConditional((cudaGraphConditionalHandle)innerHandle, 0u);
        return;
    }
    const double alphaD = in->alpha;
    const float alpha = (float)alphaD;
    float rr = 0.f, rz = 0.f;
    const int n4q = n4 >> 2;
    float4* r4 = reinterpret_cast<float4*>(r);
    const float4* a4 = reinterpret_cast<const float4*>(Ap);
    const float4* j4 = reinterpret_cast<const float4*>(J);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4q; i += gridDim.x * blockDim.x) {
        float4 rv = r4[i];
        const float4 av = __ldcs(&a4[i]), jv = j4[i];
        rv.x = fmaf(-alpha, av.x, rv.x);
        rv.y = fmaf(-alpha, av.y, rv.y);
        rv.z = fmaf(-alpha, av.z, rv.z);
        rv.w = fmaf(-alpha, av.w, rv.w);
        rr = fmaf(rv.x, rv.x, rr);
        rr = fmaf(rv.y, rv.y, rr);
        rr = fmaf(rv.z, rv.z, rr);
        rr = fmaf(rv.w, rv.w, rr);
        rz = fmaf(rv.x, rv.x * jv.x, rz);
        rz = fmaf(rv.y, rv.y * jv.y, rz);
        rz = fmaf(rv.z, rv.z * jv.z, rz);
        rz = fmaf(rv.w, rv.w * jv.w, rz);
        r4[i] = rv;
    }
    float v[2] = {rr, rz};
    block_sum<kMxThreads, 2, float>(v);
    double tot[2] = {(double)v[0], (double)v[1]}, fin[2];
    if (grid_sum_last<2>(tot, partials, &in->counters[2], fin) && threadIdx.x == 0) {
        const double rrN = fin[0], rzN = fin[1];
        const double beta = rzN / in->rz;
        in->rr = rrN;
        in->rz = rzN;
        in->beta = beta;
        uint32_t k = in->k + 1u;
        bool cont = !(rrN < in->tols) && (k < in->maxIterP1);
        if (!isfinite(alphaD) || !isfinite(beta) || !isfinite(rrN)) cont = false;
        in->k = k;
        in->done = cont ? 0u : 1u;
        if (useCond) cudaGraphSetConditional((cudaGraphConditionalHandle)innerHandle, cont ? 1u : 0u);
    }
}

// d += alpha p (moved here from the update kernel, where p is not otherwise
// read), then p = J r + beta p unless the inner loop just stopped; the
// iteration tag keeps the d update from being applied twice.
__global__ void __launch_bounds__(kMxThreads) cg32_pupdate_kernel(int n4, float* __restrict__ d, float* __restrict__ p,
                                                                  const float* __restrict__ r,
                                                                  const float* __restrict__ J, CgState* in) {
    const uint32_t k = *(volatile uint32_t*)&in->k;
    if (*(volatile uint32_t*)&in->xTag == k) return;
    const bool last = *(volatile uint32_t*)&in->done != 0u;
    const float alpha = (float)in->alpha;
    const float beta = (float)in->beta;
    const int n4q = n4 >> 2;
    float4* d4 = reinterpret_cast<float4*>(d);
    float4* p4 = reinterpret_cast<float4*>(p);
    const float4* r4 = reinterpret_cast<const float4*>(r);
    const float4* j4 = reinterpret_cast<const float4*>(J);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4q; i += gridDim.x * blockDim.x) {
        float4 dv = d4[i], pv = p4[i];
        dv.x = fmaf(alpha, pv.x, dv.x);
        dv.y = fmaf(alpha, pv.y, dv.y);
        dv.z = fmaf(alpha, pv.z, dv.z);
        dv.w = fmaf(alpha, pv.w, dv.w);
        d4[i] = dv;
        if (!last) {
            const float4 rv = r4[i], jv = j4[i];
            pv.x = fmaf(beta, pv.x, rv.x * jv.x);
            pv.y = fmaf(beta, pv.y, rv.y * jv.y);
            pv.z = fmaf(beta, pv.z, rv.z * jv.z);
            pv.w = fmaf(beta, pv.w, rv.w * jv.w);
            p4[i] = pv;
        }
    }
    __shared__ bool amLast;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        amLast = atomicAdd(&in->counters[3], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (amLast && threadIdx.x == 0) {
        in->counters[3] = 0u;
        in->xTag = k;
    }
}

__global__ void __launch_bounds__(kMxThreads) ir_update_kernel(int n4, double* __restrict__ x,
                                                               const float* __restrict__ d, CgState* st,
                                                               const CgState* in) {
    if (*(volatile uint32_t*)&st->done) return;
    const double inv = 1.0 / st->scale;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x)
        x[i] = fma((double)d[i], inv, x[i]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->innerK += in->k;
        st->outer += 1u;
        st->k = st->innerK;
    }
}

// ---- launchers ----
cudaError_t ir_init_launch(int grid, cudaStream_t s, int n, int n4, const double* b, const double* diag, double* x,
                           float* J32, CgState* st, double* partials) {
    ir_init_kernel<<<grid, kMxThreads, 0, s>>>(n, n4, b, diag, x, J32, st, partials);
    return cudaGetLastError();
}
cudaError_t ir_check_launch(cudaStream_t s, CgState* st, CgState* in, uint64_t outerHandle, uint32_t maxOuter) {
    ir_check_kernel<<<1, 32, 0, s>>>(st, in, outerHandle, maxOuter);
    return cudaGetLastError();
}
cudaError_t ir_inner_init_launch(int grid, cudaStream_t s, int n4, const double* r64, const float* J32, float* r32,
                                 float* p32, float* d32, CgState* st, CgState* in, double* partials,
                                 uint64_t innerHandle, double innerTol) {
    ir_inner_init_kernel<<<grid, kMxThreads, 0, s>>>(n4, r64, J32, r32, p32, d32, st, in, partials, innerHandle,
                                                      innerTol);
    return cudaGetLastError();
}
cudaError_t cg32_update_launch(int grid, cudaStream_t s, int n4, float* r, const float* Ap, const float* J,
                               CgState* in, double* partials, uint64_t innerHandle, int useCond) {
    cg32_update_kernel<<<grid, kMxThreads, 0, s>>>(n4, r, Ap, J, in, partials, innerHandle, useCond);
    return cudaGetLastError();
}
cudaError_t cg32_pupdate_launch(int grid, cudaStream_t s, int n4, float* d, float* p, const float* r, const float* J,
                                CgState* in) {
    cg32_pupdate_kernel<<<grid, kMxThreads, 0, s>>>(n4, d, p, r, J, in);
    return cudaGetLastError();
}
cudaError_t ir_update_launch(int grid, cudaStream_t s, int n4, double* x, const float* d, CgState* st,
                             const CgState* in) {
    ir_update_kernel<<<grid, kMxThreads, 0, s>>>(n4, x, d, st, in);
    return cudaGetLastError();
}

}  // namespace xjpcg
