// mixed_kernels.cu -- mixed-precision Jacobi-PCG with reliable updates.
//
// The CG recurrence runs in FP32: matrix values, r, p, Ap, J and the
// solution increment are FP32 and the per-thread partial sums of p.Ap, r.r
// and r.z are accumulated in FP32 (the CTA totals are combined in FP64).  FP64
// is kept for the true residual r = b - A x (FP64 matrix, FP64 x), for the
// solution x itself (the FP32 increment is folded into it at every refresh)
// and for the alpha / beta scalars.  The refinement is a reliable update
// (van der Vorst and Ye's residual replacement): when the recursive r.r has
// dropped by delta^2 from its largest value since the last refresh, or looks
// converged, or the iteration budget is spent, x += increment in FP64, the
// true residual is recomputed in FP64 and replaces the FP32 r, and the loop
// goes on with the same search direction p.  Keeping p keeps the Krylov
// progress, so the iteration count stays close to the FP64 solver's, whereas
// restarting CG at every refinement sweep would lose it.  The solve stops
// when the true residual meets ||b - A x|| <= tol ||b||.
//
// One CUDA graph per matrix:
//   rel_init                        x = 0, d = 0, J = 1/diag, r = b, p = J r
//   WHILE not done:
//     WHILE no refresh is due (eight iterations per pass):
//       SpMV fp32, kCgDot           Ap = A p, p.Ap, alpha
//       rel_fused                   d += alpha p, r -= alpha Ap, r.r, r.z; at
//                                   its grid barrier the refresh decision
//                                   (ends the inner loop) and beta; then
//                                   p = J r + beta p unless a refresh is due
//                                   (XJPCG_FUSED_UPDATE=0: rel_update, then
//                                   rel_pupdate, which skips when a refresh
//                                   is due)
//     rel_fold                      x += d (FP64), d = 0
//     SpMV fp64, kResidual          r64 = b - A x, ||r64||^2
//     rel_restart                   r = r64, r.z, beta, stop test; clears
//                                   the refresh flag, re-arms the inner loop
//     rel_pupdate                   p = J r + beta p
// The refresh runs a few times per solve, so the FP32 iterations carry no
// conditional node of their own.
// Without graphs (XJPCG_HOST_LOOP=1, for profilers) the host launches the six
// kernels of every iteration in batches; the refresh kernels then return at
// once unless the update kernel chose a refresh (reliable / skipRefresh),
// and every kernel returns once done is set.
#include <algorithm>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

constexpr int kMxThreads = 256;

__global__ void __launch_bounds__(kMxThreads) rel_init_kernel(int n, int n4, const double* __restrict__ b,
                                                              const double* __restrict__ diag, double* __restrict__ x,
                                                              float* __restrict__ d, float* __restrict__ J,
                                                              float* __restrict__ r, float* __restrict__ p,
                                                              CgState* st, double* partials) {
    double bb = 0.0;
    float rz = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const double bi = i < n ? b[i] : 0.0;
        const double di = i < n ? diag[i] : 1.0;
        const float ji = (float)(1.0 / di);
        const float ri = (float)bi;
        const float zi = ji * ri;
        x[i] = 0.0;
        d[i] = 0.f;
        J[i] = ji;
        r[i] = ri;
        p[i] = zi;
        bb = fma(bi, bi, bb);
        rz = fmaf(ri, zi, rz);
    }
    double v[2] = {bb, (double)rz};
    block_sum<kMxThreads, 2, double>(v);
    double fin[2];
    if (grid_sum_last<kMxThreads, 2>(v, partials, &st->counters[1], fin) && threadIdx.x == 0) {
        st->bb = fin[0];
        st->rz = fin[1];
        st->rr = fin[0];
        st->rrMax = fin[0];
        st->rrTrue = fin[0];
        st->tols = fin[0] * st->tol * st->tol;
        st->done = 0;
        st->outer = 0;
        st->innerK = 0;
        st->k = 0;
        st->reliable = 0;
        st->status &= ~(kStatusBreakdown | kStatusWaitTimeout);
        st->vecSize = (uint32_t)n4;
    }
}

__global__ void __launch_bounds__(kMxThreads, 5) rel_update_kernel(int n4, float* __restrict__ d, float* __restrict__ r,
                                                                const float* __restrict__ p,
                                                                const float* __restrict__ Ap,
                                                                const float* __restrict__ J, CgState* st,
                                                                double* partials) {
    if (*(volatile uint32_t*)&st->done) {
        // Reachable only after the SpMV gave up on a wait: close both loops.
        if (blockIdx.x == 0 && threadIdx.x == 0 && st->useCond) {
            cudaGraphSetConditional((cudaGraphConditionalHandle)st->relHandle, 0u);
            cudaGraphSetConditional((cudaGraphConditionalHandle)st->condHandle, 0u);
        }
        return;
    }
    // A refresh is due (an earlier copy of this kernel in the same pass of
    // the inner loop chose it): nothing to do until the refresh has run.
    if (*(volatile uint32_t*)&st->reliable) return;
    const double alphaD = st->alpha;
    const float alpha = (float)alphaD;
    float rr = 0.f, rz = 0.f;
    const int n4q = n4 >> 2;
    float4* d4 = reinterpret_cast<float4*>(d);
    float4* r4 = reinterpret_cast<float4*>(r);
    const float4* p4 = reinterpret_cast<const float4*>(p);
    const float4* a4 = reinterpret_cast<const float4*>(Ap);
    const float4* j4 = reinterpret_cast<const float4*>(J);
    // Two float4 per step, all ten loads issued before any arithmetic.
    const int stride = gridDim.x * blockDim.x;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + stride < n4q; i += 2 * stride) {
        float4 dv[2], rv[2], pv[2], av[2], jv[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int e = i + u * stride;
            dv[u] = d4[e];
            rv[u] = r4[e];
            pv[u] = p4[e];
            av[u] = __ldcs(&a4[e]);
            jv[u] = j4[e];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            dv[u].x = fmaf(alpha, pv[u].x, dv[u].x);
            dv[u].y = fmaf(alpha, pv[u].y, dv[u].y);
            dv[u].z = fmaf(alpha, pv[u].z, dv[u].z);
            dv[u].w = fmaf(alpha, pv[u].w, dv[u].w);
            rv[u].x = fmaf(-alpha, av[u].x, rv[u].x);
            rv[u].y = fmaf(-alpha, av[u].y, rv[u].y);
            rv[u].z = fmaf(-alpha, av[u].z, rv[u].z);
            rv[u].w = fmaf(-alpha, av[u].w, rv[u].w);
            rr = fmaf(rv[u].x, rv[u].x, rr);
            rr = fmaf(rv[u].y, rv[u].y, rr);
            rr = fmaf(rv[u].z, rv[u].z, rr);
            rr = fmaf(rv[u].w, rv[u].w, rr);
            rz = fmaf(rv[u].x, rv[u].x * jv[u].x, rz);
            rz = fmaf(rv[u].y, rv[u].y * jv[u].y, rz);
            rz = fmaf(rv[u].z, rv[u].z * jv[u].z, rz);
            rz = fmaf(rv[u].w, rv[u].w * jv[u].w, rz);
            d4[i + u * stride] = dv[u];
            r4[i + u * stride] = rv[u];
        }
    }
    for (; i < n4q; i += stride) {
        float4 dv = d4[i], rv = r4[i];
        const float4 pv = p4[i], av = __ldcs(&a4[i]), jv = j4[i];
        dv.x = fmaf(alpha, pv.x, dv.x);
        dv.y = fmaf(alpha, pv.y, dv.y);
        dv.z = fmaf(alpha, pv.z, dv.z);
        dv.w = fmaf(alpha, pv.w, dv.w);
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
        d4[i] = dv;
        r4[i] = rv;
    }
    float v[2] = {rr, rz};
    block_sum<kMxThreads, 2, float>(v);
    double tot[2] = {(double)v[0], (double)v[1]}, fin[2];
    if (grid_sum_last<kMxThreads, 2>(tot, partials, &st->counters[2], fin) && threadIdx.x == 0) {
        const double rrN = fin[0], rzN = fin[1];
        const uint32_t k = st->k + 1u;
        st->k = k;
        st->innerK = k;
        st->rr = rrN;
        if (rrN > st->rrMax) st->rrMax = rrN;
        bool bd = !isfinite(alphaD) || !isfinite(rrN) || !isfinite(rzN);
        // Refresh when the recursive residual fell by delta^2, looks converged,
        // or the budget is spent (the last refresh folds x and measures the
        // true residual).
        const bool refresh = bd || rrN < st->delta2 * st->rrMax || rrN < st->tols || k + 1u >= st->maxIterP1;
        st->reliable = refresh ? 1u : 0u;
        st->skipRefresh = refresh ? 0u : 1u;
        if (bd) {
            st->status |= kStatusBreakdown;
        } else if (!refresh) {
            st->beta = rzN / st->rz;
            st->rz = rzN;
        }
        if (st->useCond) cudaGraphSetConditional((cudaGraphConditionalHandle)st->relHandle, refresh ? 0u : 1u);
    }
}

// The FP32 update and the p update in one cooperative launch, the mixed
// loop's form of cg_fused_kernel:
//   phase A  rel_update_kernel's element work (d, r, the r.r and r.z partials);
//   barrier  the last CTA adds the partials in rel_update_kernel's order,
//            decides the refresh and forms beta, once;
//   phase B  when no refresh is due, p = J r + beta p over the same elements
//            (each thread reads only what it wrote in phase A).  A due refresh
//            changes r and beta first: rel_pupdate runs after it instead.
// pDone tells the standalone p update that this iteration's p is done.
constexpr uint64_t kMxBarrierBudgetNs = 2000000000ull;  // 2 s

__global__ void __launch_bounds__(kMxThreads) rel_fused_kernel(int n4, float* __restrict__ d, float* __restrict__ r,
                                                               float* __restrict__ p, const float* __restrict__ Ap,
                                                               const float* __restrict__ J, CgState* st,
                                                               double* partials) {
    if (*(volatile uint32_t*)&st->done) {
        // Reachable only after the SpMV gave up on a wait: close both loops.
        if (blockIdx.x == 0 && threadIdx.x == 0 && st->useCond) {
            cudaGraphSetConditional((cudaGraphConditionalHandle)st->relHandle, 0u);
            cudaGraphSetConditional((cudaGraphConditionalHandle)st->condHandle, 0u);
        }
        return;
    }
    // A refresh is due (an earlier copy of this kernel in the same pass of
    // the inner loop chose it): nothing to do until the refresh has run.
    if (*(volatile uint32_t*)&st->reliable) return;
    const double alphaD = st->alpha;
    const double rzOld = st->rz;  // the last CTA at the barrier overwrites it
    const uint32_t k0 = st->k;
    const float alpha = (float)alphaD;
    float rr = 0.f, rz = 0.f;
    const int n4q = n4 >> 2;
    float4* d4 = reinterpret_cast<float4*>(d);
    float4* r4 = reinterpret_cast<float4*>(r);
    float4* p4 = reinterpret_cast<float4*>(p);
    const float4* a4 = reinterpret_cast<const float4*>(Ap);
    const float4* j4 = reinterpret_cast<const float4*>(J);
    const int stride = gridDim.x * blockDim.x;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    int i = i0;
    for (; i + stride < n4q; i += 2 * stride) {
        float4 dv[2], rv[2], pv[2], av[2], jv[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int e = i + u * stride;
            dv[u] = d4[e];
            rv[u] = r4[e];
            pv[u] = p4[e];
            av[u] = __ldcs(&a4[e]);
            jv[u] = j4[e];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            dv[u].x = fmaf(alpha, pv[u].x, dv[u].x);
            dv[u].y = fmaf(alpha, pv[u].y, dv[u].y);
            dv[u].z = fmaf(alpha, pv[u].z, dv[u].z);
            dv[u].w = fmaf(alpha, pv[u].w, dv[u].w);
            rv[u].x = fmaf(-alpha, av[u].x, rv[u].x);
            rv[u].y = fmaf(-alpha, av[u].y, rv[u].y);
            rv[u].z = fmaf(-alpha, av[u].z, rv[u].z);
            rv[u].w = fmaf(-alpha, av[u].w, rv[u].w);
            rr = fmaf(rv[u].x, rv[u].x, rr);
            rr = fmaf(rv[u].y, rv[u].y, rr);
            rr = fmaf(rv[u].z, rv[u].z, rr);
            rr = fmaf(rv[u].w, rv[u].w, rr);
            rz = fmaf(rv[u].x, rv[u].x * jv[u].x, rz);
            rz = fmaf(rv[u].y, rv[u].y * jv[u].y, rz);
            rz = fmaf(rv[u].z, rv[u].z * jv[u].z, rz);
            rz = fmaf(rv[u].w, rv[u].w * jv[u].w, rz);
            d4[i + u * stride] = dv[u];
            r4[i + u * stride] = rv[u];
        }
    }
    for (; i < n4q; i += stride) {
        float4 dv = d4[i], rv = r4[i];
        const float4 pv = p4[i], av = __ldcs(&a4[i]), jv = j4[i];
        dv.x = fmaf(alpha, pv.x, dv.x);
        dv.y = fmaf(alpha, pv.y, dv.y);
        dv.z = fmaf(alpha, pv.z, dv.z);
        dv.w = fmaf(alpha, pv.w, dv.w);
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
        d4[i] = dv;
        r4[i] = rv;
    }
    float v[2] = {rr, rz};
    block_sum<kMxThreads, 2, float>(v);
    double tot[2] = {(double)v[0], (double)v[1]};
    bool refreshL = false;
    auto finish = [&](const double (&fin)[2]) {
        const double rrN = fin[0], rzN = fin[1];
        const uint32_t k = k0 + 1u;
        st->k = k;
        st->innerK = k;
        st->rr = rrN;
        if (rrN > st->rrMax) st->rrMax = rrN;
        const bool bd = !isfinite(alphaD) || !isfinite(rrN) || !isfinite(rzN);
        // Refresh when the recursive residual fell by delta^2, looks
        // converged, or the budget is spent (the last refresh folds x and
        // measures the true residual).
        const bool refresh = bd || rrN < st->delta2 * st->rrMax || rrN < st->tols || k + 1u >= st->maxIterP1;
        st->reliable = refresh ? 1u : 0u;
        st->skipRefresh = refresh ? 0u : 1u;
        st->pDone = refresh ? 0u : 1u;
        double beta = 0.0;
        if (bd) {
            st->status |= kStatusBreakdown;
        } else if (!refresh) {
            beta = rzN / rzOld;
            st->beta = beta;
            st->rz = rzN;
        }
        st->fusedBeta = beta;
        st->fusedCont = refresh ? 0u : 1u;
        refreshL = refresh;
    };
    auto after = [&]() {
        if (st->useCond) cudaGraphSetConditional((cudaGraphConditionalHandle)st->relHandle, refreshL ? 0u : 1u);
    };
    if (!grid_sum_barrier<kMxThreads, 2>(tot, partials + kFusedPartialOff, &st->counters[2], &st->counters[5], finish,
                                         after, kMxBarrierBudgetNs)) {
        if (threadIdx.x == 0) {
            atomicOr(&st->status, kStatusWaitTimeout);
            st->done = 1u;
            if (st->useCond) {
                cudaGraphSetConditional((cudaGraphConditionalHandle)st->relHandle, 0u);
                cudaGraphSetConditional((cudaGraphConditionalHandle)st->condHandle, 0u);
            }
        }
        return;
    }
    if (__ldcg(&st->fusedCont)) {
        const float beta = (float)__ldcg(&st->fusedBeta);
        for (i = i0; i < n4q; i += stride) {
            float4 pv = p4[i];
            const float4 rv = r4[i], jv = j4[i];
            pv.x = fmaf(beta, pv.x, rv.x * jv.x);
            pv.y = fmaf(beta, pv.y, rv.y * jv.y);
            pv.z = fmaf(beta, pv.z, rv.z * jv.z);
            pv.w = fmaf(beta, pv.w, rv.w * jv.w);
            p4[i] = pv;
        }
    }
}

__global__ void __launch_bounds__(kMxThreads) rel_fold_kernel(int n4, double* __restrict__ x, float* __restrict__ d,
                                                              const CgState* st) {
    if (!*(volatile const uint32_t*)&st->reliable || *(volatile const uint32_t*)&st->done) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        x[i] += (double)d[i];
        d[i] = 0.f;
    }
}

__global__ void __launch_bounds__(kMxThreads) rel_restart_kernel(int n4, const double* __restrict__ r64,
                                                                 const float* __restrict__ J, float* __restrict__ r,
                                                                 CgState* st, double* partials) {
    if (!*(volatile uint32_t*)&st->reliable || *(volatile uint32_t*)&st->done) return;
    float rz = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const float ri = (float)r64[i];
        r[i] = ri;
        rz = fmaf(ri, J[i] * ri, rz);
    }
    double v[1] = {(double)rz};
    block_sum<kMxThreads, 1, double>(v);
    double fin[1];
    if (grid_sum_last<kMxThreads, 1>(v, partials, &st->counters[3], fin) && threadIdx.x == 0) {
        const double rrT = st->rrTrue, rzN = fin[0];
        st->outer += 1u;
        st->rr = rrT;
        st->rrMax = rrT;
        bool stop = !(rrT > st->tols) || st->k + 1u >= st->maxIterP1;
        if (!isfinite(rrT) || !isfinite(rzN) || (st->status & kStatusBreakdown)) {
            st->status |= kStatusBreakdown;
            stop = true;
        }
        if (st->status & kStatusWaitTimeout) stop = true;
        if (!stop) {
            st->beta = rzN / st->rz;
            st->rz = rzN;
        }
        st->done = stop ? 1u : 0u;
        if (stop) st->skipRefresh = 1u;
        st->reliable = 0u;  // the refresh is done: the next p update runs
        if (st->useCond) {
            if (stop) cudaGraphSetConditional((cudaGraphConditionalHandle)st->condHandle, 0u);
            cudaGraphSetConditional((cudaGraphConditionalHandle)st->relHandle, stop ? 0u : 1u);
        }
    }
}

__global__ void __launch_bounds__(kMxThreads) rel_pupdate_kernel(int n4, float* __restrict__ p,
                                                                 const float* __restrict__ r,
                                                                 const float* __restrict__ J, CgState* st) {
    // A due refresh changes r and beta first; the p update after it runs then.
    if (*(volatile uint32_t*)&st->done || *(volatile uint32_t*)&st->reliable || *(volatile uint32_t*)&st->pDone)
        return;
    const float beta = (float)st->beta;
    const int n4q = n4 >> 2;
    float4* p4 = reinterpret_cast<float4*>(p);
    const float4* r4 = reinterpret_cast<const float4*>(r);
    const float4* j4 = reinterpret_cast<const float4*>(J);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4q; i += gridDim.x * blockDim.x) {
        float4 pv = p4[i];
        const float4 rv = r4[i], jv = j4[i];
        pv.x = fmaf(beta, pv.x, rv.x * jv.x);
        pv.y = fmaf(beta, pv.y, rv.y * jv.y);
        pv.z = fmaf(beta, pv.z, rv.z * jv.z);
        pv.w = fmaf(beta, pv.w, rv.w * jv.w);
        p4[i] = pv;
    }
}

// ---- launchers ----
cudaError_t rel_init_launch(int grid, cudaStream_t s, int n, int n4, const double* b, const double* diag, double* x,
                            float* d, float* J, float* r, float* p, CgState* st, double* partials) {
    rel_init_kernel<<<grid, kMxThreads, 0, s>>>(n, n4, b, diag, x, d, J, r, p, st, partials);
    return cudaGetLastError();
}
// At most the CTAs that fit at once (a cooperative launch), capped at three
// per SM as for the fp64 kernel: fewer CTAs meet at the barrier.  160^3 mixed
// solve: 74.6 ms with three or two per SM, 75.2 ms with four (the most that fit).
int rel_fused_grid(int n4, int numSms) {
    int perSm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, rel_fused_kernel, kMxThreads, 0) != cudaSuccess ||
        perSm < 1) {
        cudaGetLastError();
        perSm = 1;
    }
    perSm = std::min(perSm, 3);
    const int need = std::max(1, (n4 / 4 + kMxThreads - 1) / kMxThreads);
    return std::min(need, numSms * perSm);
}

cudaError_t rel_fused_launch(int grid, cudaStream_t s, int n4, float* d, float* r, float* p, const float* Ap,
                             const float* J, CgState* st, double* partials) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kMxThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, rel_fused_kernel, n4, d, r, p, Ap, J, st, partials);
}

cudaError_t rel_update_launch(int grid, cudaStream_t s, int n4, float* d, float* r, const float* p, const float* Ap,
                              const float* J, CgState* st, double* partials) {
    rel_update_kernel<<<grid, kMxThreads, 0, s>>>(n4, d, r, p, Ap, J, st, partials);
    return cudaGetLastError();
}
cudaError_t rel_fold_launch(int grid, cudaStream_t s, int n4, double* x, float* d, const CgState* st) {
    rel_fold_kernel<<<grid, kMxThreads, 0, s>>>(n4, x, d, st);
    return cudaGetLastError();
}
cudaError_t rel_restart_launch(int grid, cudaStream_t s, int n4, const double* r64, const float* J, float* r,
                               CgState* st, double* partials) {
    rel_restart_kernel<<<grid, kMxThreads, 0, s>>>(n4, r64, J, r, st, partials);
    return cudaGetLastError();
}
cudaError_t rel_pupdate_launch(int grid, cudaStream_t s, int n4, float* p, const float* r, const float* J,
                               CgState* st) {
    rel_pupdate_kernel<<<grid, kMxThreads, 0, s>>>(n4, p, r, J, st);
    return cudaGetLastError();
}

}  // namespace xjpcg
