// cg_kernels.cu -- the vector kernels of the fp64 Jacobi-PCG iteration.
//
// Per iteration the loop runs three launches (captured once in a CUDA graph,
// inside a conditional WHILE node):
//   1. SpMV + p.Ap + alpha            (spmv_kernels.cu, mode kCgDot)
//   2. cg_update_kernel: r -= alpha Ap, z = J r (written over the spent Ap),
//      r.r and r.z reduced over the grid; the last CTA forms beta, writes the
//      64-byte iteration record, applies the stop rule and sets the loop's
//      condition.  This fuses the reference's krnl_update_xk (L1/hpc/include/
//      hw/cgSolver/update_xk.hpp:26-67), krnl_update_rk_jacobi
//      (update_rk_jacobi.hpp:29-110) and krnl_control (pcg/hw/include/
//      control.hpp:65-92, tasks.hpp:43-47).
//   3. cg_pupdate_kernel: x += alpha p (update_xk.hpp:26-67), then
//      p = z + beta p with the z the update kernel left (update_pk.hpp:26-72).
//      x is updated here rather than in the update kernel so that x and p
//      are read once per iteration; with z stored, an iteration streams 80 n
//      bytes of vectors (update 40 n, p kernel 40 n) instead of 88 n.
// The vector init kernel restates GenCgVector::init (pcg/sw/include/impl/
// cgVector.hpp:101-114) and the instruction slot 0 (cgVector.hpp:149-159).
// Reductions are fixed-order (per-CTA tree, then the last CTA sums the CTA
// partials in index order), so a solve is bitwise reproducible.
#include <algorithm>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

constexpr int kVecThreads = 256;

__device__ __forceinline__ void write_record(CgState* s, uint32_t k, double rr, double rz, double alpha,
                                             double beta) {
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

__global__ void __launch_bounds__(kVecThreads) cg_init_kernel(int n, int n4, const double* __restrict__ b,
                                                              const double* __restrict__ diag, double* __restrict__ x,
                                                              double* __restrict__ r, double* __restrict__ p,
                                                              double* __restrict__ J, double* __restrict__ Ap,
                                                              CgState* state, double* partials) {
    double bb = 0.0, rz = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const double bi = i < n ? b[i] : 0.0;
        const double di = i < n ? diag[i] : 1.0;
        const double ji = 1.0 / di;
        const double zi = ji * bi;
        r[i] = bi;
        J[i] = ji;
        p[i] = zi;
        x[i] = 0.0;
        Ap[i] = 0.0;
        bb = fma(bi, bi, bb);
        rz = fma(bi, zi, rz);
    }
    double v[2] = {bb, rz};
    block_sum<kVecThreads, 2, double>(v);
    double fin[2];
    if (grid_sum_last<kVecThreads, 2>(v, partials, &state->counters[1], fin) && threadIdx.x == 0) {
        CgState* s = state;
        s->bb = fin[0];
        s->rz = fin[1];
        s->rr = fin[0];
        s->tols = fin[0] * s->tol * s->tol;
        s->k = 0;
        s->done = 0;
        s->counters[3] = 0u;  // the fused kernel's grid barrier
        s->status &= ~(kStatusBreakdown | kStatusWaitTimeout);
        s->vecSize = (uint32_t)n4;
        if (s->records && s->recCap > 0) {
            IterRecord rec = {};
            rec.maxIter = s->maxIterP1;
            rec.vecSize = (uint32_t)n4;
            rec.tols = s->tols;
            rec.res = fin[0];
            rec.rz = fin[1];
            rec.clock = globaltimer_ns();
            s->records[0] = rec;
        }
    }
}

__global__ void __launch_bounds__(kVecThreads, 5) cg_update_kernel(int n4, double* __restrict__ r,
                                                                   double* __restrict__ Ap,
                                                                   const double* __restrict__ J, CgState* state,
                                                                   double* partials) {
    if (*(volatile uint32_t*)&state->done) {
        // The loop is over (a host-driven batch past convergence, or an
        // earlier kernel of this iteration gave up on a wait): no x update is
        // due, and the graph's loop is closed so it cannot spin.
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            state->xSkip = 1u;
            if (state->useCond) cudaGraphSetConditional((cudaGraphConditionalHandle)state->condHandle, 0u);
        }
        return;
    }
    const double alpha = state->alpha;
    double rr = 0.0, rz = 0.0;
    const int n2 = n4 >> 1;
    double2* r2 = reinterpret_cast<double2*>(r);
    double2* a2 = reinterpret_cast<double2*>(Ap);
    const double2* j2 = reinterpret_cast<const double2*>(J);
    // Two elements per step, all six loads issued before any arithmetic.
    const int stride = gridDim.x * blockDim.x;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + stride < n2; i += 2 * stride) {
        double2 rv[2], av[2], jv[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int e = i + u * stride;
            rv[u] = r2[e];
            av[u] = __ldcs(&a2[e]);
            jv[u] = j2[e];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            rv[u].x = fma(-alpha, av[u].x, rv[u].x);
            rv[u].y = fma(-alpha, av[u].y, rv[u].y);
            const double z0 = rv[u].x * jv[u].x, z1 = rv[u].y * jv[u].y;
            rr = fma(rv[u].x, rv[u].x, rr);
            rr = fma(rv[u].y, rv[u].y, rr);
            rz = fma(rv[u].x, z0, rz);
            rz = fma(rv[u].y, z1, rz);
            r2[i + u * stride] = rv[u];
            a2[i + u * stride] = make_double2(z0, z1);  // Ap is spent: z = J r for the p kernel
        }
    }
    for (; i < n2; i += stride) {
        double2 rv = r2[i];
        const double2 av = __ldcs(&a2[i]), jv = j2[i];
        rv.x = fma(-alpha, av.x, rv.x);
        rv.y = fma(-alpha, av.y, rv.y);
        const double z0 = rv.x * jv.x, z1 = rv.y * jv.y;
        rr = fma(rv.x, rv.x, rr);
        rr = fma(rv.y, rv.y, rr);
        rz = fma(rv.x, z0, rz);
        rz = fma(rv.y, z1, rz);
        r2[i] = rv;
        a2[i] = make_double2(z0, z1);
    }
    double v[2] = {rr, rz};
    block_sum<kVecThreads, 2, double>(v);
    double fin[2];
    if (grid_sum_last<kVecThreads, 2>(v, partials, &state->counters[2], fin) && threadIdx.x == 0) {
        CgState* s = state;
        const double rrN = fin[0], rzN = fin[1];
        const double beta = rzN / s->rz;
        s->rr = rrN;
        s->rz = rzN;
        s->beta = beta;
        uint32_t k = s->k;
        write_record(s, k, rrN, rzN, alpha, beta);
        bool cont = !(rrN < s->tols);
        ++k;
        cont = cont && (k < s->maxIterP1);
        if (!isfinite(alpha) || !isfinite(beta) || !isfinite(rrN)) {
            s->status |= kStatusBreakdown;
            cont = false;
        }
        if (s->status & kStatusWaitTimeout) cont = false;
        s->k = k;
        s->xSkip = 0u;  // this iteration's x += alpha p is due in the p kernel
        s->done = cont ? 0u : 1u;
        if (s->useCond) cudaGraphSetConditional((cudaGraphConditionalHandle)s->condHandle, cont ? 1u : 0u);
    }
}

__global__ void __launch_bounds__(kVecThreads) cg_pupdate_kernel(int n4, double* __restrict__ x,
                                                                 double* __restrict__ p,
                                                                 const double* __restrict__ z, CgState* state) {
    if (*(volatile uint32_t*)&state->xSkip) return;
    const double alpha = state->alpha;
    const double beta = state->beta;
    // On the iteration that stopped the loop only x is updated.
    const bool last = *(volatile uint32_t*)&state->done != 0u;
    const int n2 = n4 >> 1;
    double2* x2 = reinterpret_cast<double2*>(x);
    double2* p2 = reinterpret_cast<double2*>(p);
    const double2* z2 = reinterpret_cast<const double2*>(z);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        double2 pv = p2[i], xv = x2[i];
        xv.x = fma(alpha, pv.x, xv.x);
        xv.y = fma(alpha, pv.y, xv.y);
        x2[i] = xv;
        if (!last) {
            const double2 zv = z2[i];
            pv.x = fma(beta, pv.x, zv.x);
            pv.y = fma(beta, pv.y, zv.y);
            p2[i] = pv;
        }
    }
}

// The update and the p update fused into one cooperative launch.
//   phase A  r' = r - alpha Ap, z = J r', x' = x + alpha p, and the CTA's
//            partial r'.r' and r'.z; r' and x' are written with streaming
//            stores, z over the spent Ap with an L2 evict-last policy, and p
//            is read with that policy, so that both are still in L2 after
//  barrier  a bounded grid barrier (all CTAs are resident: cooperative
//            launch); the last CTA to arrive adds all CTAs' partials in a
//            fixed order, forms beta, writes the record, applies the stop
//            rule and sets the loop's condition, once, and publishes beta
//            and that decision before releasing the others;
//   phase B  p' = z + beta p over the same elements (same thread, same
//            elements as phase A, so no other CTA's writes are read), with p'
//            stored evict-last for the next SpMV's gathers.
// An iteration then streams 64 n bytes of vectors from HBM (phase A reads
// r, Ap, J, x, p and writes r', x'; phase B writes p') instead of 80 n, with
// one launch and no last-CTA reduction tail.  Same arithmetic per element as
// cg_update_kernel + cg_pupdate_kernel; only the order of the r.r / r.z sums
// differs (per CTA, then over CTAs), and it is fixed.
constexpr uint64_t kBarrierBudgetNs = 2000000000ull;  // 2 s

__global__ void __launch_bounds__(kVecThreads) cg_fused_kernel(int n4, double* __restrict__ x,
                                                               double* __restrict__ r, double* __restrict__ p,
                                                               double* __restrict__ Apz,
                                                               const double* __restrict__ J, CgState* state,
                                                               double* partials, int nbSpmv) {
    // Uniform in every CTA: done only changes after the barrier below.
    if (*(volatile uint32_t*)&state->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            state->xSkip = 1u;
            if (state->useCond) cudaGraphSetConditional((cudaGraphConditionalHandle)state->condHandle, 0u);
        }
        return;
    }
    const double rzOld = state->rz;  // the last CTA at the barrier overwrites it
    const uint32_t k0 = state->k;
    const uint64_t keep = l2_policy_evict_last();
    const int n2 = n4 >> 1;
    double2* r2 = reinterpret_cast<double2*>(r);
    double2* x2 = reinterpret_cast<double2*>(x);
    double2* p2 = reinterpret_cast<double2*>(p);
    double2* z2 = reinterpret_cast<double2*>(Apz);
    const double2* j2 = reinterpret_cast<const double2*>(J);
    const int stride = gridDim.x * blockDim.x;
    double rr = 0.0, rz = 0.0;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    // The first element's loads go out before alpha is known.
    const bool have0 = i < n2;
    double2 rv0 = make_double2(0.0, 0.0), av0 = rv0, jv0 = rv0, xv0 = rv0, pv0 = rv0;
    if (have0) {
        rv0 = __ldcs(&r2[i]);
        av0 = __ldcs(&z2[i]);
        jv0 = __ldcs(&j2[i]);
        xv0 = __ldcs(&x2[i]);
        pv0 = ld2_policy(&p2[i], keep);
    }
    double alpha;
    if (nbSpmv > 0) {
        // alpha = rz / p.Ap from the SpMV's per-CTA partials (kSpmvCgPart), in
        // the order grid_sum_last<256, 1> adds them, so every CTA forms the
        // same bits that the SpMV's last CTA would have.
        __shared__ double sAlpha;
        double a = 0.0;
#pragma unroll 4
        for (int b = threadIdx.x; b < nbSpmv; b += kVecThreads) a += __ldcg(&partials[b]);
        double s1[1] = {a};
        block_sum<kVecThreads, 1, double>(s1);
        if (threadIdx.x == 0) {
            const double al = rzOld / s1[0];
            sAlpha = al;
            if (blockIdx.x == 0) {
                state->pAp = s1[0];
                state->alpha = al;
            }
        }
        __syncthreads();
        alpha = sAlpha;
    } else {
        alpha = state->alpha;
    }
    double* bar = partials + kFusedPartialOff;  // clear of the SpMV's partials
    for (bool first = true; i < n2; i += stride, first = false) {
        double2 rv, av, jv, xv, pv;
        if (first) {
            rv = rv0;
            av = av0;
            jv = jv0;
            xv = xv0;
            pv = pv0;
        } else {
            rv = __ldcs(&r2[i]);
            av = __ldcs(&z2[i]);
            jv = __ldcs(&j2[i]);
            xv = __ldcs(&x2[i]);
            pv = ld2_policy(&p2[i], keep);
        }
        rv.x = fma(-alpha, av.x, rv.x);
        rv.y = fma(-alpha, av.y, rv.y);
        const double2 zv = make_double2(rv.x * jv.x, rv.y * jv.y);
        xv.x = fma(alpha, pv.x, xv.x);
        xv.y = fma(alpha, pv.y, xv.y);
        rr = fma(rv.x, rv.x, rr);
        rr = fma(rv.y, rv.y, rr);
        rz = fma(rv.x, zv.x, rz);
        rz = fma(rv.y, zv.y, rz);
        __stcs(&r2[i], rv);
        __stcs(&x2[i], xv);
        st2_policy(&z2[i], zv, keep);
    }
    double v[2] = {rr, rz};
    block_sum<kVecThreads, 2, double>(v);
    // The last CTA at the barrier has the grid's r.r and r.z: it forms beta,
    // writes the record, applies the stop rule (control.hpp:83), sets the
    // loop's condition and publishes beta and the decision for the others.
    // The record and the loop's condition wait for no other CTA: the last CTA
    // writes them after it has released the others.
    double recRr = 0.0, recRz = 0.0, recBeta = 0.0;
    bool recCont = false;
    auto finish = [&](const double (&tot)[2]) {
        CgState* st = state;
        const double rrN = tot[0], rzN = tot[1];
        const double beta = rzN / rzOld;
        bool cont = !(rrN < st->tols) && (k0 + 1u < st->maxIterP1);
        if (!isfinite(alpha) || !isfinite(beta) || !isfinite(rrN)) {
            st->status |= kStatusBreakdown;
            cont = false;
        }
        if (st->status & kStatusWaitTimeout) cont = false;
        st->rr = rrN;
        st->rz = rzN;
        st->beta = beta;
        st->k = k0 + 1u;
        st->xSkip = 0u;
        st->done = cont ? 0u : 1u;
        st->fusedBeta = beta;
        st->fusedCont = cont ? 1u : 0u;
        recRr = rrN;
        recRz = rzN;
        recBeta = beta;
        recCont = cont;
    };
    auto after = [&]() {
        write_record(state, k0, recRr, recRz, alpha, recBeta);
        if (state->useCond) cudaGraphSetConditional((cudaGraphConditionalHandle)state->condHandle, recCont ? 1u : 0u);
    };
    if (!grid_sum_barrier<kVecThreads, 2>(v, bar, &state->counters[3], &state->counters[5], finish, after,
                                          kBarrierBudgetNs)) {
        if (threadIdx.x == 0) {
            atomicOr(&state->status, kStatusWaitTimeout);
            state->done = 1u;
            if (state->useCond) cudaGraphSetConditional((cudaGraphConditionalHandle)state->condHandle, 0u);
        }
        return;
    }
    const double beta = __ldcg(&state->fusedBeta);
    if (__ldcg(&state->fusedCont)) {
        for (i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += stride) {
            const double2 zv = ld2_policy(&z2[i], keep);
            double2 pv = ld2_policy(&p2[i], keep);
            pv.x = fma(beta, pv.x, zv.x);
            pv.y = fma(beta, pv.y, zv.y);
            st2_policy(&p2[i], pv, keep);
        }
    }
}

// Diagnostic of the bounded wait that every mbarrier wait in the library
// uses (mbar_wait_bounded).  One warp initialises an mbarrier that expects
// one arrival and never arrives, so the wait cannot complete: it must give up
// after budgetNs and report kStatusWaitTimeout, as a stalled copy would.  No
// copy is issued, so nothing is in flight when the CTA exits.  out[0] =
// status bits, out[1..2] = the wait's duration in ns.
__global__ void wait_probe_kernel(uint64_t budgetNs, uint32_t* out) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncwarp();
    const uint64_t t0 = globaltimer_ns();
    const bool ok = mbar_wait_bounded(&bar, 0u, budgetNs);
    const uint64_t dt = globaltimer_ns() - t0;
    if (__any_sync(0xffffffffu, !ok) && threadIdx.x == 0) {
        out[0] = kStatusWaitTimeout;
        out[1] = (uint32_t)dt;
        out[2] = (uint32_t)(dt >> 32);
    } else if (threadIdx.x == 0) {
        out[0] = 0u;
        out[1] = (uint32_t)dt;
        out[2] = (uint32_t)(dt >> 32);
    }
}

cudaError_t wait_probe_launch(cudaStream_t st, uint64_t budgetNs, uint32_t* out) {
    wait_probe_kernel<<<1, 32, 0, st>>>(budgetNs, out);
    return cudaGetLastError();
}

// FP64 issue-rate probe: the ceiling every fp64 kernel of the loop is held
// against.  Each thread runs kFp64Chains independent register-resident chains
// a <- fma(a, m, c) for `iters` steps (enough independent chains per warp to
// cover the pipe's latency at full occupancy), so the kernel issues nothing
// but DFMA once its few loads are done.  m < 1 keeps the chains finite; one
// store of their sum per thread keeps the compiler from removing them.
// m and c are computed per thread so that they live in registers, as the
// operands of the library's own FMAs do: a DFMA that reads an operand from
// the constant bank (a kernel parameter) issued at about 5/6 of this rate
// when measured on GB300.
constexpr int kFp64Chains = 8;

__global__ void __launch_bounds__(kVecThreads) fp64_rate_kernel(int iters, double m0, double c0, double* out) {
    const double m = m0 - 1e-12 * (double)(threadIdx.x & 31);
    const double c = c0 * (double)((threadIdx.x & 7) + 1);
    double a[kFp64Chains];
#pragma unroll
    for (int j = 0; j < kFp64Chains; ++j) a[j] = (double)(threadIdx.x + j) * 1e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < kFp64Chains; ++j) a[j] = fma(a[j], m, c);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < kFp64Chains; ++j) s += a[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Full occupancy: 2048 threads per SM.
int fp64_rate_grid(int numSms) { return numSms * (2048 / kVecThreads); }

double fp64_rate_dfma(int grid, int iters) { return (double)grid * kVecThreads * kFp64Chains * (double)iters; }

cudaError_t fp64_rate_launch(cudaStream_t st, int grid, int iters, double* out) {
    fp64_rate_kernel<<<grid, kVecThreads, 0, st>>>(iters, 0.999999, 1e-6, out);
    return cudaGetLastError();
}

// The update kernel holds two elements per step (48 registers): one wave of
// 5 CTAs per SM.
int update_grid(int n4, int numSms) {
    int need = (n4 / 2 + kVecThreads - 1) / kVecThreads;
    int cap = numSms * 5;
    if (need < 1) need = 1;
    return need < cap ? need : cap;
}

int vec_grid(int n4, int numSms) {
    int need = (n4 / 2 + kVecThreads - 1) / kVecThreads;
    int cap = numSms * 8;
    if (need < 1) need = 1;
    return need < cap ? need : cap;
}

cudaError_t cg_init_launch(int grid, cudaStream_t st, int n, int n4, const double* b, const double* diag, double* x,
                           double* r, double* p, double* J, double* Ap, CgState* state, double* partials) {
    cg_init_kernel<<<grid, kVecThreads, 0, st>>>(n, n4, b, diag, x, r, p, J, Ap, state, partials);
    return cudaGetLastError();
}

cudaError_t cg_update_launch(int grid, cudaStream_t st, int n4, double* r, double* Ap, const double* J,
                             CgState* state, double* partials) {
    cg_update_kernel<<<grid, kVecThreads, 0, st>>>(n4, r, Ap, J, state, partials);
    return cudaGetLastError();
}

// At most one CTA per resident slot: the cooperative launch needs them all at once.
int fused_grid(int n4, int numSms) {
    int perSm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, cg_fused_kernel, kVecThreads, 0) != cudaSuccess ||
        perSm < 1) {
        cudaGetLastError();
        perSm = 1;
    }
    // Three CTAs per SM (768 threads, about 18 elements each on 160^3) measured
    // best on 160^3: 0.2699 ms per iteration against 0.2713 - 0.2724 with 4 to
    // 6 and 0.2779 with 2.  Fewer CTAs shorten the barrier and its partial
    // sums.  Below about 1.2 M element pairs two CTAs per SM do better (us per
    // iteration, three against two, with the loop as it is now): 27-point
    // 160^3 265.6 / 274.8, 140^3 185.6 / 186.0, 128^3 151.0 / 145.4, 100^3
    // 80.3 / 79.2; the 885k-row 7-point system 42.4 / 41.8.
    const int n2 = n4 / 2;
    perSm = std::min(perSm, n2 < 1200000 ? 2 : 3);
    const int need = std::max(1, (n4 / 2 + kVecThreads - 1) / kVecThreads);
    return std::min(need, numSms * perSm);
}

cudaError_t cg_fused_launch(int grid, cudaStream_t st, int n4, double* x, double* r, double* p, double* Apz,
                            const double* J, CgState* state, double* partials, int nbSpmv) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kVecThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, cg_fused_kernel, n4, x, r, p, Apz, J, state, partials, nbSpmv);
}

cudaError_t cg_pupdate_launch(int grid, cudaStream_t st, int n4, double* x, double* p, const double* z,
                              CgState* state) {
    cg_pupdate_kernel<<<grid, kVecThreads, 0, st>>>(n4, x, p, z, state);
    return cudaGetLastError();
}

}  // namespace xjpcg
