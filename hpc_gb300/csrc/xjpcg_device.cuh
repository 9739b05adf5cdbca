// xjpcg_device.cuh -- device-side building blocks shared by the xJPCG kernels:
// the per-handle solver state, deterministic block/grid reductions, and the
// mbarrier + cp.async.bulk primitives (inline PTX, sm_103a) with bounded waits.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "xjpcg_state.h"

namespace xjpcg {

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------
// Deterministic reductions.  Every sum below has a fixed association order for
// a fixed launch shape, so results are bitwise stable run to run.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of NV values per thread; result valid in thread 0.
//
// FP64 adds are scarce on this part (about two per clock per SM), so the sum
// is not a shuffle tree in every warp (five add instructions per value in
// each of the NT/32 warps).  Every thread stores its value; warp 0 alone adds
// them, lane l taking l, l + 32, l + 64, ... in that order, and finishes with
// one shuffle tree: NT/32 + 4 add instructions per value for the whole block.
// The order is fixed, so results are bitwise stable run to run.
template <int NT, int NV, typename T>
__device__ __forceinline__ void block_sum(T (&v)[NV]) {
    __shared__ T part[NV][NT];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) part[i][threadIdx.x] = v[i];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            T s = part[i][lane];
#pragma unroll 8
            for (int w = 1; w < NT / 32; ++w) s += part[i][w * 32 + lane];
            v[i] = warp_sum(s);
        }
    }
    __syncthreads();
}

// block_sum with the totals returned in every thread.
template <int NT, int NV, typename T>
__device__ __forceinline__ void block_allsum(T (&v)[NV]) {
    __shared__ T part[NV][NT];
    __shared__ T tot[NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) part[i][threadIdx.x] = v[i];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            T s = part[i][lane];
#pragma unroll 8
            for (int w = 1; w < NT / 32; ++w) s += part[i][w * 32 + lane];
            s = warp_sum(s);
            if (lane == 0) tot[i] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = tot[i];
    // the next call's writes to part and tot follow its own first barrier,
    // which every thread reaches only after this read
}

// Last-block-done grid reduction of NV doubles.  Each block (NT threads)
// calls it once with its block total in thread 0.  Returns true in the block
// that finished last; in that block, out[] holds the grid totals (valid in
// all threads).  The last block adds the partials with all its threads
// (thread t takes t, t + NT, ... in order, so every load is in flight at
// once), then block_sum's fixed order.  The partial buffer must hold
// NV * gridDim.x doubles.
template <int NT, int NV>
__device__ __forceinline__ bool grid_sum_last(const double (&blockTotal)[NV], double* partials,
                                              uint32_t* counter, double (&out)[NV]) {
    __shared__ bool amLast;
    __shared__ double fin[NV];
    const int nb = gridDim.x;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[i * nb + blockIdx.x] = blockTotal[i];
        __threadfence();
        uint32_t ticket = atomicAdd(counter, 1u);
        amLast = (ticket == (uint32_t)nb - 1);
    }
    __syncthreads();
    if (!amLast) return false;
    __threadfence();
    double s[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double a = 0.0;
#pragma unroll 4
        for (int b = threadIdx.x; b < nb; b += NT) a += __ldcg(&partials[i * nb + b]);
        s[i] = a;
    }
    block_sum<NT, NV, double>(s);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) fin[i] = s[i];
        *counter = 0u;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) out[i] = fin[i];
    return true;
}

// ---------------------------------------------------------------------------
// mbarrier and bulk-copy primitives (PTX ISA 8.x, sm_90 and later).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the given phase parity.  Gives up after budgetNs of wall time and
// returns false; the caller records kStatusWaitTimeout and winds down.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t budgetNs) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t spin = 0;; ++spin) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((spin & 255u) == 255u && globaltimer_ns() - t0 > budgetNs) return false;
    }
}

__device__ __forceinline__ uint64_t l2_policy_evict_first() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ uint64_t l2_policy_evict_last() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// Streaming value load (evict-first) that asks L2 to fetch the whole 256-byte
// block: a warp reads a SELL-32 slice's columns in order, 128 B (FP32) or
// 256 B (FP64) each, so the next column's line is the neighbour.  The 160^3
// mixed solve took 74.4 ms with it against 74.8 ms with plain streaming loads.
template <typename T>
__device__ __forceinline__ T ld_val(const T* p) {
    T v;
    if (sizeof(T) == 8) {
        double d;
        asm("ld.global.cs.L2::256B.f64 %0, [%1];" : "=d"(d) : "l"(p));
        v = (T)d;
    } else {
        float f;
        asm("ld.global.cs.L2::256B.f32 %0, [%1];" : "=f"(f) : "l"(p));
        v = (T)f;
    }
    return v;
}

// 16-byte global load / store with an L2 cache policy from createpolicy.
__device__ __forceinline__ double2 ld2_policy(const double2* p, uint64_t pol) {
    double2 v;
    asm volatile("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ void st2_policy(double2* p, double2 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(p), "d"(v.x), "d"(v.y), "l"(pol)
                 : "memory");
}

// Grid-wide sum of NV doubles fused with a grid barrier, for a cooperative
// launch (every CTA resident).  Each CTA passes its block total (thread 0);
// the last CTA to arrive adds all CTAs' totals in index order (its threads
// take t, t + NT, ... then block_sum's fixed order) and calls fin(sums) in
// its thread 0 -- the one place where the grid's totals exist, so whatever
// follows from them is computed once -- then releases the others.  Writes
// made by fin are visible to every CTA after the barrier.  A wait longer
// than budgetNs of %globaltimer gives up and returns false.  count must be 0
// before the launch; partials holds NV * gridDim.x doubles.
// The same, with the last CTA's thread 0 calling after() once it has released
// the others: work that no other CTA waits for (a record, a graph condition)
// then stays off the barrier's critical path.
template <int NT, int NV, typename Fin, typename After>
__device__ __forceinline__ bool grid_sum_barrier(const double (&blockTotal)[NV], double* partials, uint32_t* count,
                                                 uint32_t* gen, Fin fin, After after, uint64_t budgetNs) {
    __shared__ bool amLast, ok;
    __shared__ uint32_t genSeen;
    const int nb = gridDim.x;
    if (threadIdx.x == 0) {
        ok = true;
        genSeen = *(volatile uint32_t*)gen;
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[i * nb + blockIdx.x] = blockTotal[i];
        __threadfence();
        amLast = atomicAdd(count, 1u) == (uint32_t)nb - 1u;
    }
    __syncthreads();
    if (amLast) {
        __threadfence();
        double s[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double a = 0.0;
            for (int b = threadIdx.x; b < nb; b += NT) a += __ldcg(&partials[i * nb + b]);
            s[i] = a;
        }
        block_sum<NT, NV, double>(s);
        if (threadIdx.x == 0) {
            fin(s);
            *(volatile uint32_t*)count = 0u;
            __threadfence();
            atomicAdd(gen, 1u);
            after();
        }
    } else if (threadIdx.x == 0) {
        const uint64_t t0 = globaltimer_ns();
        while (*(volatile uint32_t*)gen == genSeen) {
            if (globaltimer_ns() - t0 > budgetNs) {
                ok = false;
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
    }
    __syncthreads();
    return ok;
}

template <int NT, int NV, typename Fin>
__device__ __forceinline__ bool grid_sum_barrier(const double (&blockTotal)[NV], double* partials, uint32_t* count,
                                                 uint32_t* gen, Fin fin, uint64_t budgetNs) {
    __shared__ bool amLast, ok;
    __shared__ uint32_t genSeen;
    const int nb = gridDim.x;
    if (threadIdx.x == 0) {
        ok = true;
        genSeen = *(volatile uint32_t*)gen;
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[i * nb + blockIdx.x] = blockTotal[i];
        __threadfence();
        amLast = atomicAdd(count, 1u) == (uint32_t)nb - 1u;
    }
    __syncthreads();
    if (amLast) {
        __threadfence();
        double s[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double a = 0.0;
            for (int b = threadIdx.x; b < nb; b += NT) a += __ldcg(&partials[i * nb + b]);
            s[i] = a;
        }
        block_sum<NT, NV, double>(s);
        if (threadIdx.x == 0) {
            fin(s);
            *(volatile uint32_t*)count = 0u;
            __threadfence();
            atomicAdd(gen, 1u);
        }
    } else if (threadIdx.x == 0) {
        const uint64_t t0 = globaltimer_ns();
        while (*(volatile uint32_t*)gen == genSeen) {
            if (globaltimer_ns() - t0 > budgetNs) {
                ok = false;
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
    }
    __syncthreads();
    return ok;
}

// 1-D bulk copy global -> shared, completing on the mbarrier's transaction
// count.  dst, src and bytes must all be multiples of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar, uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
        : "memory");
}

}  // namespace xjpcg
