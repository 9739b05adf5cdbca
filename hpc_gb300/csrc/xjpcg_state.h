// xjpcg_state.h -- plain structs shared by host and device code: the
// per-solve device state and the 64-byte iteration record.
#pragma once
#include <cstdint>

namespace xjpcg {

// Status bits written by kernels into CgState::status.
enum : uint32_t {
    kStatusBreakdown = 1u,    // alpha, beta or r.r became non-finite
    kStatusWaitTimeout = 2u,  // an mbarrier wait ran out of its time budget
    kStatusIndexError = 4u,   // a matrix index was outside [0, n)
    kStatusCountError = 8u,   // symmetric expansion produced the wrong count
};

// One 64-byte iteration record, laid out like the reference's CGSolverInstr
// memory image (pcg/hw/include/impl/cgInstr.hpp:117-132):
// u32 ID, Iter, VecSize, MaxIter; f64 Tols, Res, RZ, Alpha, Beta; u64 Clock.
struct alignas(8) IterRecord {
    uint32_t id, iter, vecSize, maxIter;
    double tols, res, rz, alpha, beta;
    uint64_t clock;
};
static_assert(sizeof(IterRecord) == 64, "record must be 64 bytes");

// Per-solve state in device memory.  The host writes the command fields
// (tol, maxIterP1, records, recCap) before each graph launch; the kernels
// own the rest.  Reductions use counters[] for the last-block-done pattern.
struct alignas(16) CgState {
    double rz, pAp, alpha, beta, rr, bb, tols, tol;
    double rrTrue;                 // mixed precision: true residual norm^2
    double scale;                  // mixed precision: inner rhs scale
    uint32_t k;                    // iterations run so far (K)
    uint32_t maxIterP1;            // MaxIter of the record: user maxIter + 1
    uint32_t done;                 // 1 once the loop must stop
    uint32_t status;               // kStatus* bits
    uint32_t vecSize;              // n rounded up to a multiple of 4
    uint32_t recCap;               // slots in records[]
    uint32_t counters[6];          // last-block-done tickets
    IterRecord* records;           // slot 0 = command, slot k+1 = iteration k
    uint64_t condHandle;           // cudaGraphConditionalHandle of the loop
    uint32_t useCond;              // 1 when running under a conditional node
    uint32_t outer;                // mixed precision: reliable updates (true-residual refreshes)
    uint32_t innerK;               // mixed precision: FP32 iterations
    uint32_t reliable;             // mixed precision: this iteration refreshes the residual
    double rrMax;                  // mixed precision: largest r.r since the last refresh
    double delta2;                 // mixed precision: refresh when r.r < delta2 * rrMax
    uint64_t relHandle;            // mixed precision: conditional handle of the inner FP32 loop (0: a refresh is due)
    uint32_t skipRefresh;          // mixed precision: 1 = the refresh kernels of this iteration return at once
    uint32_t xSkip;                // fp64: 1 = the update kernel found the loop done (no x update due)
    uint32_t pupdateDue;           // reference-order loop: 1 = this iteration's p update is due
    uint32_t fusedCont;            // fused update: 1 = the loop goes on (the p update is due)
    double fusedBeta;              // fused update: beta, published at its grid barrier
    uint32_t pDone;                // mixed precision: 1 = the fused update already updated p this iteration
};

}  // namespace xjpcg
