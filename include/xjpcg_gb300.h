/*
 * xjpcg_gb300.h -- additional entry points of the GB300 xJPCG library.
 *
 * These symbols are new; the reference has no counterpart for most of them
 * (its FPGA runtime offers only the pcg.h API and the SpMV host classes).
 * Where one does correspond to a reference interface, its comment cites it.
 * All take the handle created by xJPCG_createHandle, return XJPCG_Status_t
 * and record status and message on the handle like the pcg.h calls.
 * Pointers are host pointers unless a parameter name starts with d_.
 */
#ifndef XJPCG_GB300_H
#define XJPCG_GB300_H

#include "pcg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Diagnostics of the last matrix set-up and solve on a handle. */
typedef struct {
    uint32_t n;            /* rows of the stored matrix */
    uint32_t n4;           /* n rounded up to a multiple of 4 (record VecSize) */
    uint64_t nnz;          /* stored entries (full matrix, duplicates kept) */
    uint32_t itersRun;     /* iterations the device executed (K) */
    uint32_t spmvLanes;    /* lanes per row chosen by the SpMV tuner */
    uint32_t spmvGrid;     /* CTAs of the SpMV launch */
    uint32_t statusBits;   /* device status word of the last solve */
    uint32_t outerSweeps;  /* mixed precision: refinement sweeps */
    uint32_t innerIters;   /* mixed precision: FP32 inner iterations, summed */
    double bb;             /* b.b of the last solve */
    double rrLast;         /* recursive r.r after the last iteration */
    double solveMs;        /* device time of the last solve (CUDA events) */
    uint32_t loopMode;     /* 1 = conditional-graph loop, 0 = host-driven */
    uint32_t spmvLayout;   /* 0 = CSR staged through shared memory, 1 = sliced (SELL-32) */
} XJPCG_GbInfo_t;

/* CSR input (0- or 1-based per the mode's index nibble), same contract as
 * xJPCG_cooSolver otherwise.  The row pointer and column arrays are int32.
 * New symbol; pcg.h:178-215 is the COO form it parallels. */
XJPCG_Status_t xJPCG_gbCsrSolver(XJPCG_Handle_t* handle, uint32_t n, uint32_t nnz, const int32_t* rowPtr,
                                 const int32_t* colIdx, const double* data, const double* diagA, const double* b,
                                 double* x, uint32_t maxIter, double tol, uint32_t* iter, double* res,
                                 XJPCG_Mode_t mode);

/* Solve with the handle's stored matrix, b / diag / x in device memory.
 * Same stop rule, counters and status as xJPCG_cooSolver in KEEP_MATRIX
 * mode, without host copies of the vectors. */
XJPCG_Status_t xJPCG_gbSolveDevice(XJPCG_Handle_t* handle, const double* d_b, const double* d_diagA, double* d_x,
                                   uint32_t maxIter, double tol, uint32_t* iter, double* res);

/* Mixed precision solve with the stored matrix: FP32 Jacobi-PCG inner loop
 * (FP32 values, vectors and accumulation) inside an FP64 iterative
 * refinement loop that recomputes r = b - A x in FP64 and updates x in FP64.
 * Stops when ||b - A x|| <= tol ||b|| (true residual) or after maxIter inner
 * iterations in total.  *iter = inner iterations, *res = final true relative
 * residual.  onDevice != 0: b, diagA and x are device pointers. */
XJPCG_Status_t xJPCG_gbMixedSolve(XJPCG_Handle_t* handle, const double* b, const double* diagA, double* x,
                                  uint32_t maxIter, double tol, uint32_t* iter, double* res, int onDevice);

/* y = A x with the stored matrix.  onDevice != 0: x and y are device
 * pointers (no host copies). */
XJPCG_Status_t xJPCG_gbSpmv(XJPCG_Handle_t* handle, const double* x, double* y, int onDevice);

/* Copies the stored CSR out: rowPtr[n+1], colIdx[nnz], values[nnz] and
 * perm[nnz] (input position of each CSR entry).  Any pointer may be NULL. */
XJPCG_Status_t xJPCG_gbGetCsr(XJPCG_Handle_t* handle, int32_t* rowPtr, int32_t* colIdx, double* values,
                              uint32_t* perm);

/* Copies up to cap 64-byte iteration records of the last solve into buf
 * (slot 0 = command, slot k+1 = iteration k; layout of the reference's
 * CGSolverInstr image, pcg/hw/include/impl/cgInstr.hpp:117-132).  *count =
 * slots written. */
XJPCG_Status_t xJPCG_gbGetRecords(XJPCG_Handle_t* handle, void* buf, uint64_t cap, uint64_t* count);

XJPCG_Status_t xJPCG_gbGetInfo(const XJPCG_Handle_t* handle, XJPCG_GbInfo_t* info);

/* SpMV tuner report of the stored matrix: for each kernel configuration c
 * (c < *count), ms[c] = median time of a plain SpMV (-1 if not timed) and
 * shape[4c..4c+3] = lanes per row, consumer threads per CTA, chunk entries,
 * pipeline stages.  At most cap configurations are written. */
XJPCG_Status_t xJPCG_gbGetSpmvTuning(const XJPCG_Handle_t* handle, float* ms, int32_t* shape, int32_t cap,
                                     int32_t* count);

/* The cudaStream_t the handle launches on (for event timing by callers). */
XJPCG_Status_t xJPCG_gbGetStream(const XJPCG_Handle_t* handle, void** stream);

/* Forces the CSR SpMV lanes-per-row (1, 2, 4, 8, 16, 32); -1 forces the
 * sliced layout; 0 restores tuning. */
XJPCG_Status_t xJPCG_gbSetSpmvLanes(XJPCG_Handle_t* handle, int lanes);

#ifdef __cplusplus
}
#endif

#endif /* XJPCG_GB300_H */
