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
    uint32_t spmvLayout;   /* 0 = CSR staged through shared memory, 1 = sliced (SELL-32), 2 = merge path,
                              3 = sliced with int16 column offsets, 4 = sliced with rows sorted by
                              length (long rows one warp each), 5 = sliced with column offsets
                              shared by the 32 rows of a slice */
    uint32_t batchThreads; /* batched solves: CTA size chosen by the tuner */
    uint32_t batchLanes;   /* batched solves: lanes per row */
    uint32_t batchSmemRows;/* batched solves: rows of p held in shared memory */
    uint32_t batchGrid;    /* batched solves: CTAs of the persistent launch */
    double batchMs;        /* batched solves: device time of the last batch (CUDA events) */
    uint32_t spmvCfg;      /* index of the FP64 SpMV configuration in the tuning table */
    uint32_t spmvCfg32;    /* index of the mixed solver's FP32 SpMV configuration (~0 until tuned) */
    uint32_t spmvLayout32; /* layout of that configuration, coded as spmvLayout */
    uint32_t batchSliced;  /* batched solves: 1 when the chosen kernel reads the per-system SELL-32 copy */
    double tuneMs;         /* wall time of the last SpMV tuning (part of m_matProc) */
    double uploadMs;       /* device time of the last COO matrix upload (H2D, part of m_matProc) */
    double uploadIdxMs;    /* of which the row and column index copies (on the handle's stream) */
    double uploadValMs;    /* of which the value copy (on the side stream, from its start) */
    uint32_t loopUnroll;   /* iterations per pass of a graph loop's body (kernels past the stop return at once) */
    uint32_t kernelsPerIter; /* kernels per fp64 iteration: 2 (SpMV, fused vector kernel) or 3 (separate) */
} XJPCG_GbInfo_t;

/* Per-system outcome of a batched solve. */
typedef struct {
    uint32_t iters;    /* fp64: min(K, maxIter) as xJPCG reports it; mixed: inner iterations */
    uint32_t itersRun; /* iterations executed (fp64: K) */
    uint32_t outer;    /* mixed: refinement sweeps */
    uint32_t status;   /* 0 = ran to its stop rule, 1 = breakdown (non-finite alpha, beta or r.r) */
    double res;        /* fp64: sqrt(r.r / b.b) of the recursive residual; mixed: true relative residual */
} XJPCG_GbBatchResult_t;

/* xJPCG_createHandle on a chosen CUDA device (no counterpart in pcg.h; the
 * reference selects its card through the FPGA object's setId,
 * L2/common/include/sw/xNativeFPGA.hpp).  deviceId < 0 takes the calling
 * thread's current device, as xJPCG_createHandle does.  The caller's current
 * device is the same after the call as before it.  Every call on the handle
 * runs on its device and leaves the caller's current device unchanged. */
XJPCG_Status_t xJPCG_gbCreateHandleOnDevice(XJPCG_Handle_t** handle, int deviceId, const char* xclbinPath);

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

/* Mixed precision solve with the stored matrix (reliable updates): the CG
 * recurrences run in FP32 (FP32 values, vectors and dot products) and keep
 * their search direction; a refresh folds the FP32 correction into the FP64
 * x, recomputes r = b - A x with an FP64 SpMV and restarts the FP32 residual
 * from it.  A refresh runs when the FP32 residual norm has fallen by a factor
 * delta below its largest value since the last refresh (delta = 1e-3, or
 * XJPCG_RELIABLE_DELTA), when it meets the tolerance, and when the iteration
 * budget runs out.  Stops when ||b - A x|| <= tol ||b|| (true FP64 residual)
 * or after maxIter iterations.  *iter = FP32 iterations, *res = final true
 * relative residual.  onDevice != 0: b, diagA and x are device pointers. */
XJPCG_Status_t xJPCG_gbMixedSolve(XJPCG_Handle_t* handle, const double* b, const double* diagA, double* x,
                                  uint32_t maxIter, double tol, uint32_t* iter, double* res, int onDevice);

/* SpmvHost drop-in (replaces L2/sparse/include/sw/fp64/spmvHost.hpp:26-103:
 * createLoadNnzBufs + createLoadParXbufs[0] + createLoadRbParamBufs +
 * sendBOs).  Takes the reference's partitioned-matrix buffers as written by
 * its host partitioner (nnzVal_0..15, parParam, rbParam; numChannels must be
 * 16), decodes them on the GPU and stores the matrix in the handle (padding
 * and zero-valued entries dropped).  The matrix is square of size
 * max(rows, padded columns); xJPCG_gbGetInfo reports it. */
XJPCG_Status_t xJPCG_gbSetSignatureMatrix(XJPCG_Handle_t* handle, uint32_t numChannels, const void* const* nnzBufs,
                                          const uint64_t* nnzBytes, const void* parParam, uint64_t parParamBytes,
                                          const void* rbParam, uint64_t rbParamBytes);

/* Sizes of the partitioned-matrix ("signature") files of the stored matrix:
 * info[6] = m, n, nnz, mPad, nPad, nnzPad (the words of info.dat). */
typedef struct {
    uint32_t info[6];
    uint32_t rowBlocks;    /* rbParam records */
    uint32_t partitions;   /* parParam records */
    uint64_t rbParamBytes;
    uint64_t parParamBytes;
    uint64_t nnzValBytes[16];
} XJPCG_GbSignature_t;

/* Signature exporter (replaces SpmPar::partitionCooMat / partitionCscSymMat /
 * updateMat + storeMatPar: L2/sparse/include/sw/fp64/gen_signature.hpp:41-73,
 * signature.hpp:471-561, gen_signature.cpp:58-81).  Partitions the stored
 * matrix on the GPU into the bytes the reference's host partitioner writes
 * for the same input: rbParam.dat, parParam.dat, nnzVal_0..15.dat and
 * info.dat, with parEntries 4, accLatency 8, 16 channels and 4096 x 4096
 * partitions.  The layout is kept until the matrix structure changes; after
 * a values-only update (XJPCG_MODE_KEEP_NZ_LAYOUT) only the value streams
 * are rewritten, as update_sig does.  Fills *sig with the buffer sizes.
 * INVALID_VALUE when no matrix is stored or the padded matrix would exceed
 * 2^31 entries. */
XJPCG_Status_t xJPCG_gbExportSignature(XJPCG_Handle_t* handle, XJPCG_GbSignature_t* sig);

/* Copies the buffers of the last xJPCG_gbExportSignature to host memory of
 * the sizes it reported; any pointer, and any of the 16 nnzVal pointers, may
 * be NULL. */
XJPCG_Status_t xJPCG_gbGetSignature(XJPCG_Handle_t* handle, void* rbParam, void* parParam, void* const* nnzVal);

/* y = A x for the matrix loaded by xJPCG_gbSetSignatureMatrix (SpmvHost run +
 * getY; the x buffer is the second createLoadParXbufs buffer).  x has xLen
 * entries (the padded column count, zero-extended), y receives yRows rows
 * (setStoreYrows).  When frame is not NULL it also receives the dSpmv
 * transY framing of those rows (dSpmv/hw/include/impl/transY.hpp:35-65): a
 * 64-byte word {startAddr, yRows, 0...} followed by the values packed eight
 * per 64-byte word, zero-filled, at least one data word; frameBytes must be
 * >= 64 + 64 * max(1, ceil(yRows / 8)). */
XJPCG_Status_t xJPCG_gbSignatureSpmv(XJPCG_Handle_t* handle, const double* x, uint32_t xLen, double* y,
                                     uint32_t yRows, uint32_t startAddr, void* frame, uint64_t frameBytes);

/* JPCG on the matrix loaded by xJPCG_gbSetSignatureMatrix (the reference's
 * partitioned buffers), leading n x n block; b, diagA and x are host arrays
 * of n entries; same stop rule, counters, records and status as
 * xJPCG_cooSolver.  With summation order 1 (xJPCG_gbSetSignatureSumOrder)
 * every operation of the loop follows the reference FPGA's arithmetic as its
 * C source states it: the vector init of pcg/sw/include/impl/cgVector.hpp:
 * 101-114 (bb and r.z summed in index order), the SpMV order of
 * xJPCG_gbSignatureSpmv, the dot products of xf::blas::DotHelper<double, 2>
 * and nrm2s (L1/blas/include/hw/blas/helpers/funcs/dotHelper.hpp, sum.hpp:
 * 4-entry trees, zero-padded 8-entry trees, then the 8-entry sums added in
 * order), the axpy updates x = alpha*p + x, r = (-alpha)*Ap + r,
 * p = beta*p + z and z = r*J, each multiply, add and divide rounded on its
 * own.  The records and x are then the bits a C execution of that source
 * gives (a checking mode: its dot sums run on one thread).  With order 0 it
 * is the tuned solver on the decoded matrix, b and diag padded to the matrix
 * size with 0 and 1.  INVALID_VALUE when no partitioned matrix is loaded (or,
 * for order 1, it changed since) or n exceeds it. */
XJPCG_Status_t xJPCG_gbSignatureSolve(XJPCG_Handle_t* handle, uint32_t n, const double* b, const double* diagA,
                                      double* x, uint32_t maxIter, double tol, uint32_t* iter, double* res);

/* dSpmv store side (replaces dSpmvStoreYhost::run + getY,
 * dSpmv/sw/include/dSpmvStoreYhost.hpp:27-55, and the krnl_dStoreY kernel,
 * dSpmv/hw/include/impl/dStoreY.hpp:36-65).  Reads numNodes transY frames
 * back to back from `frames` (frameBytes bytes, host memory) and writes each
 * into y as dStoreY does: a 64-byte header word {startAddr, rows, ...}
 * (uint32; startAddr counted in 32-byte memory words), then ceil(rows / 8)
 * 64-byte data words, stored whole from byte 32 * startAddr on, so a last
 * partial word's zero fill is written too.  No handle and no device work.
 * INVALID_VALUE for a null pointer, a frame that runs past frameBytes, a
 * frame that would write past yBytes, or a header with rows = 0 (the transY
 * kernel still emits one data word for it, which dStoreY would not read, so
 * every later frame would be misread); frames before the bad one are
 * written.  *consumedBytes (may be NULL) = bytes of frames read. */
XJPCG_Status_t xJPCG_gbStoreYFrames(const void* frames, uint64_t frameBytes, uint32_t numNodes, double* y,
                                    uint64_t yBytes, uint64_t* consumedBytes);

/* Summation order of xJPCG_gbSignatureSpmv.  0 (the default): the tuned SpMV
 * kernels, each row summed in its CSR order with fused multiply-adds.
 * 1: the order of the reference's FPGA SpMV as its C source states it
 * (L1/sparse/include/hw/xf_sparse/fp64/spmv.hpp multAddX 136-157, regAcc
 * 159-185, rowMemAcc 452-476; dataMovers.hpp accY 339-375): each group of 4
 * stored entries as four rounded products summed left to right, each run of
 * 8 groups summed left to right, each row's runs in stream order, plus 0;
 * padding entries included.  Order 1 needs a matrix loaded by
 * xJPCG_gbSetSignatureMatrix and unchanged since (INVALID_VALUE otherwise),
 * and gives the same bits as a C execution of that source. */
XJPCG_Status_t xJPCG_gbSetSignatureSumOrder(XJPCG_Handle_t* handle, int order);

/* Adjoint of the handle's last solve x = A^-1 b (no counterpart in the
 * reference).  With g = dL/dx, solves lambda = A^-1 g (A is SPD) with the
 * same fp64 JPCG and stop rule, then, when gradA is not NULL, writes
 * dL/dA = -lambda_i x_j for every stored entry: for COO / CSR input gradA is
 * indexed like the input data array (duplicates each get the full value); for
 * symmetric-CSC input it is indexed by the expanded full matrix in the
 * reference's emission order (2 nnz - n entries).  dL/db = lambda.  Only the
 * converged x and lambda are kept.  onDevice != 0: g, diagA, lambda and
 * gradA are device pointers. */
XJPCG_Status_t xJPCG_gbAdjointSolve(XJPCG_Handle_t* handle, const double* g, const double* diagA, double* lambda,
                                    double* gradA, uint32_t maxIter, double tol, uint32_t* iter, double* res,
                                    int onDevice);

/* Edge gradient of a diffusion parametrisation (no counterpart in the
 * reference): for A = sum_e c_e (e_i - e_j)(e_i - e_j)^T + G with
 * c_e = exp(theta_e), writes gradTheta[e] = -c_e (lambda_i - lambda_j)
 * (x_i - x_j) = dL/dtheta_e, from the last solve's x and the last adjoint's
 * lambda.  onDevice != 0: the edge arrays are device pointers. */
XJPCG_Status_t xJPCG_gbEdgeGrad(XJPCG_Handle_t* handle, int64_t numEdges, const int32_t* edgeI, const int32_t* edgeJ,
                                const double* conductance, double* gradTheta, int onDevice);

/* Solves numSystems independent SPD systems in one persistent launch (no
 * counterpart in the reference; its control loop carries a CG_numTasks hook,
 * pcg/hw/include/control.hpp:43-92, built with one task).  The systems are
 * concatenated: system s owns rows sysRowStart[s] .. sysRowStart[s+1]-1 of the
 * concatenated vectors; rowPtr holds global entry offsets (rowPtr[0] = 0) and
 * colIdx holds 0-based column indices local to the system.  Every system uses
 * the xJPCG stop rule (fp64, precision 0) or FP64 refinement around an FP32
 * inner CG (precision 1), x0 = 0, with its own convergence test; results[s]
 * reports it.  Returns SUCCESS when every system met tol, else
 * EXECUTION_FAILED (x and results are written either way).  onDevice != 0:
 * all arrays except results are device pointers. */
XJPCG_Status_t xJPCG_gbBatchSolve(XJPCG_Handle_t* handle, uint32_t numSystems, const int32_t* sysRowStart,
                                  const int32_t* rowPtr, const int32_t* colIdx, const double* values,
                                  const double* diagA, const double* b, double* x, uint32_t maxIter, double tol,
                                  int precision, XJPCG_GbBatchResult_t* results, int onDevice);

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
 * pipeline stages.  Sliced configurations report (1, 0, unroll, column bits:
 * 32 for absolute int32 columns, 16 for int16 offsets from the row), the
 * length-sorted sliced ones (1, 1, unroll, 32), the shared-offset sliced
 * ones (1, 2, unroll, 1 when TMA bulk copies prefetch the values, a form
 * that exists in FP32 only, 2 when runs of consecutive offsets share one
 * gather through warp shuffles, else 0) and the merge-path kernel (0, 256,
 * steps per thread, 0).  At most cap
 * configurations are written. */
XJPCG_Status_t xJPCG_gbGetSpmvTuning(const XJPCG_Handle_t* handle, float* ms, int32_t* shape, int32_t cap,
                                     int32_t* count);

/* FP32 SpMV tuner report of the mixed solver (same configuration order as
 * xJPCG_gbGetSpmvTuning): ms[c] = median time of a plain FP32 SpMV, -1 when
 * not timed (not yet tuned, configuration not available, or a forced
 * layout).  At most cap entries are written. */
XJPCG_Status_t xJPCG_gbGetSpmvTuning32(const XJPCG_Handle_t* handle, float* ms, int32_t cap, int32_t* count);

/* The cudaStream_t the handle launches on (for event timing by callers). */
XJPCG_Status_t xJPCG_gbGetStream(const XJPCG_Handle_t* handle, void** stream);

/* Forces the CSR SpMV lanes-per-row (1, 2, 4, 8, 16, 32); -1 forces the
 * sliced layout, -2 the merge-path kernel, -3 the sliced layout with int16
 * column offsets (INVALID_VALUE when some column lies more than 32767 from
 * its row), -4 the length-sorted sliced layout (INVALID_VALUE when the plain
 * sliced layout pads 20 % or less, where it is not offered), -5 the sliced
 * layout with slice-shared column offsets (INVALID_VALUE when the plain
 * sliced layout is not available); 0 restores tuning.  A forced layout applies to the FP32 SpMV of
 * the mixed solver as well. */
XJPCG_Status_t xJPCG_gbSetSpmvLanes(XJPCG_Handle_t* handle, int lanes);

/* Forces the FP64 SpMV configuration with index cfg of the tuner report
 * (xJPCG_gbGetSpmvTuning), or restores tuning with -1.  INVALID_VALUE when
 * the configuration cannot run on the stored matrix (its layout is not
 * offered); the previous choice then stays.  It takes precedence over
 * xJPCG_gbSetSpmvLanes.  The FP32 SpMV of the mixed solver uses the same
 * configuration. */
XJPCG_Status_t xJPCG_gbSetSpmvConfig(XJPCG_Handle_t* handle, int cfg);

/* Forces the mixed solver's FP32 SpMV configuration (index cfg of the tuner
 * report; -1 restores tuning).  It applies from the next mixed solve, which
 * fails with INVALID_VALUE when the configuration cannot run on the stored
 * matrix in FP32. */
XJPCG_Status_t xJPCG_gbSetSpmvConfig32(XJPCG_Handle_t* handle, int cfg);

/* Failure-detection diagnostic.  Runs, on the handle's stream, the bounded
 * mbarrier wait that every wait of the library uses, on a barrier that
 * nothing completes.  The wait gives up after budgetNs (1 ns .. 1 s) and the
 * call returns INTERNAL_ERROR with the message a timed-out solve gives;
 * *deviceStatus = the device status bits (2 = wait timeout) and *elapsedNs =
 * the wait's duration on the device clock.  No copy is in flight, the GPU
 * context stays usable and the handle's matrix and vectors are untouched.
 * INVALID_VALUE for a budget out of range or null outputs. */
XJPCG_Status_t xJPCG_gbDiagWaitTimeout(XJPCG_Handle_t* handle, uint64_t budgetNs, uint32_t* deviceStatus,
                                       uint64_t* elapsedNs);

/* FP64 issue-rate diagnostic (no counterpart in the reference).  Runs, on the
 * handle's stream, a kernel that fills every SM with register-resident
 * chains of FP64 fused multiply-adds (8 independent chains per thread, 2048
 * threads per SM, iters steps per chain) and times it with CUDA events: one
 * warm-up launch, then the best of three.  *dfmaPerSecond = DFMA instructions
 * per second over the whole GPU, *ms = the best launch's time.  This is the
 * FP64 ceiling the library's fp64 kernels are measured against.
 * INVALID_VALUE for iters outside 1 .. 2^24 or null outputs. */
XJPCG_Status_t xJPCG_gbDiagFp64Rate(XJPCG_Handle_t* handle, int32_t iters, double* dfmaPerSecond, double* ms);

/* Memory-overrun diagnostic.  A handle created while the environment holds
 * XJPCG_GUARD_BYTES=N (N > 0) allocates each of its device buffers with N
 * bytes of 0xA5 after the end.  This call waits for the handle's streams and
 * compares every guard: *corrupted = the number of buffers whose guard bytes
 * changed.  SUCCESS when none did; INTERNAL_ERROR naming the first buffer
 * when some did; INVALID_VALUE when the handle has no guards. */
XJPCG_Status_t xJPCG_gbDiagCheckGuards(XJPCG_Handle_t* handle, uint32_t* corrupted);

/* y = A x and *d_dot = x.y for callers that cannot allocate device memory.
 *
 * No counterpart in the reference.  Some callers may not allocate at the
 * point of the call: code whose framework allocator owns the device memory,
 * code that must not synchronise the device (cudaMalloc / cudaFree can), or
 * a thread that only owns the buffers it was handed.  They cannot create a
 * handle, because a handle allocates.  This call takes no handle: the CSR
 * matrix (int32 row pointers and columns, 0-based, fp64 values) and the
 * vectors are the caller's device memory, and the kernel's only other memory
 * (its per-CTA partial sums and a counter) is a 131328-byte static array
 * inside this library that every GPU loading the library keeps until exit.
 *
 * Limit: n <= 524288 rows (one partial sum per 32-row tile, 16384 tiles);
 * larger n returns XJPCG_STATUS_INVALID_VALUE without launching.  The call
 * is asynchronous on `stream` (a cudaStream_t; NULL = legacy stream), with
 * d_y and *d_dot ready when the stream reaches it.  Every call shares the
 * static array: calls whose kernels overlap on the GPU race, calls on one
 * stream do not.  The first call in a CUDA context (normally the first call
 * on a device, in its primary context) looks up the array's address
 * (cudaGetSymbolAddress) with that context current and caches it for that
 * context; make it before any stream capture.  A context created later
 * (after cudaDeviceReset, or by cuCtxCreate) gets its own lookup on its first
 * call.  Nothing here allocates or frees. */
XJPCG_Status_t xJPCG_gbSpmvDotNoAlloc(uint32_t n, const int32_t* d_rowPtr, const int32_t* d_colIdx,
                                      const double* d_values, const double* d_x, double* d_y, double* d_dot,
                                      void* stream);

#ifdef __cplusplus
}
#endif

#endif /* XJPCG_GB300_H */
