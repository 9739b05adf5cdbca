/*
 * pcg.h -- xJPCG C API, GB300 implementation.
 *
 * Drop-in for the Xilinx/HPC xJPCG interface: the same symbols, argument
 * lists, enum values, struct layout and status strings as the reference's
 * pcg/sw/include/pcg.h (declarations at pcg.h:41-254, behaviour in
 * pcg/sw/src/pcg.cpp:34-215).  Applications that compiled against the
 * reference header compile and link against libXilinxPcg.so from this
 * repository unchanged.  Each entry point below names the reference
 * declaration it replaces.
 *
 * Differences a caller can observe (all are cases where the reference's
 * behaviour is undefined):
 *   - matrix indices outside [base, n+base) give XJPCG_STATUS_INVALID_VALUE;
 *   - KEEP_MATRIX with a dimension different from the stored matrix gives
 *     XJPCG_STATUS_INVALID_VALUE;
 *   - a non-finite alpha/beta/r.r stops the loop at that iteration and gives
 *     XJPCG_STATUS_EXECUTION_FAILED (the FPGA would run on to maxIter on NaN);
 *   - a negative p_maxIter in xJPCG_cscSymSolver gives INVALID_VALUE.
 */
#ifndef XILINX_PCG_H
#define XILINX_PCG_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

/* Same inline/extern switch as the reference (pcg.h:28-32), used by the
 * header-only loader (pcg_loader.c with XILINX_PCG_INLINE). */
#ifdef XILINX_PCG_INLINE
#define XILINX_PCG_LINKAGE_DECL inline
#else
#define XILINX_PCG_LINKAGE_DECL extern
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes, declared order as the reference (pcg.h:41-49). */
typedef enum {
    XJPCG_STATUS_SUCCESS,
    XJPCG_STATUS_NOT_INITIALIZED,
    XJPCG_STATUS_ALLOC_FAILED,
    XJPCG_STATUS_INVALID_VALUE,
    XJPCG_STATUS_EXECUTION_FAILED,
    XJPCG_STATUS_INTERNAL_ERROR,
    XJPCG_STATUS_DYNAMIC_LOADING_ERROR
} XJPCG_Status_t;

/* Replaces xJPCG_getErrorString (pcg.h:56-57, pcg.cpp:196-215): returns the
 * enumerator's name, or "Unknown Error Code!". */
XILINX_PCG_LINKAGE_DECL
const char* xJPCG_getErrorString(const XJPCG_Status_t code);

/* Wall-clock phases of the last call, in seconds (pcg.h:62-67). */
typedef struct {
    double m_objInit; /* handle creation: device context, stream, state */
    double m_matProc; /* matrix upload, conversion to CSR, SpMV tuning */
    double m_vecProc; /* b and diagonal upload */
    double m_solver;  /* device JPCG loop and result read-back */
} XJPCG_Metric_t;

struct XJPCG_ObjectStruct;
typedef struct XJPCG_ObjectStruct XJPCG_Handle_t;

/* Solver modes (pcg.h:79-85): low nibble = reuse, high nibble = index base. */
typedef enum XJPCG_Mode_t {
    XJPCG_MODE_DEFAULT = 0x00,
    XJPCG_MODE_KEEP_NZ_LAYOUT = 0x01,
    XJPCG_MODE_KEEP_MATRIX = 0x02,
    XJPCG_MODE_C_INDEX = 0x00,
    XJPCG_MODE_FORTRAN_INDEX = 0x10
} XJPCG_Mode_t;

/* Replaces xJPCG_createHandle (pcg.h:94-95, pcg.cpp:34-52).  The second
 * argument (an xclbin path in the reference) is accepted and ignored; the
 * handle binds to the current CUDA device.  *handle is set even when the
 * device set-up fails, so the caller can read the message. */
XILINX_PCG_LINKAGE_DECL
XJPCG_Status_t xJPCG_createHandle(XJPCG_Handle_t** handle, const char* xclbinPath);

/* Replaces xJPCG_destroyHandle (pcg.h:103-104, pcg.cpp:54-59). */
XILINX_PCG_LINKAGE_DECL
XJPCG_Status_t xJPCG_destroyHandle(XJPCG_Handle_t* handle);

/* Replaces xJPCG_cscSymSolver (pcg.h:163-177, pcg.cpp:61-116).  p_rowIdx /
 * p_colptr / p_data hold one triangle plus the diagonal, so the full matrix
 * has 2*p_nnz - p_n entries (pcgImp.hpp:87).  x0 = 0; p_x is output only. */
XILINX_PCG_LINKAGE_DECL
XJPCG_Status_t xJPCG_cscSymSolver(XJPCG_Handle_t* handle,
                                  const int64_t p_n,
                                  const int64_t p_nnz,
                                  const int64_t* p_rowIdx,
                                  const int64_t* p_colptr,
                                  const double* p_data,
                                  const double* p_diagA,
                                  const double* p_b,
                                  const double* p_x,
                                  const int64_t p_maxIter,
                                  const double p_tol,
                                  int64_t* p_iter,
                                  double* p_res,
                                  const XJPCG_Mode_t mode);

/* Replaces xJPCG_cooSolver (pcg.h:201-215, pcg.cpp:118-173).  With
 * XJPCG_MODE_KEEP_NZ_LAYOUT the index arrays may be NULL. */
XILINX_PCG_LINKAGE_DECL
XJPCG_Status_t xJPCG_cooSolver(XJPCG_Handle_t* handle,
                               const uint32_t p_n,
                               const uint32_t p_nnz,
                               const uint32_t* p_rowIdx,
                               const uint32_t* p_colIdx,
                               const double* p_data,
                               const double* p_diagA,
                               const double* p_b,
                               const double* p_x,
                               const uint32_t p_maxIter,
                               const double p_tol,
                               uint32_t* p_iter,
                               double* p_res,
                               const XJPCG_Mode_t mode);

/* Replaces xJPCG_peekAtLastStatus (pcg.h:223-224, pcg.cpp:182-188). */
XILINX_PCG_LINKAGE_DECL
XJPCG_Status_t xJPCG_peekAtLastStatus(const XJPCG_Handle_t* handle);

/* Replaces xJPCG_getLastMessage (pcg.h:240-241, pcg.cpp:190-194).  The
 * pointer stays valid until the next call on the handle. */
XILINX_PCG_LINKAGE_DECL
const char* xJPCG_getLastMessage(const XJPCG_Handle_t* handle);

/* Replaces xJPCG_getMetrics (pcg.h:253-254, pcg.cpp:175-180). */
XILINX_PCG_LINKAGE_DECL
XJPCG_Status_t xJPCG_getMetrics(const XJPCG_Handle_t* handle, XJPCG_Metric_t* metric);

#ifdef __cplusplus
}
#endif

#endif /* XILINX_PCG_H */
