// pcg_handle.hpp -- the object behind an XJPCG_Handle_t.
//
// Mirrors the reference's PCGImpl (pcg/sw/include/impl/pcgImp.hpp:44-253):
// matrix set / values-only update / reuse, vector set, run, result, metrics,
// last status and message.  The FPGA runtime underneath it (xCgHost,
// pcg/sw/src/cgHost.cpp:356-496) becomes a CUDA stream, device buffers and a
// CUDA graph that holds the whole solve: the vector-init kernel followed by a
// conditional WHILE node whose body is the three per-iteration kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/pcg.h"
#include "../../include/xjpcg_gb300.h"
#include "xjpcg_state.h"
#include "xjpcg_internal.hpp"

namespace xjpcg {

// Exceptions carry the status they map to; messages use the reference's
// prefixes (pcg/sw/include/impl/cgException.hpp:36-54).
class CgError : public std::runtime_error {
   public:
    CgError(XJPCG_Status_t st, const std::string& msg) : std::runtime_error(msg), status(st) {}
    XJPCG_Status_t status;
};
inline CgError InvalidValue(const std::string& s) { return CgError(XJPCG_STATUS_INVALID_VALUE, "INVALID VALUE ERROR: " + s); }
inline CgError InternalError(const std::string& s) { return CgError(XJPCG_STATUS_INTERNAL_ERROR, "INTERNAL ERROR: " + s); }
inline CgError AllocFailed(const std::string& s) { return CgError(XJPCG_STATUS_ALLOC_FAILED, "Alloc Failed ERROR: " + s); }
inline CgError ExecFailed(const std::string& s) { return CgError(XJPCG_STATUS_EXECUTION_FAILED, "Solver ERROR: " + s); }

// Grow-only device buffer.  Every reallocation bumps the owner's generation
// so graphs that captured the old address are rebuilt.
constexpr unsigned char kGuardByte = 0xA5;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    size_t guard = 0;  // guard bytes allocated past `bytes` (debug builds of a handle)
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        guard = 0;
    }
    // Grows the buffer to at least b bytes; with guardBytes > 0 a new
    // allocation carries that many bytes of kGuardByte after its end.
    bool ensure(size_t b, uint64_t* generation, size_t guardBytes = 0);
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

struct Results {
    uint32_t reportedIters;  // min(K, maxIter), the reference's host scan
    uint32_t itersRun;       // K
    double rrLast;
    double bb;
    uint32_t status;
};

// The stored matrix in the reference's partitioned ("signature") format,
// built on the device (signature_export.cu).  build() computes the layout
// from the CSR structure; format() writes the channel streams from the
// values, so a values-only update reruns format() alone.
class SigExport {
   public:
    void build(cudaStream_t st, uint32_t n, uint64_t nnz, const int* rowptr, const int* col);
    void format(cudaStream_t st, const double* val);
    void copyOut(cudaStream_t st, void* rb, void* par, void* const* nnzVal) const;

    bool valid = false;
    uint64_t structGen = 0;  // matrix structure the layout was built for
    uint32_t m = 0, n = 0, nnz = 0, nnzPad = 0;
    int nb = 0, P = 0, S = 0;
    uint64_t rbBytes = 0, parBytes = 0;
    uint64_t chanBytes[16] = {}, chanBase[16] = {};

   private:
    static void grow(DevBuf& b, size_t bytes, const char* what);
    DevBuf bBlkRow0, bBlkEnt, bBlkM, bBlkMin, bBlkMax, bBlkMinG, bBlkMaxG, bBlkNcol, bBitOff, bSlotOff, bBitmap;
    DevBuf bStarts, bNPart, bParBase, bPartG0, bPartBlock, bBlockSums;
    DevBuf bSegCount, bSegBase, bSegLo, bSegHi, bSegRow, bSegLen, bSegMinG, bSegMaxG, bSegOff, bTotal, bPpad;
    DevBuf bSlotSrc, bGrpRow, bGrpG;
    DevBuf bChStart, bChLen, bChMinG, bChEndRow, bChBytes, bChOff, bChanBytes, bChanBase, bChanHdr;
    DevBuf bRb, bPar, bOut;
};

class PcgHandle {
   public:
    PcgHandle() = default;
    ~PcgHandle();
    // device < 0: the calling thread's current device.
    void init(int device = -1);
    bool initDone() const { return m_initDone; }
    int device() const { return m_device; }

    // Matrix input.  base: 0 = C, 1 = Fortran (mode >> 4).
    void setCooMat(uint32_t n, uint64_t nnz, const uint32_t* row, const uint32_t* col, const double* data, int base);
    void updateCooValues(uint32_t n, uint64_t nnz, const double* data);
    void setCscSymMat(uint32_t n, uint64_t nnzHalf, const int64_t* rowIdx, const int64_t* colPtr, const double* data,
                      int base);
    void updateCscSymValues(uint32_t n, uint64_t nnzHalf, const int64_t* rowIdx, const int64_t* colPtr,
                            const double* data, int base);
    void setCsrMat(uint32_t n, uint64_t nnz, const int32_t* rowPtr, const int32_t* colIdx, const double* data,
                   int base);
    void updateCsrValues(uint32_t n, uint64_t nnz, const double* data);

    void setVec(uint32_t n, const double* b, const double* diag, bool onDevice);
    Results run(uint32_t maxIter, double tol);
    void copyX(double* x, uint32_t n, bool toDevice);

    Results runMixed(uint32_t maxIter, double tol);
    void copyX64(double* x, uint32_t n, bool toDevice);

    void spmv(const double* x, double* y, bool onDevice);
    // The reference's partitioned-matrix buffers as the stored matrix.
    void setSignatureMatrix(uint32_t nch, const void* const* bufs, const uint64_t* bytes, const void* par,
                            uint64_t parBytes, const void* rb, uint64_t rbBytes);
    void setSignatureSumOrder(int order);
    // JPCG on the leading n x n block of the signature matrix: summation
    // order 1 = the reference FPGA's arithmetic order (fpga_order.cu), 0 =
    // the tuned solver on the decoded CSR.  Host arrays.
    Results signatureSolve(uint32_t n, const double* b, const double* diag, double* x, uint32_t maxIter, double tol);
    void signatureSpmv(const double* x, uint32_t xLen, double* y, uint32_t yRows, uint32_t startAddr,
                       unsigned char* frame, uint64_t frameBytes);
    uint32_t sigRows() const { return m_sigRows; }
    // Adjoint of the last solve: lambda = A^-1 g; optional dL/dA per input entry.
    Results adjoint(const double* g, const double* diag, double* lambda, double* gradA, uint32_t maxIter, double tol,
                    bool onDevice);
    void edgeGrad(int64_t m, const int32_t* ei, const int32_t* ej, const double* c, double* grad, bool onDevice);
    void markSolved() { m_haveX = true; }
    // Batched solve: concatenated systems (see batched_kernels.cu).  Returns the
    // number of systems that did not converge.
    uint32_t batchSolve(uint32_t nsys, const int32_t* sysRow, const int32_t* rowPtr, const int32_t* colIdx,
                        const double* values, const double* diag, const double* b, double* x, uint32_t maxIter,
                        double tol, int precision, BatchResult* results, bool onDevice);
    void getCsr(int32_t* rowPtr, int32_t* colIdx, double* values, uint32_t* perm);
    void exportSignature(XJPCG_GbSignature_t* sig);
    void getSignature(void* rb, void* par, void* const* nnzVal);
    uint64_t getRecords(void* buf, uint64_t cap);
    void fillInfo(XJPCG_GbInfo_t* info) const;
    int tuning(float* ms, int* shape, int cap) const;
    int tuning32(float* ms, int cap) const;
    void setLanes(int lanes);
    void setSpmvConfig(int cfg);
    void setSpmvConfig32(int cfg);
    void diagWaitTimeout(uint64_t budgetNs, uint32_t* deviceStatus, uint64_t* elapsedNs);
    void diagFp64Rate(int32_t iters, double* dfmaPerSecond, double* ms);
    uint32_t checkGuards(std::string* firstBad);  // buffers whose guard bytes changed
    bool guardsOn() const { return m_guardBytes > 0; }

    bool hasMatrix() const { return m_haveMatrix; }
    uint32_t matrixN() const { return m_n; }
    cudaStream_t stream() const { return m_stream; }

    XJPCG_Metric_t* metrics() { return &m_metrics; }
    const XJPCG_Metric_t* metrics() const { return &m_metrics; }
    XJPCG_Status_t setStatusMessage(XJPCG_Status_t st, const std::string& msg) const {
        m_lastStatus = st;
        m_lastMessage = msg;
        return st;
    }
    XJPCG_Status_t lastStatus() const { return m_lastStatus; }
    const std::string& lastMessage() const { return m_lastMessage; }
    bool isFirstCall() const { return m_firstCall; }
    void markCalled() { m_firstCall = false; }
    double dot() const { return m_lastBb; }

   private:
    void check(cudaError_t e, const char* what);
    void faultPoint(const char* what);
    void alloc(DevBuf& b, size_t bytes, const char* what);
    void finishMatrix();     // after CSR exists: values pad, tuning
    void tuneSpmv();
    int numSpmvCfgs() const;
    bool isSell(int cfg) const;
    bool isSellNarrow(int cfg) const;
    bool isSorted(int cfg) const;
    bool isPat(int cfg) const;
    int patCfg0() const;
    bool ensurePat();
    int sortedCfg0() const;
    int mergeCfg() const;
    uint32_t layoutCode(int cfg) const;
    bool ensureSorted();
    bool isMerge(int cfg) const;
    void ensureMergeScratch();
    int spmvGrid64(int cfg);
    int spmvGrid32(int cfg);
    bool ensureSell();
    void ensureValues32(int cfg);
    void tuneSpmv32();
    int timeConfigs(bool fp32, std::vector<float>& out);
    void refreshSellValues();
    cudaError_t spmv64(int cfg, int grid, const double* x, double* y, const double* b, CgState* st, double* part,
                       int mode, const uint32_t* done);
    cudaError_t spmv32(int cfg, int grid, const float* x, float* y, const float* b, CgState* st, double* part,
                       int mode, const uint32_t* done);
    void ensureVectors(uint32_t n);
    void buildGraph();
    int cgSpmvMode() const;
    void mixedUpdate(int n4, int vg, CgState* st, double* part, bool pUpdate = true);
    void iterationTail(int n4, CgState* st, double* part);
    void buildMixedGraph();
    Results readResults(uint32_t maxIter);

    mutable XJPCG_Status_t m_lastStatus = XJPCG_STATUS_SUCCESS;
    mutable std::string m_lastMessage;
    bool m_firstCall = true;
    XJPCG_Metric_t m_metrics = {0, 0, 0, 0};

    int m_device = 0;
    int m_numSms = 0;
    cudaStream_t m_stream = nullptr;
    cudaStream_t m_upStream = nullptr;  // COO value upload, overlapping the index conversion
    cudaEvent_t m_evIdxIn = nullptr;
    cudaEvent_t m_ev0 = nullptr, m_ev1 = nullptr;
    uint64_t m_generation = 1;

    // matrix
    bool m_haveMatrix = false;
    uint32_t m_n = 0;
    uint64_t m_nnz = 0;
    uint64_t m_nnzHalf = 0;   // symmetric CSC input only
    int m_kind = 0;           // 0 none, 1 COO, 2 CSC-sym, 3 CSR
    DevBuf m_rowptr, m_col, m_val, m_perm, m_val32;
    DevBuf m_inRow, m_inCol, m_inVal, m_inIdx64, m_inPtr64;
    DevBuf m_counts, m_fill, m_blockSums, m_keys, m_flags, m_cscScratch;
    // sliced (SELL-32) copy of the matrix, built on demand by the tuner
    DevBuf m_sliceOff, m_sellCol, m_sellVal, m_sellVal32;
    DevBuf m_sellCol16;          // int16 column offsets (when the matrix is narrow enough)
    bool m_sellNarrow = false;
    double m_sellPadRatio = 0.0;  // stored / real entries of the sliced copy
    // sliced copy with slice-shared column offsets (structured grids)
    DevBuf m_psSliceOff, m_psPatLen, m_psPatNew, m_psPatIdx, m_psPatOff, m_psGenOff, m_psPat, m_psGcol, m_psVal,
        m_psVal32;
    int m_psState = 0;  // 0 not built, 1 built, 2 not offered
    int64_t m_psTotal = 0;
    bool m_ps32Valid = false;
    // length-sorted sliced copy (irregular rows)
    DevBuf m_ssSorted, m_ssHist, m_ssStart, m_ssSliceOff, m_ssCol, m_ssVal, m_ssVal32;
    int m_ssState = 0;  // 0 not built, 1 built, 2 not offered
    int m_ssLong = 0;
    int64_t m_ssTotal = 0;
    bool m_ss32Valid = false;
    int m_sellState = 0;  // 0 not built, 1 built, 2 rejected (too much padding)
    DevBuf m_mergeRow, m_mergeVal, m_mergePart;  // merge-path carries and partials
    DevBuf m_mergeTile;                          // merge-path tile start rows
    bool m_mergeTilesValid = false;
    int64_t m_sellTotal = 0;
    bool m_sell32Valid = false;
    bool m_val32Valid = false;
    int m_forcedLanes = 0;
    int m_forcedCfg = -1;  // forced SpMV configuration index, -1 = tuned
    int m_forcedCfg32 = -1;  // forced FP32 SpMV configuration of the mixed solver, -1 = tuned
    // SpMV tuning cache: the choices stand while the structure fingerprint matches
    DevBuf m_hashBuf;
    DevBuf m_diagBuf;  // bounded-wait diagnostic output
    uint64_t m_structHash = 0, m_tunedHash = ~0ull;
    int m_tunedCfg = -1, m_tuned32Cfg = -1;
    int m_spmvCfg = 2;
    int m_spmvGrid = 0;
    std::vector<float> m_tuneMs;  // median time of each SpMV configuration at the last tuning
    // FP32 SpMV of the mixed solver: tuned separately (no FP64 issue limit)
    int m_spmvCfg32 = -1;
    int m_spmvGrid32 = 0;
    uint64_t m_tuned32Gen = ~0ull;
    std::vector<float> m_tuneMs32;
    double m_lastTuneMs = 0.0;  // wall time of the last FP64 tuning
    cudaEvent_t m_evUp0 = nullptr, m_evUp1 = nullptr;  // around the last COO upload
    cudaEvent_t m_evUpIdx = nullptr, m_evUpVal = nullptr;  // end of the index copies, start of the value copy
    bool m_uploadTimed = false;

    // vectors
    uint32_t m_vecN = 0, m_n4 = 0;
    DevBuf m_b, m_diag, m_x, m_r, m_p, m_J, m_Ap;
    DevBuf m_state, m_partials, m_records;
    uint64_t m_recCap = 0;
    DevBuf m_scratchY;
    // mixed precision
    DevBuf m_state32, m_r32, m_p32, m_d32, m_Ap32, m_J32;

    // signature input
    DevBuf m_sigBuf, m_sigChunks, m_sigRow, m_sigCol, m_sigVal, m_sigKeep, m_sigFrame;
    uint32_t m_sigRows = 0;
    // reference-order SpMV over the decoded stored entries (m_sigVal, m_sigCol)
    DevBuf m_sigRunRow, m_sigRunIdx, m_sigRunPtr, m_sigRunList, m_sigRunPerm;
    int m_sigSumOrder = 0;                         // 0 = fastest SpMV, 1 = the reference's summation order
    uint64_t m_valGen = 0, m_sigOrderedGen = ~0ull;  // matrix values generation; the one the run lists match
    SigExport m_sigExport;
    DevBuf m_foPart;  // block sums of the reference-order dots
    uint64_t m_structGen = 0;  // bumped whenever a new matrix structure is stored
    // adjoint
    DevBuf m_xKeep, m_lambda, m_grad, m_edgeI, m_edgeJ, m_edgeC, m_edgeG;
    bool m_haveX = false, m_haveLambda = false;

    // batched solves
    DevBuf m_bSysRow, m_bOrder, m_bRowptr, m_bCol, m_bVal, m_bVal32, m_bB, m_bDiag, m_bX, m_bR, m_bAp, m_bJ;
    DevBuf m_bR32, m_bD32, m_bAp32, m_bJ32, m_bP, m_bP32, m_bRes, m_bQueue;
    DevBuf m_bsBase, m_bsLen, m_bsOff, m_bsScan, m_bsVal, m_bsVal32, m_bsCol;  // per-system SELL-32 copy
    DevBuf m_bsPatLen, m_bsPatOff;  // its slices' shared column offsets
    DevBuf m_bsMeta, m_bsSysPat;    // slice records, and each system's offsets
    int m_batchCfg = -1, m_batchSmemRows = 0, m_batchGrid = 0;
    uint64_t m_batchKey = 0;
    float m_batchMs = 0.f;
    std::vector<float> m_batchTuneMs;
    cudaGraphExec_t m_batchExec = nullptr;  // queue reset + persistent kernel
    uint64_t m_batchExecKey = 0;

    // graph
    cudaGraphExec_t m_exec = nullptr;
    uint64_t m_execGen = 0;
    cudaGraphConditionalHandle m_cond = 0;
    cudaGraphExec_t m_mixedExec = nullptr;
    uint64_t m_mixedGen = 0;
    cudaGraphConditionalHandle m_condOuter = 0, m_condInner = 0;
    bool m_useGraph = true;
    bool m_fusedUpdate = true;  // XJPCG_FUSED_UPDATE
    bool m_faultAlloc = false, m_faultLaunch = false, m_initDone = false;  // XJPCG_FAULT hooks
    size_t m_guardBytes = 0;                                   // XJPCG_GUARD_BYTES
    std::vector<std::pair<DevBuf*, std::string>> m_guarded;    // buffers allocated with guards

    // last results
    double m_lastBb = 0.0;
    CgState m_lastState{};
    float m_lastMs = 0.f;
    uint32_t m_lastOuter = 0, m_lastInner = 0;
};

}  // namespace xjpcg
