// pcg_api.cpp -- the extern "C" boundary of libXilinxPcg.so.
//
// The pcg.h entry points follow pcg/sw/src/pcg.cpp:34-215 step for step: mode
// dispatch on (mode & 0x0f), index base (mode & 0xf0) >> 4, first-call check
// for the reuse modes, the four metric phases, res = sqrt(Res / bb), and
// EXECUTION_FAILED when res > tol with x, iter and res still written.  No C++
// exception crosses this boundary.
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>

#include "pcg_handle.hpp"

using xjpcg::CgError;
using xjpcg::PcgHandle;

namespace {

double elapsed(std::chrono::time_point<std::chrono::high_resolution_clock>& last) {
    auto now = std::chrono::high_resolution_clock::now();
    std::chrono::duration<double> d = now - last;
    last = now;
    return d.count();
}

PcgHandle* impl(XJPCG_Handle_t* h) { return reinterpret_cast<PcgHandle*>(h); }
const PcgHandle* impl(const XJPCG_Handle_t* h) { return reinterpret_cast<const PcgHandle*>(h); }

// Makes the handle's device current for one API call and gives the calling
// thread its previous device back afterwards, so that a handle created on
// one device keeps working whatever device the caller has current.
class DeviceScope {
   public:
    explicit DeviceScope(const PcgHandle* p) {
        if (p == nullptr || !p->initDone()) return;
        if (cudaGetDevice(&m_prev) == cudaSuccess && m_prev != p->device() && cudaSetDevice(p->device()) == cudaSuccess)
            m_switched = true;
    }
    ~DeviceScope() {
        if (m_switched) cudaSetDevice(m_prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;

   private:
    int m_prev = 0;
    bool m_switched = false;
};

// The index base of a mode; the reference rejects anything but 0 and 1 in
// SparseMatrix::loadCoo / loadCscSym (matrix_params.hpp:51-60, 82-96) with an
// SpmNotSupported exception that surfaces as INTERNAL_ERROR.
int modeBase(int mode) {
    const int base = (mode & 0xf0) >> 4;
    if (base != 0 && base != 1)
        throw xjpcg::InternalError("from getCooDatFromCscSym in gen_signature.hpp, unsupported storage mode.");
    return base;
}

void finishSolve(PcgHandle* p, const xjpcg::Results& r, double tol, double* res, uint32_t* iter32, int64_t* iter64,
                 std::chrono::time_point<std::chrono::high_resolution_clock>& last) {
    *res = std::sqrt(r.rrLast / r.bb);
    if (iter32) *iter32 = r.reportedIters;
    if (iter64) *iter64 = r.reportedIters;
    p->markCalled();
    p->markSolved();
    p->metrics()->m_solver = elapsed(last);
    if (r.status & xjpcg::kStatusBreakdown)
        throw xjpcg::ExecFailed("breakdown (non-finite alpha, beta or r.r) after " + std::to_string(r.reportedIters) +
                                " iterations.");
    if (*res > tol)
        throw xjpcg::ExecFailed("exit with divergent solution after " + std::to_string(r.reportedIters) +
                                " iterations.");
}

}  // namespace

extern "C" {

XJPCG_Status_t xJPCG_createHandle(XJPCG_Handle_t** handle, const char* xclbinPath) {
    return xJPCG_gbCreateHandleOnDevice(handle, -1, xclbinPath);
}

XJPCG_Status_t xJPCG_gbCreateHandleOnDevice(XJPCG_Handle_t** handle, int deviceId, const char* xclbinPath) {
    (void)xclbinPath;
    if (handle == nullptr) return XJPCG_STATUS_INVALID_VALUE;
    PcgHandle* p = new (std::nothrow) PcgHandle();
    if (p == nullptr) return XJPCG_STATUS_ALLOC_FAILED;
    *handle = reinterpret_cast<XJPCG_Handle_t*>(p);
    int prev = -1;
    if (deviceId >= 0 && cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    struct Restore {
        int dev;
        ~Restore() {
            if (dev >= 0) cudaSetDevice(dev);
        }
    } restore{prev};
    try {
        auto last = std::chrono::high_resolution_clock::now();
        p->init(deviceId);
        p->metrics()->m_objInit = elapsed(last);
    } catch (const CgError& e) {
        return p->setStatusMessage(e.status, e.what());
    } catch (const std::exception& e) {
        return p->setStatusMessage(XJPCG_STATUS_INTERNAL_ERROR, e.what());
    }
    return p->setStatusMessage(XJPCG_STATUS_SUCCESS, "Handle is created successfully");
}

XJPCG_Status_t xJPCG_destroyHandle(XJPCG_Handle_t* handle) {
    if (handle == nullptr) return XJPCG_STATUS_NOT_INITIALIZED;
    DeviceScope scope(impl(handle));
    delete impl(handle);
    return XJPCG_STATUS_SUCCESS;
}

XJPCG_Status_t xJPCG_cscSymSolver(XJPCG_Handle_t* handle, const int64_t p_n, const int64_t p_nnz,
                                  const int64_t* p_rowIdx, const int64_t* p_colPtr, const double* p_data,
                                  const double* p_diagA, const double* p_b, const double* p_x,
                                  const int64_t p_maxIter, const double p_tol, int64_t* p_iter, double* p_res,
                                  const XJPCG_Mode_t mode) {
    if (handle == nullptr) return XJPCG_STATUS_NOT_INITIALIZED;
    PcgHandle* p = impl(handle);
    try {
        auto last = std::chrono::high_resolution_clock::now();
        const bool first = p->isFirstCall();
        // PCGImpl::setCscSymMat / updateCscSymMat argument checks
        // (pcgImp.hpp:78-86, 124-132); the narrowing to uint32_t is the
        // reference's own (pcgImp.hpp:72-77).
        const uint32_t n = (uint32_t)p_n;
        const uint32_t nnz = (uint32_t)p_nnz;
        switch (mode & 0x0f) {
            case XJPCG_MODE_DEFAULT: {
                if (n == 0) throw xjpcg::InvalidValue("Wrong dimension size.");
                if (nnz == 0) throw xjpcg::InvalidValue("Wrong non-zero element size.");
                if (p_rowIdx == nullptr || p_colPtr == nullptr || p_data == nullptr)
                    throw xjpcg::InvalidValue("Matrix is nullptr.");
                p->setCscSymMat(n, nnz, p_rowIdx, p_colPtr, p_data, modeBase(mode));
                break;
            }
            case XJPCG_MODE_KEEP_NZ_LAYOUT: {
                if (first)
                    throw xjpcg::InvalidValue("wrong solver mode for the first call, please use XJPCG_MODEL_DEFAULT.");
                if (n == 0) throw xjpcg::InvalidValue("Wrong dimension size.");
                if (nnz == 0) throw xjpcg::InvalidValue("Wrong non-zero element size.");
                if (p_data == nullptr) throw xjpcg::InvalidValue("Matrix is nullptr.");
                p->updateCscSymValues(n, nnz, p_rowIdx, p_colPtr, p_data, modeBase(mode));
                break;
            }
            default:
                if (first)
                    throw xjpcg::InvalidValue("wrong solver mode for the first call, please use XJPCG_MODEL_DEFAULT.");
                break;
        }
        p->metrics()->m_matProc = elapsed(last);
        if (p_maxIter < 0) throw xjpcg::InvalidValue("negative maximum iteration count.");
        p->setVec(n, p_b, p_diagA, false);
        p->metrics()->m_vecProc = elapsed(last);
        xjpcg::Results r = p->run((uint32_t)p_maxIter, p_tol);
        p->copyX(const_cast<double*>(p_x), n, false);
        finishSolve(p, r, p_tol, p_res, nullptr, p_iter, last);
    } catch (const CgError& e) {
        return p->setStatusMessage(e.status, e.what());
    } catch (const std::exception& e) {
        return p->setStatusMessage(XJPCG_STATUS_INTERNAL_ERROR, e.what());
    }
    return p->setStatusMessage(XJPCG_STATUS_SUCCESS, "Solver returns successfully");
}

XJPCG_Status_t xJPCG_cooSolver(XJPCG_Handle_t* handle, const uint32_t p_n, const uint32_t p_nnz,
                               const uint32_t* p_rowIdx, const uint32_t* p_colIdx, const double* p_data,
                               const double* matJ, const double* b, const double* x, const uint32_t p_maxIter,
                               const double p_tol, uint32_t* p_iter, double* p_res, const XJPCG_Mode_t mode) {
    if (handle == nullptr) return XJPCG_STATUS_NOT_INITIALIZED;
    PcgHandle* p = impl(handle);
    try {
        auto last = std::chrono::high_resolution_clock::now();
        const bool first = p->isFirstCall();
        switch (mode & 0x0f) {
            case XJPCG_MODE_DEFAULT:
                // PCGImpl::setCooMat checks (pcgImp.hpp:55-63)
                if (p_n == 0) throw xjpcg::InvalidValue("Wrong dimension size.");
                if (p_nnz == 0) throw xjpcg::InvalidValue("Wrong non-zero element size.");
                if (p_rowIdx == nullptr || p_colIdx == nullptr || p_data == nullptr)
                    throw xjpcg::InvalidValue("Matrix is nullptr.");
                p->setCooMat(p_n, p_nnz, p_rowIdx, p_colIdx, p_data, modeBase(mode));
                break;
            case XJPCG_MODE_KEEP_NZ_LAYOUT:
                if (first)
                    throw xjpcg::InvalidValue("wrong solver mode for the first call, please use XJPCG_MODEL_DEFAULT.");
                // PCGImpl::updateMat checks (pcgImp.hpp:96-104); indices unused
                if (p_n == 0) throw xjpcg::InvalidValue("Wrong dimension size.");
                if (p_nnz == 0) throw xjpcg::InvalidValue("Wrong non-zero element size.");
                if (p_data == nullptr) throw xjpcg::InvalidValue("Matrix is nullptr.");
                p->updateCooValues(p_n, p_nnz, p_data);
                break;
            default:
                if (first)
                    throw xjpcg::InvalidValue("wrong solver mode for the first call, please use XJPCG_MODEL_DEFAULT.");
                break;
        }
        p->metrics()->m_matProc = elapsed(last);
        p->setVec(p_n, b, matJ, false);
        p->metrics()->m_vecProc = elapsed(last);
        xjpcg::Results r = p->run(p_maxIter, p_tol);
        p->copyX(const_cast<double*>(x), p_n, false);
        finishSolve(p, r, p_tol, p_res, p_iter, nullptr, last);
    } catch (const CgError& e) {
        return p->setStatusMessage(e.status, e.what());
    } catch (const std::exception& e) {
        return p->setStatusMessage(XJPCG_STATUS_INTERNAL_ERROR, e.what());
    }
    return p->setStatusMessage(XJPCG_STATUS_SUCCESS, "Solver returns successfully");
}

XJPCG_Status_t xJPCG_getMetrics(const XJPCG_Handle_t* handle, XJPCG_Metric_t* metric) {
    if (handle == nullptr) return XJPCG_STATUS_NOT_INITIALIZED;
    const PcgHandle* p = impl(handle);
    if (metric == nullptr) return p->setStatusMessage(XJPCG_STATUS_INVALID_VALUE, "INVALID VALUE ERROR: metric is nullptr.");
    *metric = *p->metrics();
    return p->setStatusMessage(XJPCG_STATUS_SUCCESS, "Get metrics successfully");
}

XJPCG_Status_t xJPCG_peekAtLastStatus(const XJPCG_Handle_t* handle) {
    if (handle == nullptr) return XJPCG_STATUS_NOT_INITIALIZED;
    return impl(handle)->lastStatus();
}

const char* xJPCG_getLastMessage(const XJPCG_Handle_t* handle) {
    if (handle == nullptr) return "Can't retrieve last error message from a null JPCG handle.";
    return impl(handle)->lastMessage().c_str();
}

const char* xJPCG_getErrorString(const XJPCG_Status_t code) {
    switch (code) {
        case XJPCG_STATUS_SUCCESS:
            return "XJPCG_STATUS_SUCCESS";
        case XJPCG_STATUS_NOT_INITIALIZED:
            return "XJPCG_STATUS_NOT_INITIALIZED";
        case XJPCG_STATUS_ALLOC_FAILED:
            return "XJPCG_STATUS_ALLOC_FAILED";
        case XJPCG_STATUS_INVALID_VALUE:
            return "XJPCG_STATUS_INVALID_VALUE";
        case XJPCG_STATUS_EXECUTION_FAILED:
            return "XJPCG_STATUS_EXECUTION_FAILED";
        case XJPCG_STATUS_INTERNAL_ERROR:
            return "XJPCG_STATUS_INTERNAL_ERROR";
        case XJPCG_STATUS_DYNAMIC_LOADING_ERROR:
            return "XJPCG_STATUS_DYNAMIC_LOADING_ERROR";
    }
    return "Unknown Error Code!";
}

// ---------------------------------------------------------------------------
// Extensions (xjpcg_gb300.h)
// ---------------------------------------------------------------------------
#define XJ_GUARD_BEGIN                                 \
    if (handle == nullptr) return XJPCG_STATUS_NOT_INITIALIZED; \
    PcgHandle* p = impl(handle);                        \
    DeviceScope deviceScope_(p);                        \
    try {
#define XJ_GUARD_END(msg)                                               \
    }                                                                   \
    catch (const CgError& e) {                                          \
        return p->setStatusMessage(e.status, e.what());                 \
    }                                                                   \
    catch (const std::exception& e) {                                   \
        return p->setStatusMessage(XJPCG_STATUS_INTERNAL_ERROR, e.what()); \
    }                                                                   \
    return p->setStatusMessage(XJPCG_STATUS_SUCCESS, msg);

XJPCG_Status_t xJPCG_gbCsrSolver(XJPCG_Handle_t* handle, uint32_t n, uint32_t nnz, const int32_t* rowPtr,
                                 const int32_t* colIdx, const double* data, const double* diagA, const double* b,
                                 double* x, uint32_t maxIter, double tol, uint32_t* iter, double* res,
                                 XJPCG_Mode_t mode) {
    XJ_GUARD_BEGIN
    auto last = std::chrono::high_resolution_clock::now();
    const bool first = p->isFirstCall();
    switch (mode & 0x0f) {
        case XJPCG_MODE_DEFAULT:
            if (n == 0) throw xjpcg::InvalidValue("Wrong dimension size.");
            if (nnz == 0) throw xjpcg::InvalidValue("Wrong non-zero element size.");
            if (rowPtr == nullptr || colIdx == nullptr || data == nullptr)
                throw xjpcg::InvalidValue("Matrix is nullptr.");
            p->setCsrMat(n, nnz, rowPtr, colIdx, data, modeBase(mode));
            break;
        case XJPCG_MODE_KEEP_NZ_LAYOUT:
            if (first) throw xjpcg::InvalidValue("wrong solver mode for the first call, please use XJPCG_MODEL_DEFAULT.");
            if (data == nullptr) throw xjpcg::InvalidValue("Matrix is nullptr.");
            p->updateCsrValues(n, nnz, data);
            break;
        default:
            if (first) throw xjpcg::InvalidValue("wrong solver mode for the first call, please use XJPCG_MODEL_DEFAULT.");
            break;
    }
    p->metrics()->m_matProc = elapsed(last);
    p->setVec(n, b, diagA, false);
    p->metrics()->m_vecProc = elapsed(last);
    xjpcg::Results r = p->run(maxIter, tol);
    p->copyX(x, n, false);
    finishSolve(p, r, tol, res, iter, nullptr, last);
    XJ_GUARD_END("Solver returns successfully")
}

XJPCG_Status_t xJPCG_gbSolveDevice(XJPCG_Handle_t* handle, const double* d_b, const double* d_diagA, double* d_x,
                                   uint32_t maxIter, double tol, uint32_t* iter, double* res) {
    XJ_GUARD_BEGIN
    auto last = std::chrono::high_resolution_clock::now();
    if (!p->hasMatrix()) throw xjpcg::InvalidValue("no matrix has been set.");
    p->metrics()->m_matProc = 0.0;
    p->setVec(p->matrixN(), d_b, d_diagA, true);
    p->metrics()->m_vecProc = elapsed(last);
    xjpcg::Results r = p->run(maxIter, tol);
    if (d_x) p->copyX(d_x, p->matrixN(), true);
    finishSolve(p, r, tol, res, iter, nullptr, last);
    XJ_GUARD_END("Solver returns successfully")
}

XJPCG_Status_t xJPCG_gbMixedSolve(XJPCG_Handle_t* handle, const double* b, const double* diagA, double* x,
                                  uint32_t maxIter, double tol, uint32_t* iter, double* res, int onDevice) {
    XJ_GUARD_BEGIN
    auto last = std::chrono::high_resolution_clock::now();
    if (!p->hasMatrix()) throw xjpcg::InvalidValue("no matrix has been set.");
    p->metrics()->m_matProc = 0.0;
    p->setVec(p->matrixN(), b, diagA, onDevice != 0);
    p->metrics()->m_vecProc = elapsed(last);
    xjpcg::Results r = p->runMixed(maxIter, tol);
    if (x) p->copyX64(x, p->matrixN(), onDevice != 0);
    p->markSolved();
    *res = std::sqrt(r.rrLast / r.bb);
    if (iter) *iter = r.reportedIters;
    p->metrics()->m_solver = elapsed(last);
    if (r.status & xjpcg::kStatusBreakdown) throw xjpcg::ExecFailed("breakdown in the refinement loop.");
    if (!(*res <= tol))
        throw xjpcg::ExecFailed("exit with divergent solution after " + std::to_string(r.reportedIters) +
                                " inner iterations.");
    XJ_GUARD_END("Solver returns successfully")
}

XJPCG_Status_t xJPCG_gbSetSignatureMatrix(XJPCG_Handle_t* handle, uint32_t numChannels, const void* const* nnzBufs,
                                          const uint64_t* nnzBytes, const void* parParam, uint64_t parParamBytes,
                                          const void* rbParam, uint64_t rbParamBytes) {
    XJ_GUARD_BEGIN
    auto last = std::chrono::high_resolution_clock::now();
    if (nnzBufs == nullptr || nnzBytes == nullptr || parParam == nullptr || rbParam == nullptr)
        throw xjpcg::InvalidValue("buffer is nullptr.");
    p->setSignatureMatrix(numChannels, nnzBufs, nnzBytes, parParam, parParamBytes, rbParam, rbParamBytes);
    p->markCalled();
    p->metrics()->m_matProc = elapsed(last);
    XJ_GUARD_END("Partitioned matrix loaded successfully")
}

XJPCG_Status_t xJPCG_gbSignatureSpmv(XJPCG_Handle_t* handle, const double* x, uint32_t xLen, double* y,
                                     uint32_t yRows, uint32_t startAddr, void* frame, uint64_t frameBytes) {
    XJ_GUARD_BEGIN
    auto last = std::chrono::high_resolution_clock::now();
    if (x == nullptr) throw xjpcg::InvalidValue("Vector is nullptr.");
    p->signatureSpmv(x, xLen, y, yRows, startAddr, static_cast<unsigned char*>(frame), frameBytes);
    p->metrics()->m_solver = elapsed(last);
    XJ_GUARD_END("SpMV returns successfully")
}

XJPCG_Status_t xJPCG_gbSignatureSolve(XJPCG_Handle_t* handle, uint32_t n, const double* b, const double* diagA,
                                      double* x, uint32_t maxIter, double tol, uint32_t* iter, double* res) {
    XJ_GUARD_BEGIN
    auto last = std::chrono::high_resolution_clock::now();
    if (iter == nullptr || res == nullptr) throw xjpcg::InvalidValue("iter and res must not be null.");
    p->metrics()->m_matProc = 0.0;
    p->metrics()->m_vecProc = 0.0;
    xjpcg::Results r = p->signatureSolve(n, b, diagA, x, maxIter, tol);
    finishSolve(p, r, tol, res, iter, nullptr, last);
    XJ_GUARD_END("Solver returns successfully")
}

XJPCG_Status_t xJPCG_gbSetSignatureSumOrder(XJPCG_Handle_t* handle, int order) {
    XJ_GUARD_BEGIN
    p->setSignatureSumOrder(order);
    XJ_GUARD_END("summation order set successfully")
}

XJPCG_Status_t xJPCG_gbExportSignature(XJPCG_Handle_t* handle, XJPCG_GbSignature_t* sig) {
    XJ_GUARD_BEGIN
    p->exportSignature(sig);
    XJ_GUARD_END("signature exported successfully")
}

XJPCG_Status_t xJPCG_gbGetSignature(XJPCG_Handle_t* handle, void* rbParam, void* parParam, void* const* nnzVal) {
    XJ_GUARD_BEGIN
    p->getSignature(rbParam, parParam, nnzVal);
    XJ_GUARD_END("signature copied successfully")
}

XJPCG_Status_t xJPCG_gbAdjointSolve(XJPCG_Handle_t* handle, const double* g, const double* diagA, double* lambda,
                                    double* gradA, uint32_t maxIter, double tol, uint32_t* iter, double* res,
                                    int onDevice) {
    XJ_GUARD_BEGIN
    auto last = std::chrono::high_resolution_clock::now();
    if (g == nullptr || diagA == nullptr) throw xjpcg::InvalidValue("Vector is nullptr.");
    xjpcg::Results r = p->adjoint(g, diagA, lambda, gradA, maxIter, tol, onDevice != 0);
    *res = std::sqrt(r.rrLast / r.bb);
    if (iter) *iter = r.reportedIters;
    p->metrics()->m_solver = elapsed(last);
    if (r.status & xjpcg::kStatusBreakdown) throw xjpcg::ExecFailed("breakdown in the adjoint solve.");
    if (*res > tol)
        throw xjpcg::ExecFailed("adjoint exit with divergent solution after " + std::to_string(r.reportedIters) +
                                " iterations.");
    XJ_GUARD_END("Adjoint solver returns successfully")
}

XJPCG_Status_t xJPCG_gbEdgeGrad(XJPCG_Handle_t* handle, int64_t numEdges, const int32_t* edgeI, const int32_t* edgeJ,
                                const double* conductance, double* gradTheta, int onDevice) {
    XJ_GUARD_BEGIN
    if (edgeI == nullptr || edgeJ == nullptr || conductance == nullptr || gradTheta == nullptr)
        throw xjpcg::InvalidValue("edge array is nullptr.");
    p->edgeGrad(numEdges, edgeI, edgeJ, conductance, gradTheta, onDevice != 0);
    XJ_GUARD_END("Edge gradient returns successfully")
}

XJPCG_Status_t xJPCG_gbBatchSolve(XJPCG_Handle_t* handle, uint32_t numSystems, const int32_t* sysRowStart,
                                  const int32_t* rowPtr, const int32_t* colIdx, const double* values,
                                  const double* diagA, const double* b, double* x, uint32_t maxIter, double tol,
                                  int precision, XJPCG_GbBatchResult_t* results, int onDevice) {
    XJ_GUARD_BEGIN
    if (sysRowStart == nullptr || rowPtr == nullptr || colIdx == nullptr || values == nullptr)
        throw xjpcg::InvalidValue("Matrix is nullptr.");
    if (diagA == nullptr || b == nullptr) throw xjpcg::InvalidValue("Vector is nullptr.");
    static_assert(sizeof(XJPCG_GbBatchResult_t) == sizeof(xjpcg::BatchResult), "result layout");
    const uint32_t failed = p->batchSolve(numSystems, sysRowStart, rowPtr, colIdx, values, diagA, b, x, maxIter, tol,
                                          precision, reinterpret_cast<xjpcg::BatchResult*>(results), onDevice != 0);
    if (failed) throw xjpcg::ExecFailed(std::to_string(failed) + " of " + std::to_string(numSystems) +
                                        " systems did not reach the tolerance.");
    XJ_GUARD_END("Batched solver returns successfully")
}

XJPCG_Status_t xJPCG_gbSpmv(XJPCG_Handle_t* handle, const double* x, double* y, int onDevice) {
    XJ_GUARD_BEGIN
    if (x == nullptr || y == nullptr) throw xjpcg::InvalidValue("Vector is nullptr.");
    p->spmv(x, y, onDevice != 0);
    XJ_GUARD_END("SpMV returns successfully")
}

XJPCG_Status_t xJPCG_gbGetCsr(XJPCG_Handle_t* handle, int32_t* rowPtr, int32_t* colIdx, double* values,
                              uint32_t* perm) {
    XJ_GUARD_BEGIN
    p->getCsr(rowPtr, colIdx, values, perm);
    XJ_GUARD_END("Get CSR successfully")
}

XJPCG_Status_t xJPCG_gbGetRecords(XJPCG_Handle_t* handle, void* buf, uint64_t cap, uint64_t* count) {
    XJ_GUARD_BEGIN
    if (buf == nullptr || count == nullptr) throw xjpcg::InvalidValue("buffer is nullptr.");
    *count = p->getRecords(buf, cap);
    XJ_GUARD_END("Get records successfully")
}

XJPCG_Status_t xJPCG_gbGetInfo(const XJPCG_Handle_t* handle, XJPCG_GbInfo_t* info) {
    if (handle == nullptr) return XJPCG_STATUS_NOT_INITIALIZED;
    if (info == nullptr) return XJPCG_STATUS_INVALID_VALUE;
    impl(handle)->fillInfo(info);
    return XJPCG_STATUS_SUCCESS;
}

XJPCG_Status_t xJPCG_gbGetSpmvTuning(const XJPCG_Handle_t* handle, float* ms, int32_t* shape, int32_t cap,
                                     int32_t* count) {
    if (handle == nullptr) return XJPCG_STATUS_NOT_INITIALIZED;
    if (ms == nullptr || shape == nullptr || count == nullptr) return XJPCG_STATUS_INVALID_VALUE;
    *count = impl(handle)->tuning(ms, shape, cap);
    return XJPCG_STATUS_SUCCESS;
}

XJPCG_Status_t xJPCG_gbGetSpmvTuning32(const XJPCG_Handle_t* handle, float* ms, int32_t cap, int32_t* count) {
    if (handle == nullptr) return XJPCG_STATUS_NOT_INITIALIZED;
    if (ms == nullptr || count == nullptr) return XJPCG_STATUS_INVALID_VALUE;
    *count = impl(handle)->tuning32(ms, cap);
    return XJPCG_STATUS_SUCCESS;
}

XJPCG_Status_t xJPCG_gbGetStream(const XJPCG_Handle_t* handle, void** stream) {
    if (handle == nullptr) return XJPCG_STATUS_NOT_INITIALIZED;
    if (stream == nullptr) return XJPCG_STATUS_INVALID_VALUE;
    *stream = (void*)impl(handle)->stream();
    return XJPCG_STATUS_SUCCESS;
}

XJPCG_Status_t xJPCG_gbSetSpmvLanes(XJPCG_Handle_t* handle, int lanes) {
    XJ_GUARD_BEGIN
    p->setLanes(lanes);
    XJ_GUARD_END("SpMV lanes set successfully")
}

XJPCG_Status_t xJPCG_gbSetSpmvConfig(XJPCG_Handle_t* handle, int cfg) {
    XJ_GUARD_BEGIN
    p->setSpmvConfig(cfg);
    XJ_GUARD_END("SpMV configuration set successfully")
}

XJPCG_Status_t xJPCG_gbSetSpmvConfig32(XJPCG_Handle_t* handle, int cfg) {
    XJ_GUARD_BEGIN
    p->setSpmvConfig32(cfg);
    XJ_GUARD_END("FP32 SpMV configuration set successfully")
}

XJPCG_Status_t xJPCG_gbDiagWaitTimeout(XJPCG_Handle_t* handle, uint64_t budgetNs, uint32_t* deviceStatus,
                                       uint64_t* elapsedNs) {
    XJ_GUARD_BEGIN
    if (deviceStatus == nullptr || elapsedNs == nullptr)
        throw xjpcg::InvalidValue("deviceStatus and elapsedNs must not be null.");
    p->diagWaitTimeout(budgetNs, deviceStatus, elapsedNs);
    XJ_GUARD_END("The device wait completed")
}

XJPCG_Status_t xJPCG_gbDiagFp64Rate(XJPCG_Handle_t* handle, int32_t iters, double* dfmaPerSecond, double* ms) {
    XJ_GUARD_BEGIN
    if (dfmaPerSecond == nullptr || ms == nullptr) throw xjpcg::InvalidValue("dfmaPerSecond and ms must not be null.");
    p->diagFp64Rate(iters, dfmaPerSecond, ms);
    XJ_GUARD_END("FP64 rate measured")
}

XJPCG_Status_t xJPCG_gbDiagCheckGuards(XJPCG_Handle_t* handle, uint32_t* corrupted) {
    XJ_GUARD_BEGIN
    if (corrupted == nullptr) throw xjpcg::InvalidValue("corrupted must not be null.");
    if (!p->guardsOn()) throw xjpcg::InvalidValue("the handle was created without guard bytes (XJPCG_GUARD_BYTES).");
    std::string first;
    *corrupted = p->checkGuards(&first);
    if (*corrupted) throw xjpcg::InternalError("a kernel wrote past the end of " + first);
    XJ_GUARD_END("Guard bytes intact")
}

// The receiving side of the dSpmv transY framing, as dStoreY writes it
// (dSpmv/hw/include/impl/dStoreY.hpp:36-65): for each of numNodes frames, a
// 64-byte header word {startAddr, rows, ...} (uint32, startAddr counted in
// 32-byte memory words), then ceil(rows / 8) 64-byte data words, each stored
// as two 32-byte memory words at startAddr, startAddr + 1, ...  Every data
// word is written whole, so the zero fill of a last partial word lands in y
// too, as on the FPGA.  Host memory only; no device work.
XJPCG_Status_t xJPCG_gbStoreYFrames(const void* frames, uint64_t frameBytes, uint32_t numNodes, double* y,
                                    uint64_t yBytes, uint64_t* consumedBytes) {
    if (frames == nullptr || y == nullptr) return XJPCG_STATUS_INVALID_VALUE;
    const unsigned char* in = static_cast<const unsigned char*>(frames);
    unsigned char* out = reinterpret_cast<unsigned char*>(y);
    uint64_t pos = 0;
    for (uint32_t node = 0; node < numNodes; ++node) {
        if (pos > frameBytes || frameBytes - pos < 64) return XJPCG_STATUS_INVALID_VALUE;
        uint32_t head[2];
        std::memcpy(head, in + pos, sizeof(head));
        const uint64_t startByte = (uint64_t)head[0] * 32u;
        const uint64_t words = ((uint64_t)head[1] + 7u) / 8u;
        // rows = 0: transY still emits one data word that dStoreY never
        // reads, which would shift every later frame; refused instead.
        if (head[1] == 0) return XJPCG_STATUS_INVALID_VALUE;
        if (frameBytes - pos - 64 < words * 64) return XJPCG_STATUS_INVALID_VALUE;
        if (startByte > yBytes || yBytes - startByte < words * 64) return XJPCG_STATUS_INVALID_VALUE;
        std::memcpy(out + startByte, in + pos + 64, words * 64);
        pos += 64 + words * 64;
        if (consumedBytes) *consumedBytes = pos;
    }
    if (consumedBytes) *consumedBytes = pos;
    return XJPCG_STATUS_SUCCESS;
}

}  // extern "C"
