// pcg_handle.cpp -- host orchestration of the GB300 xJPCG solver.
#include "pcg_handle.hpp"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace xjpcg {

namespace {
// NVTX range over a host phase (header-only NVTX v3; a no-op unless a
// profiler is attached), so a timeline shows matrix set-up, tuning and
// solves by name.
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};
constexpr uint64_t kMaxRecords = 1ull << 20;  // ring of records beyond this
constexpr int kPartialSlots = 4 * 8192;       // doubles; >= 2 * max grid
// Iterations per pass of a graph's WHILE body.  Every pass of a conditional
// node costs about 5 us on GB300; the kernels after the stop return at once.
// 160^3 fp64: 0.2694 / 0.2669 / 0.2656 / 0.2651 ms per iteration with 1 / 2 /
// 4 / 8; the mixed solve 78.5 / 77.5 / 76.8 / 76.4 ms.
constexpr int kLoopUnroll = 8;

int envInt(const char* name, int dflt) {
    const char* v = std::getenv(name);
    return v ? std::atoi(v) : dflt;
}
double envDouble(const char* name, double dflt) {
    const char* v = std::getenv(name);
    return v ? std::atof(v) : dflt;
}
bool envIs(const char* name, const char* value) {
    const char* v = std::getenv(name);
    return v && std::strcmp(v, value) == 0;
}
}  // namespace

bool DevBuf::ensure(size_t b, uint64_t* generation, size_t guardBytes) {
    if (b == 0) b = 16;
    if (b <= bytes) return true;
    release();
    if (cudaMalloc(&p, b + guardBytes) != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
        return false;
    }
    if (guardBytes > 0) {
        // Allocations happen outside stream captures; the fill completes
        // before any kernel of the handle can touch the buffer.
        if (cudaMemset(static_cast<unsigned char*>(p) + b, kGuardByte, guardBytes) != cudaSuccess ||
            cudaDeviceSynchronize() != cudaSuccess) {
            cudaGetLastError();
            release();
            return false;
        }
    }
    bytes = b;
    guard = guardBytes;
    if (generation) ++*generation;
    return true;
}

PcgHandle::~PcgHandle() {
    if (m_exec) cudaGraphExecDestroy(m_exec);
    if (m_mixedExec) cudaGraphExecDestroy(m_mixedExec);
    if (m_batchExec) cudaGraphExecDestroy(m_batchExec);
    if (m_ev0) cudaEventDestroy(m_ev0);
    if (m_ev1) cudaEventDestroy(m_ev1);
    if (m_evUp0) cudaEventDestroy(m_evUp0);
    if (m_evUp1) cudaEventDestroy(m_evUp1);
    if (m_evUpIdx) cudaEventDestroy(m_evUpIdx);
    if (m_evUpVal) cudaEventDestroy(m_evUpVal);
    if (m_evIdxIn) cudaEventDestroy(m_evIdxIn);
    if (m_upStream) cudaStreamDestroy(m_upStream);
    if (m_stream) cudaStreamDestroy(m_stream);
}

void PcgHandle::check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) throw AllocFailed(std::string(what) + ": " + cudaGetErrorString(e));
    throw InternalError(std::string(what) + ": " + cudaGetErrorString(e));
}

void PcgHandle::alloc(DevBuf& b, size_t bytes, const char* what) {
    // XJPCG_FAULT=alloc: every allocation after the handle's own set-up fails
    // as a cudaMalloc failure would (host-side fault injection).
    if (m_faultAlloc && m_initDone && bytes > b.bytes)
        throw AllocFailed(std::string("device allocation failed for ") + what);
    if (!b.ensure(bytes, &m_generation, m_guardBytes))
        throw AllocFailed(std::string("device allocation failed for ") + what);
    if (m_guardBytes > 0) {
        bool known = false;
        for (const auto& g : m_guarded) known = known || g.first == &b;
        if (!known) m_guarded.emplace_back(&b, what);
    }
}

// Debug handles (XJPCG_GUARD_BYTES > 0 when the handle is created) allocate
// every buffer with guard bytes after its end, a stand-in for a memory
// checker: a kernel that writes past the end of a buffer changes them.
// Returns the number of buffers whose guard bytes changed.
uint32_t PcgHandle::checkGuards(std::string* firstBad) {
    check(cudaStreamSynchronize(m_stream), "sync");
    check(cudaStreamSynchronize(m_upStream), "sync");
    uint32_t bad = 0;
    std::vector<unsigned char> host;
    for (const auto& g : m_guarded) {
        const DevBuf* b = g.first;
        if (b->p == nullptr || b->guard == 0) continue;
        host.resize(b->guard);
        check(cudaMemcpy(host.data(), static_cast<const unsigned char*>(b->p) + b->bytes, b->guard,
                         cudaMemcpyDeviceToHost),
              "guard check");
        bool ok = true;
        for (unsigned char c : host) ok = ok && c == kGuardByte;
        if (!ok) {
            if (bad == 0 && firstBad) *firstBad = g.second;
            ++bad;
        }
    }
    return bad;
}

// XJPCG_FAULT=launch: the solver launches (graphs, or the first kernel of
// the host-driven loops) report a launch failure before anything is queued.
void PcgHandle::faultPoint(const char* what) {
    if (m_faultLaunch) check(cudaErrorLaunchFailure, what);
}

void PcgHandle::init(int device) {
    m_guardBytes = (size_t)std::max(0, envInt("XJPCG_GUARD_BYTES", 0));
    if (device >= 0) check(cudaSetDevice(device), "cudaSetDevice");
    check(cudaGetDevice(&m_device), "cudaGetDevice");
    check(cudaDeviceGetAttribute(&m_numSms, cudaDevAttrMultiProcessorCount, m_device), "cudaDeviceGetAttribute");
    check(cudaStreamCreateWithFlags(&m_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    check(cudaEventCreate(&m_ev0), "cudaEventCreate");
    check(cudaEventCreate(&m_ev1), "cudaEventCreate");
    check(cudaEventCreate(&m_evUp0), "cudaEventCreate");
    check(cudaEventCreate(&m_evUp1), "cudaEventCreate");
    check(cudaEventCreate(&m_evUpIdx), "cudaEventCreate");
    check(cudaEventCreate(&m_evUpVal), "cudaEventCreate");
    check(cudaEventCreateWithFlags(&m_evIdxIn, cudaEventDisableTiming), "cudaEventCreate");
    check(cudaStreamCreateWithFlags(&m_upStream, cudaStreamNonBlocking), "cudaStreamCreate");
    alloc(m_state, sizeof(CgState), "solver state");
    alloc(m_state32, sizeof(CgState), "solver state");
    alloc(m_partials, sizeof(double) * kPartialSlots, "reduction partials");
    alloc(m_flags, 8 * sizeof(int), "flags");
    check(cudaMemsetAsync(m_state.p, 0, sizeof(CgState), m_stream), "memset");
    check(cudaMemsetAsync(m_state32.p, 0, sizeof(CgState), m_stream), "memset");
    check(cudaStreamSynchronize(m_stream), "sync");
    m_useGraph = envInt("XJPCG_HOST_LOOP", 0) == 0;
    m_fusedUpdate = envInt("XJPCG_FUSED_UPDATE", 1) != 0;
    m_forcedLanes = envInt("XJPCG_SPMV_LANES", 0);
    m_forcedCfg = envInt("XJPCG_SPMV_CFG", -1);
    m_faultAlloc = envIs("XJPCG_FAULT", "alloc");
    m_faultLaunch = envIs("XJPCG_FAULT", "launch");
    m_initDone = true;
}

// ---------------------------------------------------------------------------
// Matrix set-up
// ---------------------------------------------------------------------------
void PcgHandle::setCooMat(uint32_t n, uint64_t nnz, const uint32_t* row, const uint32_t* col, const double* data,
                          int base) {
    Range range_("xJPCG matrix set-up (COO)");
    if (nnz > 0x7ffffff0ull) throw InvalidValue("number of non-zeros exceeds 2^31 - 16.");
    m_haveMatrix = false;
    alloc(m_inRow, sizeof(uint32_t) * nnz, "COO rows");
    alloc(m_inCol, sizeof(uint32_t) * nnz, "COO cols");
    alloc(m_inVal, sizeof(double) * nnz, "COO values");
    // The host link (about 211 GB/s here, the same through the copy engine
    // or a kernel reading host memory) bounds the upload, so the values travel
    // on a side stream after the indices while the index conversion runs;
    // the value gather waits for them.
    check(cudaEventRecord(m_evUp0, m_stream), "event");
    check(cudaMemcpyAsync(m_inRow.p, row, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice, m_stream), "H2D rows");
    check(cudaMemcpyAsync(m_inCol.p, col, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice, m_stream), "H2D cols");
    check(cudaEventRecord(m_evIdxIn, m_stream), "event");
    check(cudaEventRecord(m_evUpIdx, m_stream), "event");
    check(cudaStreamWaitEvent(m_upStream, m_evIdxIn, 0), "stream wait");
    check(cudaEventRecord(m_evUpVal, m_upStream), "event");
    check(cudaMemcpyAsync(m_inVal.p, data, sizeof(double) * nnz, cudaMemcpyHostToDevice, m_upStream), "H2D values");
    check(cudaEventRecord(m_evUp1, m_upStream), "event");
    m_uploadTimed = true;
    const uint64_t nnzPad = (nnz + 3) / 4 * 4 + 4;
    alloc(m_rowptr, sizeof(int) * ((size_t)n + 1 + kRowptrPad), "CSR row pointers");
    alloc(m_col, sizeof(int) * nnzPad, "CSR columns");
    alloc(m_val, sizeof(double) * nnzPad, "CSR values");
    alloc(m_perm, sizeof(uint32_t) * (nnz + 1), "CSR permutation");
    alloc(m_counts, sizeof(int) * ((size_t)n + 2), "conversion counts");
    alloc(m_fill, sizeof(int) * ((size_t)n + 1), "conversion fill");
    alloc(m_blockSums, sizeof(int) * ((size_t)scan_block_count((int)std::max<uint64_t>(n + 1, nnz + 1)) + 16),
          "scan scratch");
    alloc(m_keys, sizeof(uint64_t) * (nnz + 1), "conversion keys");
    ConvertScratch s;
    s.counts = m_counts.as<int>();
    s.fill = m_fill.as<int>();
    s.blockSums = m_blockSums.as<int>();
    s.keys = m_keys.as<uint64_t>();
    s.flags = m_flags.as<int>();
    int herr = 0;
    const cudaError_t ce = coo_to_csr(m_stream, (int)n, (int64_t)nnz, m_inRow.as<uint32_t>(),
                                      m_inCol.as<uint32_t>(), base, m_rowptr.as<int>(), m_col.as<int>(),
                                      m_perm.as<uint32_t>(), s, &herr);
    check(cudaStreamWaitEvent(m_stream, m_evUp1, 0), "stream wait");  // the values have landed
    if (ce != cudaSuccess || (herr & kStatusIndexError)) {
        cudaStreamSynchronize(m_stream);  // no value copy stays in flight past a failed call
        check(ce, "COO to CSR conversion");
        throw InvalidValue("matrix index out of range [base, n + base).");
    }
    check(gather_values(m_stream, (int64_t)nnz, m_perm.as<uint32_t>(), m_inVal.as<double>(), m_val.as<double>()),
          "value gather");
    m_n = n;
    m_nnz = nnz;
    m_kind = 1;
    finishMatrix();
}

void PcgHandle::updateCooValues(uint32_t n, uint64_t nnz, const double* data) {
    Range range_("xJPCG values update");
    // Signature::checkUpdateDim (signature.hpp:575-583) raises SpmInvalidValue,
    // which the reference reports as INTERNAL_ERROR through std::exception.
    if (!m_haveMatrix || n != m_n || nnz != m_nnz)
        throw InternalError("Invalid dimension and/or number of nnzs used for updateing matrix.");
    alloc(m_inVal, sizeof(double) * nnz, "COO values");
    check(cudaMemcpyAsync(m_inVal.p, data, sizeof(double) * nnz, cudaMemcpyHostToDevice, m_stream), "H2D values");
    check(gather_values(m_stream, (int64_t)nnz, m_perm.as<uint32_t>(), m_inVal.as<double>(), m_val.as<double>()),
          "value gather");
    m_val32Valid = false;
    refreshSellValues();
    check(cudaStreamSynchronize(m_stream), "sync");
}

void PcgHandle::setCsrMat(uint32_t n, uint64_t nnz, const int32_t* rowPtr, const int32_t* colIdx,
                          const double* data, int base) {
    Range range_("xJPCG matrix set-up (CSR)");
    // Row indices are expanded on the host side of the copy: the CSR row
    // pointer is small (n + 1) and validated here; the rest is the COO path.
    if ((int64_t)rowPtr[0] - base != 0 || (uint64_t)((int64_t)rowPtr[n] - base) != nnz)
        throw InvalidValue("CSR row pointer does not span [0, nnz).");
    std::vector<uint32_t> rows(nnz);
    for (uint32_t i = 0; i < n; ++i) {
        const int64_t s = (int64_t)rowPtr[i] - base, e = (int64_t)rowPtr[i + 1] - base;
        if (e < s) throw InvalidValue("CSR row pointer is not monotone.");
        for (int64_t k = s; k < e; ++k) rows[k] = i + (uint32_t)base;
    }
    setCooMat(n, nnz, rows.data(), reinterpret_cast<const uint32_t*>(colIdx), data, base);
    m_kind = 3;
}

void PcgHandle::updateCsrValues(uint32_t n, uint64_t nnz, const double* data) { updateCooValues(n, nnz, data); }

void PcgHandle::setCscSymMat(uint32_t n, uint64_t nnzHalf, const int64_t* rowIdx, const int64_t* colPtr,
                             const double* data, int base) {
    Range range_("xJPCG matrix set-up (CSC)");
    // PCGImpl::setCscSymMat: full nnz = 2 * nnz - n (pcgImp.hpp:87).
    const uint64_t nnzFull = (uint32_t)(nnzHalf * 2 - n);
    if (base == 1 && colPtr[0] < 1)
        throw InternalError("from getCooDatFromCscSym in gen_signature.hpp, colPtr[0] start from 1 in FORTRAN storage mode.");
    if (nnzHalf > 0x7ffffff0ull || nnzFull > 0x7ffffff0ull) throw InvalidValue("number of non-zeros exceeds 2^31 - 16.");
    alloc(m_inIdx64, sizeof(int64_t) * nnzHalf, "CSC row indices");
    alloc(m_inPtr64, sizeof(int64_t) * ((size_t)n + 1), "CSC column pointers");
    alloc(m_cscScratch, sizeof(int) * (nnzHalf + 8), "CSC scratch");
    alloc(m_blockSums, sizeof(int) * ((size_t)scan_block_count((int)std::max<uint64_t>(nnzHalf + 1, nnzFull + 1)) + 16),
          "scan scratch");
    DevBuf halfVal;
    if (!halfVal.ensure(sizeof(double) * nnzHalf, nullptr)) throw AllocFailed("device allocation failed for CSC values");
    check(cudaMemcpyAsync(m_inIdx64.p, rowIdx, sizeof(int64_t) * nnzHalf, cudaMemcpyHostToDevice, m_stream), "H2D");
    check(cudaMemcpyAsync(m_inPtr64.p, colPtr, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, m_stream),
          "H2D");
    check(cudaMemcpyAsync(halfVal.p, data, sizeof(double) * nnzHalf, cudaMemcpyHostToDevice, m_stream), "H2D");
    alloc(m_inRow, sizeof(uint32_t) * nnzFull, "COO rows");
    alloc(m_inCol, sizeof(uint32_t) * nnzFull, "COO cols");
    alloc(m_inVal, sizeof(double) * nnzFull, "COO values");
    int herr = 0;
    check(cscsym_expand(m_stream, (int)n, (int64_t)nnzHalf, (int64_t)nnzFull, m_inIdx64.as<int64_t>(),
                        m_inPtr64.as<int64_t>(), halfVal.as<double>(), base, m_inRow.as<uint32_t>(),
                        m_inCol.as<uint32_t>(), m_inVal.as<double>(), nullptr, m_cscScratch.as<int>(),
                        m_blockSums.as<int>(), &herr),
          "symmetric CSC expansion");
    if (herr & kStatusIndexError) throw InvalidValue("matrix index out of range [base, n + base).");
    if (herr & kStatusCountError)
        throw InternalError("from loadCscSym in matrix_params.hpp, failed to convert indices from CscSym to COO format.");
    check(cudaStreamSynchronize(m_stream), "sync");
    // The expanded list is a COO input with base 0.
    std::vector<uint32_t> dummy;
    const uint64_t nnz = nnzFull;
    const uint64_t nnzPad = (nnz + 3) / 4 * 4 + 4;
    alloc(m_rowptr, sizeof(int) * ((size_t)n + 1 + kRowptrPad), "CSR row pointers");
    alloc(m_col, sizeof(int) * nnzPad, "CSR columns");
    alloc(m_val, sizeof(double) * nnzPad, "CSR values");
    alloc(m_perm, sizeof(uint32_t) * (nnz + 1), "CSR permutation");
    alloc(m_counts, sizeof(int) * ((size_t)n + 2), "conversion counts");
    alloc(m_fill, sizeof(int) * ((size_t)n + 1), "conversion fill");
    alloc(m_keys, sizeof(uint64_t) * (nnz + 1), "conversion keys");
    ConvertScratch s;
    s.counts = m_counts.as<int>();
    s.fill = m_fill.as<int>();
    s.blockSums = m_blockSums.as<int>();
    s.keys = m_keys.as<uint64_t>();
    s.flags = m_flags.as<int>();
    check(coo_to_csr(m_stream, (int)n, (int64_t)nnz, m_inRow.as<uint32_t>(), m_inCol.as<uint32_t>(), 0,
                     m_rowptr.as<int>(), m_col.as<int>(), m_perm.as<uint32_t>(), s, &herr),
          "COO to CSR conversion");
    if (herr & kStatusIndexError) throw InvalidValue("matrix index out of range [base, n + base).");
    check(gather_values(m_stream, (int64_t)nnz, m_perm.as<uint32_t>(), m_inVal.as<double>(), m_val.as<double>()),
          "value gather");
    m_n = n;
    m_nnz = nnz;
    m_nnzHalf = nnzHalf;
    m_kind = 2;
    finishMatrix();
}

void PcgHandle::updateCscSymValues(uint32_t n, uint64_t nnzHalf, const int64_t* rowIdx, const int64_t* colPtr,
                                   const double* data, int base) {
    const uint64_t nnzFull = (uint32_t)(nnzHalf * 2 - n);
    if (!m_haveMatrix || n != m_n || nnzFull != m_nnz)
        throw InternalError("Invalid dimension and/or number of nnzs used for updateing matrix.");
    if (rowIdx == nullptr || colPtr == nullptr) throw InvalidValue("Matrix is nullptr.");
    if (base == 1 && colPtr[0] < 1)
        throw InternalError("from getCooDatFromCscSym in gen_signature.hpp, colPtr[0] start from 1 in FORTRAN storage mode.");
    alloc(m_inIdx64, sizeof(int64_t) * nnzHalf, "CSC row indices");
    alloc(m_inPtr64, sizeof(int64_t) * ((size_t)n + 1), "CSC column pointers");
    alloc(m_cscScratch, sizeof(int) * (nnzHalf + 8), "CSC scratch");
    alloc(m_blockSums, sizeof(int) * ((size_t)scan_block_count((int)(nnzHalf + 1)) + 16), "scan scratch");
    DevBuf halfVal;
    if (!halfVal.ensure(sizeof(double) * nnzHalf, nullptr)) throw AllocFailed("device allocation failed for CSC values");
    check(cudaMemcpyAsync(m_inIdx64.p, rowIdx, sizeof(int64_t) * nnzHalf, cudaMemcpyHostToDevice, m_stream), "H2D");
    check(cudaMemcpyAsync(m_inPtr64.p, colPtr, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, m_stream),
          "H2D");
    check(cudaMemcpyAsync(halfVal.p, data, sizeof(double) * nnzHalf, cudaMemcpyHostToDevice, m_stream), "H2D");
    alloc(m_inVal, sizeof(double) * nnzFull, "COO values");
    int herr = 0;
    // getCooDatFromCscSym re-expands the values with the new indices
    // (gen_signature.hpp:73-112); the stored permutation maps them to CSR.
    check(cscsym_expand(m_stream, (int)n, (int64_t)nnzHalf, (int64_t)nnzFull, m_inIdx64.as<int64_t>(),
                        m_inPtr64.as<int64_t>(), halfVal.as<double>(), base, nullptr, nullptr, m_inVal.as<double>(),
                        nullptr, m_cscScratch.as<int>(), m_blockSums.as<int>(), &herr),
          "symmetric CSC expansion");
    if (herr & kStatusIndexError) throw InvalidValue("matrix index out of range [base, n + base).");
    if (herr & kStatusCountError)
        throw InternalError("from getCooDatFromCscSym in gen_signature.hpp, failed to convert data from CscSym to COO format.");
    check(gather_values(m_stream, (int64_t)nnzFull, m_perm.as<uint32_t>(), m_inVal.as<double>(), m_val.as<double>()),
          "value gather");
    m_val32Valid = false;
    refreshSellValues();
    check(cudaStreamSynchronize(m_stream), "sync");
}

void PcgHandle::finishMatrix() {
    // Zero the 4-element alignment pad past nnz (read by the bulk copies).
    const uint64_t nnzPad = (m_nnz + 3) / 4 * 4 + 4;
    check(cudaMemsetAsync(m_val.as<double>() + m_nnz, 0, sizeof(double) * (nnzPad - m_nnz), m_stream), "memset");
    check(cudaMemsetAsync(m_col.as<int>() + m_nnz, 0, sizeof(int) * (nnzPad - m_nnz), m_stream), "memset");
    check(cudaMemsetAsync(m_rowptr.as<int>() + m_n + 1, 0, sizeof(int) * kRowptrPad, m_stream), "memset");
    m_val32Valid = false;
    m_sellState = 0;
    m_sell32Valid = false;
    m_ssState = 0;
    m_ss32Valid = false;
    m_psState = 0;
    m_ps32Valid = false;
    m_mergeTilesValid = false;
    ++m_structGen;
    ++m_valGen;
    alloc(m_hashBuf, 16, "structure fingerprint");
    check(struct_hash(m_stream, (int)m_n, (int64_t)m_nnz, m_rowptr.as<int>(), m_col.as<int>(),
                      m_hashBuf.as<unsigned long long>(), &m_structHash),
          "structure fingerprint");
    m_haveMatrix = true;
    ensureVectors(m_n);
    tuneSpmv();
}

void PcgHandle::setLanes(int lanes) {
    m_forcedLanes = lanes;
    if (m_haveMatrix) tuneSpmv();
}

// Runs the bounded-wait diagnostic on the handle's stream: a wait that can
// never complete must give up after budgetNs and report the timeout the way a
// solve does (INTERNAL_ERROR), and the context stays usable.
void PcgHandle::diagWaitTimeout(uint64_t budgetNs, uint32_t* deviceStatus, uint64_t* elapsedNs) {
    if (budgetNs == 0 || budgetNs > 1000000000ull)
        throw InvalidValue("the wait budget must be between 1 ns and 1 s.");
    alloc(m_diagBuf, 16, "wait diagnostic");
    check(cudaMemsetAsync(m_diagBuf.p, 0xff, 16, m_stream), "memset");
    check(wait_probe_launch(m_stream, budgetNs, m_diagBuf.as<uint32_t>()), "wait diagnostic");
    uint32_t out[3] = {0u, 0u, 0u};
    check(cudaMemcpyAsync(out, m_diagBuf.p, sizeof(out), cudaMemcpyDeviceToHost, m_stream), "wait diagnostic");
    check(cudaStreamSynchronize(m_stream), "wait diagnostic");
    *deviceStatus = out[0];
    *elapsedNs = (uint64_t)out[1] | ((uint64_t)out[2] << 32);
    if (out[0] & kStatusWaitTimeout) throw InternalError("Run kernel failed: a device wait timed out.");
}

// Times the FP64 issue-rate probe on the handle's stream with CUDA events:
// one warm-up launch, then the best of three timed launches.
void PcgHandle::diagFp64Rate(int32_t iters, double* dfmaPerSecond, double* ms) {
    if (iters < 1 || iters > (1 << 24)) throw InvalidValue("iters must be between 1 and 2^24.");
    const int grid = fp64_rate_grid(m_numSms);
    alloc(m_diagBuf, (size_t)grid * 256 * sizeof(double), "fp64 rate diagnostic");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    check(cudaEventCreate(&e0), "cudaEventCreate");
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        throw InternalError("cudaEventCreate failed.");
    }
    float best = -1.0f;
    cudaError_t err = fp64_rate_launch(m_stream, grid, iters, m_diagBuf.as<double>());
    for (int rep = 0; rep < 3 && err == cudaSuccess; ++rep) {
        err = cudaEventRecord(e0, m_stream);
        if (err == cudaSuccess) err = fp64_rate_launch(m_stream, grid, iters, m_diagBuf.as<double>());
        if (err == cudaSuccess) err = cudaEventRecord(e1, m_stream);
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        float t = 0.0f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
        if (err == cudaSuccess && (best < 0.0f || t < best)) best = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    check(err, "fp64 rate diagnostic");
    *ms = best;
    *dfmaPerSecond = best > 0.0f ? fp64_rate_dfma(grid, iters) / (best * 1e-3) : 0.0;
}

void PcgHandle::setSpmvConfig32(int cfg) {
    if (cfg < -1) throw InvalidValue("SpMV configuration index must be -1 (tuned) or at least 0.");
    if (cfg >= numSpmvCfgs()) throw InvalidValue("no such SpMV configuration.");
    m_forcedCfg32 = cfg;
    m_tuned32Gen = ~0ull;  // chosen again at the next mixed solve
}

void PcgHandle::setSpmvConfig(int cfg) {
    if (cfg < -1) throw InvalidValue("SpMV configuration index must be -1 (tuned) or at least 0.");
    const int old = m_forcedCfg;
    m_forcedCfg = cfg;
    if (!m_haveMatrix) return;
    try {
        tuneSpmv();
    } catch (...) {
        m_forcedCfg = old;  // a configuration that cannot run is not kept
        throw;
    }
}

// Picks the SpMV configuration by timing every one on the stored matrix
// (plain mode, x = p buffer), median of three launches each.
void PcgHandle::refreshSellValues() {
    ++m_valGen;
    m_sell32Valid = false;
    m_ss32Valid = false;
    if (m_sellState == 1)
        check(sell_fill<double>(m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(), m_val.as<double>(),
                                m_sliceOff.as<int>(), nullptr, m_sellVal.as<double>()),
              "sliced fill");
    m_ps32Valid = false;
    if (m_psState == 1)
        check(sellpat_fill<double>(m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(), m_val.as<double>(),
                                   m_psSliceOff.as<int>(), m_psPatLen.as<int>(), m_psPatNew.as<int>(),
                                   m_psPatIdx.as<int>(), m_psPatOff.as<int>(), m_psGenOff.as<int>(), m_psVal.as<double>(),
                                   nullptr, nullptr, false),
              "shared-offset fill");
    if (m_ssState == 1)
        check(sellsort_fill<double>(m_stream, (int)m_n, m_ssLong, m_rowptr.as<int>(), m_col.as<int>(),
                                    m_val.as<double>(), m_ssSorted.as<int>(), m_ssSliceOff.as<int>(), nullptr,
                                    m_ssVal.as<double>()),
              "sorted sliced fill");
}

// Configuration index space: [0, ncsr) staged CSR shapes, [ncsr, ncsr +
// nsell) sliced unroll depths, then the sorted-sliced unroll depths, then the
// merge-path kernel.
int PcgHandle::numSpmvCfgs() const { return mergeCfg() + 1; }

int PcgHandle::patCfg0() const { return spmv_num_configs() + sell_num_configs(); }

int PcgHandle::sortedCfg0() const { return patCfg0() + sellpat_num_configs(); }

int PcgHandle::mergeCfg() const { return sortedCfg0() + sellsort_num_configs(); }

bool PcgHandle::isSell(int cfg) const {
    return cfg >= spmv_num_configs() && cfg < spmv_num_configs() + sell_num_configs();
}

bool PcgHandle::isSellNarrow(int cfg) const { return isSell(cfg) && sell_config_narrow(cfg - spmv_num_configs()); }

bool PcgHandle::isSorted(int cfg) const { return cfg >= sortedCfg0() && cfg < mergeCfg(); }

bool PcgHandle::isPat(int cfg) const { return cfg >= patCfg0() && cfg < sortedCfg0(); }

bool PcgHandle::isMerge(int cfg) const { return cfg == mergeCfg(); }

uint32_t PcgHandle::layoutCode(int cfg) const {
    if (isMerge(cfg)) return 2u;
    if (isPat(cfg)) return 5u;
    if (isSorted(cfg)) return 4u;
    if (isSellNarrow(cfg)) return 3u;
    return isSell(cfg) ? 1u : 0u;
}

// Builds (once per matrix) the sliced copy with slice-shared column offsets.
// Offered for matrices the plain sliced layout suits.
bool PcgHandle::ensurePat() {
    if (m_psState == 1) return true;
    if (m_psState == 2) return false;
    if (!ensureSell()) {
        m_psState = 2;
        return false;
    }
    const int n = (int)m_n;
    const int nslices = (n + 31) / 32;
    const size_t sb = sizeof(int) * ((size_t)nslices + 1);
    for (DevBuf* b : {&m_psSliceOff, &m_psPatLen, &m_psPatNew, &m_psPatIdx, &m_psGenOff}) alloc(*b, sb, "shared-offset slices");
    alloc(m_psPatOff, sb, "shared-offset patterns");
    alloc(m_blockSums, sizeof(int) * ((size_t)scan_block_count(std::max(nslices, n) + 1) + 16), "scan scratch");
    int64_t tot[3] = {0, 0, 0};
    check(sellpat_plan(m_stream, n, m_rowptr.as<int>(), m_col.as<int>(), m_psSliceOff.as<int>(), m_psPatLen.as<int>(),
                       m_psPatNew.as<int>(), m_psPatIdx.as<int>(), m_psGenOff.as<int>(), m_blockSums.as<int>(), tot),
          "shared-offset layout");
    if (tot[0] > 0x7fffff00ll) {
        m_psState = 2;
        return false;
    }
    int64_t patTotal = 0;
    check(sellpat_index(m_stream, n, m_psPatLen.as<int>(), m_psPatNew.as<int>(), m_psPatIdx.as<int>(), (int)tot[2],
                        m_psPatOff.as<int>(), m_blockSums.as<int>(), &patTotal),
          "shared-offset patterns");
    alloc(m_psPat, sizeof(int) * ((size_t)patTotal + 32), "shared offsets");
    alloc(m_psGcol, sizeof(int) * ((size_t)tot[1] + 32), "shared-offset general columns");
    alloc(m_psVal, sizeof(double) * ((size_t)tot[0] + 32), "shared-offset values");
    check(sellpat_fill<double>(m_stream, n, m_rowptr.as<int>(), m_col.as<int>(), m_val.as<double>(),
                               m_psSliceOff.as<int>(), m_psPatLen.as<int>(), m_psPatNew.as<int>(), m_psPatIdx.as<int>(),
                               m_psPatOff.as<int>(), m_psGenOff.as<int>(), m_psVal.as<double>(), m_psPat.as<int>(),
                               m_psGcol.as<int>(), true),
          "shared-offset fill");
    m_psTotal = tot[0];
    m_psState = 1;
    m_ps32Valid = false;
    return true;
}

// Builds (once per matrix) the length-sorted sliced copy.  Only offered when
// the plain sliced layout is rejected or pads more than 20 %: for matrices
// with near-uniform rows sorting buys nothing and costs set-up time.
bool PcgHandle::ensureSorted() {
    if (m_ssState == 1) return true;
    if (m_ssState == 2) return false;
    if (ensureSell() && m_sellPadRatio <= 1.2) {
        m_ssState = 2;
        return false;
    }
    const int n = (int)m_n;
    const int tiles = sellsort_tiles(n);
    const int binsTotal = sellsort_bins() * tiles;
    alloc(m_ssSorted, sizeof(int) * ((size_t)n + 32), "sorted rows");
    alloc(m_ssHist, sizeof(int) * ((size_t)binsTotal + 1), "sorted-row histogram");
    alloc(m_ssStart, sizeof(int) * ((size_t)binsTotal + 1), "sorted-row histogram");
    alloc(m_blockSums, sizeof(int) * ((size_t)scan_block_count(std::max(binsTotal, n) + 1) + 16), "scan scratch");
    int nLong = 0;
    check(sellsort_order(m_stream, n, m_rowptr.as<int>(), m_ssHist.as<int>(), m_ssStart.as<int>(),
                         m_blockSums.as<int>(), m_ssSorted.as<int>(), &nLong),
          "row sort");
    const int nSlices = (n - nLong + 31) / 32;
    alloc(m_ssSliceOff, sizeof(int) * ((size_t)nSlices + 1), "sorted slice offsets");
    int64_t total = 0;
    check(sellsort_slices(m_stream, n, nLong, m_rowptr.as<int>(), m_ssSorted.as<int>(), m_ssSliceOff.as<int>(),
                          m_blockSums.as<int>(), &total),
          "sorted slices");
    if (total > 0x7fffff00ll) {
        m_ssState = 2;
        return false;
    }
    alloc(m_ssCol, sizeof(int) * ((size_t)total + 32), "sorted sliced columns");
    alloc(m_ssVal, sizeof(double) * ((size_t)total + 32), "sorted sliced values");
    check(sellsort_fill<double>(m_stream, n, nLong, m_rowptr.as<int>(), m_col.as<int>(), m_val.as<double>(),
                                m_ssSorted.as<int>(), m_ssSliceOff.as<int>(), m_ssCol.as<int>(), m_ssVal.as<double>()),
          "sorted sliced fill");
    m_ssLong = nLong;
    m_ssTotal = total;
    m_ssState = 1;
    m_ss32Valid = false;
    return true;
}

void PcgHandle::ensureMergeScratch() {
    const int nt = merge_tiles((int)m_n, (int64_t)m_nnz);
    if (m_mergeTilesValid && (size_t)nt + 1 <= m_mergeTile.bytes / sizeof(int)) return;
    alloc(m_mergeTile, sizeof(int) * ((size_t)nt + 2), "merge tile rows");
    check(merge_partition(m_stream, (int)m_n, (int)m_nnz, m_rowptr.as<int>(), m_mergeTile.as<int>()), "merge tiles");
    m_mergeTilesValid = true;
    alloc(m_mergeRow, sizeof(int) * ((size_t)nt + 1), "merge carries");
    alloc(m_mergeVal, sizeof(double) * ((size_t)nt + 1), "merge carries");
    alloc(m_mergePart, sizeof(double) * ((size_t)nt + merge_fixup_grid(nt) + 1), "merge partials");
}

int PcgHandle::spmvGrid64(int cfg) {
    if (isMerge(cfg)) {
        ensureMergeScratch();
        return merge_tiles((int)m_n, (int64_t)m_nnz);
    }
    if (isSorted(cfg))
        return ensureSorted() ? sellsort_grid<double>(cfg - sortedCfg0(), (int)m_n, m_ssLong, m_numSms) : 0;
    if (isPat(cfg)) return ensurePat() ? sellpat_grid<double>(cfg - patCfg0(), (int)m_n, m_numSms) : 0;
    if (!isSell(cfg)) return spmv_grid<double>(cfg, (int)m_n, m_numSms);
    if (!ensureSell() || (isSellNarrow(cfg) && !m_sellNarrow)) return 0;
    return sell_grid<double>(cfg - spmv_num_configs(), (int)m_n, m_numSms);
}

int PcgHandle::spmvGrid32(int cfg) {
    if (isMerge(cfg)) {
        ensureMergeScratch();
        return merge_tiles((int)m_n, (int64_t)m_nnz);
    }
    if (isSorted(cfg))
        return ensureSorted() ? sellsort_grid<float>(cfg - sortedCfg0(), (int)m_n, m_ssLong, m_numSms) : 0;
    if (isPat(cfg)) return ensurePat() ? sellpat_grid<float>(cfg - patCfg0(), (int)m_n, m_numSms) : 0;
    if (!isSell(cfg)) return spmv_grid<float>(cfg, (int)m_n, m_numSms);
    if (!ensureSell() || (isSellNarrow(cfg) && !m_sellNarrow)) return 0;
    return sell_grid<float>(cfg - spmv_num_configs(), (int)m_n, m_numSms);
}

cudaError_t PcgHandle::spmv64(int cfg, int grid, const double* x, double* y, const double* b, CgState* st,
                              double* part, int mode, const uint32_t* done) {
    if (isMerge(cfg) && !m_mergeTilesValid) return cudaErrorInvalidValue;
    if (isMerge(cfg)) {
        const int m = mode == kSpmvResidual ? kSpmvPlain : mode;
        cudaError_t e = spmv_merge_launch<double>(m_stream, (int)m_n, (int)m_nnz, m_rowptr.as<int>(), m_col.as<int>(),
                                                  m_val.as<double>(), x, y, m_mergeTile.as<int>(),
                                                  m_mergeRow.as<int>(), m_mergeVal.p,
                                                  m_mergePart.as<double>(), st, m, done);
        if (e != cudaSuccess || mode != kSpmvResidual) return e;
        return residual_finish_launch<double>(m_stream, (int)m_n, b, y, part, st, done);
    }
    // a layout whose copy was not built (or was rejected) is never launched
    if ((isSorted(cfg) && m_ssState != 1) || (isSell(cfg) && m_sellState != 1) ||
        (isSellNarrow(cfg) && !m_sellNarrow) || (isPat(cfg) && m_psState != 1))
        return cudaErrorInvalidValue;
    if (isPat(cfg))
        return spmv_sellpat_launch<double>(cfg - patCfg0(), grid, m_stream, (int)m_n, m_psSliceOff.as<int>(),
                                           m_psPatLen.as<int>(), m_psPatIdx.as<int>(), m_psPatOff.as<int>(),
                                           m_psGenOff.as<int>(), m_psPat.as<int>(), m_psGcol.as<int>(),
                                           m_psVal.as<double>(), x, y, b, st, part, mode, done);
    if (isSorted(cfg))
        return spmv_sellsort_launch<double>(cfg - sortedCfg0(), grid, m_stream, (int)m_n, m_ssLong,
                                            m_ssSorted.as<int>(), m_ssSliceOff.as<int>(), m_ssCol.as<int>(),
                                            m_ssVal.as<double>(), m_rowptr.as<int>(), m_col.as<int>(),
                                            m_val.as<double>(), x, y, b, st, part, mode, done);
    if (!isSell(cfg))
        return spmv_launch<double>(cfg, grid, m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(),
                                   m_val.as<double>(), x, y, b, st, part, mode, done);
    return spmv_sell_launch<double>(cfg - spmv_num_configs(), grid, m_stream, (int)m_n, m_sliceOff.as<int>(),
                                    m_sellCol.as<int>(), m_sellNarrow ? m_sellCol16.as<int16_t>() : nullptr,
                                    m_sellVal.as<double>(), x, y, b, st, part, mode, done);
}

cudaError_t PcgHandle::spmv32(int cfg, int grid, const float* x, float* y, const float* b, CgState* st,
                              double* part, int mode, const uint32_t* done) {
    if (isMerge(cfg) && (!m_mergeTilesValid || !m_val32Valid)) return cudaErrorInvalidValue;
    if (isMerge(cfg))  // the fp32 inner loop only uses the kCgDot mode
        return spmv_merge_launch<float>(m_stream, (int)m_n, (int)m_nnz, m_rowptr.as<int>(), m_col.as<int>(),
                                        m_val32.as<float>(), x, y, m_mergeTile.as<int>(), m_mergeRow.as<int>(),
                                        m_mergeVal.p,
                                        m_mergePart.as<double>(), st, mode, done);
    if ((isSorted(cfg) && (m_ssState != 1 || !m_ss32Valid)) || (isSell(cfg) && (m_sellState != 1 || !m_sell32Valid)) ||
        (isSellNarrow(cfg) && !m_sellNarrow) || (isPat(cfg) && (m_psState != 1 || !m_ps32Valid)) || !m_val32Valid)
        return cudaErrorInvalidValue;
    if (isPat(cfg))
        return spmv_sellpat_launch<float>(cfg - patCfg0(), grid, m_stream, (int)m_n, m_psSliceOff.as<int>(),
                                          m_psPatLen.as<int>(), m_psPatIdx.as<int>(), m_psPatOff.as<int>(),
                                          m_psGenOff.as<int>(), m_psPat.as<int>(), m_psGcol.as<int>(),
                                          m_psVal32.as<float>(), x, y, b, st, part, mode, done);
    if (isSorted(cfg))
        return spmv_sellsort_launch<float>(cfg - sortedCfg0(), grid, m_stream, (int)m_n, m_ssLong,
                                           m_ssSorted.as<int>(), m_ssSliceOff.as<int>(), m_ssCol.as<int>(),
                                           m_ssVal32.as<float>(), m_rowptr.as<int>(), m_col.as<int>(),
                                           m_val32.as<float>(), x, y, b, st, part, mode, done);
    if (!isSell(cfg))
        return spmv_launch<float>(cfg, grid, m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(),
                                  m_val32.as<float>(), x, y, b, st, part, mode, done);
    return spmv_sell_launch<float>(cfg - spmv_num_configs(), grid, m_stream, (int)m_n, m_sliceOff.as<int>(),
                                   m_sellCol.as<int>(), m_sellNarrow ? m_sellCol16.as<int16_t>() : nullptr,
                                   m_sellVal32.as<float>(), x, y, b, st, part, mode, done);
}

// Builds (once per matrix) the sliced copy used by the SELL kernels.  Returns
// false when padding would exceed half the stored entries (irregular rows),
// in which case the sliced configurations are not offered.
bool PcgHandle::ensureSell() {
    if (m_sellState == 1) return true;
    if (m_sellState == 2) return false;
    const int nslices = ((int)m_n + 31) / 32;
    alloc(m_sliceOff, sizeof(int) * ((size_t)nslices + 1), "slice offsets");
    alloc(m_blockSums, sizeof(int) * ((size_t)scan_block_count(nslices + 1) + 16), "scan scratch");
    int64_t total = 0;
    check(sell_build(m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(), m_val.as<double>(), m_sliceOff.as<int>(),
                     m_blockSums.as<int>(), &total),
          "sliced layout");
    // Padding of the phantom rows past n in the last slice is a fixed cost
    // and does not count against the layout.
    int lastOff = 0;
    check(cudaMemcpyAsync(&lastOff, m_sliceOff.as<int>() + nslices - 1, sizeof(int), cudaMemcpyDeviceToHost, m_stream),
          "D2H");
    check(cudaStreamSynchronize(m_stream), "sync");
    const int64_t phantom = (int64_t)(nslices * 32 - (int64_t)m_n) * ((total - lastOff) / 32);
    m_sellPadRatio = (double)(total - phantom) / (double)std::max<uint64_t>(m_nnz, 1);
    if ((uint64_t)(total - phantom) > m_nnz + m_nnz / 2 + 64 || total > 0x7fffff00ll) {
        m_sellState = 2;
        return false;
    }
    alloc(m_sellCol, sizeof(int) * ((size_t)total + 32), "sliced columns");
    alloc(m_sellVal, sizeof(double) * ((size_t)total + 32), "sliced values");
    check(sell_fill<double>(m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(), m_val.as<double>(),
                            m_sliceOff.as<int>(), m_sellCol.as<int>(), m_sellVal.as<double>()),
          "sliced fill");
    bool fits = false;
    check(sell_narrow_fits(m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(), m_blockSums.as<int>(), &fits),
          "sliced width");
    m_sellNarrow = fits;
    if (fits) {
        alloc(m_sellCol16, sizeof(int16_t) * ((size_t)total + 64), "sliced column offsets");
        check(sell_fill_narrow(m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(), m_sliceOff.as<int>(),
                               m_sellCol16.as<int16_t>()),
              "sliced offsets");
    }
    m_sellTotal = total;
    m_sellState = 1;
    m_sell32Valid = false;
    return true;
}

// Times the SpMV configurations (plain mode, x = p, FP64 or FP32) and returns
// the fastest (-1 when none can launch).  Sliced layouts go first: on matrices they suit they are the
// fastest, and a good early time lets the rest be judged quickly.  Each
// configuration gets one launch (warm-up, timed); one that is over 1.5 times
// the best so far keeps that time, the others get three more and keep the
// median.
int PcgHandle::timeConfigs(bool fp32, std::vector<float>& out) {
    const int ncfg = numSpmvCfgs();
    std::vector<int> order;
    // Rows of near-uniform length (the sliced copy pads at most 10 %): the
    // sliced kernels move the fewest bytes with the least overhead, so only
    // they are timed; the staged-CSR, length-sorted and merge-path kernels
    // are left out.
    const bool uniformRows = ensureSell() && m_sellPadRatio <= 1.1;
    for (int c = spmv_num_configs(); c < ncfg; ++c)
        if (!uniformRows || isSell(c) || isPat(c)) order.push_back(c);
    if (!uniformRows)
        for (int c = 0; c < spmv_num_configs(); ++c) order.push_back(c);
    int best = -1;
    float bestMs = 1e30f;
    for (int c : order) {
        const int grid = fp32 ? spmvGrid32(c) : spmvGrid64(c);
        if (grid <= 0) continue;
        if (fp32) ensureValues32(c);
        float ms[4];
        int timed = 0;
        for (int rep = 0; rep < 4; ++rep) {
            check(cudaEventRecord(m_ev0, m_stream), "event");
            check(fp32 ? spmv32(c, grid, m_p32.as<float>(), m_Ap32.as<float>(), nullptr, m_state.as<CgState>(),
                                m_partials.as<double>(), kSpmvPlain, nullptr)
                       : spmv64(c, grid, m_p.as<double>(), m_Ap.as<double>(), nullptr, m_state.as<CgState>(),
                                m_partials.as<double>(), kSpmvPlain, nullptr),
                  "SpMV");
            check(cudaEventRecord(m_ev1, m_stream), "event");
            check(cudaEventSynchronize(m_ev1), "event");
            check(cudaEventElapsedTime(&ms[timed++], m_ev0, m_ev1), "event");
            if (rep == 0 && ms[0] > 1.5f * bestMs) break;
        }
        float t = ms[0];
        if (timed == 4) {  // median of the three launches after the warm-up
            std::sort(ms + 1, ms + 4);
            t = ms[2];
        }
        out[c] = t;
        if (t < bestMs) {
            bestMs = t;
            best = c;
        }
    }
    return best;
}

void PcgHandle::tuneSpmv() {
    Range range_("xJPCG SpMV tuning");
    const auto t0 = std::chrono::steady_clock::now();
    struct TuneClock {
        std::chrono::steady_clock::time_point t0;
        double* out;
        ~TuneClock() { *out = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); }
    } clk{t0, &m_lastTuneMs};
    const int ncfg = numSpmvCfgs();
    int best = -1;
    if (m_forcedCfg >= 0) {
        if (m_forcedCfg >= ncfg || spmvGrid64(m_forcedCfg) <= 0)
            throw InvalidValue("the forced SpMV configuration is not available for this matrix.");
        best = m_forcedCfg;
    } else if (m_forcedLanes == -2) {
        best = mergeCfg();
    } else if (m_forcedLanes == -5) {
        if (!ensurePat()) throw InvalidValue("the shared-offset sliced SpMV layout is not offered for this matrix.");
        best = patCfg0();  // unroll 4
    } else if (m_forcedLanes == -4) {
        if (!ensureSorted())
            throw InvalidValue("the length-sorted sliced SpMV layout is not offered for this matrix.");
        best = sortedCfg0() + 1;  // unroll 8
    } else if (m_forcedLanes == -3) {
        if (!ensureSell() || !m_sellNarrow)
            throw InvalidValue("the sliced SpMV layout with 16-bit column offsets is not available for this matrix.");
        best = spmv_num_configs() + 4;  // int16 offsets, unroll 8
    } else if (m_forcedLanes < 0) {
        if (!ensureSell()) throw InvalidValue("the sliced SpMV layout is not available for this matrix.");
        best = spmv_num_configs();
    } else if (m_forcedLanes > 0) {
        for (int c = spmv_num_configs() - 1; c >= 0; --c)
            if (spmv_config_lanes(c) == m_forcedLanes) best = c;
        if (best < 0) throw InvalidValue("unsupported SpMV lanes per row.");
    } else if (m_tunedHash == m_structHash && m_tunedCfg >= 0 && m_tunedCfg < ncfg && spmvGrid64(m_tunedCfg) > 0) {
        // The same structure as the last tuned matrix (row pointers and
        // columns fingerprinted): SpMV timings depend on the structure only,
        // so the earlier choice and its table stand.
        best = m_tunedCfg;
    } else {
        m_tuneMs.assign(ncfg, -1.f);
        check(cudaMemsetAsync(m_p.p, 0, sizeof(double) * m_n4, m_stream), "memset");
        best = timeConfigs(false, m_tuneMs);
        if (best < 0) throw InternalError("no SpMV configuration can be launched on this device.");
        m_tunedHash = m_structHash;
        m_tunedCfg = best;
        m_tuned32Cfg = -1;
    }
    m_spmvCfg = best;
    m_spmvGrid = spmvGrid64(best);
    m_spmvCfg32 = -1;  // retuned (or follows a forced choice) at the next mixed solve
    ++m_generation;  // graphs embed the configuration
}

// FP32 values of the layout `cfg` uses (CSR copy for the staged and
// merge-path kernels, sliced copy for the SELL kernels).
void PcgHandle::ensureValues32(int cfg) {
    const uint64_t nnzPad = (m_nnz + 3) / 4 * 4 + 4;
    if (!m_val32Valid) {
        alloc(m_val32, sizeof(float) * nnzPad, "fp32 values");
        check(convert_f64_to_f32(m_stream, (int64_t)nnzPad, m_val.as<double>(), m_val32.as<float>()), "fp32 values");
        m_val32Valid = true;
    }
    if (isPat(cfg) && m_psState == 1 && !m_ps32Valid) {
        alloc(m_psVal32, sizeof(float) * ((size_t)m_psTotal + 32), "shared-offset fp32 values");
        check(sellpat_fill<float>(m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(), m_val.as<double>(),
                                  m_psSliceOff.as<int>(), m_psPatLen.as<int>(), m_psPatNew.as<int>(),
                                  m_psPatIdx.as<int>(), m_psPatOff.as<int>(), m_psGenOff.as<int>(), m_psVal32.as<float>(),
                                  nullptr, nullptr, false),
              "shared-offset fp32 fill");
        m_ps32Valid = true;
    }
    if (isSorted(cfg) && m_ssState == 1 && !m_ss32Valid) {
        alloc(m_ssVal32, sizeof(float) * ((size_t)m_ssTotal + 32), "sorted sliced fp32 values");
        check(sellsort_fill<float>(m_stream, (int)m_n, m_ssLong, m_rowptr.as<int>(), m_col.as<int>(), m_val.as<double>(),
                                   m_ssSorted.as<int>(), m_ssSliceOff.as<int>(), nullptr, m_ssVal32.as<float>()),
              "sorted sliced fp32 fill");
        m_ss32Valid = true;
    }
    if (isSell(cfg) && m_sellState == 1 && !m_sell32Valid) {
        alloc(m_sellVal32, sizeof(float) * ((size_t)m_sellTotal + 32), "sliced fp32 values");
        check(sell_fill<float>(m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(), m_val.as<double>(),
                               m_sliceOff.as<int>(), nullptr, m_sellVal32.as<float>()),
              "sliced fp32 fill");
        m_sell32Valid = true;
    }
}

// The mixed solver's FP32 SpMV has no FP64 issue limit, so its best layout
// and unroll can differ from the FP64 choice: every configuration is timed
// again in FP32 (plain mode, median of 3) once per matrix structure.  With a
// forced layout (XJPCG_SPMV_LANES / _CFG or xJPCG_gbSetSpmvLanes) the FP64
// choice is kept.
void PcgHandle::tuneSpmv32() {
    Range range_("xJPCG FP32 SpMV tuning");
    if (m_tuned32Gen == m_structGen && m_spmvCfg32 >= 0) return;
    const int ncfg = numSpmvCfgs();
    const size_t vb32 = sizeof(float) * ((size_t)m_n4 + 4);
    alloc(m_p32, vb32, "p32");
    alloc(m_Ap32, vb32, "Ap32");
    int best = m_spmvCfg;
    if (m_forcedCfg32 >= 0) {
        if (m_forcedCfg32 >= ncfg || spmvGrid32(m_forcedCfg32) <= 0)
            throw InvalidValue("the forced FP32 SpMV configuration is not available for this matrix.");
        best = m_forcedCfg32;
    } else if (m_forcedLanes == 0 && m_forcedCfg < 0) {
        if (m_tuned32Cfg >= 0 && m_tunedHash == m_structHash && spmvGrid32(m_tuned32Cfg) > 0) {
            best = m_tuned32Cfg;  // same structure as when it was tuned
        } else {
            m_tuneMs32.assign(ncfg, -1.f);
            check(cudaMemsetAsync(m_p32.p, 0, vb32, m_stream), "memset");
            const int b32 = timeConfigs(true, m_tuneMs32);
            if (b32 >= 0) best = b32;
            if (m_tunedHash == m_structHash) m_tuned32Cfg = best;
        }
    }
    m_spmvCfg32 = best;
    m_spmvGrid32 = spmvGrid32(best);
    m_tuned32Gen = m_structGen;
    ++m_generation;  // the mixed graph embeds the configuration
}

int PcgHandle::tuning32(float* ms, int cap) const {
    const int ncfg = numSpmvCfgs();
    for (int c = 0; c < ncfg && c < cap; ++c) ms[c] = c < (int)m_tuneMs32.size() ? m_tuneMs32[c] : -1.f;
    return ncfg;
}

// ---------------------------------------------------------------------------
// Vectors and the solve
// ---------------------------------------------------------------------------
void PcgHandle::ensureVectors(uint32_t n) {
    const uint32_t n4 = (n + 3) / 4 * 4;
    const size_t vb = sizeof(double) * ((size_t)n4 + 4);
    alloc(m_b, vb, "b");
    alloc(m_diag, vb, "diag");
    alloc(m_x, vb, "x");
    alloc(m_r, vb, "r");
    alloc(m_p, vb, "p");
    alloc(m_J, vb, "J");
    alloc(m_Ap, vb, "Ap");
    if (n4 != m_n4) {
        for (DevBuf* v : {&m_b, &m_diag, &m_x, &m_r, &m_p, &m_J, &m_Ap})
            check(cudaMemsetAsync(v->p, 0, vb, m_stream), "memset");
        ++m_generation;
    }
    m_vecN = n;
    m_n4 = n4;
}

void PcgHandle::setVec(uint32_t n, const double* b, const double* diag, bool onDevice) {
    // GenCgVector::loadVec / updateVec (cgVector.hpp:55-93).
    if (b == nullptr || diag == nullptr) throw InvalidValue("Vector is nullptr.");
    if (!m_haveMatrix || n != m_n) throw InvalidValue("vector dimension differs from the stored matrix.");
    ensureVectors(n);
    const cudaMemcpyKind kind = onDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    check(cudaMemcpyAsync(m_b.p, b, sizeof(double) * n, kind, m_stream), "copy b");
    check(cudaMemcpyAsync(m_diag.p, diag, sizeof(double) * n, kind, m_stream), "copy diag");
    if (!onDevice) check(cudaStreamSynchronize(m_stream), "sync");
}

void PcgHandle::buildGraph() {
    if (m_exec && m_execGen == m_generation) return;
    if (m_exec) {
        cudaGraphExecDestroy(m_exec);
        m_exec = nullptr;
    }
    const int n = (int)m_n, n4 = (int)m_n4;
    const int vg = vec_grid(n4, m_numSms);
    CgState* st = m_state.as<CgState>();
    double* part = m_partials.as<double>();
    cudaGraph_t g = nullptr;
    check(cudaGraphCreate(&g, 0), "cudaGraphCreate");
    check(cudaStreamBeginCaptureToGraph(m_stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
          "capture");
    check(cg_init_launch(vg, m_stream, n, n4, m_b.as<double>(), m_diag.as<double>(), m_x.as<double>(),
                         m_r.as<double>(), m_p.as<double>(), m_J.as<double>(), m_Ap.as<double>(), st, part),
          "init kernel");
    check(cudaStreamEndCapture(m_stream, &g), "capture end");
    size_t numNodes = 0;
    check(cudaGraphGetNodes(g, nullptr, &numNodes), "graph nodes");
    std::vector<cudaGraphNode_t> nodes(numNodes);
    check(cudaGraphGetNodes(g, nodes.data(), &numNodes), "graph nodes");
    check(cudaGraphConditionalHandleCreate(&m_cond, g, 1, cudaGraphCondAssignDefault), "conditional handle");
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = m_cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t condNode;
    check(cudaGraphAddNode(&condNode, g, nodes.data(), nullptr, numNodes, &cp), "conditional node");
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    check(cudaStreamBeginCaptureToGraph(m_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
          "capture body");
    for (int u = 0; u < kLoopUnroll; ++u) {
        check(spmv64(m_spmvCfg, m_spmvGrid, m_p.as<double>(), m_Ap.as<double>(), nullptr, st, part, cgSpmvMode(),
                     &st->done),
              "SpMV kernel");
        iterationTail(n4, st, part);
    }
    check(cudaStreamEndCapture(m_stream, &body), "capture body end");
    check(cudaGraphInstantiate(&m_exec, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    m_execGen = m_generation;
}

// The SpMV mode of the fp64 loop.  With the fused vector kernel and a sliced
// layout (256-thread CTAs), the SpMV only stores its per-CTA partials of p.Ap
// and the fused kernel forms alpha from them while its first loads are in
// flight; otherwise the SpMV's last CTA forms alpha.
int PcgHandle::cgSpmvMode() const {
    const bool sliced = isSell(m_spmvCfg) || isPat(m_spmvCfg) || isSorted(m_spmvCfg);
    return (m_fusedUpdate && sliced && m_spmvGrid > 0 && m_spmvGrid <= kFusedPartialOff) ? kSpmvCgPart
                                                                                         : kSpmvCgDot;
}

// The mixed loop's FP32 update after its SpMV: the fused cooperative kernel
// (update, refresh decision, and the p update when no refresh is due), or,
// with XJPCG_FUSED_UPDATE=0, the update kernel alone (with pUpdate, the p
// update kernel after it).  On 160^3 the fused form takes the mixed solve
// from 77.9 to 74.6 ms.
void PcgHandle::mixedUpdate(int n4, int vg, CgState* st, double* part, bool pUpdate) {
    if (m_fusedUpdate) {
        check(rel_fused_launch(rel_fused_grid(n4, m_numSms), m_stream, n4, m_d32.as<float>(), m_r32.as<float>(),
                               m_p32.as<float>(), m_Ap32.as<float>(), m_J32.as<float>(), st, part),
              "mixed fused update");
        return;
    }
    check(rel_update_launch(update_grid(n4, m_numSms), m_stream, n4, m_d32.as<float>(), m_r32.as<float>(),
                            m_p32.as<float>(), m_Ap32.as<float>(), m_J32.as<float>(), st, part),
          "mixed update");
    if (pUpdate)
        check(rel_pupdate_launch(vg, m_stream, n4, m_p32.as<float>(), m_r32.as<float>(), m_J32.as<float>(), st),
              "p fp32");
}

// The vector part of an fp64 iteration after the SpMV: the fused cooperative
// kernel (update and p update in one launch), or the two separate kernels
// when XJPCG_FUSED_UPDATE=0.
void PcgHandle::iterationTail(int n4, CgState* st, double* part) {
    if (m_fusedUpdate) {
        check(cg_fused_launch(fused_grid(n4, m_numSms), m_stream, n4, m_x.as<double>(), m_r.as<double>(),
                              m_p.as<double>(), m_Ap.as<double>(), m_J.as<double>(), st, part,
                              cgSpmvMode() == kSpmvCgPart ? m_spmvGrid : 0),
              "fused update kernel");
        return;
    }
    check(cg_update_launch(update_grid(n4, m_numSms), m_stream, n4, m_r.as<double>(), m_Ap.as<double>(),
                           m_J.as<double>(), st, part),
          "update kernel");
    check(cg_pupdate_launch(vec_grid(n4, m_numSms), m_stream, n4, m_x.as<double>(), m_p.as<double>(),
                            m_Ap.as<double>(), st),
          "p kernel");
}

Results PcgHandle::run(uint32_t maxIter, double tol) {
    Range range_("xJPCG fp64 solve");
    if (!m_haveMatrix) throw InvalidValue("no matrix has been set.");
    // Records: slot 0 + one per iteration, up to a ring of kMaxRecords.
    const uint64_t want = std::min<uint64_t>((uint64_t)maxIter + 2, kMaxRecords);
    if (want > m_recCap) {
        alloc(m_records, sizeof(IterRecord) * want, "iteration records");
        m_recCap = want;
    }
    check(cudaMemsetAsync(m_records.p, 0, sizeof(IterRecord) * std::min<uint64_t>(m_recCap, want), m_stream),
          "memset records");
    CgState cmd = {};
    cmd.tol = tol;
    cmd.maxIterP1 = maxIter + 1u;
    cmd.records = m_records.as<IterRecord>();
    cmd.recCap = (uint32_t)want;
    const int n = (int)m_n, n4 = (int)m_n4;
    CgState* st = m_state.as<CgState>();
    double* part = m_partials.as<double>();
    if (m_useGraph) {
        buildGraph();
        cmd.useCond = 1;
        cmd.condHandle = (uint64_t)m_cond;
    }
    faultPoint("graph launch");
    check(cudaMemcpyAsync(st, &cmd, sizeof(CgState), cudaMemcpyHostToDevice, m_stream), "state upload");
    check(cudaEventRecord(m_ev0, m_stream), "event");
    if (m_useGraph) {
        check(cudaGraphLaunch(m_exec, m_stream), "graph launch");
    } else {
        // Host-driven loop: batches of iterations, kernels skip once done.
        const int vg = vec_grid(n4, m_numSms);
        check(cg_init_launch(vg, m_stream, n, n4, m_b.as<double>(), m_diag.as<double>(), m_x.as<double>(),
                             m_r.as<double>(), m_p.as<double>(), m_J.as<double>(), m_Ap.as<double>(), st, part),
              "init kernel");
        uint64_t ran = 0;
        for (;;) {
            for (int u = 0; u < 16; ++u) {
                check(spmv64(m_spmvCfg, m_spmvGrid, m_p.as<double>(), m_Ap.as<double>(), nullptr, st, part,
                                          cgSpmvMode(), &st->done),
                      "SpMV kernel");
                iterationTail(n4, st, part);
            }
            ran += 16;
            uint32_t done = 0;
            check(cudaMemcpyAsync(&done, &st->done, sizeof(uint32_t), cudaMemcpyDeviceToHost, m_stream), "D2H");
            check(cudaStreamSynchronize(m_stream), "sync");
            if (done || ran > (uint64_t)maxIter + 1) break;
        }
    }
    check(cudaEventRecord(m_ev1, m_stream), "event");
    check(cudaMemcpyAsync(&m_lastState, st, sizeof(CgState), cudaMemcpyDeviceToHost, m_stream), "state download");
    check(cudaStreamSynchronize(m_stream), "sync");
    check(cudaEventElapsedTime(&m_lastMs, m_ev0, m_ev1), "event");
    return readResults(maxIter);
}

Results PcgHandle::readResults(uint32_t maxIter) {
    const CgState& s = m_lastState;
    if (s.status & kStatusWaitTimeout) throw InternalError("Run kernel failed: a device wait timed out.");
    Results r;
    r.itersRun = s.k;
    // pcgImp.hpp:171-180: the scan stops at the first empty record, so a run
    // that used all maxIter + 1 slots reports maxIter.
    r.reportedIters = s.k <= maxIter ? s.k : maxIter;
    r.rrLast = s.rr;
    r.bb = s.bb;
    r.status = s.status;
    m_lastBb = s.bb;
    return r;
}

void PcgHandle::copyX(double* x, uint32_t n, bool toDevice) {
    check(cudaMemcpyAsync(x, m_x.p, sizeof(double) * n, toDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                          m_stream),
          "copy x");
    check(cudaStreamSynchronize(m_stream), "sync");
}

// ---------------------------------------------------------------------------
// Mixed precision
// ---------------------------------------------------------------------------
void PcgHandle::buildMixedGraph() {
    if (m_mixedExec && m_mixedGen == m_generation) return;
    if (m_mixedExec) {
        cudaGraphExecDestroy(m_mixedExec);
        m_mixedExec = nullptr;
    }
    const int n = (int)m_n, n4 = (int)m_n4;
    (void)n;
    const int vg = vec_grid(n4, m_numSms);
    const int cfg32 = m_spmvCfg32;
    const int grid32 = m_spmvGrid32;
    CgState* st = m_state.as<CgState>();
    double* part = m_partials.as<double>();
    cudaGraph_t g = nullptr;
    check(cudaGraphCreate(&g, 0), "cudaGraphCreate");
    check(cudaStreamBeginCaptureToGraph(m_stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
          "capture");
    check(rel_init_launch(vg, m_stream, (int)m_n, n4, m_b.as<double>(), m_diag.as<double>(), m_x.as<double>(),
                          m_d32.as<float>(), m_J32.as<float>(), m_r32.as<float>(), m_p32.as<float>(), st, part),
          "mixed init");
    check(cudaStreamEndCapture(m_stream, &g), "capture end");
    size_t nn = 0;
    check(cudaGraphGetNodes(g, nullptr, &nn), "nodes");
    std::vector<cudaGraphNode_t> nodes(nn);
    check(cudaGraphGetNodes(g, nodes.data(), &nn), "nodes");
    check(cudaGraphConditionalHandleCreate(&m_condOuter, g, 1, cudaGraphCondAssignDefault), "handle");
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = m_condOuter;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t loopNode;
    check(cudaGraphAddNode(&loopNode, g, nodes.data(), nullptr, nn, &cp), "loop node");
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    // body: WHILE no refresh is due {FP32 SpMV, update, p update}, then the
    // refresh (fold, FP64 residual, restart) and its p update
    check(cudaGraphConditionalHandleCreate(&m_condInner, body, 1, cudaGraphCondAssignDefault), "handle");
    cudaGraphNodeParams ip = {};
    ip.type = cudaGraphNodeTypeConditional;
    ip.conditional.handle = m_condInner;
    ip.conditional.type = cudaGraphCondTypeWhile;
    ip.conditional.size = 1;
    cudaGraphNode_t innerNode;
    check(cudaGraphAddNode(&innerNode, body, nullptr, nullptr, 0, &ip), "inner loop node");
    cudaGraph_t inner = ip.conditional.phGraph_out[0];
    check(cudaStreamBeginCaptureToGraph(m_stream, inner, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
          "capture");
    for (int u = 0; u < kLoopUnroll; ++u) {
        // the FP32 SpMV stops on a due refresh (reliable) as well as on done
        check(spmv32(cfg32, grid32, m_p32.as<float>(), m_Ap32.as<float>(), nullptr, st, part, kSpmvCgDot,
                     &st->reliable),
              "SpMV fp32");
        mixedUpdate(n4, vg, st, part);
    }
    check(cudaStreamEndCapture(m_stream, &inner), "capture end");
    check(cudaStreamBeginCaptureToGraph(m_stream, body, &innerNode, nullptr, 1, cudaStreamCaptureModeThreadLocal),
          "capture");
    check(rel_fold_launch(vg, m_stream, n4, m_x.as<double>(), m_d32.as<float>(), st), "fold");
    check(spmv64(m_spmvCfg, m_spmvGrid, m_x.as<double>(), m_r.as<double>(), m_b.as<double>(), st, part,
                 kSpmvResidual, nullptr),
          "residual SpMV");
    check(rel_restart_launch(vg, m_stream, n4, m_r.as<double>(), m_J32.as<float>(), m_r32.as<float>(), st, part),
          "restart");
    check(rel_pupdate_launch(vg, m_stream, n4, m_p32.as<float>(), m_r32.as<float>(), m_J32.as<float>(), st),
          "p fp32");
    check(cudaStreamEndCapture(m_stream, &body), "capture end");
    check(cudaGraphInstantiate(&m_mixedExec, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    m_mixedGen = m_generation;
}

Results PcgHandle::runMixed(uint32_t maxIter, double tol) {
    Range range_("xJPCG mixed solve");
    if (!m_haveMatrix) throw InvalidValue("no matrix has been set.");
    const size_t vb32 = sizeof(float) * ((size_t)m_n4 + 4);
    alloc(m_r32, vb32, "r32");
    alloc(m_p32, vb32, "p32");
    alloc(m_d32, vb32, "d32");
    alloc(m_Ap32, vb32, "Ap32");
    alloc(m_J32, vb32, "J32");
    tuneSpmv32();
    ensureValues32(m_spmvCfg32);
    check(cudaMemsetAsync(m_Ap32.p, 0, vb32, m_stream), "memset");
    CgState* st = m_state.as<CgState>();
    if (m_useGraph) buildMixedGraph();
    CgState cmd = {};
    cmd.tol = tol;
    cmd.maxIterP1 = maxIter + 1u;
    cmd.useCond = m_useGraph ? 1u : 0u;
    cmd.condHandle = m_useGraph ? (uint64_t)m_condOuter : 0;
    cmd.relHandle = m_useGraph ? (uint64_t)m_condInner : 0;
    // 1e-3: on the 27-point 160^3 system 0.01 and 1e-3 tie (4-5 refreshes),
    // 1e-4 adds 11 FP32 iterations and 1e-5 adds 142; on the 2M-row Zipf
    // system (22 iterations, refresh-bound) 1e-3 saves one of six refreshes.
    const double delta = envDouble("XJPCG_RELIABLE_DELTA", 1e-3);
    cmd.delta2 = delta * delta;
    faultPoint("graph launch");
    check(cudaMemcpyAsync(st, &cmd, sizeof(CgState), cudaMemcpyHostToDevice, m_stream), "state upload");
    check(cudaEventRecord(m_ev0, m_stream), "event");
    if (m_useGraph) {
        check(cudaGraphLaunch(m_mixedExec, m_stream), "graph launch");
    } else {
        // Host-driven loop (profilers): the graph's kernels in batches of 16
        // iterations; the refresh kernels skip themselves unless chosen.
        const int n4 = (int)m_n4;
        const int vg = vec_grid(n4, m_numSms);
        double* part = m_partials.as<double>();
        check(rel_init_launch(vg, m_stream, (int)m_n, n4, m_b.as<double>(), m_diag.as<double>(), m_x.as<double>(),
                              m_d32.as<float>(), m_J32.as<float>(), m_r32.as<float>(), m_p32.as<float>(), st, part),
              "mixed init");
        uint64_t ran = 0;
        for (;;) {
            for (int u = 0; u < 16; ++u) {
                check(spmv32(m_spmvCfg32, m_spmvGrid32, m_p32.as<float>(), m_Ap32.as<float>(), nullptr, st, part,
                             kSpmvCgDot, &st->done),
                      "SpMV fp32");
                mixedUpdate(n4, vg, st, part, false);
                check(rel_fold_launch(vg, m_stream, n4, m_x.as<double>(), m_d32.as<float>(), st), "fold");
                check(spmv64(m_spmvCfg, m_spmvGrid, m_x.as<double>(), m_r.as<double>(), m_b.as<double>(), st, part,
                             kSpmvResidual, &st->skipRefresh),
                      "residual SpMV");
                check(rel_restart_launch(vg, m_stream, n4, m_r.as<double>(), m_J32.as<float>(), m_r32.as<float>(),
                                         st, part),
                      "restart");
                check(rel_pupdate_launch(vg, m_stream, n4, m_p32.as<float>(), m_r32.as<float>(), m_J32.as<float>(),
                                         st),
                      "p fp32");
            }
            ran += 16;
            uint32_t done = 0;
            check(cudaMemcpyAsync(&done, &st->done, sizeof(uint32_t), cudaMemcpyDeviceToHost, m_stream), "D2H");
            check(cudaStreamSynchronize(m_stream), "sync");
            if (done || ran > (uint64_t)maxIter + 1) break;
        }
    }
    check(cudaEventRecord(m_ev1, m_stream), "event");
    check(cudaMemcpyAsync(&m_lastState, st, sizeof(CgState), cudaMemcpyDeviceToHost, m_stream), "state download");
    check(cudaStreamSynchronize(m_stream), "sync");
    check(cudaEventElapsedTime(&m_lastMs, m_ev0, m_ev1), "event");
    const CgState& s = m_lastState;
    if (s.status & kStatusWaitTimeout) throw InternalError("Run kernel failed: a device wait timed out.");
    m_lastOuter = s.outer;
    m_lastInner = s.innerK;
    Results r;
    r.itersRun = s.k;
    r.reportedIters = s.k;
    r.rrLast = s.rrTrue;
    r.bb = s.bb;
    r.status = s.status;
    m_lastBb = s.bb;
    return r;
}

void PcgHandle::copyX64(double* x, uint32_t n, bool toDevice) { copyX(x, n, toDevice); }

// ---------------------------------------------------------------------------
// Utilities
// ---------------------------------------------------------------------------
void PcgHandle::spmv(const double* x, double* y, bool onDevice) {
    if (!m_haveMatrix) throw InvalidValue("no matrix has been set.");
    const double* dx = x;
    double* dy = y;
    if (!onDevice) {
        alloc(m_scratchY, sizeof(double) * ((size_t)m_n4 + 4), "SpMV output");
        check(cudaMemcpyAsync(m_b.p, x, sizeof(double) * m_n, cudaMemcpyHostToDevice, m_stream), "H2D x");
        dx = m_b.as<double>();
        dy = m_scratchY.as<double>();
    }
    check(spmv64(m_spmvCfg, m_spmvGrid, dx, dy, nullptr, m_state.as<CgState>(), m_partials.as<double>(),
                              kSpmvPlain, nullptr),
          "SpMV");
    if (!onDevice) {
        check(cudaMemcpyAsync(y, dy, sizeof(double) * m_n, cudaMemcpyDeviceToHost, m_stream), "D2H y");
        check(cudaStreamSynchronize(m_stream), "sync");
    }
}

// ---------------------------------------------------------------------------
// The reference's partitioned-matrix buffers (SpmvHost drop-in)
// ---------------------------------------------------------------------------
namespace {
uint32_t rdU32(const unsigned char* p, uint64_t off) {
    uint32_t v;
    std::memcpy(&v, p + off, 4);
    return v;
}
uint16_t rdU16(const unsigned char* p, uint64_t off) {
    uint16_t v;
    std::memcpy(&v, p + off, 2);
    return v;
}
}  // namespace

// Layouts: RowBlockParam (matrix_params.hpp:329-471): 32-byte header
// {totalRows, totalRbs}, then per row block 8 x 32 bytes: {startRow, minCol,
// cols, numPars}, {rows, nnzs}, u16[16] channel row offsets, u16[16]
// channel rows, u32[16] channel nnzs, 32 bytes dummy.  ParParam (473-576):
// 32-byte header {totalPars}, then per partition 8 x 32 bytes: u32[16]
// channel columns, u32[16] channel nnzs, {baseColBlock, colBlocks, rows,
// nnzs}, u16[16] channel column-block offsets, u16[16] channel column blocks,
// dummy.  Chunks follow gen_nnzStore (signature.hpp:361-426).
void PcgHandle::setSignatureMatrix(uint32_t nch, const void* const* bufs, const uint64_t* bytes, const void* par,
                                   uint64_t parBytes, const void* rb, uint64_t rbBytes) {
    Range range_("xJPCG signature matrix set-up");
    if (nch != 16) throw InvalidValue("the partitioned format has 16 channels.");
    const unsigned char* R = static_cast<const unsigned char*>(rb);
    const unsigned char* P = static_cast<const unsigned char*>(par);
    if (rbBytes < 32 || parBytes < 32) throw InvalidValue("parameter buffer too small.");
    const uint32_t totalRows = rdU32(R, 0), totalRbs = rdU32(R, 4), totalPars = rdU32(P, 0);
    if (32 + (uint64_t)totalRbs * 256 > rbBytes || 32 + (uint64_t)totalPars * 256 > parBytes)
        throw InvalidValue("parameter buffer shorter than its header says.");
    std::vector<uint64_t> chanOff(nch, 32), chanBase(nch, 0);
    uint64_t totalBytes = 0;
    for (uint32_t c = 0; c < nch; ++c) {
        if (bufs[c] == nullptr || bytes[c] < 32) throw InvalidValue("channel buffer missing or too small.");
        chanBase[c] = totalBytes;
        totalBytes += (bytes[c] + 15) / 16 * 16;
    }
    std::vector<SigChunk> chunks;
    int64_t groups = 0;
    uint32_t maxColEnd = 0;
    for (uint32_t p = 0; p < totalPars; ++p) {
        const uint64_t pb = 32 + (uint64_t)p * 256;
        maxColEnd = std::max(maxColEnd, (rdU32(P, pb + 128) + rdU32(P, pb + 132)) * 4u);
    }
    uint32_t parId = 0;
    for (uint32_t r = 0; r < totalRbs; ++r) {
        const uint64_t rbb = 32 + (uint64_t)r * 256;
        const uint32_t startRow = rdU32(R, rbb), npars = rdU32(R, rbb + 12);
        if ((uint64_t)parId + npars > totalPars) throw InvalidValue("row blocks reference missing partitions.");
        for (uint32_t c = 0; c < nch; ++c) {
            const int32_t rowBase = (int32_t)(startRow + rdU16(R, rbb + 64 + 2 * c));
            for (uint32_t q = 0; q < npars; ++q) {
                const uint64_t pb = 32 + (uint64_t)(parId + q) * 256;
                const uint32_t chNnz = rdU32(P, pb + 64 + 4 * c);
                if (chNnz % 32 != 0) throw InvalidValue("channel chunk is not a multiple of 32 entries.");
                const int64_t ng = chNnz / 4;
                if (ng == 0) continue;
                const uint64_t chunkBytes = 32 * (uint64_t)(ng + (ng + 127) / 128 + (ng + 15) / 16);
                if (chanOff[c] + chunkBytes > bytes[c]) throw InvalidValue("channel buffer shorter than its chunks.");
                SigChunk ck;
                ck.byteStart = (int64_t)(chanBase[c] + chanOff[c]);
                ck.groupStart = groups;
                ck.rowBase = rowBase;
                ck.colBase = (int32_t)(rdU32(P, pb + 128) + rdU16(P, pb + 160 + 2 * c));
                chunks.push_back(ck);
                groups += ng;
                chanOff[c] += chunkBytes;
            }
        }
        parId += npars;
    }
    const uint32_t n = std::max(totalRows, maxColEnd);
    if (n == 0 || groups == 0) throw InvalidValue("empty partitioned matrix.");
    const int64_t entries = groups * 4;
    if (entries > 0x7ffffff0ll) throw InvalidValue("partitioned matrix too large for int32 indexing.");
    alloc(m_sigBuf, totalBytes + 16, "channel buffers");
    for (uint32_t c = 0; c < nch; ++c)
        check(cudaMemcpyAsync(m_sigBuf.as<unsigned char>() + chanBase[c], bufs[c], bytes[c], cudaMemcpyHostToDevice,
                              m_stream),
              "H2D channel");
    alloc(m_sigChunks, sizeof(SigChunk) * chunks.size(), "chunk table");
    check(cudaMemcpyAsync(m_sigChunks.p, chunks.data(), sizeof(SigChunk) * chunks.size(), cudaMemcpyHostToDevice,
                          m_stream),
          "H2D chunks");
    alloc(m_sigRow, sizeof(uint32_t) * entries, "decoded rows");
    alloc(m_sigCol, sizeof(uint32_t) * entries, "decoded columns");
    alloc(m_sigVal, sizeof(double) * entries, "decoded values");
    alloc(m_sigKeep, sizeof(int) * (entries + 1), "decoded mask");
    check(sig_decode(m_stream, (int)chunks.size(), m_sigChunks.as<SigChunk>(), m_sigBuf.as<unsigned char>(), groups,
                     m_sigRow.as<uint32_t>(), m_sigCol.as<uint32_t>(), m_sigVal.as<double>(), m_sigKeep.as<int>()),
          "decode");
    check(cudaMemsetAsync(m_sigKeep.as<int>() + entries, 0, sizeof(int), m_stream), "memset");
    alloc(m_cscScratch, sizeof(int) * (entries + 8), "positions");
    alloc(m_blockSums, sizeof(int) * ((size_t)scan_block_count((int)entries + 1) + 16), "scan scratch");
    check(scan_exclusive(m_stream, m_sigKeep.as<int>(), m_cscScratch.as<int>(), (int)entries + 1, m_blockSums.as<int>()),
          "scan");
    int kept = 0;
    check(cudaMemcpyAsync(&kept, m_cscScratch.as<int>() + entries, sizeof(int), cudaMemcpyDeviceToHost, m_stream),
          "D2H");
    check(cudaStreamSynchronize(m_stream), "sync");
    if (kept == 0) throw InvalidValue("partitioned matrix holds no non-zero entry.");
    alloc(m_inRow, sizeof(uint32_t) * kept, "COO rows");
    alloc(m_inCol, sizeof(uint32_t) * kept, "COO cols");
    alloc(m_inVal, sizeof(double) * kept, "COO values");
    check(sig_compact(m_stream, entries, m_cscScratch.as<int>(), m_sigKeep.as<int>(), m_sigRow.as<uint32_t>(),
                      m_sigCol.as<uint32_t>(), m_sigVal.as<double>(), m_inRow.as<uint32_t>(), m_inCol.as<uint32_t>(),
                      m_inVal.as<double>()),
          "compact");
    // The compacted list is a COO input in stored order (base 0).
    const uint64_t nnz = (uint64_t)kept;
    const uint64_t nnzPad = (nnz + 3) / 4 * 4 + 4;
    alloc(m_rowptr, sizeof(int) * ((size_t)n + 1 + kRowptrPad), "CSR row pointers");
    alloc(m_col, sizeof(int) * nnzPad, "CSR columns");
    alloc(m_val, sizeof(double) * nnzPad, "CSR values");
    alloc(m_perm, sizeof(uint32_t) * (nnz + 1), "CSR permutation");
    alloc(m_counts, sizeof(int) * ((size_t)n + 2), "conversion counts");
    alloc(m_fill, sizeof(int) * ((size_t)n + 1), "conversion fill");
    alloc(m_keys, sizeof(uint64_t) * (nnz + 1), "conversion keys");
    alloc(m_blockSums, sizeof(int) * ((size_t)scan_block_count((int)std::max<uint64_t>(n + 1, nnz + 1)) + 16),
          "scan scratch");
    ConvertScratch sc;
    sc.counts = m_counts.as<int>();
    sc.fill = m_fill.as<int>();
    sc.blockSums = m_blockSums.as<int>();
    sc.keys = m_keys.as<uint64_t>();
    sc.flags = m_flags.as<int>();
    int herr = 0;
    check(coo_to_csr(m_stream, (int)n, (int64_t)nnz, m_inRow.as<uint32_t>(), m_inCol.as<uint32_t>(), 0,
                     m_rowptr.as<int>(), m_col.as<int>(), m_perm.as<uint32_t>(), sc, &herr),
          "COO to CSR conversion");
    if (herr & kStatusIndexError) throw InvalidValue("decoded index out of range.");
    check(gather_values(m_stream, (int64_t)nnz, m_perm.as<uint32_t>(), m_inVal.as<double>(), m_val.as<double>()),
          "value gather");
    m_n = n;
    m_nnz = nnz;
    m_kind = 4;
    m_sigRows = totalRows;
    finishMatrix();
    // Run lists for the reference-order SpMV: every run of 32 stored entries
    // (one row index) listed under its row, in stream order.  The conversion
    // sorts each row's runs by run index, which is the stream order: the
    // chunks of a row's channel follow its row block's partitions in order.
    const int64_t runs = groups / 8;
    const uint32_t N = (uint32_t)std::max<int64_t>((int64_t)n, runs);
    alloc(m_sigRunRow, sizeof(uint32_t) * (size_t)runs, "run rows");
    alloc(m_sigRunIdx, sizeof(uint32_t) * (size_t)runs, "run indices");
    check(sig_run_rows(m_stream, runs, m_sigRow.as<uint32_t>(), m_sigRunRow.as<uint32_t>(), m_sigRunIdx.as<uint32_t>()),
          "run rows");
    alloc(m_sigRunPtr, sizeof(int) * ((size_t)N + 1 + kRowptrPad), "run pointers");
    alloc(m_sigRunList, sizeof(int) * ((size_t)runs + 8), "run lists");
    alloc(m_sigRunPerm, sizeof(uint32_t) * ((size_t)runs + 1), "run permutation");
    alloc(m_counts, sizeof(int) * ((size_t)N + 2), "conversion counts");
    alloc(m_fill, sizeof(int) * ((size_t)N + 1), "conversion fill");
    alloc(m_keys, sizeof(uint64_t) * ((size_t)runs + 1), "conversion keys");
    alloc(m_blockSums, sizeof(int) * ((size_t)scan_block_count((int)std::max<int64_t>((int64_t)N + 1, runs + 1)) + 16),
          "scan scratch");
    ConvertScratch rs;
    rs.counts = m_counts.as<int>();
    rs.fill = m_fill.as<int>();
    rs.blockSums = m_blockSums.as<int>();
    rs.keys = m_keys.as<uint64_t>();
    rs.flags = m_flags.as<int>();
    herr = 0;
    check(coo_to_csr(m_stream, (int)N, runs, m_sigRunRow.as<uint32_t>(), m_sigRunIdx.as<uint32_t>(), 0,
                     m_sigRunPtr.as<int>(), m_sigRunList.as<int>(), m_sigRunPerm.as<uint32_t>(), rs, &herr),
          "run lists");
    if (herr & kStatusIndexError) throw InternalError("run list conversion out of range.");
    check(cudaStreamSynchronize(m_stream), "sync");
    m_sigOrderedGen = m_valGen;
}

void PcgHandle::setSignatureSumOrder(int order) {
    if (order != 0 && order != 1) throw InvalidValue("summation order must be 0 (fastest) or 1 (the reference's).");
    m_sigSumOrder = order;
}

// JPCG over the matrix loaded by setSignatureMatrix.  Order 1: the loop of
// fpga_order.cu, driven from the host in batches of 8 iterations (each
// kernel that changes the solve returns at once when the loop is done).
// Order 0: the tuned solve on the decoded CSR, with b and diag padded to the
// matrix size (b 0, diag 1), as the 4-padding of cgVector.hpp:67-73 does.
Results PcgHandle::signatureSolve(uint32_t n, const double* b, const double* diag, double* x, uint32_t maxIter,
                                  double tol) {
    Range range_("xJPCG signature solve");
    if (b == nullptr || diag == nullptr) throw InvalidValue("Vector is nullptr.");
    if (!m_haveMatrix || m_kind != 4) throw InvalidValue("no matrix loaded by xJPCG_gbSetSignatureMatrix.");
    const uint32_t n4 = (n + 3) / 4 * 4;
    if (n == 0 || n > m_n || n4 > m_n4) throw InvalidValue("vector dimension exceeds the partitioned matrix.");
    if (m_sigSumOrder == 0) {
        std::vector<double> bp(m_n, 0.0), dp(m_n, 1.0);
        std::copy(b, b + n, bp.begin());
        std::copy(diag, diag + n, dp.begin());
        setVec(m_n, bp.data(), dp.data(), false);
        Results r = run(maxIter, tol);
        if (x) copyX(x, n, false);
        return r;
    }
    if (m_sigOrderedGen != m_valGen)
        throw InvalidValue("the reference-order solve needs a matrix loaded by xJPCG_gbSetSignatureMatrix and "
                           "unchanged since.");
    const uint64_t want = std::min<uint64_t>((uint64_t)maxIter + 2, kMaxRecords);
    if (want > m_recCap) {
        alloc(m_records, sizeof(IterRecord) * want, "iteration records");
        m_recCap = want;
    }
    check(cudaMemsetAsync(m_records.p, 0, sizeof(IterRecord) * want, m_stream), "memset records");
    CgState cmd = {};
    cmd.tol = tol;
    cmd.maxIterP1 = maxIter + 1u;
    cmd.records = m_records.as<IterRecord>();
    cmd.recCap = (uint32_t)want;
    CgState* st = m_state.as<CgState>();
    check(cudaMemcpyAsync(st, &cmd, sizeof(CgState), cudaMemcpyHostToDevice, m_stream), "state upload");
    const size_t vb = sizeof(double) * ((size_t)m_n4 + 4);
    check(cudaMemsetAsync(m_p.p, 0, vb, m_stream), "memset p");  // p past n4 stays 0 for the SpMV's gathers
    check(cudaMemsetAsync(m_Ap.p, 0, vb, m_stream), "memset Ap");
    check(cudaMemcpyAsync(m_b.p, b, sizeof(double) * n, cudaMemcpyHostToDevice, m_stream), "H2D b");
    check(cudaMemcpyAsync(m_diag.p, diag, sizeof(double) * n, cudaMemcpyHostToDevice, m_stream), "H2D diag");
    alloc(m_foPart, sizeof(double) * (2 * (size_t)fo_blocks((int)n4) + 2), "reference-order dot blocks");
    faultPoint("reference-order solve");
    check(cudaEventRecord(m_ev0, m_stream), "event");
    check(fo_init(m_stream, (int)n, (int)n4, m_b.as<double>(), m_diag.as<double>(), m_x.as<double>(),
                  m_r.as<double>(), m_p.as<double>(), m_J.as<double>(), m_Ap.as<double>(), st),
          "reference-order init");
    uint64_t ran = 0;
    for (;;) {
        for (int u = 0; u < 8; ++u) {
            check(sig_ordered_spmv(m_stream, (int)m_n, m_sigRunPtr.as<int>(), m_sigRunList.as<int>(),
                                   m_sigVal.as<double>(), m_sigCol.as<uint32_t>(), m_p.as<double>(),
                                   m_Ap.as<double>()),
                  "reference-order SpMV");
            check(fo_iteration_tail(m_stream, (int)n4, m_x.as<double>(), m_p.as<double>(), m_r.as<double>(),
                                    m_Ap.as<double>(), m_J.as<double>(), m_foPart.as<double>(), st),
                  "reference-order iteration");
        }
        ran += 8;
        uint32_t done = 0;
        check(cudaMemcpyAsync(&done, &st->done, sizeof(uint32_t), cudaMemcpyDeviceToHost, m_stream), "D2H");
        check(cudaStreamSynchronize(m_stream), "sync");
        if (done || ran > (uint64_t)maxIter + 1) break;
    }
    check(cudaEventRecord(m_ev1, m_stream), "event");
    check(cudaMemcpyAsync(&m_lastState, st, sizeof(CgState), cudaMemcpyDeviceToHost, m_stream), "state download");
    if (x) check(cudaMemcpyAsync(x, m_x.p, sizeof(double) * n, cudaMemcpyDeviceToHost, m_stream), "D2H x");
    check(cudaStreamSynchronize(m_stream), "sync");
    check(cudaEventElapsedTime(&m_lastMs, m_ev0, m_ev1), "event");
    return readResults(maxIter);
}

void PcgHandle::signatureSpmv(const double* x, uint32_t xLen, double* y, uint32_t yRows, uint32_t startAddr,
                              unsigned char* frame, uint64_t frameBytes) {
    if (!m_haveMatrix) throw InvalidValue("no matrix has been set.");
    if (xLen > m_n || yRows > m_n) throw InvalidValue("vector longer than the matrix.");
    const bool ordered = m_sigSumOrder == 1;
    if (ordered && !(m_kind == 4 && m_sigOrderedGen == m_valGen))
        throw InvalidValue("the reference-order SpMV needs a matrix loaded by xJPCG_gbSetSignatureMatrix and "
                           "unchanged since.");
    alloc(m_scratchY, sizeof(double) * ((size_t)m_n4 + 4), "SpMV output");
    check(cudaMemsetAsync(m_b.p, 0, sizeof(double) * m_n4, m_stream), "memset");
    check(cudaMemcpyAsync(m_b.p, x, sizeof(double) * xLen, cudaMemcpyHostToDevice, m_stream), "H2D x");
    if (ordered)
        check(sig_ordered_spmv(m_stream, (int)m_n, m_sigRunPtr.as<int>(), m_sigRunList.as<int>(),
                               m_sigVal.as<double>(), m_sigCol.as<uint32_t>(), m_b.as<double>(),
                               m_scratchY.as<double>()),
              "reference-order SpMV");
    else
        check(spmv64(m_spmvCfg, m_spmvGrid, m_b.as<double>(), m_scratchY.as<double>(), nullptr,
                     m_state.as<CgState>(), m_partials.as<double>(), kSpmvPlain, nullptr),
              "SpMV");
    if (y) check(cudaMemcpyAsync(y, m_scratchY.p, sizeof(double) * yRows, cudaMemcpyDeviceToHost, m_stream), "D2H y");
    if (frame) {
        const uint64_t need = 64 + 64 * (uint64_t)(yRows == 0 ? 1 : (yRows + 7) / 8);
        if (frameBytes < need) throw InvalidValue("frame buffer too small.");
        alloc(m_sigFrame, need, "frame");
        check(transy_frame(m_stream, startAddr, yRows, m_scratchY.as<double>(), m_sigFrame.as<unsigned char>()),
              "frame");
        check(cudaMemcpyAsync(frame, m_sigFrame.p, need, cudaMemcpyDeviceToHost, m_stream), "D2H frame");
    }
    check(cudaStreamSynchronize(m_stream), "sync");
}

// ---------------------------------------------------------------------------
// Adjoint
// ---------------------------------------------------------------------------
Results PcgHandle::adjoint(const double* g, const double* diag, double* lambda, double* gradA, uint32_t maxIter,
                           double tol, bool onDevice) {
    Range range_("xJPCG adjoint solve");
    if (!m_haveMatrix || !m_haveX) throw InvalidValue("the adjoint needs a completed solve on this handle.");
    const size_t vb = sizeof(double) * ((size_t)m_n4 + 4);
    alloc(m_xKeep, vb, "adjoint x");
    alloc(m_lambda, vb, "adjoint lambda");
    check(cudaMemcpyAsync(m_xKeep.p, m_x.p, vb, cudaMemcpyDeviceToDevice, m_stream), "keep x");
    setVec(m_n, g, diag, onDevice);
    Results r = run(maxIter, tol);
    check(cudaMemcpyAsync(m_lambda.p, m_x.p, vb, cudaMemcpyDeviceToDevice, m_stream), "lambda");
    check(cudaMemcpyAsync(m_x.p, m_xKeep.p, vb, cudaMemcpyDeviceToDevice, m_stream), "restore x");
    m_haveLambda = true;
    const cudaMemcpyKind out = onDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (lambda) check(cudaMemcpyAsync(lambda, m_lambda.p, sizeof(double) * m_n, out, m_stream), "copy lambda");
    if (gradA) {
        // dL/dA per input entry: COO / CSR inputs index gradA like their data
        // array (perm maps CSR slots back); symmetric CSC input indexes it by
        // the expanded full matrix (2 nnz - n entries, emission order).
        alloc(m_grad, sizeof(double) * (m_nnz + 4), "dA");
        check(grad_nnz_launch(m_stream, (int)m_n, m_rowptr.as<int>(), m_col.as<int>(), m_perm.as<uint32_t>(),
                              m_xKeep.as<double>(), m_lambda.as<double>(), m_grad.as<double>()),
              "dA kernel");
        check(cudaMemcpyAsync(gradA, m_grad.p, sizeof(double) * m_nnz, out, m_stream), "copy dA");
    }
    check(cudaStreamSynchronize(m_stream), "sync");
    return r;
}

void PcgHandle::edgeGrad(int64_t m, const int32_t* ei, const int32_t* ej, const double* c, double* grad,
                         bool onDevice) {
    Range range_("xJPCG edge gradient");
    if (!m_haveLambda) throw InvalidValue("the edge gradient needs a completed adjoint solve.");
    if (m <= 0) throw InvalidValue("number of edges must be positive.");
    const int* dI = ei;
    const int* dJ = ej;
    const double* dC = c;
    double* dG = grad;
    if (!onDevice) {
        alloc(m_edgeI, sizeof(int) * m, "edges");
        alloc(m_edgeJ, sizeof(int) * m, "edges");
        alloc(m_edgeC, sizeof(double) * m, "edges");
        alloc(m_edgeG, sizeof(double) * m, "edge gradient");
        check(cudaMemcpyAsync(m_edgeI.p, ei, sizeof(int) * m, cudaMemcpyHostToDevice, m_stream), "H2D");
        check(cudaMemcpyAsync(m_edgeJ.p, ej, sizeof(int) * m, cudaMemcpyHostToDevice, m_stream), "H2D");
        check(cudaMemcpyAsync(m_edgeC.p, c, sizeof(double) * m, cudaMemcpyHostToDevice, m_stream), "H2D");
        dI = m_edgeI.as<int>();
        dJ = m_edgeJ.as<int>();
        dC = m_edgeC.as<double>();
        dG = m_edgeG.as<double>();
    }
    int bad = 0;
    check(edge_grad_launch(m_stream, m, (int)m_n, dI, dJ, dC, m_x.as<double>(), m_lambda.as<double>(), dG,
                           m_flags.as<int>(), &bad),
          "edge gradient");
    if (bad) throw InvalidValue("an edge endpoint lies outside [0, n).");
    if (!onDevice) check(cudaMemcpyAsync(grad, dG, sizeof(double) * m, cudaMemcpyDeviceToHost, m_stream), "D2H");
    check(cudaStreamSynchronize(m_stream), "sync");
}

// ---------------------------------------------------------------------------
// Batched solves
// ---------------------------------------------------------------------------
namespace {
__attribute__((unused)) uint64_t mixKey(uint64_t h, uint64_t v) { return (h ^ v) * 0x100000001b3ull; }
}  // namespace

uint32_t PcgHandle::batchSolve(uint32_t nsys, const int32_t* sysRow, const int32_t* rowPtr, const int32_t* colIdx,
                               const double* values, const double* diag, const double* b, double* x,
                               uint32_t maxIter, double tol, int precision, BatchResult* results, bool onDevice) {
    Range range_("xJPCG batched solve");
    if (nsys == 0) throw InvalidValue("number of systems is zero.");
    if (precision != 0 && precision != 1) throw InvalidValue("precision must be 0 (fp64) or 1 (mixed).");
    const bool mixed = precision == 1;
    // System and row offsets are small: validate them on the host.
    std::vector<int32_t> hSys(nsys + 1);
    check(cudaMemcpy(hSys.data(), sysRow, sizeof(int32_t) * (nsys + 1), onDevice ? cudaMemcpyDeviceToHost
                                                                                  : cudaMemcpyHostToHost),
          "system offsets");
    if (hSys[0] != 0) throw InvalidValue("system row offsets must start at 0.");
    int maxN = 0;
    for (uint32_t s = 0; s < nsys; ++s) {
        const int ns = hSys[s + 1] - hSys[s];
        if (ns <= 0) throw InvalidValue("every system needs at least one row.");
        maxN = std::max(maxN, ns);
    }
    const int total = hSys[nsys];
    std::vector<int32_t> hRp((size_t)total + 1);
    check(cudaMemcpy(hRp.data(), rowPtr, sizeof(int32_t) * ((size_t)total + 1),
                     onDevice ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost),
          "row pointers");
    if (hRp[0] != 0) throw InvalidValue("row pointers must start at 0.");
    int maxRowLen = 0;
    for (int i = 0; i < total; ++i) {
        if (hRp[i + 1] < hRp[i]) throw InvalidValue("row pointers are not monotone.");
        maxRowLen = std::max(maxRowLen, hRp[i + 1] - hRp[i]);
    }
    const int64_t nnz = hRp[total];
    // Queue order: largest systems first so the long solves start early.
    std::vector<int32_t> order(nsys);
    for (uint32_t s = 0; s < nsys; ++s) order[s] = (int32_t)s;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t c) {
        return (hRp[hSys[a + 1]] - hRp[hSys[a]]) > (hRp[hSys[c + 1]] - hRp[hSys[c]]);
    });
    const size_t vb = sizeof(double) * ((size_t)total + 4), fb = sizeof(float) * ((size_t)total + 4);
    alloc(m_bSysRow, sizeof(int32_t) * (nsys + 1), "batch offsets");
    alloc(m_bOrder, sizeof(int32_t) * nsys, "batch order");
    alloc(m_bRowptr, sizeof(int32_t) * ((size_t)total + 1), "batch row pointers");
    alloc(m_bCol, sizeof(int32_t) * ((size_t)nnz + 4), "batch columns");
    alloc(m_bVal, sizeof(double) * ((size_t)nnz + 4), "batch values");
    for (DevBuf* v : {&m_bB, &m_bDiag, &m_bX, &m_bR, &m_bAp, &m_bJ, &m_bP}) alloc(*v, vb, "batch vector");
    if (mixed) {
        alloc(m_bVal32, sizeof(float) * ((size_t)nnz + 4), "batch fp32 values");
        for (DevBuf* v : {&m_bR32, &m_bD32, &m_bAp32, &m_bJ32, &m_bP32}) alloc(*v, fb, "batch vector");
    }
    alloc(m_bRes, sizeof(BatchResult) * nsys, "batch results");
    alloc(m_bQueue, 16, "batch queue");
    const cudaMemcpyKind k = onDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    check(cudaMemcpyAsync(m_bSysRow.p, hSys.data(), sizeof(int32_t) * (nsys + 1), cudaMemcpyHostToDevice, m_stream),
          "H2D");
    check(cudaMemcpyAsync(m_bOrder.p, order.data(), sizeof(int32_t) * nsys, cudaMemcpyHostToDevice, m_stream), "H2D");
    check(cudaMemcpyAsync(m_bRowptr.p, hRp.data(), sizeof(int32_t) * ((size_t)total + 1), cudaMemcpyHostToDevice,
                          m_stream),
          "H2D");
    check(cudaMemcpyAsync(m_bCol.p, colIdx, sizeof(int32_t) * nnz, k, m_stream), "copy columns");
    check(cudaMemcpyAsync(m_bVal.p, values, sizeof(double) * nnz, k, m_stream), "copy values");
    check(cudaMemcpyAsync(m_bB.p, b, sizeof(double) * total, k, m_stream), "copy b");
    check(cudaMemcpyAsync(m_bDiag.p, diag, sizeof(double) * total, k, m_stream), "copy diag");
    check(batch_validate_columns(m_stream, (int)nsys, m_bSysRow.as<int>(), m_bRowptr.as<int>(), m_bCol.as<int>(),
                                 m_flags.as<int>()),
          "column check");
    int bad = 0;
    check(cudaMemcpyAsync(&bad, m_flags.p, sizeof(int), cudaMemcpyDeviceToHost, m_stream), "D2H");
    check(cudaStreamSynchronize(m_stream), "sync");
    if (bad) throw InvalidValue("a column index lies outside its system.");
    if (mixed) check(convert_f64_to_f32(m_stream, nnz, m_bVal.as<double>(), m_bVal32.as<float>()), "fp32 values");

    // Per-system SELL-32 copy for the sliced kernels: 32-row slices of each
    // system, values slice-column-major, 16-bit local columns.  Offered when
    // every system has at most 65,536 rows and the copy fits 32-bit offsets.
    int64_t nslices = 0;
    for (uint32_t s = 0; s < nsys; ++s) nslices += (hSys[s + 1] - hSys[s] + 31) / 32;
    const bool sliced = maxN <= 65536 &&
                        nslices * 32 * (int64_t)std::max(maxRowLen, kBatchPatMax) < 0x7fffff00ll &&
                        envInt("XJPCG_BATCH_SLICED", 1) != 0;
    if (sliced) {
        const int nsl = (int)nslices;
        std::vector<int32_t> hBase(nsys + 1, 0);
        for (uint32_t s = 0; s < nsys; ++s) hBase[s + 1] = hBase[s] + (hSys[s + 1] - hSys[s] + 31) / 32;
        alloc(m_bsBase, sizeof(int32_t) * (nsys + 1), "batch slice bases");
        alloc(m_bsLen, sizeof(int32_t) * ((size_t)nsl + 1), "batch slice lengths");
        alloc(m_bsOff, sizeof(int32_t) * ((size_t)nsl + 1), "batch slice offsets");
        alloc(m_bsScan, sizeof(int32_t) * ((size_t)scan_block_count(nsl + 1) + 1), "scan scratch");
        alloc(m_bsPatLen, sizeof(int32_t) * ((size_t)nsl + 1), "batch slice patterns");
        alloc(m_bsPatOff, sizeof(int32_t) * (size_t)kBatchPatMax * ((size_t)nsl + 1), "batch slice offsets");
        check(cudaMemcpyAsync(m_bsBase.p, hBase.data(), sizeof(int32_t) * (nsys + 1), cudaMemcpyHostToDevice,
                              m_stream),
              "H2D");
        check(cudaMemsetAsync(m_bsLen.p, 0, sizeof(int32_t) * ((size_t)nsl + 1), m_stream), "memset");
        check(batch_sell_widths(m_stream, (int)nsys, nsl, m_bSysRow.as<int>(), m_bsBase.as<int>(),
                                m_bRowptr.as<int>(), m_bCol.as<int>(), m_bsLen.as<int>(), m_bsOff.as<int>(),
                                m_bsScan.as<int>(), m_bsPatLen.as<int>(), m_bsPatOff.as<int>(),
                                envInt("XJPCG_BATCH_PATTERNS", 1) != 0),
              "batch slices");
        alloc(m_bsMeta, sizeof(int32_t) * 2 * ((size_t)nsl + 1), "batch slice records");
        alloc(m_bsSysPat, sizeof(int32_t) * (size_t)(kBatchPatMax + 1) * (nsys + 1), "batch system offsets");
        check(batch_sell_meta(m_stream, (int)nsys, nsl, m_bSysRow.as<int>(), m_bsBase.as<int>(), m_bsOff.as<int>(),
                              m_bsPatLen.as<int>(), m_bsPatOff.as<int>(), static_cast<int2*>(m_bsMeta.p),
                              m_bsSysPat.as<int>()),
              "batch slice records");
        int stored = 0;
        check(cudaMemcpyAsync(&stored, m_bsOff.as<int>() + nsl, sizeof(int), cudaMemcpyDeviceToHost, m_stream),
              "D2H");
        check(cudaStreamSynchronize(m_stream), "sync");
        alloc(m_bsCol, sizeof(uint16_t) * ((size_t)stored + 64), "batch sliced columns");
        if (mixed) {
            alloc(m_bsVal32, sizeof(float) * ((size_t)stored + 32), "batch sliced fp32 values");
            check(batch_sell_fill<float>(m_stream, (int)nsys, nsl, m_bSysRow.as<int>(), m_bsBase.as<int>(),
                                         m_bRowptr.as<int>(), m_bCol.as<int>(), m_bVal.as<double>(), m_bsOff.as<int>(),
                                         m_bsPatLen.as<int>(), m_bsPatOff.as<int>(), m_bsVal32.as<float>(),
                                         m_bsCol.as<uint16_t>()),
                  "batch sliced fp32 fill");
        } else {
            alloc(m_bsVal, sizeof(double) * ((size_t)stored + 32), "batch sliced values");
            check(batch_sell_fill<double>(m_stream, (int)nsys, nsl, m_bSysRow.as<int>(), m_bsBase.as<int>(),
                                          m_bRowptr.as<int>(), m_bCol.as<int>(), m_bVal.as<double>(),
                                          m_bsOff.as<int>(), m_bsPatLen.as<int>(), m_bsPatOff.as<int>(),
                                          m_bsVal.as<double>(), m_bsCol.as<uint16_t>()),
                  "batch sliced fill");
        }
    }

    BatchLaunch L;
    L.nsys = (int)nsys;
    L.sysRow = m_bSysRow.as<int>();
    L.order = m_bOrder.as<int>();
    L.rowptr = m_bRowptr.as<int>();
    L.col = m_bCol.as<int>();
    L.val = m_bVal.as<double>();
    L.val32 = mixed ? m_bVal32.as<float>() : nullptr;
    L.b = m_bB.as<double>();
    L.diag = m_bDiag.as<double>();
    L.x = m_bX.as<double>();
    L.r = m_bR.as<double>();
    L.Ap = m_bAp.as<double>();
    L.J = m_bJ.as<double>();
    L.r32 = mixed ? m_bR32.as<float>() : nullptr;
    L.d32 = mixed ? m_bD32.as<float>() : nullptr;
    L.Ap32 = mixed ? m_bAp32.as<float>() : nullptr;
    L.J32 = mixed ? m_bJ32.as<float>() : nullptr;
    L.pGlobal = m_bP.as<double>();
    L.p32Global = mixed ? m_bP32.as<float>() : nullptr;
    L.res = m_bRes.as<BatchResult>();
    L.queue = m_bQueue.as<uint32_t>();
    L.maxIterP1 = maxIter + 1u;
    L.tol = tol;
    {
        // 0.01 per system: on the 4,096-system batch 1e-3 adds 0.9 % and
        // 1e-4 adds 6.5 % FP32 iterations.
        const double delta = envDouble("XJPCG_RELIABLE_DELTA", 0.01);
        L.delta2 = delta * delta;
    }
    if (sliced) {
        L.sliceBase = m_bsBase.as<int>();
        L.sliceOff = m_bsOff.as<int>();
        L.sval = mixed ? nullptr : m_bsVal.as<double>();
        L.sval32 = mixed ? m_bsVal32.as<float>() : nullptr;
        L.scol = m_bsCol.as<uint16_t>();
        L.patLen = m_bsPatLen.as<int>();
        L.patOff = m_bsPatOff.as<int>();
        L.meta = static_cast<const int2*>(m_bsMeta.p);
        L.sysPat = m_bsSysPat.as<int>();
    }

    // Shape candidates: CTA size x lanes per row x rows of p kept in shared
    // memory: the largest system (up to 200 KB), 4,096 rows, or 44 KB.  More
    // shared memory leaves less L1 for the matrix and the vectors: on 4,096
    // systems the fp64 batch took 148.1 / 149.6 / 171.8 ms with 4,096 / 8,192 /
    // 11,264 rows, and the mixed one 81.6 / 78.8 ms with 4,096 / 11,264 rows.
    const size_t esz = mixed ? sizeof(float) : sizeof(double);
    const int smemCap = (int)(200 * 1024 / esz);
    std::vector<int> smemRows;
    for (int rows : {smemCap, 4096, (int)(44 * 1024 / esz)}) {
        rows = std::min(maxN, rows);
        if (std::find(smemRows.begin(), smemRows.end(), rows) == smemRows.end()) smemRows.push_back(rows);
    }
    const uint64_t key = mixKey(mixKey(mixKey(nsys, (uint64_t)total), (uint64_t)nnz),
                                (uint64_t)precision + 7 + (sliced ? 1000 : 0));
    const int forced = envInt("XJPCG_BATCH_CFG", -1);
    auto runOnce = [&](int cfg, int rows, float* ms) {
        check(cudaMemsetAsync(m_bQueue.p, 0, 16, m_stream), "memset queue");
        check(cudaEventRecord(m_ev0, m_stream), "event");
        int grid = 0;
        check(batch_launch(cfg, mixed, m_numSms, rows, m_stream, L, &grid), "batched kernel");
        check(cudaEventRecord(m_ev1, m_stream), "event");
        check(cudaEventSynchronize(m_ev1), "event");
        check(cudaEventElapsedTime(ms, m_ev0, m_ev1), "event");
        m_batchGrid = grid;
    };
    const int ncfg = batch_num_configs();
    if (forced >= 0 && forced < ncfg * (int)smemRows.size()) {
        m_batchCfg = forced % ncfg;
        m_batchSmemRows = smemRows[forced / ncfg];
    } else if (m_batchKey != key || m_batchCfg < 0) {
        m_batchTuneMs.assign((size_t)ncfg * smemRows.size(), -1.f);
        float best = 1e30f;
        for (size_t si = 0; si < smemRows.size(); ++si)
            for (int c = 0; c < ncfg; ++c) {
                if (batch_config_sliced(c) && !sliced) continue;
                float ms = 0;
                runOnce(c, smemRows[si], &ms);
                m_batchTuneMs[si * ncfg + c] = ms;
                if (ms < best) {
                    best = ms;
                    m_batchCfg = c;
                    m_batchSmemRows = smemRows[si];
                }
            }
        m_batchKey = key;
    }
    // The production launch is a CUDA graph (queue reset + persistent
    // kernel), instantiated once per shape and buffer set.
    const uint64_t gkey = mixKey(mixKey(mixKey(key, (uint64_t)m_batchCfg), (uint64_t)m_batchSmemRows), m_generation);
    if (!m_batchExec || m_batchExecKey != gkey) {
        if (m_batchExec) {
            cudaGraphExecDestroy(m_batchExec);
            m_batchExec = nullptr;
        }
        cudaGraph_t g = nullptr;
        check(cudaStreamBeginCapture(m_stream, cudaStreamCaptureModeThreadLocal), "capture");
        int grid = 0;
        cudaError_t e1 = cudaMemsetAsync(m_bQueue.p, 0, 16, m_stream);
        cudaError_t e2 = e1 == cudaSuccess ? batch_launch(m_batchCfg, mixed, m_numSms, m_batchSmemRows, m_stream, L, &grid)
                                           : e1;
        cudaError_t e3 = cudaStreamEndCapture(m_stream, &g);
        check(e2, "batched kernel capture");
        check(e3, "capture end");
        check(cudaGraphInstantiate(&m_batchExec, g, 0), "graph instantiate");
        cudaGraphDestroy(g);
        m_batchGrid = grid;
        m_batchExecKey = gkey;
    }
    faultPoint("graph launch");
    check(cudaEventRecord(m_ev0, m_stream), "event");
    check(cudaGraphLaunch(m_batchExec, m_stream), "graph launch");
    check(cudaEventRecord(m_ev1, m_stream), "event");
    check(cudaEventSynchronize(m_ev1), "event");
    check(cudaEventElapsedTime(&m_batchMs, m_ev0, m_ev1), "event");
    std::vector<BatchResult> hr(nsys);
    check(cudaMemcpyAsync(results ? (void*)results : (void*)hr.data(), m_bRes.p, sizeof(BatchResult) * nsys,
                          cudaMemcpyDeviceToHost, m_stream),
          "D2H results");
    if (x)
        check(cudaMemcpyAsync(x, m_bX.p, sizeof(double) * total, onDevice ? cudaMemcpyDeviceToDevice
                                                                          : cudaMemcpyDeviceToHost, m_stream),
              "copy x");
    check(cudaStreamSynchronize(m_stream), "sync");
    const BatchResult* rr = results ? results : hr.data();
    uint32_t failed = 0;
    for (uint32_t s = 0; s < nsys; ++s)
        if (rr[s].status != 0 || !(rr[s].res <= tol)) ++failed;
    return failed;
}

void PcgHandle::getCsr(int32_t* rowPtr, int32_t* colIdx, double* values, uint32_t* perm) {
    if (!m_haveMatrix) throw InvalidValue("no matrix has been set.");
    if (rowPtr)
        check(cudaMemcpyAsync(rowPtr, m_rowptr.p, sizeof(int) * ((size_t)m_n + 1), cudaMemcpyDeviceToHost, m_stream),
              "D2H");
    if (colIdx) check(cudaMemcpyAsync(colIdx, m_col.p, sizeof(int) * m_nnz, cudaMemcpyDeviceToHost, m_stream), "D2H");
    if (values)
        check(cudaMemcpyAsync(values, m_val.p, sizeof(double) * m_nnz, cudaMemcpyDeviceToHost, m_stream), "D2H");
    if (perm) check(cudaMemcpyAsync(perm, m_perm.p, sizeof(uint32_t) * m_nnz, cudaMemcpyDeviceToHost, m_stream), "D2H");
    check(cudaStreamSynchronize(m_stream), "sync");
}

void PcgHandle::exportSignature(XJPCG_GbSignature_t* sig) {
    Range range_("xJPCG signature export");
    if (!m_haveMatrix) throw InvalidValue("no matrix has been set.");
    if (!m_sigExport.valid || m_sigExport.structGen != m_structGen) {
        m_sigExport.build(m_stream, m_n, m_nnz, m_rowptr.as<int>(), m_col.as<int>());
        m_sigExport.structGen = m_structGen;
    }
    m_sigExport.format(m_stream, m_val.as<double>());
    if (sig) {
        std::memset(sig, 0, sizeof(*sig));
        const SigExport& e = m_sigExport;
        const uint32_t info[6] = {e.m, e.n, e.nnz, e.m, (e.n + 3) / 4 * 4, e.nnzPad};
        std::memcpy(sig->info, info, sizeof(info));
        sig->rowBlocks = (uint32_t)e.nb;
        sig->partitions = (uint32_t)e.P;
        sig->rbParamBytes = e.rbBytes;
        sig->parParamBytes = e.parBytes;
        for (int c = 0; c < 16; ++c) sig->nnzValBytes[c] = e.chanBytes[c];
    }
}

void PcgHandle::getSignature(void* rb, void* par, void* const* nnzVal) {
    m_sigExport.copyOut(m_stream, rb, par, nnzVal);
}

uint64_t PcgHandle::getRecords(void* buf, uint64_t cap) {
    if (m_recCap == 0) return 0;
    const uint64_t used = std::min<uint64_t>((uint64_t)m_lastState.k + 1, m_recCap);
    const uint64_t cnt = std::min<uint64_t>(used, cap);
    check(cudaMemcpyAsync(buf, m_records.p, sizeof(IterRecord) * cnt, cudaMemcpyDeviceToHost, m_stream), "D2H");
    check(cudaStreamSynchronize(m_stream), "sync");
    return cnt;
}

int PcgHandle::tuning(float* ms, int* shape, int cap) const {
    const int ncfg = numSpmvCfgs();
    for (int c = 0; c < ncfg && c < cap; ++c) {
        ms[c] = c < (int)m_tuneMs.size() ? m_tuneMs[c] : -1.f;
        if (isMerge(c)) {
            // merge path: lanes 0, 256 threads, path steps per thread
            shape[4 * c] = 0;
            shape[4 * c + 1] = 256;
            shape[4 * c + 2] = merge_items_per_thread();
            shape[4 * c + 3] = 0;
        } else if (isPat(c)) {
            // shared-offset sliced layout: (1, 2, unroll, 1 when the values
            // are prefetched by TMA bulk copies (FP32 only) else 0)
            shape[4 * c] = 1;
            shape[4 * c + 1] = 2;
            shape[4 * c + 2] = sellpat_config_unroll(c - patCfg0());
            shape[4 * c + 3] = sellpat_config_tma(c - patCfg0()) ? 1 : (sellpat_config_runs(c - patCfg0()) ? 2 : 0);
        } else if (isSorted(c)) {
            // length-sorted sliced layout: (1, 1, unroll, 32)
            shape[4 * c] = 1;
            shape[4 * c + 1] = 1;
            shape[4 * c + 2] = sellsort_config_unroll(c - sortedCfg0());
            shape[4 * c + 3] = 32;
        } else if (isSell(c)) {
            // sliced layout: one lane per row, no CTA staging; chunk = unroll,
            // last field = bits per stored column (32 absolute, 16 offset)
            shape[4 * c] = 1;
            shape[4 * c + 1] = 0;
            shape[4 * c + 2] = sell_config_unroll(c - spmv_num_configs());
            shape[4 * c + 3] = isSellNarrow(c) ? 16 : 32;
        } else {
            spmv_config_shape(c, &shape[4 * c], &shape[4 * c + 1], &shape[4 * c + 2], &shape[4 * c + 3]);
        }
    }
    return ncfg;
}

void PcgHandle::fillInfo(XJPCG_GbInfo_t* info) const {
    std::memset(info, 0, sizeof(*info));
    info->n = m_n;
    info->n4 = m_n4;
    info->nnz = m_nnz;
    info->itersRun = m_lastState.k;
    info->spmvLanes = isMerge(m_spmvCfg) ? 0u : (isSell(m_spmvCfg) ? 1u : (uint32_t)spmv_config_lanes(m_spmvCfg));
    info->spmvLayout = layoutCode(m_spmvCfg);
    info->spmvGrid = (uint32_t)m_spmvGrid;
    info->statusBits = m_lastState.status;
    info->outerSweeps = m_lastOuter;
    info->innerIters = m_lastInner;
    info->bb = m_lastState.bb;
    info->rrLast = m_lastState.rr;
    info->solveMs = m_lastMs;
    info->loopMode = m_useGraph ? 1u : 0u;
    info->loopUnroll = m_useGraph ? (uint32_t)kLoopUnroll : 16u;  // the host loop issues batches of 16
    info->kernelsPerIter = m_fusedUpdate ? 2u : 3u;
    if (m_batchCfg >= 0) {
        int t = 0, l = 0;
        batch_config_shape(m_batchCfg, &t, &l);
        info->batchThreads = (uint32_t)t;
        info->batchLanes = (uint32_t)l;
        info->batchSliced = batch_config_sliced(m_batchCfg) ? 1u : 0u;
    }
    info->batchSmemRows = (uint32_t)m_batchSmemRows;
    info->batchGrid = (uint32_t)m_batchGrid;
    info->batchMs = m_batchMs;
    const int c32 = m_spmvCfg32 >= 0 ? m_spmvCfg32 : m_spmvCfg;
    info->spmvLayout32 = layoutCode(c32);
    info->spmvCfg32 = m_spmvCfg32 >= 0 ? (uint32_t)m_spmvCfg32 : 0xffffffffu;
    info->spmvCfg = (uint32_t)m_spmvCfg;
    info->tuneMs = m_lastTuneMs;
    float up = 0.f;
    if (m_uploadTimed && cudaEventElapsedTime(&up, m_evUp0, m_evUp1) == cudaSuccess) info->uploadMs = up;
    if (m_uploadTimed && cudaEventElapsedTime(&up, m_evUp0, m_evUpIdx) == cudaSuccess) info->uploadIdxMs = up;
    if (m_uploadTimed && cudaEventElapsedTime(&up, m_evUpVal, m_evUp1) == cudaSuccess) info->uploadValMs = up;
}

}  // namespace xjpcg
