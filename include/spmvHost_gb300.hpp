/*
 * spmvHost_gb300.hpp -- the reference's SpMV host classes, over this
 * library's C ABI, with a GPU in place of the Alveo card.
 *
 * Drop-in for
 *   xilinx_apps::sparse::SpmvHost<16>          L2/sparse/include/sw/fp64/spmvHost.hpp:26-103
 *   xilinx_apps::dspmv::dSpmvComputeHost<16>   dSpmv/sw/include/dSpmvComputeHost.hpp:27-96
 *   xilinx_apps::dspmv::dSpmvStoreYhost<16>    dSpmv/sw/include/dSpmvStoreYhost.hpp:27-55
 * and of the card object they are handed,
 *   xilinx_apps::hpc_common::FPGA              L2/common/include/sw/xNativeFPGA.hpp:33-45
 * with the same method names, argument meanings and call order: an
 * application written against those headers compiles against this one and
 * links with -lXilinxPcg (header only; nothing here needs CUDA headers).
 *
 * What stands behind each method:
 *   FPGA::setId / load_xclbin   the CUDA device and one xJPCG handle on it
 *                               (xJPCG_gbCreateHandleOnDevice); the xclbin
 *                               path is accepted and ignored, as by
 *                               xJPCG_createHandle.
 *   init / createKernels        bind the card; the kernels are in the library.
 *   createLoadNnzBufs etc.      record the caller's host buffers (the
 *                               reference wraps them in buffer objects).
 *   sendBOs                     xJPCG_gbSetSignatureMatrix: the partitioned
 *                               matrix (16 nnzVal channels, parParam, rbParam)
 *                               is copied to the GPU and decoded there.
 *   run                         xJPCG_gbSignatureSpmv: y = A x on the GPU
 *                               (x = the second createLoadParXbufs buffer);
 *                               the compute host also builds the transY frame.
 *   getY                        copies the result into the caller's y buffer.
 *   finish                      nothing left to wait for (every call above is
 *                               synchronous).
 * The transY network link between a compute card and the store card becomes
 * a byte stream in host memory (NetStream): dSpmvComputeHost::run appends its
 * frame to the stream it is connected to, and dSpmvStoreYhost::run consumes
 * setStoreYargs(numNodes) frames from its stream (xJPCG_gbStoreYFrames).
 *
 * Errors: a failing library call throws SpmvHostError with the XJPCG status
 * and the handle's message (the reference's kernel wrappers abort or throw).
 */
#ifndef XJPCG_SPMVHOST_GB300_HPP
#define XJPCG_SPMVHOST_GB300_HPP

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "xjpcg_gb300.h"

namespace xilinx_apps {

namespace hpc_common {

// The accelerator: one CUDA device and one xJPCG handle on it.
class FPGA {
   public:
    FPGA() = default;
    ~FPGA() {
        if (m_handle != nullptr) xJPCG_destroyHandle(m_handle);
    }
    FPGA(const FPGA&) = delete;
    FPGA& operator=(const FPGA&) = delete;

    void setId(const int p_id) { m_id = p_id; }
    // Creates the handle on device setId (or the current device when setId
    // was not called).  The path is accepted and ignored.
    void load_xclbin(const std::string& xclbin_fnm) {
        if (m_handle != nullptr) return;
        const XJPCG_Status_t st = xJPCG_gbCreateHandleOnDevice(&m_handle, m_id, xclbin_fnm.c_str());
        if (st != XJPCG_STATUS_SUCCESS) {
            std::string msg = m_handle ? xJPCG_getLastMessage(m_handle) : xJPCG_getErrorString(st);
            if (m_handle != nullptr) xJPCG_destroyHandle(m_handle);
            m_handle = nullptr;
            throw std::runtime_error("load_xclbin: " + msg);
        }
    }
    int getId() const { return m_id; }
    XJPCG_Handle_t* handle() const { return m_handle; }

   private:
    int m_id = -1;
    XJPCG_Handle_t* m_handle = nullptr;
};

}  // namespace hpc_common

namespace sparse {

class SpmvHostError : public std::runtime_error {
   public:
    SpmvHostError(XJPCG_Status_t p_status, const std::string& p_msg)
        : std::runtime_error(p_msg), m_status(p_status) {}
    XJPCG_Status_t getStatus() const { return m_status; }

   private:
    XJPCG_Status_t m_status;
};

namespace detail {

inline void check(XJPCG_Handle_t* h, XJPCG_Status_t st, const char* what) {
    if (st == XJPCG_STATUS_SUCCESS) return;
    std::string msg = std::string(what) + ": ";
    msg += h != nullptr ? xJPCG_getLastMessage(h) : xJPCG_getErrorString(st);
    throw SpmvHostError(st, msg);
}

// The buffers and calls SpmvHost and dSpmvComputeHost share: the matrix
// (nnz channels, parParam, rbParam) and x, sent with sendBOs and multiplied
// with run.
template <unsigned int t_NumChannels>
class SpmvCompute {
   public:
    void init(hpc_common::FPGA* p_fpga) { m_card = p_fpga; }
    void createKernels() {
        if (m_card == nullptr) throw SpmvHostError(XJPCG_STATUS_NOT_INITIALIZED, "createKernels: init() first");
        if (m_card->handle() == nullptr) m_card->load_xclbin("");
    }
    void createLoadNnzBufs(const size_t p_bytes[t_NumChannels], void* p_hostPtr[t_NumChannels]) {
        for (unsigned int i = 0; i < t_NumChannels; ++i) {
            m_nnzBytes[i] = p_bytes[i];
            m_nnzPtr[i] = p_hostPtr[i];
        }
    }
    // [0] = parParam, [1] = x (the padded column count of doubles).
    void createLoadParXbufs(const size_t p_bytes[2], void* p_hostPtr[2]) {
        for (unsigned int i = 0; i < 2; ++i) {
            m_parXbytes[i] = p_bytes[i];
            m_parXptr[i] = p_hostPtr[i];
        }
    }
    void createLoadRbParamBufs(const size_t p_bytes, void* p_hostPtr) {
        m_rbBytes = p_bytes;
        m_rbPtr = p_hostPtr;
    }
    void sendBOs() {
        XJPCG_Handle_t* h = handle("sendBOs");
        uint64_t bytes[t_NumChannels];
        for (unsigned int i = 0; i < t_NumChannels; ++i) bytes[i] = m_nnzBytes[i];
        check(h,
              xJPCG_gbSetSignatureMatrix(h, t_NumChannels, const_cast<const void* const*>(m_nnzPtr), bytes,
                                         m_parXptr[0], m_parXbytes[0], m_rbPtr, m_rbBytes),
              "sendBOs");
        m_sent = true;
    }
    void finish() {}

   protected:
    XJPCG_Handle_t* handle(const char* what) const {
        if (m_card == nullptr || m_card->handle() == nullptr)
            throw SpmvHostError(XJPCG_STATUS_NOT_INITIALIZED, std::string(what) + ": init() and createKernels() first");
        return m_card->handle();
    }
    // y = A x for the sent matrix: `rows` values into m_y and, when frame is
    // wanted, the transY frame of them with startAddr into m_frame.
    void multiply(uint32_t rows, uint32_t startAddr, bool frame) {
        XJPCG_Handle_t* h = handle("run");
        if (!m_sent) throw SpmvHostError(XJPCG_STATUS_INVALID_VALUE, "run: sendBOs() first");
        m_y.assign(rows, 0.0);
        const uint64_t words = rows == 0 ? 1 : (rows + 7) / 8;
        if (frame) m_frame.assign(64 + 64 * words, 0u);
        check(h,
              xJPCG_gbSignatureSpmv(h, static_cast<const double*>(m_parXptr[1]),
                                    (uint32_t)(m_parXbytes[1] / sizeof(double)), m_y.data(), rows, startAddr,
                                    frame ? m_frame.data() : nullptr, frame ? (uint64_t)m_frame.size() : 0),
              "run");
    }

    hpc_common::FPGA* m_card = nullptr;
    size_t m_nnzBytes[t_NumChannels] = {};
    void* m_nnzPtr[t_NumChannels] = {};
    size_t m_parXbytes[2] = {};
    void* m_parXptr[2] = {};
    size_t m_rbBytes = 0;
    void* m_rbPtr = nullptr;
    bool m_sent = false;
    std::vector<double> m_y;
    std::vector<unsigned char> m_frame;
};

}  // namespace detail

template <unsigned int t_NumChannels>
class SpmvHost : public detail::SpmvCompute<t_NumChannels> {
    static_assert(t_NumChannels == 16, "the partitioned format has 16 channels");
    using Base = detail::SpmvCompute<t_NumChannels>;

   public:
    SpmvHost() {}
    void createStoreYbufs(const size_t p_bytes, void* p_hostPtr) {
        m_yBytes = p_bytes;
        m_yPtr = p_hostPtr;
    }
    void setStoreYrows(const unsigned int p_rows) { m_rows = p_rows; }
    void run() { this->multiply(m_rows, 0u, false); }
    void getY() {
        const size_t bytes = this->m_y.size() * sizeof(double);
        if (m_yPtr == nullptr || bytes > m_yBytes)
            throw SpmvHostError(XJPCG_STATUS_INVALID_VALUE, "getY: the y buffer is missing or smaller than the rows");
        std::memcpy(m_yPtr, this->m_y.data(), bytes);
    }

   private:
    size_t m_yBytes = 0;
    void* m_yPtr = nullptr;
    unsigned int m_rows = 0;
};

}  // namespace sparse

namespace dspmv {

using sparse::SpmvHostError;

// The network link from compute cards to the store card: frames appended
// back to back, consumed from the front.
class NetStream {
   public:
    void write(const std::vector<unsigned char>& p_frame) { m_bytes.insert(m_bytes.end(), p_frame.begin(), p_frame.end()); }
    const unsigned char* data() const { return m_bytes.data() + m_head; }
    size_t size() const { return m_bytes.size() - m_head; }
    void consume(size_t p_bytes) {
        m_head += p_bytes;
        if (m_head == m_bytes.size()) {
            m_bytes.clear();
            m_head = 0;
        }
    }

   private:
    std::vector<unsigned char> m_bytes;
    size_t m_head = 0;
};

template <unsigned int t_NumChannels>
class dSpmvComputeHost : public sparse::detail::SpmvCompute<t_NumChannels> {
    static_assert(t_NumChannels == 16, "the partitioned format has 16 channels");

   public:
    dSpmvComputeHost() {}
    // startAddr: where the store card writes these rows, in 32-byte memory
    // words; rows: how many rows of y this card sends.
    void setKrnTransYargs(const unsigned int p_startAddr, const unsigned int p_rows) {
        m_startAddr = p_startAddr;
        m_rows = p_rows;
    }
    void connect(NetStream* p_net) { m_net = p_net; }
    // y = A x, framed by transY and sent on the connected stream.
    void run() {
        this->multiply(m_rows, m_startAddr, true);
        if (m_net != nullptr) m_net->write(this->m_frame);
    }
    // The last frame run() built (a 64-byte header word, then the rows eight
    // per 64-byte word).
    const std::vector<unsigned char>& frame() const { return this->m_frame; }
    const std::vector<double>& y() const { return this->m_y; }

   private:
    unsigned int m_startAddr = 0, m_rows = 0;
    NetStream* m_net = nullptr;
};

template <unsigned int t_NumChannels>
class dSpmvStoreYhost {
   public:
    dSpmvStoreYhost() {}
    void init(hpc_common::FPGA* p_fpga) { m_card = p_fpga; }
    void createKernels() {}
    void createStoreYbufs(const size_t p_bytes, void* p_hostPtr) {
        m_yBytes = p_bytes;
        m_yPtr = p_hostPtr;
    }
    void setStoreYargs(const unsigned int p_numComputeNodes) { m_nodes = p_numComputeNodes; }
    void connect(NetStream* p_net) { m_net = p_net; }
    // Consumes one frame per compute node into the result memory (a copy of
    // the y buffer as run() found it; getY hands it back).
    void run() {
        if (m_net == nullptr || m_yPtr == nullptr)
            throw SpmvHostError(XJPCG_STATUS_NOT_INITIALIZED, "run: connect() and createStoreYbufs() first");
        m_mem.assign(static_cast<const unsigned char*>(m_yPtr), static_cast<const unsigned char*>(m_yPtr) + m_yBytes);
        m_mem.resize((m_yBytes + 7) / 8 * 8, 0u);
        uint64_t used = 0;
        const XJPCG_Status_t st = xJPCG_gbStoreYFrames(m_net->data(), m_net->size(), m_nodes,
                                                       reinterpret_cast<double*>(m_mem.data()), m_yBytes, &used);
        m_net->consume((size_t)used);
        if (st != XJPCG_STATUS_SUCCESS)
            throw SpmvHostError(st, "run: a transY frame is malformed or writes past the y buffer");
    }
    void getY() { std::memcpy(m_yPtr, m_mem.data(), m_yBytes); }

   private:
    hpc_common::FPGA* m_card = nullptr;
    size_t m_yBytes = 0;
    void* m_yPtr = nullptr;
    unsigned int m_nodes = 0;
    NetStream* m_net = nullptr;
    std::vector<unsigned char> m_mem;
};

}  // namespace dspmv
}  // namespace xilinx_apps

#endif  // XJPCG_SPMVHOST_GB300_HPP
