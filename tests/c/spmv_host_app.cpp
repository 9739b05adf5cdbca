// spmv_host_app.cpp -- an application written against the reference's SpMV
// host classes, built against include/spmvHost_gb300.hpp and libXilinxPcg.so.
//
// Part 1 replays the call sequence of the reference's SpMV test
// (L2/sparse/tests/fp64/spmv/main.cpp:71-191): read the partitioned matrix
// (nnzVal_0..15.dat, parParam.dat, rbParam.dat, info.dat) and the vectors
// (inVec.dat, refVec.dat), run SpmvHost<16> (init, createKernels, create*Bufs,
// setStoreYrows, sendBOs, run, getY, finish), write outVec.dat and compare
// with refVec.dat as that test does (isClose<float>(1e-4, 3e-6) per entry,
// utils/include/sw/utils.hpp:82-97).
//
// Part 2 is the distributed form (dSpmv): two compute cards each run
// dSpmvComputeHost<16> on the same matrix and send their rows over a
// NetStream, card 0 at memory word 0 and card 1 right after card 0's rows
// (rounded up to whole 64-byte words); the store card's dSpmvStoreYhost<16>
// assembles them.  Each half must equal its card's y bit for bit (the
// compute -> frame -> store round trip), the words after each half must hold
// the transY zero fill, and each card's y must pass the reference test's
// compare against refVec (each card tunes its own SpMV, so the cards' sums
// may differ from part 1's in the last bits).
//
// Usage: spmv_host_app <sig_dir> <vec_dir> [device id]; prints
// "INFO: Test pass!" and exits 0 when every check holds.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "spmvHost_gb300.hpp"

static std::vector<unsigned char> readBin(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        std::cerr << "ERROR: cannot open " << path << std::endl;
        std::exit(EXIT_FAILURE);
    }
    return std::vector<unsigned char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

static void writeBin(const std::string& path, const void* p, size_t bytes) {
    std::ofstream f(path, std::ios::binary);
    f.write(static_cast<const char*>(p), (std::streamsize)bytes);
}

// The reference test's compare for doubles: both values taken to float,
// |x - ref| <= 3e-6 + 1e-4 |ref| in float.
static bool isClose(double v, double ref) {
    const float fv = (float)v, fr = (float)ref;
    return std::fabs(fv - fr) <= (3e-6f + 1e-4f * std::fabs(fr));
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cerr << "Usage: " << argv[0] << " <sig_dir> <vec_dir> [device id]" << std::endl;
        return EXIT_FAILURE;
    }
    const std::string sigDir = argv[1], vecDir = argv[2];
    const int deviceId = argc > 3 ? std::atoi(argv[3]) : 0;
    constexpr unsigned int kCh = 16;

    std::vector<unsigned char> nnzBuf[kCh];
    void* nnzPtr[kCh];
    size_t nnzBytes[kCh];
    for (unsigned int i = 0; i < kCh; ++i) {
        nnzBuf[i] = readBin(sigDir + "/nnzVal_" + std::to_string(i) + ".dat");
        nnzPtr[i] = nnzBuf[i].data();
        nnzBytes[i] = nnzBuf[i].size();
    }
    std::vector<unsigned char> parXbuf[2] = {readBin(sigDir + "/parParam.dat"), readBin(vecDir + "/inVec.dat")};
    void* parXptr[2] = {parXbuf[0].data(), parXbuf[1].data()};
    size_t parXbytes[2] = {parXbuf[0].size(), parXbuf[1].size()};
    std::vector<unsigned char> rbBuf = readBin(sigDir + "/rbParam.dat");
    std::vector<unsigned char> refBuf = readBin(vecDir + "/refVec.dat");
    std::vector<unsigned char> infoBuf = readBin(sigDir + "/info.dat");
    const unsigned int yRows = (unsigned int)(refBuf.size() / sizeof(double));
    std::vector<double> y(yRows, 0.0);
    const double* ref = reinterpret_cast<const double*>(refBuf.data());

    uint32_t info[6] = {};
    std::memcpy(info, infoBuf.data(), std::min(sizeof(info), infoBuf.size()));
    std::cout << "INFO: matrix original m n nnz; padded m n nnz: ";
    for (unsigned int i = 0; i < 6; ++i) std::cout << info[i] << " ";
    std::cout << std::endl;

    try {
        // ---- part 1: SpmvHost, the reference test's sequence ----
        xilinx_apps::hpc_common::FPGA card;
        card.setId(deviceId);
        card.load_xclbin("spmv.xclbin");
        xilinx_apps::sparse::SpmvHost<kCh> spmvHost;
        spmvHost.init(&card);
        spmvHost.createKernels();
        spmvHost.createLoadNnzBufs(nnzBytes, nnzPtr);
        spmvHost.createLoadParXbufs(parXbytes, parXptr);
        spmvHost.createLoadRbParamBufs(rbBuf.size(), rbBuf.data());
        spmvHost.createStoreYbufs(y.size() * sizeof(double), y.data());
        spmvHost.setStoreYrows(yRows);
        spmvHost.sendBOs();
        spmvHost.run();
        spmvHost.getY();
        spmvHost.finish();
        writeBin(vecDir + "/outVec.dat", y.data(), y.size() * sizeof(double));
        int errs = 0;
        for (unsigned int i = 0; i < yRows; ++i) errs += isClose(y[i], ref[i]) ? 0 : 1;
        if (errs != 0) {
            std::cout << "ERROR: SpmvHost: " << errs << " of " << yRows << " entries mismatch" << std::endl;
            return EXIT_FAILURE;
        }

        // ---- part 2: two compute cards, one store card ----
        const unsigned int words0 = (yRows + 7) / 8;  // 64-byte words card 0 sends
        const unsigned int start1 = 2 * words0;       // card 1's rows, in 32-byte memory words
        const size_t memDoubles = 8 * (size_t)words0 * 2;
        std::vector<double> mem(memDoubles, -1.0);    // the store card's result memory
        xilinx_apps::dspmv::NetStream net;
        xilinx_apps::hpc_common::FPGA cards[2];
        xilinx_apps::dspmv::dSpmvComputeHost<kCh> compute[2];
        for (int c = 0; c < 2; ++c) {
            cards[c].setId(deviceId);
            cards[c].load_xclbin("dspmv_compute.xclbin");
            compute[c].init(&cards[c]);
            compute[c].createKernels();
            compute[c].createLoadNnzBufs(nnzBytes, nnzPtr);
            compute[c].createLoadParXbufs(parXbytes, parXptr);
            compute[c].createLoadRbParamBufs(rbBuf.size(), rbBuf.data());
            compute[c].setKrnTransYargs(c == 0 ? 0u : start1, yRows);
            compute[c].connect(&net);
            compute[c].sendBOs();
            compute[c].run();
            compute[c].finish();
        }
        xilinx_apps::hpc_common::FPGA storeCard;
        storeCard.setId(deviceId);
        xilinx_apps::dspmv::dSpmvStoreYhost<kCh> store;
        store.init(&storeCard);
        store.createKernels();
        store.createStoreYbufs(mem.size() * sizeof(double), mem.data());
        store.setStoreYargs(2);
        store.connect(&net);
        store.run();
        store.getY();
        if (net.size() != 0) {
            std::cout << "ERROR: dSpmv: " << net.size() << " bytes of frames left unread" << std::endl;
            return EXIT_FAILURE;
        }
        for (int c = 0; c < 2; ++c) {
            const double* part = mem.data() + (c == 0 ? 0 : 4 * (size_t)start1);
            const std::vector<double>& yc = compute[c].y();
            if (yc.size() != yRows || std::memcmp(part, yc.data(), yRows * sizeof(double)) != 0) {
                std::cout << "ERROR: dSpmv: the stored rows of card " << c << " differ from its y" << std::endl;
                return EXIT_FAILURE;
            }
            int cerrs = 0;
            for (unsigned int i = 0; i < yRows; ++i) cerrs += isClose(yc[i], ref[i]) ? 0 : 1;
            if (cerrs != 0) {
                std::cout << "ERROR: dSpmv: card " << c << ": " << cerrs << " entries mismatch refVec" << std::endl;
                return EXIT_FAILURE;
            }
            for (size_t i = yRows; i < 8 * (size_t)words0; ++i)
                if (part[i] != 0.0 || std::signbit(part[i])) {
                    std::cout << "ERROR: dSpmv: card " << c << " zero fill missing at " << i << std::endl;
                    return EXIT_FAILURE;
                }
        }
    } catch (const std::exception& e) {
        std::cout << "ERROR: " << e.what() << std::endl;
        return EXIT_FAILURE;
    }
    std::cout << "INFO: Test pass!" << std::endl;
    return EXIT_SUCCESS;
}
