/*
 * ref_partition_harness.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A small driver of our own that links the reference's host partitioner
 * (Xilinx/HPC L2/sparse/src/sw/c++/gen_signature.cpp and the headers under
 * L2/sparse/include/sw/fp64, utils/include/sw) so that the oracle and the
 * product's format conversion can be pinned against the reference itself.
 * It is compiled by oracle/build_ref.sh from the reference sources where they
 * lie; the binary goes to oracle/_ref/ and is never shipped or linked by the
 * product.
 *
 * Usage:
 *   ref_partition_harness coo <dir> <base>
 *       reads dir/meta.txt ("n nnz"), dir/row.bin, dir/col.bin (uint32),
 *       dir/data.bin (f64).  Writes:
 *         dir/ref_sorted_{row,col,data}.bin   SparseMatrix::loadCoo +
 *                                             sort_by_row (matrix_params.hpp)
 *         dir/sig/{rbParam,parParam,info,nnzVal_c}.dat
 *                                             SpmPar::partitionCooMat + storeMatPar
 *       and, if dir/data2.bin exists, dir/sig2/ from SpmPar::updateMat(data2)
 *       (the KEEP_NZ_LAYOUT path, signature.hpp:534-555).
 *   ref_partition_harness csc <dir> <base>
 *       reads dir/meta.txt ("n nnzHalf"), dir/rowidx.bin, dir/colptr.bin
 *       (int64), dir/data.bin (f64); full nnz = 2*nnzHalf - n
 *       (pcg/sw/include/impl/pcgImp.hpp:87).  Writes dir/ref_sorted_*.bin from
 *       loadCscSym + sort_by_row and dir/sig/ from partitionCscSymMat, and
 *       dir/sig2/ from updateCscSymMat(data2) when dir/data2.bin exists.
 * Exit status 0 on success, 3 when the reference raised an exception (its
 * message goes to dir/ref_error.txt).
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>
#include <sys/stat.h>

#include "gen_signature.hpp"
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T>
std::vector<T> readVec(const std::string& path, size_t count) {
    std::vector<T> v(count);
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path.c_str());
        exit(2);
    }
    size_t got = fread(v.data(), sizeof(T), count, f);
    fclose(f);
    if (got != count) {
        fprintf(stderr, "short read %s\n", path.c_str());
        exit(2);
    }
    return v;
}

template <typename T>
void writeVec(const std::string& path, const std::vector<T>& v) {
    FILE* f = fopen(path.c_str(), "wb");
    fwrite(v.data(), sizeof(T), v.size(), f);
    fclose(f);
}

bool exists(const std::string& p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

void dumpSorted(const std::string& dir, xf::sparse::SparseMatrix& m) {
    m.sort_by_row();
    writeVec(dir + "/ref_sorted_row.bin", m.m_row_list);
    writeVec(dir + "/ref_sorted_col.bin", m.m_col_list);
    writeVec(dir + "/ref_sorted_data.bin", m.m_data_list);
}

// Wall time of the reference's partition call alone (no file I/O), written to
// dir/ref_time.txt as "seconds threads" (threads = OpenMP's maximum).
void recordTime(const std::string& dir, double s) {
    std::ofstream t(dir + "/ref_time.txt");
#ifdef _OPENMP
    t << s << " " << omp_get_max_threads() << "\n";
#else
    t << s << " 1\n";
#endif
}

void storeTo(const std::string& dir, xf::sparse::MatPartition& par) {
    mkdir(dir.c_str(), 0755);
    xf::sparse::storeMatPar(dir, par);
}

} // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s coo|csc <dir> <base>\n", argv[0]);
        return 1;
    }
    std::string kind = argv[1], dir = argv[2];
    int base = atoi(argv[3]);
    uint32_t n = 0;
    uint64_t nnz = 0;
    {
        std::ifstream meta(dir + "/meta.txt");
        meta >> n >> nnz;
    }
    xf::sparse::SpmPar<double> spm(SPARSE_parEntries, SPARSE_accLatency, SPARSE_hbmChannels, SPARSE_maxRows,
                                   SPARSE_maxCols, SPARSE_hbmMemBits);
    try {
        if (kind == "coo") {
            auto row = readVec<uint32_t>(dir + "/row.bin", nnz);
            auto col = readVec<uint32_t>(dir + "/col.bin", nnz);
            auto data = readVec<double>(dir + "/data.bin", nnz);
            xf::sparse::SparseMatrix m;
            m.loadCoo(n, n, (uint32_t)nnz, row.data(), col.data(), base);
            dumpSorted(dir, m);
            const auto t0 = std::chrono::steady_clock::now();
            xf::sparse::MatPartition par = spm.partitionCooMat(n, n, (uint32_t)nnz, row.data(), col.data(), data.data(), base);
            recordTime(dir, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
            storeTo(dir + "/sig", par);
            if (exists(dir + "/data2.bin")) {
                auto data2 = readVec<double>(dir + "/data2.bin", nnz);
                spm.checkUpdateDim(n, n, (uint32_t)nnz);
                xf::sparse::MatPartition par2 = spm.updateMat(data2.data());
                storeTo(dir + "/sig2", par2);
            }
        } else {
            auto rowIdx = readVec<int64_t>(dir + "/rowidx.bin", nnz);
            auto colPtr = readVec<int64_t>(dir + "/colptr.bin", (size_t)n + 1);
            auto data = readVec<double>(dir + "/data.bin", nnz);
            uint32_t full = (uint32_t)(nnz * 2 - n);
            xf::sparse::SparseMatrix m;
            m.loadCscSym(n, full, rowIdx.data(), colPtr.data(), base);
            dumpSorted(dir, m);
            const auto t0 = std::chrono::steady_clock::now();
            xf::sparse::MatPartition par = spm.partitionCscSymMat(n, full, rowIdx.data(), colPtr.data(), data.data(), base);
            recordTime(dir, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
            storeTo(dir + "/sig", par);
            if (exists(dir + "/data2.bin")) {
                auto data2 = readVec<double>(dir + "/data2.bin", nnz);
                spm.checkUpdateDim(n, n, full);
                xf::sparse::MatPartition par2 =
                    spm.updateCscSymMat(n, full, rowIdx.data(), colPtr.data(), data2.data(), base);
                storeTo(dir + "/sig2", par2);
            }
        }
    } catch (const std::exception& e) {
        std::ofstream err(dir + "/ref_error.txt");
        err << e.what() << "\n";
        return 3;
    }
    return 0;
}
