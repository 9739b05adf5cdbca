// xjpcg_internal.hpp -- host-visible declarations of the device launchers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace xjpcg {

struct CgState;

// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount),
// read once per device and cached; grid-stride launches cap their grids at a
// multiple of it.  Falls back to 1 if the query fails (the launch stays correct,
// grid-stride loops cover the work).
inline int device_sm_count() {
    constexpr int kMaxDev = 64;
    static int cache[kMaxDev] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) {
        cudaGetLastError();
        return 1;
    }
    int v = __atomic_load_n(&cache[dev], __ATOMIC_RELAXED);
    if (v > 0) return v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
        cudaGetLastError();
        return 1;
    }
    __atomic_store_n(&cache[dev], v, __ATOMIC_RELAXED);
    return v;
}

// ---- SpMV (spmv_kernels.cu) ----
int spmv_num_configs();
int spmv_config_lanes(int cfg);
void spmv_config_shape(int cfg, int* lanes, int* consumers, int* chunk, int* stages);
// Row-pointer arrays must hold n + 1 + kRowptrPad entries (the SpMV copies
// fixed-size, 16-byte aligned slices of them).
constexpr int kRowptrPad = 160;
template <typename VT>
int spmv_grid(int cfg, int n, int numSms);
template <typename VT>
cudaError_t spmv_launch(int cfg, int grid, cudaStream_t st, int n, const int* rowptr, const int* col, const VT* val,
                        const VT* x, VT* y, const VT* b, CgState* state, double* partials, int mode,
                        const uint32_t* doneFlag);
// kSpmvCgPart: y = A p and each CTA's partial p.y in partials[blockIdx.x],
// with no grid reduction: the fused vector kernel adds them (kernels with
// 256-thread CTAs, whose order it repeats; spmv_config_partials says which).
enum : int { kSpmvPlain = 0, kSpmvCgDot = 1, kSpmvResidual = 2, kSpmvCgPart = 3 };

// ---- sliced SpMV layout (spmv_kernels.cu) ----
int sell_num_configs();
int sell_config_unroll(int cfg);
bool sell_config_narrow(int cfg);  // int16 column offsets instead of int32 columns
// sliceOff must hold nslices + 1 ints; *total = stored entries (padded).
cudaError_t sell_build(cudaStream_t st, int n, const int* rowptr, const int* col, const double* val, int* sliceOff,
                       int* blockSums, int64_t* total);
template <typename VT>
cudaError_t sell_fill(cudaStream_t st, int n, const int* rowptr, const int* col, const double* val,
                      const int* sliceOff, int* scol, VT* sval);
// *fits = every |col - row| <= 32767 (flag: one device int of scratch).
cudaError_t sell_narrow_fits(cudaStream_t st, int n, const int* rowptr, const int* col, int* flag, bool* fits);
cudaError_t sell_fill_narrow(cudaStream_t st, int n, const int* rowptr, const int* col, const int* sliceOff,
                             int16_t* scol16);
template <typename VT>
int sell_grid(int cfg, int n, int numSms);
template <typename VT>
cudaError_t spmv_sell_launch(int cfg, int grid, cudaStream_t st, int n, const int* sliceOff, const int* scol,
                             const int16_t* scol16, const VT* sval, const VT* x, VT* y, const VT* b, CgState* state,
                             double* partials, int mode, const uint32_t* doneFlag);

// ---- sliced SpMV with slice-shared column offsets (spmv_sellpat.cu) ----
int sellpat_num_configs();
int sellpat_config_unroll(int cfg);
int sellpat_config_tma(int cfg);  // 1: values prefetched by TMA bulk copies (FP32 only)
int sellpat_config_runs(int cfg);  // 1: run-aware x gathers (consecutive offsets passed by shuffle)
// All per-slice arrays hold nslices + 1 ints.  totals = {stored values,
// general-slice columns, stored patterns}.
cudaError_t sellpat_plan(cudaStream_t st, int n, const int* rowptr, const int* col, int* sliceOff, int* patLen,
                         int* patNew, int* patIdx, int* genOff, int* blockSums, int64_t* totals);
// patOff: nPatterns + 1 ints; *patTotal = stored pattern entries.
cudaError_t sellpat_index(cudaStream_t st, int n, const int* patLen, const int* patNew, int* patIdx, int nPatterns,
                          int* patOff, int* blockSums, int64_t* patTotal);
template <typename VT>
cudaError_t sellpat_fill(cudaStream_t st, int n, const int* rowptr, const int* col, const double* val,
                         const int* sliceOff, const int* patLen, const int* patNew, const int* patIdx,
                         const int* patOff, const int* genOff, VT* sval, int* pat, int* gcol, bool writeIndex);
template <typename VT>
int sellpat_grid(int cfg, int n, int numSms);
template <typename VT>
cudaError_t spmv_sellpat_launch(int cfg, int grid, cudaStream_t st, int n, const int* sliceOff, const int* patLen,
                                const int* patIdx, const int* patOff, const int* genOff, const int* pat,
                                const int* gcol, const VT* sval, const VT* x, VT* y, const VT* b, CgState* state,
                                double* partials, int mode, const uint32_t* doneFlag);

// ---- bounded-wait diagnostic (cg_kernels.cu) ----
// out: 3 uint32 (status bits, wait duration in ns as two halves).
cudaError_t wait_probe_launch(cudaStream_t st, uint64_t budgetNs, uint32_t* out);
// The JPCG loop in the reference FPGA's arithmetic order (fpga_order.cu).
// z is written over Ap (Apz); t holds 2 * fo_blocks(n4) doubles.
int fo_blocks(int n4);
cudaError_t fo_init(cudaStream_t st, int n, int n4, const double* b, const double* diag, double* x, double* r,
                    double* p, double* J, double* z, CgState* s);
cudaError_t fo_iteration_tail(cudaStream_t st, int n4, double* x, double* p, double* r, double* Apz, const double* J,
                              double* t, CgState* s);
// FP64 issue-rate probe (cg_kernels.cu): out holds grid * 256 doubles.
int fp64_rate_grid(int numSms);
double fp64_rate_dfma(int grid, int iters);
cudaError_t fp64_rate_launch(cudaStream_t st, int grid, int iters, double* out);

// ---- length-sorted sliced SpMV (spmv_sellsort.cu) ----
int sellsort_num_configs();
int sellsort_config_unroll(int cfg);
int sellsort_tiles(int n);
int sellsort_bins();
// hist/start: sellsort_bins() * sellsort_tiles(n) ints each; sorted: n ints.
cudaError_t sellsort_order(cudaStream_t st, int n, const int* rowptr, int* hist, int* start, int* blockSums,
                           int* sorted, int* nLong);
// sliceOff: (n - nLong + 31) / 32 + 1 ints; *total = stored slice entries.
cudaError_t sellsort_slices(cudaStream_t st, int n, int nLong, const int* rowptr, const int* sorted, int* sliceOff,
                            int* blockSums, int64_t* total);
template <typename VT>
cudaError_t sellsort_fill(cudaStream_t st, int n, int nLong, const int* rowptr, const int* col, const double* val,
                          const int* sorted, const int* sliceOff, int* scol, VT* sval);
template <typename VT>
int sellsort_grid(int cfg, int n, int nLong, int numSms);
template <typename VT>
cudaError_t spmv_sellsort_launch(int cfg, int grid, cudaStream_t st, int n, int nLong, const int* sorted,
                                 const int* sliceOff, const int* scol, const VT* sval, const int* rowptr,
                                 const int* col, const VT* val, const VT* x, VT* y, const VT* b, CgState* state,
                                 double* partials, int mode, const uint32_t* doneFlag);

// ---- merge-path SpMV (spmv_merge.cu) ----
// Scratch per matrix: tileRow[ntiles + 1] ints (merge_partition), carryRow[ntiles] ints, carryVal[ntiles] accumulators
// (double for fp64, float for fp32), partials[ntiles + merge_fixup_grid(ntiles)].
int merge_tiles(int n, int64_t nnz);
int merge_items_per_thread();
int merge_fixup_grid(int ntiles);
cudaError_t merge_partition(cudaStream_t st, int n, int nnz, const int* rowptr, int* tileRow);
template <typename VT>
cudaError_t spmv_merge_launch(cudaStream_t st, int n, int nnz, const int* rowptr, const int* col, const VT* val,
                              const VT* x, VT* y, const int* tileRow, int* carryRow, void* carryVal, double* partials,
                              CgState* state, int mode, const uint32_t* doneFlag);
template <typename VT>
cudaError_t residual_finish_launch(cudaStream_t st, int n, const VT* b, VT* y, double* partials, CgState* state,
                                   const uint32_t* doneFlag);

// ---- CG vector kernels (cg_kernels.cu) ----
int vec_grid(int n4, int numSms);
int update_grid(int n4, int numSms);
// update + p update in one cooperative launch (cg_kernels.cu); grid from
// fused_grid (every CTA resident); partials hold 2 * grid doubles.
int fused_grid(int n4, int numSms);
// The fused kernel's barrier uses partials[kFusedPartialOff ...), clear of an
// SpMV's per-CTA partials (at most kFusedPartialOff CTAs); nbSpmv > 0: alpha
// from the SpMV's kSpmvCgPart partials, 0: alpha from the state.
constexpr int kFusedPartialOff = 8192;
cudaError_t cg_fused_launch(int grid, cudaStream_t st, int n4, double* x, double* r, double* p, double* Apz,
                            const double* J, CgState* state, double* partials, int nbSpmv);
cudaError_t cg_init_launch(int grid, cudaStream_t st, int n, int n4, const double* b, const double* diag, double* x,
                           double* r, double* p, double* J, double* Ap, CgState* state, double* partials);
// update: r -= alpha Ap, then z = J r is written over Ap; p update reads it
cudaError_t cg_update_launch(int grid, cudaStream_t st, int n4, double* r, double* Ap, const double* J,
                             CgState* state, double* partials);
cudaError_t cg_pupdate_launch(int grid, cudaStream_t st, int n4, double* x, double* p, const double* z,
                              CgState* state);

// ---- mixed precision, reliable updates (mixed_kernels.cu) ----
cudaError_t rel_init_launch(int grid, cudaStream_t s, int n, int n4, const double* b, const double* diag, double* x,
                            float* d, float* J, float* r, float* p, CgState* st, double* partials);
int rel_fused_grid(int n4, int numSms);
cudaError_t rel_fused_launch(int grid, cudaStream_t s, int n4, float* d, float* r, float* p, const float* Ap,
                             const float* J, CgState* st, double* partials);
cudaError_t rel_update_launch(int grid, cudaStream_t s, int n4, float* d, float* r, const float* p, const float* Ap,
                              const float* J, CgState* st, double* partials);
cudaError_t rel_fold_launch(int grid, cudaStream_t s, int n4, double* x, float* d, const CgState* st);
cudaError_t rel_restart_launch(int grid, cudaStream_t s, int n4, const double* r64, const float* J, float* r,
                               CgState* st, double* partials);
cudaError_t rel_pupdate_launch(int grid, cudaStream_t s, int n4, float* p, const float* r, const float* J,
                               CgState* st);

// ---- batched solves (batched_kernels.cu) ----
struct BatchResult {      // layout of XJPCG_GbBatchResult_t
    uint32_t iters;       // reported iterations (min(K, maxIter)); mixed: inner iterations
    uint32_t itersRun;    // iterations executed (K)
    uint32_t outer;       // mixed: refinement sweeps
    uint32_t status;      // 0 ok, 1 breakdown (non-finite alpha / beta / r.r)
    double res;           // fp64: sqrt(r.r / b.b) of the recursive residual; mixed: true residual
};
struct BatchLaunch {
    int nsys;
    const int* sysRow;
    const int* order;
    const int* rowptr;
    const int* col;
    const double* val;
    const float* val32;
    const double* b;
    const double* diag;
    double* x;
    double* r;
    double* Ap;
    double* J;
    float* r32;
    float* d32;
    float* Ap32;
    float* J32;
    double* pGlobal;
    float* p32Global;
    BatchResult* res;
    uint32_t* queue;
    uint32_t maxIterP1;
    double tol;
    double delta2;  // mixed: reliable-update threshold, squared
    // per-system SELL-32 copy for the sliced kernels (null: not built)
    const int* sliceBase = nullptr;
    const int* sliceOff = nullptr;
    const double* sval = nullptr;
    const float* sval32 = nullptr;
    const uint16_t* scol = nullptr;
    const int* patLen = nullptr;  // per slice: shared column offsets, or 0
    const int* patOff = nullptr;  // kBatchPatMax per slice
    const int2* meta = nullptr;   // per slice: {value offset, width | kSliceSysPat}
    const int* sysPat = nullptr;  // per system: pattern length, then kBatchPatMax offsets
};
int batch_num_configs();
cudaError_t batch_validate_columns(cudaStream_t st, int nsys, const int* sysRow, const int* rowptr, const int* col,
                                   int* flag);
void batch_config_shape(int cfg, int* threads, int* lanes);
bool batch_config_sliced(int cfg);  // the kernel reads the per-system SELL-32 copy
// Shared column offsets per slice of the batched SELL-32 copy: at most this
// many, stored kBatchPatMax ints per slice.
constexpr int kBatchPatMax = 8;
// Flag in a slice record's width word: the slice uses its system's offsets.
constexpr int kSliceSysPat = 1 << 30;
cudaError_t batch_sell_meta(cudaStream_t st, int nsys, int nslices, const int* sysRow, const int* sliceBase,
                            const int* sliceOff, const int* patLen, const int* patOff, int2* meta, int* sysPat);
cudaError_t batch_sell_widths(cudaStream_t st, int nsys, int nslices, const int* sysRow, const int* sliceBase,
                              const int* rowptr, const int* col, int* sliceLen, int* sliceOff, int* blockSums,
                              int* patLen, int* patOff, bool patterns);
template <typename VT>
cudaError_t batch_sell_fill(cudaStream_t st, int nsys, int nslices, const int* sysRow, const int* sliceBase,
                            const int* rowptr, const int* col, const double* val, const int* sliceOff,
                            const int* patLen, const int* patOff, VT* sval, uint16_t* scol);
cudaError_t batch_launch(int cfg, bool mixed, int numSms, int smemRows, cudaStream_t st, const BatchLaunch& L,
                         int* gridOut);


// ---- partitioned-matrix ("signature") input (signature_kernels.cu) ----
struct SigChunk {
    int64_t byteStart;   // offset of the chunk in the concatenated channel buffers
    int64_t groupStart;  // first global 4-entry group of the chunk
    int32_t rowBase;     // row-block start + the channel's row offset
    int32_t colBase;     // partition base column block + the channel's offset
};
cudaError_t sig_decode(cudaStream_t st, int nchunks, const SigChunk* chunks, const unsigned char* buf, int64_t groups,
                       uint32_t* row, uint32_t* col, double* val, int* keep);
cudaError_t sig_compact(cudaStream_t st, int64_t count, const int* pos, const int* keep, const uint32_t* row,
                        const uint32_t* col, const double* val, uint32_t* rowOut, uint32_t* colOut, double* valOut);
cudaError_t transy_frame(cudaStream_t st, uint32_t startAddr, uint32_t rows, const double* y, unsigned char* frame);
// runs of 32 stored entries (one row index each): their rows and indices
cudaError_t sig_run_rows(cudaStream_t st, int64_t runs, const uint32_t* row, uint32_t* runRow, uint32_t* runIdx);
// y = A x in the reference FPGA's summation order over the decoded stored entries
cudaError_t sig_ordered_spmv(cudaStream_t st, int rows, const int* runPtr, const int* runIdx, const double* val,
                             const uint32_t* col, const double* x, double* y);

// ---- adjoint (adjoint_kernels.cu) ----
cudaError_t grad_nnz_launch(cudaStream_t st, int n, const int* rowptr, const int* col, const uint32_t* perm,
                            const double* x, const double* lambda, double* grad);
cudaError_t edge_grad_launch(cudaStream_t st, int64_t m, int n, const int* ei, const int* ej, const double* c,
                             const double* x, const double* lambda, double* grad, int* flag, int* hostBad);

// ---- conversion (convert_kernels.cu) ----
// All return cudaSuccess or the first CUDA error; data errors are reported
// through *errFlag (device int) as kStatusIndexError / kStatusCountError.
struct ConvertScratch {
    int* counts = nullptr;      // n + 1
    int* fill = nullptr;        // n
    int* blockSums = nullptr;   // scan scratch
    uint64_t* keys = nullptr;   // nnz
    int* flags = nullptr;       // device int flags[4]
    size_t countsCap = 0, keysCap = 0, blockCap = 0;
};
cudaError_t scan_exclusive(cudaStream_t st, const int* in, int* out, int count, int* blockSums);
int scan_block_count(int count);
cudaError_t coo_to_csr(cudaStream_t st, int n, int64_t nnz, const uint32_t* row, const uint32_t* col, int base,
                       int* rowptr, int* colOut, uint32_t* perm, ConvertScratch& scratch, int* hostErr);
cudaError_t gather_values(cudaStream_t st, int64_t nnz, const uint32_t* perm, const double* src, double* dst);
// 64-bit fingerprint of a CSR structure (row pointers and columns).
cudaError_t struct_hash(cudaStream_t st, int n, int64_t nnz, const int* rowptr, const int* col,
                        unsigned long long* scratch, uint64_t* hash);
cudaError_t cscsym_expand(cudaStream_t st, int n, int64_t nnzHalf, int64_t nnzFull, const int64_t* rowIdx,
                          const int64_t* colPtr, const double* data, int base, uint32_t* rowOut, uint32_t* colOut,
                          double* valOut, int64_t* posScratch, int* flagScratch, int* blockSums, int* hostErr);
cudaError_t convert_f64_to_f32(cudaStream_t st, int64_t count, const double* src, float* dst);

}  // namespace xjpcg
