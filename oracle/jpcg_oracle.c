/*
 * jpcg_oracle.c -- CPU restatement of the xJPCG hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/, the smoke
 * test in __graft_entry__.py and the cpu_baseline / reference arm of bench.py
 * may load it.  The product library (hpc_gb300/) never links or calls it.
 *
 * What is restated, with the reference file each part follows (paths are
 * relative to the Xilinx/HPC tree):
 *
 *   orc_coo_to_csr      COO (C or Fortran base) -> row-major order that the
 *                       reference partitioner stores: stable sort by row
 *                       (L2/sparse/include/sw/fp64/matrix_params.hpp:51-79,
 *                       219-246), then per row block a stable sort by column
 *                       (signature.hpp:135-169) and per partition a stable sort
 *                       by row (signature.hpp:233-236).  Net effect per row:
 *                       entries ordered by (column, original position).
 *   orc_cscsym_expand   symmetric half-CSC -> full COO list in the reference's
 *                       emission order (matrix_params.hpp:82-134 for indices,
 *                       gen_signature.hpp:73-112 for values).
 *   orc_spmv            y = A x over that CSR, one sequential sum per row.
 *   orc_jpcg            the Jacobi-PCG loop with the xJPCG semantics:
 *                       vector init and 4-padding (pcg/sw/include/impl/
 *                       cgVector.hpp:55-114), instruction slot 0 with
 *                       MaxIter = maxIter+1 and Tols = bb*tol^2
 *                       (cgVector.hpp:149-159, pcgImp.hpp:157-158), per
 *                       iteration SpMV + p.Ap + alpha (pcg/hw/src/
 *                       krnl_storeApk.cpp:63-73), x update (L1/hpc/include/hw/
 *                       cgSolver/update_xk.hpp:26-67), r/z/rr/rz/beta
 *                       (update_rk_jacobi.hpp:29-110), p update
 *                       (update_pk.hpp:26-72), loop control and per-iteration
 *                       record (pcg/hw/include/control.hpp:65-92, L1/hpc/
 *                       include/hw/cgSolver/tasks.hpp:43-47), result scan
 *                       (pcgImp.hpp:171-180) and res = sqrt(Res/bb)
 *                       (pcg/sw/src/pcg.cpp:159).
 *
 * Summation order.  The FPGA's dot products are a 4-lane tree followed by a
 * delayed-adder accumulation (L1/blas/include/hw/blas/helpers/funcs/
 * dotHelper.hpp, sum.hpp).  The oracle keeps the 4-lane tree and accumulates
 * the 4-lane sums in fixed blocks of ORC_BLOCK elements that are combined in
 * order, so results do not depend on the number of OpenMP threads.  The vector
 * init sums (bb, rz) are sequential, as in cgVector.hpp:106-113.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_BLOCK 4096

typedef struct {
    uint32_t id, iter, vecSize, maxIter;
    double tols, res, rz, alpha, beta;
    uint64_t clock;
} orc_record_t; /* 64-byte record: pcg/hw/include/impl/cgInstr.hpp:117-132 */

static void orc_set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Format conversion                                                          */
/* ------------------------------------------------------------------------ */

/* Stable merge sort of (col, orig) pairs inside one row; insertion sort for
 * short rows.  Keys compare by column only, so equal columns keep their
 * original order (duplicates are kept, as the reference keeps them). */
static void row_sort(int32_t* col, uint32_t* perm, int64_t len, int32_t* tc, uint32_t* tp) {
    if (len <= 32) {
        for (int64_t i = 1; i < len; ++i) {
            int32_t c = col[i];
            uint32_t p = perm[i];
            int64_t j = i - 1;
            while (j >= 0 && col[j] > c) {
                col[j + 1] = col[j];
                perm[j + 1] = perm[j];
                --j;
            }
            col[j + 1] = c;
            perm[j + 1] = p;
        }
        return;
    }
    int64_t h = len / 2;
    row_sort(col, perm, h, tc, tp);
    row_sort(col + h, perm + h, len - h, tc, tp);
    int64_t i = 0, j = h, o = 0;
    while (i < h && j < len) {
        if (col[j] < col[i]) {
            tc[o] = col[j];
            tp[o++] = perm[j++];
        } else {
            tc[o] = col[i];
            tp[o++] = perm[i++];
        }
    }
    while (i < h) { tc[o] = col[i]; tp[o++] = perm[i++]; }
    while (j < len) { tc[o] = col[j]; tp[o++] = perm[j++]; }
    memcpy(col, tc, sizeof(int32_t) * len);
    memcpy(perm, tp, sizeof(uint32_t) * len);
}

/* Returns 0 on success, -1 on an index outside [base, n+base). */
int orc_coo_to_csr(uint32_t n, uint64_t nnz, const uint32_t* row, const uint32_t* col, int base,
                   int32_t* rowptr, int32_t* colOut, uint32_t* perm) {
    int64_t* cnt = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    if (!cnt) return -2;
    for (uint64_t k = 0; k < nnz; ++k) {
        uint32_t r = row[k] - (uint32_t)base, c = col[k] - (uint32_t)base;
        if (r >= n || c >= n) {
            free(cnt);
            return -1;
        }
        cnt[r + 1]++;
    }
    for (uint32_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    for (uint32_t i = 0; i <= n; ++i) rowptr[i] = (int32_t)cnt[i];
    for (uint64_t k = 0; k < nnz; ++k) { /* stable scatter by row */
        uint32_t r = row[k] - (uint32_t)base;
        int64_t pos = cnt[r]++;
        colOut[pos] = (int32_t)(col[k] - (uint32_t)base);
        perm[pos] = (uint32_t)k;
    }
    free(cnt);
    int64_t maxLen = 0;
    for (uint32_t i = 0; i < n; ++i) {
        int64_t l = rowptr[i + 1] - rowptr[i];
        if (l > maxLen) maxLen = l;
    }
    int32_t* tc = (int32_t*)malloc(sizeof(int32_t) * (maxLen + 1));
    uint32_t* tp = (uint32_t*)malloc(sizeof(uint32_t) * (maxLen + 1));
    for (uint32_t i = 0; i < n; ++i)
        row_sort(colOut + rowptr[i], perm + rowptr[i], rowptr[i + 1] - rowptr[i], tc, tp);
    free(tc);
    free(tp);
    return 0;
}

/* Symmetric half-CSC -> full COO in emission order.  valOut may be NULL.
 * Returns 0, or -1 when the emitted count differs from nnzFull (the reference
 * raises SpmAllocFailed / SpmInternalError there), -3 for a bad colPtr[0] in
 * Fortran mode (SpmInvalidValue in the reference). */
int orc_cscsym_expand(uint32_t n, uint64_t nnzFull, const int64_t* rowIdx, const int64_t* colPtr,
                      const double* data, int base, uint32_t* rowOut, uint32_t* colOut, double* valOut) {
    if (base == 1 && colPtr[0] < 1) return -3;
    uint64_t idx = 0;
    for (uint32_t j = 0; j < n; ++j) {
        for (int64_t k = colPtr[j] - base; k < colPtr[j + 1] - base; ++k) {
            int64_t i = rowIdx[k] - base;
            if (idx >= nnzFull) return -1;
            rowOut[idx] = (uint32_t)i;
            colOut[idx] = j;
            if (valOut) valOut[idx] = data[k];
            idx++;
            if (i != (int64_t)j) {
                if (idx >= nnzFull) return -1;
                rowOut[idx] = j;
                colOut[idx] = (uint32_t)i;
                if (valOut) valOut[idx] = data[k];
                idx++;
            }
        }
    }
    return idx == nnzFull ? 0 : -1;
}

/* ------------------------------------------------------------------------ */
/* Kernels of the loop                                                        */
/* ------------------------------------------------------------------------ */

void orc_spmv(uint32_t n, const int32_t* rowptr, const int32_t* col, const double* val, const double* x,
              double* y, int nthreads) {
    orc_set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        double s = 0.0;
        for (int32_t e = rowptr[i]; e < rowptr[i + 1]; ++e) s += val[e] * x[col[e]];
        y[i] = s;
    }
}

/* 4-lane tree of products, blocks of ORC_BLOCK combined in order.  n4 is a
 * multiple of 4. */
static double dot4(int64_t n4, const double* a, const double* b) {
    int64_t nb = (n4 + ORC_BLOCK - 1) / ORC_BLOCK;
    double* part = (double*)malloc(sizeof(double) * (nb > 0 ? nb : 1));
#pragma omp parallel for schedule(static)
    for (int64_t blk = 0; blk < nb; ++blk) {
        int64_t s = blk * ORC_BLOCK, e = s + ORC_BLOCK < n4 ? s + ORC_BLOCK : n4;
        double acc = 0.0;
        for (int64_t i = s; i < e; i += 4)
            acc += (a[i] * b[i] + a[i + 1] * b[i + 1]) + (a[i + 2] * b[i + 2] + a[i + 3] * b[i + 3]);
        part[blk] = acc;
    }
    double t = 0.0;
    for (int64_t blk = 0; blk < nb; ++blk) t += part[blk];
    free(part);
    return t;
}

/* r.r and r.(J*r) in one pass, same order as dot4. */
static void dot_rr_rz(int64_t n4, const double* r, const double* J, double* rr, double* rz) {
    int64_t nb = (n4 + ORC_BLOCK - 1) / ORC_BLOCK;
    double* part = (double*)malloc(sizeof(double) * 2 * (nb > 0 ? nb : 1));
#pragma omp parallel for schedule(static)
    for (int64_t blk = 0; blk < nb; ++blk) {
        int64_t s = blk * ORC_BLOCK, e = s + ORC_BLOCK < n4 ? s + ORC_BLOCK : n4;
        double a1 = 0.0, a2 = 0.0;
        for (int64_t i = s; i < e; i += 4) {
            double z0 = r[i] * J[i], z1 = r[i + 1] * J[i + 1], z2 = r[i + 2] * J[i + 2], z3 = r[i + 3] * J[i + 3];
            a1 += (r[i] * r[i] + r[i + 1] * r[i + 1]) + (r[i + 2] * r[i + 2] + r[i + 3] * r[i + 3]);
            a2 += (r[i] * z0 + r[i + 1] * z1) + (r[i + 2] * z2 + r[i + 3] * z3);
        }
        part[2 * blk] = a1;
        part[2 * blk + 1] = a2;
    }
    double t1 = 0.0, t2 = 0.0;
    for (int64_t blk = 0; blk < nb; ++blk) {
        t1 += part[2 * blk];
        t2 += part[2 * blk + 1];
    }
    free(part);
    *rr = t1;
    *rz = t2;
}

/*
 * Jacobi-PCG with the xJPCG contract.
 *   x        out, n entries (x0 = 0 always; the caller's x is never read)
 *   iterOut  reported iteration count (min(K, maxIter), K = iterations run)
 *   resOut   sqrt(Res_last / bb)
 *   kOut     K, the number of iterations that actually ran (may be NULL)
 *   records  optional, recCap slots; slot 0 = host command, slot k+1 = iteration k
 *   maxRun   if nonzero, stop after this many iterations (bounded CPU sample);
 *            the result is then not a converged solve.
 * Returns 0, or 1 when the run stopped on a non-finite alpha/beta/rr.
 */
int orc_jpcg(uint32_t n, const int32_t* rowptr, const int32_t* col, const double* val, const double* diag,
             const double* b, uint32_t maxIter, double tol, double* x, uint32_t* iterOut, double* resOut,
             uint32_t* kOut, orc_record_t* records, uint64_t recCap, uint32_t maxRun, int nthreads) {
    orc_set_threads(nthreads);
    int64_t n4 = ((int64_t)n + 3) / 4 * 4;
    double* J = (double*)malloc(sizeof(double) * n4);
    double* r = (double*)malloc(sizeof(double) * n4);
    double* p = (double*)malloc(sizeof(double) * n4);
    double* Ap = (double*)malloc(sizeof(double) * n4);
    double* xk = (double*)malloc(sizeof(double) * n4);
    double bb = 0.0, rz = 0.0;
    for (int64_t i = 0; i < n4; ++i) { /* cgVector.hpp:101-114 */
        double bi = i < (int64_t)n ? b[i] : 0.0;
        double di = i < (int64_t)n ? diag[i] : 1.0;
        r[i] = bi;
        J[i] = 1.0 / di;
        double z = J[i] * r[i];
        bb += bi * bi;
        rz += r[i] * z;
        p[i] = z;
        xk[i] = 0.0;
        Ap[i] = 0.0;
    }
    uint32_t maxIterP1 = maxIter + 1u;
    double tols = bb * tol * tol;
    if (records && recCap > 0) {
        memset(records, 0, sizeof(orc_record_t) * recCap);
        records[0].maxIter = maxIterP1;
        records[0].tols = tols;
        records[0].res = bb;
        records[0].rz = rz;
        records[0].vecSize = (uint32_t)n4;
    }
    uint32_t k = 0;
    double rr = bb, lastRes = 0.0;
    int status = 0;
    for (;;) {
        orc_spmv(n, rowptr, col, val, p, Ap, 0);
        for (int64_t i = n; i < n4; ++i) Ap[i] = 0.0;
        double pAp = dot4(n4, p, Ap);
        double alpha = rz / pAp;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n4; ++i) {
            xk[i] = alpha * p[i] + xk[i];
            r[i] = (-alpha) * Ap[i] + r[i];
        }
        double rzn;
        dot_rr_rz(n4, r, J, &rr, &rzn);
        double beta = rzn / rz;
        rz = rzn;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n4; ++i) p[i] = beta * p[i] + r[i] * J[i];
        if (records && (uint64_t)k + 1 < recCap) {
            orc_record_t* rec = &records[k + 1];
            rec->id = 0;
            rec->iter = k;
            rec->vecSize = (uint32_t)n4;
            rec->maxIter = maxIterP1;
            rec->tols = tols;
            rec->res = rr;
            rec->rz = rzn;
            rec->alpha = alpha;
            rec->beta = beta;
        }
        lastRes = rr;
        if (!isfinite(alpha) || !isfinite(beta) || !isfinite(rr)) {
            status = 1;
            k++;
            break;
        }
        /* control.hpp:83: continue iff !(rr < Tols) && ++iter < MaxIter */
        int cont = !(rr < tols);
        k++;
        cont = cont && (k < maxIterP1);
        if (maxRun && k >= maxRun) break;
        if (!cont) break;
    }
    /* pcgImp.hpp:171-180: the host scan reports min(K, maxIter) */
    uint32_t reported = k <= maxIter ? k : maxIter;
    if (iterOut) *iterOut = reported;
    if (kOut) *kOut = k;
    if (resOut) *resOut = sqrt(lastRes / bb);
    memcpy(x, xk, sizeof(double) * n);
    free(J);
    free(r);
    free(p);
    free(Ap);
    free(xk);
    return status;
}

/* Plain FP64 CG norm helpers used by tests for true-residual checks. */
double orc_true_relres(uint32_t n, const int32_t* rowptr, const int32_t* col, const double* val, const double* b,
                       const double* x, int nthreads) {
    double* y = (double*)malloc(sizeof(double) * n);
    orc_spmv(n, rowptr, col, val, x, y, nthreads);
    double num = 0.0, den = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        double d = b[i] - y[i];
        num += d * d;
        den += b[i] * b[i];
    }
    free(y);
    return sqrt(num / den);
}
