/* An application of the xJPCG C API linked against libXilinxPcg_loader.a
 * (-ldl) instead of libXilinxPcg.so: every call goes through the dlopen
 * loader.  Modes:
 *   loader_app errstr        error strings and the loader's error state
 *   loader_app create        createHandle / destroyHandle status
 *   loader_app solve N       tridiagonal COO solve (diag 4, off-diagonal -1,
 *                            b = 1), prints status, iterations, the reported
 *                            residual and the true relative residual
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pcg.h"

static int run_errstr(void) {
    printf("str3=%s\n", xJPCG_getErrorString(XJPCG_STATUS_INVALID_VALUE));
    printf("str6=%s\n", xJPCG_getErrorString(XJPCG_STATUS_DYNAMIC_LOADING_ERROR));
    printf("peek=%d\n", (int)xJPCG_peekAtLastStatus(NULL));
    const char* m = xJPCG_getLastMessage(NULL);
    printf("msg=%s\n", m ? m : "(null)");
    return 0;
}

static int run_create(void) {
    XJPCG_Handle_t* h = NULL;
    XJPCG_Status_t st = xJPCG_createHandle(&h, "");
    printf("create=%d\n", (int)st);
    const char* m = xJPCG_getLastMessage(h);
    printf("msg=%s\n", m ? m : "(null)");
    if (h != NULL) printf("destroy=%d\n", (int)xJPCG_destroyHandle(h));
    return 0;
}

static int run_solve(uint32_t n) {
    uint32_t nnz = 3 * n - 2, k = 0;
    uint32_t* row = malloc(sizeof(uint32_t) * nnz);
    uint32_t* col = malloc(sizeof(uint32_t) * nnz);
    double* val = malloc(sizeof(double) * nnz);
    double* diag = malloc(sizeof(double) * n);
    double* b = malloc(sizeof(double) * n);
    double* x = malloc(sizeof(double) * n);
    for (uint32_t i = 0; i < n; ++i) {
        if (i > 0) { row[k] = i; col[k] = i - 1; val[k++] = -1.0; }
        row[k] = i; col[k] = i; val[k++] = 4.0;
        if (i + 1 < n) { row[k] = i; col[k] = i + 1; val[k++] = -1.0; }
        diag[i] = 4.0;
        b[i] = 1.0;
        x[i] = 0.0;
    }
    XJPCG_Handle_t* h = NULL;
    XJPCG_Status_t st = xJPCG_createHandle(&h, "");
    if (st != XJPCG_STATUS_SUCCESS) {
        printf("create=%d msg=%s\n", (int)st, xJPCG_getLastMessage(h));
        return 1;
    }
    uint32_t iter = 0;
    double res = 0.0;
    st = xJPCG_cooSolver(h, n, nnz, row, col, val, diag, b, x, 1000, 1e-10, &iter, &res, XJPCG_MODE_DEFAULT);
    XJPCG_Metric_t met;
    XJPCG_Status_t stm = xJPCG_getMetrics(h, &met);
    double rr = 0.0, bb = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        double ax = 4.0 * x[i] - (i > 0 ? x[i - 1] : 0.0) - (i + 1 < n ? x[i + 1] : 0.0);
        rr += (b[i] - ax) * (b[i] - ax);
        bb += b[i] * b[i];
    }
    printf("status=%d iter=%u res=%.6e true=%.6e metrics=%d peek=%d\n", (int)st, iter, res, sqrt(rr / bb),
           (int)stm, (int)xJPCG_peekAtLastStatus(h));
    xJPCG_destroyHandle(h);
    free(row); free(col); free(val); free(diag); free(b); free(x);
    return st == XJPCG_STATUS_SUCCESS ? 0 : 1;
}

int main(int argc, char** argv) {
    if (argc >= 2 && strcmp(argv[1], "errstr") == 0) return run_errstr();
    if (argc >= 2 && strcmp(argv[1], "create") == 0) return run_create();
    if (argc >= 3 && strcmp(argv[1], "solve") == 0) return run_solve((uint32_t)strtoul(argv[2], NULL, 10));
    fprintf(stderr, "usage: loader_app errstr | create | solve N\n");
    return 2;
}
