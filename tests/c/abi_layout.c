/* Prints the sizes and field offsets of the extension header's structs, for
 * the check that the Python binding's ctypes mirrors match them. */
#include <stddef.h>
#include <stdio.h>

#include "xjpcg_gb300.h"

#define F(T, f) printf("%s.%s=%zu\n", #T, #f, offsetof(T, f))

int main(void) {
    printf("XJPCG_GbInfo_t=%zu\n", sizeof(XJPCG_GbInfo_t));
    F(XJPCG_GbInfo_t, nnz);
    F(XJPCG_GbInfo_t, bb);
    F(XJPCG_GbInfo_t, solveMs);
    F(XJPCG_GbInfo_t, spmvLayout);
    F(XJPCG_GbInfo_t, batchMs);
    F(XJPCG_GbInfo_t, spmvCfg32);
    F(XJPCG_GbInfo_t, tuneMs);
    F(XJPCG_GbInfo_t, uploadMs);
    printf("XJPCG_GbSignature_t=%zu\n", sizeof(XJPCG_GbSignature_t));
    F(XJPCG_GbSignature_t, rowBlocks);
    F(XJPCG_GbSignature_t, rbParamBytes);
    F(XJPCG_GbSignature_t, nnzValBytes);
    printf("XJPCG_GbBatchResult_t=%zu\n", sizeof(XJPCG_GbBatchResult_t));
    F(XJPCG_GbBatchResult_t, res);
    printf("XJPCG_Metric_t=%zu\n", sizeof(XJPCG_Metric_t));
    return 0;
}
