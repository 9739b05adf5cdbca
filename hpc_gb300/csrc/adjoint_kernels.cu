// adjoint_kernels.cu -- gradients of a converged solve x = A^-1 b.
//
// For a loss L(x) with g = dL/dx, the adjoint is lambda = A^-T g = A^-1 g (A is
// SPD), a second JPCG solve through the same kernels.  Then
//   dL/db    = lambda
//   dL/dA_ij = -lambda_i x_j            (per stored entry: grad_nnz_kernel)
// and for a diffusion matrix A = sum_e c_e (e_i - e_j)(e_i - e_j)^T + G with
// c_e = exp(theta_e):
//   dL/dc_e     = -(lambda_i - lambda_j)(x_i - x_j)
//   dL/dtheta_e = c_e dL/dc_e             (edge_grad_kernel)
// Only the converged x and lambda are used; no iterate history is kept.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "xjpcg_device.cuh"
#include "xjpcg_internal.hpp"

namespace xjpcg {

// One warp per row: slot j of row i gets -lambda_i x_col(j), written at the
// input position perm[j] (or at j when perm is null).
__global__ void grad_nnz_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                const uint32_t* __restrict__ perm, const double* __restrict__ x,
                                const double* __restrict__ lambda, double* __restrict__ grad) {
    const int lane = threadIdx.x & 31;
    const int warpsPerGrid = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warpsPerGrid) {
        const double li = -lambda[i];
        for (int j = rowptr[i] + lane; j < rowptr[i + 1]; j += 32) {
            const double gv = li * x[col[j]];
            grad[perm ? perm[j] : (uint32_t)j] = gv;
        }
    }
}

__global__ void edge_grad_kernel(int64_t m, const int* __restrict__ ei, const int* __restrict__ ej,
                                 const double* __restrict__ c, const double* __restrict__ x,
                                 const double* __restrict__ lambda, double* __restrict__ grad) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const int i = ei[e], j = ej[e];
        grad[e] = -c[e] * (lambda[i] - lambda[j]) * (x[i] - x[j]);
    }
}

__global__ void edge_check_kernel(int64_t m, int n, const int* __restrict__ ei, const int* __restrict__ ej, int* flag) {
    bool bad = false;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x)
        bad |= (ei[e] < 0 || ei[e] >= n || ej[e] < 0 || ej[e] >= n);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

cudaError_t grad_nnz_launch(cudaStream_t st, int n, const int* rowptr, const int* col, const uint32_t* perm,
                            const double* x, const double* lambda, double* grad) {
    const int grid = std::max(1, std::min((int)(((int64_t)n * 32 + 255) / 256), device_sm_count() * 32));
    grad_nnz_kernel<<<grid, 256, 0, st>>>(n, rowptr, col, perm, x, lambda, grad);
    return cudaGetLastError();
}

cudaError_t edge_grad_launch(cudaStream_t st, int64_t m, int n, const int* ei, const int* ej, const double* c,
                             const double* x, const double* lambda, double* grad, int* flag, int* hostBad) {
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((m + 255) / 256, device_sm_count() * 32));
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    edge_check_kernel<<<grid, 256, 0, st>>>(m, n, ei, ej, flag);
    e = cudaMemcpyAsync(hostBad, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess || *hostBad) return e;
    edge_grad_kernel<<<grid, 256, 0, st>>>(m, ei, ej, c, x, lambda, grad);
    return cudaGetLastError();
}

}  // namespace xjpcg
