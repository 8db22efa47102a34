// Dense inverse of a small coarsest-level operator, built on the device (sm_103a).
//
// The coarsest level of a multigrid hierarchy (at most a few thousand unknowns) is
// solved with one dense matrix-vector product by its explicit inverse.  The matrix
// comes from n applies of the level's operator to unit vectors (any operator:
// Laplacian or elasticity, matrix-free, stored element matrices or assembled), each
// writing one column of a device array with no host round trip; the inverse is formed
// in FP64 by Gauss-Jordan elimination (no pivoting: the operator's free block is SPD,
// every pivot is a positive Schur complement), one rank-1 update launch per column.
//
// Dirichlet dofs appear as identity rows (the operator copies constrained entries)
// while their columns keep the couplings: M = [[A_II, A_ID], [0, I]].  The SPD part S
// (constrained columns zeroed, symmetrised) is inverted and the couplings N folded
// back: M^-1 = S^-1 (I - N).
//
// No reference counterpart: the reference's coarsest level runs an iterative solver
// (algebra/sfem_Multigrid.hpp, the coarse solver slot).
#include <algorithm>

#include "common.cuh"

namespace sfem_gb300 {
namespace {

template <typename T>
__global__ void unit_vector_kernel(ptrdiff_t n, ptrdiff_t j, T *e) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        e[i] = i == j ? T(1) : T(0);
}

// A[i][j] = cols[j * ld + i]: column j holds A e_j
template <typename T>
__global__ void gather_matrix_kernel(ptrdiff_t n, ptrdiff_t ld, const T *__restrict__ cols, double *__restrict__ A) {
    for (ptrdiff_t k = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; k < n * n;
         k += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t i = k / n, j = k % n;
        A[k] = (double)cols[j * ld + i];
    }
}

// flags[i] = 1 if row i of A is the identity row e_i^T (a constrained dof); one warp per row
__global__ void identity_rows_kernel(ptrdiff_t n, const double *__restrict__ A, int *__restrict__ flags) {
    const ptrdiff_t i = (ptrdiff_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    bool id = true;
    for (ptrdiff_t j = lane; j < n; j += 32) id = id && (A[i * n + j] == (j == i ? 1.0 : 0.0));
    id = __all_sync(0xffffffffu, id);
    if (lane == 0) flags[i] = id ? 1 : 0;
}

// S = the symmetrised free block; constrained rows and columns the identity
__global__ void spd_part_kernel(ptrdiff_t n, const double *__restrict__ A, const int *__restrict__ flags,
                                double *__restrict__ S) {
    for (ptrdiff_t k = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; k < n * n;
         k += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t i = k / n, j = k % n;
        double v;
        if (flags[i] || flags[j])
            v = i == j ? 1.0 : 0.0;
        else
            v = 0.5 * (A[i * n + j] + A[j * n + i]);
        S[k] = v;
    }
}

// row k and column k of S before step k
__global__ void gj_save_kernel(ptrdiff_t n, ptrdiff_t k, const double *__restrict__ S, double *__restrict__ rc) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        rc[i] = S[i * n + k];
        rc[n + i] = S[k * n + i];
    }
}

// Gauss-Jordan step k in place: afterwards S holds the inverse in the columns 0..k
__global__ void gj_update_kernel(ptrdiff_t n, ptrdiff_t k, double *__restrict__ S, const double *__restrict__ rc,
                                 int *__restrict__ status) {
    const double p = rc[k];
    if (blockIdx.x == 0 && threadIdx.x == 0 && !(p > 0.0)) atomicExch(status, 1);
    const double ip = 1.0 / p;
    for (ptrdiff_t q = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; q < n * n;
         q += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t i = q / n, j = q % n;
        double v;
        if (i == k && j == k)
            v = ip;
        else if (i == k)
            v = rc[n + j] * ip;
        else if (j == k)
            v = -rc[i] * ip;
        else
            v = S[q] - rc[i] * ip * rc[n + j];
        S[q] = v;
    }
}

// inv[r][c] = Sinv[r][c] for a free column c; for a constrained c the folded coupling
// Sinv[r][c] - sum_{k != c} Sinv[r][k] A[k][c]; one warp per entry
template <typename T>
__global__ void fold_couplings_kernel(ptrdiff_t n, const double *__restrict__ Sinv, const double *__restrict__ A,
                                      const int *__restrict__ flags, T *__restrict__ inv) {
    const ptrdiff_t w = (ptrdiff_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n * n) return;
    const ptrdiff_t r = w / n, c = w % n;
    double v = 0;
    if (flags[c]) {
        for (ptrdiff_t k = lane; k < n; k += 32)
            if (k != c) v += Sinv[r * n + k] * A[k * n + c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    if (lane == 0) inv[w] = (T)(Sinv[w] - v);
}

template <typename T>
int dense_inverse_tpl(ptrdiff_t n, ptrdiff_t ld, const T *cols, double *A, double *S, double *rc, int *flags, T *inv,
                      cudaStream_t s) {
    const ptrdiff_t nn = n * n;
    int *status = flags + n;
    if (cudaMemsetAsync(status, 0, sizeof(int), s) != cudaSuccess) return set_error("dense inverse: memset failed");
    gather_matrix_kernel<T><<<grid_for(nn, 256), 256, 0, s>>>(n, ld, cols, A);
    identity_rows_kernel<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(n, A, flags);
    spd_part_kernel<<<grid_for(nn, 256), 256, 0, s>>>(n, A, flags, S);
    if (check_launch("dense inverse (matrix)")) return SFEM_GB300_FAILURE;
    for (ptrdiff_t k = 0; k < n; k++) {
        gj_save_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, k, S, rc);
        gj_update_kernel<<<grid_for(nn, 256), 256, 0, s>>>(n, k, S, rc, status);
    }
    if (check_launch("dense inverse (elimination)")) return SFEM_GB300_FAILURE;
    fold_couplings_kernel<T><<<(unsigned)((nn + 7) / 8), 256, 0, s>>>(n, S, A, flags, inv);
    if (check_launch("dense inverse (couplings)")) return SFEM_GB300_FAILURE;
    int bad = 0;
    if (cudaMemcpyAsync(&bad, status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return set_error("dense inverse: reading the pivot status failed");
    if (bad) return set_error("dense inverse: matrix not positive definite on its free dofs");
    return SFEM_GB300_SUCCESS;
}

}  // namespace

int dense_unit_vector(int real_type, ptrdiff_t n, ptrdiff_t j, void *e, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    if (real_type == SFEM_GB300_FLOAT32)
        unit_vector_kernel<float><<<grid_for(n, 256), 256, 0, stream_of(stream)>>>(n, j, (float *)e);
    else
        unit_vector_kernel<double><<<grid_for(n, 256), 256, 0, stream_of(stream)>>>(n, j, (double *)e);
    return check_launch("dense_unit_vector");
}

int dense_inverse(int real_type, ptrdiff_t n, ptrdiff_t ld, const void *cols, double *A, double *S, double *rc,
                  int *flags, void *inv, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    if (ld < n) return set_error("dense inverse: column stride %td below %td", ld, n);
    const cudaStream_t s = stream_of(stream);
    if (real_type == SFEM_GB300_FLOAT32)
        return dense_inverse_tpl<float>(n, ld, (const float *)cols, A, S, rc, flags, (float *)inv, s);
    return dense_inverse_tpl<double>(n, ld, (const double *)cols, A, S, rc, flags, (double *)inv, s);
}

}  // namespace sfem_gb300
