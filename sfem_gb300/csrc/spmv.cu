// Symmetric sparse formats and their assembly from the hex8 operators.
//
//  * CRS sym  (CRSSymSpMV, algebra/sfem_crs_sym_SpMV.hpp:8-91):
//      y = scale_output * y + D x + U x + U^T x,  U = strict upper triangle in CRS.
//  * BSR sym  (BCRSSymSpMV, algebra/sfem_bcrs_sym_SpMV.hpp:9-279): block size 2 or 3,
//      diagonal blocks as their bs(bs+1)/2 upper entries; off-diagonal blocks of the
//      strict upper block triangle either full (bs*bs, row-major) or, as the
//      reference stores them, as symmetric bs(bs+1)/2 upper entries.  Values AoS.
//  * assembly of the hex8 Laplacian into CRS sym (hex8_laplacian_crs_sym,
//    operators/hex8/hex8_laplacian.cpp:148-221) and of hex8 linear elasticity into
//    BSR sym (affine_hex8_linear_elasticity_bsr / crs_sym, hex8_linear_elasticity.cpp:789-857).
//
// The row part is a gather (one thread per row, plain store); the transpose part
// scatters with atomics in a second launch, as the reference does with omp atomic.
#include "common.cuh"
#include "laplacian_kernels.cuh"

namespace sfem_gb300 {

template <typename T>
__global__ void crs_sym_rows_kernel(ptrdiff_t n, const idx_t *__restrict__ rowptr, const idx_t *__restrict__ colidx,
                                    const T *__restrict__ diag, const T *__restrict__ offdiag, T scale,
                                    const T *__restrict__ x, T *__restrict__ y) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        T acc = diag[i] * x[i];
        for (idx_t k = rowptr[i]; k < rowptr[i + 1]; k++) acc += offdiag[k] * x[colidx[k]];
        y[i] = (scale != T(0) ? scale * y[i] : T(0)) + acc;
    }
}

template <typename T>
__global__ void crs_sym_transpose_kernel(ptrdiff_t n, const idx_t *__restrict__ rowptr,
                                         const idx_t *__restrict__ colidx, const T *__restrict__ offdiag,
                                         const T *__restrict__ x, T *__restrict__ y) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        const T xi = x[i];
        for (idx_t k = rowptr[i]; k < rowptr[i + 1]; k++) atomicAdd(&y[colidx[k]], offdiag[k] * xi);
    }
}

template <typename T, int BS>
__device__ __forceinline__ void load_block(const T *v, bool sym, T B[BS][BS]) {
    if (sym) {
        int k = 0;
#pragma unroll
        for (int a = 0; a < BS; a++)
#pragma unroll
            for (int b = a; b < BS; b++, k++) {
                B[a][b] = v[k];
                B[b][a] = v[k];
            }
    } else {
#pragma unroll
        for (int a = 0; a < BS; a++)
#pragma unroll
            for (int b = 0; b < BS; b++) B[a][b] = v[a * BS + b];
    }
}

template <typename T, int BS>
__global__ void bsr_sym_rows_kernel(ptrdiff_t nb, const idx_t *__restrict__ rowptr, const idx_t *__restrict__ colidx,
                                    const T *__restrict__ diag, const T *__restrict__ offdiag, int off_sym, T scale,
                                    const T *__restrict__ x, T *__restrict__ y) {
    constexpr int NS = BS * (BS + 1) / 2;
    const int off_stride = off_sym ? NS : BS * BS;
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < nb; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        T B[BS][BS], acc[BS], xl[BS];
        load_block<T, BS>(&diag[i * NS], true, B);
#pragma unroll
        for (int b = 0; b < BS; b++) xl[b] = x[i * BS + b];
#pragma unroll
        for (int a = 0; a < BS; a++) {
            acc[a] = 0;
#pragma unroll
            for (int b = 0; b < BS; b++) acc[a] += B[a][b] * xl[b];
        }
        for (idx_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
            load_block<T, BS>(&offdiag[(ptrdiff_t)k * off_stride], off_sym, B);
            const ptrdiff_t j = colidx[k];
#pragma unroll
            for (int b = 0; b < BS; b++) xl[b] = x[j * BS + b];
#pragma unroll
            for (int a = 0; a < BS; a++)
#pragma unroll
                for (int b = 0; b < BS; b++) acc[a] += B[a][b] * xl[b];
        }
#pragma unroll
        for (int a = 0; a < BS; a++) y[i * BS + a] = (scale != T(0) ? scale * y[i * BS + a] : T(0)) + acc[a];
    }
}

template <typename T, int BS>
__global__ void bsr_sym_transpose_kernel(ptrdiff_t nb, const idx_t *__restrict__ rowptr,
                                         const idx_t *__restrict__ colidx, const T *__restrict__ offdiag, int off_sym,
                                         const T *__restrict__ x, T *__restrict__ y) {
    constexpr int NS = BS * (BS + 1) / 2;
    const int off_stride = off_sym ? NS : BS * BS;
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < nb; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        T xl[BS], B[BS][BS];
#pragma unroll
        for (int a = 0; a < BS; a++) xl[a] = x[i * BS + a];
        for (idx_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
            load_block<T, BS>(&offdiag[(ptrdiff_t)k * off_stride], off_sym, B);
            const ptrdiff_t j = colidx[k];
#pragma unroll
            for (int b = 0; b < BS; b++) {
                T s = 0;
#pragma unroll
                for (int a = 0; a < BS; a++) s += B[a][b] * xl[a];
                atomicAdd(&y[j * BS + b], s);
            }
        }
    }
}

// position of column `col` in row `row` of a sorted CRS graph, or -1
__device__ __forceinline__ idx_t find_col(const idx_t *rowptr, const idx_t *colidx, idx_t row, idx_t col) {
    idx_t lo = rowptr[row], hi = rowptr[row + 1] - 1;
    while (lo <= hi) {
        const idx_t mid = (lo + hi) >> 1;
        const idx_t c = colidx[mid];
        if (c == col) return mid;
        if (c < col)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    return -1;
}

// hex8 Laplacian -> CRS sym (diag + strict upper), one thread per element.
template <typename T>
__global__ void hex8_laplacian_crs_sym_kernel(ptrdiff_t nelements, const idx_t *const *elements, ptrdiff_t fff_stride,
                                              const float *fff, const idx_t *rowptr, const idx_t *colidx, T *diag,
                                              T *offdiag, int *missing) {
    for (ptrdiff_t e = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; e < nelements;
         e += (ptrdiff_t)gridDim.x * blockDim.x) {
        idx_t ev[8];
        T f[6];
#pragma unroll
        for (int v = 0; v < 8; v++) ev[v] = elements[v][e];
#pragma unroll
        for (int m = 0; m < 6; m++) f[m] = (T)fff[m * fff_stride + e];
        for (int i = 0; i < 8; i++) {
            for (int j = 0; j < 8; j++) {
                if (i != j && ev[j] <= ev[i]) continue;
                T a = 0;
#pragma unroll
                for (int m = 0; m < 6; m++) a += f[m] * lap_w<T>(i * 8 + j, m);
                if (i == j) {
                    atomicAdd(&diag[ev[i]], a);
                } else {
                    const idx_t k = find_col(rowptr, colidx, ev[i], ev[j]);
                    if (k < 0)
                        atomicAdd(missing, 1);
                    else
                        atomicAdd(&offdiag[k], a);
                }
            }
        }
    }
}

// hex8 Laplacian -> full CRS (every coupling, both triangles), one thread per element
// (hex8_laplacian_crs, operators/hex8/hex8_laplacian.cpp:223).
template <typename T>
__global__ void hex8_laplacian_crs_kernel(ptrdiff_t nelements, const idx_t *const *elements, ptrdiff_t fff_stride,
                                          const float *fff, const idx_t *rowptr, const idx_t *colidx, T *values,
                                          int *missing) {
    for (ptrdiff_t e = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; e < nelements;
         e += (ptrdiff_t)gridDim.x * blockDim.x) {
        idx_t ev[8];
        T f[6];
#pragma unroll
        for (int v = 0; v < 8; v++) ev[v] = elements[v][e];
#pragma unroll
        for (int m = 0; m < 6; m++) f[m] = (T)fff[m * fff_stride + e];
        for (int i = 0; i < 8; i++) {
            for (int j = 0; j < 8; j++) {
                T a = 0;
#pragma unroll
                for (int m = 0; m < 6; m++) a += f[m] * lap_w<T>(i * 8 + j, m);
                const idx_t k = find_col(rowptr, colidx, ev[i], ev[j]);
                if (k < 0)
                    atomicAdd(missing, 1);
                else
                    atomicAdd(&values[k], a);
            }
        }
    }
}

template <typename T>
static int crs_sym_spmv_tpl(ptrdiff_t n, const idx_t *rowptr, const idx_t *colidx, const void *diag,
                            const void *offdiag, double scale, const void *x, void *y, cudaStream_t s) {
    const int g = grid_for(n, 128, kNumSMs * 16);
    crs_sym_rows_kernel<T><<<g, 128, 0, s>>>(n, rowptr, colidx, (const T *)diag, (const T *)offdiag, (T)scale,
                                             (const T *)x, (T *)y);
    crs_sym_transpose_kernel<T><<<g, 128, 0, s>>>(n, rowptr, colidx, (const T *)offdiag, (const T *)x, (T *)y);
    return check_launch("sfem_gb300_crs_sym_spmv");
}

template <typename T, int BS>
static int bsr_sym_spmv_tpl(ptrdiff_t nb, const idx_t *rowptr, const idx_t *colidx, const void *diag,
                            const void *offdiag, int off_sym, double scale, const void *x, void *y, cudaStream_t s) {
    const int g = grid_for(nb, 128, kNumSMs * 16);
    bsr_sym_rows_kernel<T, BS><<<g, 128, 0, s>>>(nb, rowptr, colidx, (const T *)diag, (const T *)offdiag, off_sym,
                                                 (T)scale, (const T *)x, (T *)y);
    bsr_sym_transpose_kernel<T, BS><<<g, 128, 0, s>>>(nb, rowptr, colidx, (const T *)offdiag, off_sym, (const T *)x,
                                                      (T *)y);
    return check_launch("sfem_gb300_bsr_sym_spmv");
}

}  // namespace sfem_gb300

using namespace sfem_gb300;

extern "C" int sfem_gb300_crs_sym_spmv(int real_type, ptrdiff_t nrows, const int32_t *rowptr, const int32_t *colidx,
                                       const void *diag, const void *offdiag, double scale_output, const void *x,
                                       void *y, void *stream) {
    if (nrows <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    if (real_type == SFEM_GB300_FLOAT32)
        return crs_sym_spmv_tpl<float>(nrows, rowptr, colidx, diag, offdiag, scale_output, x, y, s);
    if (real_type == SFEM_GB300_FLOAT64 || real_type == SFEM_GB300_REAL_DEFAULT)
        return crs_sym_spmv_tpl<double>(nrows, rowptr, colidx, diag, offdiag, scale_output, x, y, s);
    return set_error("sfem_gb300_crs_sym_spmv: unsupported real type %d", real_type);
}

extern "C" int sfem_gb300_bsr_sym_spmv(int real_type, int block_size, ptrdiff_t nblock_rows, const int32_t *rowptr,
                                       const int32_t *colidx, const void *diag_sym, const void *offdiag,
                                       int offdiag_symmetric, double scale_output, const void *x, void *y,
                                       void *stream) {
    if (nblock_rows <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    const bool f32 = real_type == SFEM_GB300_FLOAT32;
    if (!f32 && real_type != SFEM_GB300_FLOAT64 && real_type != SFEM_GB300_REAL_DEFAULT)
        return set_error("sfem_gb300_bsr_sym_spmv: unsupported real type %d", real_type);
    switch (block_size) {
        case 2:
            return f32 ? bsr_sym_spmv_tpl<float, 2>(nblock_rows, rowptr, colidx, diag_sym, offdiag, offdiag_symmetric,
                                                     scale_output, x, y, s)
                       : bsr_sym_spmv_tpl<double, 2>(nblock_rows, rowptr, colidx, diag_sym, offdiag, offdiag_symmetric,
                                                      scale_output, x, y, s);
        case 3:
            return f32 ? bsr_sym_spmv_tpl<float, 3>(nblock_rows, rowptr, colidx, diag_sym, offdiag, offdiag_symmetric,
                                                     scale_output, x, y, s)
                       : bsr_sym_spmv_tpl<double, 3>(nblock_rows, rowptr, colidx, diag_sym, offdiag, offdiag_symmetric,
                                                      scale_output, x, y, s);
        default:
            return set_error("sfem_gb300_bsr_sym_spmv: block size %d not supported (2 or 3)", block_size);
    }
}

extern "C" int sfem_gb300_hex8_laplacian_crs_sym(ptrdiff_t nelements, idx_t **elements, ptrdiff_t fff_stride,
                                                 const float *fff, const int32_t *rowptr, const int32_t *colidx,
                                                 int real_type, void *diag, void *offdiag, void *stream) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    int *missing = nullptr;
    if (cudaMallocAsync((void **)&missing, sizeof(int), s) != cudaSuccess)
        return set_error("sfem_gb300_hex8_laplacian_crs_sym: allocation failed");
    cudaMemsetAsync(missing, 0, sizeof(int), s);
    const int g = grid_for(nelements, 128, kNumSMs * 16);
    if (real_type == SFEM_GB300_FLOAT32)
        hex8_laplacian_crs_sym_kernel<float><<<g, 128, 0, s>>>(nelements, elements, fff_stride, fff, rowptr, colidx,
                                                               (float *)diag, (float *)offdiag, missing);
    else
        hex8_laplacian_crs_sym_kernel<double><<<g, 128, 0, s>>>(nelements, elements, fff_stride, fff, rowptr, colidx,
                                                                (double *)diag, (double *)offdiag, missing);
    int h_missing = 0;
    cudaMemcpyAsync(&h_missing, missing, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    cudaFreeAsync(missing, s);
    if (check_launch("sfem_gb300_hex8_laplacian_crs_sym")) return SFEM_GB300_FAILURE;
    if (h_missing) return set_error("sfem_gb300_hex8_laplacian_crs_sym: %d element couplings missing from the graph", h_missing);
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_hex8_laplacian_crs(ptrdiff_t nelements, idx_t **elements, ptrdiff_t fff_stride,
                                             const float *fff, const int32_t *rowptr, const int32_t *colidx,
                                             int real_type, void *values, void *stream) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    if (real_type != SFEM_GB300_FLOAT32 && real_type != SFEM_GB300_FLOAT64 && real_type != SFEM_GB300_REAL_DEFAULT)
        return set_error("sfem_gb300_hex8_laplacian_crs: unsupported real type %d", real_type);
    const cudaStream_t s = stream_of(stream);
    int *missing = nullptr;
    if (cudaMallocAsync((void **)&missing, sizeof(int), s) != cudaSuccess)
        return set_error("sfem_gb300_hex8_laplacian_crs: allocation failed");
    cudaMemsetAsync(missing, 0, sizeof(int), s);
    const int g = grid_for(nelements, 128, kNumSMs * 16);
    if (real_type == SFEM_GB300_FLOAT32)
        hex8_laplacian_crs_kernel<float><<<g, 128, 0, s>>>(nelements, elements, fff_stride, fff, rowptr, colidx,
                                                           (float *)values, missing);
    else
        hex8_laplacian_crs_kernel<double><<<g, 128, 0, s>>>(nelements, elements, fff_stride, fff, rowptr, colidx,
                                                            (double *)values, missing);
    const int lerr = check_launch("sfem_gb300_hex8_laplacian_crs");
    int h_missing = 0;
    cudaMemcpyAsync(&h_missing, missing, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    cudaFreeAsync(missing, s);
    if (lerr) return SFEM_GB300_FAILURE;
    if (h_missing) return set_error("sfem_gb300_hex8_laplacian_crs: %d element couplings missing from the graph", h_missing);
    return SFEM_GB300_SUCCESS;
}
