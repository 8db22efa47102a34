// Vector kernels of the solver path (BLAS<T> seam, algebra/sfem_tpl_blas.hpp:11-35)
// plus fused CG / Chebyshev updates and Dirichlet constraint kernels.
//
// Reductions are deterministic: a fixed grid (a function of n only), one
// double partial per block, and the last block to finish sums the partials in
// block order.  The caller provides the scratch (sfem_gb300_reduce_workspace_size
// bytes); the reference instead cudaMallocs and frees a result buffer on every
// dot (algebra/cuda/sfem_cuda_blas.cu:280-297).
#include "blas.cuh"
#include "common.cuh"

namespace sfem_gb300 {

// ------------------------------------------------------------------ reductions

int reduce_grid(ptrdiff_t n) {
    ptrdiff_t g = (n + kReduceBlock * 4 - 1) / (kReduceBlock * 4);
    if (g < 1) g = 1;
    if (g > kReduceMaxBlocks) g = kReduceMaxBlocks;
    return (int)g;
}

template <typename T>
__global__ void __launch_bounds__(kReduceBlock) dot_kernel(ptrdiff_t n, const T *__restrict__ x,
                                                           const T *__restrict__ y, ReduceWorkspace ws,
                                                           double *result, int do_sqrt) {
    T acc = 0;
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)kReduceBlock + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * kReduceBlock)
        acc += x[i] * y[i];
    reduce_epilogue((double)acc, ws, result, do_sqrt);
}

// ------------------------------------------------------------------ elementwise

template <typename T>
__global__ void axpby_kernel(ptrdiff_t n, T alpha, const T *__restrict__ x, T beta, T *__restrict__ y) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        y[i] = alpha * x[i] + beta * y[i];
}

template <typename T>
__global__ void zaxpby_kernel(ptrdiff_t n, T alpha, const T *__restrict__ x, T beta, const T *__restrict__ y,
                              T *__restrict__ z) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        z[i] = alpha * x[i] + beta * y[i];
}

template <typename T>
__global__ void scal_kernel(ptrdiff_t n, T alpha, T *__restrict__ x) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        x[i] *= alpha;
}

template <typename T>
__global__ void values_kernel(ptrdiff_t n, T v, T *__restrict__ x) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        x[i] = v;
}

template <typename T>
__global__ void reciprocal_kernel(ptrdiff_t n, T alpha, T *__restrict__ x) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        const T v = x[i];
        if (v != T(0)) x[i] = alpha / v;
    }
}

template <typename T>
__global__ void xypaz_kernel(ptrdiff_t n, const T *__restrict__ x, const T *__restrict__ y, T alpha, T *__restrict__ z) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        z[i] = x[i] * y[i] + alpha * z[i];
}

// ------------------------------------------------------------------ fused solver updates

// alpha = scal[ia] / scal[ib] (device scalars);  x += alpha p;  r -= alpha Ap;  optionally rr = (r, r)
template <typename T>
__global__ void __launch_bounds__(kReduceBlock) cg_update_x_r_kernel(ptrdiff_t n, const double *__restrict__ num,
                                                                     const double *__restrict__ den,
                                                                     const T *__restrict__ p, const T *__restrict__ Ap,
                                                                     T *__restrict__ x, T *__restrict__ r,
                                                                     ReduceWorkspace ws, double *rr) {
    const T alpha = (T)(*num / *den);
    T acc = 0;
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)kReduceBlock + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * kReduceBlock) {
        x[i] += alpha * p[i];
        const T ri = r[i] - alpha * Ap[i];
        r[i] = ri;
        acc += ri * ri;
    }
    if (rr) reduce_epilogue((double)acc, ws, rr, 0);
}

// beta = (num - sub) / den ;  p = z + beta p   (sub may be NULL)
template <typename T>
__global__ void cg_update_p_kernel(ptrdiff_t n, const double *__restrict__ num, const double *__restrict__ den,
                                   const double *__restrict__ sub, const T *__restrict__ z, T *__restrict__ p) {
    const T beta = (T)((*num - (sub ? *sub : 0.0)) / *den);
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        p[i] = z[i] + beta * p[i];
}

// Chebyshev3 step (algebra/sfem_Chebyshev3.hpp:36-52): p = beta p - rhs + Ax ; x -= alpha p.
// With inv_diag the step runs on D^-1 A: p = beta p + D^-1 (Ax - rhs).  beta == 0 ignores the old p.
template <typename T>
__global__ void cheb_update_kernel(ptrdiff_t n, T alpha, T beta, const T *__restrict__ inv_diag,
                                   const T *__restrict__ rhs, const T *__restrict__ Ax, T *__restrict__ p,
                                   T *__restrict__ x) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        T g = Ax[i] - rhs[i];
        if (inv_diag) g *= inv_diag[i];
        const T pi = (beta != T(0) ? beta * p[i] : T(0)) + g;
        p[i] = pi;
        x[i] -= alpha * pi;
    }
}

// ------------------------------------------------------------------ constraints

// dest[node*block + comp] = src[node*block + comp] for the constrained nodes
// (constraint_nodes_copy_vec, operators/boundary_conditions/dirichlet.hpp:124)
template <typename T>
__global__ void constraint_copy_kernel(ptrdiff_t nn, const idx_t *__restrict__ nodes, int block, int comp,
                                       const T *__restrict__ src, T *__restrict__ dst) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < nn; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t k = (ptrdiff_t)nodes[i] * block + comp;
        dst[k] = src[k];
    }
}

// every component of the constrained nodes in one launch: dst[node*block + c] = src[...], c < block
template <typename T>
__global__ void constraint_copy_block_kernel(ptrdiff_t nn, const idx_t *__restrict__ nodes, int block,
                                             const T *__restrict__ src, T *__restrict__ dst) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < nn * block;
         i += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t k = (ptrdiff_t)nodes[i / block] * block + i % block;
        dst[k] = src[k];
    }
}

template <typename T>
__global__ void constraint_value_block_kernel(ptrdiff_t nn, const idx_t *__restrict__ nodes, int block, T value,
                                              T *__restrict__ x) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < nn * block;
         i += (ptrdiff_t)gridDim.x * blockDim.x)
        x[(ptrdiff_t)nodes[i / block] * block + i % block] = value;
}

template <typename T>
__global__ void constraint_value_kernel(ptrdiff_t nn, const idx_t *__restrict__ nodes, int block, int comp, T value,
                                        T *__restrict__ x) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < nn; i += (ptrdiff_t)gridDim.x * blockDim.x)
        x[(ptrdiff_t)nodes[i] * block + comp] = value;
}

// ------------------------------------------------------------------ seeded uniform values

// x[i] = U(-1, 1) from a counter-based hash (splitmix64) of (seed, i): reproducible for any launch shape.
template <typename T>
__global__ void random_uniform_kernel(ptrdiff_t n, unsigned long long seed, T *__restrict__ x) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z = z ^ (z >> 31);
        x[i] = (T)((double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0);
    }
}

// ------------------------------------------------------------------ precision conversion

template <typename S, typename D>
__global__ void convert_kernel(ptrdiff_t n, const S *__restrict__ src, D *__restrict__ dst) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        dst[i] = (D)src[i];
}

// y += alpha * (double) x   (x float)
__global__ void axpy_f32_to_f64_kernel(ptrdiff_t n, double alpha, const float *__restrict__ x, double *__restrict__ y) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        y[i] += alpha * (double)x[i];
}

// dst = (float)(src / *nrm)  (device-resident scale; 0 if *nrm == 0)
__global__ void scaled_to_f32_kernel(ptrdiff_t n, const double *__restrict__ nrm, const double *__restrict__ src,
                                     float *__restrict__ dst) {
    const double s = *nrm > 0 ? 1.0 / *nrm : 0.0;
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        dst[i] = (float)(src[i] * s);
}

// y += *nrm * (double) x
__global__ void scaled_axpy_f32_to_f64_kernel(ptrdiff_t n, const double *__restrict__ nrm, const float *__restrict__ x,
                                              double *__restrict__ y) {
    const double s = *nrm;
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x)
        y[i] += s * (double)x[i];
}

// x += M b, M dense row-major n x n: one warp per row
template <typename T>
__global__ void dense_mv_add_kernel(ptrdiff_t n, const T *__restrict__ M, const T *__restrict__ b, T *__restrict__ x) {
    const ptrdiff_t row = (ptrdiff_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    T acc = 0;
    for (ptrdiff_t j = lane; j < n; j += 32) acc += M[row * n + j] * b[j];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) x[row] += acc;
}

// ------------------------------------------------------------------ host helpers

static inline int ew_grid(ptrdiff_t n) { return grid_for(n, 256, kNumSMs * 16); }

template <typename T>
int dot_tpl(ptrdiff_t n, const void *x, const void *y, void *workspace, double *result, int do_sqrt, cudaStream_t s) {
    if (!workspace) return set_error("sfem_gb300_dot: workspace is NULL");
    ReduceWorkspace ws = workspace_of(workspace);
    dot_kernel<T><<<reduce_grid(n), kReduceBlock, 0, s>>>(n, (const T *)x, (const T *)y, ws, result, do_sqrt);
    return check_launch("sfem_gb300_dot");
}

}  // namespace sfem_gb300

using namespace sfem_gb300;

#define SFEM_DISPATCH_REAL(rt, what, CALL_F64, CALL_F32)                     \
    switch (rt) {                                                            \
        case SFEM_GB300_REAL_DEFAULT:                                        \
        case SFEM_GB300_FLOAT64: {                                           \
            typedef double T;                                                \
            CALL_F64;                                                        \
            break;                                                           \
        }                                                                    \
        case SFEM_GB300_FLOAT32: {                                           \
            typedef float T;                                                 \
            CALL_F32;                                                        \
            break;                                                           \
        }                                                                    \
        default:                                                             \
            return set_error("%s: unsupported real type %d", what, (int)rt); \
    }

extern "C" size_t sfem_gb300_reduce_workspace_size(void) { return kReduceWorkspaceBytes; }

extern "C" int sfem_gb300_dot(int real_type, ptrdiff_t n, const void *x, const void *y, void *workspace,
                              double *result, void *stream) {
    const cudaStream_t s = stream_of(stream);
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_dot", return dot_tpl<T>(n, x, y, workspace, result, 0, s),
                       return dot_tpl<T>(n, x, y, workspace, result, 0, s));
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_norm2(int real_type, ptrdiff_t n, const void *x, void *workspace, double *result,
                                void *stream) {
    const cudaStream_t s = stream_of(stream);
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_norm2", return dot_tpl<T>(n, x, x, workspace, result, 1, s),
                       return dot_tpl<T>(n, x, x, workspace, result, 1, s));
    return SFEM_GB300_SUCCESS;
}

#define SFEM_EW_LAUNCH(kernel, ...) \
    kernel<T><<<ew_grid(n), 256, 0, stream_of(stream)>>>(__VA_ARGS__)

extern "C" int sfem_gb300_axpby(int real_type, ptrdiff_t n, double alpha, const void *x, double beta, void *y,
                                void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_axpby", SFEM_EW_LAUNCH(axpby_kernel, n, (T)alpha, (const T *)x, (T)beta, (T *)y),
                       SFEM_EW_LAUNCH(axpby_kernel, n, (T)alpha, (const T *)x, (T)beta, (T *)y));
    return check_launch("sfem_gb300_axpby");
}

extern "C" int sfem_gb300_axpy(int real_type, ptrdiff_t n, double alpha, const void *x, void *y, void *stream) {
    return sfem_gb300_axpby(real_type, n, alpha, x, 1.0, y, stream);
}

extern "C" int sfem_gb300_zaxpby(int real_type, ptrdiff_t n, double alpha, const void *x, double beta, const void *y,
                                 void *z, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_zaxpby",
                       SFEM_EW_LAUNCH(zaxpby_kernel, n, (T)alpha, (const T *)x, (T)beta, (const T *)y, (T *)z),
                       SFEM_EW_LAUNCH(zaxpby_kernel, n, (T)alpha, (const T *)x, (T)beta, (const T *)y, (T *)z));
    return check_launch("sfem_gb300_zaxpby");
}

extern "C" int sfem_gb300_scal(int real_type, ptrdiff_t n, double alpha, void *x, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_scal", SFEM_EW_LAUNCH(scal_kernel, n, (T)alpha, (T *)x),
                       SFEM_EW_LAUNCH(scal_kernel, n, (T)alpha, (T *)x));
    return check_launch("sfem_gb300_scal");
}

extern "C" int sfem_gb300_values(int real_type, ptrdiff_t n, double value, void *x, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_values", SFEM_EW_LAUNCH(values_kernel, n, (T)value, (T *)x),
                       SFEM_EW_LAUNCH(values_kernel, n, (T)value, (T *)x));
    return check_launch("sfem_gb300_values");
}

extern "C" int sfem_gb300_reciprocal(int real_type, ptrdiff_t n, double alpha, void *x, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_reciprocal", SFEM_EW_LAUNCH(reciprocal_kernel, n, (T)alpha, (T *)x),
                       SFEM_EW_LAUNCH(reciprocal_kernel, n, (T)alpha, (T *)x));
    return check_launch("sfem_gb300_reciprocal");
}

extern "C" int sfem_gb300_xypaz(int real_type, ptrdiff_t n, const void *x, const void *y, double alpha, void *z,
                                void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_xypaz",
                       SFEM_EW_LAUNCH(xypaz_kernel, n, (const T *)x, (const T *)y, (T)alpha, (T *)z),
                       SFEM_EW_LAUNCH(xypaz_kernel, n, (const T *)x, (const T *)y, (T)alpha, (T *)z));
    return check_launch("sfem_gb300_xypaz");
}

extern "C" int sfem_gb300_cg_update_x_r(int real_type, ptrdiff_t n, const double *alpha_num, const double *alpha_den,
                                        const void *p, const void *Ap, void *x, void *r, void *workspace, double *rr,
                                        void *stream) {
    if (rr && !workspace) return set_error("sfem_gb300_cg_update_x_r: workspace is NULL");
    ReduceWorkspace ws = workspace ? workspace_of(workspace) : ReduceWorkspace{nullptr, nullptr};
    const cudaStream_t s = stream_of(stream);
    const int grid = reduce_grid(n);
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_cg_update_x_r",
                       (cg_update_x_r_kernel<T><<<grid, kReduceBlock, 0, s>>>(n, alpha_num, alpha_den, (const T *)p,
                                                                              (const T *)Ap, (T *)x, (T *)r, ws, rr)),
                       (cg_update_x_r_kernel<T><<<grid, kReduceBlock, 0, s>>>(n, alpha_num, alpha_den, (const T *)p,
                                                                              (const T *)Ap, (T *)x, (T *)r, ws, rr)));
    return check_launch("sfem_gb300_cg_update_x_r");
}

extern "C" int sfem_gb300_cg_update_p(int real_type, ptrdiff_t n, const double *beta_num, const double *beta_den,
                                      const double *beta_sub, const void *z, void *p, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_cg_update_p",
                       SFEM_EW_LAUNCH(cg_update_p_kernel, n, beta_num, beta_den, beta_sub, (const T *)z, (T *)p),
                       SFEM_EW_LAUNCH(cg_update_p_kernel, n, beta_num, beta_den, beta_sub, (const T *)z, (T *)p));
    return check_launch("sfem_gb300_cg_update_p");
}

extern "C" int sfem_gb300_chebyshev_update(int real_type, ptrdiff_t n, double alpha, double beta, const void *inv_diag,
                                           const void *rhs, const void *Ax, void *p, void *x, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_chebyshev_update",
                       SFEM_EW_LAUNCH(cheb_update_kernel, n, (T)alpha, (T)beta, (const T *)inv_diag, (const T *)rhs,
                                      (const T *)Ax, (T *)p, (T *)x),
                       SFEM_EW_LAUNCH(cheb_update_kernel, n, (T)alpha, (T)beta, (const T *)inv_diag, (const T *)rhs,
                                      (const T *)Ax, (T *)p, (T *)x));
    return check_launch("sfem_gb300_chebyshev_update");
}

extern "C" int sfem_gb300_constraint_nodes_copy(int real_type, ptrdiff_t n_nodes, const int32_t *nodes, int block_size,
                                                int component, const void *src, void *dest, void *stream) {
    const ptrdiff_t n = n_nodes;
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_constraint_nodes_copy",
                       SFEM_EW_LAUNCH(constraint_copy_kernel, n, nodes, block_size, component, (const T *)src, (T *)dest),
                       SFEM_EW_LAUNCH(constraint_copy_kernel, n, nodes, block_size, component, (const T *)src, (T *)dest));
    return check_launch("sfem_gb300_constraint_nodes_copy");
}

extern "C" int sfem_gb300_constraint_nodes_to_value(int real_type, ptrdiff_t n_nodes, const int32_t *nodes,
                                                    int block_size, int component, double value, void *x,
                                                    void *stream) {
    const ptrdiff_t n = n_nodes;
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_constraint_nodes_to_value",
                       SFEM_EW_LAUNCH(constraint_value_kernel, n, nodes, block_size, component, (T)value, (T *)x),
                       SFEM_EW_LAUNCH(constraint_value_kernel, n, nodes, block_size, component, (T)value, (T *)x));
    return check_launch("sfem_gb300_constraint_nodes_to_value");
}

namespace sfem_gb300 {
int constraint_copy_block(int real_type, ptrdiff_t n_nodes, const int32_t *nodes, int block_size, const void *src,
                          void *dest, void *stream) {
    const ptrdiff_t n = n_nodes * block_size;
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "constraint_copy_block",
                       SFEM_EW_LAUNCH(constraint_copy_block_kernel, n_nodes, nodes, block_size, (const T *)src,
                                      (T *)dest),
                       SFEM_EW_LAUNCH(constraint_copy_block_kernel, n_nodes, nodes, block_size, (const T *)src,
                                      (T *)dest));
    return check_launch("constraint_copy_block");
}

int constraint_value_block(int real_type, ptrdiff_t n_nodes, const int32_t *nodes, int block_size, double value,
                           void *x, void *stream) {
    const ptrdiff_t n = n_nodes * block_size;
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "constraint_value_block",
                       SFEM_EW_LAUNCH(constraint_value_block_kernel, n_nodes, nodes, block_size, (T)value, (T *)x),
                       SFEM_EW_LAUNCH(constraint_value_block_kernel, n_nodes, nodes, block_size, (T)value, (T *)x));
    return check_launch("constraint_value_block");
}
}  // namespace sfem_gb300

extern "C" int sfem_gb300_convert(ptrdiff_t n, int src_type, const void *src, int dst_type, void *dst, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    const bool s64 = src_type != SFEM_GB300_FLOAT32, d64 = dst_type != SFEM_GB300_FLOAT32;
    if (s64 && !d64)
        convert_kernel<double, float><<<ew_grid(n), 256, 0, s>>>(n, (const double *)src, (float *)dst);
    else if (!s64 && d64)
        convert_kernel<float, double><<<ew_grid(n), 256, 0, s>>>(n, (const float *)src, (double *)dst);
    else if (s64)
        convert_kernel<double, double><<<ew_grid(n), 256, 0, s>>>(n, (const double *)src, (double *)dst);
    else
        convert_kernel<float, float><<<ew_grid(n), 256, 0, s>>>(n, (const float *)src, (float *)dst);
    return check_launch("sfem_gb300_convert");
}

extern "C" int sfem_gb300_random_uniform(int real_type, ptrdiff_t n, unsigned long long seed, void *x, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    SFEM_DISPATCH_REAL(real_type, "sfem_gb300_random_uniform",
                       SFEM_EW_LAUNCH(random_uniform_kernel, n, seed, (T *)x),
                       SFEM_EW_LAUNCH(random_uniform_kernel, n, seed, (T *)x));
    return check_launch("sfem_gb300_random_uniform");
}

extern "C" int sfem_gb300_axpy_f32_to_f64(ptrdiff_t n, double alpha, const float *x, double *y, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    axpy_f32_to_f64_kernel<<<ew_grid(n), 256, 0, stream_of(stream)>>>(n, alpha, x, y);
    return check_launch("sfem_gb300_axpy_f32_to_f64");
}

extern "C" int sfem_gb300_scaled_to_f32(ptrdiff_t n, const double *nrm, const double *src, float *dst, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    scaled_to_f32_kernel<<<ew_grid(n), 256, 0, stream_of(stream)>>>(n, nrm, src, dst);
    return check_launch("sfem_gb300_scaled_to_f32");
}

extern "C" int sfem_gb300_scaled_axpy_f32_to_f64(ptrdiff_t n, const double *nrm, const float *x, double *y,
                                                 void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    scaled_axpy_f32_to_f64_kernel<<<ew_grid(n), 256, 0, stream_of(stream)>>>(n, nrm, x, y);
    return check_launch("sfem_gb300_scaled_axpy_f32_to_f64");
}

namespace sfem_gb300 {
int dense_symv_add(int real_type, ptrdiff_t n, const void *M, const void *b, void *x, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    const int blocks = (int)((n + 7) / 8);
    if (real_type == SFEM_GB300_FLOAT32)
        dense_mv_add_kernel<float><<<blocks, 256, 0, stream_of(stream)>>>(n, (const float *)M, (const float *)b,
                                                                           (float *)x);
    else
        dense_mv_add_kernel<double><<<blocks, 256, 0, stream_of(stream)>>>(n, (const double *)M, (const double *)b,
                                                                            (double *)x);
    return check_launch("dense_symv_add");
}
}  // namespace sfem_gb300
