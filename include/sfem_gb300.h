/*
 * sfem_gb300 -- C ABI of the GB300-native (sm_103a) matrix-free operator path
 * for sshex8 / hex8 meshes.  Drop-in for the reference's CUDA element-kernel
 * ABI (operators/cuda/cu_laplacian.hpp, operators/cuda/cu_linear_elasticity.hpp,
 * operators/sshex8/cuda/*.cu) and its BLAS / solver seams.
 *
 * Conventions (same as the reference's CUDA ABI):
 *  - every entry point returns 0 (SFEM_GB300_SUCCESS) or 1 (SFEM_GB300_FAILURE);
 *    unsupported types or levels return FAILURE with a message available from
 *    sfem_gb300_last_error() instead of aborting;
 *  - "apply" entry points ACCUMULATE: y += A x (callers zero y first);
 *  - `elements` is a DEVICE array of device pointers (idx**, SoA,
 *    elements[v][e]); geometry is SoA with a stride (fff[d*stride + e]);
 *  - `stream` is a pointer to a cudaStream_t, or NULL for the default stream;
 *    all launches are asynchronous on that stream;
 *  - all pointers are device pointers unless stated otherwise.
 */
#ifndef SFEM_GB300_H
#define SFEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SFEM_GB300_SUCCESS 0
#define SFEM_GB300_FAILURE 1

/* Element types.  The reference passes smesh::ElemType (whose numeric values
 * live in the absent smesh submodule); a caller maps HEX8 to SFEM_GB300_HEX8
 * and a semi-structured hex8 of level L to SFEM_GB300_SSHEX8(L). */
#define SFEM_GB300_HEX8 8
#define SFEM_GB300_SSHEX8_BASE 1000
#define SFEM_GB300_SSHEX8(L) (SFEM_GB300_SSHEX8_BASE + (L))

/* Primitive types of x / y (smesh::PrimitiveType: SMESH_DEFAULT = real_t = double). */
#define SFEM_GB300_REAL_DEFAULT 0
#define SFEM_GB300_FLOAT32 1
#define SFEM_GB300_FLOAT64 2

typedef int32_t sfem_gb300_idx_t;

/* Last error message of the calling thread ("" if none). */
const char *sfem_gb300_last_error(void);

/* Library version string. */
const char *sfem_gb300_version(void);

/* ---------------------------------------------------------------- geometry */

/* Per-element FFF metric det(J) J^-1 J^-T (6 floats, SoA fff[d*fff_stride+e])
 * at the element centre from the 8 corner index arrays (hex8 order) and SoA
 * float32 points.  Replaces cu_hex8_fff_fill (operators/hex8/cuda/cu_hex8_fff.cu:179)
 * and the host FFF cache (operators/hex8/hex8_fff.cpp:5-37). */
int sfem_gb300_hex8_fff_fill(ptrdiff_t nelements, sfem_gb300_idx_t **corners, float **points, ptrdiff_t fff_stride,
                             float *fff, void *stream);

/* Per-element adjugate det(J) J^-1 (9 floats SoA adj[d*stride+e]) and
 * determinant (det[e]) at the element centre.  Replaces cu_hex8_adjugate_fill
 * (operators/hex8/cuda/cu_hex8_adjugate.cu:17). */
int sfem_gb300_hex8_adjugate_fill(ptrdiff_t nelements, sfem_gb300_idx_t **corners, float **points,
                                  ptrdiff_t jacobian_stride, float *adjugate, float *determinant, void *stream);

/* --------------------------------------------------------------- Laplacian */

/* y += A x for the affine hex8 / sshex8 Laplacian (cached float FFF).
 * Replaces cu_laplacian_apply (operators/cuda/cu_laplacian.hpp:13-21;
 * dispatch operators/cuda/cu_laplacian.cpp:21-37). */
int cu_laplacian_apply(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements, ptrdiff_t fff_stride,
                       const void *fff, int real_type_xy, const void *x, void *y, void *stream);

/* diag += diag(A).  Replaces cu_laplacian_diag (operators/cuda/cu_laplacian.hpp:23-30). */
int cu_laplacian_diag(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements, ptrdiff_t fff_stride,
                      const void *fff, int real_type_diag, void *diag, void *stream);

/* ------------------------------------------------------------ vector BLAS */
/* Device-vector kernels of the BLAS<T> seam (algebra/sfem_tpl_blas.hpp:11-35;
 * CUDA_BLAS, algebra/cuda/sfem_cuda_blas.hpp:55-77).  real_type selects
 * double (REAL_DEFAULT / FLOAT64) or float (FLOAT32) vectors; scalars are
 * passed as double. */

/* Bytes of scratch the reductions need.  The caller allocates it once, zero-fills
 * it once, and may reuse it for any number of reductions issued in stream order
 * (each reduction leaves it ready for the next).  Reductions that run
 * concurrently on different streams need separate workspaces. */
size_t sfem_gb300_reduce_workspace_size(void);

/* *result (device double) = x . y, deterministic (fixed reduction order for a given n).
 * Replaces CUDA_BLAS::dot (algebra/cuda/sfem_cuda_blas.cu:249-297). */
int sfem_gb300_dot(int real_type, ptrdiff_t n, const void *x, const void *y, void *workspace, double *result,
                   void *stream);
/* *result (device double) = ||x||_2.  Replaces CUDA_BLAS::norm2. */
int sfem_gb300_norm2(int real_type, ptrdiff_t n, const void *x, void *workspace, double *result, void *stream);
/* y = alpha x + beta y  (BLAS<T>::axpby) */
int sfem_gb300_axpby(int real_type, ptrdiff_t n, double alpha, const void *x, double beta, void *y, void *stream);
/* y += alpha x  (BLAS<T>::axpy) */
int sfem_gb300_axpy(int real_type, ptrdiff_t n, double alpha, const void *x, void *y, void *stream);
/* z = alpha x + beta y  (BLAS<T>::zaxpby) */
int sfem_gb300_zaxpby(int real_type, ptrdiff_t n, double alpha, const void *x, double beta, const void *y, void *z,
                      void *stream);
/* x *= alpha  (BLAS<T>::scal) */
int sfem_gb300_scal(int real_type, ptrdiff_t n, double alpha, void *x, void *stream);
/* x[:] = value  (BLAS<T>::values) */
int sfem_gb300_values(int real_type, ptrdiff_t n, double value, void *x, void *stream);
/* x = alpha / x where x != 0  (BLAS<T>::reciprocal) */
int sfem_gb300_reciprocal(int real_type, ptrdiff_t n, double alpha, void *x, void *stream);
/* z = x * y + alpha z  (BLAS<T>::xypaz; the Jacobi smoother step) */
int sfem_gb300_xypaz(int real_type, ptrdiff_t n, const void *x, const void *y, double alpha, void *z, void *stream);

/* Fused CG updates with device-resident scalars (no host round trip), cf. the
 * host fusion in algebra/sfem_cg.hpp:26-72:
 *   alpha = *alpha_num / *alpha_den;  x += alpha p;  r -= alpha Ap;  if rr: *rr = (r, r). */
int sfem_gb300_cg_update_x_r(int real_type, ptrdiff_t n, const double *alpha_num, const double *alpha_den,
                             const void *p, const void *Ap, void *x, void *r, void *workspace, double *rr,
                             void *stream);
/*   beta = *beta_num / *beta_den;  p = z + beta p. */
int sfem_gb300_cg_update_p(int real_type, ptrdiff_t n, const double *beta_num, const double *beta_den, const void *z,
                           void *p, void *stream);
/* Chebyshev3 step p = beta p - rhs + Ax;  x -= alpha p (algebra/sfem_Chebyshev3.hpp:36-52). */
int sfem_gb300_chebyshev_update(int real_type, ptrdiff_t n, double alpha, double beta, const void *rhs, const void *Ax,
                                void *p, void *x, void *stream);

/* Dirichlet constraints on interleaved vectors (operators/boundary_conditions/dirichlet.hpp:44-130):
 * dest[node*block+comp] = src[node*block+comp], resp. x[node*block+comp] = value. */
int sfem_gb300_constraint_nodes_copy(int real_type, ptrdiff_t n_nodes, const int32_t *nodes, int block_size,
                                     int component, const void *src, void *dest, void *stream);
int sfem_gb300_constraint_nodes_to_value(int real_type, ptrdiff_t n_nodes, const int32_t *nodes, int block_size,
                                         int component, double value, void *x, void *stream);

/* Precision conversion dst = (dst_type) src, and y += alpha (double) x for float x. */
int sfem_gb300_convert(ptrdiff_t n, int src_type, const void *src, int dst_type, void *dst, void *stream);
int sfem_gb300_axpy_f32_to_f64(ptrdiff_t n, double alpha, const float *x, double *y, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SFEM_GB300_H */
