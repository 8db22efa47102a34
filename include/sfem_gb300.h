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
/* float vectors with the element contraction on the tensor cores in BF16
 * (FP32 accumulate); accepted by the linear-elasticity apply only.  Entry
 * error is about 1e-2 of |K||u|: for smoothers inside a multigrid
 * preconditioner, not for the operator of a Krylov method. */
#define SFEM_GB300_FLOAT32_BF16TC 3

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

/* Kernel used for float sshex8 applies (process-wide tuning knob, no reference
 * counterpart): -1 per-level default, 0 shared-memory staged tile, 1 warp per
 * element, 2 thread per element in registers, 3 cp.async staged tile with two
 * threads per element, 4 persistent cp.async pipeline with one warp per micro
 * layer (3 and 4: even L; other levels use the staged tile), 8 node-centric
 * stencil form (L = 2, 3, 4; the default at L = 3, 4 and in FP64 at L = 2).
 * Returns the previous setting (-1 if none was forced). */
int sfem_gb300_set_laplacian_kernel(int variant);

/* Non-affine sshex8 Laplacian, y += A x (replaces sshex8_laplacian_apply,
 * operators/sshex8/sshex8_laplacian.cpp:39-182, on the GPU): macro elements with the
 * trilinear geometry of their 8 corner nodes (points_x/y/z: device float arrays, the
 * reference's SoA geom_t** points), every micro element integrated with the six-point
 * face-centre rule at the FFF of the macro map.  element_type SSHEX8(L), 1 <= L <= 16;
 * FP32 or FP64 x / y; a correctness path (one CTA per macro element), not tuned. */
int sfem_gb300_sshex8_laplacian_apply_nonaffine(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                                                const float *points_x, const float *points_y, const float *points_z,
                                                int real_type_xy, const void *x, void *y, void *stream);

/* Packed tiles (no reference counterpart; an operator-creation step like the
 * reference's FFF cache): the connectivity and FFF of sshex8 L = 3 or 4 repacked
 * into one contiguous block per 32 consecutive macro elements ([(L+1)^3][el] int32
 * node ids, then [6][el] FFF floats; elements past the end: node 0, FFF 0) so an
 * apply fetches a tile's ids and metric with one bulk copy.
 * sfem_gb300_sshex8_packed_bytes gives the block array's size (-1: unsupported
 * type), sfem_gb300_sshex8_pack fills it (16-byte aligned),
 * sfem_gb300_sshex8_laplacian_apply_packed computes y += A x from it (FP32 and
 * FP64 x / y: the node-centric stencil kernel; FP32 at L = 4 with another kernel
 * variant forced: the element-matrix kernel); the result equals cu_laplacian_apply's on the same
 * connectivity and FFF up to rounding order.  sfem_gb300_laplacian_status returns
 * (and clears) 1 if a packed apply gave up waiting for its bulk copy (2 if the
 * drain after that gave up too), else 0.
 * sfem_gb300_set_tile_wait_polls (test knob, no reference counterpart) bounds the
 * FIRST wait of every tile on its bulk copy (0: give up without polling; < 0: the
 * default bound) so a test can make it give up; the drain wait that follows keeps
 * its long bound, so no copy is left in flight when the CTA exits.  Returns the
 * previous bound. */
/* Stored element matrices (the reference's "ss:em" Laplacian,
 * frontend/ops/sfem_SemiStructuredEMLaplacian.cpp:77-117: sshex8_laplacian_element_matrix,
 * operators/sshex8/sshex8_laplacian.cpp:595-634, + sshex8_stencil_element_matrix_apply):
 * em[e * 64 + i * 8 + j] = the micro element matrix of macro element e (FFF / L, hex8
 * corner order) in real_type, and y += A x from them (any sshex8 level 1..16). */
int sfem_gb300_sshex8_laplacian_element_matrix(int element_type, ptrdiff_t nelements, ptrdiff_t fff_stride,
                                               const float *fff, int real_type, void *em, void *stream);
int sfem_gb300_sshex8_laplacian_apply_em(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                                         const void *em, int real_type, const void *x, void *y, void *stream);

ptrdiff_t sfem_gb300_sshex8_packed_bytes(int element_type, ptrdiff_t nelements);
int sfem_gb300_sshex8_pack(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements, ptrdiff_t fff_stride,
                           const float *fff, void *packed, void *stream);
int sfem_gb300_sshex8_laplacian_apply_packed(int element_type, ptrdiff_t nelements, const void *packed,
                                             int real_type_xy, const void *x, void *y, void *stream);
int sfem_gb300_laplacian_status(void);
int sfem_gb300_set_tile_wait_polls(int polls);

/* Compensated residual (no reference counterpart; the reference evaluates residuals
 * in the working precision, drivers/mgsolve.cpp:315): r = b - A x for the FP64
 * operator given by its stored micro element matrices (row-major (8 bs) x (8 bs) per
 * macro element, row / column = component * 8 + corner: the layout of
 * sfem_gb300_sshex8_laplacian_element_matrix and
 * sfem_gb300_linear_elasticity_element_matrices), block_size 1 or 3 (interleaved
 * components), with every product and sum of A x carried in double-double and the
 * scatter to shared nodes kept error-free, then rounded to double; constrained rows
 * get b - x.  x may be an unevaluated sum x + x_lo (x_lo NULL: zero), so a solution
 * kept in double-double is judged exactly.  `work` holds 2 n_dofs doubles.  Certifies
 * residuals far below the plain FP64 evaluation floor (about 1e-16 of (|A||x|)_i per
 * entry).  sfem_gb300_dd_axpy: (x_hi, x_lo) += alpha e with an error-free sum. */
int sfem_gb300_residual_dd(int element_type, int block_size, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                           const double *element_matrices, ptrdiff_t n_dofs, const double *x, const double *x_lo,
                           const double *b, ptrdiff_t n_dirichlet, const int32_t *dirichlet, double *work, double *r,
                           void *stream);
int sfem_gb300_dd_axpy(ptrdiff_t n, double alpha, const double *e, double *x_hi, double *x_lo, void *stream);

/* ------------------------------------------------------- linear elasticity */

/* out += K u for the affine hex8 / sshex8 linear-elasticity operator with
 * interleaved vectors (u[3*node + d]) and SoA float adjugate (9 x stride) /
 * determinant (stride).  Replaces cu_linear_elasticity_apply
 * (operators/cuda/cu_linear_elasticity.hpp:15) / cu_affine_hex8_linear_elasticity_apply
 * (operators/hex8/cuda/cu_hex8_linear_elasticity.cu:181). */
int sfem_gb300_linear_elasticity_apply(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                                       ptrdiff_t jacobian_stride, const float *adjugate, const float *determinant,
                                       double mu, double lambda, int real_type, const void *u, void *out,
                                       void *stream);

/* Stored element matrices (no reference counterpart; the reference rebuilds them per apply):
 * K[e] (24 x 24 row-major, row/column = component * 8 + corner, real_type) of every macro
 * element from the level's sub-adjugate, and out += K u with them.  Used on coarse levels
 * (hex8, L <= 2), where building the matrix costs more than applying it. */
int sfem_gb300_linear_elasticity_element_matrices(int element_type, ptrdiff_t nelements, ptrdiff_t jacobian_stride,
                                                  const float *adjugate, const float *determinant, double mu,
                                                  double lambda, int real_type, void *K, void *stream);
int sfem_gb300_linear_elasticity_apply_em(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                                          const void *K, int real_type, const void *u, void *out, void *stream);

/* FP32 sshex8 kernel choice (no reference counterpart): -1 default, 0 the SIMT warp
 * kernel, 1 the tcgen05 kernel (L = 4: element-matrix contraction on the tensor cores in
 * 3xTF32, FP32-level accuracy; the default at L = 4).  sfem_gb300_elasticity_status
 * returns (and clears) 1 if a tcgen05 kernel gave up waiting for its MMAs, else 0. */
int sfem_gb300_set_elasticity_kernel(int variant);
int sfem_gb300_elasticity_status(void);

/* The reference's linear-elasticity entry points under its names and argument order
 * (operators/cuda/cu_linear_elasticity.hpp:15-60): interleaved xyz vectors, SoA float
 * adjugate (9 x jacobian_stride) and determinant.
 *  - cu_linear_elasticity_apply: y += K x, HEX8 or SSHEX8(L) (:15-26);
 *  - cu_linear_elasticity_diag: diag += diag(K) (3 per node, :28-38);
 *  - cu_linear_elasticity_block_diag_sym_aos: out += the symmetric 3 x 3 node blocks
 *    (6 per node: 00, 01, 02, 11, 12, 22, :55-65);
 *  - cu_linear_elasticity_bsr: values += K on a block sparse row pattern with 3 x 3
 *    row-major blocks (HEX8, as the reference, :41-53; fails if an element node pair is
 *    missing from the pattern). */
int cu_linear_elasticity_apply(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                               ptrdiff_t jacobian_stride, const void *jacobian_adjugate,
                               const void *jacobian_determinant, double mu, double lambda, int real_type,
                               const void *x, void *y, void *stream);
int cu_linear_elasticity_diag(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                              ptrdiff_t jacobian_stride, const void *jacobian_adjugate,
                              const void *jacobian_determinant, double mu, double lambda, int real_type, void *diag,
                              void *stream);
int cu_linear_elasticity_block_diag_sym_aos(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                                            ptrdiff_t jacobian_stride, const void *jacobian_adjugate,
                                            const void *jacobian_determinant, double mu, double lambda,
                                            int real_type, void *out, void *stream);
int cu_linear_elasticity_bsr(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                             ptrdiff_t jacobian_stride, const void *jacobian_adjugate, const void *jacobian_determinant,
                             double mu, double lambda, int real_type, const int32_t *rowptr, const int32_t *colidx,
                             void *values, void *stream);

/* The reference's exact sshex8 entry point (operators/sshex8/cuda/cu_sshex8_linear_elasticity.cu:1730-1748):
 * component d of node g at u{x,y,z}[g * u_stride] and out{x,y,z}[g * out_stride].  The
 * interleaved layout (stride 3, uy = ux + 1, uz = ux + 2) runs the tuned kernels; any
 * other (separate arrays, padded strides) the CTA-per-macro-element kernel, L = 1..16. */
int cu_affine_sshex8_linear_elasticity_apply(int level, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                                             ptrdiff_t jacobian_stride, const void *jacobian_adjugate,
                                             const void *jacobian_determinant, double mu, double lambda,
                                             int real_type, ptrdiff_t u_stride, const void *ux, const void *uy,
                                             const void *uz, ptrdiff_t out_stride, void *outx, void *outy, void *outz,
                                             void *stream);

/* diag3 += diagonal (3 per node) and/or block6 += symmetric 3x3 block diagonal
 * (00,01,02,11,12,22 per node); either may be NULL.  Replaces
 * cu_affine_sshex8_linear_elasticity_diag / _block_diag_sym
 * (operators/sshex8/cuda/cu_sshex8_linear_elasticity.cu:1938, :2171). */
int sfem_gb300_linear_elasticity_block_diag(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                                            ptrdiff_t jacobian_stride, const float *adjugate, const float *determinant,
                                            double mu, double lambda, int real_type, void *diag3, void *block6,
                                            void *stream);

/* block6 <- omega * inverse(block6) per node; Dirichlet nodes become identity
 * (algebra/cuda/sfem_cuda_ShiftableJacobi.cu:14-100). */
int sfem_gb300_block3_invert(int real_type, ptrdiff_t n_nodes, void *block6, double omega, ptrdiff_t n_dirichlet,
                             const int32_t *dirichlet_nodes, void *stream);
/* x += B r per node with symmetric 3x3 blocks B (block Jacobi step). */
int sfem_gb300_block3_apply(int real_type, ptrdiff_t n_nodes, const void *block6, const void *r, void *x, void *stream);

/* ------------------------------------------------------ multigrid transfer */

/* to = P from: nested trilinear prolongation inside each macro element from
 * level from_level to to_level (to_level % from_level == 0), vec_size
 * interleaved components.  Both connectivities are in sshex8 lidx order (for
 * level 1 pass the macro corners in lidx order).  Output overwritten.
 * Replaces sshex8_prolongate / sshex8_hierarchical_prolongation
 * (operators/sshex8/sshex8_interpolate.cpp:259, :129) and smesh's device path. */
int sfem_gb300_sshex8_prolongate(ptrdiff_t nelements, int from_level, sfem_gb300_idx_t **from_elements, int to_level,
                                 sfem_gb300_idx_t **to_elements, int vec_size, int real_type, const void *from,
                                 void *to, void *stream);

/* to += R from with R = P^T and the fine input divided by the element-node
 * incidence count.  Replaces sshex8_restrict / sshex8_hierarchical_restriction
 * (operators/sshex8/sshex8_interpolate.cpp:633, :12). */
int sfem_gb300_sshex8_restrict(ptrdiff_t nelements, int from_level, sfem_gb300_idx_t **from_elements,
                               const uint16_t *from_element_to_node_incidence_count, int to_level,
                               sfem_gb300_idx_t **to_elements, int vec_size, int real_type, const void *from, void *to,
                               void *stream);

/* y[vec*i + c] = sum_k weights[k] x[vec*colidx[k] + c] over the CSR row i (overwrites y):
 * nested interpolation between plain hex8 grids below the macro mesh, or its transpose.
 * No reference counterpart (the reference's hierarchy ends at the macro mesh). */
int sfem_gb300_crs_transfer(int real_type, ptrdiff_t nrows, int vec_size, const sfem_gb300_idx_t *rowptr,
                            const sfem_gb300_idx_t *colidx, const double *weights, const void *x, void *y,
                            void *stream);

/* count[node] += number of macro elements containing the node (count zeroed by the caller).
 * Replaces sshex8_element_node_incidence_count (operators/sshex8/sshex8_interpolate.cpp:239). */
int sfem_gb300_sshex8_element_node_incidence_count(int level, ptrdiff_t nelements, sfem_gb300_idx_t **elements,
                                                   uint16_t *count, void *stream);

/* ------------------------------------------------- symmetric sparse formats */

/* y = scale_output * y + (D + U + U^T) x for a symmetric matrix stored as its
 * diagonal and strict upper triangle U in CRS (sorted columns > row).
 * Replaces CRSSymSpMV (algebra/sfem_crs_sym_SpMV.hpp:8-91) and the cuSPARSE
 * two-pass COO path (algebra/cuda/sfem_cuda_crs_SpMV.cpp:190-330). */
int sfem_gb300_crs_sym_spmv(int real_type, ptrdiff_t nrows, const int32_t *rowptr, const int32_t *colidx,
                            const void *diag, const void *offdiag, double scale_output, const void *x, void *y,
                            void *stream);

/* Block version, block_size 2 or 3: diagonal blocks as bs(bs+1)/2 upper entries
 * per block row (AoS); strict-upper off-diagonal blocks full bs*bs row-major, or
 * (offdiag_symmetric != 0) as bs(bs+1)/2 upper entries as the reference stores
 * them.  Replaces BCRSSymSpMV (algebra/sfem_bcrs_sym_SpMV.hpp:9-279). */
int sfem_gb300_bsr_sym_spmv(int real_type, int block_size, ptrdiff_t nblock_rows, const int32_t *rowptr,
                            const int32_t *colidx, const void *diag_sym, const void *offdiag, int offdiag_symmetric,
                            double scale_output, const void *x, void *y, void *stream);

/* diag += diag(A), offdiag += strict upper part of the hex8 Laplacian on a given
 * upper CRS graph (elements in hex8 corner order).  Fails if an element coupling
 * is missing from the graph.  Replaces cu_laplacian_crs_sym / hex8_laplacian_crs_sym
 * (operators/cuda/cu_laplacian.hpp:44-53, operators/hex8/hex8_laplacian.cpp:148-221). */
int sfem_gb300_hex8_laplacian_crs_sym(ptrdiff_t nelements, sfem_gb300_idx_t **elements, ptrdiff_t fff_stride,
                                      const float *fff, const int32_t *rowptr, const int32_t *colidx, int real_type,
                                      void *diag, void *offdiag, void *stream);

/* values += the hex8 Laplacian on a full CRS graph (both triangles; elements in hex8
 * corner order).  Fails if an element coupling is missing from the graph.  The
 * reference's hex8_laplacian_crs (operators/hex8/hex8_laplacian.cpp:223) on the GPU. */
int sfem_gb300_hex8_laplacian_crs(ptrdiff_t nelements, sfem_gb300_idx_t **elements, ptrdiff_t fff_stride,
                                  const float *fff, const int32_t *rowptr, const int32_t *colidx, int real_type,
                                  void *values, void *stream);

/* The reference's Laplacian assembly entry points under its names and argument order
 * (operators/cuda/cu_laplacian.hpp:32-53): element_type HEX8 (the reference's CUDA
 * crs_sym serves HEX8 only; its crs serves tetrahedra only, which are out of scope here,
 * so cu_laplacian_crs serves HEX8 instead); others return FAILURE with a message. */
int cu_laplacian_crs(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements, ptrdiff_t fff_stride,
                     const void *fff, const int32_t *rowptr, const int32_t *colidx, int real_type, void *values,
                     void *stream);
int cu_laplacian_crs_sym(int element_type, ptrdiff_t nelements, sfem_gb300_idx_t **elements, ptrdiff_t fff_stride,
                         const void *fff, const int32_t *rowptr, const int32_t *colidx, int real_type, void *diag,
                         void *offdiag, void *stream);

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

/* Allocation-free dot product for callers that cannot allocate device memory:
 * code running while someone else's stream capture is building a CUDA graph,
 * code inside a memory arena or pool that forbids cudaMalloc, plugins whose host
 * application owns every allocation.  No reference counterpart.  Same result as
 * sfem_gb300_dot (deterministic order), but the scratch is a fixed array inside
 * the library (1024 block partial sums + a ticket word, 8.25 KiB per GPU, held
 * until the process exits) instead of a caller workspace.  n above
 * SFEM_GB300_NOALLOC_MAX_N is rejected.  All calls on a GPU share that scratch:
 * calls that may overlap on the GPU (different streams, unordered threads) race
 * and must be serialised by the caller.  Every call looks up the scratch address
 * in the current context (host-side, no allocation); the first call that sees an
 * address on a device (the first there, or the first after a device reset or a
 * context change) clears the scratch; make that first call before any stream
 * capture.  *result is a device pointer. */
#define SFEM_GB300_NOALLOC_MAX_N 2147483647LL
int sfem_gb300_dot_noalloc(int real_type, ptrdiff_t n, const void *x, const void *y, double *result, void *stream);

/* Fused CG updates with device-resident scalars (no host round trip), cf. the
 * host fusion in algebra/sfem_cg.hpp:26-72:
 *   alpha = *alpha_num / *alpha_den;  x += alpha p;  r -= alpha Ap;  if rr: *rr = (r, r). */
int sfem_gb300_cg_update_x_r(int real_type, ptrdiff_t n, const double *alpha_num, const double *alpha_den,
                             const void *p, const void *Ap, void *x, void *r, void *workspace, double *rr,
                             void *stream);
/*   beta = (*beta_num - *beta_sub) / *beta_den;  p = z + beta p  (beta_sub may be NULL;
 * with it this is the flexible-CG Polak-Ribiere update). */
int sfem_gb300_cg_update_p(int real_type, ptrdiff_t n, const double *beta_num, const double *beta_den,
                           const double *beta_sub, const void *z, void *p, void *stream);
/* Chebyshev3 step p = beta p - rhs + Ax;  x -= alpha p (algebra/sfem_Chebyshev3.hpp:36-52).
 * With a non-NULL inv_diag the step runs on the Jacobi-scaled operator: p = beta p + D^-1 (Ax - rhs).
 * beta == 0 ignores the previous p. */
int sfem_gb300_chebyshev_update(int real_type, ptrdiff_t n, double alpha, double beta, const void *inv_diag,
                                const void *rhs, const void *Ax, void *p, void *x, void *stream);

/* Dirichlet constraints on interleaved vectors (operators/boundary_conditions/dirichlet.hpp:44-130):
 * dest[node*block+comp] = src[node*block+comp], resp. x[node*block+comp] = value. */
int sfem_gb300_constraint_nodes_copy(int real_type, ptrdiff_t n_nodes, const int32_t *nodes, int block_size,
                                     int component, const void *src, void *dest, void *stream);
int sfem_gb300_constraint_nodes_to_value(int real_type, ptrdiff_t n_nodes, const int32_t *nodes, int block_size,
                                         int component, double value, void *x, void *stream);

/* x[i] = U(-1, 1), a counter-based hash of (seed, i): reproducible start vectors
 * (the reference's Chebyshev3::init_with_random, algebra/sfem_Chebyshev3.hpp:148-160). */
int sfem_gb300_random_uniform(int real_type, ptrdiff_t n, unsigned long long seed, void *x, void *stream);

/* Precision conversion dst = (dst_type) src, and y += alpha (double) x for float x. */
int sfem_gb300_convert(ptrdiff_t n, int src_type, const void *src, int dst_type, void *dst, void *stream);
int sfem_gb300_axpy_f32_to_f64(ptrdiff_t n, double alpha, const float *x, double *y, void *stream);
/* Precision bridge with a device-resident scale (no host round trip):
 * dst = (float)(src / *nrm) (0 if *nrm == 0);  y += *nrm * (double) x. */
int sfem_gb300_scaled_to_f32(ptrdiff_t n, const double *nrm, const double *src, float *dst, void *stream);
int sfem_gb300_scaled_axpy_f32_to_f64(ptrdiff_t n, const double *nrm, const float *x, double *y, void *stream);

/* ------------------------------------------------------- learned smoother */
/* No reference counterpart.  A patch is the 5x5x5 node grid of one level-4
 * sshex8 macro element (lidx order).  Activations are BF16, channels-last
 * [P][125][C]; weights BF16 [cout][cin][27] (3x3x3 offsets, x fastest); FP32
 * arithmetic.  Channel pairs (cin, cout) in {1, 16} x {1, 16}. */

/* out = act(conv3x3x3(in, W)) with zero padding; act = ReLU if relu != 0. */
int sfem_gb300_patchconv_forward(ptrdiff_t P, int cin, int cout, const void *in, const void *W, int relu, void *out,
                                 void *stream);
/* gin = conv^T(gout, W), multiplied by ReLU'(in_act) when in_act is not NULL. */
int sfem_gb300_patchconv_backward_data(ptrdiff_t P, int cin, int cout, const void *gout, const void *W,
                                       const void *in_act, void *gin, void *stream);
/* dW (FP32, cout*cin*27) += sum over patches and positions of gout (x) in. */
int sfem_gb300_patchconv_backward_weights(ptrdiff_t P, int cin, int cout, const void *gout, const void *in, float *dW,
                                          void *stream);
/* Patches of (scale .* r) normalised by their RMS (patch_scale[p], 1 for an all-zero patch);
 * elements = level-4 sshex8 connectivity, scale may be NULL. */
int sfem_gb300_gather_patches(int real_type, ptrdiff_t P, sfem_gb300_idx_t **elements, const void *r,
                              const void *scale, void *out_bf16, float *patch_scale, void *stream);
/* x[g] += alpha * patch_scale[p] * in[p][v] / count[g] (corrections averaged over shared nodes). */
int sfem_gb300_scatter_patches(int real_type, ptrdiff_t P, sfem_gb300_idx_t **elements, const void *in_bf16,
                               const float *patch_scale, const uint16_t *count, double alpha, void *x, void *stream);

/* Fused learned correction (inference): for every patch p, gather s^-1 (inv_diag . r)
 * (s = patch RMS), run the three BF16 convolutions on the tensor cores (FP32
 * accumulate), and d[g] += omega * s * out[v] / count[g].  `frag` holds the
 * weights as tensor-core operands (sfem_gb300_learned_fragments_size() bytes,
 * 16-byte aligned, built by sfem_gb300_learned_fragments from the [co][ci][27]
 * BF16 weights of the 1 -> 16 -> 16 -> 1 network).  Same result as
 * gather_patches + patchconv_forward x3 + scatter_patches up to accumulation order.
 * Kernel variant (sfem_gb300_set_learned_kernel): 0 = tcgen05.mma with the
 * accumulators in tensor memory (default), 1 = warp-level mma.sync.
 * sfem_gb300_learned_status returns (and clears) 1 if a tcgen05 kernel gave up
 * waiting for its tensor-core work (its corrections are then incomplete), 0 if not. */
size_t sfem_gb300_learned_fragments_size(void);
int sfem_gb300_learned_fragments(const void *W1, const void *W2, const void *W3, void *frag, void *stream);
int sfem_gb300_learned_correction(int real_type, ptrdiff_t P, sfem_gb300_idx_t **elements, const void *r,
                                  const void *inv_diag, const void *frag, const uint16_t *count, double omega,
                                  void *d, void *stream);
int sfem_gb300_set_learned_kernel(int variant);
int sfem_gb300_learned_status(void);
/* gy = 2 (y - target) / n (BF16), *loss += mean squared error (FP32, may be NULL). */
int sfem_gb300_mse_grad(ptrdiff_t n, const void *y, const void *target, void *gy, float *loss, void *stream);
/* Adam step on FP32 master weights, mirrored into BF16 (t = 1-based step). */
int sfem_gb300_adam_step(int n, float *w, const float *g, float *m, float *v, void *w_bf16, float lr, float beta1,
                         float beta2, float eps, int t, void *stream);

/* ------------------------------------------------- operators and solvers */
/* Opaque handles (void *) over the device solver layer, mirroring the
 * reference's frontend factories (frontend/sfem_API.hpp: create_cg :143,
 * create_shiftable_jacobi :180, create_stationary :247, create_cheb3 :287,
 * create_mg :323) and Operator<T>::apply (algebra/sfem_Operator.hpp:13-33).
 * The caller owns every device array passed in and keeps it alive while the
 * handle exists; handles own their work vectors.  Every handle is released
 * with sfem_gb300_handle_destroy.  Linear operators accumulate (y += A x);
 * solvers take (b, x) with x as the initial guess. */

/* Stream (pointer to cudaStream_t or NULL) + reduction workspace shared by the handles built on it. */
int sfem_gb300_context_create(void *stream, void **context);
int sfem_gb300_handle_destroy(void *handle);

/* Function-level Laplacian: y += A x, then y[c] = x[c] on Dirichlet nodes
 * (Function::apply + copy_constrained_dofs, frontend/sfem_Function.cpp:481-496).
 * An FP32 sshex8 L = 4 operator packs the connectivity and FFF at creation
 * (sfem_gb300_sshex8_pack) and applies from the packed tiles, so it keeps the
 * geometry it was created with; other operators read `fff` at every apply. */
int sfem_gb300_laplacian_op_create(void *context, int real_type, int element_type, ptrdiff_t nelements,
                                   sfem_gb300_idx_t **elements, ptrdiff_t fff_stride, const float *fff,
                                   ptrdiff_t n_nodes, ptrdiff_t n_dirichlet, const int32_t *dirichlet_nodes,
                                   void **op);
/* Function-level linear elasticity (3 dofs/node, all components fixed on Dirichlet nodes).
 * On hex8 and L <= 2 levels the element matrices are built once here, from the geometry
 * as it is at creation, and applied from memory (sfem_gb300_linear_elasticity_apply_em). */
int sfem_gb300_elasticity_op_create(void *context, int real_type, int element_type, ptrdiff_t nelements,
                                    sfem_gb300_idx_t **elements, ptrdiff_t jacobian_stride, const float *adjugate,
                                    const float *determinant, double mu, double lambda, ptrdiff_t n_nodes,
                                    ptrdiff_t n_dirichlet, const int32_t *dirichlet_nodes, void **op);
/* Prolongation (coarse level -> fine level) then zero fine Dirichlet dofs
 * (algebra/mg/sfem_GeometricMultigrid.cpp:54-66). */
int sfem_gb300_prolongation_op_create(void *context, int real_type, ptrdiff_t nelements, int from_level,
                                      sfem_gb300_idx_t **from_elements, ptrdiff_t n_from, int to_level,
                                      sfem_gb300_idx_t **to_elements, ptrdiff_t n_to, int vec_size,
                                      ptrdiff_t n_dirichlet_to, const int32_t *dirichlet_to, void **op);
/* Restriction (fine -> coarse) then zero coarse Dirichlet dofs (:38-52). */
int sfem_gb300_restriction_op_create(void *context, int real_type, ptrdiff_t nelements, int from_level,
                                     sfem_gb300_idx_t **from_elements, const uint16_t *count, ptrdiff_t n_from,
                                     int to_level, sfem_gb300_idx_t **to_elements, ptrdiff_t n_to, int vec_size,
                                     ptrdiff_t n_dirichlet_to, const int32_t *dirichlet_to, void **op);
/* Symmetric CRS operator (y += A x) with Dirichlet rows treated as identity: an
 * assembled coarse-level operator for the multigrid hierarchy. */
int sfem_gb300_crs_sym_op_create(void *context, int real_type, ptrdiff_t nrows, const int32_t *rowptr,
                                 const int32_t *colidx, const void *diag, const void *offdiag, ptrdiff_t n_dirichlet,
                                 const int32_t *dirichlet_nodes, void **op);
int sfem_gb300_op_apply(void *op, const void *x, void *y);
int sfem_gb300_op_size(void *op, ptrdiff_t *rows, ptrdiff_t *cols);

/* Jacobi smoother x += relaxation D^-1 b (ShiftableJacobi, algebra/sfem_ShiftableJacobi.hpp:15-65). */
int sfem_gb300_jacobi_create(void *context, int real_type, ptrdiff_t n, const void *diag, double relaxation,
                             void **solver);
/* 3x3 block Jacobi x += B b with block6 already inverted by sfem_gb300_block3_invert
 * (ShiftableBlockSymJacobi, algebra/sfem_ShiftableJacobi.hpp:67-155). */
int sfem_gb300_block_jacobi_create(void *context, int real_type, ptrdiff_t n_nodes, const void *inv_block6,
                                   void **solver);
/* Stationary iteration x += P (b - A x), max_it sweeps (algebra/sfem_Stationary.hpp:19-133). */
int sfem_gb300_stationary_create(void *context, void *op, void *precond, int max_it, void **solver);
/* Chebyshev3 smoother; runs the power method from a vector of ones at creation
 * (algebra/sfem_Chebyshev3.hpp:56-312, algebra/sfem_PowerMethod.hpp:18-55).
 * inv_diag (n entries, may be NULL) selects the Jacobi-scaled iteration on D^-1 A; the
 * caller keeps it alive.  Unscaled, the identity rows of Dirichlet nodes (eigenvalue 1)
 * dominate the spectrum estimate on fine meshes, where the stiffness eigenvalues scale with h. */
int sfem_gb300_chebyshev3_create(void *context, void *op, const void *inv_diag, int max_it, double scale_eig_max,
                                 double scale_eig_min, int eigen_max_it, double eigen_tol, void **solver);
int sfem_gb300_chebyshev3_eig_max(void *solver, double *eig_max);
int sfem_gb300_chebyshev3_set_eig_max(void *solver, double eig_max);
/* (Preconditioned) conjugate gradient (algebra/sfem_cg.hpp:79-453); precond may be NULL.
 * Default stopping test is the reference's: sqrt(r.z) < atol or sqrt(r.z)/sqrt(r0.z0) < rtol. */
int sfem_gb300_cg_create(void *context, void *op, void *precond, int max_it, double rtol, double atol, void **solver);
/* Options: residual_norm != 0 stops on ||r||_2 / ||r0||_2 < rtol (the true residual for
 * x0 = 0) instead of the preconditioned norm; flexible != 0 uses the Polak-Ribiere beta
 * (r_k . (z_k - z_{k-1})) / (r_{k-1} . z_{k-1}), i.e. flexible CG for variable or
 * inexact preconditioners (no reference counterpart); check_every = k reads the
 * convergence scalar from the device only every k iterations (>= 1). */
int sfem_gb300_cg_set_options(void *solver, int residual_norm, int flexible, int check_every);
int sfem_gb300_cg_set_verbose(void *solver, int verbose);
/* Multigrid V/W cycle (algebra/sfem_Multigrid.hpp:27-354); levels added finest first. */
int sfem_gb300_mg_create(void *context, int real_type, int max_it, int cycle_type, void **solver);
int sfem_gb300_mg_add_level(void *mg, void *op, void *smoother, void *prolongation, void *restriction);
/* Learned smoother for level-4 sshex8 Laplacians: `sweeps` times
 *   r = b - A x;  x += omega * scatter(net(gather(D^-1 r)))
 * with the 3-layer patch network (W1: channels x 1 x 27, W2: channels x channels x 27,
 * W3: 1 x channels x 27, BF16).  Usable as a multigrid smoother or, with a Chebyshev3
 * handle as `fallback`, switched to the fallback by sfem_gb300_learned_smoother_use_fallback. */
int sfem_gb300_learned_smoother_create(void *context, void *op, sfem_gb300_idx_t **elements, ptrdiff_t nelements,
                                       const uint16_t *count, const void *inv_diag, const void *W1, const void *W2,
                                       const void *W3, int channels, double omega, int sweeps, void *fallback,
                                       void **solver);
int sfem_gb300_learned_smoother_use_fallback(void *solver, int use_fallback);
/* chain 1: the fallback smoother first, then the learned corrections; chain 2: the
 * learned corrections first (on the coarse-grid-corrected iterate), then the fallback. */
int sfem_gb300_learned_smoother_set_chain(void *solver, int chain);
/* Let a CG (residual not decreasing for 2 checks) or an iterative refinement (FP64
 * residual not halved by an outer step) switch the learned smoother to its fallback. */
int sfem_gb300_solver_set_fallback(void *solver, void *learned_smoother);
int sfem_gb300_solver_fallback_used(void *solver, int *used);
/* Replace the (pre-)smoother of a level, or set a separate post-smoother (level 0 = finest). */
int sfem_gb300_mg_set_pre_smoother(void *mg, int level, void *smoother);
int sfem_gb300_mg_set_post_smoother(void *mg, int level, void *smoother);
/* Copy of the finest-level iterate after each coarse-grid correction into x_cc (device, n entries). */
int sfem_gb300_mg_set_harvest(void *mg, void *x_cc);
/* Graph mode (no reference counterpart): the V-cycles of each (b, x) pair are
 * captured once into a CUDA graph and replayed.  Requires host-synchronisation-free
 * levels (Chebyshev3 / Jacobi smoothers, a dense coarse solver). */
int sfem_gb300_mg_set_graph(void *mg, int enable);
/* Dense direct solver for a small (<= 1536 unknowns) SPD coarsest level: the matrix is
 * built from the operator, inverted once by Cholesky, applied as x += A^-1 b. */
int sfem_gb300_dense_solver_create(void *context, void *op, void **solver);
/* Operator y = P x (CSR, see sfem_gb300_crs_transfer), output Dirichlet dofs zeroed. */
int sfem_gb300_crs_transfer_op_create(void *context, int real_type, ptrdiff_t nrows, ptrdiff_t ncols,
                                      const sfem_gb300_idx_t *rowptr, const sfem_gb300_idx_t *colidx,
                                      const double *weights, int vec_size, ptrdiff_t n_dirichlet,
                                      const sfem_gb300_idx_t *dirichlet, void **op);

/* FP64 iterative refinement around a float inner solver (no reference counterpart):
 * r = b - A x in double, d = inner(r/|r|) in float, x += |r| d, until |r| <= rtol |b|. */
int sfem_gb300_ir_create(void *context, void *op64, void *inner32, int max_it, double rtol, void **solver);
/* Float preconditioner for a double Krylov method (no reference counterpart):
 * z = |r| inner(r / |r|) with the norm kept on the device, so FP64 carries the
 * Krylov recurrence, true residual and solution while the preconditioner (e.g. a
 * float multigrid V-cycle) runs in FP32. */
int sfem_gb300_mixed_precond_create(void *context, void *inner32, void **op64);
int sfem_gb300_solver_apply(void *solver, const void *b, void *x);
int sfem_gb300_solver_stats(void *solver, int *iterations, double *last_relative);

/* ------------------------------------------------------------ batched solves
 * No reference counterpart (the reference runs one solve per process).  The
 * vectors of P independent problems are concatenated, problem p owning the
 * dof range [offsets[p], offsets[p+1]).  Element operators need no batched
 * form: connectivity of several problems concatenated with node offsets is a
 * larger mesh.  The calls below add the per-problem Krylov algebra. */

/* Work list of (problem, dof range) chunks of at most `chunk` dofs (host offsets, P + 1). */
int sfem_gb300_batch_layout_create(void *context, int n_problems, const int64_t *offsets, int chunk, void **layout);
/* Launch shape of the batched vector kernels: chunk, threads per CTA (multiple of 32,
 * <= 1024), CTAs per SM of the persistent grid.  Graphs captured before are rebuilt. */
int sfem_gb300_batch_layout_set_launch(void *layout, int chunk, int threads, int ctas_per_sm);
/* d_out[p] = (x_p, y_p) for every problem (device array of P doubles), deterministic. */
int sfem_gb300_batch_dot(void *layout, int real_type, const void *x, const void *y, double *d_out);
/* Block-diagonal operator: ops[g] acts on [offsets[g], offsets[g+1]) (host offsets). */
int sfem_gb300_batch_grouped_op_create(void *context, int real_type, int n_ops, void **ops, const int64_t *offsets,
                                       void **op);
/* Chebyshev3 on D^-1 A with one eigenvalue estimate per problem (batched power method,
 * eigen_max_it normalised iterations from a seeded U(-1,1) vector). */
int sfem_gb300_batch_chebyshev3_create(void *context, void *layout, void *op, const void *inv_diag, int max_it,
                                       double scale_eig_max, double scale_eig_min, int eigen_max_it,
                                       unsigned long long seed, void **solver);
int sfem_gb300_batch_chebyshev3_eig_max(void *solver, double *eig_max_out /* host, P */);
/* (Flexible) preconditioned CG over the batch: exactly `iterations` iterations per
 * apply, per-problem scalars on the device, problem p stops updating once
 * ||r_p|| <= rtol ||r0_p||.  Never synchronises with the host. */
int sfem_gb300_batch_cg_create(void *context, void *layout, void *op, void *precond, int iterations, double rtol,
                               int flexible, void **solver);
/* z += ||r_p|| M32(r_p / ||r_p||): a float preconditioner (the grouped float
 * multigrid) under a double batched Krylov method, norms kept on the device. */
int sfem_gb300_batch_bridge_create(void *context, void *layout, void *inner32, void **op64);
/* Host driver of a double batched CG: start, then chunks of check_every iterations
 * captured into one CUDA graph (use_graph) and replayed until every problem has
 * ||r_p|| <= rtol ||b_p|| (the CG's rtol; zero initial guess). */
int sfem_gb300_batch_solve_create(void *context, void *layout, void *cg64, int check_every, int max_it,
                                  int use_graph, void **solver);
int sfem_gb300_batch_solve_set_launch(void *solver, int check_every);
/* Host outputs (each may be NULL): seconds from start until problem p was seen
 * converged, the iteration count at that check, total seconds. */
int sfem_gb300_batch_solve_run(void *solver, const double *b, double *x, double *latency_s,
                               int *iterations_per_problem, double *seconds);
/* The same with staggered arrivals: release_s[p] (host) is problem p's release time in
 * seconds from the start of the call.  A problem keeps its start state until the first
 * chunk boundary after its release, then iterates; latency_s and the iteration counts
 * are counted from its release. */
int sfem_gb300_batch_solve_run_released(void *solver, const double *b, double *x, const double *release_s,
                                        double *latency_s, int *iterations_per_problem, double *seconds);
/* Non-blocking driver, for several batched solvers (each with its own context) that
 * advance independently on their own streams: begin captures the chunk if needed and
 * starts the CG; step launches one chunk and the copy of the active mask; poll returns
 * 2 while that mask is in flight (SFEM_GB300_FAILURE on an error), else 0 with the mask
 * in active[P] (may be NULL), the
 * number of active problems and the iterations done.  A problem has converged when its
 * flag drops to 0; step again only after poll returned 0 with problems still active. */
int sfem_gb300_batch_solve_begin(void *solver, const double *b, double *x);
/* Stream priority of the solver's own stream: level 0 the default, each level one step
 * higher, clamped to the device's priority range (not while a chunk is in flight). */
int sfem_gb300_batch_solve_set_priority(void *solver, int level);
int sfem_gb300_batch_solve_step(void *solver);
int sfem_gb300_batch_solve_poll(void *solver, int *active, int *n_active, int *iterations);
/* Mean milliseconds of `reps` replays of the captured chunk starting from x (x is
 * modified): the autotuner's measurement. */
int sfem_gb300_batch_solve_time_chunk(void *solver, const double *b, double *x, int reps, double *ms);

#ifdef __cplusplus
}
#endif

#endif /* SFEM_GB300_H */
