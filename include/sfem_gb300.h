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

#ifdef __cplusplus
}
#endif

#endif /* SFEM_GB300_H */
