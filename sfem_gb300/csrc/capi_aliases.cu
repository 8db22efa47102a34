// Entry points under the reference's own CUDA ABI names (operators/cuda/cu_laplacian.hpp,
// operators/cuda/cu_linear_elasticity.hpp) that forward to this library's kernels with the
// reference's argument order and meaning: interleaved xyz vectors for elasticity, SoA
// float geometry with a stride, accumulate semantics, `stream` a pointer to a
// cudaStream_t.  Unsupported element or real types return FAILURE with a message.
#include "common.cuh"

extern "C" {
int sfem_gb300_linear_elasticity_apply(int element_type, ptrdiff_t nelements, sfem_gb300::idx_t **elements,
                                       ptrdiff_t jacobian_stride, const float *adjugate, const float *determinant,
                                       double mu, double lambda, int real_type, const void *u, void *out,
                                       void *stream);
int sfem_gb300_linear_elasticity_block_diag(int element_type, ptrdiff_t nelements, sfem_gb300::idx_t **elements,
                                            ptrdiff_t jacobian_stride, const float *adjugate,
                                            const float *determinant, double mu, double lambda, int real_type,
                                            void *diag3, void *block6, void *stream);
int sfem_gb300_hex8_laplacian_crs_sym(ptrdiff_t nelements, sfem_gb300::idx_t **elements, ptrdiff_t fff_stride,
                                      const float *fff, const int32_t *rowptr, const int32_t *colidx, int real_type,
                                      void *diag, void *offdiag, void *stream);
int sfem_gb300_hex8_laplacian_crs(ptrdiff_t nelements, sfem_gb300::idx_t **elements, ptrdiff_t fff_stride,
                                  const float *fff, const int32_t *rowptr, const int32_t *colidx, int real_type,
                                  void *values, void *stream);
}

using namespace sfem_gb300;

extern "C" int cu_linear_elasticity_apply(int element_type, ptrdiff_t nelements, idx_t **elements,
                                          ptrdiff_t jacobian_stride, const void *jacobian_adjugate,
                                          const void *jacobian_determinant, double mu, double lambda, int real_type,
                                          const void *x, void *y, void *stream) {
    return sfem_gb300_linear_elasticity_apply(element_type, nelements, elements, jacobian_stride,
                                              (const float *)jacobian_adjugate, (const float *)jacobian_determinant,
                                              mu, lambda, real_type, x, y, stream);
}

extern "C" int cu_linear_elasticity_diag(int element_type, ptrdiff_t nelements, idx_t **elements,
                                         ptrdiff_t jacobian_stride, const void *jacobian_adjugate,
                                         const void *jacobian_determinant, double mu, double lambda, int real_type,
                                         void *diag, void *stream) {
    return sfem_gb300_linear_elasticity_block_diag(element_type, nelements, elements, jacobian_stride,
                                                   (const float *)jacobian_adjugate,
                                                   (const float *)jacobian_determinant, mu, lambda, real_type, diag,
                                                   nullptr, stream);
}

extern "C" int cu_linear_elasticity_block_diag_sym_aos(int element_type, ptrdiff_t nelements, idx_t **elements,
                                                       ptrdiff_t jacobian_stride, const void *jacobian_adjugate,
                                                       const void *jacobian_determinant, double mu, double lambda,
                                                       int real_type, void *out, void *stream) {
    return sfem_gb300_linear_elasticity_block_diag(element_type, nelements, elements, jacobian_stride,
                                                   (const float *)jacobian_adjugate,
                                                   (const float *)jacobian_determinant, mu, lambda, real_type, nullptr,
                                                   out, stream);
}

extern "C" int cu_laplacian_crs_sym(int element_type, ptrdiff_t nelements, idx_t **elements, ptrdiff_t fff_stride,
                                    const void *fff, const int32_t *rowptr, const int32_t *colidx, int real_type,
                                    void *diag, void *offdiag, void *stream) {
    if (element_type != SFEM_GB300_HEX8)
        return set_error("cu_laplacian_crs_sym: element type %d (HEX8 only, as the reference)", element_type);
    return sfem_gb300_hex8_laplacian_crs_sym(nelements, elements, fff_stride, (const float *)fff, rowptr, colidx,
                                             real_type, diag, offdiag, stream);
}

extern "C" int cu_laplacian_crs(int element_type, ptrdiff_t nelements, idx_t **elements, ptrdiff_t fff_stride,
                                const void *fff, const int32_t *rowptr, const int32_t *colidx, int real_type,
                                void *values, void *stream) {
    if (element_type != SFEM_GB300_HEX8)
        return set_error("cu_laplacian_crs: element type %d (HEX8 only)", element_type);
    return sfem_gb300_hex8_laplacian_crs(nelements, elements, fff_stride, (const float *)fff, rowptr, colidx,
                                         real_type, values, stream);
}
