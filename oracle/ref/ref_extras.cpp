// Thin extern "C" entry points around the reference's header-inline kernels,
// compiled together with the reference's own operator sources into
// oracle/_ref/libsfem_ref.so (see oracle/build.py).  Test infrastructure only:
// this library is the checker for the oracle restatement and is never part of
// the product.
#include "sfem_base.hpp"
#include "sfem_macros.hpp"

#include "hex8_inline_cpu.hpp"
#include "hex8_laplacian_inline_cpu.hpp"
#include "hex8_linear_elasticity_inline_cpu.hpp"

#include <stdlib.h>

extern "C" void sfem_abort() { abort(); }

// operators/hex8/hex8_laplacian_inline_cpu.hpp:213
extern "C" void ref_hex8_laplacian_matrix_fff_integral(const double *fff, double *element_matrix) {
    hex8_laplacian_matrix_fff_integral(fff, element_matrix);
}

// operators/hex8/hex8_laplacian_inline_cpu.hpp:332
extern "C" void ref_hex8_laplacian_apply_fff_integral(const double *fff, const double *u, double *out) {
    hex8_laplacian_apply_fff_integral(fff, u, out);
}

// operators/hex8/hex8_linear_elasticity_inline_cpu.hpp:207
extern "C" void ref_hex8_linear_elasticity_matrix(double mu, double lambda, const double *adjugate, double det,
                                                  double *element_matrix) {
    hex8_linear_elasticity_matrix(mu, lambda, adjugate, det, element_matrix);
}

// operators/hex8/hex8_inline_cpu.hpp:13 evaluated at the element centre, as the
// reference's FFF cache does (operators/hex8/hex8_fff.cpp:5-37).  The 8 corner
// index arrays are given in standard hex8 order.
extern "C" int ref_hex8_fff_fill(ptrdiff_t nelements, idx_t **corners, geom_t **points, jacobian_t *fff) {
    const geom_t *const x = points[0];
    const geom_t *const y = points[1];
    const geom_t *const z = points[2];
#pragma omp parallel for
    for (ptrdiff_t e = 0; e < nelements; e++) {
        scalar_t lx[8], ly[8], lz[8], f[6];
        for (int v = 0; v < 8; v++) {
            const idx_t n = corners[v][e];
            lx[v] = x[n];
            ly[v] = y[n];
            lz[v] = z[n];
        }
        hex8_fff(lx, ly, lz, 0.5, 0.5, 0.5, f);
        for (int d = 0; d < 6; d++) fff[e * 6 + d] = (jacobian_t)f[d];
    }
    return 0;
}

// operators/hex8/hex8_inline_cpu.hpp:90 at the element centre, stored AoS as
// the reference's macro adjugate cache (frontend/ops/sfem_LinearElasticity.cpp:252-289).
extern "C" int ref_hex8_adjugate_and_det_fill(ptrdiff_t nelements, idx_t **corners, geom_t **points,
                                              jacobian_t *adjugate, jacobian_t *determinant) {
    const geom_t *const x = points[0];
    const geom_t *const y = points[1];
    const geom_t *const z = points[2];
#pragma omp parallel for
    for (ptrdiff_t e = 0; e < nelements; e++) {
        scalar_t lx[8], ly[8], lz[8], adj[9], det;
        for (int v = 0; v < 8; v++) {
            const idx_t n = corners[v][e];
            lx[v] = x[n];
            ly[v] = y[n];
            lz[v] = z[n];
        }
        hex8_adjugate_and_det(lx, ly, lz, 0.5, 0.5, 0.5, adj, &det);
        for (int d = 0; d < 9; d++) adjugate[e * 9 + d] = (jacobian_t)adj[d];
        determinant[e] = (jacobian_t)det;
    }
    return 0;
}
