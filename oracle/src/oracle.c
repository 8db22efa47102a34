/*
 * CPU oracle: a plain-C restatement of the reference's (zulianp/sfem) CPU
 * algorithms on the matrix-free operator path.  TEST INFRASTRUCTURE ONLY:
 * the parity tests, smoke() and bench.py's CPU-baseline leg are the only
 * users; the product never links or calls this file.
 *
 * Conventions follow the reference's CPU path:
 *   real_t = double (vectors, accumulation), geom_t = jacobian_t = float
 *   (coordinates and cached geometry), idx_t = int32 (cmake/SFEMNumbers.cmake:5-14);
 *   connectivity is SoA elements[v][e]; the CPU FFF / adjugate caches are AoS
 *   (fff[e*6+d], adj[e*9+d]) as in operators/hex8/hex8_fff.cpp:31-33.
 *
 * Element matrices are derived here from the tensor-product structure of the
 * Q1 basis on [0,1]^3 (exact integration of the affine-element bilinear
 * forms); the reference uses generated closed forms with the same values.
 * The oracle is pinned against the reference's own compiled sources by the
 * CPU test-suite (oracle/_ref, built from the reference tree).
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int32_t idx_t;
typedef float geom_t;
typedef float jacobian_t;

/* standard hex8 corner order (operators/sshex8/sshex8.hpp:53-62) */
static const int C8[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

static inline int lidx(int L, int x, int y, int z) { return z * (L + 1) * (L + 1) + y * (L + 1) + x; }

static inline void atomic_add(double *p, double v) {
#pragma omp atomic update
    *p += v;
}

/* ------------------------------------------------------------------------ */
/* 1D integrals of the linear basis psi0 = 1-t, psi1 = t on [0,1]           */
/* ------------------------------------------------------------------------ */
static inline double m1(int a, int b) { return a == b ? 1.0 / 3.0 : 1.0 / 6.0; }  /* int psi_a psi_b   */
static inline double k1(int a, int b) { return a == b ? 1.0 : -1.0; }             /* int psi'_a psi'_b */
static inline double g1(int a, int b) { (void)b; return a ? 0.5 : -0.5; }         /* int psi'_a psi_b  */

/* int d_p phi_c d_q phi_e over the unit cube (p, q in 0..2) */
static double grad_integral(int c, int e, int p, int q) {
    double r = 1.0;
    for (int d = 0; d < 3; d++) {
        const int a = C8[c][d], b = C8[e][d];
        if (d == p && d == q)
            r *= k1(a, b);
        else if (d == p)
            r *= g1(a, b);
        else if (d == q)
            r *= g1(b, a);
        else
            r *= m1(a, b);
    }
    return r;
}

static double I_table[8][8][3][3];
static int I_ready = 0;
static void ensure_tables(void) {
    if (I_ready) return;
#pragma omp critical(oracle_tables)
    {
        if (!I_ready) {
            for (int c = 0; c < 8; c++)
                for (int e = 0; e < 8; e++)
                    for (int p = 0; p < 3; p++)
                        for (int q = 0; q < 3; q++) I_table[c][e][p][q] = grad_integral(c, e, p, q);
            I_ready = 1;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Geometry                                                                 */
/* ------------------------------------------------------------------------ */

/* Jacobian J[i][p] = d x_i / d xi_p of the trilinear map at (qx,qy,qz).
 * The reference evaluates it at the element centre (hex8_inline_cpu.hpp:13-73, :90-150). */
static void hex8_jacobian(const double *x, const double *y, const double *z, double qx, double qy, double qz,
                          double J[3][3]) {
    const double q[3] = {qx, qy, qz};
    const double *X[3] = {x, y, z};
    for (int i = 0; i < 3; i++)
        for (int p = 0; p < 3; p++) J[i][p] = 0;
    for (int c = 0; c < 8; c++) {
        double w[3], dw[3];
        for (int d = 0; d < 3; d++) {
            w[d] = C8[c][d] ? q[d] : 1 - q[d];
            dw[d] = C8[c][d] ? 1.0 : -1.0;
        }
        const double dphi[3] = {dw[0] * w[1] * w[2], w[0] * dw[1] * w[2], w[0] * w[1] * dw[2]};
        for (int i = 0; i < 3; i++)
            for (int p = 0; p < 3; p++) J[i][p] += X[i][c] * dphi[p];
    }
}

/* adj = det(J) J^{-1} (row-major), det = det(J) */
static void adjugate_det(const double J[3][3], double adj[9], double *det) {
    adj[0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    adj[1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    adj[2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    adj[3] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    adj[4] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    adj[5] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    adj[6] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    adj[7] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    adj[8] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    *det = J[0][0] * adj[0] + J[0][1] * adj[3] + J[0][2] * adj[6];
}

/* FFF = det(J) J^{-1} J^{-T}, symmetric, stored (00,01,02,11,12,22)
 * (operators/hex8/hex8_inline_cpu.hpp:13-73). */
static void fff_from_jacobian(const double J[3][3], double fff[6]) {
    double adj[9], det;
    adjugate_det(J, adj, &det);
    /* J^{-1} = adj/det ;  FFF = det * Jinv Jinv^T = (adj adj^T) / det */
    double G[3][3];
    for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += adj[3 * p + k] * adj[3 * q + k];
            G[p][q] = s / det;
        }
    fff[0] = G[0][0];
    fff[1] = G[0][1];
    fff[2] = G[0][2];
    fff[3] = G[1][1];
    fff[4] = G[1][2];
    fff[5] = G[2][2];
}

static void gather_corners(ptrdiff_t e, idx_t **corners, geom_t **points, double x[8], double y[8], double z[8]) {
    for (int v = 0; v < 8; v++) {
        const idx_t n = corners[v][e];
        x[v] = points[0][n];
        y[v] = points[1][n];
        z[v] = points[2][n];
    }
}

/* hex8_fff_fill (operators/hex8/hex8_fff.cpp:5-37): corners in hex8 order. */
int or_hex8_fff_fill(ptrdiff_t nelements, idx_t **corners, geom_t **points, jacobian_t *fff) {
#pragma omp parallel for
    for (ptrdiff_t e = 0; e < nelements; e++) {
        double x[8], y[8], z[8], J[3][3], f[6];
        gather_corners(e, corners, points, x, y, z);
        hex8_jacobian(x, y, z, 0.5, 0.5, 0.5, J);
        fff_from_jacobian(J, f);
        for (int d = 0; d < 6; d++) fff[e * 6 + d] = (jacobian_t)f[d];
    }
    return 0;
}

/* macro adjugate + determinant cache (hex8_adjugate_and_det at the centre,
 * operators/hex8/hex8_inline_cpu.hpp:90; frontend/ops/sfem_LinearElasticity.cpp:252-289). */
int or_hex8_adjugate_and_det_fill(ptrdiff_t nelements, idx_t **corners, geom_t **points, jacobian_t *adjugate,
                                  jacobian_t *determinant) {
#pragma omp parallel for
    for (ptrdiff_t e = 0; e < nelements; e++) {
        double x[8], y[8], z[8], J[3][3], adj[9], det;
        gather_corners(e, corners, points, x, y, z);
        hex8_jacobian(x, y, z, 0.5, 0.5, 0.5, J);
        adjugate_det(J, adj, &det);
        for (int d = 0; d < 9; d++) adjugate[e * 9 + d] = (jacobian_t)adj[d];
        determinant[e] = (jacobian_t)det;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Laplacian                                                                */
/* ------------------------------------------------------------------------ */

/* 8x8 Q1 Laplacian element matrix from the FFF of the (sub-)element
 * (operators/hex8/hex8_laplacian_inline_cpu.hpp:213). */
void or_hex8_laplacian_matrix(const double fff[6], double A[64]) {
    ensure_tables();
    const double F[3][3] = {{fff[0], fff[1], fff[2]}, {fff[1], fff[3], fff[4]}, {fff[2], fff[4], fff[5]}};
    for (int c = 0; c < 8; c++)
        for (int e = 0; e < 8; e++) {
            double s = 0;
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++) s += F[p][q] * I_table[c][e][p][q];
            A[c * 8 + e] = s;
        }
}

static void sshex8_micro_nodes(int L, int xi, int yi, int zi, int lev[8]) {
    for (int c = 0; c < 8; c++) lev[c] = lidx(L, xi + C8[c][0], yi + C8[c][1], zi + C8[c][2]);
}

/* Affine sshex8 Laplacian apply, values += A u.
 * Same operator as affine_sshex8_laplacian_stencil_apply_fff
 * (operators/sshex8/sshex8_laplacian.cpp:698-769): one metric per macro
 * element, sub-FFF = FFF / L (:19-28), applied micro element by micro element
 * as sshex8_apply_element_matrix (operators/sshex8/sshex8.hpp:44-86). */
int or_sshex8_laplacian_apply(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff, const double *u,
                              double *values) {
    const int nxe = (L + 1) * (L + 1) * (L + 1);
#pragma omp parallel
    {
        double *eu = (double *)malloc(nxe * sizeof(double));
        double *ev = (double *)malloc(nxe * sizeof(double));
        idx_t *idx = (idx_t *)malloc(nxe * sizeof(idx_t));
#pragma omp for
        for (ptrdiff_t e = 0; e < nelements; e++) {
            double sub[6], A[64];
            const double h = 1.0 / L;
            for (int d = 0; d < 6; d++) sub[d] = (double)fff[e * 6 + d] * h;
            or_hex8_laplacian_matrix(sub, A);
            for (int v = 0; v < nxe; v++) {
                idx[v] = elements[v][e];
                eu[v] = u[idx[v]];
                ev[v] = 0;
            }
            for (int zi = 0; zi < L; zi++)
                for (int yi = 0; yi < L; yi++)
                    for (int xi = 0; xi < L; xi++) {
                        int lev[8];
                        sshex8_micro_nodes(L, xi, yi, zi, lev);
                        for (int i = 0; i < 8; i++) {
                            double acc = 0;
                            for (int j = 0; j < 8; j++) acc += A[i * 8 + j] * eu[lev[j]];
                            ev[lev[i]] += acc;
                        }
                    }
            for (int v = 0; v < nxe; v++) atomic_add(&values[idx[v]], ev[v]);
        }
        free(eu);
        free(ev);
        free(idx);
    }
    return 0;
}

static inline void atomic_add_f(float *p, float v) {
#pragma omp atomic update
    *p += v;
}

/* The same apply in the reference's float32 number configuration
 * (SFEM_REAL_TYPE=float32, cmake/SFEMNumbers.cmake:5-10: real, scalar and
 * accumulator all float): element matrix, gathers, products and sums in float. */
int or_sshex8_laplacian_apply_f32(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff, const float *u,
                                  float *values) {
    const int nxe = (L + 1) * (L + 1) * (L + 1);
#pragma omp parallel
    {
        float *eu = (float *)malloc(nxe * sizeof(float));
        float *ev = (float *)malloc(nxe * sizeof(float));
        idx_t *idx = (idx_t *)malloc(nxe * sizeof(idx_t));
#pragma omp for
        for (ptrdiff_t e = 0; e < nelements; e++) {
            double sub[6], Ad[64];
            float A[64];
            const float h = 1.0f / (float)L;
            for (int d = 0; d < 6; d++) sub[d] = (double)(fff[e * 6 + d] * h);
            or_hex8_laplacian_matrix(sub, Ad);
            for (int k = 0; k < 64; k++) A[k] = (float)Ad[k];
            for (int v = 0; v < nxe; v++) {
                idx[v] = elements[v][e];
                eu[v] = u[idx[v]];
                ev[v] = 0;
            }
            for (int zi = 0; zi < L; zi++)
                for (int yi = 0; yi < L; yi++)
                    for (int xi = 0; xi < L; xi++) {
                        int lev[8];
                        sshex8_micro_nodes(L, xi, yi, zi, lev);
                        for (int i = 0; i < 8; i++) {
                            float acc = 0;
                            for (int j = 0; j < 8; j++) acc += A[i * 8 + j] * eu[lev[j]];
                            ev[lev[i]] += acc;
                        }
                    }
            for (int v = 0; v < nxe; v++) atomic_add_f(&values[idx[v]], ev[v]);
        }
        free(eu);
        free(ev);
        free(idx);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Node-centric (stencil) form: the reference's CPU default                 */
/* ------------------------------------------------------------------------ */

/* Tap tables of the node-centric form, by node class (per axis: 0 = low face, 1 = inside,
 * 2 = high face of the macro element; class = cz*9 + cy*3 + cx): the offsets d of the
 * neighbours a node of that class couples to inside its macro element, and for each the
 * element-matrix entries A[k][k+d] (k over the micro elements of this macro element that
 * contain both nodes) whose sum is the coefficient.  Class 13 (inside) is the 27-point
 * stencil; the other 26 are the partial stencils of the surface. */
typedef struct {
    int ntaps[27];
    int off[27][27][3];
    int pos[27][27];  /* (dz+1)*9 + (dy+1)*3 + (dx+1): the tap's slot in a full 3x3x3 block */
    int nsum[27][27];
    int a[27][27][8];
} stencil_taps_t;

static void stencil_taps(stencil_taps_t *t) {
    memset(t, 0, sizeof(*t));
    for (int cls = 0; cls < 27; cls++) {
        const int c[3] = {cls % 3, (cls / 3) % 3, cls / 9};
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    const int d[3] = {dx, dy, dz};
                    int n = 0, idx[8];
                    for (int k = 0; k < 8; k++) {
                        int ok = 1;
                        for (int ax = 0; ax < 3; ax++) {
                            const int kk = C8[k][ax], jj = kk + d[ax];
                            /* the micro element with the node at corner kk lies inside the macro
                             * element: low face -> corner 0 only, high face -> corner 1 only */
                            if (jj < 0 || jj > 1 || (c[ax] == 0 && kk != 0) || (c[ax] == 2 && kk != 1)) ok = 0;
                        }
                        if (!ok) continue;
                        int j = 0;
                        while (C8[j][0] != C8[k][0] + dx || C8[j][1] != C8[k][1] + dy || C8[j][2] != C8[k][2] + dz) j++;
                        idx[n++] = k * 8 + j;
                    }
                    if (!n) continue;
                    const int q = t->ntaps[cls]++;
                    t->off[cls][q][0] = dx;
                    t->off[cls][q][1] = dy;
                    t->off[cls][q][2] = dz;
                    t->pos[cls][q] = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
                    t->nsum[cls][q] = n;
                    for (int i = 0; i < n; i++) t->a[cls][q][i] = idx[i];
                }
    }
}

static inline int node_class(int L, int i) { return i == 0 ? 0 : (i == L ? 2 : 1); }

/* class of every local node and the tap offsets as local-index differences */
static void stencil_linear_offsets(int L, const stencil_taps_t *T, int *vcls, int offl[27][27]) {
    const int N1 = L + 1;
    for (int zi = 0; zi <= L; zi++)
        for (int yi = 0; yi <= L; yi++)
            for (int xi = 0; xi <= L; xi++)
                vcls[lidx(L, xi, yi, zi)] = node_class(L, zi) * 9 + node_class(L, yi) * 3 + node_class(L, xi);
    for (int cls = 0; cls < 27; cls++)
        for (int q = 0; q < T->ntaps[cls]; q++)
            offl[cls][q] = T->off[cls][q][0] + N1 * (T->off[cls][q][1] + N1 * T->off[cls][q][2]);
}

/* L = 2, 3, 4: one function per node class with every loop bound a compile-time
 * constant (nodes of the class, and its taps dz, dy, dx in that order, the order of the
 * tap tables), so the compiler unrolls them into straight-line code with fixed offsets
 * on the (L+1)^3 micro grid.  c27: the class's coefficients as a full 3x3x3 block indexed
 * (dz+1)*9 + (dy+1)*3 + (dx+1); a tap that does not exist is never read. */
#define OR_LO(LL, c) ((c) == 0 ? 0 : ((c) == 1 ? 1 : (LL)))
#define OR_HI(LL, c) ((c) == 1 ? (LL) - 1 : OR_LO(LL, c))
#define OR_D0(c) ((c) == 0 ? 0 : -1)
#define OR_D1(c) ((c) == 2 ? 0 : 1)
#define OR_CLASS(REAL, P, LL, CX, CY, CZ)                                                                  \
    static inline void P##_##CX##CY##CZ(const REAL *restrict c27, const REAL *restrict in,                \
                                        REAL *restrict out) {                                             \
        enum { N1_ = (LL) + 1, NP_ = N1_ * N1_ };                                                          \
        for (int z = OR_LO(LL, CZ); z <= OR_HI(LL, CZ); z++)                                               \
            for (int y = OR_LO(LL, CY); y <= OR_HI(LL, CY); y++)                                           \
                for (int x = OR_LO(LL, CX); x <= OR_HI(LL, CX); x++) {                                     \
                    REAL acc = 0;                                                                          \
                    for (int dz = OR_D0(CZ); dz <= OR_D1(CZ); dz++)                                        \
                        for (int dy = OR_D0(CY); dy <= OR_D1(CY); dy++)                                    \
                            for (int dx = OR_D0(CX); dx <= OR_D1(CX); dx++)                                \
                                acc += c27[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)] *                       \
                                       in[(z + dz) * NP_ + (y + dy) * N1_ + x + dx];                       \
                    out[z * NP_ + y * N1_ + x] = acc;                                                      \
                }                                                                                          \
    }
#define OR_CLASSES_Z(REAL, P, LL, CZ)                                                                      \
    OR_CLASS(REAL, P, LL, 0, 0, CZ) OR_CLASS(REAL, P, LL, 1, 0, CZ) OR_CLASS(REAL, P, LL, 2, 0, CZ)         \
    OR_CLASS(REAL, P, LL, 0, 1, CZ) OR_CLASS(REAL, P, LL, 1, 1, CZ) OR_CLASS(REAL, P, LL, 2, 1, CZ)         \
    OR_CLASS(REAL, P, LL, 0, 2, CZ) OR_CLASS(REAL, P, LL, 1, 2, CZ) OR_CLASS(REAL, P, LL, 2, 2, CZ)
#define OR_ALL(REAL, P, LL)                                                                                \
    OR_CLASSES_Z(REAL, P, LL, 0) OR_CLASSES_Z(REAL, P, LL, 1) OR_CLASSES_Z(REAL, P, LL, 2)                  \
    static inline void P##_apply(const REAL (*full)[27], const REAL *restrict in, REAL *restrict out) {    \
        P##_000(full[0], in, out);  P##_100(full[1], in, out);  P##_200(full[2], in, out);                 \
        P##_010(full[3], in, out);  P##_110(full[4], in, out);  P##_210(full[5], in, out);                 \
        P##_020(full[6], in, out);  P##_120(full[7], in, out);  P##_220(full[8], in, out);                 \
        P##_001(full[9], in, out);  P##_101(full[10], in, out); P##_201(full[11], in, out);                \
        P##_011(full[12], in, out); P##_111(full[13], in, out); P##_211(full[14], in, out);                \
        P##_021(full[15], in, out); P##_121(full[16], in, out); P##_221(full[17], in, out);                \
        P##_002(full[18], in, out); P##_102(full[19], in, out); P##_202(full[20], in, out);                \
        P##_012(full[21], in, out); P##_112(full[22], in, out); P##_212(full[23], in, out);                \
        P##_022(full[24], in, out); P##_122(full[25], in, out); P##_222(full[26], in, out);                \
    }
OR_ALL(double, or_l2d, 2)
OR_ALL(float, or_l2f, 2)
OR_ALL(double, or_l3d, 3)
OR_ALL(float, or_l3f, 3)
OR_ALL(double, or_l4d, 4)
OR_ALL(float, or_l4f, 4)

/* affine_sshex8_laplacian_stencil_apply_fff (operators/sshex8/sshex8_laplacian.cpp:698-769),
 * values += A u.  Per macro element: sub-FFF = FFF / L (:19-28), element matrix A, the
 * 27-point stencil of A (hex8_matrix_to_stencil, operators/stencil/stencil3.hpp:205)
 * applied at every node strictly inside the macro element (sshex8_stencil,
 * stencil3.hpp:167), the partial stencils of A at its surface nodes (the 26 cases of
 * sshex8_surface_stencil, operators/stencil/sshex8_skeleton_stencil.hpp:1683-1720), then
 * the (L+1)^3 results are added to values with atomics.  Coefficients are built once per
 * macro element and class, as the reference does. */
int or_sshex8_laplacian_stencil_apply(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff,
                                      const double *u, double *values) {
    const int N1 = L + 1, nxe = N1 * N1 * N1;
    stencil_taps_t *T = (stencil_taps_t *)malloc(sizeof(stencil_taps_t));
    stencil_taps(T);
    int *vcls = (int *)malloc(nxe * sizeof(int));
    int offl[27][27];
    stencil_linear_offsets(L, T, vcls, offl);
#pragma omp parallel
    {
        double *eu = (double *)malloc(nxe * sizeof(double));
        double *ev = (double *)malloc(nxe * sizeof(double));
        idx_t *idx = (idx_t *)malloc(nxe * sizeof(idx_t));
        double coef[27][27];
        double full[27][27];
        memset(full, 0, sizeof(full));  /* slots of taps that do not exist stay zero */
#pragma omp for
        for (ptrdiff_t e = 0; e < nelements; e++) {
            double sub[6], A[64];
            const double h = 1.0 / L;
            for (int d = 0; d < 6; d++) sub[d] = (double)fff[e * 6 + d] * h;
            or_hex8_laplacian_matrix(sub, A);
            for (int cls = 0; cls < 27; cls++)
                for (int q = 0; q < T->ntaps[cls]; q++) {
                    double c = 0;
                    for (int i = 0; i < T->nsum[cls][q]; i++) c += A[T->a[cls][q][i]];
                    coef[cls][q] = c;
                    full[cls][T->pos[cls][q]] = c;
                }
            for (int v = 0; v < nxe; v++) {
                idx[v] = elements[v][e];
                eu[v] = u[idx[v]];
            }
            if (L >= 2 && L <= 4) {
                const double(*cf)[27] = (const double(*)[27])full;
                if (L == 4)
                    or_l4d_apply(cf, eu, ev);
                else if (L == 3)
                    or_l3d_apply(cf, eu, ev);
                else
                    or_l2d_apply(cf, eu, ev);
            } else
            /* class by class, rows of nodes along x (the reference's stencil sweeps run
             * along x too); fixed tap counts so the x loop unrolls and vectorises */
            for (int cls = 0; cls < 27; cls++) {
                const int cx = cls % 3, cy = (cls / 3) % 3, cz = cls / 9;
                const int x0 = cx == 0 ? 0 : (cx == 1 ? 1 : L), x1 = cx == 1 ? L - 1 : x0;
                const int y0 = cy == 0 ? 0 : (cy == 1 ? 1 : L), y1 = cy == 1 ? L - 1 : y0;
                const int z0 = cz == 0 ? 0 : (cz == 1 ? 1 : L), z1 = cz == 1 ? L - 1 : z0;
                const int nt = T->ntaps[cls];
                const int *restrict o = offl[cls];
                const double *restrict c = coef[cls];
                const double *restrict xin = eu;
                double *restrict yout = ev;
                for (int zi = z0; zi <= z1; zi++)
                    for (int yi = y0; yi <= y1; yi++) {
                        const int row = lidx(L, 0, yi, zi);
                        switch (nt) {
                            case 27:
                                for (int xi = x0; xi <= x1; xi++) {
                                    double acc = 0;
#pragma GCC unroll 27
                                    for (int q = 0; q < 27; q++) acc += c[q] * xin[row + xi + o[q]];
                                    yout[row + xi] = acc;
                                }
                                break;
                            case 18:
                                for (int xi = x0; xi <= x1; xi++) {
                                    double acc = 0;
#pragma GCC unroll 18
                                    for (int q = 0; q < 18; q++) acc += c[q] * xin[row + xi + o[q]];
                                    yout[row + xi] = acc;
                                }
                                break;
                            case 12:
                                for (int xi = x0; xi <= x1; xi++) {
                                    double acc = 0;
#pragma GCC unroll 12
                                    for (int q = 0; q < 12; q++) acc += c[q] * xin[row + xi + o[q]];
                                    yout[row + xi] = acc;
                                }
                                break;
                            default:
                                for (int xi = x0; xi <= x1; xi++) {
                                    double acc = 0;
                                    for (int q = 0; q < nt; q++) acc += c[q] * xin[row + xi + o[q]];
                                    yout[row + xi] = acc;
                                }
                        }
                    }
            }
            for (int v = 0; v < nxe; v++) atomic_add(&values[idx[v]], ev[v]);
        }
        free(eu);
        free(ev);
        free(idx);
    }
    free(vcls);
    free(T);
    return 0;
}

/* The same stencil apply in the reference's float32 number configuration
 * (real, scalar and accumulator float, cmake/SFEMNumbers.cmake:5-10): element
 * matrix rounded to float, stencil sums, products and sums in float. */
int or_sshex8_laplacian_stencil_apply_f32(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff,
                                          const float *u, float *values) {
    const int N1 = L + 1, nxe = N1 * N1 * N1;
    stencil_taps_t *T = (stencil_taps_t *)malloc(sizeof(stencil_taps_t));
    stencil_taps(T);
    int *vcls = (int *)malloc(nxe * sizeof(int));
    int offl[27][27];
    stencil_linear_offsets(L, T, vcls, offl);
#pragma omp parallel
    {
        float *eu = (float *)malloc(nxe * sizeof(float));
        float *ev = (float *)malloc(nxe * sizeof(float));
        idx_t *idx = (idx_t *)malloc(nxe * sizeof(idx_t));
        float coef[27][27];
        float full[27][27];
        memset(full, 0, sizeof(full));  /* slots of taps that do not exist stay zero */
#pragma omp for
        for (ptrdiff_t e = 0; e < nelements; e++) {
            double sub[6], Ad[64];
            float A[64];
            const float h = 1.0f / (float)L;
            for (int d = 0; d < 6; d++) sub[d] = (double)(fff[e * 6 + d] * h);
            or_hex8_laplacian_matrix(sub, Ad);
            for (int k = 0; k < 64; k++) A[k] = (float)Ad[k];
            for (int cls = 0; cls < 27; cls++)
                for (int q = 0; q < T->ntaps[cls]; q++) {
                    float c = 0;
                    for (int i = 0; i < T->nsum[cls][q]; i++) c += A[T->a[cls][q][i]];
                    coef[cls][q] = c;
                    full[cls][T->pos[cls][q]] = c;
                }
            for (int v = 0; v < nxe; v++) {
                idx[v] = elements[v][e];
                eu[v] = u[idx[v]];
            }
            if (L >= 2 && L <= 4) {
                const float(*cf)[27] = (const float(*)[27])full;
                if (L == 4)
                    or_l4f_apply(cf, eu, ev);
                else if (L == 3)
                    or_l3f_apply(cf, eu, ev);
                else
                    or_l2f_apply(cf, eu, ev);
            } else
            /* class by class, rows of nodes along x (the reference's stencil sweeps run
             * along x too); fixed tap counts so the x loop unrolls and vectorises */
            for (int cls = 0; cls < 27; cls++) {
                const int cx = cls % 3, cy = (cls / 3) % 3, cz = cls / 9;
                const int x0 = cx == 0 ? 0 : (cx == 1 ? 1 : L), x1 = cx == 1 ? L - 1 : x0;
                const int y0 = cy == 0 ? 0 : (cy == 1 ? 1 : L), y1 = cy == 1 ? L - 1 : y0;
                const int z0 = cz == 0 ? 0 : (cz == 1 ? 1 : L), z1 = cz == 1 ? L - 1 : z0;
                const int nt = T->ntaps[cls];
                const int *restrict o = offl[cls];
                const float *restrict c = coef[cls];
                const float *restrict xin = eu;
                float *restrict yout = ev;
                for (int zi = z0; zi <= z1; zi++)
                    for (int yi = y0; yi <= y1; yi++) {
                        const int row = lidx(L, 0, yi, zi);
                        switch (nt) {
                            case 27:
                                for (int xi = x0; xi <= x1; xi++) {
                                    float acc = 0;
#pragma GCC unroll 27
                                    for (int q = 0; q < 27; q++) acc += c[q] * xin[row + xi + o[q]];
                                    yout[row + xi] = acc;
                                }
                                break;
                            case 18:
                                for (int xi = x0; xi <= x1; xi++) {
                                    float acc = 0;
#pragma GCC unroll 18
                                    for (int q = 0; q < 18; q++) acc += c[q] * xin[row + xi + o[q]];
                                    yout[row + xi] = acc;
                                }
                                break;
                            case 12:
                                for (int xi = x0; xi <= x1; xi++) {
                                    float acc = 0;
#pragma GCC unroll 12
                                    for (int q = 0; q < 12; q++) acc += c[q] * xin[row + xi + o[q]];
                                    yout[row + xi] = acc;
                                }
                                break;
                            default:
                                for (int xi = x0; xi <= x1; xi++) {
                                    float acc = 0;
                                    for (int q = 0; q < nt; q++) acc += c[q] * xin[row + xi + o[q]];
                                    yout[row + xi] = acc;
                                }
                        }
                    }
            }
            for (int v = 0; v < nxe; v++) atomic_add_f(&values[idx[v]], ev[v]);
        }
        free(eu);
        free(ev);
        free(idx);
    }
    free(vcls);
    free(T);
    return 0;
}

/* hex8_laplacian_apply_opt (operators/hex8/hex8_laplacian.cpp:309-345);
 * elements in hex8 corner order. */
int or_hex8_laplacian_apply(ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff, const double *u,
                            double *values) {
#pragma omp parallel for
    for (ptrdiff_t e = 0; e < nelements; e++) {
        double f[6], A[64], eu[8];
        for (int d = 0; d < 6; d++) f[d] = fff[e * 6 + d];
        or_hex8_laplacian_matrix(f, A);
        for (int v = 0; v < 8; v++) eu[v] = u[elements[v][e]];
        for (int i = 0; i < 8; i++) {
            double acc = 0;
            for (int j = 0; j < 8; j++) acc += A[i * 8 + j] * eu[j];
            atomic_add(&values[elements[i][e]], acc);
        }
    }
    return 0;
}

/* affine_sshex8_laplacian_diag (operators/sshex8/sshex8_laplacian.cpp:333-435)
 * and hex8_laplacian_diag (operators/hex8/hex8_laplacian.cpp:262-307), from
 * the cached FFF.  L == 0 selects the plain hex8 corner ordering. */
int or_laplacian_diag(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff, double *diag) {
    const int Lm = L > 0 ? L : 1;
#pragma omp parallel for
    for (ptrdiff_t e = 0; e < nelements; e++) {
        double sub[6], A[64];
        for (int d = 0; d < 6; d++) sub[d] = (double)fff[e * 6 + d] / Lm;
        or_hex8_laplacian_matrix(sub, A);
        if (L == 0) {
            for (int i = 0; i < 8; i++) atomic_add(&diag[elements[i][e]], A[i * 9]);
            continue;
        }
        for (int zi = 0; zi < L; zi++)
            for (int yi = 0; yi < L; yi++)
                for (int xi = 0; xi < L; xi++) {
                    int lev[8];
                    sshex8_micro_nodes(L, xi, yi, zi, lev);
                    for (int i = 0; i < 8; i++) atomic_add(&diag[elements[lev[i]][e]], A[i * 9]);
                }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Linear elasticity                                                        */
/* ------------------------------------------------------------------------ */

/* 24x24 element matrix, row/col index = component*8 + node, from the
 * (sub-)adjugate and determinant (operators/hex8/hex8_linear_elasticity_inline_cpu.hpp:207).
 * K[(a,i),(b,j)] = int mu (grad phi_a . grad phi_b) delta_ij + mu d_j phi_a d_i phi_b
 *                      + lambda d_i phi_a d_j phi_b  dx,  grad phi = adj^T grad_ref phi / det. */
void or_hex8_linear_elasticity_matrix(double mu, double lambda, const double adj[9], double det, double K[576]) {
    ensure_tables();
    double AA[3][3];
    for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += adj[3 * p + k] * adj[3 * q + k];
            AA[p][q] = s;
        }
    const double inv_det = 1.0 / det;
    for (int i = 0; i < 3; i++)
        for (int a = 0; a < 8; a++)
            for (int j = 0; j < 3; j++)
                for (int b = 0; b < 8; b++) {
                    double s = 0;
                    for (int p = 0; p < 3; p++)
                        for (int q = 0; q < 3; q++) {
                            const double I = I_table[a][b][p][q];
                            double w = mu * adj[3 * p + j] * adj[3 * q + i] + lambda * adj[3 * p + i] * adj[3 * q + j];
                            if (i == j) w += mu * AA[p][q];
                            s += I * w;
                        }
                    K[(i * 8 + a) * 24 + (j * 8 + b)] = s * inv_det;
                }
}

static void sub_adjugate(const jacobian_t *adjugate, const jacobian_t *determinant, ptrdiff_t e, int L, double adj[9],
                         double *det) {
    const double h = 1.0 / L;
    for (int d = 0; d < 9; d++) adj[d] = (double)adjugate[e * 9 + d] * (h * h);
    *det = (double)determinant[e] * (h * h * h);
}

/* affine_sshex8_linear_elasticity_apply_macro_adjugate (operators/sshex8/sshex8_linear_elasticity.cpp:275-424):
 * sub-adjugate = adj h^2, sub-det = det h^3 (operators/sshex8/sshex8.hpp:26-42);
 * u and out are interleaved with stride 3 (ux = u, uy = u+1, uz = u+2).
 * L == 0 selects a plain hex8 mesh (affine_hex8_linear_elasticity_apply_adjugate,
 * operators/hex8/hex8_linear_elasticity.cpp:458). */
static int linear_elasticity_apply_impl(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *adjugate,
                                        const jacobian_t *determinant, double mu, double lambda, const double *u,
                                        double *out, int absolute);

int or_linear_elasticity_apply(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *adjugate,
                               const jacobian_t *determinant, double mu, double lambda, const double *u, double *out) {
    return linear_elasticity_apply_impl(L, nelements, elements, adjugate, determinant, mu, lambda, u, out, 0);
}

/* out += |K| u with every element-matrix entry replaced by its magnitude: with u = |x|
 * this is the row scale sum_j |K_ij| |x_j| (summed element by element, so an upper
 * bound of the assembled one) that floating-point parity is measured against. */
int or_linear_elasticity_apply_abs(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *adjugate,
                                   const jacobian_t *determinant, double mu, double lambda, const double *u,
                                   double *out) {
    return linear_elasticity_apply_impl(L, nelements, elements, adjugate, determinant, mu, lambda, u, out, 1);
}

static int linear_elasticity_apply_impl(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *adjugate,
                                        const jacobian_t *determinant, double mu, double lambda, const double *u,
                                        double *out, int absolute) {
    const int Lm = L > 0 ? L : 1;
    const int nxe = (Lm + 1) * (Lm + 1) * (Lm + 1);
#pragma omp parallel
    {
        double *eu = (double *)malloc(3 * nxe * sizeof(double));
        double *ev = (double *)malloc(3 * nxe * sizeof(double));
        idx_t *idx = (idx_t *)malloc(nxe * sizeof(idx_t));
        double *K = (double *)malloc(576 * sizeof(double));
#pragma omp for
        for (ptrdiff_t e = 0; e < nelements; e++) {
            double adj[9], det;
            sub_adjugate(adjugate, determinant, e, Lm, adj, &det);
            or_hex8_linear_elasticity_matrix(mu, lambda, adj, det, K);
            if (absolute)
                for (int k = 0; k < 576; k++) K[k] = fabs(K[k]);
            if (L == 0) {
                double ue[24], oe[24];
                for (int v = 0; v < 8; v++)
                    for (int d = 0; d < 3; d++) ue[d * 8 + v] = u[3 * (ptrdiff_t)elements[v][e] + d];
                for (int i = 0; i < 24; i++) {
                    double s = 0;
                    for (int j = 0; j < 24; j++) s += K[i * 24 + j] * ue[j];
                    oe[i] = s;
                }
                for (int v = 0; v < 8; v++)
                    for (int d = 0; d < 3; d++) atomic_add(&out[3 * (ptrdiff_t)elements[v][e] + d], oe[d * 8 + v]);
                continue;
            }
            for (int v = 0; v < nxe; v++) {
                idx[v] = elements[v][e];
                for (int d = 0; d < 3; d++) {
                    eu[d * nxe + v] = u[3 * (ptrdiff_t)idx[v] + d];
                    ev[d * nxe + v] = 0;
                }
            }
            for (int zi = 0; zi < L; zi++)
                for (int yi = 0; yi < L; yi++)
                    for (int xi = 0; xi < L; xi++) {
                        int lev[8];
                        double ue[24];
                        sshex8_micro_nodes(L, xi, yi, zi, lev);
                        for (int d = 0; d < 3; d++)
                            for (int v = 0; v < 8; v++) ue[d * 8 + v] = eu[d * nxe + lev[v]];
                        for (int i = 0; i < 24; i++) {
                            double s = 0;
                            for (int j = 0; j < 24; j++) s += K[i * 24 + j] * ue[j];
                            ev[(i / 8) * nxe + lev[i % 8]] += s;
                        }
                    }
            for (int v = 0; v < nxe; v++)
                for (int d = 0; d < 3; d++) atomic_add(&out[3 * (ptrdiff_t)idx[v] + d], ev[d * nxe + v]);
        }
        free(eu);
        free(ev);
        free(idx);
        free(K);
    }
    return 0;
}

/* Diagonal (3 per node, interleaved) and symmetric 3x3 block diagonal
 * (6 per node: 00,01,02,11,12,22, interleaved)
 * (operators/sshex8/sshex8_linear_elasticity.cpp:971-1257). L == 0: plain hex8. */
int or_linear_elasticity_block_diag_sym(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *adjugate,
                                        const jacobian_t *determinant, double mu, double lambda, double *diag3,
                                        double *block6) {
    const int Lm = L > 0 ? L : 1;
    static const int bi[6] = {0, 0, 0, 1, 1, 2}, bj[6] = {0, 1, 2, 1, 2, 2};
#pragma omp parallel
    {
        double *K = (double *)malloc(576 * sizeof(double));
#pragma omp for
        for (ptrdiff_t e = 0; e < nelements; e++) {
            double adj[9], det;
            sub_adjugate(adjugate, determinant, e, Lm, adj, &det);
            or_hex8_linear_elasticity_matrix(mu, lambda, adj, det, K);
            const int nmicro = L > 0 ? L * L * L : 1;
            for (int m = 0; m < nmicro; m++) {
                int lev[8];
                if (L > 0) {
                    const int xi = m % L, yi = (m / L) % L, zi = m / (L * L);
                    sshex8_micro_nodes(L, xi, yi, zi, lev);
                } else {
                    for (int v = 0; v < 8; v++) lev[v] = v;
                }
                for (int a = 0; a < 8; a++) {
                    const ptrdiff_t n = elements[lev[a]][e];
                    if (diag3)
                        for (int d = 0; d < 3; d++) atomic_add(&diag3[3 * n + d], K[(d * 8 + a) * 24 + d * 8 + a]);
                    if (block6)
                        for (int k = 0; k < 6; k++)
                            atomic_add(&block6[6 * n + k], K[(bi[k] * 8 + a) * 24 + bj[k] * 8 + a]);
                }
            }
        }
        free(K);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Transfer operators                                                       */
/* ------------------------------------------------------------------------ */

/* sshex8_element_node_incidence_count (operators/sshex8/sshex8_interpolate.cpp:239-257) */
int or_incidence_count(int L, ptrdiff_t nelements, idx_t **elements, uint16_t *count) {
    const int nxe = (L + 1) * (L + 1) * (L + 1);
    for (int v = 0; v < nxe; v++)
        for (ptrdiff_t e = 0; e < nelements; e++) count[elements[v][e]]++;
    return 0;
}

/* Nested prolongation, to = P from (overwrite), trilinear in each macro element
 * (sshex8_prolongate, operators/sshex8/sshex8_interpolate.cpp:259-558; with
 * from_level == 1 and the macro corners of to_elements this is
 * sshex8_hierarchical_prolongation, :129-237).  vec_size components interleaved. */
int or_sshex8_prolongate(ptrdiff_t nelements, int from_level, idx_t **from_elements, int to_level,
                         idx_t **to_elements, int vec_size, const double *from, double *to) {
    if (to_level % from_level) return 1;
    const int s = to_level / from_level;
#pragma omp parallel for
    for (ptrdiff_t e = 0; e < nelements; e++) {
        for (int zi = 0; zi <= to_level; zi++)
            for (int yi = 0; yi <= to_level; yi++)
                for (int xi = 0; xi <= to_level; xi++) {
                    const int cx = xi / s < from_level ? xi / s : from_level - 1;
                    const int cy = yi / s < from_level ? yi / s : from_level - 1;
                    const int cz = zi / s < from_level ? zi / s : from_level - 1;
                    const double tx = (double)(xi - cx * s) / s, ty = (double)(yi - cy * s) / s,
                                 tz = (double)(zi - cz * s) / s;
                    const ptrdiff_t gid = to_elements[lidx(to_level, xi, yi, zi)][e];
                    for (int d = 0; d < vec_size; d++) {
                        double acc = 0;
                        for (int c = 0; c < 8; c++) {
                            const double w = (C8[c][0] ? tx : 1 - tx) * (C8[c][1] ? ty : 1 - ty) * (C8[c][2] ? tz : 1 - tz);
                            if (w == 0) continue;
                            const ptrdiff_t src =
                                    from_elements[lidx(from_level, cx + C8[c][0], cy + C8[c][1], cz + C8[c][2])][e];
                            acc += w * from[src * vec_size + d];
                        }
                        to[gid * vec_size + d] = acc;
                    }
                }
    }
    return 0;
}

/* Restriction R = P^T with the fine input divided by the element-node incidence
 * count (sshex8_restrict, operators/sshex8/sshex8_interpolate.cpp:633-760;
 * sshex8_hierarchical_restriction, :12-127).  to += R from. */
int or_sshex8_restrict(ptrdiff_t nelements, int from_level, idx_t **from_elements, const uint16_t *count,
                       int to_level, idx_t **to_elements, int vec_size, const double *from, double *to) {
    if (from_level % to_level) return 1;
    const int s = from_level / to_level;
#pragma omp parallel for
    for (ptrdiff_t e = 0; e < nelements; e++) {
        for (int zi = 0; zi <= from_level; zi++)
            for (int yi = 0; yi <= from_level; yi++)
                for (int xi = 0; xi <= from_level; xi++) {
                    const int cx = xi / s < to_level ? xi / s : to_level - 1;
                    const int cy = yi / s < to_level ? yi / s : to_level - 1;
                    const int cz = zi / s < to_level ? zi / s : to_level - 1;
                    const double tx = (double)(xi - cx * s) / s, ty = (double)(yi - cy * s) / s,
                                 tz = (double)(zi - cz * s) / s;
                    const ptrdiff_t gid = from_elements[lidx(from_level, xi, yi, zi)][e];
                    for (int d = 0; d < vec_size; d++) {
                        const double val = from[gid * vec_size + d] / count[gid];
                        for (int c = 0; c < 8; c++) {
                            const double w = (C8[c][0] ? tx : 1 - tx) * (C8[c][1] ? ty : 1 - ty) * (C8[c][2] ? tz : 1 - tz);
                            if (w == 0) continue;
                            const ptrdiff_t dst = to_elements[lidx(to_level, cx + C8[c][0], cy + C8[c][1], cz + C8[c][2])][e];
                            atomic_add(&to[dst * vec_size + d], w * val);
                        }
                    }
                }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Symmetric sparse formats                                                 */
/* ------------------------------------------------------------------------ */

/* y = (D + U + U^T) x with D the diagonal and U the strict upper triangle in
 * CRS (CRSSymSpMV, algebra/sfem_crs_sym_SpMV.hpp:8-91).  y is overwritten. */
int or_crs_sym_spmv(ptrdiff_t n, const idx_t *rowptr, const idx_t *colidx, const double *diag, const double *offdiag,
                    const double *x, double *y) {
    for (ptrdiff_t i = 0; i < n; i++) y[i] = diag[i] * x[i];
    for (ptrdiff_t i = 0; i < n; i++)
        for (idx_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
            const idx_t j = colidx[k];
            y[i] += offdiag[k] * x[j];
            y[j] += offdiag[k] * x[i];
        }
    return 0;
}

/* Symmetric block CRS, block size bs: diagonal blocks stored as the bs(bs+1)/2
 * upper entries per row, off-diagonal blocks (strict upper) full bs*bs row-major
 * (BCRSSymSpMV, algebra/sfem_bcrs_sym_SpMV.hpp:9-279; values are kept AoS here). */
int or_bsr_sym_spmv(ptrdiff_t nb, int bs, const idx_t *rowptr, const idx_t *colidx, const double *diag_sym,
                    const double *offdiag, const double *x, double *y) {
    const int nsym = bs * (bs + 1) / 2;
    for (ptrdiff_t i = 0; i < nb; i++) {
        const double *D = &diag_sym[i * nsym];
        int k = 0;
        double Df[16];
        for (int a = 0; a < bs; a++)
            for (int b = a; b < bs; b++, k++) {
                Df[a * bs + b] = D[k];
                Df[b * bs + a] = D[k];
            }
        for (int a = 0; a < bs; a++) {
            double s = 0;
            for (int b = 0; b < bs; b++) s += Df[a * bs + b] * x[i * bs + b];
            y[i * bs + a] = s;
        }
    }
    for (ptrdiff_t i = 0; i < nb; i++)
        for (idx_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
            const idx_t j = colidx[k];
            const double *B = &offdiag[(ptrdiff_t)k * bs * bs];
            for (int a = 0; a < bs; a++)
                for (int b = 0; b < bs; b++) {
                    y[i * bs + a] += B[a * bs + b] * x[j * bs + b];
                    y[j * bs + b] += B[a * bs + b] * x[i * bs + a];
                }
        }
    return 0;
}

/* Symmetric CRS assembly of the hex8 Laplacian from the FFF cache: diag and
 * strict upper triangle on a given graph (hex8_laplacian_crs_sym,
 * operators/hex8/hex8_laplacian.cpp:148-221).  rowptr/colidx hold only the
 * strict upper part (col > row), sorted. */
int or_hex8_laplacian_crs_sym(ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff, const idx_t *rowptr,
                              const idx_t *colidx, double *diag, double *offdiag) {
#pragma omp parallel for
    for (ptrdiff_t e = 0; e < nelements; e++) {
        double f[6], A[64];
        idx_t ev[8];
        for (int d = 0; d < 6; d++) f[d] = fff[e * 6 + d];
        or_hex8_laplacian_matrix(f, A);
        for (int v = 0; v < 8; v++) ev[v] = elements[v][e];
        for (int i = 0; i < 8; i++) {
            atomic_add(&diag[ev[i]], A[i * 9]);
            for (int j = 0; j < 8; j++) {
                if (ev[j] <= ev[i]) continue;
                for (idx_t k = rowptr[ev[i]]; k < rowptr[ev[i] + 1]; k++)
                    if (colidx[k] == ev[j]) {
                        atomic_add(&offdiag[k], A[i * 8 + j]);
                        break;
                    }
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Learned smoother network (no reference counterpart): 3x3x3 convolutions  */
/* on 5x5x5 patches, zero padding, channels-last activations [p][v][c],      */
/* weights [co][ci][27] with offset o = (dz+1)*9 + (dy+1)*3 + (dx+1).        */
/* Plain loop nests in double for gradient checks of the GPU kernels.        */
/* ------------------------------------------------------------------------ */

static int pc_neighbor(int v, int o) {
    const int x = v % 5, y = (v / 5) % 5, z = v / 25;
    const int X = x + o % 3 - 1, Y = y + (o / 3) % 3 - 1, Z = z + o / 9 - 1;
    if (X < 0 || X > 4 || Y < 0 || Y > 4 || Z < 0 || Z > 4) return -1;
    return Z * 25 + Y * 5 + X;
}

void or_patchconv_forward(ptrdiff_t P, int cin, int cout, const float *in, const float *W, int relu, double *out) {
#pragma omp parallel for
    for (ptrdiff_t p = 0; p < P; p++)
        for (int v = 0; v < 125; v++)
            for (int co = 0; co < cout; co++) {
                double acc = 0;
                for (int o = 0; o < 27; o++) {
                    const int u = pc_neighbor(v, o);
                    if (u < 0) continue;
                    for (int ci = 0; ci < cin; ci++)
                        acc += (double)W[(co * cin + ci) * 27 + o] * in[(p * 125 + u) * cin + ci];
                }
                out[(p * 125 + v) * cout + co] = relu && acc < 0 ? 0 : acc;
            }
}

void or_patchconv_backward_data(ptrdiff_t P, int cin, int cout, const float *gout, const float *W, const float *in_act,
                                double *gin) {
#pragma omp parallel for
    for (ptrdiff_t p = 0; p < P; p++)
        for (int u = 0; u < 125; u++)
            for (int ci = 0; ci < cin; ci++) {
                double acc = 0;
                for (int o = 0; o < 27; o++) {
                    /* u = v + o  <=>  v = u - o: the neighbour of u at the mirrored offset */
                    const int v = pc_neighbor(u, 26 - o);
                    if (v < 0) continue;
                    for (int co = 0; co < cout; co++) acc += (double)W[(co * cin + ci) * 27 + o] * gout[(p * 125 + v) * cout + co];
                }
                if (in_act && in_act[(p * 125 + u) * cin + ci] <= 0) acc = 0;
                gin[(p * 125 + u) * cin + ci] = acc;
            }
}

void or_patchconv_backward_weights(ptrdiff_t P, int cin, int cout, const float *gout, const float *in, double *dW) {
    for (int co = 0; co < cout; co++)
        for (int ci = 0; ci < cin; ci++)
            for (int o = 0; o < 27; o++) {
                double acc = 0;
#pragma omp parallel for reduction(+ : acc)
                for (ptrdiff_t p = 0; p < P; p++)
                    for (int v = 0; v < 125; v++) {
                        const int u = pc_neighbor(v, o);
                        if (u < 0) continue;
                        acc += (double)gout[(p * 125 + v) * cout + co] * in[(p * 125 + u) * cin + ci];
                    }
                dW[(co * cin + ci) * 27 + o] += acc;
            }
}

/* ------------------------------------------------------------------------ */
/* Compensated (double-double) residuals                                    */
/* ------------------------------------------------------------------------ */

/* Error-free transformations (Knuth's TwoSum; TwoProduct with a fused multiply-add):
 * a + b = s + e and a * b = p + e exactly. */
static inline void two_sum(double a, double b, double *s, double *e) {
    const double x = a + b, bb = x - a;
    *s = x;
    *e = (a - (x - bb)) + (b - bb);
}
static inline void dd_add(double *hi, double *lo, double v) {
    double s, e;
    two_sum(*hi, v, &s, &e);
    *hi = s;
    *lo += e;
}
static inline void dd_fma(double *hi, double *lo, double a, double b) {
    const double p = a * b, pe = fma(a, b, -p);
    dd_add(hi, lo, p);
    *lo += pe;
}

/* r = b - A x with the products and sums of A x carried in double-double: the
 * residual of the FP64 operator (element matrices in double, as the apply) evaluated
 * to about 1e-30 relative to |A||x| instead of 1e-16, so residuals far below the
 * plain-FP64 evaluation floor can be measured.  Element contributions are formed in
 * parallel and summed node by node in element order.  kind 0: sshex8 Laplacian from
 * the FFF (L >= 2), kind 1: linear elasticity (3 interleaved components; L = 0 plain
 * hex8).  Rows of the constrained dofs are left to the caller. */
static int residual_dd(int kind, int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *geom,
                       const jacobian_t *det, double mu, double lambda, const double *em, const double *x,
                       const double *x_lo, const double *b, ptrdiff_t ndofs, double *r) {
    const int bs = kind == 1 ? 3 : 1;
    const int Lm = L > 0 ? L : 1;
    const int nxe = L > 0 ? (L + 1) * (L + 1) * (L + 1) : 8;
    const int nloc = nxe * bs;
    double *buf = (double *)malloc((size_t)nelements * nloc * 2 * sizeof(double));
    if (!buf) return 1;
#pragma omp parallel
    {
        double *K = (double *)malloc(576 * sizeof(double));
#pragma omp for
        for (ptrdiff_t e = 0; e < nelements; e++) {
            double *hi = buf + (size_t)e * nloc * 2, *lo = hi + nloc;
            for (int i = 0; i < nloc; i++) hi[i] = lo[i] = 0;
            const int ne = kind == 1 ? 24 : 8;
            if (em) {
                memcpy(K, em + (size_t)e * ne * ne, (size_t)ne * ne * sizeof(double));
            } else if (kind == 0) {
                double sub[6];
                for (int d = 0; d < 6; d++) sub[d] = (double)geom[e * 6 + d] * (1.0 / Lm);
                or_hex8_laplacian_matrix(sub, K);
            } else {
                double adj[9], dt;
                sub_adjugate(geom, det, e, Lm, adj, &dt);
                or_hex8_linear_elasticity_matrix(mu, lambda, adj, dt, K);
            }
            for (int zi = 0; zi < Lm; zi++)
                for (int yi = 0; yi < Lm; yi++)
                    for (int xi = 0; xi < Lm; xi++) {
                        int lev[8];
                        if (L > 0)
                            sshex8_micro_nodes(L, xi, yi, zi, lev);
                        else
                            for (int c = 0; c < 8; c++) lev[c] = c;
                        double ue[24], ul[24];
                        for (int c = 0; c < 8; c++)
                            for (int d = 0; d < bs; d++) {
                                const ptrdiff_t q = (ptrdiff_t)elements[lev[c]][e] * bs + d;
                                ue[d * 8 + c] = x[q];
                                ul[d * 8 + c] = x_lo ? x_lo[q] : 0.0;
                            }
                        for (int i = 0; i < ne; i++) {
                            double h = 0, l = 0;
                            for (int j = 0; j < ne; j++) {
                                dd_fma(&h, &l, K[i * ne + j], ue[j]);
                                l = fma(K[i * ne + j], ul[j], l);
                            }
                            const int slot = lev[i % 8] * bs + i / 8;
                            dd_add(&hi[slot], &lo[slot], h);
                            lo[slot] += l;
                        }
                    }
        }
        free(K);
    }
    double *ahi = (double *)calloc(ndofs, sizeof(double)), *alo = (double *)calloc(ndofs, sizeof(double));
    for (ptrdiff_t e = 0; e < nelements; e++) {
        const double *hi = buf + (size_t)e * nloc * 2, *lo = hi + nloc;
        for (int v = 0; v < nxe; v++) {
            const ptrdiff_t g = elements[v][e];
            for (int d = 0; d < bs; d++) {
                dd_add(&ahi[g * bs + d], &alo[g * bs + d], hi[v * bs + d]);
                alo[g * bs + d] += lo[v * bs + d];
            }
        }
    }
#pragma omp parallel for
    for (ptrdiff_t i = 0; i < ndofs; i++) {
        double h = b[i], l = 0;
        dd_add(&h, &l, -ahi[i]);
        l -= alo[i];
        r[i] = h + l;
    }
    free(ahi);
    free(alo);
    free(buf);
    return 0;
}

int or_sshex8_laplacian_residual_dd(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff,
                                    const double *x, const double *b, ptrdiff_t n, double *r) {
    return residual_dd(0, L, nelements, elements, fff, NULL, 0, 0, NULL, x, NULL, b, n, r);
}

int or_linear_elasticity_residual_dd(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *adjugate,
                                     const jacobian_t *determinant, double mu, double lambda, const double *x,
                                     const double *b, ptrdiff_t ndofs, double *r) {
    return residual_dd(1, L, nelements, elements, adjugate, determinant, mu, lambda, NULL, x, NULL, b, ndofs, r);
}

/* The same from given micro element matrices em[e][(8 bs)^2] (bs 1: kind 0, bs 3: kind 1)
 * and a solution given as x + x_lo (x_lo may be NULL). */
int or_residual_dd_em(int bs, int L, ptrdiff_t nelements, idx_t **elements, const double *em, const double *x,
                      const double *x_lo, const double *b, ptrdiff_t ndofs, double *r) {
    return residual_dd(bs == 3 ? 1 : 0, L, nelements, elements, NULL, NULL, 0, 0, em, x, x_lo, b, ndofs, r);
}

/* ------------------------------------------------------------------------ */
/* Non-affine sshex8 Laplacian                                               */
/* ------------------------------------------------------------------------ */

/* sshex8_laplacian_apply (operators/sshex8/sshex8_laplacian.cpp:39-182), values += A u
 * for macro elements whose geometry is the trilinear map of their 8 corner nodes.
 * Per micro element (xi, yi, zi): the six-point rule at the face centres of the micro
 * reference cube, weights 1/6 (q6, operators/hex8/hex8_quadrature.hpp:4-15); at each
 * point the FFF of the macro map at the macro coordinates ((xi, yi, zi) + q) / L, scaled
 * by h = 1/L to the micro element (hex8_sub_fff_0, :19-28), and
 * v_i += w grad phi_i(q) . (G grad u(q)) (what hex8_laplacian_apply_fff evaluates,
 * operators/hex8/hex8_laplacian_inline_cpu.hpp:6). */
static const double OR_Q6[6][3] = {{0.0, 0.5, 0.5}, {0.5, 0.0, 0.5}, {0.5, 0.5, 0.0},
                                   {0.5, 0.5, 1.0}, {0.5, 1.0, 0.5}, {1.0, 0.5, 0.5}};

int or_sshex8_laplacian_apply_nonaffine(int L, ptrdiff_t nelements, idx_t **elements, geom_t **points,
                                        const double *u, double *values) {
    if (L < 1 || L > 16) return -1;
    const int N1 = L + 1, nxe = N1 * N1 * N1;
#pragma omp parallel
    {
        double *eu = (double *)malloc(nxe * sizeof(double));
        double *ev = (double *)malloc(nxe * sizeof(double));
        idx_t *idx = (idx_t *)malloc(nxe * sizeof(idx_t));
#pragma omp for
        for (ptrdiff_t e = 0; e < nelements; e++) {
            double x[8], y[8], z[8];
            for (int c = 0; c < 8; c++) {
                const idx_t n = elements[lidx(L, C8[c][0] * L, C8[c][1] * L, C8[c][2] * L)][e];
                x[c] = points[0][n];
                y[c] = points[1][n];
                z[c] = points[2][n];
            }
            for (int v = 0; v < nxe; v++) {
                idx[v] = elements[v][e];
                eu[v] = u[idx[v]];
                ev[v] = 0;
            }
            const double h = 1.0 / L;
            for (int zi = 0; zi < L; zi++)
                for (int yi = 0; yi < L; yi++)
                    for (int xi = 0; xi < L; xi++) {
                        int lev[8];
                        double ue[8], ve[8] = {0};
                        for (int c = 0; c < 8; c++) {
                            lev[c] = lidx(L, xi + C8[c][0], yi + C8[c][1], zi + C8[c][2]);
                            ue[c] = eu[lev[c]];
                        }
                        for (int k = 0; k < 6; k++) {
                            double J[3][3], f[6], dphi[8][3], gu[3] = {0, 0, 0}, t[3];
                            hex8_jacobian(x, y, z, h * (xi + OR_Q6[k][0]), h * (yi + OR_Q6[k][1]),
                                          h * (zi + OR_Q6[k][2]), J);
                            fff_from_jacobian(J, f);
                            const double G[3][3] = {{f[0] * h, f[1] * h, f[2] * h},
                                                    {f[1] * h, f[3] * h, f[4] * h},
                                                    {f[2] * h, f[4] * h, f[5] * h}};
                            for (int c = 0; c < 8; c++) {
                                double w[3], dw[3];
                                for (int d = 0; d < 3; d++) {
                                    w[d] = C8[c][d] ? OR_Q6[k][d] : 1 - OR_Q6[k][d];
                                    dw[d] = C8[c][d] ? 1.0 : -1.0;
                                }
                                dphi[c][0] = dw[0] * w[1] * w[2];
                                dphi[c][1] = w[0] * dw[1] * w[2];
                                dphi[c][2] = w[0] * w[1] * dw[2];
                                for (int p = 0; p < 3; p++) gu[p] += dphi[c][p] * ue[c];
                            }
                            for (int p = 0; p < 3; p++) t[p] = (G[p][0] * gu[0] + G[p][1] * gu[1] + G[p][2] * gu[2]) / 6.0;
                            for (int c = 0; c < 8; c++) ve[c] += dphi[c][0] * t[0] + dphi[c][1] * t[1] + dphi[c][2] * t[2];
                        }
                        for (int c = 0; c < 8; c++) ev[lev[c]] += ve[c];
                    }
            for (int v = 0; v < nxe; v++) atomic_add(&values[idx[v]], ev[v]);
        }
        free(eu);
        free(ev);
        free(idx);
    }
    return 0;
}
