/*
 * CPU oracle: multigrid-preconditioned CG on the sshex8 hierarchy, a plain-C
 * (OpenMP) restatement of the reference's solver templates.  TEST INFRASTRUCTURE
 * ONLY: it gives the FP64 reference solution the GPU solves are compared with and
 * the CPU solve time the benchmark reports beside them.
 *
 *   ConjugateGradient::apply        algebra/sfem_cg.hpp:200-443 (preconditioned form)
 *   Multigrid::cycle (V-cycle)      algebra/sfem_Multigrid.hpp:242-346
 *   Chebyshev3::precond_apply       algebra/sfem_Chebyshev3.hpp:183-242 (lambda_min =
 *                                   0.06 lambda_max, lambda_max from the power method
 *                                   algebra/sfem_PowerMethod.hpp:18-55, scaled by 1.02)
 *   coarse solve                    Jacobi-preconditioned CG to a relative tolerance
 *                                   (1e-8 in drivers/mgsolve.cpp:210-222, 1e-6 in the
 *                                   default geometric multigrid,
 *                                   algebra/mg/sfem_GeometricMultigrid.cpp:149-163); no
 *                                   absolute tolerance (mgsolve's atol 1e-10 assumes its
 *                                   right-hand-side scale and would stop the coarse solves of
 *                                   small residuals after a few iterations)
 *   Dirichlet rows                  identity rows in the operator, zero constraints on the
 *                                   restricted residual and the prolongated correction
 *                                   (frontend/sfem_Function.cpp:481-586)
 *
 * The hierarchy is the sshex8 derefinement (L, L/2, ..., 1) on one macro mesh with
 * nested transfers (sshex8_prolongate / sshex8_restrict); level 1 is applied as hex8.
 * The smoother may run on the Jacobi-scaled operator (D^-1 A), as the GPU solvers do.
 */
#include <math.h>
#include <omp.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int32_t idx_t;
typedef float jacobian_t;

/* oracle.c */
int or_sshex8_laplacian_stencil_apply(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff,
                                      const double *u, double *values);
int or_hex8_laplacian_apply(ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff, const double *u,
                            double *values);
int or_laplacian_diag(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *fff, double *diag);
int or_linear_elasticity_apply(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *adjugate,
                               const jacobian_t *determinant, double mu, double lambda, const double *u, double *out);
int or_linear_elasticity_block_diag_sym(int L, ptrdiff_t nelements, idx_t **elements, const jacobian_t *adjugate,
                                        const jacobian_t *determinant, double mu, double lambda, double *diag3,
                                        double *block6);
int or_sshex8_prolongate(ptrdiff_t nelements, int from_level, idx_t **from_elements, int to_level,
                         idx_t **to_elements, int vec_size, const double *from, double *to);
int or_sshex8_restrict(ptrdiff_t nelements, int from_level, idx_t **from_elements, const uint16_t *count,
                       int to_level, idx_t **to_elements, int vec_size, const double *from, double *to);

/* One level of the hierarchy (filled by the caller). */
typedef struct {
    int L;                    /* sshex8 level; 1 = the macro hex8 mesh */
    idx_t **elements;         /* sshex8 connectivity of this level (lidx order; at L = 1 the 8 corners) */
    idx_t **hex8_elements;    /* L = 1 only: the corners in hex8 order (the hex8 apply's layout) */
    ptrdiff_t n_nodes;
    ptrdiff_t n_dirichlet;
    const idx_t *dirichlet;   /* constrained node ids */
    const uint16_t *count;    /* element-node incidence count of this level (restriction from it) */
} or_level_t;

typedef struct {
    int kind;                 /* 0 Laplacian, 1 linear elasticity (3 interleaved components) */
    ptrdiff_t nelements;      /* macro elements */
    const jacobian_t *geom;   /* FFF AoS [E][6] (Laplacian) or adjugate AoS [E][9] (elasticity) */
    const jacobian_t *det;    /* elasticity: determinant [E] */
    double mu, lambda;
    int nlevels;
    or_level_t *levels;       /* finest first */
    int sweeps;               /* Chebyshev3 sweeps, pre and post */
    int scaled;               /* smoother on D^-1 A */
    double scale_eig_max;     /* 1.02 in the reference's mgsolve */
    double coarse_rtol;       /* coarse CG: 1e-8 in mgsolve, 1e-6 in the default geometric multigrid */
    double rtol;              /* outer stop: true ||b - A x|| / ||b|| */
    int max_it;
    int flexible;             /* Polak-Ribiere beta (flexible CG) instead of Fletcher-Reeves */
} or_mg_problem_t;

typedef struct {
    int iterations;           /* outer CG iterations */
    int restarts;             /* residual replacements after the recurrence met rtol */
    int coarse_iterations;    /* all coarse CG iterations */
    double true_rel_residual;
    double setup_seconds, solve_seconds;
} or_mg_stats_t;

/* ---------------------------------------------------------------- vectors */
static double vdot(ptrdiff_t n, const double *x, const double *y) {
    double s = 0;
#pragma omp parallel for reduction(+ : s)
    for (ptrdiff_t i = 0; i < n; i++) s += x[i] * y[i];
    return s;
}
static void vzero(ptrdiff_t n, double *x) {
#pragma omp parallel for
    for (ptrdiff_t i = 0; i < n; i++) x[i] = 0;
}
static void vcopy(ptrdiff_t n, const double *x, double *y) {
#pragma omp parallel for
    for (ptrdiff_t i = 0; i < n; i++) y[i] = x[i];
}
/* y = a x + b y */
static void vaxpby(ptrdiff_t n, double a, const double *x, double b, double *y) {
#pragma omp parallel for
    for (ptrdiff_t i = 0; i < n; i++) y[i] = a * x[i] + b * y[i];
}
/* z = x * y */
static void vmul(ptrdiff_t n, const double *x, const double *y, double *z) {
#pragma omp parallel for
    for (ptrdiff_t i = 0; i < n; i++) z[i] = x[i] * y[i];
}

/* ---------------------------------------------------------------- levels */
typedef struct {
    const or_mg_problem_t *P;
    int k;
    ptrdiff_t n;              /* dofs */
    double *inv_diag;
    double eig_max;
    double *rhs, *sol, *work, *p, *t;
} level_state_t;

static int bs_of(const or_mg_problem_t *P) { return P->kind == 1 ? 3 : 1; }

/* y = A x with identity Dirichlet rows */
static void level_apply(const level_state_t *S, const double *x, double *y) {
    const or_mg_problem_t *P = S->P;
    const or_level_t *lv = &P->levels[S->k];
    vzero(S->n, y);
    if (P->kind == 0) {
        if (lv->L == 1)
            or_hex8_laplacian_apply(P->nelements, lv->hex8_elements, P->geom, x, y);
        else
            or_sshex8_laplacian_stencil_apply(lv->L, P->nelements, lv->elements, P->geom, x, y);
    } else {
        if (lv->L == 1)
            or_linear_elasticity_apply(0, P->nelements, lv->hex8_elements, P->geom, P->det, P->mu, P->lambda, x, y);
        else
            or_linear_elasticity_apply(lv->L, P->nelements, lv->elements, P->geom, P->det, P->mu, P->lambda, x, y);
    }
    const int bs = bs_of(P);
    for (ptrdiff_t i = 0; i < lv->n_dirichlet; i++)
        for (int d = 0; d < bs; d++) y[(ptrdiff_t)lv->dirichlet[i] * bs + d] = x[(ptrdiff_t)lv->dirichlet[i] * bs + d];
}

static void zero_constraints(const level_state_t *S, double *x) {
    const or_level_t *lv = &S->P->levels[S->k];
    const int bs = bs_of(S->P);
    for (ptrdiff_t i = 0; i < lv->n_dirichlet; i++)
        for (int d = 0; d < bs; d++) x[(ptrdiff_t)lv->dirichlet[i] * bs + d] = 0;
}

static void level_inverse_diagonal(level_state_t *S) {
    const or_mg_problem_t *P = S->P;
    const or_level_t *lv = &P->levels[S->k];
    double *d = S->inv_diag;
    vzero(S->n, d);
    if (P->kind == 0) {
        or_laplacian_diag(lv->L == 1 ? 0 : lv->L, P->nelements, lv->L == 1 ? lv->hex8_elements : lv->elements, P->geom, d);
    } else {
        double *b6 = (double *)calloc((size_t)lv->n_nodes * 6, sizeof(double));
        or_linear_elasticity_block_diag_sym(lv->L == 1 ? 0 : lv->L, P->nelements,
                                            lv->L == 1 ? lv->hex8_elements : lv->elements, P->geom, P->det, P->mu,
                                            P->lambda, d, b6);
        free(b6);
    }
    const int bs = bs_of(P);
    for (ptrdiff_t i = 0; i < lv->n_dirichlet; i++)
        for (int c = 0; c < bs; c++) d[(ptrdiff_t)lv->dirichlet[i] * bs + c] = 1;
#pragma omp parallel for
    for (ptrdiff_t i = 0; i < S->n; i++) d[i] = 1.0 / d[i];
}

/* the operator the smoother sees: A or D^-1 A */
static void smoother_op(const level_state_t *S, const double *x, double *y) {
    level_apply(S, x, y);
    if (S->P->scaled) vmul(S->n, S->inv_diag, y, y);
}

/* PowerMethod::max_eigen_value (algebra/sfem_PowerMethod.hpp:18-55): start from ones,
 * |lambda_k - lambda_{k-1}| <= 1e-5 checked on even steps, at most 100 (odd) steps. */
static double power_method(level_state_t *S) {
    const ptrdiff_t n = S->n;
    double *v0 = (double *)malloc(n * sizeof(double)), *v1 = (double *)malloc(n * sizeof(double));
    double *w = (double *)malloc(n * sizeof(double));
    for (ptrdiff_t i = 0; i < n; i++) v0[i] = 1;
    smoother_op(S, v0, v1);
    double nrm = sqrt(vdot(n, v1, v1));
    vaxpby(n, 0, v1, 1.0 / nrm, v1);
    double *vecs[2] = {v0, v1};
    double lam = 0, lam_old = 0;
    for (int k = 0; k < 101; k++) {
        smoother_op(S, vecs[(k + 1) % 2], w);
        lam = sqrt(vdot(n, w, w));
        vaxpby(n, 0, w, 1.0 / lam, w);
        vcopy(n, w, vecs[k % 2]);
        if (fabs(lam - lam_old) <= 1e-5 && k % 2 == 0) break;
        lam_old = lam;
    }
    free(v0);
    free(v1);
    free(w);
    return lam;
}

/* Chebyshev3::precond_apply with a nonzero initial guess; on D^-1 A when scaled
 * (residuals scaled by D^-1). */
static void chebyshev3(level_state_t *S, const double *rhs, double *x) {
    const ptrdiff_t n = S->n;
    const int scaled = S->P->scaled;
    const double emax = S->eig_max * S->P->scale_eig_max, emin = 0.06 * emax;
    const double eavg = (emin + emax) / 2, ediff = (emin - emax) / 2;
    double alpha = 1.0 / eavg, beta = 0;
    double *p = S->p, *t = S->t;
    level_apply(S, x, p);
#pragma omp parallel for
    for (ptrdiff_t i = 0; i < n; i++) {
        p[i] = (p[i] - rhs[i]) * (scaled ? S->inv_diag[i] : 1.0);
        x[i] -= alpha * p[i];
    }
    for (int it = 1; it < S->P->sweeps; it++) {
        const double dea = ediff * alpha;
        beta = (it == 1 ? 0.5 : 0.25) * dea * dea;
        alpha = 1.0 / (eavg - beta / alpha);
        level_apply(S, x, t);
#pragma omp parallel for
        for (ptrdiff_t i = 0; i < n; i++) {
            p[i] = beta * p[i] + (t[i] - rhs[i]) * (scaled ? S->inv_diag[i] : 1.0);
            x[i] -= alpha * p[i];
        }
    }
}

/* Jacobi-preconditioned CG (ConjugateGradient with an inverse-diagonal preconditioner),
 * zero initial guess; stops on sqrt(rtz)/sqrt(rtz0) < rtol or sqrt(rtz) < atol. */
static int jacobi_pcg(level_state_t *S, const double *b, double *x, double rtol, double atol, int max_it) {
    const ptrdiff_t n = S->n;
    double *r = (double *)malloc(n * sizeof(double)), *z = (double *)malloc(n * sizeof(double));
    double *p = (double *)malloc(n * sizeof(double)), *Ap = (double *)malloc(n * sizeof(double));
    vzero(n, x);
    vcopy(n, b, r);
    vmul(n, S->inv_diag, r, z);
    vcopy(n, z, p);
    double rtz = vdot(n, r, z);
    const double rtz0 = rtz;
    int it = 0;
    if (rtz0 > 0 && sqrt(rtz0) >= atol) {
        for (it = 1; it <= max_it; it++) {
            level_apply(S, p, Ap);
            const double alpha = rtz / vdot(n, p, Ap);
            vaxpby(n, alpha, p, 1, x);
            vaxpby(n, -alpha, Ap, 1, r);
            vmul(n, S->inv_diag, r, z);
            const double rtz_new = vdot(n, r, z);
            if (sqrt(fabs(rtz_new)) < atol || sqrt(fabs(rtz_new / rtz0)) < rtol) break;
            vaxpby(n, 1, z, rtz_new / rtz, p);
            rtz = rtz_new;
        }
    }
    free(r);
    free(z);
    free(p);
    free(Ap);
    return it;
}

typedef struct {
    level_state_t *L;
    int nlevels;
    int coarse_iterations;
} mg_t;

/* Multigrid::cycle, V-cycle, zero initial guess at every level */
static void vcycle(mg_t *M, int k) {
    level_state_t *S = &M->L[k];
    if (k == M->nlevels - 1) {
        M->coarse_iterations += jacobi_pcg(S, S->rhs, S->sol, S->P->coarse_rtol, 0.0, 40000);
        return;
    }
    level_state_t *C = &M->L[k + 1];
    const or_mg_problem_t *P = S->P;
    const or_level_t *lf = &P->levels[k], *lc = &P->levels[k + 1];
    const int bs = bs_of(P);
    chebyshev3(S, S->rhs, S->sol);
    level_apply(S, S->sol, S->work);
    vaxpby(S->n, 1, S->rhs, -1, S->work);
    vzero(C->n, C->rhs);
    or_sshex8_restrict(P->nelements, lf->L, lf->elements, lf->count, lc->L, lc->elements, bs, S->work, C->rhs);
    zero_constraints(C, C->rhs);
    vzero(C->n, C->sol);
    vcycle(M, k + 1);
    or_sshex8_prolongate(P->nelements, lc->L, lc->elements, lf->L, lf->elements, bs, C->sol, S->work);
    zero_constraints(S, S->work);
    vaxpby(S->n, 1, S->work, 1, S->sol);
    chebyshev3(S, S->rhs, S->sol);
}

/* x = V-cycle(r) from x = 0 */
static void mg_precond(mg_t *M, const double *r, double *z) {
    level_state_t *S = &M->L[0];
    vcopy(S->n, r, S->rhs);
    vzero(S->n, S->sol);
    vcycle(M, 0);
    vcopy(S->n, S->sol, z);
}

static double wall(void) { return omp_get_wtime(); }

/* MG-preconditioned CG from x = 0 to ||b - A x|| / ||b|| <= rtol (true residual).
 * The outer CG stops on its recurrence residual; the true residual is then evaluated
 * and, if it misses rtol, CG restarts from the current x with r = b - A x. */
int or_mg_pcg_solve(const or_mg_problem_t *P, const double *b, double *x, or_mg_stats_t *stats) {
    const double t0 = wall();
    mg_t M;
    M.nlevels = P->nlevels;
    M.coarse_iterations = 0;
    M.L = (level_state_t *)calloc(P->nlevels, sizeof(level_state_t));
    const int bs = bs_of(P);
    for (int k = 0; k < P->nlevels; k++) {
        level_state_t *S = &M.L[k];
        S->P = P;
        S->k = k;
        S->n = P->levels[k].n_nodes * bs;
        S->inv_diag = (double *)malloc(S->n * sizeof(double));
        S->rhs = (double *)calloc(S->n, sizeof(double));
        S->sol = (double *)calloc(S->n, sizeof(double));
        S->work = (double *)calloc(S->n, sizeof(double));
        S->p = (double *)calloc(S->n, sizeof(double));
        S->t = (double *)calloc(S->n, sizeof(double));
        level_inverse_diagonal(S);
        if (k < P->nlevels - 1) S->eig_max = power_method(S);
    }
    const double t1 = wall();
    level_state_t *F = &M.L[0];
    const ptrdiff_t n = F->n;
    double *r = (double *)malloc(n * sizeof(double)), *z = (double *)malloc(n * sizeof(double));
    double *p = (double *)malloc(n * sizeof(double)), *Ap = (double *)malloc(n * sizeof(double));
    double *zold = P->flexible ? (double *)malloc(n * sizeof(double)) : NULL;
    const double bnorm = sqrt(vdot(n, b, b));
    vzero(n, x);
    int it = 0, restarts = 0;
    double rel = 1;
    while (it < P->max_it) {
        level_apply(F, x, Ap);
#pragma omp parallel for
        for (ptrdiff_t i = 0; i < n; i++) r[i] = b[i] - Ap[i];
        rel = sqrt(vdot(n, r, r)) / bnorm;
        if (rel <= P->rtol) break;
        if (it > 0) restarts++;
        mg_precond(&M, r, z);
        vcopy(n, z, p);
        double rtz = vdot(n, r, z);
        for (; it < P->max_it;) {
            it++;
            level_apply(F, p, Ap);
            const double alpha = rtz / vdot(n, p, Ap);
            vaxpby(n, alpha, p, 1, x);
            vaxpby(n, -alpha, Ap, 1, r);
            if (sqrt(vdot(n, r, r)) / bnorm <= P->rtol) break;
            if (zold) vcopy(n, z, zold);
            mg_precond(&M, r, z);
            const double rtz_new = vdot(n, r, z);
            /* flexible: beta = r.(z - z_old) / rtz_old, so a preconditioner that changes
             * between iterations (inexact coarse solves) keeps the search directions useful */
            const double beta = zold ? (rtz_new - vdot(n, r, zold)) / rtz : rtz_new / rtz;
            vaxpby(n, 1, z, beta, p);
            rtz = rtz_new;
        }
    }
    const double t2 = wall();
    level_apply(F, x, Ap);
#pragma omp parallel for
    for (ptrdiff_t i = 0; i < n; i++) r[i] = b[i] - Ap[i];
    rel = sqrt(vdot(n, r, r)) / bnorm;
    if (stats) {
        stats->iterations = it;
        stats->restarts = restarts;
        stats->coarse_iterations = M.coarse_iterations;
        stats->true_rel_residual = rel;
        stats->setup_seconds = t1 - t0;
        stats->solve_seconds = t2 - t1;
    }
    for (int k = 0; k < P->nlevels; k++) {
        level_state_t *S = &M.L[k];
        free(S->inv_diag);
        free(S->rhs);
        free(S->sol);
        free(S->work);
        free(S->p);
        free(S->t);
    }
    free(M.L);
    free(r);
    free(z);
    free(p);
    free(Ap);
    free(zold);
    return rel <= P->rtol ? 0 : 1;
}
