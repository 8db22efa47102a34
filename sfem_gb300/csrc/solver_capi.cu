// C ABI object layer over the device solver templates: operators (Laplacian,
// linear elasticity, transfer), smoothers and solvers as opaque handles, composed
// the way the reference's frontend composes them (frontend/sfem_API.hpp:
// create_cg :143, create_shiftable_jacobi :180, create_stationary :247,
// create_cheb3 :287, create_mg :323, create_hierarchical_prolongation :409,
// create_hierarchical_restriction :575) and as drivers/mgsolve.cpp:128-330 uses them.
#include <cstdarg>
#include <cstring>
#include <functional>
#include <memory>
#include <string>

#include "common.cuh"
#include "capi_handle.hpp"
#include "solvers.hpp"

namespace sfem_gb300 {

// ---------------------------------------------------------------- operators

// Function-level Laplacian: y += A x, then y[c] = x[c] on Dirichlet nodes
// (Function::apply + copy_constrained_dofs, frontend/sfem_Function.cpp:481-496).
template <typename T>
class LaplacianOp final : public Operator<T> {
public:
    std::shared_ptr<Context> ctx;
    int element_type{0};
    ptrdiff_t nelements{0}, n_nodes{0}, fff_stride{0}, n_dirichlet{0};
    idx_t **elements{nullptr};
    const float *fff{nullptr};
    const idx_t *dirichlet{nullptr};
    // FP32 sshex8 L = 3, 4: connectivity + FFF repacked per 32-element tile, built at creation
    // (the operator keeps the geometry it was created with, as the reference's op keeps its FFF)
    DeviceBuffer<int32_t> packed;
    int prepare() {
        if (real_type_v<T> != SFEM_GB300_FLOAT32) return 0;
        const ptrdiff_t nb = sfem_gb300_sshex8_packed_bytes(element_type, nelements);
        if (nb <= 0) return 0;
        SFEM_GB300_CHECK(packed.resize(nb / (ptrdiff_t)sizeof(int32_t)));
        return sfem_gb300_sshex8_pack(element_type, nelements, elements, fff_stride, fff, packed.ptr, ctx->sp());
    }
    int apply(const T *x, T *y) override {
        if (packed.n > 0) {
            SFEM_GB300_CHECK(sfem_gb300_sshex8_laplacian_apply_packed(element_type, nelements, packed.ptr,
                                                                      real_type_v<T>, x, y, ctx->sp()));
        } else {
            SFEM_GB300_CHECK(cu_laplacian_apply(element_type, nelements, elements, fff_stride, fff, real_type_v<T>, x,
                                                y, ctx->sp()));
        }
        return sfem_gb300_constraint_nodes_copy(real_type_v<T>, n_dirichlet, dirichlet, 1, 0, x, y, ctx->sp());
    }
    ptrdiff_t rows() const override { return n_nodes; }
    ptrdiff_t cols() const override { return n_nodes; }
};

// Function-level linear elasticity (3 dofs per node, interleaved), Dirichlet on all components.
template <typename T>
class ElasticityOp final : public Operator<T> {
public:
    std::shared_ptr<Context> ctx;
    int element_type{0};
    ptrdiff_t nelements{0}, n_nodes{0}, jac_stride{0}, n_dirichlet{0};
    idx_t **elements{nullptr};
    const float *adjugate{nullptr}, *determinant{nullptr};
    double mu{1}, lambda{1};
    const idx_t *dirichlet{nullptr};
    int contraction{real_type_v<T>};  // FLOAT32_BF16TC: tensor-core BF16 element contraction
    DeviceBuffer<T> em;                // stored element matrices (coarse levels), built by prepare()
    bool stored() const {
        const bool coarse = element_type == SFEM_GB300_HEX8 ||
                            (element_type >= SFEM_GB300_SSHEX8(1) && element_type <= SFEM_GB300_SSHEX8(2));
        // at most 4 GiB of matrices (576 values per element); larger meshes build them per apply
        const bool fits = (double)nelements * 576 * sizeof(T) <= 4.0 * 1024 * 1024 * 1024;
        return coarse && fits && contraction == real_type_v<T>;
    }
    // called at creation and whenever the geometry or the contraction changes (outside any capture)
    int prepare() {
        if (!stored()) return 0;
        SFEM_GB300_CHECK(em.resize(576 * nelements));
        return sfem_gb300_linear_elasticity_element_matrices(element_type, nelements, jac_stride, adjugate,
                                                             determinant, mu, lambda, real_type_v<T>, em.ptr,
                                                             ctx->sp());
    }
    int apply(const T *x, T *y) override {
        if (stored() && em.n == 576 * nelements) {
            SFEM_GB300_CHECK(sfem_gb300_linear_elasticity_apply_em(element_type, nelements, elements, em.ptr,
                                                                   real_type_v<T>, x, y, ctx->sp()));
        } else {
            SFEM_GB300_CHECK(sfem_gb300_linear_elasticity_apply(element_type, nelements, elements, jac_stride,
                                                                adjugate, determinant, mu, lambda, contraction, x, y,
                                                                ctx->sp()));
        }
        SFEM_GB300_CHECK(constraint_copy_block(real_type_v<T>, n_dirichlet, dirichlet, 3, x, y, ctx->sp()));
        return 0;
    }
    ptrdiff_t rows() const override { return 3 * n_nodes; }
    ptrdiff_t cols() const override { return 3 * n_nodes; }
};

// Prolongation (overwrites y) followed by zeroing the fine Dirichlet dofs
// (algebra/mg/sfem_GeometricMultigrid.cpp:54-66).
template <typename T>
class ProlongationOp final : public Operator<T> {
public:
    std::shared_ptr<Context> ctx;
    ptrdiff_t nelements{0}, n_from{0}, n_to{0}, n_dirichlet{0};
    int from_level{0}, to_level{0}, vec{1};
    idx_t **from_elements{nullptr}, **to_elements{nullptr};
    const idx_t *dirichlet{nullptr};
    int apply(const T *x, T *y) override {
        SFEM_GB300_CHECK(sfem_gb300_sshex8_prolongate(nelements, from_level, from_elements, to_level, to_elements, vec,
                                                      real_type_v<T>, x, y, ctx->sp()));
        SFEM_GB300_CHECK(constraint_value_block(real_type_v<T>, n_dirichlet, dirichlet, vec, 0.0, y, ctx->sp()));
        return 0;
    }
    ptrdiff_t rows() const override { return vec * n_to; }
    ptrdiff_t cols() const override { return vec * n_from; }
    bool overwrites_output() const override { return true; }
};

// Nested interpolation (or its transpose) stored as CSR: overwrites y, then zeroes
// the output Dirichlet dofs (used for the hex8 levels below the macro mesh).
template <typename T>
class CrsTransferOp final : public Operator<T> {
public:
    std::shared_ptr<Context> ctx;
    ptrdiff_t nrows{0}, ncols{0}, n_dirichlet{0};
    int vec{1};
    const idx_t *rowptr{nullptr}, *colidx{nullptr};
    const double *weights{nullptr};
    const idx_t *dirichlet{nullptr};
    int apply(const T *x, T *y) override {
        SFEM_GB300_CHECK(sfem_gb300_crs_transfer(real_type_v<T>, nrows, vec, rowptr, colidx, weights, x, y, ctx->sp()));
        SFEM_GB300_CHECK(constraint_value_block(real_type_v<T>, n_dirichlet, dirichlet, vec, 0.0, y, ctx->sp()));
        return 0;
    }
    ptrdiff_t rows() const override { return vec * nrows; }
    ptrdiff_t cols() const override { return vec * ncols; }
    bool overwrites_output() const override { return true; }
};

// Restriction (accumulates into y) followed by zeroing the coarse Dirichlet dofs
// (algebra/mg/sfem_GeometricMultigrid.cpp:38-52).
template <typename T>
class RestrictionOp final : public Operator<T> {
public:
    std::shared_ptr<Context> ctx;
    ptrdiff_t nelements{0}, n_from{0}, n_to{0}, n_dirichlet{0};
    int from_level{0}, to_level{0}, vec{1};
    idx_t **from_elements{nullptr}, **to_elements{nullptr};
    const uint16_t *count{nullptr};
    const idx_t *dirichlet{nullptr};
    int apply(const T *x, T *y) override {
        SFEM_GB300_CHECK(sfem_gb300_sshex8_restrict(nelements, from_level, from_elements, count, to_level, to_elements,
                                                    vec, real_type_v<T>, x, y, ctx->sp()));
        SFEM_GB300_CHECK(constraint_value_block(real_type_v<T>, n_dirichlet, dirichlet, vec, 0.0, y, ctx->sp()));
        return 0;
    }
    ptrdiff_t rows() const override { return vec * n_to; }
    ptrdiff_t cols() const override { return vec * n_from; }
};

// Assembled symmetric CRS operator: y += A x via a scratch vector, Dirichlet rows identity.
template <typename T>
class CrsSymOp final : public Operator<T> {
public:
    std::shared_ptr<Context> ctx;
    ptrdiff_t nrows{0}, n_dirichlet{0};
    const idx_t *rowptr{nullptr}, *colidx{nullptr}, *dirichlet{nullptr};
    const T *diag{nullptr}, *offdiag{nullptr};
    DeviceBuffer<T> tmp;
    int apply(const T *x, T *y) override {
        SFEM_GB300_CHECK(tmp.resize(nrows));
        SFEM_GB300_CHECK(sfem_gb300_crs_sym_spmv(real_type_v<T>, nrows, rowptr, colidx, diag, offdiag, 0.0, x,
                                                 tmp.ptr, ctx->sp()));
        SFEM_GB300_CHECK(sfem_gb300_axpy(real_type_v<T>, nrows, 1.0, tmp.ptr, y, ctx->sp()));
        return sfem_gb300_constraint_nodes_copy(real_type_v<T>, n_dirichlet, dirichlet, 1, 0, x, y, ctx->sp());
    }
    ptrdiff_t rows() const override { return nrows; }
    ptrdiff_t cols() const override { return nrows; }
};

// Iterative refinement (no reference counterpart): outer loop in double with the
// double operator, inner solve in float on the normalised residual.
//   r = b - A x ; d = inner(r / |r|) ; x += |r| d ; until |r| <= rtol |b|.
class IterativeRefinement final : public Solver<double> {
public:
    std::shared_ptr<Context> ctx;
    std::shared_ptr<Operator<double>> op;
    std::shared_ptr<Operator<float>> inner;
    DeviceBuffer<double> r;
    DeviceBuffer<float> r32, d32;
    int max_it{50};
    double rtol{1e-10}, atol{0};
    double last_rel{0};
    double *s{nullptr};
    std::function<void()> on_stagnation;  // FP64 residual failed to decrease by half
    bool stagnated{false};
    int apply(const double *b, double *x) override {
        const ptrdiff_t n = op->rows();
        if (!s) s = ctx->slots(2);
        SFEM_GB300_CHECK(r.resize(n));
        SFEM_GB300_CHECK(r32.resize(n));
        SFEM_GB300_CHECK(d32.resize(n));
        Blas<double> bd = blas_of<double>(ctx);
        bd.norm2(n, b, &s[1]);
        const double bnorm = ctx->read(&s[1]);
        double prev = -1;
        int flat = 0;
        stagnated = false;
        for (this->iterations_ = 0;; this->iterations_++) {
            bd.zeros(n, r.ptr);
            SFEM_GB300_CHECK(op->apply(x, r.ptr));
            bd.axpby(n, 1.0, b, -1.0, r.ptr);
            bd.norm2(n, r.ptr, &s[0]);
            const double rnorm = ctx->read(&s[0]);
            last_rel = bnorm > 0 ? rnorm / bnorm : rnorm;
            if (prev >= 0 && rnorm > 0.5 * prev && on_stagnation && !stagnated) {
                stagnated = true;
                on_stagnation();
            }
            // FP64 attainable accuracy reached: two outer steps without a 10 % reduction
            if (prev >= 0 && rnorm > 0.9 * prev) {
                if (++flat >= 2)
                    return set_error("IterativeRefinement: residual stagnated at %g (rtol %g not attainable)", last_rel,
                                     rtol);
            } else {
                flat = 0;
            }
            prev = rnorm;
            if (rnorm <= rtol * bnorm || rnorm <= atol || rnorm == 0) return 0;
            if (!std::isfinite(rnorm)) return set_error("IterativeRefinement: non-finite residual");
            if (this->iterations_ >= max_it) return set_error("IterativeRefinement: no convergence (rel %g)", last_rel);
            bd.scal(n, 1.0 / rnorm, r.ptr);
            SFEM_GB300_CHECK(sfem_gb300_convert(n, SFEM_GB300_FLOAT64, r.ptr, SFEM_GB300_FLOAT32, r32.ptr, ctx->sp()));
            cudaMemsetAsync(d32.ptr, 0, n * sizeof(float), ctx->stream);
            inner->apply(r32.ptr, d32.ptr);  // inner may stop at its own max_it: refinement absorbs it
            SFEM_GB300_CHECK(sfem_gb300_axpy_f32_to_f64(n, rnorm, d32.ptr, x, ctx->sp()));
        }
    }
    ptrdiff_t rows() const override { return op->rows(); }
    ptrdiff_t cols() const override { return op->cols(); }
};

}  // namespace sfem_gb300

using namespace sfem_gb300;

typedef Handle sfem_gb300_handle;


extern "C" {

int sfem_gb300_context_create(void *stream, void **out) {
    cudaStream_t s = stream_of(stream);
    auto ctx = Context::create(s);
    if (!ctx) return set_error("sfem_gb300_context_create: allocation failed");
    auto *h = new Handle();
    h->kind = "context";
    h->ctx = ctx;
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_handle_destroy(void *handle) {
    delete H(handle);
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_laplacian_op_create(void *context, int real_type, int element_type, ptrdiff_t nelements,
                                   idx_t **elements, ptrdiff_t fff_stride, const float *fff, ptrdiff_t n_nodes,
                                   ptrdiff_t n_dirichlet, const int32_t *dirichlet_nodes, void **out) {
    auto *c = H(context);
    auto *h = new Handle();
    h->kind = "laplacian";
    h->ctx = c->ctx;
    h->real_type = is_f32(real_type) ? SFEM_GB300_FLOAT32 : SFEM_GB300_FLOAT64;
    auto fill = [&](auto op) {
        op->ctx = c->ctx;
        op->element_type = element_type;
        op->nelements = nelements;
        op->elements = elements;
        op->fff_stride = fff_stride;
        op->fff = fff;
        op->n_nodes = n_nodes;
        op->n_dirichlet = n_dirichlet;
        op->dirichlet = dirichlet_nodes;
    };
    int rc = 0;
    if (is_f32(real_type)) {
        auto op = std::make_shared<LaplacianOp<float>>();
        fill(op);
        rc = op->prepare();
        h->f = op;
    } else {
        auto op = std::make_shared<LaplacianOp<double>>();
        fill(op);
        h->d = op;
    }
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_elasticity_op_create(void *context, int real_type, int element_type, ptrdiff_t nelements,
                                    idx_t **elements, ptrdiff_t jacobian_stride, const float *adjugate,
                                    const float *determinant, double mu, double lambda, ptrdiff_t n_nodes,
                                    ptrdiff_t n_dirichlet, const int32_t *dirichlet_nodes, void **out) {
    auto *c = H(context);
    auto *h = new Handle();
    h->kind = "elasticity";
    h->ctx = c->ctx;
    h->real_type = is_f32(real_type) ? SFEM_GB300_FLOAT32 : SFEM_GB300_FLOAT64;
    auto fill = [&](auto op) {
        op->ctx = c->ctx;
        op->element_type = element_type;
        op->nelements = nelements;
        op->elements = elements;
        op->jac_stride = jacobian_stride;
        op->adjugate = adjugate;
        op->determinant = determinant;
        op->mu = mu;
        op->lambda = lambda;
        op->n_nodes = n_nodes;
        op->n_dirichlet = n_dirichlet;
        op->dirichlet = dirichlet_nodes;
    };
    int rc = 0;
    if (is_f32(real_type)) {
        auto op = std::make_shared<ElasticityOp<float>>();
        fill(op);
        if (real_type == SFEM_GB300_FLOAT32_BF16TC) op->contraction = SFEM_GB300_FLOAT32_BF16TC;
        rc = op->prepare();
        h->f = op;
    } else {
        auto op = std::make_shared<ElasticityOp<double>>();
        fill(op);
        rc = op->prepare();
        h->d = op;
    }
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_prolongation_op_create(void *context, int real_type, ptrdiff_t nelements, int from_level,
                                      idx_t **from_elements, ptrdiff_t n_from, int to_level, idx_t **to_elements,
                                      ptrdiff_t n_to, int vec_size, ptrdiff_t n_dirichlet_to,
                                      const int32_t *dirichlet_to, void **out) {
    auto *c = H(context);
    auto *h = new Handle();
    h->kind = "prolongation";
    h->ctx = c->ctx;
    h->real_type = is_f32(real_type) ? SFEM_GB300_FLOAT32 : SFEM_GB300_FLOAT64;
    auto fill = [&](auto op) {
        op->ctx = c->ctx;
        op->nelements = nelements;
        op->from_level = from_level;
        op->from_elements = from_elements;
        op->n_from = n_from;
        op->to_level = to_level;
        op->to_elements = to_elements;
        op->n_to = n_to;
        op->vec = vec_size;
        op->n_dirichlet = n_dirichlet_to;
        op->dirichlet = dirichlet_to;
    };
    if (is_f32(real_type)) {
        auto op = std::make_shared<ProlongationOp<float>>();
        fill(op);
        h->f = op;
    } else {
        auto op = std::make_shared<ProlongationOp<double>>();
        fill(op);
        h->d = op;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_restriction_op_create(void *context, int real_type, ptrdiff_t nelements, int from_level,
                                     idx_t **from_elements, const uint16_t *count, ptrdiff_t n_from, int to_level,
                                     idx_t **to_elements, ptrdiff_t n_to, int vec_size, ptrdiff_t n_dirichlet_to,
                                     const int32_t *dirichlet_to, void **out) {
    auto *c = H(context);
    auto *h = new Handle();
    h->kind = "restriction";
    h->ctx = c->ctx;
    h->real_type = is_f32(real_type) ? SFEM_GB300_FLOAT32 : SFEM_GB300_FLOAT64;
    auto fill = [&](auto op) {
        op->ctx = c->ctx;
        op->nelements = nelements;
        op->from_level = from_level;
        op->from_elements = from_elements;
        op->count = count;
        op->n_from = n_from;
        op->to_level = to_level;
        op->to_elements = to_elements;
        op->n_to = n_to;
        op->vec = vec_size;
        op->n_dirichlet = n_dirichlet_to;
        op->dirichlet = dirichlet_to;
    };
    if (is_f32(real_type)) {
        auto op = std::make_shared<RestrictionOp<float>>();
        fill(op);
        h->f = op;
    } else {
        auto op = std::make_shared<RestrictionOp<double>>();
        fill(op);
        h->d = op;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_crs_sym_op_create(void *context, int real_type, ptrdiff_t nrows, const int32_t *rowptr,
                                 const int32_t *colidx, const void *diag, const void *offdiag, ptrdiff_t n_dirichlet,
                                 const int32_t *dirichlet_nodes, void **out) {
    auto *c = H(context);
    auto *h = new Handle();
    h->kind = "crs_sym";
    h->ctx = c->ctx;
    h->real_type = is_f32(real_type) ? SFEM_GB300_FLOAT32 : SFEM_GB300_FLOAT64;
    auto fill = [&](auto op, auto tag) {
        using T = decltype(tag);
        op->ctx = c->ctx;
        op->nrows = nrows;
        op->rowptr = rowptr;
        op->colidx = colidx;
        op->diag = (const T *)diag;
        op->offdiag = (const T *)offdiag;
        op->n_dirichlet = n_dirichlet;
        op->dirichlet = dirichlet_nodes;
    };
    if (is_f32(real_type)) {
        auto op = std::make_shared<CrsSymOp<float>>();
        fill(op, 0.0f);
        h->f = op;
    } else {
        auto op = std::make_shared<CrsSymOp<double>>();
        fill(op, 0.0);
        h->d = op;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_op_apply(void *op, const void *x, void *y) {
    auto *h = H(op);
    if (h->d) return h->d->apply((const double *)x, (double *)y);
    if (h->f) return h->f->apply((const float *)x, (float *)y);
    return set_error("sfem_gb300_op_apply: handle of kind '%s' is not an operator", h->kind.c_str());
}

int sfem_gb300_op_size(void *op, ptrdiff_t *rows, ptrdiff_t *cols) {
    auto *h = H(op);
    *rows = h->rows();
    *cols = h->cols();
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_jacobi_create(void *context, int real_type, ptrdiff_t n, const void *diag, double relaxation,
                             void **out) {
    auto *c = H(context);
    auto *h = new Handle();
    h->kind = "jacobi";
    h->ctx = c->ctx;
    h->real_type = is_f32(real_type) ? SFEM_GB300_FLOAT32 : SFEM_GB300_FLOAT64;
    int rc;
    if (is_f32(real_type)) {
        auto j = std::make_shared<Jacobi<float>>();
        j->blas = blas_of<float>(c->ctx);
        j->relaxation = relaxation;
        rc = j->set_diag((const float *)diag, n);
        h->f = j;
    } else {
        auto j = std::make_shared<Jacobi<double>>();
        j->blas = blas_of<double>(c->ctx);
        j->relaxation = relaxation;
        rc = j->set_diag((const double *)diag, n);
        h->d = j;
    }
    *out = h;
    return rc;
}

int sfem_gb300_block_jacobi_create(void *context, int real_type, ptrdiff_t n_nodes, const void *inv_block6,
                                   void **out) {
    auto *c = H(context);
    auto *h = new Handle();
    h->kind = "block_jacobi";
    h->ctx = c->ctx;
    h->real_type = is_f32(real_type) ? SFEM_GB300_FLOAT32 : SFEM_GB300_FLOAT64;
    if (is_f32(real_type)) {
        auto j = std::make_shared<BlockJacobi<float>>();
        j->blas = blas_of<float>(c->ctx);
        j->inv_block6 = (const float *)inv_block6;
        j->n_nodes = n_nodes;
        h->f = j;
    } else {
        auto j = std::make_shared<BlockJacobi<double>>();
        j->blas = blas_of<double>(c->ctx);
        j->inv_block6 = (const double *)inv_block6;
        j->n_nodes = n_nodes;
        h->d = j;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_stationary_create(void *context, void *op, void *precond, int max_it, void **out) {
    auto *c = H(context);
    auto *o = H(op), *p = H(precond);
    auto *h = new Handle();
    h->kind = "stationary";
    h->ctx = c->ctx;
    h->real_type = o->real_type;
    if (o->f) {
        auto s = std::make_shared<Stationary<float>>();
        s->blas = blas_of<float>(c->ctx);
        s->op = o->f;
        s->precond = p->f;
        s->max_it = max_it;
        h->f = s;
    } else {
        auto s = std::make_shared<Stationary<double>>();
        s->blas = blas_of<double>(c->ctx);
        s->op = o->d;
        s->precond = p->d;
        s->max_it = max_it;
        h->d = s;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_chebyshev3_create(void *context, void *op, const void *inv_diag, int max_it, double scale_eig_max,
                                 double scale_eig_min, int eigen_max_it, double eigen_tol, void **out) {
    auto *c = H(context);
    auto *o = H(op);
    auto *h = new Handle();
    h->kind = "chebyshev3";
    h->ctx = c->ctx;
    h->real_type = o->real_type;
    int rc;
    if (o->f) {
        auto s = std::make_shared<Chebyshev3<float>>();
        s->blas = blas_of<float>(c->ctx);
        s->op = o->f;
        s->inv_diag = (const float *)inv_diag;
        s->max_it = max_it;
        s->scale_eig_max = scale_eig_max;
        s->scale_eig_min = scale_eig_min;
        s->eigen_max_it = eigen_max_it;
        s->eigen_tol = eigen_tol;
        rc = eigen_max_it > 1 ? s->init_with_random(0x5eed5eedull) : s->init_with_ones();
        h->f = s;
        h->impl = s;
    } else {
        auto s = std::make_shared<Chebyshev3<double>>();
        s->blas = blas_of<double>(c->ctx);
        s->op = o->d;
        s->inv_diag = (const double *)inv_diag;
        s->max_it = max_it;
        s->scale_eig_max = scale_eig_max;
        s->scale_eig_min = scale_eig_min;
        s->eigen_max_it = eigen_max_it;
        s->eigen_tol = eigen_tol;
        rc = eigen_max_it > 1 ? s->init_with_random(0x5eed5eedull) : s->init_with_ones();
        h->d = s;
        h->impl = s;
    }
    *out = h;
    return rc;
}

int sfem_gb300_chebyshev3_eig_max(void *cheb, double *eig_max) {
    auto *h = H(cheb);
    if (h->kind != "chebyshev3") return set_error("not a chebyshev3 handle");
    if (h->f)
        *eig_max = std::static_pointer_cast<Chebyshev3<float>>(h->impl)->eig_max;
    else
        *eig_max = std::static_pointer_cast<Chebyshev3<double>>(h->impl)->eig_max;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_chebyshev3_set_eig_max(void *cheb, double eig_max) {
    auto *h = H(cheb);
    if (h->kind != "chebyshev3") return set_error("not a chebyshev3 handle");
    if (h->f)
        std::static_pointer_cast<Chebyshev3<float>>(h->impl)->eig_max = eig_max;
    else
        std::static_pointer_cast<Chebyshev3<double>>(h->impl)->eig_max = eig_max;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_cg_create(void *context, void *op, void *precond, int max_it, double rtol, double atol, void **out) {
    auto *c = H(context);
    auto *o = H(op);
    auto *p = precond ? H(precond) : nullptr;
    auto *h = new Handle();
    h->kind = "cg";
    h->ctx = c->ctx;
    h->real_type = o->real_type;
    if (o->f) {
        auto s = std::make_shared<ConjugateGradient<float>>();
        s->blas = blas_of<float>(c->ctx);
        s->op = o->f;
        if (p) s->precond = p->f;
        s->max_it = max_it;
        s->rtol = rtol;
        s->atol = atol;
        h->f = s;
        h->impl = s;
    } else {
        auto s = std::make_shared<ConjugateGradient<double>>();
        s->blas = blas_of<double>(c->ctx);
        s->op = o->d;
        if (p) s->precond = p->d;
        s->max_it = max_it;
        s->rtol = rtol;
        s->atol = atol;
        h->d = s;
        h->impl = s;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_mg_create(void *context, int real_type, int max_it, int cycle_type, void **out) {
    auto *c = H(context);
    auto *h = new Handle();
    h->kind = "mg";
    h->ctx = c->ctx;
    h->real_type = is_f32(real_type) ? SFEM_GB300_FLOAT32 : SFEM_GB300_FLOAT64;
    if (is_f32(real_type)) {
        auto m = std::make_shared<Multigrid<float>>();
        m->blas = blas_of<float>(c->ctx);
        m->max_it = max_it;
        m->cycle_type = cycle_type;
        h->f = m;
        h->impl = m;
    } else {
        auto m = std::make_shared<Multigrid<double>>();
        m->blas = blas_of<double>(c->ctx);
        m->max_it = max_it;
        m->cycle_type = cycle_type;
        h->d = m;
        h->impl = m;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

// Levels are added finest first; prolongation maps the next coarser level to this one,
// restriction maps this level to the next coarser one (both NULL on the coarsest level).
int sfem_gb300_mg_add_level(void *mg, void *op, void *smoother, void *prolongation, void *restriction) {
    auto *h = H(mg);
    if (h->kind != "mg") return set_error("sfem_gb300_mg_add_level: not a multigrid handle");
    auto *o = H(op), *s = H(smoother);
    auto *p = prolongation ? H(prolongation) : nullptr, *r = restriction ? H(restriction) : nullptr;
    if (h->f) {
        auto m = std::static_pointer_cast<Multigrid<float>>(h->impl);
        m->add_level(o->f, s->f, p ? p->f : nullptr, r ? r->f : nullptr);
    } else {
        auto m = std::static_pointer_cast<Multigrid<double>>(h->impl);
        m->add_level(o->d, s->d, p ? p->d : nullptr, r ? r->d : nullptr);
    }
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_learned_smoother_create(void *context, void *op, idx_t **elements, ptrdiff_t nelements,
                                       const uint16_t *count, const void *inv_diag, const void *W1, const void *W2,
                                       const void *W3, int channels, double omega, int sweeps, void *fallback,
                                       void **out) {
    auto *c = H(context);
    auto *o = H(op);
    auto *fb = fallback ? H(fallback) : nullptr;
    if (channels != 16) return set_error("sfem_gb300_learned_smoother_create: channels must be 16");
    auto *h = new Handle();
    h->kind = "learned";
    h->ctx = c->ctx;
    h->real_type = o->real_type;
    auto fill = [&](auto s, auto tag) {
        using T = decltype(tag);
        s->blas = blas_of<T>(c->ctx);
        s->elements = elements;
        s->nelements = nelements;
        s->count = count;
        s->inv_diag = (const T *)inv_diag;
        s->W[0] = W1;
        s->W[1] = W2;
        s->W[2] = W3;
        s->channels = channels;
        s->omega = omega;
        s->sweeps = sweeps;
    };
    // the correction is zeroed on the operator's Dirichlet nodes
    auto constraints = [](auto s, auto op) {
        using T = typename std::remove_reference_t<decltype(*op)>::value_type;
        if (auto lop = std::dynamic_pointer_cast<LaplacianOp<T>>(op)) {
            s->dirichlet = lop->dirichlet;
            s->n_dirichlet = lop->n_dirichlet;
        }
    };
    if (o->f) {
        auto s = std::make_shared<LearnedSmoother<float>>();
        fill(s, 0.0f);
        s->op = o->f;
        constraints(s, o->f);
        if (fb) s->fallback = fb->f;
        h->f = s;
        h->impl = s;
    } else {
        auto s = std::make_shared<LearnedSmoother<double>>();
        fill(s, 0.0);
        s->op = o->d;
        constraints(s, o->d);
        if (fb) s->fallback = fb->d;
        h->d = s;
        h->impl = s;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_solver_set_fallback(void *solver, void *learned) {
    auto *h = H(solver);
    auto *l = H(learned);
    if (l->kind != "learned") return set_error("sfem_gb300_solver_set_fallback: not a learned-smoother handle");
    std::function<void()> fn;
    if (l->f) {
        auto ls = std::static_pointer_cast<LearnedSmoother<float>>(l->impl);
        fn = [ls]() {
            ls->use_fallback = true;
            ls->blas.ctx->epoch++;
        };
    } else {
        auto ls = std::static_pointer_cast<LearnedSmoother<double>>(l->impl);
        fn = [ls]() {
            ls->use_fallback = true;
            ls->blas.ctx->epoch++;
        };
    }
    if (h->kind == "cg") {
        if (h->f)
            std::static_pointer_cast<ConjugateGradient<float>>(h->impl)->on_stagnation = fn;
        else
            std::static_pointer_cast<ConjugateGradient<double>>(h->impl)->on_stagnation = fn;
    } else if (h->kind == "ir") {
        std::static_pointer_cast<IterativeRefinement>(h->impl)->on_stagnation = fn;
    } else {
        return set_error("sfem_gb300_solver_set_fallback: handle of kind '%s' has no residual monitor", h->kind.c_str());
    }
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_solver_fallback_used(void *solver, int *used) {
    auto *h = H(solver);
    *used = 0;
    if (h->kind == "cg")
        *used = h->f ? std::static_pointer_cast<ConjugateGradient<float>>(h->impl)->stagnated
                     : std::static_pointer_cast<ConjugateGradient<double>>(h->impl)->stagnated;
    else if (h->kind == "ir")
        *used = std::static_pointer_cast<IterativeRefinement>(h->impl)->stagnated;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_learned_smoother_set_chain(void *solver, int chain) {
    auto *h = H(solver);
    if (h->kind != "learned") return set_error("not a learned-smoother handle");
    if (chain < 0 || chain > 2) return set_error("sfem_gb300_learned_smoother_set_chain: chain must be 0, 1 or 2");
    if (h->f) {
        auto ls = std::static_pointer_cast<LearnedSmoother<float>>(h->impl);
        ls->chain = chain;
        ls->blas.ctx->epoch++;
    } else {
        auto ls = std::static_pointer_cast<LearnedSmoother<double>>(h->impl);
        ls->chain = chain;
        ls->blas.ctx->epoch++;
    }
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_learned_smoother_use_fallback(void *solver, int use_fallback) {
    auto *h = H(solver);
    if (h->kind != "learned") return set_error("not a learned-smoother handle");
    if (h->f) {
        auto ls = std::static_pointer_cast<LearnedSmoother<float>>(h->impl);
        ls->use_fallback = use_fallback != 0;
        ls->blas.ctx->epoch++;
    } else {
        auto ls = std::static_pointer_cast<LearnedSmoother<double>>(h->impl);
        ls->use_fallback = use_fallback != 0;
        ls->blas.ctx->epoch++;
    }
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_mg_set_post_smoother(void *mg, int level, void *smoother) {
    auto *h = H(mg);
    if (h->kind != "mg") return set_error("not a multigrid handle");
    auto *s = H(smoother);
    if (h->f) {
        auto m = std::static_pointer_cast<Multigrid<float>>(h->impl);
        if (level < 0 || level >= (int)m->levels.size()) return set_error("mg_set_post_smoother: bad level");
        m->levels[level].post_smoother = s->f;
        m->release_graphs();
    } else {
        auto m = std::static_pointer_cast<Multigrid<double>>(h->impl);
        if (level < 0 || level >= (int)m->levels.size()) return set_error("mg_set_post_smoother: bad level");
        m->levels[level].post_smoother = s->d;
        m->release_graphs();
    }
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_mg_set_pre_smoother(void *mg, int level, void *smoother) {
    auto *h = H(mg);
    if (h->kind != "mg") return set_error("not a multigrid handle");
    auto *s = H(smoother);
    if (h->f) {
        auto m = std::static_pointer_cast<Multigrid<float>>(h->impl);
        if (level < 0 || level >= (int)m->levels.size()) return set_error("mg_set_pre_smoother: bad level");
        m->levels[level].smoother = s->f;
        m->release_graphs();
    } else {
        auto m = std::static_pointer_cast<Multigrid<double>>(h->impl);
        if (level < 0 || level >= (int)m->levels.size()) return set_error("mg_set_pre_smoother: bad level");
        m->levels[level].smoother = s->d;
        m->release_graphs();
    }
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_crs_transfer_op_create(void *context, int real_type, ptrdiff_t nrows, ptrdiff_t ncols,
                                      const idx_t *rowptr, const idx_t *colidx, const double *weights, int vec_size,
                                      ptrdiff_t n_dirichlet, const idx_t *dirichlet, void **out) {
    auto *c = H(context);
    auto *h = new Handle();
    h->kind = "crs_transfer";
    h->ctx = c->ctx;
    h->real_type = is_f32(real_type) ? SFEM_GB300_FLOAT32 : SFEM_GB300_FLOAT64;
    auto fill = [&](auto op) {
        op->ctx = c->ctx;
        op->nrows = nrows;
        op->ncols = ncols;
        op->rowptr = rowptr;
        op->colidx = colidx;
        op->weights = weights;
        op->vec = vec_size;
        op->n_dirichlet = n_dirichlet;
        op->dirichlet = dirichlet;
    };
    if (is_f32(real_type)) {
        auto op = std::make_shared<CrsTransferOp<float>>();
        fill(op);
        h->f = op;
    } else {
        auto op = std::make_shared<CrsTransferOp<double>>();
        fill(op);
        h->d = op;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_dense_solver_create(void *context, void *op, void **out) {
    auto *c = H(context);
    auto *o = H(op);
    auto *h = new Handle();
    h->kind = "dense";
    h->ctx = c->ctx;
    h->real_type = o->real_type;
    auto make = [&](auto tag) -> int {
        using T = decltype(tag);
        auto s = std::make_shared<DenseCoarseSolver<T>>();
        s->blas = blas_of<T>(c->ctx);
        s->op = op_of<T>(o);
        op_of<T>(h) = s;
        h->impl = s;
        return s->setup();
    };
    const int rc = o->f ? make(0.0f) : make(0.0);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_mg_set_graph(void *mg, int enable) {
    auto *h = H(mg);
    if (h->kind != "mg") return set_error("not a multigrid handle");
    if (h->f) {
        auto m = std::static_pointer_cast<Multigrid<float>>(h->impl);
        m->release_graphs();
        m->use_graph = enable != 0;
    } else {
        auto m = std::static_pointer_cast<Multigrid<double>>(h->impl);
        m->release_graphs();
        m->use_graph = enable != 0;
    }
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_mg_set_harvest(void *mg, void *x_cc) {
    auto *h = H(mg);
    if (h->kind != "mg") return set_error("not a multigrid handle");
    if (h->f)
    {
        auto m = std::static_pointer_cast<Multigrid<float>>(h->impl);
        m->harvest = (float *)x_cc;
        m->release_graphs();
    } else {
        auto m = std::static_pointer_cast<Multigrid<double>>(h->impl);
        m->harvest = (double *)x_cc;
        m->release_graphs();
    }
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_ir_create(void *context, void *op64, void *inner32, int max_it, double rtol, void **out) {
    auto *c = H(context);
    auto *o = H(op64), *in = H(inner32);
    if (!o->d || !in->f) return set_error("sfem_gb300_ir_create: needs a double operator and a float inner solver");
    auto *h = new Handle();
    h->kind = "ir";
    h->ctx = c->ctx;
    h->real_type = SFEM_GB300_FLOAT64;
    auto s = std::make_shared<IterativeRefinement>();
    s->ctx = c->ctx;
    s->op = o->d;
    s->inner = in->f;
    s->max_it = max_it;
    s->rtol = rtol;
    h->d = s;
    h->impl = s;
    *out = h;
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_solver_apply(void *solver, const void *b, void *x) { return sfem_gb300_op_apply(solver, b, x); }
int sfem_gb300_mixed_precond_create(void *context, void *inner32, void **out) {
    auto *c = H(context);
    auto *in = H(inner32);
    if (!in->f) return set_error("sfem_gb300_mixed_precond_create: inner operator must be float");
    auto inner = in->f;
    auto ctx = c->ctx;
    double *slot = ctx->slots(1);
    if (!slot) return set_error("sfem_gb300_mixed_precond_create: out of scalar slots");
    const ptrdiff_t n = inner->rows();
    auto r32 = std::make_shared<DeviceBuffer<float>>(n);
    auto z32 = std::make_shared<DeviceBuffer<float>>(n);
    if (n > 0 && (!r32->ptr || !z32->ptr)) return set_error("sfem_gb300_mixed_precond_create: allocation failed");
    auto op = make_op<double>(n, n, [ctx, inner, slot, r32, z32, n](const double *r, double *z) {
        void *sp = ctx->sp();
        SFEM_GB300_CHECK(sfem_gb300_norm2(SFEM_GB300_FLOAT64, n, r, ctx->workspace, slot, sp));
        SFEM_GB300_CHECK(sfem_gb300_scaled_to_f32(n, slot, r, r32->ptr, sp));
        SFEM_GB300_CUDA(cudaMemsetAsync(z32->ptr, 0, n * sizeof(float), ctx->stream));
        SFEM_GB300_CHECK(inner->apply(r32->ptr, z32->ptr));
        return sfem_gb300_scaled_axpy_f32_to_f64(n, slot, z32->ptr, z, sp);
    });
    auto *h = new Handle();
    h->kind = "mixed_precond";
    h->ctx = ctx;
    h->real_type = SFEM_GB300_FLOAT64;
    h->d = op;
    *out = h;
    return SFEM_GB300_SUCCESS;
}


int sfem_gb300_solver_stats(void *solver, int *iterations, double *last_relative) {
    auto *h = H(solver);
    *iterations = 0;
    if (last_relative) *last_relative = 0;
    if (h->kind == "cg") {
        if (h->f) {
            auto s = std::static_pointer_cast<ConjugateGradient<float>>(h->impl);
            *iterations = s->iterations_;
            if (last_relative) *last_relative = s->last_rel;
        } else {
            auto s = std::static_pointer_cast<ConjugateGradient<double>>(h->impl);
            *iterations = s->iterations_;
            if (last_relative) *last_relative = s->last_rel;
        }
    } else if (h->kind == "ir") {
        auto s = std::static_pointer_cast<IterativeRefinement>(h->impl);
        *iterations = s->iterations_;
        if (last_relative) *last_relative = s->last_rel;
    } else if (h->kind == "mg") {
        if (h->f)
            *iterations = std::static_pointer_cast<Multigrid<float>>(h->impl)->iterations_;
        else
            *iterations = std::static_pointer_cast<Multigrid<double>>(h->impl)->iterations_;
    }
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_cg_set_options(void *solver, int residual_norm, int flexible, int check_every) {
    auto *h = H(solver);
    if (h->kind != "cg") return set_error("not a cg handle");
    auto set = [&](auto cg) {
        cg->residual_norm = residual_norm != 0;
        cg->flexible = flexible != 0;
        cg->check_every = check_every < 1 ? 1 : check_every;
    };
    if (h->f)
        set(std::static_pointer_cast<ConjugateGradient<float>>(h->impl));
    else
        set(std::static_pointer_cast<ConjugateGradient<double>>(h->impl));
    return SFEM_GB300_SUCCESS;
}

int sfem_gb300_cg_set_verbose(void *solver, int verbose) {
    auto *h = H(solver);
    if (h->kind != "cg") return set_error("not a cg handle");
    if (h->f)
        std::static_pointer_cast<ConjugateGradient<float>>(h->impl)->verbose = verbose;
    else
        std::static_pointer_cast<ConjugateGradient<double>>(h->impl)->verbose = verbose;
    return SFEM_GB300_SUCCESS;
}

}  // extern "C"
