// Device-resident host solver layer: C++ mirror of the reference's solver
// templates on top of the sfem_gb300 C ABI.
//
//   Operator<T>            algebra/sfem_Operator.hpp:13-33   (apply(x, y), rows, cols)
//   ConjugateGradient<T>   algebra/sfem_cg.hpp:79-453        (PCG; stop on sqrt(rtz)/sqrt(rtz0))
//   Chebyshev3<T>          algebra/sfem_Chebyshev3.hpp:56-312 + PowerMethod (sfem_PowerMethod.hpp:12-55)
//   ShiftableJacobi<T>     algebra/sfem_ShiftableJacobi.hpp:15-65
//   StationaryIteration<T> algebra/sfem_Stationary.hpp:19-133
//   Multigrid<T>           algebra/sfem_Multigrid.hpp:27-354 (V/W cycle)
//
// All vectors live on the GPU; scalars produced by reductions stay on the
// device and feed the fused update kernels directly.  The host reads one
// scalar per Krylov iteration (the convergence test), like the reference's
// device BLAS does for every dot.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "sfem_gb300.h"

namespace sfem_gb300 {

template <typename T>
constexpr int real_type_v = sizeof(T) == 8 ? SFEM_GB300_FLOAT64 : SFEM_GB300_FLOAT32;

#define SFEM_GB300_CHECK(expr)                  \
    do {                                        \
        if ((expr) != SFEM_GB300_SUCCESS) {     \
            return SFEM_GB300_FAILURE;          \
        }                                       \
    } while (0)

#define SFEM_GB300_CUDA(expr)                                                                                   \
    do {                                                                                                        \
        cudaError_t _e = (expr);                                                                                \
        if (_e != cudaSuccess) return set_error("%s:%d: %s", __FILE__, __LINE__, cudaGetErrorString(_e)); \
    } while (0)

int set_error(const char *fmt, ...);

// Dirichlet dofs of every block component in one launch (the per-component C entry points
// sfem_gb300_constraint_nodes_copy / _to_value launch once per component)
int constraint_copy_block(int real_type, ptrdiff_t n_nodes, const int32_t *nodes, int block_size, const void *src,
                          void *dest, void *stream);
int constraint_value_block(int real_type, ptrdiff_t n_nodes, const int32_t *nodes, int block_size, double value,
                           void *x, void *stream);

// -------------------------------------------------------------------------- buffers

// Owning device buffer.
template <typename T>
struct DeviceBuffer {
    T *ptr{nullptr};
    ptrdiff_t n{0};
    DeviceBuffer() = default;
    explicit DeviceBuffer(ptrdiff_t size) { resize(size); }
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    DeviceBuffer(DeviceBuffer &&o) noexcept : ptr(o.ptr), n(o.n) {
        o.ptr = nullptr;
        o.n = 0;
    }
    DeviceBuffer &operator=(DeviceBuffer &&o) noexcept {
        if (this != &o) {
            release();
            ptr = o.ptr;
            n = o.n;
            o.ptr = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DeviceBuffer() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        n = 0;
    }
    int resize(ptrdiff_t size) {
        if (size == n && ptr) return 0;
        release();
        n = size;
        if (size > 0 && cudaMalloc((void **)&ptr, size * sizeof(T)) != cudaSuccess) {
            ptr = nullptr;
            n = 0;
            return set_error("cudaMalloc of %zd bytes failed", (size_t)(size * sizeof(T)));
        }
        return 0;
    }
    T *data() const { return ptr; }
};

// Stream + reduction workspace + device scalar slots shared by the solvers of one
// hierarchy.  Slots are handed out from blocks of kSlotBlock doubles; a full block
// is kept (its slots stay valid) and a new one is allocated, so a context can
// serve any number of solver objects.
struct Context {
    static constexpr int kSlotBlock = 1024;
    cudaStream_t stream{0};
    void *workspace{nullptr};
    std::vector<double *> blocks;
    int next_slot{kSlotBlock};
    double *h_scalar{nullptr};  // pinned staging for host reads
    // bumped whenever a solver changes which kernels it launches (e.g. a learned
    // smoother switching to its fallback): captured CUDA graphs of older epochs are stale
    uint64_t epoch{0};

    static std::shared_ptr<Context> create(cudaStream_t s, int = 0) {
        auto c = std::make_shared<Context>();
        c->stream = s;
        if (cudaMalloc(&c->workspace, sfem_gb300_reduce_workspace_size()) != cudaSuccess) return nullptr;
        if (cudaMemset(c->workspace, 0, sfem_gb300_reduce_workspace_size()) != cudaSuccess) return nullptr;
        if (cudaMallocHost((void **)&c->h_scalar, sizeof(double)) != cudaSuccess) return nullptr;
        return c;
    }
    ~Context() {
        if (workspace) cudaFree(workspace);
        for (double *b : blocks) cudaFree(b);
        if (h_scalar) cudaFreeHost(h_scalar);
    }
    // Reserve k consecutive device scalar slots (zero-initialised).
    double *slots(int k) {
        if (k > kSlotBlock) return nullptr;
        if (next_slot + k > kSlotBlock) {
            double *b = nullptr;
            if (cudaMalloc((void **)&b, kSlotBlock * sizeof(double)) != cudaSuccess) return nullptr;
            if (cudaMemset(b, 0, kSlotBlock * sizeof(double)) != cudaSuccess) return nullptr;
            blocks.push_back(b);
            next_slot = 0;
        }
        double *p = blocks.back() + next_slot;
        next_slot += k;
        return p;
    }
    void *sp() { return stream ? (void *)&stream : nullptr; }
    // Copy one device scalar to the host (synchronizes the stream).
    double read(const double *d) {
        cudaMemcpyAsync(h_scalar, d, sizeof(double), cudaMemcpyDeviceToHost, stream);
        cudaStreamSynchronize(stream);
        return *h_scalar;
    }
};

// BLAS<T> on the device (algebra/sfem_tpl_blas.hpp:11-35) through the C ABI.
template <typename T>
struct Blas {
    std::shared_ptr<Context> ctx;
    static constexpr int rt = real_type_v<T>;
    int zeros(ptrdiff_t n, T *x) const {
        return n > 0 && cudaMemsetAsync(x, 0, n * sizeof(T), ctx->stream) != cudaSuccess ? set_error("memset") : 0;
    }
    int copy(ptrdiff_t n, const T *src, T *dst) const {
        return n > 0 && cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess
                       ? set_error("memcpy")
                       : 0;
    }
    int values(ptrdiff_t n, T v, T *x) const { return sfem_gb300_values(rt, n, v, x, ctx->sp()); }
    int axpby(ptrdiff_t n, T a, const T *x, T b, T *y) const { return sfem_gb300_axpby(rt, n, a, x, b, y, ctx->sp()); }
    int axpy(ptrdiff_t n, T a, const T *x, T *y) const { return sfem_gb300_axpy(rt, n, a, x, y, ctx->sp()); }
    int zaxpby(ptrdiff_t n, T a, const T *x, T b, const T *y, T *z) const {
        return sfem_gb300_zaxpby(rt, n, a, x, b, y, z, ctx->sp());
    }
    int scal(ptrdiff_t n, T a, T *x) const { return sfem_gb300_scal(rt, n, a, x, ctx->sp()); }
    int reciprocal(ptrdiff_t n, T a, T *x) const { return sfem_gb300_reciprocal(rt, n, a, x, ctx->sp()); }
    int xypaz(ptrdiff_t n, const T *x, const T *y, T a, T *z) const { return sfem_gb300_xypaz(rt, n, x, y, a, z, ctx->sp()); }
    int dot(ptrdiff_t n, const T *x, const T *y, double *d_result) const {
        return sfem_gb300_dot(rt, n, x, y, ctx->workspace, d_result, ctx->sp());
    }
    int norm2(ptrdiff_t n, const T *x, double *d_result) const {
        return sfem_gb300_norm2(rt, n, x, ctx->workspace, d_result, ctx->sp());
    }
};

// -------------------------------------------------------------------------- operators

// algebra/sfem_Operator.hpp:13-33.  Linear operators accumulate (y += A x);
// solvers used as operators take (b, x) with x as the initial guess.
template <typename T>
class Operator {
public:
    using value_type = T;
    virtual ~Operator() = default;
    virtual int apply(const T *x, T *y) = 0;
    virtual ptrdiff_t rows() const = 0;
    virtual ptrdiff_t cols() const = 0;
    // true if apply overwrites y instead of accumulating
    virtual bool overwrites_output() const { return false; }
};

template <typename T>
class LambdaOperator final : public Operator<T> {
public:
    ptrdiff_t r{0}, c{0};
    bool overwrites{false};
    std::function<int(const T *, T *)> fn;
    int apply(const T *x, T *y) override { return fn(x, y); }
    ptrdiff_t rows() const override { return r; }
    ptrdiff_t cols() const override { return c; }
    bool overwrites_output() const override { return overwrites; }
};

template <typename T>
std::shared_ptr<Operator<T>> make_op(ptrdiff_t rows, ptrdiff_t cols, std::function<int(const T *, T *)> fn,
                                     bool overwrites = false) {
    auto op = std::make_shared<LambdaOperator<T>>();
    op->r = rows;
    op->c = cols;
    op->fn = std::move(fn);
    op->overwrites = overwrites;
    return op;
}

// -------------------------------------------------------------------------- solvers

template <typename T>
class Solver : public Operator<T> {
public:
    int iterations_{0};
    virtual int iterations() const { return iterations_; }
};

// PowerMethod (algebra/sfem_PowerMethod.hpp:18-55): largest eigenvalue by normalised power iteration.
template <typename T>
double power_method_max_eigenvalue(const Blas<T> &blas, Operator<T> &op, int max_it, double tol, ptrdiff_t n,
                                   T *ev, T *work, double *d_slot) {
    const int max_it_odd = max_it + (max_it % 2 == 0);
    blas.zeros(n, work);
    op.apply(ev, work);
    blas.norm2(n, work, d_slot);
    double nrm = blas.ctx->read(d_slot);
    blas.scal(n, T(1.0 / nrm), work);
    T *vecs[2] = {ev, work};
    double lambda = 0, lambda_old = 0;
    for (int k = 0; k < max_it_odd; k++) {
        T *w = vecs[k % 2];
        T *v = vecs[(k + 1) % 2];
        blas.zeros(n, w);
        op.apply(v, w);
        blas.norm2(n, w, d_slot);
        lambda = blas.ctx->read(d_slot);
        blas.scal(n, T(1.0 / lambda), w);
        if (std::fabs(lambda - lambda_old) <= tol && k % 2 == 0) break;
        lambda_old = lambda;
    }
    return lambda;
}

// Chebyshev3 (algebra/sfem_Chebyshev3.hpp:183-302).  With inv_diag set, the
// iteration (and the power method) run on the Jacobi-scaled operator D^-1 A.
template <typename T>
class Chebyshev3 final : public Solver<T> {
public:
    Blas<T> blas;
    std::shared_ptr<Operator<T>> op;
    const T *inv_diag{nullptr};
    DeviceBuffer<T> p, temp;
    double eig_max{0}, scale_eig_max{1.02}, scale_eig_min{0.06};
    int max_it{3};
    bool initial_guess_zero{false};
    int eigen_max_it{1000};
    double eigen_tol{1e-6};

    int init(const T *guess) {
        const ptrdiff_t n = op->rows();
        SFEM_GB300_CHECK(p.resize(n));
        SFEM_GB300_CHECK(temp.resize(n));
        blas.copy(n, guess, temp.ptr);
        double *slot = blas.ctx->slots(1);
        if (!slot) return set_error("Chebyshev3: out of scalar slots");
        std::shared_ptr<Operator<T>> pm_op = op;
        DeviceBuffer<T> scratch;
        if (inv_diag) {
            SFEM_GB300_CHECK(scratch.resize(n));
            auto A = op;
            auto b = blas;
            const T *d = inv_diag;
            T *tmp = scratch.ptr;
            pm_op = make_op<T>(n, n, [A, b, d, tmp, n](const T *x, T *y) {
                b.zeros(n, tmp);
                A->apply(x, tmp);
                return b.xypaz(n, d, tmp, T(1), y);
            });
        }
        eig_max = power_method_max_eigenvalue(blas, *pm_op, eigen_max_it, eigen_tol, n, temp.ptr, p.ptr, slot);
        return blas.zeros(n, p.ptr);
    }
    int init_with_ones() {
        DeviceBuffer<T> ones(op->rows());
        blas.values(op->rows(), T(1), ones.ptr);
        return init(ones.ptr);
    }
    // Seeded U(-1,1) start vector: unlike the constant vector it has components
    // in the highest modes, so the power method does not underestimate lambda_max.
    int init_with_random(unsigned long long seed) {
        DeviceBuffer<T> v(op->rows());
        SFEM_GB300_CHECK(sfem_gb300_random_uniform(real_type_v<T>, op->rows(), seed, v.ptr, blas.ctx->sp()));
        return init(v.ptr);
    }
    int apply(const T *b, T *x) override {
        const ptrdiff_t n = op->rows();
        if (max_it <= 0) return 0;
        const double emax = eig_max * scale_eig_max;
        const double emin = scale_eig_min * emax;
        const double eavg = (emin + emax) / 2, ediff = (emin - emax) / 2;
        double alpha = 1.0 / eavg, beta = 0, dea = 0;
        blas.zeros(n, temp.ptr);
        if (!initial_guess_zero) op->apply(x, temp.ptr);
        SFEM_GB300_CHECK(sfem_gb300_chebyshev_update(real_type_v<T>, n, alpha, 0.0, inv_diag, b, temp.ptr, p.ptr, x,
                                                     blas.ctx->sp()));
        this->iterations_ = 1;
        for (; this->iterations_ < max_it; this->iterations_++) {
            dea = ediff * alpha;
            beta = (this->iterations_ == 1 ? 0.5 : 0.25) * dea * dea;
            alpha = 1.0 / (eavg - beta / alpha);
            if (!op->overwrites_output()) blas.zeros(n, temp.ptr);
            op->apply(x, temp.ptr);
            SFEM_GB300_CHECK(sfem_gb300_chebyshev_update(real_type_v<T>, n, alpha, beta, inv_diag, b, temp.ptr, p.ptr, x,
                                                         blas.ctx->sp()));
        }
        return 0;
    }
    ptrdiff_t rows() const override { return op->rows(); }
    ptrdiff_t cols() const override { return op->cols(); }
};

// ShiftableJacobi (algebra/sfem_ShiftableJacobi.hpp:15-65): x += omega D^{-1} b.
template <typename T>
class Jacobi final : public Solver<T> {
public:
    Blas<T> blas;
    DeviceBuffer<T> inv_diag;
    double relaxation{1.0};
    int set_diag(const T *diag, ptrdiff_t n) {
        SFEM_GB300_CHECK(inv_diag.resize(n));
        blas.copy(n, diag, inv_diag.ptr);
        return blas.reciprocal(n, T(relaxation), inv_diag.ptr);
    }
    int apply(const T *b, T *x) override { return blas.xypaz(inv_diag.n, inv_diag.ptr, b, T(1), x); }
    ptrdiff_t rows() const override { return inv_diag.n; }
    ptrdiff_t cols() const override { return inv_diag.n; }
};

// ShiftableBlockSymJacobi (algebra/sfem_ShiftableJacobi.hpp:67-155): x += B b with
// pre-inverted symmetric 3x3 blocks (6 per node).
template <typename T>
class BlockJacobi final : public Solver<T> {
public:
    Blas<T> blas;
    const T *inv_block6{nullptr};
    ptrdiff_t n_nodes{0};
    int apply(const T *b, T *x) override {
        return sfem_gb300_block3_apply(real_type_v<T>, n_nodes, inv_block6, b, x, blas.ctx->sp());
    }
    ptrdiff_t rows() const override { return 3 * n_nodes; }
    ptrdiff_t cols() const override { return 3 * n_nodes; }
};

// Learned patch smoother (no reference counterpart), see sfem_gb300_learned_smoother_create.
template <typename T>
class LearnedSmoother final : public Solver<T> {
public:
    Blas<T> blas;
    std::shared_ptr<Operator<T>> op, fallback;
    idx_t **elements{nullptr};
    ptrdiff_t nelements{0};
    const uint16_t *count{nullptr};
    const T *inv_diag{nullptr};
    const idx_t *dirichlet{nullptr};  // the correction is zero on these nodes
    ptrdiff_t n_dirichlet{0};
    const void *W[3]{nullptr, nullptr, nullptr};
    int channels{16}, sweeps{1};
    double omega{1.0};
    bool use_fallback{false};
    int chain{0};  // 1: the fallback smoother first, then the learned corrections; 2: learned first, then fallback
    bool line_search{true};   // step length minimising the energy norm of the error along the correction
    bool fused{true};  // one tensor-core kernel for gather + network + scatter
    DeviceBuffer<T> r, d, Ad;
    DeviceBuffer<uint16_t> a0, a1, a2, a3;  // BF16 activations (unfused path)
    DeviceBuffer<float> pscale;
    DeviceBuffer<unsigned char> frag;  // B fragments of the three layers (fused path)
    double *s{nullptr};  // device scalars: (d, r), (d, A d)
    // One sweep: r = b - A x; d = net(D^-1 r patches) scattered and zeroed on
    // Dirichlet nodes; x += alpha d with alpha = (d, r) / (d, A d) computed on the
    // device.  For SPD A that alpha minimises ||x* - x - alpha d||_A, so a poor
    // correction can only be scaled down, never increase the error energy.
    int apply(const T *b, T *x) override {
        if (fallback && (chain == 1 || use_fallback)) SFEM_GB300_CHECK(fallback->apply(b, x));
        if (use_fallback) return 0;
        SFEM_GB300_CHECK(learned_sweeps(b, x));
        if (fallback && chain == 2) SFEM_GB300_CHECK(fallback->apply(b, x));
        return 0;
    }
    int learned_sweeps(const T *b, T *x) {
        const ptrdiff_t n = op->rows();
        const ptrdiff_t P = nelements;
        SFEM_GB300_CHECK(r.resize(n));
        SFEM_GB300_CHECK(d.resize(n));
        SFEM_GB300_CHECK(Ad.resize(n));
        if (fused) {
            SFEM_GB300_CHECK(frag.resize((ptrdiff_t)sfem_gb300_learned_fragments_size()));
        } else {
            SFEM_GB300_CHECK(a0.resize(P * 125));
            SFEM_GB300_CHECK(a1.resize(P * 125 * channels));
            SFEM_GB300_CHECK(a2.resize(P * 125 * channels));
            SFEM_GB300_CHECK(a3.resize(P * 125));
            SFEM_GB300_CHECK(pscale.resize(P));
        }
        if (!s) s = blas.ctx->slots(2);
        if (!s) return set_error("LearnedSmoother: out of scalar slots");
        void *sp = blas.ctx->sp();
        if (fused) SFEM_GB300_CHECK(sfem_gb300_learned_fragments(W[0], W[1], W[2], frag.ptr, sp));
        for (this->iterations_ = 0; this->iterations_ < sweeps; this->iterations_++) {
            blas.zeros(n, r.ptr);
            SFEM_GB300_CHECK(op->apply(x, r.ptr));
            blas.axpby(n, T(1), b, T(-1), r.ptr);
            T *target = line_search ? d.ptr : x;
            if (line_search) blas.zeros(n, d.ptr);
            if (fused) {
                SFEM_GB300_CHECK(sfem_gb300_learned_correction(real_type_v<T>, P, elements, r.ptr, inv_diag, frag.ptr,
                                                               count, omega, target, sp));
            } else {
                SFEM_GB300_CHECK(sfem_gb300_gather_patches(real_type_v<T>, P, elements, r.ptr, inv_diag, a0.ptr,
                                                           pscale.ptr, sp));
                SFEM_GB300_CHECK(sfem_gb300_patchconv_forward(P, 1, channels, a0.ptr, W[0], 1, a1.ptr, sp));
                SFEM_GB300_CHECK(sfem_gb300_patchconv_forward(P, channels, channels, a1.ptr, W[1], 1, a2.ptr, sp));
                SFEM_GB300_CHECK(sfem_gb300_patchconv_forward(P, channels, 1, a2.ptr, W[2], 0, a3.ptr, sp));
                SFEM_GB300_CHECK(sfem_gb300_scatter_patches(real_type_v<T>, P, elements, a3.ptr, pscale.ptr, count,
                                                            omega, target, sp));
            }
            if (!line_search) continue;
            if (n_dirichlet > 0)
                SFEM_GB300_CHECK(sfem_gb300_constraint_nodes_to_value(real_type_v<T>, n_dirichlet, dirichlet, 1, 0, 0.0,
                                                                      d.ptr, sp));
            blas.zeros(n, Ad.ptr);
            SFEM_GB300_CHECK(op->apply(d.ptr, Ad.ptr));
            SFEM_GB300_CHECK(blas.dot(n, d.ptr, r.ptr, &s[0]));
            SFEM_GB300_CHECK(blas.dot(n, d.ptr, Ad.ptr, &s[1]));
            // x += alpha d (r is scratch from here on)
            SFEM_GB300_CHECK(sfem_gb300_cg_update_x_r(real_type_v<T>, n, &s[0], &s[1], d.ptr, Ad.ptr, x, r.ptr,
                                                      blas.ctx->workspace, nullptr, sp));
        }
        return 0;
    }
    ptrdiff_t rows() const override { return op->rows(); }
    ptrdiff_t cols() const override { return op->cols(); }
};

// StationaryIteration (algebra/sfem_Stationary.hpp:19-133): x += P (b - A x), max_it sweeps.
template <typename T>
class Stationary final : public Solver<T> {
public:
    Blas<T> blas;
    std::shared_ptr<Operator<T>> op, precond;
    DeviceBuffer<T> r;
    int max_it{3};
    int apply(const T *b, T *x) override {
        const ptrdiff_t n = op->rows();
        SFEM_GB300_CHECK(r.resize(n));
        for (this->iterations_ = 0; this->iterations_ < max_it; this->iterations_++) {
            if (!op->overwrites_output()) blas.zeros(n, r.ptr);
            op->apply(x, r.ptr);
            blas.axpby(n, T(1), b, T(-1), r.ptr);
            precond->apply(r.ptr, x);
        }
        return 0;
    }
    ptrdiff_t rows() const override { return op->rows(); }
    ptrdiff_t cols() const override { return op->cols(); }
};

// ConjugateGradient (algebra/sfem_cg.hpp:79-453).  Default stopping test is the
// reference's: sqrt(rtz) < atol or sqrt(rtz)/sqrt(rtz0) < rtol.  Options:
// residual_norm (stop on ||r||/||r0||), flexible (Polak-Ribiere beta, FCG) and
// check_every (read the convergence scalar every k iterations only; all other
// scalars stay on the device).
template <typename T>
class ConjugateGradient final : public Solver<T> {
public:
    Blas<T> blas;
    std::shared_ptr<Operator<T>> op, precond;
    DeviceBuffer<T> r, z, zprev, p, Ap;
    int max_it{10000};
    double atol{1e-30}, rtol{1e-10};
    bool verbose{false};
    bool residual_norm{false}, flexible{false};
    int check_every{1};
    double last_rel{0};
    // called once when the monitored residual has not decreased for `patience`
    // consecutive checks (e.g. to switch a learned smoother to its fallback)
    std::function<void()> on_stagnation;
    int patience{2};
    bool stagnated{false};
    // slots: 0 rz, 1 rz_old, 2 pAp, 3 rr, 4 r.z_prev, 5 rr0
    double *s{nullptr};

    int apply(const T *b, T *x) override {
        const ptrdiff_t n = op->rows();
        if (!s) s = blas.ctx->slots(6);
        if (!s) return set_error("ConjugateGradient: out of scalar slots");
        SFEM_GB300_CHECK(r.resize(n));
        SFEM_GB300_CHECK(p.resize(n));
        SFEM_GB300_CHECK(Ap.resize(n));
        const bool pre = (bool)precond;
        const bool flex = pre && flexible;
        if (pre) SFEM_GB300_CHECK(z.resize(n));
        if (flex) SFEM_GB300_CHECK(zprev.resize(n));
        T *zz = pre ? z.ptr : r.ptr;
        T *zp = flex ? zprev.ptr : nullptr;
        if (!op->overwrites_output()) blas.zeros(n, r.ptr);
        op->apply(x, r.ptr);
        blas.axpby(n, T(1), b, T(-1), r.ptr);  // r = b - A x
        if (pre) {
            if (!precond->overwrites_output()) blas.zeros(n, z.ptr);
            precond->apply(r.ptr, z.ptr);
        }
        blas.copy(n, zz, p.ptr);
        blas.dot(n, r.ptr, zz, &s[0]);
        const bool use_rr = residual_norm && pre;
        if (use_rr) blas.dot(n, r.ptr, r.ptr, &s[5]);
        const double rz0 = blas.ctx->read(&s[0]);
        const double crit0 = use_rr ? blas.ctx->read(&s[5]) : rz0;
        last_rel = 1;
        this->iterations_ = 0;
        if (rz0 == 0 || crit0 == 0) return 0;
        const double norm0 = std::sqrt(std::fabs(crit0));
        const int every = check_every < 1 ? 1 : check_every;
        double best = 1.0;
        int bad = 0;
        stagnated = false;
        for (this->iterations_ = 0; this->iterations_ < max_it;) {
            if (!op->overwrites_output()) blas.zeros(n, Ap.ptr);
            op->apply(p.ptr, Ap.ptr);
            blas.dot(n, p.ptr, Ap.ptr, &s[2]);
            if (pre) {
                SFEM_GB300_CHECK(sfem_gb300_cg_update_x_r(real_type_v<T>, n, &s[0], &s[2], p.ptr, Ap.ptr, x, r.ptr,
                                                          blas.ctx->workspace, use_rr ? &s[3] : nullptr,
                                                          blas.ctx->sp()));
                if (flex) std::swap(zz, zp);
                if (!precond->overwrites_output()) blas.zeros(n, zz);
                precond->apply(r.ptr, zz);
                cudaMemcpyAsync(&s[1], &s[0], sizeof(double), cudaMemcpyDeviceToDevice, blas.ctx->stream);
                blas.dot(n, r.ptr, zz, &s[0]);
                if (flex) blas.dot(n, r.ptr, zp, &s[4]);
            } else {
                cudaMemcpyAsync(&s[1], &s[0], sizeof(double), cudaMemcpyDeviceToDevice, blas.ctx->stream);
                SFEM_GB300_CHECK(sfem_gb300_cg_update_x_r(real_type_v<T>, n, &s[1], &s[2], p.ptr, Ap.ptr, x, r.ptr,
                                                          blas.ctx->workspace, &s[0], blas.ctx->sp()));
            }
            this->iterations_++;
            if (this->iterations_ % every == 0 || this->iterations_ == max_it) {
                const double crit = blas.ctx->read(use_rr ? &s[3] : &s[0]);
                const double anorm = std::sqrt(std::fabs(crit));
                last_rel = anorm / norm0;
                if (verbose) printf("cg %d: %g %g\n", this->iterations_, anorm, last_rel);
                if (!std::isfinite(crit)) return set_error("ConjugateGradient: non-finite residual");
                if (anorm < atol || last_rel < rtol || crit == 0) return 0;
                if (last_rel < best) {
                    best = last_rel;
                    bad = 0;
                } else if (on_stagnation && !stagnated && ++bad >= patience) {
                    stagnated = true;
                    on_stagnation();
                }
            }
            SFEM_GB300_CHECK(sfem_gb300_cg_update_p(real_type_v<T>, n, &s[0], &s[1], flex ? &s[4] : nullptr, zz,
                                                    p.ptr, blas.ctx->sp()));
        }
        return set_error("ConjugateGradient: no convergence in %d iterations (rel %g)", max_it, last_rel);
    }
    ptrdiff_t rows() const override { return op->rows(); }
    ptrdiff_t cols() const override { return op->cols(); }
};

// Dense direct solve for a small coarsest level (no reference counterpart; the
// reference runs an iterative coarse solver).  The operator's n x n matrix is
// built on the device by n applies to unit vectors (one column each, no host round
// trip), inverted once on the device in FP64 (Gauss-Jordan, Dirichlet couplings
// folded back, dense.cu), and applied as x += A^-1 b with one dense matrix-vector
// kernel: no iteration count, no host synchronisation.
int dense_symv_add(int real_type, ptrdiff_t n, const void *M, const void *b, void *x, void *stream);
int dense_unit_vector(int real_type, ptrdiff_t n, ptrdiff_t j, void *e, void *stream);
int dense_inverse(int real_type, ptrdiff_t n, ptrdiff_t ld, const void *cols, double *A, double *S, double *rc,
                  int *flags, void *inv, void *stream);

template <typename T>
class DenseCoarseSolver final : public Solver<T> {
public:
    Blas<T> blas;
    std::shared_ptr<Operator<T>> op;
    DeviceBuffer<T> inv;  // row-major n x n
    static constexpr ptrdiff_t kMaxN = 1536;
    int setup() {
        const ptrdiff_t n = op->rows();
        if (n > kMaxN) return set_error("DenseCoarseSolver: %td unknowns exceed the dense limit %td", n, kMaxN);
        const ptrdiff_t ld = (n + 7) / 8 * 8;  // columns start 32-byte aligned
        DeviceBuffer<T> e(n), cols(ld * n);
        DeviceBuffer<double> A(n * n), S(n * n), rc(2 * n);
        DeviceBuffer<int> flags(n + 1);
        SFEM_GB300_CHECK(blas.zeros(ld * n, cols.ptr));
        for (ptrdiff_t j = 0; j < n; j++) {
            SFEM_GB300_CHECK(dense_unit_vector(real_type_v<T>, n, j, e.ptr, blas.ctx->sp()));
            SFEM_GB300_CHECK(op->apply(e.ptr, cols.ptr + j * ld));
        }
        SFEM_GB300_CHECK(inv.resize(n * n));
        return dense_inverse(real_type_v<T>, n, ld, cols.ptr, A.ptr, S.ptr, rc.ptr, flags.ptr, inv.ptr,
                             blas.ctx->sp());
    }
    int apply(const T *b, T *x) override {
        this->iterations_ = 1;
        return dense_symv_add(real_type_v<T>, op->rows(), inv.ptr, b, x, blas.ctx->sp());
    }
    ptrdiff_t rows() const override { return op->rows(); }
    ptrdiff_t cols() const override { return op->cols(); }
};

// Multigrid (algebra/sfem_Multigrid.hpp:27-354).  Level 0 is the finest.
template <typename T>
class Multigrid final : public Solver<T> {
public:
    struct Level {
        std::shared_ptr<Operator<T>> op, smoother, prolongation /* from next coarser */, restriction /* to coarser */;
        std::shared_ptr<Operator<T>> post_smoother;  // optional, defaults to smoother
        DeviceBuffer<T> rhs, sol, work;
    };
    Blas<T> blas;
    std::vector<Level> levels;
    int max_it{1};
    int cycle_type{1};
    // atol > 0 checks ||b - A x|| on the finest level after every pre-smoothing
    // (one host read per cycle, as algebra/sfem_Multigrid.hpp does); the default 0
    // skips the check, which is what a preconditioner (one cycle) wants and what
    // keeps a cycle free of host synchronisation (graph capture)
    double atol{0};
    double *s{nullptr};
    bool wrap_input{true};
    double norm_residual0{0}, norm_residual{0};
    // optional copy of the finest-level iterate after the coarse-grid correction
    // (before post-smoothing): the residual / error pairs a learned smoother trains on
    T *harvest{nullptr};

    void add_level(std::shared_ptr<Operator<T>> op, std::shared_ptr<Operator<T>> smoother,
                   std::shared_ptr<Operator<T>> prolongation, std::shared_ptr<Operator<T>> restriction) {
        Level l;
        l.op = op;
        l.smoother = smoother;
        l.prolongation = prolongation;
        l.restriction = restriction;
        levels.push_back(std::move(l));
    }
    int ensure_init() {
        if (!s) s = blas.ctx->slots(1);
        for (size_t i = 0; i < levels.size(); i++) {
            const ptrdiff_t n = levels[i].op->rows();
            if (i > 0 || !wrap_input) {
                SFEM_GB300_CHECK(levels[i].rhs.resize(n));
                SFEM_GB300_CHECK(levels[i].sol.resize(n));
            }
            SFEM_GB300_CHECK(levels[i].work.resize(n));
        }
        return 0;
    }
    // returns 1 if converged
    int cycle(int l, const T *rhs, T *sol) {
        Level &L = levels[l];
        const ptrdiff_t n = L.op->rows();
        if (l == (int)levels.size() - 1) {
            blas.zeros(n, sol);
            L.smoother->apply(rhs, sol);
            return 0;
        }
        Level &C = levels[l + 1];
        const ptrdiff_t nc = C.op->rows();
        for (int k = 0; k < cycle_type; k++) {
            L.smoother->apply(rhs, sol);
            if (!L.op->overwrites_output()) blas.zeros(n, L.work.ptr);
            L.op->apply(sol, L.work.ptr);
            blas.axpby(n, T(1), rhs, T(-1), L.work.ptr);
            if (l == 0 && atol > 0) {
                blas.norm2(n, L.work.ptr, s);
                norm_residual = blas.ctx->read(s);
                if (this->iterations_ == 0) norm_residual0 = norm_residual;
                if (norm_residual < atol) return 1;
            }
            blas.zeros(nc, C.rhs.ptr);
            L.restriction->apply(L.work.ptr, C.rhs.ptr);
            blas.zeros(nc, C.sol.ptr);
            cycle(l + 1, C.rhs.ptr, C.sol.ptr);
            blas.zeros(n, L.work.ptr);
            L.prolongation->apply(C.sol.ptr, L.work.ptr);
            blas.axpby(n, T(1), L.work.ptr, T(1), sol);
            if (l == 0 && harvest) blas.copy(n, sol, harvest);
            (L.post_smoother ? L.post_smoother : L.smoother)->apply(rhs, sol);
        }
        return 0;
    }
    // Graph mode: each (b, x) pair's cycles are captured once into a CUDA graph on
    // a private stream and replayed, ordered after / before the context stream
    // with events.  Every level operator and smoother must then be free of host
    // synchronisation (no iterative coarse solver with convergence checks).
    bool use_graph{false};
    struct GraphEntry {
        const T *b;
        T *x;
        cudaGraphExec_t exec;
    };
    std::vector<GraphEntry> graphs;
    uint64_t graph_epoch{0};
    cudaStream_t gstream{nullptr};
    cudaEvent_t ev_in{nullptr}, ev_out{nullptr};
    int warm{0};
    ~Multigrid() {
        release_graphs();
        if (ev_in) cudaEventDestroy(ev_in);
        if (ev_out) cudaEventDestroy(ev_out);
        if (gstream) cudaStreamDestroy(gstream);
    }
    void release_graphs() {
        for (auto &g : graphs) cudaGraphExecDestroy(g.exec);
        graphs.clear();
        warm = 0;
    }
    int run_cycles(const T *b, T *x) {
        for (this->iterations_ = 0; this->iterations_ < max_it; this->iterations_++) {
            if (cycle(0, b, x)) break;
        }
        return 0;
    }
    int apply(const T *b, T *x) override {
        SFEM_GB300_CHECK(ensure_init());
        if (use_graph && graph_epoch != blas.ctx->epoch) {
            release_graphs();
            graph_epoch = blas.ctx->epoch;
        }
        if (!use_graph || atol > 0 || warm < 1) {
            if (use_graph) warm++;  // first call eager: sizes every lazily allocated buffer
            return run_cycles(b, x);
        }
        Context &c = *blas.ctx;
        if (!gstream) {
            SFEM_GB300_CUDA(cudaStreamCreateWithFlags(&gstream, cudaStreamNonBlocking));
            SFEM_GB300_CUDA(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
            SFEM_GB300_CUDA(cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming));
        }
        cudaGraphExec_t exec = nullptr;
        for (auto &g : graphs)
            if (g.b == b && g.x == x) exec = g.exec;
        SFEM_GB300_CUDA(cudaEventRecord(ev_in, c.stream));
        SFEM_GB300_CUDA(cudaStreamWaitEvent(gstream, ev_in, 0));
        if (!exec) {
            if (graphs.size() >= 8) release_graphs();
            const cudaStream_t saved = c.stream;
            c.stream = gstream;
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamBeginCapture(gstream, cudaStreamCaptureModeThreadLocal);
            int rc = e == cudaSuccess ? run_cycles(b, x) : set_error("Multigrid capture: %s", cudaGetErrorString(e));
            cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(gstream, &graph) : cudaSuccess;
            c.stream = saved;
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (e2 != cudaSuccess) return set_error("Multigrid capture: %s", cudaGetErrorString(e2));
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return set_error("Multigrid graph instantiate: %s", cudaGetErrorString(e));
            graphs.push_back({b, x, exec});
        }
        SFEM_GB300_CUDA(cudaGraphLaunch(exec, gstream));
        SFEM_GB300_CUDA(cudaEventRecord(ev_out, gstream));
        SFEM_GB300_CUDA(cudaStreamWaitEvent(c.stream, ev_out, 0));
        return 0;
    }
    ptrdiff_t rows() const override { return levels[0].op->rows(); }
    ptrdiff_t cols() const override { return levels[0].op->cols(); }
};

}  // namespace sfem_gb300
