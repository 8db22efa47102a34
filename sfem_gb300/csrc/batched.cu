// Batched solves of many independent problems of uneven size (no reference
// counterpart: the reference solves one problem per process).
//
// Vectors of all problems are concatenated, problem p owning the dof range
// [offsets[p], offsets[p+1]).  Element operators and transfers need no batched
// form: the connectivity of several problems, concatenated with node offsets,
// is just a larger mesh, so one launch of the existing element kernels applies
// every problem of a (kind, level) group.  What is per problem is handled here:
//
//  * a work list of (problem, dof range) chunks drives every vector kernel;
//    kernels are persistent (grid = SMs x CTAs per SM, looping over the list);
//  * reductions write one partial per chunk, then one thread per problem sums
//    its partials in list order: results are deterministic;
//  * Krylov scalars (alpha, beta, residual norms, convergence masks) live in
//    device arrays of length P, so no iteration reads anything on the host;
//  * the outer solver is a batched FP64 flexible CG whose preconditioner runs the
//    per-group FP32 multigrid on per-problem normalised residuals (FP64 only for
//    the residual recurrence, dot products and solution update); chunks of
//    iterations are captured once into a CUDA graph and replayed, the host reads
//    the per-problem active mask once per chunk;
//  * the work-list chunk, the CTA shape of the vector kernels and the chunk length
//    are picked by an autotuner that times the captured chunk for each candidate.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>
#include <vector>

#include "common.cuh"
#include "capi_handle.hpp"
#include "solvers.hpp"

namespace sfem_gb300 {

struct BatchVecWork {
    int problem;
    int pad;
    long long start;  // first dof (concatenated index)
    long long end;    // one past the last dof of the chunk
};

constexpr int kBatchMaxThreads = 1024;

__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[w] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < nw; k++) s += red[k];
    return s;
}

// ---------------------------------------------------------------- reductions

template <typename TX, typename TY>
__global__ void bdot_kernel(int n_items, const BatchVecWork *__restrict__ work, const TX *__restrict__ x,
                            const TY *__restrict__ y, double *__restrict__ partials) {
    __shared__ double red[kBatchMaxThreads / 32];
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BatchVecWork w = work[it];
        double acc = 0;
        for (long long i = w.start + threadIdx.x; i < w.end; i += blockDim.x) acc += (double)x[i] * (double)y[i];
        const double s = block_sum(acc, red);
        if (threadIdx.x == 0) partials[it] = s;
    }
}

// out[p] = sum of the partials of problem p, items [first[p], first[p+1])
__global__ void bsum_kernel(int P, const int *__restrict__ first_item, const double *__restrict__ partials,
                            double *__restrict__ out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    double s = 0;
    for (int k = first_item[p]; k < first_item[p + 1]; k++) s += partials[k];
    out[p] = s;
}

// ---------------------------------------------------------------- elementwise

// alpha_p = num_p / den_p for active problems;  x += alpha p;  r -= alpha Ap;  partial (r, r)
template <typename T>
__global__ void bcg_update_x_r_kernel(int n_items, const BatchVecWork *__restrict__ work,
                                      const double *__restrict__ num, const double *__restrict__ den,
                                      const int *__restrict__ active, const T *__restrict__ p,
                                      const T *__restrict__ Ap, T *__restrict__ x, T *__restrict__ r,
                                      double *__restrict__ partials) {
    __shared__ double red[kBatchMaxThreads / 32];
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BatchVecWork w = work[it];
        const bool on = active[w.problem] != 0 && den[w.problem] != 0;
        const T alpha = on ? (T)(num[w.problem] / den[w.problem]) : T(0);
        double acc = 0;
        for (long long i = w.start + threadIdx.x; i < w.end; i += blockDim.x) {
            T ri = r[i];
            if (on) {
                x[i] += alpha * p[i];
                ri -= alpha * Ap[i];
                r[i] = ri;
            }
            acc += (double)ri * (double)ri;
        }
        const double s = block_sum(acc, red);
        if (threadIdx.x == 0) partials[it] = s;
    }
}

// beta_p = (num_p - sub_p) / den_p (0 if den_p == 0);  p = z + beta p  (active problems only)
template <typename T>
__global__ void bcg_update_p_kernel(int n_items, const BatchVecWork *__restrict__ work,
                                    const double *__restrict__ num, const double *__restrict__ den, const double *sub,
                                    const int *__restrict__ active, const T *__restrict__ z, T *__restrict__ p) {
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BatchVecWork w = work[it];
        if (!active[w.problem]) continue;
        const double d = den[w.problem];
        const T beta = d != 0 ? (T)((num[w.problem] - (sub ? sub[w.problem] : 0.0)) / d) : T(0);
        for (long long i = w.start + threadIdx.x; i < w.end; i += blockDim.x) p[i] = z[i] + beta * p[i];
    }
}

// Chebyshev step with per-problem coefficients: p = beta_p p + D^-1 (rhs - Ax); x += alpha_p p
template <typename T>
__global__ void bcheb_update_kernel(int n_items, const BatchVecWork *__restrict__ work,
                                    const double *__restrict__ alpha, const double *__restrict__ beta,
                                    const T *__restrict__ inv_diag, const T *__restrict__ rhs,
                                    const T *__restrict__ Ax, T *__restrict__ p, T *__restrict__ x) {
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BatchVecWork w = work[it];
        const T a = (T)alpha[w.problem], b = (T)beta[w.problem];
        for (long long i = w.start + threadIdx.x; i < w.end; i += blockDim.x) {
            T g = rhs[i] - Ax[i];
            if (inv_diag) g *= inv_diag[i];
            const T pi = (b != T(0) ? b * p[i] : T(0)) + g;
            p[i] = pi;
            x[i] += a * pi;
        }
    }
}

// v = w / sqrt(ww_p)  (power-method normalisation; 0 if ww_p == 0)
template <typename T>
__global__ void bnormalize_kernel(int n_items, const BatchVecWork *__restrict__ work, const double *__restrict__ ww,
                                  const T *__restrict__ w_in, T *__restrict__ v) {
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BatchVecWork w = work[it];
        const double n2 = ww[w.problem];
        const T s = n2 > 0 ? (T)(1.0 / sqrt(n2)) : T(0);
        for (long long i = w.start + threadIdx.x; i < w.end; i += blockDim.x) v[i] = w_in[i] * s;
    }
}

// r32 = inv_p * r64 (inv_p = 0 for inactive problems)
__global__ void bconvert_scaled_kernel(int n_items, const BatchVecWork *__restrict__ work,
                                       const double *__restrict__ inv, const double *__restrict__ r64,
                                       float *__restrict__ r32) {
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BatchVecWork w = work[it];
        const double s = inv[w.problem];
        for (long long i = w.start + threadIdx.x; i < w.end; i += blockDim.x) r32[i] = (float)(s * r64[i]);
    }
}

// x64 += scale_p * e32
__global__ void baxpy_f32_to_f64_kernel(int n_items, const BatchVecWork *__restrict__ work,
                                        const double *__restrict__ scale, const float *__restrict__ e32,
                                        double *__restrict__ x64) {
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BatchVecWork w = work[it];
        const double s = scale[w.problem];
        if (s == 0) continue;
        for (long long i = w.start + threadIdx.x; i < w.end; i += blockDim.x) x64[i] += s * (double)e32[i];
    }
}

// ---------------------------------------------------------------- per-problem scalar kernels

// CG start: active_p = rr0_p > 0 (and not NaN)
__global__ void bcg_start_kernel(int P, const double *__restrict__ rr0, int *__restrict__ active) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < P) active[p] = rr0[p] > 0 && rr0[p] == rr0[p];
}

// active_p <- active_p && rr_p > tol2 * rr0_p (a NaN also stops the problem)
__global__ void bcg_check_kernel(int P, const double *__restrict__ rr, const double *__restrict__ rr0, double tol2,
                                 int *__restrict__ active) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P || !active[p]) return;
    if (!(rr[p] > tol2 * rr0[p])) active[p] = 0;
}

// ---------------------------------------------------------------- layout

// Dof layout of one batch of concatenated vectors and its work list.
struct BatchLayout {
    std::shared_ptr<Context> ctx;
    int P{0};
    std::vector<long long> offsets;  // host, P + 1
    int chunk{4096};
    int threads{256};
    int ctas_per_sm{8};
    int n_items{0};
    DeviceBuffer<BatchVecWork> work;
    DeviceBuffer<int> first_item;
    DeviceBuffer<double> partials;

    long long n() const { return offsets.empty() ? 0 : offsets.back(); }
    int grid() const {
        const int g = kNumSMs * ctas_per_sm;
        return n_items < g ? (n_items > 0 ? n_items : 1) : g;
    }
    int pgrid() const { return (P + 127) / 128; }

    int build() {
        std::vector<BatchVecWork> items;
        std::vector<int> first(P + 1, 0);
        for (int p = 0; p < P; p++) {
            first[p] = (int)items.size();
            for (long long s = offsets[p]; s < offsets[p + 1]; s += chunk)
                items.push_back({p, 0, s, std::min<long long>(s + chunk, offsets[p + 1])});
        }
        first[P] = (int)items.size();
        n_items = (int)items.size();
        SFEM_GB300_CHECK(work.resize(std::max(1, n_items)));
        SFEM_GB300_CHECK(first_item.resize(P + 1));
        SFEM_GB300_CHECK(partials.resize(std::max(1, n_items)));
        if (n_items)
            SFEM_GB300_CUDA(cudaMemcpy(work.ptr, items.data(), n_items * sizeof(BatchVecWork), cudaMemcpyHostToDevice));
        SFEM_GB300_CUDA(cudaMemcpy(first_item.ptr, first.data(), (P + 1) * sizeof(int), cudaMemcpyHostToDevice));
        return 0;
    }

    template <typename TX, typename TY>
    int dot(const TX *x, const TY *y, double *out) {
        const cudaStream_t s = ctx->stream;
        bdot_kernel<TX, TY><<<grid(), threads, 0, s>>>(n_items, work.ptr, x, y, partials.ptr);
        bsum_kernel<<<pgrid(), 128, 0, s>>>(P, first_item.ptr, partials.ptr, out);
        return check_launch("batched dot");
    }
};

// ---------------------------------------------------------------- operators

// Block-diagonal operator: op g acts on the dof range [offsets[g], offsets[g+1]).
template <typename T>
class GroupedOperator final : public Operator<T> {
public:
    std::vector<std::shared_ptr<Operator<T>>> ops;
    std::vector<long long> offsets;
    int apply(const T *x, T *y) override {
        for (size_t g = 0; g < ops.size(); g++) SFEM_GB300_CHECK(ops[g]->apply(x + offsets[g], y + offsets[g]));
        return 0;
    }
    ptrdiff_t rows() const override { return offsets.back(); }
    ptrdiff_t cols() const override { return offsets.back(); }
};

// ---------------------------------------------------------------- solvers

// Chebyshev3 on the Jacobi-scaled operator with per-problem eigenvalue bounds
// (same recurrence as the single-problem Chebyshev3; the power method runs a
// fixed number of normalised iterations for all problems at once).
template <typename T>
class BatchChebyshev3 final : public Solver<T> {
public:
    std::shared_ptr<BatchLayout> lay;
    std::shared_ptr<Operator<T>> op;
    const T *inv_diag{nullptr};
    DeviceBuffer<T> p, temp;
    DeviceBuffer<double> coef;  // [2 * max_it][P]: alpha_k then beta_k
    std::vector<double> eig_max;
    double scale_eig_max{1.02}, scale_eig_min{0.06};
    int max_it{2};

    int init(int eigen_max_it, unsigned long long seed) {
        const ptrdiff_t n = op->rows();
        const int P = lay->P;
        SFEM_GB300_CHECK(p.resize(n));
        SFEM_GB300_CHECK(temp.resize(n));
        DeviceBuffer<T> v(n);
        DeviceBuffer<double> ww(P);
        const cudaStream_t s = lay->ctx->stream;
        SFEM_GB300_CHECK(sfem_gb300_random_uniform(real_type_v<T>, n, seed, v.ptr, lay->ctx->sp()));
        for (int k = 0; k < eigen_max_it; k++) {
            SFEM_GB300_CUDA(cudaMemsetAsync(temp.ptr, 0, n * sizeof(T), s));
            SFEM_GB300_CHECK(op->apply(v.ptr, temp.ptr));
            if (inv_diag)
                SFEM_GB300_CHECK(sfem_gb300_xypaz(real_type_v<T>, n, inv_diag, temp.ptr, 0.0, temp.ptr, lay->ctx->sp()));
            SFEM_GB300_CHECK(lay->dot(temp.ptr, temp.ptr, ww.ptr));
            bnormalize_kernel<T><<<lay->grid(), lay->threads, 0, s>>>(lay->n_items, lay->work.ptr, ww.ptr, temp.ptr,
                                                                       v.ptr);
        }
        std::vector<double> h(P);
        SFEM_GB300_CUDA(cudaMemcpyAsync(h.data(), ww.ptr, P * sizeof(double), cudaMemcpyDeviceToHost, s));
        SFEM_GB300_CUDA(cudaStreamSynchronize(s));
        eig_max.resize(P);
        for (int q = 0; q < P; q++) eig_max[q] = std::sqrt(h[q]);
        return set_coefficients();
    }
    int set_coefficients() {
        const int P = lay->P;
        std::vector<double> c(2 * (size_t)max_it * P, 0.0);
        for (int q = 0; q < P; q++) {
            const double emax = eig_max[q] * scale_eig_max;
            const double emin = scale_eig_min * emax;
            const double eavg = (emin + emax) / 2, ediff = (emin - emax) / 2;
            double alpha = emax > 0 ? 1.0 / eavg : 0.0, beta = 0;
            for (int k = 0; k < max_it; k++) {
                if (k > 0 && emax > 0) {
                    const double dea = ediff * alpha;
                    beta = (k == 1 ? 0.5 : 0.25) * dea * dea;
                    alpha = 1.0 / (eavg - beta / alpha);
                }
                c[(size_t)k * P + q] = alpha;
                c[((size_t)max_it + k) * P + q] = beta;
            }
        }
        SFEM_GB300_CHECK(coef.resize(c.size()));
        SFEM_GB300_CUDA(cudaMemcpy(coef.ptr, c.data(), c.size() * sizeof(double), cudaMemcpyHostToDevice));
        return 0;
    }
    int apply(const T *b, T *x) override {
        const ptrdiff_t n = op->rows();
        const int P = lay->P;
        const cudaStream_t s = lay->ctx->stream;
        for (int k = 0; k < max_it; k++) {
            if (!op->overwrites_output()) SFEM_GB300_CUDA(cudaMemsetAsync(temp.ptr, 0, n * sizeof(T), s));
            SFEM_GB300_CHECK(op->apply(x, temp.ptr));
            bcheb_update_kernel<T><<<lay->grid(), lay->threads, 0, s>>>(
                    lay->n_items, lay->work.ptr, coef.ptr + (size_t)k * P, coef.ptr + ((size_t)max_it + k) * P,
                    inv_diag, b, temp.ptr, p.ptr, x);
        }
        this->iterations_ = max_it;
        return check_launch("BatchChebyshev3");
    }
    ptrdiff_t rows() const override { return op->rows(); }
    ptrdiff_t cols() const override { return op->cols(); }
};

// Preconditioned (flexible, Polak-Ribiere) CG over a batch: per-problem scalars on
// the device, a problem stops updating once ||r_p|| <= rtol ||r0_p||.  No host
// synchronisation: apply() runs exactly max_it iterations; start() / iterate()
// let an outer driver run (and graph-capture) the iterations in chunks.
template <typename T>
class BatchCG final : public Solver<T> {
public:
    std::shared_ptr<BatchLayout> lay;
    std::shared_ptr<Operator<T>> op, precond;
    DeviceBuffer<T> r, z, zprev, p, Ap;
    DeviceBuffer<double> sc;  // [6][P]: rz, rz_old, pAp, rr, r.z_prev, rr0
    DeviceBuffer<int> active;
    int max_it{10};
    double rtol{1e-4};
    bool flexible{true};
    T *zz{nullptr}, *zp{nullptr};  // current / previous preconditioned residual

    int prepare() {
        const ptrdiff_t n = op->rows();
        SFEM_GB300_CHECK(r.resize(n));
        SFEM_GB300_CHECK(z.resize(n));
        SFEM_GB300_CHECK(p.resize(n));
        SFEM_GB300_CHECK(Ap.resize(n));
        if (flexible) SFEM_GB300_CHECK(zprev.resize(n));
        SFEM_GB300_CHECK(sc.resize(6 * (ptrdiff_t)lay->P));
        SFEM_GB300_CHECK(active.resize(lay->P));
        return 0;
    }
    double *scal(int k) { return sc.ptr + (ptrdiff_t)k * lay->P; }
    int start(const T *b, const T *x) {
        const ptrdiff_t n = op->rows();
        const int P = lay->P;
        if (!active.ptr) SFEM_GB300_CHECK(prepare());
        const cudaStream_t s = lay->ctx->stream;
        const bool pre = (bool)precond;
        zz = pre ? z.ptr : r.ptr;
        zp = pre && flexible ? zprev.ptr : nullptr;
        if (!op->overwrites_output()) SFEM_GB300_CUDA(cudaMemsetAsync(r.ptr, 0, n * sizeof(T), s));
        SFEM_GB300_CHECK(op->apply(x, r.ptr));
        SFEM_GB300_CHECK(sfem_gb300_axpby(real_type_v<T>, n, 1.0, b, -1.0, r.ptr, lay->ctx->sp()));  // r = b - A x
        if (pre) {
            if (!precond->overwrites_output()) SFEM_GB300_CUDA(cudaMemsetAsync(z.ptr, 0, n * sizeof(T), s));
            SFEM_GB300_CHECK(precond->apply(r.ptr, z.ptr));
        }
        SFEM_GB300_CUDA(cudaMemcpyAsync(p.ptr, zz, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
        SFEM_GB300_CHECK(lay->dot(r.ptr, zz, scal(0)));
        SFEM_GB300_CHECK(lay->dot(r.ptr, r.ptr, scal(5)));
        bcg_start_kernel<<<lay->pgrid(), 128, 0, s>>>(P, scal(5), active.ptr);
        return check_launch("BatchCG start");
    }
    // k iterations from the current state; rr0 (scal(5)) is the reference of the test
    int iterate(int k, T *x) {
        const ptrdiff_t n = op->rows();
        const int P = lay->P;
        const cudaStream_t s = lay->ctx->stream;
        const bool pre = (bool)precond;
        const bool flex = zp != nullptr;
        const double tol2 = rtol * rtol;
        for (int it = 0; it < k; it++) {
            if (!op->overwrites_output()) SFEM_GB300_CUDA(cudaMemsetAsync(Ap.ptr, 0, n * sizeof(T), s));
            SFEM_GB300_CHECK(op->apply(p.ptr, Ap.ptr));
            SFEM_GB300_CHECK(lay->dot(p.ptr, Ap.ptr, scal(2)));
            bcg_update_x_r_kernel<T><<<lay->grid(), lay->threads, 0, s>>>(lay->n_items, lay->work.ptr, scal(0),
                                                                           scal(2), active.ptr, p.ptr, Ap.ptr, x,
                                                                           r.ptr, lay->partials.ptr);
            bsum_kernel<<<lay->pgrid(), 128, 0, s>>>(P, lay->first_item.ptr, lay->partials.ptr, scal(3));
            bcg_check_kernel<<<lay->pgrid(), 128, 0, s>>>(P, scal(3), scal(5), tol2, active.ptr);
            SFEM_GB300_CUDA(cudaMemcpyAsync(scal(1), scal(0), P * sizeof(double), cudaMemcpyDeviceToDevice, s));
            if (pre) {
                if (flex) std::swap(zz, zp);
                if (!precond->overwrites_output()) SFEM_GB300_CUDA(cudaMemsetAsync(zz, 0, n * sizeof(T), s));
                SFEM_GB300_CHECK(precond->apply(r.ptr, zz));
                SFEM_GB300_CHECK(lay->dot(r.ptr, zz, scal(0)));
                if (flex) SFEM_GB300_CHECK(lay->dot(r.ptr, zp, scal(4)));
            } else {
                SFEM_GB300_CUDA(cudaMemcpyAsync(scal(0), scal(3), P * sizeof(double), cudaMemcpyDeviceToDevice, s));
            }
            bcg_update_p_kernel<T><<<lay->grid(), lay->threads, 0, s>>>(lay->n_items, lay->work.ptr, scal(0), scal(1),
                                                                         flex ? scal(4) : nullptr, active.ptr, zz,
                                                                         p.ptr);
        }
        if (pre && flex && (k & 1)) {
            // An odd number of buffer swaps: move the latest z back into the buffer the
            // chunk started with, so every chunk starts from the same (zz, zp) pair -- a
            // captured chunk replays with the pointers it was captured with.
            SFEM_GB300_CUDA(cudaMemcpyAsync(zp, zz, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
            std::swap(zz, zp);
        }
        return check_launch("BatchCG iterate");
    }
    int apply(const T *b, T *x) override {
        SFEM_GB300_CHECK(start(b, x));
        SFEM_GB300_CHECK(iterate(max_it, x));
        this->iterations_ = max_it;
        return 0;
    }
    ptrdiff_t rows() const override { return op->rows(); }
    ptrdiff_t cols() const override { return op->cols(); }
};

// Per-problem precision bridge: z += ||r_p|| M32(r_p / ||r_p||) for a float
// preconditioner M32 (e.g. the grouped float multigrid) under a double Krylov method.
__global__ void bbridge_scale_kernel(int P, const double *__restrict__ rr, double *__restrict__ inv,
                                     double *__restrict__ scale) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const double n = sqrt(rr[p]);
    inv[p] = n > 0 ? 1.0 / n : 0.0;
    scale[p] = n;
}

class BatchBridge final : public Operator<double> {
public:
    std::shared_ptr<BatchLayout> lay;
    std::shared_ptr<Operator<float>> inner;
    DeviceBuffer<float> r32, z32;
    DeviceBuffer<double> rr, inv, scale;
    int apply(const double *r, double *z) override {
        const ptrdiff_t n = inner->rows();
        const int P = lay->P;
        const cudaStream_t s = lay->ctx->stream;
        if (!r32.ptr) {
            SFEM_GB300_CHECK(r32.resize(n));
            SFEM_GB300_CHECK(z32.resize(n));
            SFEM_GB300_CHECK(rr.resize(P));
            SFEM_GB300_CHECK(inv.resize(P));
            SFEM_GB300_CHECK(scale.resize(P));
        }
        SFEM_GB300_CHECK(lay->dot(r, r, rr.ptr));
        bbridge_scale_kernel<<<lay->pgrid(), 128, 0, s>>>(P, rr.ptr, inv.ptr, scale.ptr);
        bconvert_scaled_kernel<<<lay->grid(), lay->threads, 0, s>>>(lay->n_items, lay->work.ptr, inv.ptr, r, r32.ptr);
        SFEM_GB300_CUDA(cudaMemsetAsync(z32.ptr, 0, n * sizeof(float), s));
        SFEM_GB300_CHECK(inner->apply(r32.ptr, z32.ptr));
        baxpy_f32_to_f64_kernel<<<lay->grid(), lay->threads, 0, s>>>(lay->n_items, lay->work.ptr, scale.ptr, z32.ptr,
                                                                     z);
        return check_launch("BatchBridge");
    }
    ptrdiff_t rows() const override { return inner->rows(); }
    ptrdiff_t cols() const override { return inner->cols(); }
};

// Host driver of a batched double CG (typically flexible, preconditioned by a
// BatchBridge over the grouped float multigrid): chunks of `check_every`
// iterations are captured into one CUDA graph on a private stream and replayed;
// after each chunk the host reads the per-problem active mask (one small copy)
// to time every problem's convergence and to stop when all have converged.
class BatchSolve {
public:
    std::shared_ptr<Context> ctx;
    std::shared_ptr<BatchLayout> lay;
    std::shared_ptr<BatchCG<double>> cg;
    int check_every{5};
    int max_it{300};
    bool use_graph{true};
    cudaStream_t stream{nullptr};
    cudaGraphExec_t exec{nullptr};
    double *g_x{nullptr};
    std::vector<double> h_latency;
    std::vector<int> h_iters;
    int iterations{0};
    double seconds{0};
    // non-blocking driver (begin / step / poll): pinned copy of the active mask, the
    // event that marks its arrival
    int *h_mask{nullptr};
    cudaEvent_t mask_ready{nullptr};
    bool pending{false};
    double *run_x{nullptr};
    int priority{0};  // CUDA stream priority of this solver's stream (0: the default)

    int make_stream() {
        if (stream) return 0;
        SFEM_GB300_CUDA(cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, priority));
        return 0;
    }
    // level 0: default priority; each level up one step higher, clamped to the device's range
    int set_priority(int level) {
        if (pending) return set_error("BatchSolve: priority change while a chunk is in flight");
        int least = 0, greatest = 0;
        SFEM_GB300_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        priority = std::max(greatest, least - std::max(level, 0));
        if (stream) {
            SFEM_GB300_CUDA(cudaStreamSynchronize(stream));
            SFEM_GB300_CUDA(cudaStreamDestroy(stream));
            stream = nullptr;
        }
        return make_stream();
    }

    ~BatchSolve() {
        exec_reset();
        if (mask_ready) cudaEventDestroy(mask_ready);
        if (h_mask) cudaFreeHost(h_mask);
        if (stream) cudaStreamDestroy(stream);
    }
    void exec_reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        g_x = nullptr;
    }
    int on_stream(const std::function<int()> &fn) {
        const cudaStream_t saved = ctx->stream;
        ctx->stream = stream;
        const int rc = fn();
        ctx->stream = saved;
        return rc;
    }
    int capture(double *x) {
        exec_reset();
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
        int rc = e == cudaSuccess ? on_stream([&] { return cg->iterate(check_every, x); })
                                  : set_error("cudaStreamBeginCapture: %s", cudaGetErrorString(e));
        cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(stream, &graph) : cudaSuccess;
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e2 != cudaSuccess) return set_error("cudaStreamEndCapture: %s", cudaGetErrorString(e2));
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
        g_x = x;
        return 0;
    }
    int chunk(double *x) {
        if (use_graph) {
            SFEM_GB300_CUDA(cudaGraphLaunch(exec, stream));
            return 0;
        }
        return on_stream([&] { return cg->iterate(check_every, x); });
    }
    // Capture (if needed) and start the CG on this solver's own stream; then step() launches
    // one chunk and the copy of the active mask without waiting, and poll() reports whether
    // that mask has arrived.  Several solvers on their own streams (and contexts) advance
    // independently: a host loop steps each one whose last mask has arrived.
    int begin(const double *b, double *x) {
        const int P = lay->P;
        SFEM_GB300_CHECK(make_stream());
        if (!h_mask) SFEM_GB300_CUDA(cudaMallocHost(&h_mask, (size_t)P * sizeof(int)));
        if (!mask_ready) SFEM_GB300_CUDA(cudaEventCreateWithFlags(&mask_ready, cudaEventDisableTiming));
        SFEM_GB300_CUDA(cudaStreamSynchronize(ctx->stream));
        if (use_graph && (!exec || g_x != x)) {
            DeviceBuffer<double> xs(cg->rows());
            SFEM_GB300_CUDA(cudaMemcpyAsync(xs.ptr, x, cg->rows() * sizeof(double), cudaMemcpyDeviceToDevice, stream));
            SFEM_GB300_CHECK(on_stream([&] { return cg->start(b, xs.ptr); }));
            SFEM_GB300_CHECK(on_stream([&] { return cg->iterate(1, xs.ptr); }));
            SFEM_GB300_CUDA(cudaStreamSynchronize(stream));
            SFEM_GB300_CHECK(capture(x));
        }
        SFEM_GB300_CHECK(on_stream([&] { return cg->start(b, x); }));
        SFEM_GB300_CUDA(cudaMemcpyAsync(h_mask, cg->active.ptr, P * sizeof(int), cudaMemcpyDeviceToHost, stream));
        SFEM_GB300_CUDA(cudaEventRecord(mask_ready, stream));
        pending = true;
        iterations = 0;
        run_x = x;
        return 0;
    }
    int step() {
        if (pending) return set_error("BatchSolve: step before the previous mask arrived");
        if (iterations >= max_it) return set_error("BatchSolve: no convergence in %d iterations", max_it);
        SFEM_GB300_CHECK(chunk(run_x));
        iterations += check_every;
        SFEM_GB300_CUDA(cudaMemcpyAsync(h_mask, cg->active.ptr, lay->P * sizeof(int), cudaMemcpyDeviceToHost, stream));
        SFEM_GB300_CUDA(cudaEventRecord(mask_ready, stream));
        pending = true;
        return 0;
    }
    // 0: the mask of the last step (or of begin) is in `active`; kPollNotReady: not yet
    static constexpr int kPollNotReady = 2;
    int poll(int *active, int *n_active) {
        if (!pending) return set_error("BatchSolve: poll without a step");
        const cudaError_t e = cudaEventQuery(mask_ready);
        if (e == cudaErrorNotReady) return kPollNotReady;
        if (e != cudaSuccess) return set_error("BatchSolve: %s", cudaGetErrorString(e));
        pending = false;
        int n = 0;
        for (int q = 0; q < lay->P; q++) {
            if (active) active[q] = h_mask[q];
            n += h_mask[q] != 0;
        }
        if (n_active) *n_active = n;
        return 0;
    }

    // release_s (host, optional): release time of every problem in seconds from the start
    // of the solve.  A problem joins the iteration at the first chunk boundary after its
    // release (until then it keeps its start state: the CG update kernels skip inactive
    // problems); its latency is counted from its release.
    int solve(const double *b, double *x, const double *release_s = nullptr) {
        const int P = lay->P;
        SFEM_GB300_CHECK(make_stream());
        SFEM_GB300_CUDA(cudaStreamSynchronize(ctx->stream));  // caller's work on b, x is done
        if (use_graph && (!exec || g_x != x)) {
            // eager warm-up on a scratch iterate sizes every lazily allocated buffer
            DeviceBuffer<double> xs(cg->rows());
            SFEM_GB300_CUDA(cudaMemcpyAsync(xs.ptr, x, cg->rows() * sizeof(double), cudaMemcpyDeviceToDevice, stream));
            SFEM_GB300_CHECK(on_stream([&] { return cg->start(b, xs.ptr); }));
            SFEM_GB300_CHECK(on_stream([&] { return cg->iterate(1, xs.ptr); }));
            SFEM_GB300_CUDA(cudaStreamSynchronize(stream));
            SFEM_GB300_CHECK(capture(x));
        }
        std::vector<int> h_active(P, 1), prev(P, 1), started(P, 1), released(P, 1), it0(P, 0);
        h_latency.assign(P, -1.0);
        h_iters.assign(P, -1);
        auto elapsed = [](std::chrono::steady_clock::time_point a) {
            return std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
        };
        const auto t0 = std::chrono::steady_clock::now();
        SFEM_GB300_CHECK(on_stream([&] { return cg->start(b, x); }));
        int n_pending = 0;
        if (release_s) {
            // the start state of every problem is kept; only the released ones iterate
            SFEM_GB300_CUDA(cudaMemcpyAsync(started.data(), cg->active.ptr, P * sizeof(int), cudaMemcpyDeviceToHost,
                                            stream));
            SFEM_GB300_CUDA(cudaStreamSynchronize(stream));
            for (int q = 0; q < P; q++) {
                released[q] = release_s[q] <= 0.0;
                h_active[q] = started[q] && released[q];
                n_pending += !released[q];
            }
            SFEM_GB300_CUDA(cudaMemcpyAsync(cg->active.ptr, h_active.data(), P * sizeof(int), cudaMemcpyHostToDevice,
                                            stream));
            prev = h_active;
        }
        int n_active = 0;
        for (int q = 0; q < P; q++) n_active += h_active[q] != 0;
        for (iterations = 0; iterations < max_it && (n_active > 0 || n_pending > 0);) {
            if (n_pending > 0) {
                // join the problems released by now; with nothing to iterate, wait for the next release
                double now = elapsed(t0);
                if (n_active == 0) {
                    double next = 1e300;
                    for (int q = 0; q < P; q++)
                        if (!released[q]) next = std::min(next, release_s[q]);
                    while (now < next) now = elapsed(t0);
                }
                bool changed = false;
                for (int q = 0; q < P; q++) {
                    if (released[q] || release_s[q] > now) continue;
                    released[q] = 1;
                    n_pending--;
                    it0[q] = iterations;
                    if (started[q]) {
                        h_active[q] = 1;
                        n_active++;
                    }
                    changed = true;
                }
                if (changed)
                    SFEM_GB300_CUDA(cudaMemcpyAsync(cg->active.ptr, h_active.data(), P * sizeof(int),
                                                    cudaMemcpyHostToDevice, stream));
                prev = h_active;
                if (n_active == 0) continue;
            }
            SFEM_GB300_CHECK(chunk(x));
            iterations += check_every;
            SFEM_GB300_CUDA(cudaMemcpyAsync(h_active.data(), cg->active.ptr, P * sizeof(int), cudaMemcpyDeviceToHost,
                                            stream));
            SFEM_GB300_CUDA(cudaStreamSynchronize(stream));
            const double now = elapsed(t0);
            n_active = 0;
            for (int q = 0; q < P; q++) {
                if (prev[q] && !h_active[q]) {
                    h_latency[q] = now - (release_s ? std::max(release_s[q], 0.0) : 0.0);
                    h_iters[q] = iterations - it0[q];
                }
                n_active += h_active[q] != 0;
            }
            prev = h_active;
        }
        seconds = elapsed(t0);
        if (n_active || n_pending)
            return set_error("BatchSolve: %d problems not converged in %d iterations", n_active + n_pending, max_it);
        return 0;
    }
};

}  // namespace sfem_gb300

using namespace sfem_gb300;

namespace {
std::shared_ptr<BatchLayout> layout_of(Handle *h) { return std::static_pointer_cast<BatchLayout>(h->impl); }
}  // namespace

extern "C" int sfem_gb300_batch_layout_create(void *context, int n_problems, const int64_t *offsets, int chunk,
                                              void **out) {
    if (n_problems <= 0) return set_error("sfem_gb300_batch_layout_create: n_problems must be > 0");
    if (chunk < 32) return set_error("sfem_gb300_batch_layout_create: chunk must be >= 32");
    for (int p = 0; p < n_problems; p++)
        if (offsets[p + 1] < offsets[p]) return set_error("sfem_gb300_batch_layout_create: offsets must not decrease");
    auto lay = std::make_shared<BatchLayout>();
    lay->ctx = H(context)->ctx;
    lay->P = n_problems;
    lay->offsets.assign(offsets, offsets + n_problems + 1);
    lay->chunk = chunk;
    SFEM_GB300_CHECK(lay->build());
    auto *h = new Handle();
    h->kind = "batch_layout";
    h->ctx = lay->ctx;
    h->impl = lay;
    *out = h;
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_batch_layout_set_launch(void *layout, int chunk, int threads, int ctas_per_sm) {
    auto lay = layout_of(H(layout));
    if (threads < 32 || threads > kBatchMaxThreads || threads % 32)
        return set_error("sfem_gb300_batch_layout_set_launch: threads must be a multiple of 32 in [32, 1024]");
    if (ctas_per_sm < 1 || ctas_per_sm > 32 || chunk < 32)
        return set_error("sfem_gb300_batch_layout_set_launch: bad ctas_per_sm or chunk");
    lay->threads = threads;
    lay->ctas_per_sm = ctas_per_sm;
    if (chunk != lay->chunk) {
        lay->chunk = chunk;
        SFEM_GB300_CHECK(lay->build());
    }
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_batch_dot(void *layout, int real_type, const void *x, const void *y, double *d_out) {
    auto lay = layout_of(H(layout));
    if (real_type == SFEM_GB300_FLOAT32) return lay->dot((const float *)x, (const float *)y, d_out);
    return lay->dot((const double *)x, (const double *)y, d_out);
}

extern "C" int sfem_gb300_batch_grouped_op_create(void *context, int real_type, int n_ops, void **ops,
                                                  const int64_t *offsets, void **out) {
    auto *c = H(context);
    auto *h = new Handle();
    h->kind = "grouped";
    h->ctx = c->ctx;
    h->real_type = is_f32(real_type) ? SFEM_GB300_FLOAT32 : SFEM_GB300_FLOAT64;
    auto fill = [&](auto g, auto tag) -> int {
        using T = decltype(tag);
        g->offsets.assign(offsets, offsets + n_ops + 1);
        for (int k = 0; k < n_ops; k++) {
            auto &o = op_of<T>(H(ops[k]));
            if (!o) return set_error("sfem_gb300_batch_grouped_op_create: operator %d has the wrong precision", k);
            if (o->rows() != offsets[k + 1] - offsets[k])
                return set_error("sfem_gb300_batch_grouped_op_create: operator %d has %td rows, its range %lld", k,
                                 o->rows(), (long long)(offsets[k + 1] - offsets[k]));
            g->ops.push_back(o);
        }
        return 0;
    };
    int rc;
    if (is_f32(real_type)) {
        auto g = std::make_shared<GroupedOperator<float>>();
        rc = fill(g, 0.0f);
        h->f = g;
    } else {
        auto g = std::make_shared<GroupedOperator<double>>();
        rc = fill(g, 0.0);
        h->d = g;
    }
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_batch_chebyshev3_create(void *context, void *layout, void *op, const void *inv_diag,
                                                  int max_it, double scale_eig_max, double scale_eig_min,
                                                  int eigen_max_it, unsigned long long seed, void **out) {
    auto *c = H(context);
    auto *o = H(op);
    auto lay = layout_of(H(layout));
    if (o->rows() != lay->n()) return set_error("sfem_gb300_batch_chebyshev3_create: operator / layout size mismatch");
    auto *h = new Handle();
    h->kind = "batch_chebyshev3";
    h->ctx = c->ctx;
    h->real_type = o->real_type;
    auto make = [&](auto tag) -> int {
        using T = decltype(tag);
        auto s = std::make_shared<BatchChebyshev3<T>>();
        s->lay = lay;
        s->op = op_of<T>(o);
        s->inv_diag = (const T *)inv_diag;
        s->max_it = max_it;
        s->scale_eig_max = scale_eig_max;
        s->scale_eig_min = scale_eig_min;
        op_of<T>(h) = s;
        h->impl = s;
        return s->init(eigen_max_it, seed);
    };
    const int rc = o->f ? make(0.0f) : make(0.0);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_batch_chebyshev3_eig_max(void *solver, double *eig_max_out) {
    auto *h = H(solver);
    const std::vector<double> &v = h->f ? std::static_pointer_cast<BatchChebyshev3<float>>(h->impl)->eig_max
                                        : std::static_pointer_cast<BatchChebyshev3<double>>(h->impl)->eig_max;
    std::memcpy(eig_max_out, v.data(), v.size() * sizeof(double));
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_batch_cg_create(void *context, void *layout, void *op, void *precond, int iterations,
                                          double rtol, int flexible, void **out) {
    auto *c = H(context);
    auto *o = H(op);
    auto lay = layout_of(H(layout));
    if (o->rows() != lay->n()) return set_error("sfem_gb300_batch_cg_create: operator / layout size mismatch");
    if (iterations < 1) return set_error("sfem_gb300_batch_cg_create: iterations must be >= 1");
    auto *h = new Handle();
    h->kind = "batch_cg";
    h->ctx = c->ctx;
    h->real_type = o->real_type;
    auto make = [&](auto tag) {
        using T = decltype(tag);
        auto s = std::make_shared<BatchCG<T>>();
        s->lay = lay;
        s->op = op_of<T>(o);
        if (precond) s->precond = op_of<T>(H(precond));
        s->max_it = iterations;
        s->rtol = rtol;
        s->flexible = flexible != 0;
        op_of<T>(h) = s;
        h->impl = s;
    };
    if (o->f)
        make(0.0f);
    else
        make(0.0);
    *out = h;
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_batch_bridge_create(void *context, void *layout, void *inner32, void **out) {
    auto *c = H(context);
    auto lay = layout_of(H(layout));
    if (!H(inner32)->f) return set_error("sfem_gb300_batch_bridge_create: inner operator must be float");
    if (H(inner32)->rows() != lay->n()) return set_error("sfem_gb300_batch_bridge_create: size mismatch");
    auto b = std::make_shared<BatchBridge>();
    b->lay = lay;
    b->inner = H(inner32)->f;
    auto *h = new Handle();
    h->kind = "batch_bridge";
    h->ctx = c->ctx;
    h->real_type = SFEM_GB300_FLOAT64;
    h->d = b;
    *out = h;
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_batch_solve_create(void *context, void *layout, void *cg64, int check_every, int max_it,
                                             int use_graph, void **out) {
    auto *c = H(context);
    auto lay = layout_of(H(layout));
    auto *h_cg = H(cg64);
    if (h_cg->kind != "batch_cg" || !h_cg->d) return set_error("sfem_gb300_batch_solve_create: needs a double batch CG");
    if (check_every < 1) return set_error("sfem_gb300_batch_solve_create: check_every must be >= 1");
    auto bs = std::make_shared<BatchSolve>();
    bs->ctx = c->ctx;
    bs->lay = lay;
    bs->cg = std::static_pointer_cast<BatchCG<double>>(h_cg->impl);
    bs->check_every = check_every;
    bs->max_it = max_it;
    bs->use_graph = use_graph != 0;
    auto *h = new Handle();
    h->kind = "batch_solve";
    h->ctx = c->ctx;
    h->impl = bs;
    *out = h;
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_batch_solve_set_launch(void *solver, int check_every) {
    auto bs = std::static_pointer_cast<BatchSolve>(H(solver)->impl);
    if (check_every < 1) return set_error("sfem_gb300_batch_solve_set_launch: check_every must be >= 1");
    bs->check_every = check_every;
    bs->exec_reset();
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_batch_solve_run_released(void *solver, const double *b, double *x,
                                                   const double *release_s, double *latency_s,
                                                   int *iterations_per_problem, double *seconds) {
    auto bs = std::static_pointer_cast<BatchSolve>(H(solver)->impl);
    const int rc = bs->solve(b, x, release_s);
    const int P = bs->lay->P;
    if (latency_s && (int)bs->h_latency.size() == P) std::memcpy(latency_s, bs->h_latency.data(), P * sizeof(double));
    if (iterations_per_problem && (int)bs->h_iters.size() == P)
        std::memcpy(iterations_per_problem, bs->h_iters.data(), P * sizeof(int));
    if (seconds) *seconds = bs->seconds;
    return rc;
}

extern "C" int sfem_gb300_batch_solve_set_priority(void *solver, int level) {
    return std::static_pointer_cast<BatchSolve>(H(solver)->impl)->set_priority(level);
}

extern "C" int sfem_gb300_batch_solve_begin(void *solver, const double *b, double *x) {
    return std::static_pointer_cast<BatchSolve>(H(solver)->impl)->begin(b, x);
}

extern "C" int sfem_gb300_batch_solve_step(void *solver) {
    return std::static_pointer_cast<BatchSolve>(H(solver)->impl)->step();
}

extern "C" int sfem_gb300_batch_solve_poll(void *solver, int *active, int *n_active, int *iterations) {
    auto bs = std::static_pointer_cast<BatchSolve>(H(solver)->impl);
    const int rc = bs->poll(active, n_active);
    if (iterations) *iterations = bs->iterations;
    return rc;
}

extern "C" int sfem_gb300_batch_solve_run(void *solver, const double *b, double *x, double *latency_s,
                                          int *iterations_per_problem, double *seconds) {
    return sfem_gb300_batch_solve_run_released(solver, b, x, nullptr, latency_s, iterations_per_problem, seconds);
}

extern "C" int sfem_gb300_batch_solve_time_chunk(void *solver, const double *b, double *x, int reps, double *ms) {
    auto bs = std::static_pointer_cast<BatchSolve>(H(solver)->impl);
    SFEM_GB300_CHECK(bs->make_stream());
    SFEM_GB300_CUDA(cudaStreamSynchronize(bs->ctx->stream));
    bs->use_graph = true;
    SFEM_GB300_CHECK(bs->on_stream([&] { return bs->cg->start(b, x); }));
    SFEM_GB300_CHECK(bs->on_stream([&] { return bs->cg->iterate(1, x); }));  // eager warm-up
    SFEM_GB300_CUDA(cudaStreamSynchronize(bs->stream));
    SFEM_GB300_CHECK(bs->capture(x));
    cudaEvent_t e0, e1;
    SFEM_GB300_CUDA(cudaEventCreate(&e0));
    SFEM_GB300_CUDA(cudaEventCreate(&e1));
    cudaEventRecord(e0, bs->stream);
    for (int k = 0; k < reps; k++) cudaGraphLaunch(bs->exec, bs->stream);
    cudaEventRecord(e1, bs->stream);
    const cudaError_t e = cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    bs->exec_reset();
    if (e != cudaSuccess) return set_error("sfem_gb300_batch_solve_time_chunk: %s", cudaGetErrorString(e));
    *ms = t / (reps > 0 ? reps : 1);
    return SFEM_GB300_SUCCESS;
}
