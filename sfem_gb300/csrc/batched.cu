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
//  * an outer FP64 refinement step (residual, inner FP32 batched flexible CG
//    preconditioned by per-group multigrid, update) is captured once into a CUDA
//    graph and replayed; the host reads the active mask once per step;
//  * the work-list chunk and the CTA shape of the vector kernels are picked by
//    an autotuner that times the captured step for each candidate.
#include <chrono>
#include <cmath>
#include <cstring>
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

// Outer refinement check on the FP64 residual: a problem stays active while
// ||r_p|| > rtol ||b_p||; then inv_p = 1 / ||r_p|| and scale_p = ||r_p||,
// both 0 for inactive problems.  Counts the active problems.
__global__ void bir_check_kernel(int P, const double *__restrict__ rr, const double *__restrict__ bb, double rtol,
                                 const int *__restrict__ step, int *__restrict__ active, int *__restrict__ done_step,
                                 double *__restrict__ rel, double *__restrict__ inv, double *__restrict__ scale,
                                 int *__restrict__ n_active) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const double rn = sqrt(rr[p]), bn = sqrt(bb[p]);
    if (active[p]) {
        rel[p] = bn > 0 ? rn / bn : 0.0;
        if (!(rn > rtol * bn) || !(rn == rn)) {
            active[p] = 0;
            done_step[p] = *step;
        }
    }
    const bool on = active[p] != 0;
    inv[p] = on ? 1.0 / rn : 0.0;
    scale[p] = on ? rn : 0.0;
    if (on) atomicAdd(n_active, 1);
}

__global__ void bstep_kernel(int *step) { *step += 1; }

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

// Preconditioned (flexible, Polak-Ribiere) CG over a batch: a fixed number of
// iterations per apply, per-problem scalars on the device, a problem stops
// updating once ||r_p|| <= rtol ||r0_p||.  No host synchronisation.
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
    int apply(const T *b, T *x) override {
        const ptrdiff_t n = op->rows();
        const int P = lay->P;
        if (!active.ptr) SFEM_GB300_CHECK(prepare());
        const cudaStream_t s = lay->ctx->stream;
        void *sp = lay->ctx->sp();
        const int rt = real_type_v<T>;
        double *rz = sc.ptr, *rz_old = sc.ptr + P, *pAp = sc.ptr + 2 * P, *rr = sc.ptr + 3 * P,
               *rzp = sc.ptr + 4 * P, *rr0 = sc.ptr + 5 * P;
        const bool pre = (bool)precond;
        const bool flex = pre && flexible;
        T *zz = pre ? z.ptr : r.ptr;
        T *zp = flex ? zprev.ptr : nullptr;
        if (!op->overwrites_output()) SFEM_GB300_CUDA(cudaMemsetAsync(r.ptr, 0, n * sizeof(T), s));
        SFEM_GB300_CHECK(op->apply(x, r.ptr));
        SFEM_GB300_CHECK(sfem_gb300_axpby(rt, n, 1.0, b, -1.0, r.ptr, sp));  // r = b - A x
        if (pre) {
            if (!precond->overwrites_output()) SFEM_GB300_CUDA(cudaMemsetAsync(z.ptr, 0, n * sizeof(T), s));
            SFEM_GB300_CHECK(precond->apply(r.ptr, z.ptr));
        }
        SFEM_GB300_CUDA(cudaMemcpyAsync(p.ptr, zz, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
        SFEM_GB300_CHECK(lay->dot(r.ptr, zz, rz));
        SFEM_GB300_CHECK(lay->dot(r.ptr, r.ptr, rr0));
        bcg_start_kernel<<<lay->pgrid(), 128, 0, s>>>(P, rr0, active.ptr);
        const double tol2 = rtol * rtol;
        for (int it = 0; it < max_it; it++) {
            if (!op->overwrites_output()) SFEM_GB300_CUDA(cudaMemsetAsync(Ap.ptr, 0, n * sizeof(T), s));
            SFEM_GB300_CHECK(op->apply(p.ptr, Ap.ptr));
            SFEM_GB300_CHECK(lay->dot(p.ptr, Ap.ptr, pAp));
            bcg_update_x_r_kernel<T><<<lay->grid(), lay->threads, 0, s>>>(lay->n_items, lay->work.ptr, rz, pAp,
                                                                           active.ptr, p.ptr, Ap.ptr, x, r.ptr,
                                                                           lay->partials.ptr);
            bsum_kernel<<<lay->pgrid(), 128, 0, s>>>(P, lay->first_item.ptr, lay->partials.ptr, rr);
            bcg_check_kernel<<<lay->pgrid(), 128, 0, s>>>(P, rr, rr0, tol2, active.ptr);
            if (it + 1 == max_it) break;
            SFEM_GB300_CUDA(cudaMemcpyAsync(rz_old, rz, P * sizeof(double), cudaMemcpyDeviceToDevice, s));
            if (pre) {
                if (flex) std::swap(zz, zp);
                if (!precond->overwrites_output()) SFEM_GB300_CUDA(cudaMemsetAsync(zz, 0, n * sizeof(T), s));
                SFEM_GB300_CHECK(precond->apply(r.ptr, zz));
                SFEM_GB300_CHECK(lay->dot(r.ptr, zz, rz));
                if (flex) SFEM_GB300_CHECK(lay->dot(r.ptr, zp, rzp));
            } else {
                SFEM_GB300_CUDA(cudaMemcpyAsync(rz, rr, P * sizeof(double), cudaMemcpyDeviceToDevice, s));
            }
            bcg_update_p_kernel<T><<<lay->grid(), lay->threads, 0, s>>>(lay->n_items, lay->work.ptr, rz, rz_old,
                                                                         flex ? rzp : nullptr, active.ptr, zz, p.ptr);
        }
        this->iterations_ = max_it;
        return check_launch("BatchCG");
    }
    ptrdiff_t rows() const override { return op->rows(); }
    ptrdiff_t cols() const override { return op->cols(); }
};

// FP64 iterative refinement over a batch around an FP32 batched inner solver.
// One outer step (residual, per-problem check, normalised FP32 residual, inner
// solve, update) is captured into a CUDA graph and replayed.
class BatchIR {
public:
    std::shared_ptr<Context> ctx;
    std::shared_ptr<BatchLayout> lay;
    std::shared_ptr<Operator<double>> op;
    std::shared_ptr<Operator<float>> inner;
    int max_outer{30};
    double rtol{1e-10};
    bool use_graph{true};
    DeviceBuffer<double> r64, bb, rr, inv, scale, rel;
    DeviceBuffer<float> r32, e32;
    DeviceBuffer<int> active, done_step, counters;  // counters: [0] active problems, [1] step
    int *h_counters{nullptr};
    cudaStream_t stream{nullptr};
    cudaGraphExec_t exec{nullptr};
    const double *g_b{nullptr};
    double *g_x{nullptr};
    // results of the last solve (host)
    std::vector<int> h_done;
    std::vector<double> h_rel, h_latency;
    int outer_steps{0};
    double seconds{0};

    ~BatchIR() {
        if (exec) cudaGraphExecDestroy(exec);
        if (stream) cudaStreamDestroy(stream);
        if (h_counters) cudaFreeHost(h_counters);
    }
    int prepare() {
        const ptrdiff_t n = op->rows();
        const int P = lay->P;
        SFEM_GB300_CHECK(r64.resize(n));
        SFEM_GB300_CHECK(r32.resize(n));
        SFEM_GB300_CHECK(e32.resize(n));
        for (auto *b : {&bb, &rr, &inv, &scale, &rel}) SFEM_GB300_CHECK(b->resize(P));
        SFEM_GB300_CHECK(active.resize(P));
        SFEM_GB300_CHECK(done_step.resize(P));
        SFEM_GB300_CHECK(counters.resize(2));
        if (!h_counters) SFEM_GB300_CUDA(cudaMallocHost((void **)&h_counters, 2 * sizeof(int)));
        if (!stream) SFEM_GB300_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        return 0;
    }
    // one outer step on the context stream
    int step(const double *b, double *x) {
        const ptrdiff_t n = op->rows();
        const int P = lay->P;
        const cudaStream_t s = ctx->stream;
        void *sp = ctx->sp();
        SFEM_GB300_CUDA(cudaMemsetAsync(counters.ptr, 0, sizeof(int), s));
        if (!op->overwrites_output()) SFEM_GB300_CUDA(cudaMemsetAsync(r64.ptr, 0, n * sizeof(double), s));
        SFEM_GB300_CHECK(op->apply(x, r64.ptr));
        SFEM_GB300_CHECK(sfem_gb300_axpby(SFEM_GB300_FLOAT64, n, 1.0, b, -1.0, r64.ptr, sp));
        SFEM_GB300_CHECK(lay->dot(r64.ptr, r64.ptr, rr.ptr));
        bir_check_kernel<<<lay->pgrid(), 128, 0, s>>>(P, rr.ptr, bb.ptr, rtol, counters.ptr + 1, active.ptr,
                                                      done_step.ptr, rel.ptr, inv.ptr, scale.ptr, counters.ptr);
        bconvert_scaled_kernel<<<lay->grid(), lay->threads, 0, s>>>(lay->n_items, lay->work.ptr, inv.ptr, r64.ptr,
                                                                    r32.ptr);
        SFEM_GB300_CUDA(cudaMemsetAsync(e32.ptr, 0, n * sizeof(float), s));
        SFEM_GB300_CHECK(inner->apply(r32.ptr, e32.ptr));
        baxpy_f32_to_f64_kernel<<<lay->grid(), lay->threads, 0, s>>>(lay->n_items, lay->work.ptr, scale.ptr, e32.ptr,
                                                                     x);
        bstep_kernel<<<1, 1, 0, s>>>(counters.ptr + 1);
        SFEM_GB300_CUDA(cudaMemcpyAsync(h_counters, counters.ptr, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
        return check_launch("BatchIR step");
    }
    void exec_reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        g_b = nullptr;
        g_x = nullptr;
    }
    int capture(const double *b, double *x) {
        exec_reset();
        const cudaStream_t saved = ctx->stream;
        ctx->stream = stream;
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
        int rc = e == cudaSuccess ? step(b, x) : set_error("cudaStreamBeginCapture: %s", cudaGetErrorString(e));
        cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(stream, &graph) : cudaSuccess;
        ctx->stream = saved;
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e2 != cudaSuccess) return set_error("cudaStreamEndCapture: %s", cudaGetErrorString(e2));
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
        g_b = b;
        g_x = x;
        return 0;
    }
    // Per-problem state for right-hand side b, on the solver stream (synchronises it).
    int reset(const double *b) {
        const int P = lay->P;
        const cudaStream_t saved = ctx->stream;
        ctx->stream = stream;
        const int rc = lay->dot(b, b, bb.ptr);
        ctx->stream = saved;
        if (rc) return rc;
        std::vector<int> ones(P, 1), minus(P, -1);
        SFEM_GB300_CUDA(cudaMemcpyAsync(active.ptr, ones.data(), P * sizeof(int), cudaMemcpyHostToDevice, stream));
        SFEM_GB300_CUDA(cudaMemcpyAsync(done_step.ptr, minus.data(), P * sizeof(int), cudaMemcpyHostToDevice, stream));
        SFEM_GB300_CUDA(cudaMemsetAsync(counters.ptr, 0, 2 * sizeof(int), stream));
        SFEM_GB300_CUDA(cudaStreamSynchronize(stream));  // the host vectors above are temporaries
        return 0;
    }
    int eager_step(const double *b, double *x) {
        const cudaStream_t saved = ctx->stream;
        ctx->stream = stream;
        const int rc = step(b, x);
        ctx->stream = saved;
        return rc;
    }
    // Makes sure a graph of the step for (b, x) exists; a warm-up step on a
    // scratch copy of x first sizes every lazily allocated buffer.
    int ensure_graph(const double *b, double *x) {
        if (exec && g_b == b && g_x == x) return 0;
        DeviceBuffer<double> xs(op->rows());
        SFEM_GB300_CUDA(cudaMemcpyAsync(xs.ptr, x, op->rows() * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        SFEM_GB300_CHECK(eager_step(b, xs.ptr));
        SFEM_GB300_CUDA(cudaStreamSynchronize(stream));
        return capture(b, x);
    }
    int solve(const double *b, double *x) {
        const int P = lay->P;
        SFEM_GB300_CHECK(prepare());
        // the solver stream runs after all work the caller queued on the context stream
        SFEM_GB300_CUDA(cudaStreamSynchronize(ctx->stream));
        if (use_graph) SFEM_GB300_CHECK(ensure_graph(b, x));
        SFEM_GB300_CHECK(reset(b));
        h_latency.assign(P, -1.0);
        std::vector<int> h_active(P, 1), prev(P, 1);
        const auto t0 = std::chrono::steady_clock::now();
        outer_steps = 0;
        for (int k = 0; k <= max_outer; k++) {
            if (use_graph)
                SFEM_GB300_CUDA(cudaGraphLaunch(exec, stream));
            else
                SFEM_GB300_CHECK(eager_step(b, x));
            SFEM_GB300_CUDA(cudaMemcpyAsync(h_active.data(), active.ptr, P * sizeof(int), cudaMemcpyDeviceToHost,
                                            stream));
            SFEM_GB300_CUDA(cudaStreamSynchronize(stream));
            const double now = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            outer_steps = k + 1;
            for (int q = 0; q < P; q++)
                if (prev[q] && !h_active[q]) h_latency[q] = now;
            prev = h_active;
            if (h_counters[0] == 0) break;
        }
        seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        h_done.resize(P);
        h_rel.resize(P);
        SFEM_GB300_CUDA(cudaMemcpy(h_done.data(), done_step.ptr, P * sizeof(int), cudaMemcpyDeviceToHost));
        SFEM_GB300_CUDA(cudaMemcpy(h_rel.data(), rel.ptr, P * sizeof(double), cudaMemcpyDeviceToHost));
        if (h_counters[0] != 0)
            return set_error("BatchIR: %d problems not converged in %d outer steps", h_counters[0], max_outer);
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

extern "C" int sfem_gb300_batch_ir_create(void *context, void *layout, void *op64, void *inner32, int max_outer,
                                          double rtol, int use_graph, void **out) {
    auto *c = H(context);
    auto lay = layout_of(H(layout));
    if (!H(op64)->d || !H(inner32)->f)
        return set_error("sfem_gb300_batch_ir_create: needs a double operator and a float inner solver");
    if (H(op64)->rows() != lay->n() || H(inner32)->rows() != lay->n())
        return set_error("sfem_gb300_batch_ir_create: operator / layout size mismatch");
    auto ir = std::make_shared<BatchIR>();
    ir->ctx = c->ctx;
    ir->lay = lay;
    ir->op = H(op64)->d;
    ir->inner = H(inner32)->f;
    ir->max_outer = max_outer;
    ir->rtol = rtol;
    ir->use_graph = use_graph != 0;
    auto *h = new Handle();
    h->kind = "batch_ir";
    h->ctx = c->ctx;
    h->impl = ir;
    *out = h;
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_batch_ir_solve(void *solver, const double *b, double *x, double *latency_s,
                                         int *outer_steps_per_problem, double *final_rel, double *seconds) {
    auto ir = std::static_pointer_cast<BatchIR>(H(solver)->impl);
    const int rc = ir->solve(b, x);
    const int P = ir->lay->P;
    if (latency_s && (int)ir->h_latency.size() == P) std::memcpy(latency_s, ir->h_latency.data(), P * sizeof(double));
    if (outer_steps_per_problem && (int)ir->h_done.size() == P)
        std::memcpy(outer_steps_per_problem, ir->h_done.data(), P * sizeof(int));
    if (final_rel && (int)ir->h_rel.size() == P) std::memcpy(final_rel, ir->h_rel.data(), P * sizeof(double));
    if (seconds) *seconds = ir->seconds;
    return rc;
}

extern "C" int sfem_gb300_batch_ir_time_step(void *solver, const double *b, double *x, int reps, double *ms) {
    auto ir = std::static_pointer_cast<BatchIR>(H(solver)->impl);
    SFEM_GB300_CHECK(ir->prepare());
    SFEM_GB300_CUDA(cudaStreamSynchronize(ir->ctx->stream));
    ir->exec_reset();
    SFEM_GB300_CHECK(ir->ensure_graph(b, x));
    SFEM_GB300_CHECK(ir->reset(b));
    cudaEvent_t e0, e1;
    SFEM_GB300_CUDA(cudaEventCreate(&e0));
    SFEM_GB300_CUDA(cudaEventCreate(&e1));
    cudaGraphLaunch(ir->exec, ir->stream);
    cudaEventRecord(e0, ir->stream);
    for (int k = 0; k < reps; k++) cudaGraphLaunch(ir->exec, ir->stream);
    cudaEventRecord(e1, ir->stream);
    const cudaError_t e = cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return set_error("sfem_gb300_batch_ir_time_step: %s", cudaGetErrorString(e));
    *ms = t / (reps > 0 ? reps : 1);
    return SFEM_GB300_SUCCESS;
}
