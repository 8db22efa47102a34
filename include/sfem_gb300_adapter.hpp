/*
 * sfem_gb300_adapter.hpp -- header-only C++ adapters that put the sfem_gb300 C ABI
 * behind the reference's own C++ seams, so the GPU path drops in where the reference
 * registers its CUDA operators:
 *
 *   DeviceBLAS<T, Base>            implements sfem::BLAS<T>      (algebra/sfem_tpl_blas.hpp:11-35)
 *   DeviceOperator<T, Base, ES>    implements sfem::Operator<T>  (algebra/sfem_Operator.hpp:13-33)
 *   LaplacianOp<Base, ES>          implements sfem::Op as the reference's "gpu:Laplacian"
 *                                  (frontend/ops/sfem_Op.hpp:42-324; GPULaplacian,
 *                                  frontend/cuda/sfem_Function_incore_cuda.cpp:545-751)
 *   LinearElasticityOp<Base, ES>   "gpu:LinearElasticity" (GPULinearElasticity, :753-1013)
 *
 * Base is the reference class (sfem::BLAS<real_t>, sfem::Operator<real_t>, sfem::Op) in
 * a reference build; ES is its device execution-space value (sfem::EXECUTION_SPACE_DEVICE,
 * an enum of the smesh submodule).  Every member these adapters define carries
 * `override`, so a signature that drifts from the reference's fails to compile.  For
 * builds without the reference tree, sfem_gb300::adapter::interfaces declares abstract
 * classes with the reference's virtual signatures (used by this library's own C++ test).
 *
 * Registration in the reference (sketch):
 *     using GpuLaplacian = sfem_gb300::adapter::LaplacianOp<sfem::Op, sfem::EXECUTION_SPACE_DEVICE>;
 *     sfem::Factory::register_op("gpu:Laplacian", [](const std::shared_ptr<sfem::FunctionSpace> &fs) {
 *         return std::make_shared<GpuLaplacian>(element_type, nelements, device_elements,
 *                                               device_corners, device_points, fs->n_dofs(), stream); });
 *
 * Conventions are those of the C ABI (include/sfem_gb300.h): device pointers, apply
 * entry points accumulate (out += A h), the caller owns inputs and outputs.  The
 * adapters own what the reference's GPU ops own: the cached geometry (FFF or adjugate and
 * determinant) and, for BLAS, the reduction workspace.  Errors of the C ABI come back as
 * SFEM_GB300_FAILURE from the int-returning members; members returning values throw
 * std::runtime_error with sfem_gb300_last_error().
 */
#ifndef SFEM_GB300_ADAPTER_HPP
#define SFEM_GB300_ADAPTER_HPP

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "sfem_gb300.h"

namespace sfem_gb300 {
namespace adapter {

// The reference's default number selection (cmake/SFEMNumbers.cmake:5-14).
using real_t = double;
using count_t = int32_t;
using idx_t = int32_t;

template <typename T>
constexpr int real_type_of();
template <>
constexpr int real_type_of<double>() {
    return SFEM_GB300_FLOAT64;
}
template <>
constexpr int real_type_of<float>() {
    return SFEM_GB300_FLOAT32;
}

inline void check(int rc, const char *what) {
    if (rc != SFEM_GB300_SUCCESS) throw std::runtime_error(std::string(what) + ": " + sfem_gb300_last_error());
}
inline void check_cuda(cudaError_t err, const char *what) {
    if (err != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(err));
}

namespace interfaces {
// Abstract classes with the reference's virtual signatures, for builds without it.
template <typename T>
class BLAS {
public:
    virtual ~BLAS() = default;
    virtual T *allocate(const std::size_t n) = 0;
    virtual void destroy(void *a) = 0;
    virtual void zeros(const std::size_t size, T *const x) = 0;
    virtual void values(const std::size_t size, const T value, T *const x) = 0;
    virtual void copy(const ptrdiff_t n, const T *const src, T *const dest) = 0;
    virtual T dot(const ptrdiff_t n, const T *const l, const T *const r) = 0;
    virtual void axpy(const ptrdiff_t n, const T alpha, const T *const x, T *const y) = 0;
    virtual void axpby(const ptrdiff_t n, const T alpha, const T *const x, const T beta, T *const y) = 0;
    virtual void scal(const std::ptrdiff_t n, const T alpha, T *const x) = 0;
    virtual void reciprocal(const std::ptrdiff_t n, const T alpha, T *const x) = 0;
    virtual T norm2(const ptrdiff_t n, const T *const x) = 0;
    virtual void zaxpby(const ptrdiff_t n, const T alpha, const T *const x, const T beta, const T *const y,
                        T *const z) = 0;
    virtual void xypaz(const ptrdiff_t n, const T *const x, const T *const y, const T alpha, T *const z) = 0;
    virtual bool good() const { return true; }
};

enum ExecutionSpace { EXECUTION_SPACE_HOST = 0, EXECUTION_SPACE_DEVICE = 1 };

template <typename T>
class Operator {
public:
    virtual ~Operator() = default;
    virtual int apply(const T *const x, T *const y) = 0;
    virtual std::ptrdiff_t rows() const = 0;
    virtual std::ptrdiff_t cols() const = 0;
    virtual ExecutionSpace execution_space() const = 0;
};

class Op {
public:
    virtual ~Op() = default;
    virtual const char *name() const = 0;
    virtual bool is_linear() const = 0;
    virtual int initialize(const std::vector<std::string> &block_names = {}) { return SFEM_GB300_SUCCESS; }
    virtual int hessian_crs(const real_t *const x, const count_t *const rowptr, const idx_t *const colidx,
                            real_t *const values) = 0;
    virtual int hessian_crs_sym(const real_t *const x, const count_t *const rowptr, const idx_t *const colidx,
                                real_t *const diag_values, real_t *const off_diag_values) {
        return SFEM_GB300_FAILURE;
    }
    virtual int hessian_block_diag_sym(const real_t *const x, real_t *const values) { return SFEM_GB300_FAILURE; }
    virtual int hessian_bsr(const real_t *const x, const count_t *const rowptr, const idx_t *const colidx,
                            real_t *const values) {
        return SFEM_GB300_FAILURE;
    }
    virtual int hessian_diag(const real_t *const x, real_t *const values) { return SFEM_GB300_FAILURE; }
    virtual int gradient(const real_t *const x, real_t *const out) = 0;
    virtual int apply(const real_t *const x, const real_t *const h, real_t *const out) = 0;
    virtual int value(const real_t *x, real_t *const out) = 0;
    virtual ExecutionSpace execution_space() const { return EXECUTION_SPACE_HOST; }
    virtual ptrdiff_t n_dofs_domain() const = 0;
    virtual ptrdiff_t n_dofs_image() const = 0;
};
}  // namespace interfaces

// The stream every adapter launches on (the C ABI's `stream` is a pointer to it).
class Stream {
public:
    explicit Stream(cudaStream_t s = nullptr) : s_(s) {}
    void *abi() { return &s_; }
    cudaStream_t get() const { return s_; }
    void synchronize() const { check_cuda(cudaStreamSynchronize(s_), "cudaStreamSynchronize"); }

private:
    cudaStream_t s_;
};

// sfem::BLAS<T> over the C ABI: every vector kernel of the reference's CUDA_BLAS
// (algebra/cuda/sfem_cuda_blas.hpp:55-77), with deterministic reductions.  dot / norm2
// return to the host (one synchronisation, as the reference's device dot does).
template <typename T, class Base>
class DeviceBLAS : public Base {
public:
    explicit DeviceBLAS(cudaStream_t stream = nullptr) : stream_(stream) {
        const size_t bytes = sfem_gb300_reduce_workspace_size();
        check_cuda(cudaMalloc(&workspace_, bytes), "DeviceBLAS workspace");
        check_cuda(cudaMemsetAsync(workspace_, 0, bytes, stream_.get()), "DeviceBLAS workspace");
        check_cuda(cudaMalloc((void **)&d_result_, sizeof(double)), "DeviceBLAS result");
    }
    ~DeviceBLAS() override {
        cudaFree(workspace_);
        cudaFree(d_result_);
    }
    DeviceBLAS(const DeviceBLAS &) = delete;
    DeviceBLAS &operator=(const DeviceBLAS &) = delete;

    T *allocate(const std::size_t n) override {
        T *p = nullptr;
        check_cuda(cudaMalloc((void **)&p, n * sizeof(T)), "DeviceBLAS::allocate");
        check_cuda(cudaMemsetAsync(p, 0, n * sizeof(T), stream_.get()), "DeviceBLAS::allocate");
        return p;
    }
    void destroy(void *a) override { cudaFree(a); }
    void zeros(const std::size_t size, T *const x) override { values(size, T(0), x); }
    void values(const std::size_t size, const T value, T *const x) override {
        check(sfem_gb300_values(rt, (ptrdiff_t)size, (double)value, x, stream_.abi()), "values");
    }
    void copy(const ptrdiff_t n, const T *const src, T *const dest) override {
        check_cuda(cudaMemcpyAsync(dest, src, n * sizeof(T), cudaMemcpyDeviceToDevice, stream_.get()), "copy");
    }
    T dot(const ptrdiff_t n, const T *const l, const T *const r) override {
        check(sfem_gb300_dot(rt, n, l, r, workspace_, d_result_, stream_.abi()), "dot");
        return (T)read_result();
    }
    void axpy(const ptrdiff_t n, const T alpha, const T *const x, T *const y) override {
        check(sfem_gb300_axpy(rt, n, (double)alpha, x, y, stream_.abi()), "axpy");
    }
    void axpby(const ptrdiff_t n, const T alpha, const T *const x, const T beta, T *const y) override {
        check(sfem_gb300_axpby(rt, n, (double)alpha, x, (double)beta, y, stream_.abi()), "axpby");
    }
    void scal(const std::ptrdiff_t n, const T alpha, T *const x) override {
        check(sfem_gb300_scal(rt, n, (double)alpha, x, stream_.abi()), "scal");
    }
    void reciprocal(const std::ptrdiff_t n, const T alpha, T *const x) override {
        check(sfem_gb300_reciprocal(rt, n, (double)alpha, x, stream_.abi()), "reciprocal");
    }
    T norm2(const ptrdiff_t n, const T *const x) override {
        check(sfem_gb300_norm2(rt, n, x, workspace_, d_result_, stream_.abi()), "norm2");
        return (T)read_result();
    }
    void zaxpby(const ptrdiff_t n, const T alpha, const T *const x, const T beta, const T *const y,
                T *const z) override {
        check(sfem_gb300_zaxpby(rt, n, (double)alpha, x, (double)beta, y, z, stream_.abi()), "zaxpby");
    }
    void xypaz(const ptrdiff_t n, const T *const x, const T *const y, const T alpha, T *const z) override {
        check(sfem_gb300_xypaz(rt, n, x, y, (double)alpha, z, stream_.abi()), "xypaz");
    }

private:
    static constexpr int rt = real_type_of<T>();
    double read_result() {
        double h = 0;
        check_cuda(cudaMemcpyAsync(&h, d_result_, sizeof(double), cudaMemcpyDeviceToHost, stream_.get()), "result");
        stream_.synchronize();
        return h;
    }
    Stream stream_;
    void *workspace_{nullptr};
    double *d_result_{nullptr};
};

// sfem::Operator<T> around any apply (the reference's make_op lambdas,
// algebra/sfem_Operator.hpp:141-147), typically an Op's apply with its constraints.
template <typename T, class Base, auto ES>
class DeviceOperator : public Base {
public:
    DeviceOperator(std::ptrdiff_t rows, std::ptrdiff_t cols, std::function<int(const T *, T *)> fn)
        : rows_(rows), cols_(cols), fn_(std::move(fn)) {}
    int apply(const T *const x, T *const y) override { return fn_(x, y); }
    std::ptrdiff_t rows() const override { return rows_; }
    std::ptrdiff_t cols() const override { return cols_; }
    decltype(ES) execution_space() const override { return ES; }

private:
    std::ptrdiff_t rows_, cols_;
    std::function<int(const T *, T *)> fn_;
};

// Shared part of the GPU ops: energy value 1/2 x.A x from an apply.
namespace detail {
inline int quadratic_value(ptrdiff_t n, const real_t *x, real_t *out, void *stream,
                           const std::function<int(const real_t *, real_t *)> &apply_fn) {
    real_t *y = nullptr;
    void *ws = nullptr;
    double *d = nullptr;
    int rc = SFEM_GB300_FAILURE;
    const cudaStream_t s = stream ? *static_cast<cudaStream_t *>(stream) : nullptr;
    if (cudaMalloc((void **)&y, n * sizeof(real_t)) == cudaSuccess &&
        cudaMalloc(&ws, sfem_gb300_reduce_workspace_size()) == cudaSuccess &&
        cudaMalloc((void **)&d, sizeof(double)) == cudaSuccess) {
        cudaMemsetAsync(ws, 0, sfem_gb300_reduce_workspace_size(), s);
        cudaMemsetAsync(y, 0, n * sizeof(real_t), s);
        rc = apply_fn(x, y);
        if (rc == SFEM_GB300_SUCCESS) rc = sfem_gb300_dot(SFEM_GB300_FLOAT64, n, x, y, ws, d, stream);
        double h = 0;
        if (rc == SFEM_GB300_SUCCESS) {
            cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, s);
            cudaStreamSynchronize(s);
            *out += 0.5 * h;
        }
    }
    cudaFree(y);
    cudaFree(ws);
    cudaFree(d);
    return rc;
}
}  // namespace detail

// The reference's GPU Laplacian op on the C ABI.  The caller passes what the reference's
// FunctionSpace holds on the device: the element index arrays (device array of device
// pointers, SoA), the 8 macro-corner index arrays in hex8 order (for the metric) and the
// 3 coordinate arrays.  initialize() computes and caches the FFF (SoA float).
template <class Base, auto ES>
class LaplacianOp : public Base {
public:
    LaplacianOp(int element_type, ptrdiff_t nelements, idx_t **elements, idx_t **corners, float **points,
                ptrdiff_t n_nodes, cudaStream_t stream = nullptr)
        : element_type_(element_type), nelements_(nelements), elements_(elements), corners_(corners),
          points_(points), n_nodes_(n_nodes), stream_(stream) {}
    ~LaplacianOp() override { cudaFree(fff_); }
    LaplacianOp(const LaplacianOp &) = delete;
    LaplacianOp &operator=(const LaplacianOp &) = delete;

    const char *name() const override { return "gpu:Laplacian"; }
    bool is_linear() const override { return true; }
    int initialize(const std::vector<std::string> & = {}) override {
        if (!fff_ && cudaMalloc((void **)&fff_, 6 * (size_t)nelements_ * sizeof(float)) != cudaSuccess)
            return SFEM_GB300_FAILURE;
        return sfem_gb300_hex8_fff_fill(nelements_, corners_, points_, nelements_, fff_, stream_.abi());
    }
    int hessian_crs(const real_t *const, const count_t *const rowptr, const idx_t *const colidx,
                    real_t *const values) override {
        return cu_laplacian_crs(element_type_, nelements_, elements_, nelements_, fff_, rowptr, colidx,
                                SFEM_GB300_FLOAT64, values, stream_.abi());
    }
    int hessian_crs_sym(const real_t *const, const count_t *const rowptr, const idx_t *const colidx,
                        real_t *const diag_values, real_t *const off_diag_values) override {
        return cu_laplacian_crs_sym(element_type_, nelements_, elements_, nelements_, fff_, rowptr, colidx,
                                    SFEM_GB300_FLOAT64, diag_values, off_diag_values, stream_.abi());
    }
    int hessian_diag(const real_t *const, real_t *const values) override {
        return cu_laplacian_diag(element_type_, nelements_, elements_, nelements_, fff_, SFEM_GB300_FLOAT64, values,
                                 stream_.abi());
    }
    int gradient(const real_t *const x, real_t *const out) override { return apply(nullptr, x, out); }
    int apply(const real_t *const, const real_t *const h, real_t *const out) override {
        return cu_laplacian_apply(element_type_, nelements_, elements_, nelements_, fff_, SFEM_GB300_FLOAT64, h, out,
                                  stream_.abi());
    }
    int value(const real_t *x, real_t *const out) override {
        return detail::quadratic_value(n_nodes_, x, out, stream_.abi(),
                                       [this](const real_t *a, real_t *b) { return apply(nullptr, a, b); });
    }
    decltype(ES) execution_space() const override { return ES; }
    ptrdiff_t n_dofs_domain() const override { return n_nodes_; }
    ptrdiff_t n_dofs_image() const override { return n_nodes_; }
    const float *fff() const { return fff_; }

private:
    int element_type_;
    ptrdiff_t nelements_;
    idx_t **elements_, **corners_;
    float **points_;
    ptrdiff_t n_nodes_;
    Stream stream_;
    float *fff_{nullptr};
};

// The reference's GPU linear-elasticity op (interleaved xyz dofs) on the C ABI;
// initialize() caches the adjugate and determinant (SoA float).
template <class Base, auto ES>
class LinearElasticityOp : public Base {
public:
    LinearElasticityOp(int element_type, ptrdiff_t nelements, idx_t **elements, idx_t **corners, float **points,
                       ptrdiff_t n_nodes, real_t mu, real_t lambda, cudaStream_t stream = nullptr)
        : element_type_(element_type), nelements_(nelements), elements_(elements), corners_(corners),
          points_(points), n_nodes_(n_nodes), mu_(mu), lambda_(lambda), stream_(stream) {}
    ~LinearElasticityOp() override {
        cudaFree(adj_);
        cudaFree(det_);
    }
    LinearElasticityOp(const LinearElasticityOp &) = delete;
    LinearElasticityOp &operator=(const LinearElasticityOp &) = delete;

    const char *name() const override { return "gpu:LinearElasticity"; }
    bool is_linear() const override { return true; }
    int initialize(const std::vector<std::string> & = {}) override {
        if (!adj_ && (cudaMalloc((void **)&adj_, 9 * (size_t)nelements_ * sizeof(float)) != cudaSuccess ||
                      cudaMalloc((void **)&det_, (size_t)nelements_ * sizeof(float)) != cudaSuccess))
            return SFEM_GB300_FAILURE;
        return sfem_gb300_hex8_adjugate_fill(nelements_, corners_, points_, nelements_, adj_, det_, stream_.abi());
    }
    int hessian_crs(const real_t *const, const count_t *const, const idx_t *const, real_t *const) override {
        return SFEM_GB300_FAILURE;  // the vector operator assembles into BSR (hessian_bsr)
    }
    int hessian_bsr(const real_t *const, const count_t *const rowptr, const idx_t *const colidx,
                    real_t *const values) override {
        return cu_linear_elasticity_bsr(element_type_, nelements_, elements_, nelements_, adj_, det_, mu_, lambda_,
                                        SFEM_GB300_FLOAT64, rowptr, colidx, values, stream_.abi());
    }
    int hessian_diag(const real_t *const, real_t *const values) override {
        return cu_linear_elasticity_diag(element_type_, nelements_, elements_, nelements_, adj_, det_, mu_, lambda_,
                                         SFEM_GB300_FLOAT64, values, stream_.abi());
    }
    int hessian_block_diag_sym(const real_t *const, real_t *const values) override {
        return cu_linear_elasticity_block_diag_sym_aos(element_type_, nelements_, elements_, nelements_, adj_, det_,
                                                       mu_, lambda_, SFEM_GB300_FLOAT64, values, stream_.abi());
    }
    int gradient(const real_t *const x, real_t *const out) override { return apply(nullptr, x, out); }
    int apply(const real_t *const, const real_t *const h, real_t *const out) override {
        return cu_linear_elasticity_apply(element_type_, nelements_, elements_, nelements_, adj_, det_, mu_, lambda_,
                                          SFEM_GB300_FLOAT64, h, out, stream_.abi());
    }
    int value(const real_t *x, real_t *const out) override {
        return detail::quadratic_value(3 * n_nodes_, x, out, stream_.abi(),
                                       [this](const real_t *a, real_t *b) { return apply(nullptr, a, b); });
    }
    decltype(ES) execution_space() const override { return ES; }
    ptrdiff_t n_dofs_domain() const override { return 3 * n_nodes_; }
    ptrdiff_t n_dofs_image() const override { return 3 * n_nodes_; }

private:
    int element_type_;
    ptrdiff_t nelements_;
    idx_t **elements_, **corners_;
    float **points_;
    ptrdiff_t n_nodes_;
    real_t mu_, lambda_;
    Stream stream_;
    float *adj_{nullptr}, *det_{nullptr};
};

}  // namespace adapter
}  // namespace sfem_gb300

#endif  // SFEM_GB300_ADAPTER_HPP
