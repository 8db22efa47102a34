// Opaque handle of the solver object layer and helpers shared by the C ABI
// translation units (single-problem solvers and batched solvers).
#pragma once

#include <memory>
#include <string>

#include "common.cuh"
#include "solvers.hpp"

namespace sfem_gb300 {

struct Handle {
    int real_type{SFEM_GB300_FLOAT64};
    std::string kind;
    std::shared_ptr<Context> ctx;
    std::shared_ptr<Operator<double>> d;
    std::shared_ptr<Operator<float>> f;
    // typed views for kind-specific calls
    std::shared_ptr<void> impl;
    ptrdiff_t rows() const { return d ? d->rows() : (f ? f->rows() : 0); }
    ptrdiff_t cols() const { return d ? d->cols() : (f ? f->cols() : 0); }
};

inline bool is_f32(int rt) { return rt == SFEM_GB300_FLOAT32 || rt == SFEM_GB300_FLOAT32_BF16TC; }

template <typename T>
std::shared_ptr<Operator<T>> &op_of(Handle *h);
template <>
inline std::shared_ptr<Operator<double>> &op_of<double>(Handle *h) {
    return h->d;
}
template <>
inline std::shared_ptr<Operator<float>> &op_of<float>(Handle *h) {
    return h->f;
}

template <typename T>
Blas<T> blas_of(const std::shared_ptr<Context> &ctx) {
    Blas<T> b;
    b.ctx = ctx;
    return b;
}

#define H(p) reinterpret_cast<::sfem_gb300::Handle *>(p)

}  // namespace sfem_gb300
