// Shared definitions for the sfem_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "sfem_gb300.h"

namespace sfem_gb300 {

typedef int32_t idx_t;

// Records a formatted error message for sfem_gb300_last_error() and returns SFEM_GB300_FAILURE.
int set_error(const char *fmt, ...);

// Resolves the reference's stream convention: a pointer to a cudaStream_t, or NULL for the default stream.
static inline cudaStream_t stream_of(void *stream) { return stream ? *static_cast<cudaStream_t *>(stream) : (cudaStream_t)0; }

// Checks the launch status of the last kernel (non-blocking).
int check_launch(const char *what);

static inline int grid_for(ptrdiff_t n, int block, int max_blocks = 152 * 32) {
    ptrdiff_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > max_blocks) g = max_blocks;
    return (int)g;
}

constexpr int kNumSMs = 152;

// sshex8 local index (operators/sshex8/sshex8.hpp:18-24)
__host__ __device__ constexpr int lidx(int L, int x, int y, int z) { return z * (L + 1) * (L + 1) + y * (L + 1) + x; }

// standard hex8 corner offsets (operators/sshex8/sshex8.hpp:53-62)
__host__ __device__ constexpr int c8x(int c) { return (c == 1 || c == 2 || c == 5 || c == 6) ? 1 : 0; }
__host__ __device__ constexpr int c8y(int c) { return (c == 2 || c == 3 || c == 6 || c == 7) ? 1 : 0; }
__host__ __device__ constexpr int c8z(int c) { return c >= 4 ? 1 : 0; }

// Q1 reference integrals on [0,1]^3: int d_p phi_c d_q phi_e.
// 1D: int psi_a psi_b = 1/3 | 1/6 ; int psi'_a psi'_b = +-1 ; int psi'_a psi_b = -+1/2.
__host__ __device__ constexpr double q1_m(int a, int b) { return a == b ? (1.0 / 3.0) : (1.0 / 6.0); }
__host__ __device__ constexpr double q1_k(int a, int b) { return a == b ? 1.0 : -1.0; }
__host__ __device__ constexpr double q1_g(int a) { return a ? 0.5 : -0.5; }
__host__ __device__ constexpr int c8(int c, int d) { return d == 0 ? c8x(c) : (d == 1 ? c8y(c) : c8z(c)); }
__host__ __device__ constexpr double q1_grad_integral(int c, int e, int p, int q) {
    double r = 1.0;
    for (int d = 0; d < 3; d++) {
        const int a = c8(c, d), b = c8(e, d);
        if (d == p && d == q)
            r *= q1_k(a, b);
        else if (d == p)
            r *= q1_g(a);
        else if (d == q)
            r *= q1_g(b);
        else
            r *= q1_m(a, b);
    }
    return r;
}

// Weight of sym. metric entry m (00,01,02,11,12,22) in Laplacian element-matrix entry (c,e).
__host__ __device__ constexpr double lap_weight(int c, int e, int m) {
    return m == 0   ? q1_grad_integral(c, e, 0, 0)
           : m == 1 ? q1_grad_integral(c, e, 0, 1) + q1_grad_integral(c, e, 1, 0)
           : m == 2 ? q1_grad_integral(c, e, 0, 2) + q1_grad_integral(c, e, 2, 0)
           : m == 3 ? q1_grad_integral(c, e, 1, 1)
           : m == 4 ? q1_grad_integral(c, e, 1, 2) + q1_grad_integral(c, e, 2, 1)
                    : q1_grad_integral(c, e, 2, 2);
}

template <typename T>
__device__ __forceinline__ void atomic_add(T *p, T v) {
    atomicAdd(p, v);
}

}  // namespace sfem_gb300
