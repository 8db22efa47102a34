// Compensated residual r = b - A x (double-double accumulation), sm_103a.
//
// The FP64 operator's entries are doubles (stored micro element matrices); the products
// A_ij x_j are split exactly into p + e with a fused multiply-add, the sums are carried as
// (hi, lo) pairs with TwoSum, and the scatter to shared nodes stays error-free: an
// atomicAdd on hi returns the value it added to, so the rounding error of that addition is
// recomputed exactly (TwoSum of the returned value and the addend) and added to lo.  The
// result equals the exact residual of the FP64 operator to about 1e-30 relative to
// (|A||x|)_i, where a plain FP64 evaluation carries errors near 1e-16 (|A||x|)_i -- the
// difference that decides whether a relative residual of 1e-10 can be certified on
// ill-conditioned problems (a clamped 4:1 cantilever: |A||x| / |b| near 1e6).
//
// No reference counterpart: the reference evaluates residuals in the working precision
// (drivers/mgsolve.cpp:315, algebra/sfem_cg.hpp:226-230).
#include <algorithm>

#include "common.cuh"

namespace sfem_gb300 {
namespace {

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void dd_fma(double &hi, double &lo, double a, double b) {
    const double p = a * b;
    const double pe = fma(a, b, -p);
    double s, e;
    two_sum(hi, p, s, e);
    hi = s;
    lo += e + pe;
}

// hex8 corner c of micro element m of an sshex8 level-L macro element: its local node
// (lidx order); L == 0 is a plain hex8 mesh whose 8 index arrays are already in corner order
__device__ __forceinline__ int micro_node(int L, int m, int c) {
    if (L == 0) return c;
    const int xi = m % L, yi = (m / L) % L, zi = m / (L * L);
    return lidx(L, xi + c8x(c), yi + c8y(c), zi + c8z(c));
}

// One CTA per macro element: stage the element matrix and the element's x in shared
// memory, then every (micro element, row) pair forms its row product in double-double
// and scatters it error-free into (hi, lo).
template <int BS>
__global__ void __launch_bounds__(128) residual_dd_scatter_kernel(int L, ptrdiff_t nelements,
                                                                  const idx_t *const *elements,
                                                                  const double *__restrict__ em,
                                                                  const double *__restrict__ x,
                                                                  const double *__restrict__ x_lo, double *hi,
                                                                  double *lo) {
    constexpr int NE = 8 * BS;
    extern __shared__ __align__(16) unsigned char rdd_smem[];
    double *K = reinterpret_cast<double *>(rdd_smem);
    const int Lm = L > 0 ? L : 1;
    const int nxe = L > 0 ? (L + 1) * (L + 1) * (L + 1) : 8;
    double *xe = K + NE * NE;
    double *xl = xe + nxe * BS;
    idx_t *ids = reinterpret_cast<idx_t *>(xl + nxe * BS);
    const int nm = Lm * Lm * Lm;
    for (ptrdiff_t e = blockIdx.x; e < nelements; e += gridDim.x) {
        for (int k = threadIdx.x; k < NE * NE; k += blockDim.x) K[k] = em[e * NE * NE + k];
        for (int v = threadIdx.x; v < nxe; v += blockDim.x) {
            const idx_t g = elements[v][e];
            ids[v] = g;
#pragma unroll
            for (int d = 0; d < BS; d++) {
                xe[v * BS + d] = x[(ptrdiff_t)g * BS + d];
                xl[v * BS + d] = x_lo ? x_lo[(ptrdiff_t)g * BS + d] : 0.0;
            }
        }
        __syncthreads();
        for (int w = threadIdx.x; w < nm * NE; w += blockDim.x) {
            const int m = w / NE, i = w % NE;
            double h = 0, l = 0;
            for (int j = 0; j < NE; j++) {
                const int q = micro_node(L, m, j % 8) * BS + j / 8;
                dd_fma(h, l, K[i * NE + j], xe[q]);
                l = fma(K[i * NE + j], xl[q], l);  // the low part of x: its product's error is negligible
            }
            const ptrdiff_t dof = (ptrdiff_t)ids[micro_node(L, m, i % 8)] * BS + i / 8;
            const double old = atomicAdd(&hi[dof], h);
            double s, err;
            two_sum(old, h, s, err);  // s is the value the atomic stored
            atomicAdd(&lo[dof], err + l);
        }
        __syncthreads();
    }
}

__global__ void residual_dd_finish_kernel(ptrdiff_t n, const double *__restrict__ b, const double *__restrict__ hi,
                                          const double *__restrict__ lo, double *r) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        double s, e;
        two_sum(b[i], -hi[i], s, e);
        r[i] = s + (e - lo[i]);
    }
}

__global__ void residual_dd_dirichlet_kernel(ptrdiff_t nd, const int32_t *nodes, int bs, const double *b,
                                             const double *x, const double *x_lo, double *r) {
    for (ptrdiff_t k = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; k < nd * bs;
         k += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t dof = (ptrdiff_t)nodes[k / bs] * bs + k % bs;
        r[dof] = (b[dof] - x[dof]) - (x_lo ? x_lo[dof] : 0.0);
    }
}

// (x_hi, x_lo) += e with TwoSum: the solution kept as an unevaluated double-double sum
__global__ void dd_axpy_kernel(ptrdiff_t n, double alpha, const double *__restrict__ e, double *x_hi, double *x_lo) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        double s, err;
        two_sum(x_hi[i], alpha * e[i], s, err);
        x_hi[i] = s;
        x_lo[i] += err;
    }
}

}  // namespace
}  // namespace sfem_gb300

using namespace sfem_gb300;

extern "C" int sfem_gb300_residual_dd(int element_type, int block_size, ptrdiff_t nelements, idx_t **elements,
                                      const double *element_matrices, ptrdiff_t n_dofs, const double *x,
                                      const double *x_lo, const double *b, ptrdiff_t n_dirichlet,
                                      const int32_t *dirichlet, double *work, double *r, void *stream) {
    const cudaStream_t s = stream_of(stream);
    int L;
    if (element_type == SFEM_GB300_HEX8)
        L = 0;
    else
        L = element_type - SFEM_GB300_SSHEX8_BASE;
    if (L < 0 || L > 16 || (L == 0 && element_type != SFEM_GB300_HEX8))
        return set_error("sfem_gb300_residual_dd: unsupported element type %d", element_type);
    if (block_size != 1 && block_size != 3)
        return set_error("sfem_gb300_residual_dd: block size %d (1 or 3)", block_size);
    if (n_dofs < 0 || nelements < 0) return set_error("sfem_gb300_residual_dd: negative size");
    double *hi = work, *lo = work + n_dofs;
    if (cudaMemsetAsync(work, 0, 2 * (size_t)n_dofs * sizeof(double), s) != cudaSuccess)
        return set_error("sfem_gb300_residual_dd: clearing the work array failed");
    if (nelements > 0) {
        const int ne = 8 * block_size;
        const int nxe = L > 0 ? (L + 1) * (L + 1) * (L + 1) : 8;
        const size_t smem = (size_t)ne * ne * sizeof(double) + 2 * (size_t)nxe * block_size * sizeof(double) +
                            (size_t)nxe * sizeof(idx_t);
        if (smem > 200 * 1024) return set_error("sfem_gb300_residual_dd: level %d too large", L);
        const int grid = (int)std::min<ptrdiff_t>(nelements, (ptrdiff_t)kNumSMs * 8);
        if (block_size == 1) {
            if (smem > 48 * 1024)
                cudaFuncSetAttribute(residual_dd_scatter_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
            residual_dd_scatter_kernel<1><<<grid, 128, smem, s>>>(L, nelements, elements, element_matrices, x, x_lo,
                                                                   hi, lo);
        } else {
            if (smem > 48 * 1024)
                cudaFuncSetAttribute(residual_dd_scatter_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
            residual_dd_scatter_kernel<3><<<grid, 128, smem, s>>>(L, nelements, elements, element_matrices, x, x_lo,
                                                                   hi, lo);
        }
        if (check_launch("sfem_gb300_residual_dd (scatter)")) return SFEM_GB300_FAILURE;
    }
    if (n_dofs > 0) {
        residual_dd_finish_kernel<<<grid_for(n_dofs, 256), 256, 0, s>>>(n_dofs, b, hi, lo, r);
        if (check_launch("sfem_gb300_residual_dd (finish)")) return SFEM_GB300_FAILURE;
    }
    if (n_dirichlet > 0) {
        residual_dd_dirichlet_kernel<<<grid_for(n_dirichlet * block_size, 256), 256, 0, s>>>(n_dirichlet, dirichlet,
                                                                                             block_size, b, x, x_lo, r);
        return check_launch("sfem_gb300_residual_dd (constraints)");
    }
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_dd_axpy(ptrdiff_t n, double alpha, const double *e, double *x_hi, double *x_lo,
                                  void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    dd_axpy_kernel<<<grid_for(n, 256), 256, 0, stream_of(stream)>>>(n, alpha, e, x_hi, x_lo);
    return check_launch("sfem_gb300_dd_axpy");
}
