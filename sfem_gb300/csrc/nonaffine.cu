// Non-affine sshex8 Laplacian apply, sm_103a (a correctness path, not tuned).
//
// Reference: sshex8_laplacian_apply (operators/sshex8/sshex8_laplacian.cpp:39-182).  A
// macro element's geometry is the trilinear map of its 8 corner nodes; every micro
// element is integrated with the six-point rule at the face centres of its reference
// cube (weights 1/6, the reference's q6 rule, operators/hex8/hex8_quadrature.hpp:4-15),
// the FFF det(J) J^-1 J^-T of the macro map evaluated at each point's macro coordinates
// and scaled by h = 1/L to the micro element (the reference's hex8_sub_fff_0, :19-28):
// v_i += w grad phi_i(q) . (G grad u(q)).  One CTA per macro element (grid-stride), one
// thread per micro element, the element's values and results in shared memory
// (shared-memory atomics for the micro elements around a node), atomics into y.
#include <algorithm>

#include "common.cuh"

namespace sfem_gb300 {
namespace {

// face centre k of the unit cube
__device__ __forceinline__ void q6_point(int k, double &qx, double &qy, double &qz) {
    qx = k == 0 ? 0.0 : k == 5 ? 1.0 : 0.5;
    qy = k == 1 ? 0.0 : k == 4 ? 1.0 : 0.5;
    qz = k == 2 ? 0.0 : k == 3 ? 1.0 : 0.5;
}

// gradient of the trilinear basis function of corner c at (qx, qy, qz)
template <typename T>
__device__ __forceinline__ void q1_grad(int c, T qx, T qy, T qz, T (&g)[3]) {
    const T wx = c8x(c) ? qx : T(1) - qx, wy = c8y(c) ? qy : T(1) - qy, wz = c8z(c) ? qz : T(1) - qz;
    const T sx = c8x(c) ? T(1) : T(-1), sy = c8y(c) ? T(1) : T(-1), sz = c8z(c) ? T(1) : T(-1);
    g[0] = sx * wy * wz;
    g[1] = wx * sy * wz;
    g[2] = wx * wy * sz;
}

template <typename T>
__global__ void __launch_bounds__(128) sshex8_laplacian_nonaffine_kernel(int L, ptrdiff_t nelements,
                                                                         const idx_t *const *elements,
                                                                         const float *__restrict__ px,
                                                                         const float *__restrict__ py,
                                                                         const float *__restrict__ pz,
                                                                         const T *__restrict__ x, T *__restrict__ y) {
    extern __shared__ __align__(16) unsigned char na_smem[];
    const int N1 = L + 1, NXE = N1 * N1 * N1, NM = L * L * L;
    T *eu = reinterpret_cast<T *>(na_smem);
    T *ev = eu + NXE;
    idx_t *ids = reinterpret_cast<idx_t *>(ev + NXE);
    __shared__ T cx[8], cy[8], cz[8];
    const T h = T(1) / T(L);
    for (ptrdiff_t e = blockIdx.x; e < nelements; e += gridDim.x) {
        for (int v = threadIdx.x; v < NXE; v += blockDim.x) {
            const idx_t g = elements[v][e];
            ids[v] = g;
            eu[v] = x[g];
            ev[v] = T(0);
        }
        if (threadIdx.x < 8) {
            const int c = threadIdx.x;
            const idx_t g = elements[lidx(L, c8x(c) * L, c8y(c) * L, c8z(c) * L)][e];
            cx[c] = (T)px[g];
            cy[c] = (T)py[g];
            cz[c] = (T)pz[g];
        }
        __syncthreads();
        for (int m = threadIdx.x; m < NM; m += blockDim.x) {
            const int xi = m % L, yi = (m / L) % L, zi = m / (L * L);
            int lev[8];
            T ue[8], ve[8];
#pragma unroll
            for (int c = 0; c < 8; c++) {
                lev[c] = lidx(L, xi + c8x(c), yi + c8y(c), zi + c8z(c));
                ue[c] = eu[lev[c]];
                ve[c] = T(0);
            }
#pragma unroll 1
            for (int k = 0; k < 6; k++) {
                double dqx, dqy, dqz;
                q6_point(k, dqx, dqy, dqz);
                const T qx = (T)dqx, qy = (T)dqy, qz = (T)dqz;
                // Jacobian of the macro map at the point's macro coordinates
                T J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                const T mx = h * (T(xi) + qx), my = h * (T(yi) + qy), mz = h * (T(zi) + qz);
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    T g[3];
                    q1_grad<T>(c, mx, my, mz, g);
#pragma unroll
                    for (int p = 0; p < 3; p++) {
                        J[0][p] += cx[c] * g[p];
                        J[1][p] += cy[c] * g[p];
                        J[2][p] += cz[c] * g[p];
                    }
                }
                // adj = det(J) J^-1; sub-FFF G = h adj adj^T / det
                const T a0 = J[1][1] * J[2][2] - J[1][2] * J[2][1], a1 = J[0][2] * J[2][1] - J[0][1] * J[2][2],
                        a2 = J[0][1] * J[1][2] - J[0][2] * J[1][1], a3 = J[1][2] * J[2][0] - J[1][0] * J[2][2],
                        a4 = J[0][0] * J[2][2] - J[0][2] * J[2][0], a5 = J[0][2] * J[1][0] - J[0][0] * J[1][2],
                        a6 = J[1][0] * J[2][1] - J[1][1] * J[2][0], a7 = J[0][1] * J[2][0] - J[0][0] * J[2][1],
                        a8 = J[0][0] * J[1][1] - J[0][1] * J[1][0];
                const T det = J[0][0] * a0 + J[0][1] * a3 + J[0][2] * a6;
                const T s = h / det;
                const T G00 = s * (a0 * a0 + a1 * a1 + a2 * a2), G01 = s * (a0 * a3 + a1 * a4 + a2 * a5),
                        G02 = s * (a0 * a6 + a1 * a7 + a2 * a8), G11 = s * (a3 * a3 + a4 * a4 + a5 * a5),
                        G12 = s * (a3 * a6 + a4 * a7 + a5 * a8), G22 = s * (a6 * a6 + a7 * a7 + a8 * a8);
                // grad u at the point (micro reference coordinates), then w G grad u
                T gu[3] = {0, 0, 0};
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    T g[3];
                    q1_grad<T>(c, qx, qy, qz, g);
#pragma unroll
                    for (int p = 0; p < 3; p++) gu[p] += g[p] * ue[c];
                }
                const T w = T(1) / T(6);
                const T t0 = w * (G00 * gu[0] + G01 * gu[1] + G02 * gu[2]);
                const T t1 = w * (G01 * gu[0] + G11 * gu[1] + G12 * gu[2]);
                const T t2 = w * (G02 * gu[0] + G12 * gu[1] + G22 * gu[2]);
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    T g[3];
                    q1_grad<T>(c, qx, qy, qz, g);
                    ve[c] += g[0] * t0 + g[1] * t1 + g[2] * t2;
                }
            }
#pragma unroll
            for (int c = 0; c < 8; c++) atomicAdd(&ev[lev[c]], ve[c]);
        }
        __syncthreads();
        for (int v = threadIdx.x; v < NXE; v += blockDim.x) atomicAdd(&y[ids[v]], ev[v]);
        __syncthreads();
    }
}

template <typename T>
int nonaffine_launch(int L, ptrdiff_t nelements, idx_t **elements, const float *px, const float *py, const float *pz,
                     const T *x, T *y, cudaStream_t s) {
    const int nxe = (L + 1) * (L + 1) * (L + 1);
    const size_t smem = (size_t)nxe * (2 * sizeof(T) + sizeof(idx_t));
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(sshex8_laplacian_nonaffine_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    const int grid = (int)std::min<ptrdiff_t>(nelements, (ptrdiff_t)kNumSMs * 8);
    sshex8_laplacian_nonaffine_kernel<T><<<grid, 128, smem, s>>>(L, nelements, elements, px, py, pz, x, y);
    return check_launch("sfem_gb300_sshex8_laplacian_apply_nonaffine");
}

}  // namespace
}  // namespace sfem_gb300

using namespace sfem_gb300;

extern "C" int sfem_gb300_sshex8_laplacian_apply_nonaffine(int element_type, ptrdiff_t nelements, idx_t **elements,
                                                           const float *points_x, const float *points_y,
                                                           const float *points_z, int real_type_xy, const void *x,
                                                           void *y, void *stream) {
    const int L = element_type - SFEM_GB300_SSHEX8_BASE;
    if (L < 1 || L > 16)
        return set_error("sfem_gb300_sshex8_laplacian_apply_nonaffine: element type %d is not sshex8 L = 1..16",
                         element_type);
    if (nelements < 0) return set_error("sfem_gb300_sshex8_laplacian_apply_nonaffine: negative element count");
    if (nelements == 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    if (real_type_xy == SFEM_GB300_FLOAT32)
        return nonaffine_launch<float>(L, nelements, elements, points_x, points_y, points_z, (const float *)x,
                                       (float *)y, s);
    if (real_type_xy == SFEM_GB300_FLOAT64 || real_type_xy == SFEM_GB300_REAL_DEFAULT)
        return nonaffine_launch<double>(L, nelements, elements, points_x, points_y, points_z, (const double *)x,
                                        (double *)y, s);
    return set_error("sfem_gb300_sshex8_laplacian_apply_nonaffine: unsupported real type %d", real_type_xy);
}
