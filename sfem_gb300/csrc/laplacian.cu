// Matrix-free Laplacian on hex8 and semi-structured hex8 (sshex8) meshes, sm_103a.
//
// Operator (reference: affine_sshex8_laplacian_stencil_apply_fff,
// operators/sshex8/sshex8_laplacian.cpp:698-769, and hex8_laplacian_apply_opt,
// operators/hex8/hex8_laplacian.cpp:309-345): one metric (FFF, 6 floats) per
// macro element, sub-metric FFF/L for each of the L^3 micro elements, element
// matrix A = sum_m f_m W_m with the exact Q1 integrals W_m, y += A x.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <atomic>
#include <mutex>

#include "common.cuh"
#include "laplacian_kernels.cuh"
#include "tcgen05.cuh"
#include "tiles.cuh"

namespace sfem_gb300 {

// ------------------------------------------------------------------ geometry

__device__ inline void hex8_center_jacobian(const double *x, const double *y, const double *z, double J[3][3]) {
    // d x_i / d xi_p at (1/2,1/2,1/2) of the trilinear map
    for (int i = 0; i < 3; i++)
        for (int p = 0; p < 3; p++) J[i][p] = 0;
    const double *X[3] = {x, y, z};
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const double dphi[3] = {(c8x(c) ? 0.25 : -0.25), (c8y(c) ? 0.25 : -0.25), (c8z(c) ? 0.25 : -0.25)};
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int p = 0; p < 3; p++) J[i][p] += X[i][c] * dphi[p];
    }
}

__device__ inline double adjugate_det(const double J[3][3], double adj[9]) {
    adj[0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    adj[1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    adj[2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    adj[3] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    adj[4] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    adj[5] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    adj[6] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    adj[7] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    adj[8] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    return J[0][0] * adj[0] + J[0][1] * adj[3] + J[0][2] * adj[6];
}

__global__ void hex8_geometry_kernel(ptrdiff_t nelements, const idx_t *const *corners, const float *const *points,
                                     ptrdiff_t stride, float *fff, float *adjugate, float *determinant) {
    for (ptrdiff_t e = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; e < nelements;
         e += (ptrdiff_t)gridDim.x * blockDim.x) {
        double x[8], y[8], z[8];
#pragma unroll
        for (int v = 0; v < 8; v++) {
            const idx_t n = corners[v][e];
            x[v] = points[0][n];
            y[v] = points[1][n];
            z[v] = points[2][n];
        }
        double J[3][3], adj[9];
        hex8_center_jacobian(x, y, z, J);
        const double det = adjugate_det(J, adj);
        if (fff) {
            double G[6];
            const int pq[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
#pragma unroll
            for (int m = 0; m < 6; m++) {
                const int p = pq[m][0], q = pq[m][1];
                G[m] = (adj[3 * p] * adj[3 * q] + adj[3 * p + 1] * adj[3 * q + 1] + adj[3 * p + 2] * adj[3 * q + 2]) / det;
                fff[m * stride + e] = (float)G[m];
            }
        }
        if (adjugate) {
#pragma unroll
            for (int d = 0; d < 9; d++) adjugate[d * stride + e] = (float)adj[d];
            determinant[e] = (float)det;
        }
    }
}

// ------------------------------------------------------------------ hex8 apply

// One thread per element: coalesced SoA index / FFF loads, 8 gathers, 8 atomic scatters.
template <typename T>
__global__ void __launch_bounds__(128) hex8_laplacian_apply_kernel(ptrdiff_t nelements, const idx_t *const *elements,
                                                                   ptrdiff_t fff_stride, const float *fff, const T *x,
                                                                   T *y) {
    for (ptrdiff_t e = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; e < nelements;
         e += (ptrdiff_t)gridDim.x * blockDim.x) {
        idx_t ev[8];
        T u[8], f[6];
#pragma unroll
        for (int v = 0; v < 8; v++) ev[v] = elements[v][e];
#pragma unroll
        for (int m = 0; m < 6; m++) f[m] = (T)fff[m * fff_stride + e];
#pragma unroll
        for (int v = 0; v < 8; v++) u[v] = x[ev[v]];
#pragma unroll
        for (int i = 0; i < 8; i++) {
            T acc = 0;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                T a = 0;
#pragma unroll
                for (int m = 0; m < 6; m++) a += f[m] * lap_w<T>(i * 8 + j, m);
                acc += a * u[j];
            }
            atomicAdd(&y[ev[i]], acc);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(128) hex8_laplacian_diag_kernel(ptrdiff_t nelements, const idx_t *const *elements,
                                                                  ptrdiff_t fff_stride, const float *fff, T *diag) {
    for (ptrdiff_t e = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; e < nelements;
         e += (ptrdiff_t)gridDim.x * blockDim.x) {
        T f[6];
#pragma unroll
        for (int m = 0; m < 6; m++) f[m] = (T)fff[m * fff_stride + e];
#pragma unroll
        for (int i = 0; i < 8; i++) {
            T a = 0;
#pragma unroll
            for (int m = 0; m < 6; m++) a += f[m] * lap_w<T>(i * 9, m);
            atomicAdd(&diag[elements[i][e]], a);
        }
    }
}

// ------------------------------------------------------------------ sshex8 apply

// v1: one warp per macro element.  Lanes compute the element matrix entries
// (A = sum_m (fff_m / L) W_m), gather the (L+1)^3 micro-grid values into shared
// memory, apply the 8x8 element matrix per micro element with shared-memory
// accumulation, then scatter: nodes strictly inside the macro element are owned
// (plain read-modify-write), surface nodes are shared (atomicAdd).
template <typename T, int L>
__global__ void __launch_bounds__(128) sshex8_laplacian_apply_warp_kernel(ptrdiff_t nelements,
                                                                          const idx_t *const *elements,
                                                                          ptrdiff_t fff_stride, const float *fff,
                                                                          const T *x, T *y, const T *Ag = nullptr) {
    constexpr int N1 = L + 1;
    constexpr int NXE = N1 * N1 * N1;
    constexpr int NM = L * L * L;
    constexpr int WPB = 4;
    constexpr int NR = (NXE + 31) / 32;
    __shared__ T xs[WPB][NXE];
    __shared__ T ys[WPB][NXE];
    __shared__ T As[WPB][64];
    __shared__ T Wt[64 * 6];  // element-matrix weights: lanes read different rows
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T *xw = xs[warp];
    T *yw = ys[warp];
    T *Aw = As[warp];
    const T h = T(1) / T(L);
    for (int k = threadIdx.x; k < 64 * 6; k += blockDim.x) Wt[k] = lap_w<T>(k / 6, k % 6);
    __syncthreads();

    for (ptrdiff_t e = (ptrdiff_t)blockIdx.x * WPB + warp; e < nelements; e += (ptrdiff_t)gridDim.x * WPB) {
        if (Ag) {
            // stored micro element matrix of this macro element (row-major 8 x 8)
            for (int k = lane; k < 64; k += 32) Aw[k] = Ag[64 * e + k];
        } else {
            T f = 0;
            if (lane < 6) f = (T)fff[lane * fff_stride + e] * h;
            T sub[6];
#pragma unroll
            for (int m = 0; m < 6; m++) sub[m] = __shfl_sync(0xffffffffu, f, m);
#pragma unroll
            for (int k = lane; k < 64; k += 32) {
                T a = 0;
#pragma unroll
                for (int m = 0; m < 6; m++) a += sub[m] * Wt[k * 6 + m];
                Aw[k] = a;
            }
        }

        idx_t gi[NR];
#pragma unroll
        for (int r = 0; r < NR; r++) {
            const int l = lane + 32 * r;
            if (l < NXE) {
                gi[r] = elements[l][e];
                xw[l] = x[gi[r]];
                yw[l] = 0;
            }
        }
        __syncwarp();

        for (int m = lane; m < NM; m += 32) {
            const int xi = m % L, yi = (m / L) % L, zi = m / (L * L);
            int v[8];
            T u[8];
#pragma unroll
            for (int c = 0; c < 8; c++) {
                v[c] = lidx(L, xi + c8x(c), yi + c8y(c), zi + c8z(c));
                u[c] = xw[v[c]];
            }
#pragma unroll
            for (int i = 0; i < 8; i++) {
                T acc = 0;
#pragma unroll
                for (int j = 0; j < 8; j++) acc += Aw[i * 8 + j] * u[j];
                atomicAdd(&yw[v[i]], acc);
            }
        }
        __syncwarp();

#pragma unroll
        for (int r = 0; r < NR; r++) {
            const int l = lane + 32 * r;
            if (l < NXE) {
                const int xi = l % N1, yi = (l / N1) % N1, zi = l / (N1 * N1);
                const bool interior = xi > 0 && xi < L && yi > 0 && yi < L && zi > 0 && zi < L;
                const T val = yw[l];
                if (interior)
                    y[gi[r]] += val;
                else
                    atomicAdd(&y[gi[r]], val);
            }
        }
        __syncwarp();
    }
}

// v2 (bandwidth path): one THREAD per macro element, everything in registers.
// Consecutive threads own consecutive macro elements, so every connectivity
// load elements[v][e] of a warp is one coalesced 128-byte line and the x
// gathers of a warp fall on a few lines (neighbouring macro elements are
// neighbours in the mesh).  The thread sweeps the micro-element layers in z
// with two node planes of x and y in registers; when a layer is done the lower
// y plane is final and is scattered (plain read-modify-write for nodes strictly
// inside the macro element, atomicAdd for its surface).  The element matrix is
// built once per thread from the 6 metric entries (compile-time weights).
template <typename T, int L>
__global__ void __launch_bounds__(128) sshex8_laplacian_apply_tpe_kernel(ptrdiff_t nelements,
                                                                         const idx_t *const *elements,
                                                                         ptrdiff_t fff_stride, const float *fff,
                                                                         const T *__restrict__ x, T *__restrict__ y) {
    constexpr int N1 = L + 1;
    constexpr int NP = N1 * N1;
    constexpr int NXE = NP * N1;
    // the row pointers in shared memory: one global load each per block instead of
    // one per thread and row ahead of every dependent index load
    __shared__ const idx_t *srow_tpe[NXE];
    for (int v = threadIdx.x; v < NXE; v += blockDim.x) srow_tpe[v] = elements[v];
    __syncthreads();
    const idx_t *const *rows = srow_tpe;
    const ptrdiff_t e = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x;
    if (e >= nelements) return;
    const T h = T(1) / T(L);
    T f[6];
#pragma unroll
    for (int m = 0; m < 6; m++) f[m] = (T)__ldg(&fff[m * fff_stride + e]) * h;
    T A[64];
#pragma unroll
    for (int k = 0; k < 64; k++) {
        T a = 0;
#pragma unroll
        for (int m = 0; m < 6; m++) {
            const double w = LapTable().w[k][m];
            if (w != 0.0) a += f[m] * T(w);
        }
        A[k] = a;
    }
    T xa[NP], xb[NP], ya[NP], yb[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) {
        xa[p] = __ldg(&x[__ldg(&rows[p][e])]);
        ya[p] = 0;
    }
#pragma unroll
    for (int zi = 0; zi < L; zi++) {
#pragma unroll
        for (int p = 0; p < NP; p++) {
            xb[p] = __ldg(&x[__ldg(&rows[(zi + 1) * NP + p][e])]);
            yb[p] = 0;
        }
#pragma unroll
        for (int yi = 0; yi < L; yi++) {
#pragma unroll
            for (int xi = 0; xi < L; xi++) {
                T u[8];
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    const int p = (yi + c8y(c)) * N1 + xi + c8x(c);
                    u[c] = c8z(c) ? xb[p] : xa[p];
                }
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    T acc = 0;
#pragma unroll
                    for (int j = 0; j < 8; j++) acc += A[i * 8 + j] * u[j];
                    const int p = (yi + c8y(i)) * N1 + xi + c8x(i);
                    if (c8z(i))
                        yb[p] += acc;
                    else
                        ya[p] += acc;
                }
            }
        }
        // plane zi is final
#pragma unroll
        for (int p = 0; p < NP; p++) {
            const int xi = p % N1, yi = p / N1;
            const idx_t g = __ldg(&rows[zi * NP + p][e]);
            if (zi > 0 && xi > 0 && xi < L && yi > 0 && yi < L)
                y[g] += ya[p];
            else
                atomicAdd(&y[g], ya[p]);
        }
#pragma unroll
        for (int p = 0; p < NP; p++) {
            xa[p] = xb[p];
            ya[p] = yb[p];
        }
    }
#pragma unroll
    for (int p = 0; p < NP; p++) atomicAdd(&y[__ldg(&rows[L * NP + p][e])], ya[p]);
}

// v3 (bandwidth path, staged): a CTA owns a tile of TILE consecutive macro
// elements, one thread per element.  Phase 1 gathers the tile's micro grids into
// shared memory plane by plane (one coalesced connectivity line per warp and
// plane node, then the x gathers, many loads in flight per thread); phase 2
// applies the element matrix from shared memory with the two active y planes in
// registers, writing each finished y plane over the x plane it no longer needs;
// phase 3 scatters (plain read-modify-write inside the macro element, atomics
// on its surface).  Shared layout [node][TILE] keeps every warp access
// conflict-free.
template <typename T, int L, int TILE>
__global__ void __launch_bounds__(TILE) sshex8_laplacian_apply_staged_kernel(ptrdiff_t nelements,
                                                                             const idx_t *const *elements,
                                                                             ptrdiff_t fff_stride, const float *fff,
                                                                             const T *__restrict__ x,
                                                                             T *__restrict__ y) {
    constexpr int N1 = L + 1;
    constexpr int NP = N1 * N1;
    constexpr int NXE = NP * N1;
    extern __shared__ unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);  // [NXE][TILE]
    const int t = threadIdx.x;
    const ptrdiff_t e = (ptrdiff_t)blockIdx.x * TILE + t;
    const bool active = e < nelements;
    // phase 1: gather
#pragma unroll 1
    for (int z = 0; z < N1; z++) {
        idx_t g[NP];
#pragma unroll
        for (int p = 0; p < NP; p++) g[p] = active ? __ldg(&elements[z * NP + p][e]) : 0;
#pragma unroll
        for (int p = 0; p < NP; p++) xs[(z * NP + p) * TILE + t] = active ? __ldg(&x[g[p]]) : T(0);
    }
    if (!active) return;  // no block-wide synchronisation below: each thread owns its column
    const T h = T(1) / T(L);
    T f[6];
#pragma unroll
    for (int m = 0; m < 6; m++) f[m] = (T)__ldg(&fff[m * fff_stride + e]) * h;
    T A[64];
#pragma unroll
    for (int k = 0; k < 64; k++) {
        T a = 0;
#pragma unroll
        for (int m = 0; m < 6; m++) {
            const double w = LapTable().w[k][m];
            if (w != 0.0) a += f[m] * T(w);
        }
        A[k] = a;
    }
    // phase 2: apply, planes of y in registers
    T ya[NP], yb[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) ya[p] = 0;
#pragma unroll
    for (int zi = 0; zi < L; zi++) {
#pragma unroll
        for (int p = 0; p < NP; p++) yb[p] = 0;
#pragma unroll
        for (int yi = 0; yi < L; yi++) {
#pragma unroll
            for (int xi = 0; xi < L; xi++) {
                T u[8];
#pragma unroll
                for (int c = 0; c < 8; c++)
                    u[c] = xs[((zi + c8z(c)) * NP + (yi + c8y(c)) * N1 + xi + c8x(c)) * TILE + t];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    T acc = 0;
#pragma unroll
                    for (int j = 0; j < 8; j++) acc += A[i * 8 + j] * u[j];
                    const int p = (yi + c8y(i)) * N1 + xi + c8x(i);
                    if (c8z(i))
                        yb[p] += acc;
                    else
                        ya[p] += acc;
                }
            }
        }
        // x plane zi is no longer needed: it receives the finished y plane zi
#pragma unroll
        for (int p = 0; p < NP; p++) {
            xs[(zi * NP + p) * TILE + t] = ya[p];
            ya[p] = yb[p];
        }
    }
#pragma unroll
    for (int p = 0; p < NP; p++) xs[(L * NP + p) * TILE + t] = ya[p];
    // phase 3: scatter
#pragma unroll 1
    for (int z = 0; z < N1; z++) {
        idx_t g[NP];
#pragma unroll
        for (int p = 0; p < NP; p++) g[p] = __ldg(&elements[z * NP + p][e]);
#pragma unroll
        for (int p = 0; p < NP; p++) {
            const int xi = p % N1, yi = p / N1;
            const T v = xs[(z * NP + p) * TILE + t];
            if (z > 0 && z < L && xi > 0 && xi < L && yi > 0 && yi < L)
                y[g[p]] += v;
            else
                atomicAdd(&y[g[p]], v);
        }
    }
}

// v4 (float bandwidth path, asynchronous staging): a CTA of 2*TILE threads owns
// TILE consecutive macro elements.
//  1. the tile's connectivity rows elements[v][e0 .. e0+TILE) are copied to shared
//     memory with cp.async (16-byte copies where the row is 16-byte aligned), one
//     coalesced line per row and no register round trip;
//  2. x[idx] is gathered into shared memory with 4-byte cp.async copies (the
//     dependent load chain costs no registers and every thread keeps dozens of
//     copies in flight);
//  3. two threads per element apply the element matrix, warp 0 the micro layers
//     0 .. L/2-1 bottom-up, warp 1 the layers L/2 .. L-1 top-down, two node planes
//     of y in registers, FP32x2 packed FMAs (A as 32 float2: rows 2k, 2k+1 of a
//     column); each finished y plane overwrites its x plane, the shared middle
//     plane is summed after a barrier;
//  4. the y values of the tile are scattered with atomics, one coalesced pass.
// Shared layout [node][TILE] keeps every access conflict-free.

// Inversion symmetry of the affine element matrix: the point reflection
// xi -> 1 - xi maps hex8 corner c to pi(c) = (0 6)(1 7)(2 4)(3 5) and leaves
// grad(phi_i) . G grad(phi_j) unchanged, so A[pi(i)][pi(j)] = A[i][j].  Rows 6, 7
// and 4, 5 are therefore rows 0, 1 and 2, 3 read at permuted columns: the packed
// FP32x2 form needs only A2[j][k] = (A[2k][j], A[2k+1][j]) for k = 0, 1.
__host__ __device__ constexpr int hex8_inv(int c) { return c == 0 ? 6 : c == 1 ? 7 : c == 2 ? 4 : c == 3 ? 5 : c == 4 ? 2 : c == 5 ? 3 : c == 6 ? 0 : 1; }

// one micro layer (base = x column of plane zi): lo (plane zi) and up (plane zi+1) accumulate A u
template <int L, int TILE>
__device__ __forceinline__ void lap_layer_f32x2(const float *__restrict__ xbase, const float2 (&A2)[8][2],
                                                float (&lo)[(L + 1) * (L + 1)], float (&up)[(L + 1) * (L + 1)]) {
    constexpr int N1 = L + 1;
    constexpr int NP = N1 * N1;
#pragma unroll
    for (int yi = 0; yi < L; yi++) {
#pragma unroll
        for (int xi = 0; xi < L; xi++) {
            float u[8];
#pragma unroll
            for (int c = 0; c < 8; c++) u[c] = xbase[(c8z(c) * NP + (yi + c8y(c)) * N1 + xi + c8x(c)) * TILE];
            float2 acc[4];
#pragma unroll
            for (int k = 0; k < 4; k++) acc[k] = make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const float2 uu = make_float2(u[j], u[j]);
                acc[0] = __ffma2_rn(A2[j][0], uu, acc[0]);                 // rows 0, 1
                acc[1] = __ffma2_rn(A2[j][1], uu, acc[1]);                 // rows 2, 3
                acc[2] = __ffma2_rn(A2[hex8_inv(j)][1], uu, acc[2]);       // rows 4, 5
                acc[3] = __ffma2_rn(A2[hex8_inv(j)][0], uu, acc[3]);       // rows 6, 7
            }
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const float v = (i & 1) ? acc[i >> 1].y : acc[i >> 1].x;
                const int p = (yi + c8y(i)) * N1 + xi + c8x(i);
                if (c8z(i))
                    up[p] += v;
                else
                    lo[p] += v;
            }
        }
    }
}

template <int L, int TILE, int NQ = 2>
__global__ void __launch_bounds__(NQ * TILE, NQ == 2 ? (TILE == 32 ? 6 : 3) : 4) sshex8_laplacian_apply_async_kernel(
        ptrdiff_t nelements, const idx_t *const *elements, ptrdiff_t fff_stride, const float *fff,
        const float *__restrict__ x, float *__restrict__ y) {
    static_assert(L % NQ == 0, "NQ threads per element split the micro layers evenly");
    constexpr int N1 = L + 1;
    constexpr int NP = N1 * N1;
    constexpr int NXE = NP * N1;
    constexpr int H = L / NQ;  // layers per thread; thread q's bottom plane q H is shared with thread q - 1
    __shared__ __align__(16) idx_t sidx[NXE * TILE];
    __shared__ __align__(16) float sx[NXE * TILE];
    __shared__ float spart[(NQ - 1) * NP * TILE];  // partial sums of the shared planes (from the upper thread)
    __shared__ const idx_t *srow[NXE];  // the row pointers: one global load each, then shared
    const int tid = threadIdx.x;
    const ptrdiff_t e0 = (ptrdiff_t)blockIdx.x * TILE;
    const int nvalid = (int)((nelements - e0) < TILE ? (nelements - e0) : TILE);
    for (int v = tid; v < NXE; v += NQ * TILE) srow[v] = elements[v];
    __syncthreads();
    // 1. connectivity rows
    for (int v = tid / (TILE / 4); v < NXE; v += (NQ * TILE) / (TILE / 4)) {
        const int q = tid % (TILE / 4);  // 16-byte quarter of the row segment
        const idx_t *row = srow[v] + e0;
        if (nvalid == TILE && ((reinterpret_cast<uintptr_t>(row) & 15) == 0)) {
            cp_async16(&sidx[v * TILE + 4 * q], row + 4 * q);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (4 * q + k < nvalid) cp_async4(&sidx[v * TILE + 4 * q + k], row + 4 * q + k);
        }
    }
    cp_async_wait_all();
    __syncthreads();
    // 2. gather x
    for (int t = tid; t < NXE * TILE; t += NQ * TILE) {
        const int el = t % TILE;
        if (el < nvalid) cp_async4(&sx[t], x + sidx[t]);
    }
    const int el = tid % TILE;
    const int half = tid / TILE;  // the thread's layer group q; warp-uniform for TILE = 32
    const bool valid = el < nvalid;
    // element matrix, rows 0..3 packed by pairs (overlaps the gathers in flight)
    float2 A2[8][2];
    {
        float f[6];
        const float h = 1.f / (float)L;
#pragma unroll
        for (int m = 0; m < 6; m++) f[m] = valid ? __ldg(&fff[m * fff_stride + e0 + el]) * h : 0.f;
#pragma unroll
        for (int j = 0; j < 8; j++) {
#pragma unroll
            for (int k = 0; k < 2; k++) {
                float a0 = 0.f, a1 = 0.f;
#pragma unroll
                for (int m = 0; m < 6; m++) {
                    const double w0 = LapTable().w[(2 * k) * 8 + j][m];
                    const double w1 = LapTable().w[(2 * k + 1) * 8 + j][m];
                    if (w0 != 0.0) a0 += f[m] * (float)w0;
                    if (w1 != 0.0) a1 += f[m] * (float)w1;
                }
                A2[j][k] = make_float2(a0, a1);
            }
        }
    }
    cp_async_wait_all();
    __syncthreads();
    // 3. apply: thread group q runs layers q*H .. q*H + H - 1 upwards (same code for every q)
    float *col = sx + el;
    const int z0 = half * H;
    float lo[NP], up[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) lo[p] = 0.f;
#pragma unroll 1
    for (int zi = z0; zi < z0 + H; zi++) {
#pragma unroll
        for (int p = 0; p < NP; p++) up[p] = 0.f;
        lap_layer_f32x2<L, TILE>(col + zi * NP * TILE, A2, lo, up);
        // plane zi is complete for this thread; its x is not read again by it.  A bottom
        // plane shared with the group below (zi == z0 > 0) is kept aside.
        float *dst = (zi == z0 && half > 0) ? (spart + (half - 1) * NP * TILE + el) : (col + zi * NP * TILE);
#pragma unroll
        for (int p = 0; p < NP; p++) {
            dst[p * TILE] = lo[p];
            lo[p] = up[p];
        }
    }
    // lo = plane z0 + H: the top group's last plane, the others' partial of a shared plane
    if (half == NQ - 1) {
#pragma unroll
        for (int p = 0; p < NP; p++) col[(L * NP + p) * TILE] = lo[p];
    }
    __syncthreads();  // every x read of the shared planes is done
    if (half < NQ - 1) {
        const float *sp = spart + half * NP * TILE + el;
#pragma unroll
        for (int p = 0; p < NP; p++) col[((z0 + H) * NP + p) * TILE] = lo[p] + sp[p * TILE];
    }
    __syncthreads();
    // 4. scatter
    for (int t = tid; t < NXE * TILE; t += NQ * TILE) {
        if (t % TILE < nvalid) atomicAdd(&y[sidx[t]], sx[t]);
    }
}

// v5 (float bandwidth path, persistent and pipelined): each CTA of L warps loops
// over tiles of TILE = 32 consecutive macro elements.  While tile t is applied,
// the x gathers of tile t+G (G = grid size) and the connectivity + metric rows of
// tile t+2G are in flight (cp.async into three index stages and two x stages),
// so HBM streams continuously instead of stopping at every tile's barriers.
// Warp q applies micro layer q of all 32 elements (lane = element); the two
// partial sums of each inner plane are combined in shared memory after the
// layer pass.  Same packed FP32x2 / inversion-symmetry arithmetic as v4.
template <int L, int TILE>
__device__ __forceinline__ void pipe_load_rows(const idx_t *const *srow, const float *fff, ptrdiff_t fff_stride,
                                               ptrdiff_t e0, int nvalid, idx_t *sidx, float *sfff) {
    constexpr int N1 = L + 1;
    constexpr int NXE = N1 * N1 * N1;
    constexpr int NT = 32 * L;
    constexpr int Q = TILE / 4;  // 16-byte chunks per row segment
    for (int t = threadIdx.x; t < NXE * Q; t += NT) {
        const int v = t / Q, q = t % Q;
        const idx_t *row = srow[v] + e0;
        if (nvalid == TILE && ((reinterpret_cast<uintptr_t>(row) & 15) == 0)) {
            cp_async16(&sidx[v * TILE + 4 * q], row + 4 * q);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (4 * q + k < nvalid) cp_async4(&sidx[v * TILE + 4 * q + k], row + 4 * q + k);
        }
    }
    for (int t = threadIdx.x; t < 6 * TILE; t += NT) {
        const int m = t / TILE, el = t % TILE;
        if (el < nvalid) cp_async4(&sfff[t], fff + m * fff_stride + e0 + el);
    }
}

template <int L, int TILE>
__device__ __forceinline__ void pipe_gather(const float *__restrict__ x, const idx_t *sidx, int nvalid, float *sx) {
    constexpr int N1 = L + 1;
    constexpr int NXE = N1 * N1 * N1;
    constexpr int NT = 32 * L;
    for (int t = threadIdx.x; t < NXE * TILE; t += NT)
        if (t % TILE < nvalid) cp_async4(&sx[t], x + sidx[t]);
}

template <int L, int TILE>
__global__ void __launch_bounds__(32 * L, 2) sshex8_laplacian_apply_pipe_kernel(ptrdiff_t nelements,
                                                                              const idx_t *const *elements,
                                                                              ptrdiff_t fff_stride,
                                                                              const float *fff,
                                                                              const float *__restrict__ x,
                                                                              float *__restrict__ y) {
    constexpr int N1 = L + 1;
    constexpr int NP = N1 * N1;
    constexpr int NXE = NP * N1;
    constexpr int NT = 32 * L;
    constexpr int SI = NXE * TILE;  // one stage of indices or values
    extern __shared__ __align__(16) unsigned char smem_pipe[];
    idx_t *sidx = reinterpret_cast<idx_t *>(smem_pipe);              // [3][SI]
    float *sx = reinterpret_cast<float *>(sidx + 3 * SI);            // [2][SI]
    float *sfff = sx + 2 * SI;                                       // [3][6 * TILE]
    __shared__ const idx_t *srow[NXE];                               // row pointers, loaded once
    for (int v = threadIdx.x; v < NXE; v += NT) srow[v] = elements[v];
    __syncthreads();
    const ptrdiff_t ntiles = (nelements + TILE - 1) / TILE;
    const ptrdiff_t G = gridDim.x;
    auto nvalid_of = [&](ptrdiff_t t) {
        const ptrdiff_t r = nelements - t * TILE;
        return (int)(r < TILE ? r : TILE);
    };
    const int q = threadIdx.x >> 5;  // micro layer of this warp
    const int el = threadIdx.x & 31;
    ptrdiff_t t = blockIdx.x;
    if (t >= ntiles) return;
    // prologue: rows of t and t+G, gather of t
    pipe_load_rows<L, TILE>(srow, fff, fff_stride, t * TILE, nvalid_of(t), sidx, sfff);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    if (t + G < ntiles)
        pipe_load_rows<L, TILE>(srow, fff, fff_stride, (t + G) * TILE, nvalid_of(t + G), sidx + SI,
                                sfff + 6 * TILE);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    __syncthreads();
    pipe_gather<L, TILE>(x, sidx, nvalid_of(t), sx);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    for (int k = 0; t < ntiles; k++, t += G) {
        const int si = k % 3, sxs = k & 1;
        const int nvalid = nvalid_of(t);
        cp_async_wait_all();  // x(t) and the rows of t+G
        __syncthreads();
        if (t + G < ntiles) pipe_gather<L, TILE>(x, sidx + ((k + 1) % 3) * SI, nvalid_of(t + G), sx + (sxs ^ 1) * SI);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        if (t + 2 * G < ntiles)
            pipe_load_rows<L, TILE>(srow, fff, fff_stride, (t + 2 * G) * TILE, nvalid_of(t + 2 * G),
                                    sidx + ((k + 2) % 3) * SI, sfff + ((k + 2) % 3) * 6 * TILE);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        // element matrix of this lane's element
        float2 A2[8][2];
        {
            const float *ff = sfff + si * 6 * TILE + el;
            const float h = 1.f / (float)L;
            float f[6];
#pragma unroll
            for (int m = 0; m < 6; m++) f[m] = el < nvalid ? ff[m * TILE] * h : 0.f;
#pragma unroll
            for (int j = 0; j < 8; j++) {
#pragma unroll
                for (int kk = 0; kk < 2; kk++) {
                    float a0 = 0.f, a1 = 0.f;
#pragma unroll
                    for (int m = 0; m < 6; m++) {
                        const double w0 = LapTable().w[(2 * kk) * 8 + j][m];
                        const double w1 = LapTable().w[(2 * kk + 1) * 8 + j][m];
                        if (w0 != 0.0) a0 += f[m] * (float)w0;
                        if (w1 != 0.0) a1 += f[m] * (float)w1;
                    }
                    A2[j][kk] = make_float2(a0, a1);
                }
            }
        }
        float *col = sx + sxs * SI + el;
        float lo[NP], up[NP];
#pragma unroll
        for (int p = 0; p < NP; p++) {
            lo[p] = 0.f;
            up[p] = 0.f;
        }
        lap_layer_f32x2<L, TILE>(col + q * NP * TILE, A2, lo, up);
        __syncthreads();  // every x read of this tile is done
#pragma unroll
        for (int p = 0; p < NP; p++) col[((q + 1) * NP + p) * TILE] = up[p];
        if (q == 0) {
#pragma unroll
            for (int p = 0; p < NP; p++) col[p * TILE] = lo[p];
        }
        __syncthreads();
        if (q > 0) {
#pragma unroll
            for (int p = 0; p < NP; p++) col[(q * NP + p) * TILE] += lo[p];
        }
        __syncthreads();
        const idx_t *ri = sidx + si * SI;
        const float *rv = sx + sxs * SI;
        for (int i = threadIdx.x; i < SI; i += NT)
            if (i % TILE < nvalid) atomicAdd(&y[ri[i]], rv[i]);
        __syncthreads();  // stage buffers of t are free
    }
    cp_async_wait_all();
}

// ------------------------------------------------------------------ packed tiles
// (layout in tiles.cuh)
__device__ int g_lap_status;  // nonzero: a bulk-copy wait gave up

__global__ void sshex8_pack_kernel(ptrdiff_t nelements, int nxe, const idx_t *const *elements, ptrdiff_t fff_stride,
                                   const float *fff, int32_t *packed) {
    const int words = PK_TILE * (nxe + 6);
    const ptrdiff_t total = (nelements + PK_TILE - 1) / PK_TILE * words;
    for (ptrdiff_t g = (ptrdiff_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
         g += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t t = g / words;
        const int w = (int)(g - t * words);
        const ptrdiff_t e = t * PK_TILE + w % PK_TILE;
        int32_t val = 0;
        if (e < nelements)
            val = w < PK_TILE * nxe ? elements[w / PK_TILE][e]
                                    : __float_as_int(fff[(w / PK_TILE - nxe) * fff_stride + e]);
        packed[g] = val;
    }
}

// Rows 0..3 of the micro element matrix (packed by pairs) from the macro metric f
// already scaled by 1/L.
__device__ __forceinline__ void lap_A2_from_metric(const float (&f)[6], float2 (&A2)[8][2]) {
#pragma unroll
    for (int j = 0; j < 8; j++) {
#pragma unroll
        for (int k = 0; k < 2; k++) {
            float a0 = 0.f, a1 = 0.f;
#pragma unroll
            for (int m = 0; m < 6; m++) {
                const double w0 = LapTable().w[(2 * k) * 8 + j][m];
                const double w1 = LapTable().w[(2 * k + 1) * 8 + j][m];
                if (w0 != 0.0) a0 += f[m] * (float)w0;
                if (w1 != 0.0) a1 += f[m] * (float)w1;
            }
            A2[j][k] = make_float2(a0, a1);
        }
    }
}

// FP32 apply of one packed tile per CTA: bulk copy of the block, x gathered with
// 4-byte cp.async (lanes = the tile's elements), two threads per element each running
// half of the micro layers (the async tile kernel's arithmetic), atomic scatter.
// Shared memory (dynamic, 35,968 B at L = 4: 6 CTAs per SM): the block, x [node][el],
// the partial sums of the middle plane [p][el].
template <int L>
__global__ void __launch_bounds__(2 * PK_TILE, 6) sshex8_laplacian_apply_packed_kernel(
        ptrdiff_t nelements, const int32_t *__restrict__ packed, const float *__restrict__ x,
        float *__restrict__ y, int first_polls) {
    constexpr int N1 = L + 1;
    constexpr int NP = N1 * N1;
    constexpr int NXE = NP * N1;
    constexpr int H = L / 2;
    constexpr int WORDS = pk_words(L);
    extern __shared__ __align__(128) int32_t pk_smem[];
    __shared__ __align__(8) uint64_t mbar;
    const int32_t *sidx = pk_smem;
    const float *smet = reinterpret_cast<const float *>(pk_smem + PK_TILE * NXE);
    float *sx = reinterpret_cast<float *>(pk_smem + WORDS);
    float *spart = sx + NXE * PK_TILE;
    const int tid = threadIdx.x;
    const ptrdiff_t t = blockIdx.x;
    if (tid == 0) {
        tc::mbar_init(&mbar, 1);
        tc::mbar_arrive_expect_tx(&mbar, WORDS * 4);
        tc::bulk_load(pk_smem, packed + t * WORDS, WORDS * 4, &mbar);
    }
    __syncthreads();
    if (!__syncthreads_and(tc::mbar_wait(&mbar, 0, first_polls))) {
        // leave no copy in flight into this CTA's shared memory: thread 0 drains the
        // copy (with a far longer bound) before its CTA exits
        if (tid == 0) {
            atomicExch(&g_lap_status, 1);
            if (!tc::mbar_wait(&mbar, 0, LAP_DRAIN_POLLS)) atomicExch(&g_lap_status, 2);
        }
        return;
    }
    const int nvalid = (int)((nelements - t * PK_TILE) < PK_TILE ? (nelements - t * PK_TILE) : PK_TILE);
    // 1. gather x (full tiles without the per-node validity test)
    if (nvalid == PK_TILE) {
#pragma unroll 8
        for (int i = tid; i < NXE * PK_TILE; i += 2 * PK_TILE) cp_async4(&sx[i], x + sidx[i]);
    } else {
        for (int i = tid; i < NXE * PK_TILE; i += 2 * PK_TILE)
            if (i % PK_TILE < nvalid) cp_async4(&sx[i], x + sidx[i]);
    }
    const int el = tid % PK_TILE;
    const int half = tid / PK_TILE;  // warp-uniform layer group
    float2 A2[8][2];
    {
        float f[6];
        const float h = 1.f / (float)L;
#pragma unroll
        for (int m = 0; m < 6; m++) f[m] = el < nvalid ? smet[m * PK_TILE + el] * h : 0.f;
        lap_A2_from_metric(f, A2);
    }
    cp_async_wait_all();
    __syncthreads();
    // 2. apply: thread group `half` runs layers half*H .. half*H + H - 1 upwards
    float *col = sx + el;
    const int z0 = half * H;
    float lo[NP], up[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) lo[p] = 0.f;
#pragma unroll 1
    for (int zi = z0; zi < z0 + H; zi++) {
#pragma unroll
        for (int p = 0; p < NP; p++) up[p] = 0.f;
        lap_layer_f32x2<L, PK_TILE>(col + zi * NP * PK_TILE, A2, lo, up);
        // plane zi is complete for this thread; the middle plane's lower part (from the
        // upper group) is kept aside until every x read of it is done
        float *dst = (zi == z0 && half > 0) ? spart + el : col + zi * NP * PK_TILE;
#pragma unroll
        for (int p = 0; p < NP; p++) {
            dst[p * PK_TILE] = lo[p];
            lo[p] = up[p];
        }
    }
    if (half == 1) {
#pragma unroll
        for (int p = 0; p < NP; p++) col[(L * NP + p) * PK_TILE] = lo[p];
    }
    __syncthreads();
    if (half == 0) {
#pragma unroll
        for (int p = 0; p < NP; p++) col[(H * NP + p) * PK_TILE] = lo[p] + spart[p * PK_TILE + el];
    }
    __syncthreads();
    // 3. scatter
    if (nvalid == PK_TILE) {
#pragma unroll 8
        for (int i = tid; i < NXE * PK_TILE; i += 2 * PK_TILE) atomicAdd(&y[sidx[i]], sx[i]);
    } else {
        for (int i = tid; i < NXE * PK_TILE; i += 2 * PK_TILE)
            if (i % PK_TILE < nvalid) atomicAdd(&y[sidx[i]], sx[i]);
    }
}

// Diagonal: node value = sum over the micro elements of this macro element that
// contain it of A[a][a] (a = the node's corner in that micro element).
template <typename T, int L>
__global__ void __launch_bounds__(128) sshex8_laplacian_diag_kernel(ptrdiff_t nelements, const idx_t *const *elements,
                                                                    ptrdiff_t fff_stride, const float *fff, T *diag) {
    constexpr int N1 = L + 1;
    constexpr int NXE = N1 * N1 * N1;
    constexpr int WPB = 4;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const T h = T(1) / T(L);
    for (ptrdiff_t e = (ptrdiff_t)blockIdx.x * WPB + warp; e < nelements; e += (ptrdiff_t)gridDim.x * WPB) {
        T sub[6];
#pragma unroll
        for (int m = 0; m < 6; m++) sub[m] = (T)fff[m * fff_stride + e] * h;
        T Ad[8];
#pragma unroll
        for (int a = 0; a < 8; a++) {
            T s = 0;
#pragma unroll
            for (int m = 0; m < 6; m++) s += sub[m] * lap_w<T>(a * 9, m);
            Ad[a] = s;
        }
        for (int l = lane; l < NXE; l += 32) {
            const int xi = l % N1, yi = (l / N1) % N1, zi = l / (N1 * N1);
            T s = 0;
#pragma unroll
            for (int a = 0; a < 8; a++) {
                const bool ok = (c8x(a) ? xi > 0 : xi < L) && (c8y(a) ? yi > 0 : yi < L) && (c8z(a) ? zi > 0 : zi < L);
                if (ok) s += Ad[a];
            }
            const bool interior = xi > 0 && xi < L && yi > 0 && yi < L && zi > 0 && zi < L;
            const idx_t g = elements[l][e];
            if (interior)
                diag[g] += s;
            else
                atomicAdd(&diag[g], s);
        }
    }
}

// Any level 2 <= L <= LAP_MAX_L without a compile-time kernel (5, 7, 9..16): one CTA
// per macro element, the (L+1)^3 values of x and y in dynamic shared memory
// (2 (L+1)^3 T: 78.6 KB for FP64 at L = 16), micro elements spread over the
// threads with shared-memory atomics, node ids read again for the scatter
// (interior nodes plain read-modify-write, surface nodes atomics).
constexpr int LAP_MAX_L = 16;
template <typename T>
__global__ void __launch_bounds__(256) sshex8_laplacian_apply_cta_kernel(int L, ptrdiff_t nelements,
                                                                         const idx_t *const *elements,
                                                                         ptrdiff_t fff_stride, const float *fff,
                                                                         const T *x, T *y, const T *Ag = nullptr) {
    extern __shared__ __align__(16) unsigned char lap_cta_smem[];
    const int N1 = L + 1, NXE = N1 * N1 * N1, NM = L * L * L;
    T *xs = reinterpret_cast<T *>(lap_cta_smem);
    T *ys = xs + NXE;
    T *As = ys + NXE;
    const T h = T(1) / T(L);
    for (ptrdiff_t e = blockIdx.x; e < nelements; e += gridDim.x) {
        if (threadIdx.x < 64) {
            T a = 0;
            if (Ag)
                a = Ag[64 * e + threadIdx.x];
            else
                for (int m = 0; m < 6; m++) a += (T)fff[m * fff_stride + e] * h * lap_w<T>(threadIdx.x, m);
            As[threadIdx.x] = a;
        }
        for (int l = threadIdx.x; l < NXE; l += blockDim.x) {
            xs[l] = x[elements[l][e]];
            ys[l] = 0;
        }
        __syncthreads();
        for (int m = threadIdx.x; m < NM; m += blockDim.x) {
            const int xi = m % L, yi = (m / L) % L, zi = m / (L * L);
            int v[8];
            T u[8];
#pragma unroll
            for (int c = 0; c < 8; c++) {
                v[c] = lidx(L, xi + c8x(c), yi + c8y(c), zi + c8z(c));
                u[c] = xs[v[c]];
            }
#pragma unroll
            for (int i = 0; i < 8; i++) {
                T acc = 0;
#pragma unroll
                for (int j = 0; j < 8; j++) acc += As[i * 8 + j] * u[j];
                atomicAdd(&ys[v[i]], acc);
            }
        }
        __syncthreads();
        for (int l = threadIdx.x; l < NXE; l += blockDim.x) {
            const int xi = l % N1, yi = (l / N1) % N1, zi = l / (N1 * N1);
            const bool interior = xi > 0 && xi < L && yi > 0 && yi < L && zi > 0 && zi < L;
            const idx_t g = elements[l][e];
            if (interior)
                y[g] += ys[l];
            else
                atomicAdd(&y[g], ys[l]);
        }
        __syncthreads();
    }
}

// Diagonal at any level (runtime L), warp per macro element as the compile-time kernel.
template <typename T>
__global__ void __launch_bounds__(128) sshex8_laplacian_diag_any_kernel(int L, ptrdiff_t nelements,
                                                                        const idx_t *const *elements,
                                                                        ptrdiff_t fff_stride, const float *fff, T *diag) {
    const int N1 = L + 1, NXE = N1 * N1 * N1;
    constexpr int WPB = 4;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const T h = T(1) / T(L);
    for (ptrdiff_t e = (ptrdiff_t)blockIdx.x * WPB + warp; e < nelements; e += (ptrdiff_t)gridDim.x * WPB) {
        T Ad[8];
#pragma unroll
        for (int a = 0; a < 8; a++) {
            T s = 0;
#pragma unroll
            for (int m = 0; m < 6; m++) s += (T)fff[m * fff_stride + e] * h * lap_w<T>(a * 9, m);
            Ad[a] = s;
        }
        for (int l = lane; l < NXE; l += 32) {
            const int xi = l % N1, yi = (l / N1) % N1, zi = l / (N1 * N1);
            T s = 0;
#pragma unroll
            for (int a = 0; a < 8; a++) {
                const bool ok = (c8x(a) ? xi > 0 : xi < L) && (c8y(a) ? yi > 0 : yi < L) && (c8z(a) ? zi > 0 : zi < L);
                if (ok) s += Ad[a];
            }
            const bool interior = xi > 0 && xi < L && yi > 0 && yi < L && zi > 0 && zi < L;
            const idx_t g = elements[l][e];
            if (interior)
                diag[g] += s;
            else
                atomicAdd(&diag[g], s);
        }
    }
}

template <typename T>
static int launch_lap_cta(int L, ptrdiff_t nelements, idx_t **elements, ptrdiff_t fff_stride, const float *fff,
                          const T *x, T *y, cudaStream_t s, const T *Ag = nullptr) {
    const size_t smem = (2 * (size_t)(L + 1) * (L + 1) * (L + 1) + 64) * sizeof(T);
    static std::atomic<size_t> attr{0};  // largest shared-memory opt-in so far (per T)
    if (smem > 48 * 1024 && smem > attr.load(std::memory_order_relaxed)) {
        cudaFuncSetAttribute(sshex8_laplacian_apply_cta_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        attr.store(smem, std::memory_order_relaxed);  // a racing caller at worst repeats the opt-in
    }
    const int grid = (int)std::min<ptrdiff_t>(nelements, (ptrdiff_t)kNumSMs * 8);
    sshex8_laplacian_apply_cta_kernel<T><<<grid, 256, smem, s>>>(L, nelements, elements, fff_stride, fff, x, y, Ag);
    return check_launch("cu_laplacian_apply(SSHEX8, CTA per element)");
}

// ------------------------------------------------------------------ dispatch

// Kernel variant override for benchmarking and the batched autotuner
// (SFEM_GB300_LAPLACIAN_KERNEL or sfem_gb300_set_laplacian_kernel); without one the
// applies pick per level: the node-centric stencil kernel (8) at L = 3, 4 and, in
// FP64, at L = 2; the thread-per-element kernel (2) for float at L = 2.
// "staged" (0) = shared-memory staged tile kernel for float, L <= 4;
// "warp" (1) = warp per element; "thread" (2) = registers-only thread per element;
// "async" (3) = cp.async staged tile, two threads per element, packed FP32x2 FMAs (even L);
// "pipe" (4) = persistent CTAs, cp.async pipeline across tiles, one warp per micro layer (even L);
// 6 = the async tile with four threads per element (one micro layer each, L = 4);
// 7 = the async tile of 64 elements (128 threads per CTA, L = 4);
// "stencil" (8) = node-centric stencil tiles of 32 elements (stencil.cu), L = 2..4.
static int g_laplacian_variant = -1;
static int g_laplacian_variant_forced = 0;  // set by sfem_gb300_set_laplacian_kernel
static int laplacian_variant() {
    int v = __atomic_load_n(&g_laplacian_variant, __ATOMIC_RELAXED);
    if (v < 0) {
        const char *e = getenv("SFEM_GB300_LAPLACIAN_KERNEL");
        v = (e && e[0] == 'w')   ? 1
            : (e && e[0] == 't') ? 2
            : (e && e[0] == 'a') ? 3
            : (e && e[0] == 'p') ? 4
            : (e && e[0] == 's') ? 8
                                 : 0;
        if (e && e[0]) __atomic_store_n(&g_laplacian_variant_forced, 1, __ATOMIC_RELAXED);
        __atomic_store_n(&g_laplacian_variant, v, __ATOMIC_RELAXED);
    }
    return v;
}

template <typename T>
static int laplacian_apply_tpl(int element_type, ptrdiff_t nelements, idx_t **elements, ptrdiff_t fff_stride,
                               const float *fff, const T *x, T *y, cudaStream_t s) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    if (element_type == SFEM_GB300_HEX8) {
        hex8_laplacian_apply_kernel<T><<<grid_for(nelements, 128), 128, 0, s>>>(nelements, elements, fff_stride, fff, x, y);
        return check_launch("cu_laplacian_apply(HEX8)");
    }
    const int L = element_type - SFEM_GB300_SSHEX8_BASE;
    const int blocks = grid_for((nelements + 3) / 4, 1, kNumSMs * 64);
    // default per level (measured at 7.2M nodes): L=4 async tile, L=2 thread per element, else staged tile
    int variant = laplacian_variant();
    const bool forced = __atomic_load_n(&g_laplacian_variant_forced, __ATOMIC_RELAXED) != 0;
    if (!forced) variant = (L == 3 || L == 4 || (L == 2 && sizeof(T) == 8)) ? 8 : (L == 2) ? 2 : 0;
    // node-centric stencil form (variant 8): the default where it is faster (7.2M nodes,
    // L2 flushed).  L = 4: FP64 0.53 ms against 0.99 ms for the warp element-matrix
    // kernel (about half the FP64 operations), FP32 45 us against 58 us for the async
    // tile.  L = 3: FP64 0.63 against 0.96 ms, FP32 51 against 80 us for the staged tile.
    // L = 2: FP64 0.97 against 1.04 ms; FP32 keeps the thread-per-element kernel.
    if (variant == 8 && sshex8_laplacian_stencil_supported(L))
        return sshex8_laplacian_stencil_apply<T>(L, nelements, nullptr, elements, fff_stride, fff, x, y, s);
    // FP64 at L = 2, 3: few micro elements per macro element leave most lanes of the warp
    // kernel idle; the staged tile (one thread per element) keeps them busy
    if (sizeof(T) == 8 && (L == 2 || L == 3) && variant != 1) variant = 5;
    if ((sizeof(T) == 4 && L >= 2 && L <= 4 && variant == 0) || variant == 5) {
        constexpr int TILE = 64;
        const int tb = (int)((nelements + TILE - 1) / TILE);
        auto launch = [&](auto kernel, int nxe) {
            const size_t smem = (size_t)nxe * TILE * sizeof(T);
            if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            kernel<<<tb, TILE, smem, s>>>(nelements, elements, fff_stride, fff, x, y);
        };
        switch (L) {
            case 2:
                launch(sshex8_laplacian_apply_staged_kernel<T, 2, TILE>, 27);
                break;
            case 3:
                launch(sshex8_laplacian_apply_staged_kernel<T, 3, TILE>, 64);
                break;
            default:
                launch(sshex8_laplacian_apply_staged_kernel<T, 4, TILE>, 125);
                break;
        }
        return check_launch("cu_laplacian_apply(SSHEX8, staged tile)");
    }
    if (sizeof(T) == 4 && (L == 2 || L == 4) && variant == 4) {
        constexpr int TILE = 32;
        const ptrdiff_t ntiles = (nelements + TILE - 1) / TILE;
        auto launch = [&](auto kernel, int LL) {
            const int nxe = (LL + 1) * (LL + 1) * (LL + 1);
            const size_t smem = (size_t)5 * nxe * TILE * sizeof(float) + 3 * 6 * TILE * sizeof(float);
            static int per_sm_cache[8] = {0};  // CTAs per SM, set on first use of each level
            int per_sm = per_sm_cache[LL];
            if (per_sm == 0) {
                cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * LL, smem);
                if (per_sm < 1) per_sm = 1;
                per_sm_cache[LL] = per_sm;
            }
            const ptrdiff_t grid = std::min<ptrdiff_t>(ntiles, (ptrdiff_t)kNumSMs * per_sm);
            kernel<<<(int)grid, 32 * LL, smem, s>>>(nelements, elements, fff_stride, fff, (const float *)x, (float *)y);
        };
        if (L == 2)
            launch(sshex8_laplacian_apply_pipe_kernel<2, TILE>, 2);
        else
            launch(sshex8_laplacian_apply_pipe_kernel<4, TILE>, 4);
        return check_launch("cu_laplacian_apply(SSHEX8, pipelined tile)");
    }
    if (sizeof(T) == 4 && L == 4 && variant == 7) {
        constexpr int TILE = 64;
        const int tb = (int)((nelements + TILE - 1) / TILE);
        sshex8_laplacian_apply_async_kernel<4, TILE, 2><<<tb, 2 * TILE, 0, s>>>(nelements, elements, fff_stride, fff,
                                                                                (const float *)x, (float *)y);
        return check_launch("cu_laplacian_apply(SSHEX8, async tile of 64 elements)");
    }
    if (sizeof(T) == 4 && L == 4 && variant == 6) {
        constexpr int TILE = 32;
        const int tb = (int)((nelements + TILE - 1) / TILE);
        sshex8_laplacian_apply_async_kernel<4, TILE, 4><<<tb, 4 * TILE, 0, s>>>(nelements, elements, fff_stride, fff,
                                                                                (const float *)x, (float *)y);
        return check_launch("cu_laplacian_apply(SSHEX8, async tile, four threads per element)");
    }
    if (sizeof(T) == 4 && (L == 2 || L == 4) && variant == 3) {
        constexpr int TILE = 32;
        const int tb = (int)((nelements + TILE - 1) / TILE);
        if (L == 2)
            sshex8_laplacian_apply_async_kernel<2, TILE><<<tb, 2 * TILE, 0, s>>>(
                    nelements, elements, fff_stride, fff, (const float *)x, (float *)y);
        else
            sshex8_laplacian_apply_async_kernel<4, TILE><<<tb, 2 * TILE, 0, s>>>(
                    nelements, elements, fff_stride, fff, (const float *)x, (float *)y);
        return check_launch("cu_laplacian_apply(SSHEX8, async tile)");
    }
    const bool tpe = sizeof(T) == 4 && L >= 2 && L <= 4 && variant == 2;
    if (tpe) {
        const int tb = (int)((nelements + 127) / 128);
        switch (L) {
            case 2:
                sshex8_laplacian_apply_tpe_kernel<T, 2><<<tb, 128, 0, s>>>(nelements, elements, fff_stride, fff, x, y);
                break;
            case 3:
                sshex8_laplacian_apply_tpe_kernel<T, 3><<<tb, 128, 0, s>>>(nelements, elements, fff_stride, fff, x, y);
                break;
            default:
                sshex8_laplacian_apply_tpe_kernel<T, 4><<<tb, 128, 0, s>>>(nelements, elements, fff_stride, fff, x, y);
                break;
        }
        return check_launch("cu_laplacian_apply(SSHEX8, thread per element)");
    }
#define SFEM_LAP_CASE(LL)                                                                                     \
    case LL:                                                                                                  \
        sshex8_laplacian_apply_warp_kernel<T, LL><<<blocks, 128, 0, s>>>(nelements, elements, fff_stride, fff, x, y); \
        return check_launch("cu_laplacian_apply(SSHEX8)");
    switch (L) {
        SFEM_LAP_CASE(1)
        SFEM_LAP_CASE(2)
        SFEM_LAP_CASE(3)
        SFEM_LAP_CASE(4)
        SFEM_LAP_CASE(6)
        SFEM_LAP_CASE(8)
        default:
            if (L >= 2 && L <= LAP_MAX_L) return launch_lap_cta<T>(L, nelements, elements, fff_stride, fff, x, y, s);
            return set_error("cu_laplacian_apply: unsupported element type %d", element_type);
    }
#undef SFEM_LAP_CASE
}

template <typename T>
static int laplacian_diag_tpl(int element_type, ptrdiff_t nelements, idx_t **elements, ptrdiff_t fff_stride,
                              const float *fff, T *diag, cudaStream_t s) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    if (element_type == SFEM_GB300_HEX8) {
        hex8_laplacian_diag_kernel<T><<<grid_for(nelements, 128), 128, 0, s>>>(nelements, elements, fff_stride, fff, diag);
        return check_launch("cu_laplacian_diag(HEX8)");
    }
    const int L = element_type - SFEM_GB300_SSHEX8_BASE;
    const int blocks = grid_for((nelements + 3) / 4, 1, kNumSMs * 64);
#define SFEM_LAP_CASE(LL)                                                                                   \
    case LL:                                                                                                \
        sshex8_laplacian_diag_kernel<T, LL><<<blocks, 128, 0, s>>>(nelements, elements, fff_stride, fff, diag); \
        return check_launch("cu_laplacian_diag(SSHEX8)");
    switch (L) {
        SFEM_LAP_CASE(1)
        SFEM_LAP_CASE(2)
        SFEM_LAP_CASE(3)
        SFEM_LAP_CASE(4)
        SFEM_LAP_CASE(6)
        SFEM_LAP_CASE(8)
        default:
            if (L >= 2 && L <= LAP_MAX_L) {
                sshex8_laplacian_diag_any_kernel<T><<<blocks, 128, 0, s>>>(L, nelements, elements, fff_stride, fff,
                                                                           diag);
                return check_launch("cu_laplacian_diag(SSHEX8, any level)");
            }
            return set_error("cu_laplacian_diag: unsupported element type %d", element_type);
    }
#undef SFEM_LAP_CASE
}

}  // namespace sfem_gb300

using namespace sfem_gb300;

extern "C" int sfem_gb300_hex8_fff_fill(ptrdiff_t nelements, idx_t **corners, float **points, ptrdiff_t fff_stride,
                                        float *fff, void *stream) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    hex8_geometry_kernel<<<grid_for(nelements, 128), 128, 0, stream_of(stream)>>>(nelements, corners, points,
                                                                                  fff_stride, fff, nullptr, nullptr);
    return check_launch("sfem_gb300_hex8_fff_fill");
}

extern "C" int sfem_gb300_hex8_adjugate_fill(ptrdiff_t nelements, idx_t **corners, float **points,
                                             ptrdiff_t jacobian_stride, float *adjugate, float *determinant,
                                             void *stream) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    hex8_geometry_kernel<<<grid_for(nelements, 128), 128, 0, stream_of(stream)>>>(
            nelements, corners, points, jacobian_stride, nullptr, adjugate, determinant);
    return check_launch("sfem_gb300_hex8_adjugate_fill");
}

extern "C" int cu_laplacian_apply(int element_type, ptrdiff_t nelements, idx_t **elements, ptrdiff_t fff_stride,
                                  const void *fff, int real_type_xy, const void *x, void *y, void *stream) {
    const cudaStream_t s = stream_of(stream);
    switch (real_type_xy) {
        case SFEM_GB300_REAL_DEFAULT:
        case SFEM_GB300_FLOAT64:
            return laplacian_apply_tpl<double>(element_type, nelements, elements, fff_stride, (const float *)fff,
                                               (const double *)x, (double *)y, s);
        case SFEM_GB300_FLOAT32:
            return laplacian_apply_tpl<float>(element_type, nelements, elements, fff_stride, (const float *)fff,
                                              (const float *)x, (float *)y, s);
        default:
            return set_error("cu_laplacian_apply: unsupported real type %d", real_type_xy);
    }
}

extern "C" int cu_laplacian_diag(int element_type, ptrdiff_t nelements, idx_t **elements, ptrdiff_t fff_stride,
                                 const void *fff, int real_type_diag, void *diag, void *stream) {
    const cudaStream_t s = stream_of(stream);
    switch (real_type_diag) {
        case SFEM_GB300_REAL_DEFAULT:
        case SFEM_GB300_FLOAT64:
            return laplacian_diag_tpl<double>(element_type, nelements, elements, fff_stride, (const float *)fff,
                                              (double *)diag, s);
        case SFEM_GB300_FLOAT32:
            return laplacian_diag_tpl<float>(element_type, nelements, elements, fff_stride, (const float *)fff,
                                             (float *)diag, s);
        default:
            return set_error("cu_laplacian_diag: unsupported real type %d", real_type_diag);
    }
}

extern "C" int sfem_gb300_set_laplacian_kernel(int variant) {
    if (variant < -1 || variant > 8 || variant == 5)
        return set_error("sfem_gb300_set_laplacian_kernel: variant must be -1..4, 6, 7 or 8");
    const int cur = laplacian_variant();
    const int prev = __atomic_load_n(&g_laplacian_variant_forced, __ATOMIC_RELAXED) ? cur : -1;
    __atomic_store_n(&g_laplacian_variant, variant < 0 ? 0 : variant, __ATOMIC_RELAXED);
    __atomic_store_n(&g_laplacian_variant_forced, variant < 0 ? 0 : 1, __ATOMIC_RELAXED);
    return prev;
}

// ------------------------------------------------------------------ packed tiles (C ABI)

// levels served from packed tiles: 4 (stencil or element-matrix kernel) and 3 (stencil)
static int packed_level(int element_type) {
    return element_type == SFEM_GB300_SSHEX8(PK_L) ? PK_L : element_type == SFEM_GB300_SSHEX8(3) ? 3 : -1;
}

extern "C" ptrdiff_t sfem_gb300_sshex8_packed_bytes(int element_type, ptrdiff_t nelements) {
    const int L = packed_level(element_type);
    if (L < 0 || nelements < 0) return -1;
    return (nelements + PK_TILE - 1) / PK_TILE * (ptrdiff_t)pk_words(L) * (ptrdiff_t)sizeof(int32_t);
}

extern "C" int sfem_gb300_sshex8_pack(int element_type, ptrdiff_t nelements, idx_t **elements, ptrdiff_t fff_stride,
                                      const float *fff, void *packed, void *stream) {
    const int L = packed_level(element_type);
    if (L < 0) return set_error("sfem_gb300_sshex8_pack: element type %d is not sshex8 L = 3 or 4", element_type);
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    if (reinterpret_cast<uintptr_t>(packed) & 15) return set_error("sfem_gb300_sshex8_pack: packed is not 16-byte aligned");
    const int nxe = (L + 1) * (L + 1) * (L + 1);
    const ptrdiff_t total = (nelements + PK_TILE - 1) / PK_TILE * (ptrdiff_t)pk_words(L);
    sshex8_pack_kernel<<<grid_for(total, 256), 256, 0, stream_of(stream)>>>(nelements, nxe, elements, fff_stride, fff,
                                                                           (int32_t *)packed);
    return check_launch("sfem_gb300_sshex8_pack");
}

extern "C" int sfem_gb300_sshex8_laplacian_apply_packed(int element_type, ptrdiff_t nelements, const void *packed,
                                                        int real_type_xy, const void *x, void *y, void *stream) {
    const int L = packed_level(element_type);
    if (L < 0)
        return set_error("sfem_gb300_sshex8_laplacian_apply_packed: element type %d is not sshex8 L = 3 or 4",
                         element_type);
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    if (reinterpret_cast<uintptr_t>(packed) & 15)
        return set_error("sfem_gb300_sshex8_laplacian_apply_packed: packed is not 16-byte aligned");
    // FP64 always, FP32 with variant 8 or at L = 3: the node-centric stencil kernel on the blocks
    if (real_type_xy == SFEM_GB300_FLOAT64 || real_type_xy == SFEM_GB300_REAL_DEFAULT)
        return sshex8_laplacian_stencil_apply<double>(L, nelements, (const int32_t *)packed, nullptr, 0, nullptr,
                                                      (const double *)x, (double *)y, stream_of(stream));
    if (real_type_xy != SFEM_GB300_FLOAT32)
        return set_error("sfem_gb300_sshex8_laplacian_apply_packed: unsupported real type %d", real_type_xy);
    // the stencil kernel unless another kernel was forced at L = 4 (packed element-matrix
    // kernel: 50.8 us against 45.0 us on the 48^3 L = 4 mesh)
    if (L != PK_L || laplacian_variant() == 8 || !__atomic_load_n(&g_laplacian_variant_forced, __ATOMIC_RELAXED))
        return sshex8_laplacian_stencil_apply<float>(L, nelements, (const int32_t *)packed, nullptr, 0, nullptr,
                                                     (const float *)x, (float *)y, stream_of(stream));
    const ptrdiff_t ntiles = (nelements + PK_TILE - 1) / PK_TILE;
    if (ntiles > 0x7fffffff) return set_error("sfem_gb300_sshex8_laplacian_apply_packed: too many tiles");
    constexpr int NXE = (PK_L + 1) * (PK_L + 1) * (PK_L + 1);
    constexpr size_t smem = ((size_t)pk_words(PK_L) + (size_t)NXE * PK_TILE + (size_t)(PK_L + 1) * (PK_L + 1) * PK_TILE) *
                            sizeof(float);
    static std::once_flag attr;  // shared-memory opt-in, once
    std::call_once(attr, [] {
        cudaFuncSetAttribute(sshex8_laplacian_apply_packed_kernel<PK_L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    });
    sshex8_laplacian_apply_packed_kernel<PK_L><<<(unsigned)ntiles, 2 * PK_TILE, smem, stream_of(stream)>>>(
            nelements, (const int32_t *)packed, (const float *)x, (float *)y, first_wait_polls());
    return check_launch("sfem_gb300_sshex8_laplacian_apply_packed");
}

extern "C" int sfem_gb300_laplacian_status(void) {
    int st = 0;
    if (cudaMemcpyFromSymbol(&st, g_lap_status, sizeof(int)) != cudaSuccess) return -1;
    if (st) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_lap_status, &zero, sizeof(int));
    }
    const int st2 = sshex8_laplacian_stencil_status();
    if (st2 < 0) return -1;
    return st > st2 ? st : st2;
}

// ------------------------------------------------------------------ stored element matrices

// em[e][i][j] = A_ij of the micro elements of macro element e (metric / L), row-major 8 x 8
// in hex8 corner order (the layout of sshex8_laplacian_element_matrix's `values`).
template <typename T>
__global__ void sshex8_laplacian_element_matrix_kernel(ptrdiff_t nelements, int L, ptrdiff_t fff_stride,
                                                       const float *fff, T *em) {
    const T h = T(1) / T(L);
    for (ptrdiff_t t = (ptrdiff_t)blockIdx.x * blockDim.x + threadIdx.x; t < nelements * 64;
         t += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t e = t / 64;
        const int k = (int)(t % 64);
        T a = 0;
        for (int m = 0; m < 6; m++) a += (T)fff[m * fff_stride + e] * h * lap_w<T>(k, m);
        em[t] = a;
    }
}

template <typename T>
static int laplacian_apply_em_tpl(int L, ptrdiff_t nelements, idx_t **elements, const T *em, const T *x, T *y,
                                  cudaStream_t s) {
    const int blocks = grid_for((nelements + 3) / 4, 1, kNumSMs * 64);
#define SFEM_LAP_EM_CASE(LL)                                                                                   \
    case LL:                                                                                                   \
        sshex8_laplacian_apply_warp_kernel<T, LL><<<blocks, 128, 0, s>>>(nelements, elements, 0, nullptr, x, y, em); \
        return check_launch("sfem_gb300_sshex8_laplacian_apply_em");
    switch (L) {
        SFEM_LAP_EM_CASE(1)
        SFEM_LAP_EM_CASE(2)
        SFEM_LAP_EM_CASE(3)
        SFEM_LAP_EM_CASE(4)
        SFEM_LAP_EM_CASE(6)
        SFEM_LAP_EM_CASE(8)
        default:
            return launch_lap_cta<T>(L, nelements, elements, 0, nullptr, x, y, s, em);
    }
#undef SFEM_LAP_EM_CASE
}

extern "C" int sfem_gb300_sshex8_laplacian_element_matrix(int element_type, ptrdiff_t nelements, ptrdiff_t fff_stride,
                                                          const float *fff, int real_type, void *em, void *stream) {
    const int L = element_type - SFEM_GB300_SSHEX8_BASE;
    if (L < 1 || L > LAP_MAX_L)
        return set_error("sfem_gb300_sshex8_laplacian_element_matrix: unsupported element type %d", element_type);
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    const int grid = grid_for(nelements * 64, 256);
    switch (real_type) {
        case SFEM_GB300_REAL_DEFAULT:
        case SFEM_GB300_FLOAT64:
            sshex8_laplacian_element_matrix_kernel<double><<<grid, 256, 0, s>>>(nelements, L, fff_stride, fff,
                                                                                 (double *)em);
            break;
        case SFEM_GB300_FLOAT32:
            sshex8_laplacian_element_matrix_kernel<float><<<grid, 256, 0, s>>>(nelements, L, fff_stride, fff,
                                                                                (float *)em);
            break;
        default:
            return set_error("sfem_gb300_sshex8_laplacian_element_matrix: unsupported real type %d", real_type);
    }
    return check_launch("sfem_gb300_sshex8_laplacian_element_matrix");
}

extern "C" int sfem_gb300_sshex8_laplacian_apply_em(int element_type, ptrdiff_t nelements, idx_t **elements,
                                                    const void *em, int real_type, const void *x, void *y,
                                                    void *stream) {
    const int L = element_type - SFEM_GB300_SSHEX8_BASE;
    if (L < 1 || L > LAP_MAX_L)
        return set_error("sfem_gb300_sshex8_laplacian_apply_em: unsupported element type %d", element_type);
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    switch (real_type) {
        case SFEM_GB300_REAL_DEFAULT:
        case SFEM_GB300_FLOAT64:
            return laplacian_apply_em_tpl<double>(L, nelements, elements, (const double *)em, (const double *)x,
                                                  (double *)y, s);
        case SFEM_GB300_FLOAT32:
            return laplacian_apply_em_tpl<float>(L, nelements, elements, (const float *)em, (const float *)x,
                                                 (float *)y, s);
        default:
            return set_error("sfem_gb300_sshex8_laplacian_apply_em: unsupported real type %d", real_type);
    }
}
