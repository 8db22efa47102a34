// Matrix-free linear elasticity (3 dofs per node, interleaved u[3*node+d]) on
// hex8 and sshex8 meshes, sm_103a.
//
// Operator (reference: affine_sshex8_linear_elasticity_apply_macro_adjugate,
// operators/sshex8/sshex8_linear_elasticity.cpp:275-424): one adjugate (9
// floats) and determinant per macro element; sub-adjugate = adj h^2 and
// sub-det = det h^3 with h = 1/L (operators/sshex8/sshex8.hpp:26-42); the 24x24
// element stiffness K (row/column = component*8 + corner) is applied to every
// micro element.  K[(i,a),(j,b)] = 1/det sum_pq I_ab^pq (mu adj_pj adj_qi +
// lambda adj_pi adj_qj + delta_ij mu (adj adj^T)_pq), I_ab^pq the exact Q1
// integrals of d_p phi_a d_q phi_b on the unit cube.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>
#include <atomic>
#include <mutex>

#include "common.cuh"
#include "tcgen05.cuh"

namespace sfem_gb300 {

struct GradTable {
    double I[8][8][3][3];
    constexpr GradTable() : I() {
        for (int a = 0; a < 8; a++)
            for (int b = 0; b < 8; b++)
                for (int p = 0; p < 3; p++)
                    for (int q = 0; q < 3; q++) I[a][b][p][q] = q1_grad_integral(a, b, p, q);
    }
};
// global (not __constant__): lanes read different entries, which the constant cache would serialise
static __device__ GradTable kGrad = GradTable();

// sshex8 lidx of the hex8 corner c at level 1 (used when a hex8 mesh is given in hex8 order)
__host__ __device__ constexpr int hex8_corner_of_lidx1(int l) {
    return l == 0 ? 0 : l == 1 ? 1 : l == 2 ? 3 : l == 3 ? 2 : l == 4 ? 4 : l == 5 ? 5 : l == 6 ? 7 : 6;
}

// Entry k (0..575) of the 24x24 element matrix from sub-adjugate / sub-det.
template <typename T>
__device__ __forceinline__ T elasticity_entry(int k, const T adj[9], const T AA[9], T inv_det, T mu, T lambda) {
    const int row = k / 24, col = k % 24;
    const int i = row / 8, a = row % 8, j = col / 8, b = col % 8;
    T s = 0;
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int q = 0; q < 3; q++) {
            T w = mu * adj[3 * p + j] * adj[3 * q + i] + lambda * adj[3 * p + i] * adj[3 * q + j];
            if (i == j) w += mu * AA[3 * p + q];
            s += (T)kGrad.I[a][b][p][q] * w;
        }
    return s * inv_det;
}

template <typename T>
__device__ __forceinline__ void load_sub_adjugate(const float *adjugate, const float *determinant, ptrdiff_t stride,
                                                  ptrdiff_t e, int L, T adj[9], T AA[9], T &inv_det) {
    const T h = T(1) / T(L);
#pragma unroll
    for (int d = 0; d < 9; d++) adj[d] = (T)adjugate[d * stride + e] * (h * h);
    const T det = (T)determinant[e] * (h * h * h);
    inv_det = T(1) / det;
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int q = 0; q < 3; q++) AA[3 * p + q] = adj[3 * p] * adj[3 * q] + adj[3 * p + 1] * adj[3 * q + 1] + adj[3 * p + 2] * adj[3 * q + 2];
}

// Cooperative K build by one warp: W[i][j][p][q] = mu adj_pj adj_qi + lambda adj_pi adj_qj
// + delta_ij mu (adj adj^T)_pq (81 values) then K[(i,a),(j,b)] = inv_det sum_pq I_ab^pq W_ij^pq.
// I (the unit-cube Q1 gradient integrals) comes from a per-block shared copy: lanes read
// different entries, which constant memory would serialise.
template <typename T>
__device__ __forceinline__ void build_K_warp(const T adj[9], const T AA[9], T inv_det, T mu, T lambda,
                                             const T *__restrict__ Is, T *__restrict__ Wsm, T *__restrict__ K,
                                             int ld, int lane) {
    for (int k = lane; k < 81; k += 32) {
        const int i = k / 27, j = (k / 9) % 3, p = (k / 3) % 3, q = k % 3;
        T w = mu * adj[3 * p + j] * adj[3 * q + i] + lambda * adj[3 * p + i] * adj[3 * q + j];
        if (i == j) w += mu * AA[3 * p + q];
        Wsm[k] = w;
    }
    __syncwarp();
    for (int k = lane; k < 576; k += 32) {
        const int row = k / 24, col = k % 24;
        const int i = row >> 3, a = row & 7, j = col >> 3, b = col & 7;
        const T *Iab = &Is[(a * 8 + b) * 9];
        const T *Wij = &Wsm[(i * 3 + j) * 9];
        T acc = 0;
#pragma unroll
        for (int pq = 0; pq < 9; pq++) acc += Iab[pq] * Wij[pq];
        K[row * ld + col] = acc * inv_det;
    }
    __syncwarp();
}

// Same K from its six distinct 8x8 blocks (K_ji = K_ij^T): lane l owns the entries
// (a, b) = (l / 8, l % 8) and (l / 8 + 4, l % 8) of every block, with their Q1
// gradient integrals I_ab^pq held in registers (Ir, loaded once per kernel) and the 81
// W values read from shared memory as warp-wide broadcasts.
template <typename T>
__device__ __forceinline__ void load_grad_regs(int lane, T (&Ir)[2][9]) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int l = lane + 32 * h;
#pragma unroll
        for (int pq = 0; pq < 9; pq++) Ir[h][pq] = (T)kGrad.I[l >> 3][l & 7][pq / 3][pq % 3];
    }
}

template <typename T>
__device__ __forceinline__ void build_K_warp_sym(const T adj[9], const T AA[9], T inv_det, T mu, T lambda,
                                                 const T (&Ir)[2][9], T *__restrict__ Wsm, T *__restrict__ K,
                                                 int ld, int lane) {
    for (int k = lane; k < 81; k += 32) {
        const int i = k / 27, j = (k / 9) % 3, p = (k / 3) % 3, q = k % 3;
        T w = mu * adj[3 * p + j] * adj[3 * q + i] + lambda * adj[3 * p + i] * adj[3 * q + j];
        if (i == j) w += mu * AA[3 * p + q];
        Wsm[k] = w;
    }
    __syncwarp();
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int l = lane + 32 * h, a = l >> 3, b = l & 7;
#pragma unroll
        for (int blk = 0; blk < 6; blk++) {
            const int i = blk < 3 ? 0 : (blk < 5 ? 1 : 2);
            const int j = blk < 3 ? blk : (blk < 5 ? blk - 2 : 2);  // (0,0) (0,1) (0,2) (1,1) (1,2) (2,2)
            const T *Wij = &Wsm[(i * 3 + j) * 9];
            T acc = 0;
#pragma unroll
            for (int pq = 0; pq < 9; pq++) acc += Ir[h][pq] * Wij[pq];
            acc *= inv_det;
            K[(i * 8 + a) * ld + j * 8 + b] = acc;
            if (i != j) K[(j * 8 + b) * ld + i * 8 + a] = acc;
        }
    }
    __syncwarp();
}

template <typename T>
__device__ __forceinline__ void load_grad_table(T *Is) {
    for (int k = threadIdx.x; k < 576; k += blockDim.x) Is[k] = (T)(&kGrad.I[0][0][0][0])[k];
    __syncthreads();
}

// v1: one warp per macro element.  The warp builds K (576 entries) in shared
// memory, stages the (L+1)^3 x 3 micro-grid values, lanes apply K per micro
// element with shared-memory accumulation, then scatter (owned interior nodes
// plain, shared surface nodes atomic).  HEX8 = plain hex8 mesh in hex8 corner order.
// Element matrices of every macro element of a level (sub-adjugate at level L), stored
// row-major [e][(i, a)][(j, b)]: one warp per element.
template <typename T>
__global__ void __launch_bounds__(64) elasticity_element_matrices_kernel(ptrdiff_t nelements, int L, ptrdiff_t stride,
                                                                         const float *adjugate,
                                                                         const float *determinant, T mu, T lambda,
                                                                         T *__restrict__ Kout) {
    __shared__ T Ws[2][81];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T Ir[2][9];
    load_grad_regs<T>(lane, Ir);
    for (ptrdiff_t e = (ptrdiff_t)blockIdx.x * 2 + warp; e < nelements; e += (ptrdiff_t)gridDim.x * 2) {
        T adj[9], AA[9], inv_det;
        load_sub_adjugate<T>(adjugate, determinant, stride, e, L, adj, AA, inv_det);
        build_K_warp_sym<T>(adj, AA, inv_det, mu, lambda, Ir, Ws[warp], Kout + 576 * e, 24, lane);
    }
}

// STORED: the element matrices come from Kg (elasticity_element_matrices_kernel) instead
// of being built from the sub-adjugate (used on coarse levels, where building a 24x24
// matrix costs more than applying it to the 8 or 1 micro elements).
template <typename T, int L, bool HEX8, bool STORED = false>
__global__ void __launch_bounds__(64) elasticity_apply_warp_kernel(ptrdiff_t nelements, const idx_t *const *elements,
                                                                   ptrdiff_t stride, const float *adjugate,
                                                                   const float *determinant, T mu, T lambda,
                                                                   const T *__restrict__ x, T *__restrict__ y,
                                                                   const T *__restrict__ Kg = nullptr) {
    constexpr int N1 = L + 1;
    constexpr int NXE = N1 * N1 * N1;
    constexpr int NM = L * L * L;
    constexpr int WPB = 2;
    constexpr int NR = (NXE + 31) / 32;
    __shared__ T Ks[WPB][576];
    __shared__ T xs[WPB][3 * NXE];
    __shared__ T ys[WPB][3 * NXE];
    __shared__ T Ws[WPB][81];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T *K = Ks[warp];
    T *xw = xs[warp];
    T *yw = ys[warp];
    T Ir[2][9];
    if constexpr (!STORED) load_grad_regs<T>(lane, Ir);
    for (ptrdiff_t e = (ptrdiff_t)blockIdx.x * WPB + warp; e < nelements; e += (ptrdiff_t)gridDim.x * WPB) {
        if constexpr (STORED) {
            const T *src = Kg + 576 * e;
            for (int k = lane; k < 576; k += 32) K[k] = src[k];
            __syncwarp();
        } else {
            T adj[9], AA[9], inv_det;
            load_sub_adjugate<T>(adjugate, determinant, stride, e, L, adj, AA, inv_det);
            build_K_warp_sym<T>(adj, AA, inv_det, mu, lambda, Ir, Ws[warp], K, 24, lane);
        }
        idx_t gi[NR];
#pragma unroll
        for (int r = 0; r < NR; r++) {
            const int l = lane + 32 * r;
            if (l < NXE) {
                gi[r] = elements[HEX8 ? hex8_corner_of_lidx1(l) : l][e];
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    xw[d * NXE + l] = x[3 * (ptrdiff_t)gi[r] + d];
                    yw[d * NXE + l] = 0;
                }
            }
        }
        __syncwarp();
        if constexpr (sizeof(T) == 4 && NM == 64) {
            // two micro elements per lane (m and m + 32) in one pass: each element-matrix
            // entry read from shared memory feeds one packed FP32x2 FMA for both
            int va[8], vb[8];
            float2 uu[24];
            {
                const int ma = lane, mb = lane + 32;
                const int xa = ma % L, ya = (ma / L) % L, za = ma / (L * L);
                const int xb = mb % L, yb = (mb / L) % L, zb = mb / (L * L);
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    va[c] = lidx(L, xa + c8x(c), ya + c8y(c), za + c8z(c));
                    vb[c] = lidx(L, xb + c8x(c), yb + c8y(c), zb + c8z(c));
                }
#pragma unroll
                for (int d = 0; d < 3; d++)
#pragma unroll
                    for (int c = 0; c < 8; c++)
                        uu[d * 8 + c] = make_float2((float)xw[d * NXE + va[c]], (float)xw[d * NXE + vb[c]]);
            }
#pragma unroll 1
            for (int d = 0; d < 3; d++) {
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    const int i = d * 8 + c;
                    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
                    for (int j = 0; j < 24; j++) {
                        const float k = (float)K[i * 24 + j];
                        acc = __ffma2_rn(make_float2(k, k), uu[j], acc);
                    }
                    atomicAdd(&yw[d * NXE + va[c]], (T)acc.x);
                    atomicAdd(&yw[d * NXE + vb[c]], (T)acc.y);
                }
            }
        } else if constexpr (NM >= 32) {
            // one micro element per lane: u read once, reused by the 24 rows
            for (int m = lane; m < NM; m += 32) {
                const int xi = m % L, yi = (m / L) % L, zi = m / (L * L);
                int v[8];
                T u[24];
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    v[c] = lidx(L, xi + c8x(c), yi + c8y(c), zi + c8z(c));
#pragma unroll
                    for (int d = 0; d < 3; d++) u[d * 8 + c] = xw[d * NXE + v[c]];
                }
#pragma unroll 4
                for (int i = 0; i < 24; i++) {
                    T acc = 0;
#pragma unroll
                    for (int j = 0; j < 24; j++) acc += K[i * 24 + j] * u[j];
                    atomicAdd(&yw[(i / 8) * NXE + v[i % 8]], acc);
                }
            }
        } else {
            // few micro elements (hex8, L = 2, 3 with L^3 < 32): one (micro element, row) pair per lane
            for (int t = lane; t < NM * 24; t += 32) {
                const int m = t / 24, i = t % 24;
                const int xi = m % L, yi = (m / L) % L, zi = m / (L * L);
                T acc = 0;
#pragma unroll
                for (int j = 0; j < 24; j++) {
                    const int c = j % 8;
                    acc += K[i * 24 + j] * xw[(j / 8) * NXE + lidx(L, xi + c8x(c), yi + c8y(c), zi + c8z(c))];
                }
                const int ci = i % 8;
                atomicAdd(&yw[(i / 8) * NXE + lidx(L, xi + c8x(ci), yi + c8y(ci), zi + c8z(ci))], acc);
            }
        }
        __syncwarp();
#pragma unroll
        for (int r = 0; r < NR; r++) {
            const int l = lane + 32 * r;
            if (l < NXE) {
                const int xi = l % N1, yi = (l / N1) % N1, zi = l / (N1 * N1);
                const bool interior = xi > 0 && xi < L && yi > 0 && yi < L && zi > 0 && zi < L;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const T val = yw[d * NXE + l];
                    T *dst = &y[3 * (ptrdiff_t)gi[r] + d];
                    if (interior)
                        *dst += val;
                    else
                        atomicAdd(dst, val);
                }
            }
        }
        __syncwarp();
    }
}


// Tensor-core variant (FP32 vectors, BF16 element contraction, FP32 accumulate):
// per macro element Y(24 x L^3) = K(24 x 24) U(24 x L^3), U[:, m] the 24 dofs of micro
// element m, with warp-level mma.sync.m16n8k16 (K padded to 32 x 32 in BF16).  One warp
// per macro element; the micro-grid values are staged in shared memory, outputs are
// accumulated with shared-memory atomics and scattered like the SIMT kernel.
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float d[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};\n"
            : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int L, bool HEX8>
__global__ void __launch_bounds__(128) elasticity_apply_tc_kernel(ptrdiff_t nelements, const idx_t *const *elements,
                                                                  ptrdiff_t stride, const float *adjugate,
                                                                  const float *determinant, float mu, float lambda,
                                                                  const float *__restrict__ x, float *__restrict__ y) {
    constexpr int N1 = L + 1;
    constexpr int NXE = N1 * N1 * N1;
    constexpr int NM = L * L * L;
    constexpr int NT = (NM + 7) / 8;  // n-tiles of 8 micro elements
    constexpr int WPB = 4;
    constexpr int NR = (NXE + 31) / 32;
    __shared__ float Ks[WPB][32 * 32];
    __shared__ float xs[WPB][3 * NXE];
    __shared__ float ys[WPB][3 * NXE];
    __shared__ float Is[576];
    __shared__ float Ws[WPB][81];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gid = lane >> 2, tig = lane & 3;
    float *K = Ks[warp];
    float *xw = xs[warp];
    float *yw = ys[warp];
    load_grad_table<float>(Is);
    for (int k = lane; k < 1024; k += 32) K[k] = 0.f;  // zero padding rows/cols 24..31
    __syncwarp();
    for (ptrdiff_t e = (ptrdiff_t)blockIdx.x * WPB + warp; e < nelements; e += (ptrdiff_t)gridDim.x * WPB) {
        float adj[9], AA[9], inv_det;
        load_sub_adjugate<float>(adjugate, determinant, stride, e, L, adj, AA, inv_det);
        build_K_warp<float>(adj, AA, inv_det, mu, lambda, Is, Ws[warp], K, 32, lane);
        idx_t gi[NR];
#pragma unroll
        for (int r = 0; r < NR; r++) {
            const int l = lane + 32 * r;
            if (l < NXE) {
                gi[r] = elements[HEX8 ? hex8_corner_of_lidx1(l) : l][e];
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    xw[d * NXE + l] = x[3 * (ptrdiff_t)gi[r] + d];
                    yw[d * NXE + l] = 0.f;
                }
            }
        }
        __syncwarp();
        // A fragments of K: a[mt][kt]
        uint32_t a[2][2][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int kt = 0; kt < 2; kt++) {
                const int r0 = mt * 16 + gid, c0 = kt * 16 + tig * 2;
                a[mt][kt][0] = pack_bf16x2(K[r0 * 32 + c0], K[r0 * 32 + c0 + 1]);
                a[mt][kt][1] = pack_bf16x2(K[(r0 + 8) * 32 + c0], K[(r0 + 8) * 32 + c0 + 1]);
                a[mt][kt][2] = pack_bf16x2(K[r0 * 32 + c0 + 8], K[r0 * 32 + c0 + 9]);
                a[mt][kt][3] = pack_bf16x2(K[(r0 + 8) * 32 + c0 + 8], K[(r0 + 8) * 32 + c0 + 9]);
            }
#pragma unroll 1
        for (int nt = 0; nt < NT; nt++) {
            // B fragment: U[k][m], m = nt*8 + gid (this thread's column)
            const int m = nt * 8 + gid;
            const bool mvalid = m < NM;
            const int xi = m % L, yi = (m / L) % L, zi = m / (L * L);
            auto U = [&](int k) -> float {
                if (!mvalid || k >= 24) return 0.f;
                const int comp = k >> 3, c = k & 7;
                return xw[comp * NXE + lidx(L, xi + c8x(c), yi + c8y(c), zi + c8z(c))];
            };
            uint32_t b[2][2];
#pragma unroll
            for (int kt = 0; kt < 2; kt++) {
                const int k0 = kt * 16 + tig * 2;
                b[kt][0] = pack_bf16x2(U(k0), U(k0 + 1));
                b[kt][1] = pack_bf16x2(U(k0 + 8), U(k0 + 9));
            }
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {
                float d[4] = {0.f, 0.f, 0.f, 0.f};
                mma_bf16_16816(d, a[mt][0], b[0]);
                mma_bf16_16816(d, a[mt][1], b[1]);
                // d[0..1]: row mt*16+gid, cols tig*2+{0,1};  d[2..3]: row +8
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int row = mt * 16 + gid + (q >= 2 ? 8 : 0);
                    const int col = nt * 8 + tig * 2 + (q & 1);
                    if (row < 24 && col < NM) {
                        const int cx = col % L, cy = (col / L) % L, cz = col / (L * L);
                        const int comp = row >> 3, c = row & 7;
                        atomicAdd(&yw[comp * NXE + lidx(L, cx + c8x(c), cy + c8y(c), cz + c8z(c))], d[q]);
                    }
                }
            }
        }
        __syncwarp();
#pragma unroll
        for (int r = 0; r < NR; r++) {
            const int l = lane + 32 * r;
            if (l < NXE) {
                const int px = l % N1, py = (l / N1) % N1, pz = l / (N1 * N1);
                const bool interior = px > 0 && px < L && py > 0 && py < L && pz > 0 && pz < L;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const float val = yw[d * NXE + l];
                    float *dst = &y[3 * (ptrdiff_t)gi[r] + d];
                    if (interior)
                        *dst += val;
                    else
                        atomicAdd(dst, val);
                }
            }
        }
        __syncwarp();
    }
}

// Diagonal (diag3: 3 per node) and symmetric 3x3 block diagonal (block6: 00,01,02,11,12,22 per node).
template <typename T, int L, bool HEX8>
__global__ void __launch_bounds__(64) elasticity_block_diag_kernel(ptrdiff_t nelements, const idx_t *const *elements,
                                                                   ptrdiff_t stride, const float *adjugate,
                                                                   const float *determinant, T mu, T lambda, T *diag3,
                                                                   T *block6) {
    constexpr int N1 = L + 1;
    constexpr int NXE = N1 * N1 * N1;
    constexpr int WPB = 2;
    __shared__ T Bs[WPB][8][6];
    __shared__ T Ks[WPB][576];
    __shared__ T Is[576];
    __shared__ T Ws[WPB][81];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bi[6] = {0, 0, 0, 1, 1, 2}, bj[6] = {0, 1, 2, 1, 2, 2};
    load_grad_table<T>(Is);
    for (ptrdiff_t e = (ptrdiff_t)blockIdx.x * WPB + warp; e < nelements; e += (ptrdiff_t)gridDim.x * WPB) {
        T adj[9], AA[9], inv_det;
        load_sub_adjugate<T>(adjugate, determinant, stride, e, L, adj, AA, inv_det);
        build_K_warp<T>(adj, AA, inv_det, mu, lambda, Is, Ws[warp], Ks[warp], 24, lane);
        for (int k = lane; k < 48; k += 32) {
            const int a = k / 6, c = k % 6;
            Bs[warp][a][c] = Ks[warp][(bi[c] * 8 + a) * 24 + bj[c] * 8 + a];
        }
        __syncwarp();
        for (int l = lane; l < NXE; l += 32) {
            const int xi = l % N1, yi = (l / N1) % N1, zi = l / (N1 * N1);
            T s[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
            for (int a = 0; a < 8; a++) {
                const bool ok = (c8x(a) ? xi > 0 : xi < L) && (c8y(a) ? yi > 0 : yi < L) && (c8z(a) ? zi > 0 : zi < L);
                if (ok)
#pragma unroll
                    for (int c = 0; c < 6; c++) s[c] += Bs[warp][a][c];
            }
            const ptrdiff_t g = elements[HEX8 ? hex8_corner_of_lidx1(l) : l][e];
            const bool interior = xi > 0 && xi < L && yi > 0 && yi < L && zi > 0 && zi < L;
            if (diag3) {
                const T dv[3] = {s[0], s[3], s[5]};
                for (int d = 0; d < 3; d++) {
                    if (interior)
                        diag3[3 * g + d] += dv[d];
                    else
                        atomicAdd(&diag3[3 * g + d], dv[d]);
                }
            }
            if (block6) {
                for (int c = 0; c < 6; c++) {
                    if (interior)
                        block6[6 * g + c] += s[c];
                    else
                        atomicAdd(&block6[6 * g + c], s[c]);
                }
            }
        }
        __syncwarp();
    }
}

// In-place inversion of symmetric 3x3 blocks (6 per node) scaled by omega, with
// Dirichlet nodes set to identity (inverse3_inplace_apply_AoS + mask3_apply,
// algebra/cuda/sfem_cuda_ShiftableJacobi.cu:14-100).
template <typename T>
__global__ void block_inverse_kernel(ptrdiff_t n_nodes, T *block6, T omega) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n_nodes; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        T *b = &block6[6 * i];
        const T a00 = b[0], a01 = b[1], a02 = b[2], a11 = b[3], a12 = b[4], a22 = b[5];
        const T c00 = a11 * a22 - a12 * a12, c01 = a02 * a12 - a01 * a22, c02 = a01 * a12 - a02 * a11;
        const T c11 = a00 * a22 - a02 * a02, c12 = a01 * a02 - a00 * a12, c22 = a00 * a11 - a01 * a01;
        const T det = a00 * c00 + a01 * c01 + a02 * c02;
        const T s = det != T(0) ? omega / det : T(0);
        b[0] = c00 * s;
        b[1] = c01 * s;
        b[2] = c02 * s;
        b[3] = c11 * s;
        b[4] = c12 * s;
        b[5] = c22 * s;
    }
}

template <typename T>
__global__ void block_identity_kernel(ptrdiff_t nn, const idx_t *nodes, T *block6) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < nn; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        T *b = &block6[6 * (ptrdiff_t)nodes[i]];
        b[0] = 1;
        b[1] = 0;
        b[2] = 0;
        b[3] = 1;
        b[4] = 0;
        b[5] = 1;
    }
}

// x += B r for symmetric 3x3 blocks B (block Jacobi step)
template <typename T>
__global__ void block_apply_kernel(ptrdiff_t n_nodes, const T *__restrict__ block6, const T *__restrict__ r,
                                   T *__restrict__ x) {
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n_nodes; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        const T *b = &block6[6 * i];
        const T r0 = r[3 * i], r1 = r[3 * i + 1], r2 = r[3 * i + 2];
        x[3 * i] += b[0] * r0 + b[1] * r1 + b[2] * r2;
        x[3 * i + 1] += b[1] * r0 + b[3] * r1 + b[4] * r2;
        x[3 * i + 2] += b[2] * r0 + b[4] * r1 + b[5] * r2;
    }
}

static int elasticity_apply_tc(int element_type, ptrdiff_t nelements, idx_t **elements, ptrdiff_t stride,
                               const float *adj, const float *det, float mu, float lambda, const float *x, float *y,
                               cudaStream_t s) {
    const int blocks = grid_for((nelements + 3) / 4, 1, kNumSMs * 64);
    if (element_type == SFEM_GB300_HEX8) {
        elasticity_apply_tc_kernel<1, true><<<blocks, 128, 0, s>>>(nelements, elements, stride, adj, det, mu, lambda, x, y);
        return check_launch("sfem_gb300_linear_elasticity_apply(HEX8, tensor cores)");
    }
    switch (element_type - SFEM_GB300_SSHEX8_BASE) {
        case 1:
            elasticity_apply_tc_kernel<1, false><<<blocks, 128, 0, s>>>(nelements, elements, stride, adj, det, mu, lambda, x, y);
            break;
        case 2:
            elasticity_apply_tc_kernel<2, false><<<blocks, 128, 0, s>>>(nelements, elements, stride, adj, det, mu, lambda, x, y);
            break;
        case 3:
            elasticity_apply_tc_kernel<3, false><<<blocks, 128, 0, s>>>(nelements, elements, stride, adj, det, mu, lambda, x, y);
            break;
        case 4:
            elasticity_apply_tc_kernel<4, false><<<blocks, 128, 0, s>>>(nelements, elements, stride, adj, det, mu, lambda, x, y);
            break;
        default:
            return set_error("sfem_gb300_linear_elasticity_apply: unsupported element type %d", element_type);
    }
    return check_launch("sfem_gb300_linear_elasticity_apply(SSHEX8, tensor cores)");
}

// ---------------------------------------------------------------------------- tcgen05, 3xTF32
// FP32 sshex8 apply at L = 4 with the element-matrix contraction on the 5th-generation
// tensor cores.  A CTA of four warps takes macro elements in pairs (e0, e1): one M = 128
// tile holds the 64 micro elements of each (rows 0..63: e0, 64..127: e1) by their 24
// dofs, A[m][(j, b)] = u_j(corner b of micro element m); B_e = K_e (24 x 24, N padded
// to 32, K-major); D_e = A K_e^T in tensor memory (the rows of e are kept).  Operands
// are split into TF32 hi = tf32(x) and lo = x - hi and multiplied as hi.hi + hi.lo +
// lo.hi (kind::tf32, K = 8 per MMA, FP32 accumulate): 9 MMAs per element, issued by
// lane 0 of warp e, FP32-level accuracy (the dropped lo.lo term is ~2^-22 relative).
// K is built from its six distinct 8x8 blocks (K_ji = K_ij^T).  The next pair's
// metric, node indices and values are loaded while the current pair is processed.
// Epilogue: the D rows go to shared memory; each thread then sums the (up to 8)
// micro-element contributions of its nodes and adds them to y with atomics.
constexpr int ETC_L = 4, ETC_N1 = ETC_L + 1, ETC_NXE = ETC_N1 * ETC_N1 * ETC_N1;  // 125 nodes
constexpr int ETC_A_CHUNK = 128 * 16;   // [chunk of 4 dofs][row 128][16 B]
constexpr int ETC_A_BYTES = 6 * ETC_A_CHUNK;
constexpr int ETC_B_CHUNK = 32 * 16;    // [chunk][n 32][16 B]
constexpr int ETC_B_BYTES = 6 * ETC_B_CHUNK;  // one element
constexpr int ETC_YLD = 25;             // row stride (floats) of the D rows in shared memory
constexpr int ETC_OFF_AHI = 0, ETC_OFF_ALO = ETC_A_BYTES;  // D rows alias both after the MMAs
constexpr int ETC_OFF_BHI = 2 * ETC_A_BYTES, ETC_OFF_BLO = ETC_OFF_BHI + 2 * ETC_B_BYTES;
constexpr int ETC_OFF_X = ETC_OFF_BLO + 2 * ETC_B_BYTES;   // [2][3][125] floats
constexpr int ETC_SMEM = ETC_OFF_X + 2 * 3 * ETC_NXE * 4;
constexpr int ETC_CTAS_PER_SM = 4;
constexpr uint32_t ETC_TMEM_COLS = 64;  // D_e at cols 32 e
constexpr int ETC_WAIT_POLLS = 1 << 20;
static_assert((ETC_SMEM + 2048) * ETC_CTAS_PER_SM <= 228 * 1024, "shared memory of the resident CTAs");
static_assert(128 * ETC_YLD * 4 <= 2 * ETC_A_BYTES, "D rows fit in the A region");
__device__ int g_etc_status;  // nonzero: a tensor-core wait gave up

__global__ void __launch_bounds__(128, ETC_CTAS_PER_SM) elasticity_apply_tf32x3_kernel(
        ptrdiff_t nelements, const idx_t *const *elements, ptrdiff_t stride, const float *adjugate,
        const float *determinant, float mu, float lambda, const float *__restrict__ x, float *__restrict__ y) {
    extern __shared__ __align__(16) unsigned char es[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_holder;
    __shared__ const idx_t *srow[ETC_NXE];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int e_loc = tid >> 6, u = tid & 63;  // element of the pair this thread serves
    float *xs = reinterpret_cast<float *>(es + ETC_OFF_X);
    float *Yd = reinterpret_cast<float *>(es + ETC_OFF_AHI);  // D rows after the MMAs
    for (int i = tid; i < ETC_OFF_X / 16; i += 128) reinterpret_cast<uint4 *>(es)[i] = make_uint4(0, 0, 0, 0);
    // this thread builds the entries (a, b) = (u / 8, u % 8) of the six distinct 8x8 blocks
    // of K: its nine gradient integrals I_ab^pq stay in registers
    float Ir[9];
#pragma unroll
    for (int pq = 0; pq < 9; pq++) Ir[pq] = (float)kGrad.I[u >> 3][u & 7][pq / 3][pq % 3];
    if (tid < ETC_NXE) srow[tid] = elements[tid];
    if (tid + 128 < ETC_NXE) srow[tid + 128] = elements[tid + 128];
    if (warp == 0) tc::tmem_alloc(&tmem_holder, ETC_TMEM_COLS);
    if (tid == 0) tc::mbar_init(&mbar, 2);  // one arrival per issuing warp (0, 1)
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_holder;
    uint32_t phase = 0;
    bool ok = true;
    // this thread's A row: micro element u of element e_loc; its nodes' lidx base
    const int mbase = lidx(ETC_L, u % ETC_L, (u / ETC_L) % ETC_L, u / (ETC_L * ETC_L));
    // this thread's nodes (v = u and u + 64 < 125) of element e_loc: prefetched metric,
    // indices and values of the next pair
    float pad_[10];
    idx_t pg[2] = {0, 0};
    float px[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    auto fetch_meta = [&](ptrdiff_t e) {
#pragma unroll
        for (int d = 0; d < 9; d++) pad_[d] = adjugate[d * stride + e];
        pad_[9] = determinant[e];
#pragma unroll
        for (int k = 0; k < 2; k++) pg[k] = (u + 64 * k < ETC_NXE) ? srow[u + 64 * k][e] : 0;
    };
    auto fetch_x = [&]() {
#pragma unroll
        for (int k = 0; k < 2; k++)
            if (u + 64 * k < ETC_NXE)
#pragma unroll
                for (int d = 0; d < 3; d++) px[k][d] = x[3 * (ptrdiff_t)pg[k] + d];
    };
    {
        const ptrdiff_t e = 2 * (ptrdiff_t)blockIdx.x + e_loc;
        if (e < nelements) {
            fetch_meta(e);
            fetch_x();
        }
    }
    for (ptrdiff_t pr = blockIdx.x; 2 * pr < nelements && ok; pr += gridDim.x) {
        const ptrdiff_t e = 2 * pr + e_loc;
        const bool valid = e < nelements;
        const bool pair = 2 * pr + 1 < nelements;
        // 1. sub-adjugate from the prefetched metric (registers), the element's values into
        // shared memory
        idx_t gcur[2] = {pg[0], pg[1]};
        float inv_det = 0.f;
        float adj[9], AA[9];
        {
            const float h = 1.f / (float)ETC_L;
#pragma unroll
            for (int d = 0; d < 9; d++) adj[d] = pad_[d] * (h * h);
            inv_det = valid ? 1.f / (pad_[9] * (h * h * h)) : 0.f;
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int q = 0; q < 3; q++)
                    AA[3 * p + q] = adj[3 * p] * adj[3 * q] + adj[3 * p + 1] * adj[3 * q + 1] + adj[3 * p + 2] * adj[3 * q + 2];
        }
        if (valid) {
#pragma unroll
            for (int k = 0; k < 2; k++)
                if (u + 64 * k < ETC_NXE)
#pragma unroll
                    for (int d = 0; d < 3; d++) xs[(e_loc * 3 + d) * ETC_NXE + u + 64 * k] = px[k][d];
        }
        // next pair's metric and node indices (consumed next iteration)
        const ptrdiff_t en = 2 * (pr + gridDim.x) + e_loc;
        const bool has_next = en < nelements;
        if (has_next) fetch_meta(en);
        __syncthreads();
        // 2. B_e = K_e (hi / lo) from its six distinct 8x8 blocks (entry (a, b) of each by this
        // thread, W_ij^pq = mu adj_pj adj_qi + lambda adj_pi adj_qj + delta_ij mu (adj adj^T)_pq
        // in registers), and this thread's A row
        if (valid) {
            const int a = u >> 3, b = u & 7;
#pragma unroll
            for (int blk = 0; blk < 6; blk++) {
                const int i = blk < 3 ? 0 : (blk < 5 ? 1 : 2);
                const int j = blk < 3 ? blk : (blk < 5 ? blk - 2 : 2);  // (0,0) (0,1) (0,2) (1,1) (1,2) (2,2)
                float acc = 0.f;
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        float w = mu * adj[3 * p + j] * adj[3 * q + i] + lambda * adj[3 * p + i] * adj[3 * q + j];
                        if (i == j) w += mu * AA[3 * p + q];
                        acc += Ir[3 * p + q] * w;
                    }
                acc *= inv_det;
                const float hi = tc::tf32_round(acc), lo = acc - hi;
                const int r1 = i * 8 + a, c1 = j * 8 + b;
                const int o1 = e_loc * ETC_B_BYTES + (c1 >> 2) * ETC_B_CHUNK + r1 * 16 + (c1 & 3) * 4;
                const int o2 = e_loc * ETC_B_BYTES + (r1 >> 2) * ETC_B_CHUNK + c1 * 16 + (r1 & 3) * 4;
                *reinterpret_cast<float *>(es + ETC_OFF_BHI + o1) = hi;
                *reinterpret_cast<float *>(es + ETC_OFF_BLO + o1) = lo;
                *reinterpret_cast<float *>(es + ETC_OFF_BHI + o2) = hi;  // K symmetric
                *reinterpret_cast<float *>(es + ETC_OFF_BLO + o2) = lo;
            }
            const float *xe = xs + e_loc * 3 * ETC_NXE + mbase;
#pragma unroll
            for (int c4 = 0; c4 < 6; c4++) {
                float hv[4], lv[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int col = 4 * c4 + k, j = col >> 3, b = col & 7;
                    const float val = xe[j * ETC_NXE + lidx(ETC_L, c8x(b), c8y(b), c8z(b))];
                    hv[k] = tc::tf32_round(val);
                    lv[k] = val - hv[k];
                }
                *reinterpret_cast<float4 *>(es + ETC_OFF_AHI + c4 * ETC_A_CHUNK + tid * 16) =
                        make_float4(hv[0], hv[1], hv[2], hv[3]);
                *reinterpret_cast<float4 *>(es + ETC_OFF_ALO + c4 * ETC_A_CHUNK + tid * 16) =
                        make_float4(lv[0], lv[1], lv[2], lv[3]);
            }
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        // 3. MMAs: lane 0 of warp el issues D_el (+)= A_hi B_hi + A_hi B_lo + A_lo B_hi, 3 K steps
        if (lane == 0 && warp < 2) {
            const int el = warp;
            if (el == 0 || pair) {
                constexpr uint32_t id = tc::idesc_tf32_f32(128, 32);
                const uint64_t ahi = tc::sdesc(tc::smem_u32(es + ETC_OFF_AHI), ETC_A_CHUNK, 128);
                const uint64_t alo = tc::sdesc(tc::smem_u32(es + ETC_OFF_ALO), ETC_A_CHUNK, 128);
                const uint64_t bhi = tc::sdesc(tc::smem_u32(es + ETC_OFF_BHI), ETC_B_CHUNK, 128);
                const uint64_t blo = tc::sdesc(tc::smem_u32(es + ETC_OFF_BLO), ETC_B_CHUNK, 128);
#pragma unroll
                for (int st = 0; st < 3; st++) {
                    const uint64_t ao = (uint64_t)(2 * st * ETC_A_CHUNK / 16);
                    const uint64_t bo = (uint64_t)((el * ETC_B_BYTES + 2 * st * ETC_B_CHUNK) / 16);
                    tc::mma_tf32(tmem + 32 * el, ahi + ao, bhi + bo, id, st > 0);
                    tc::mma_tf32(tmem + 32 * el, ahi + ao, blo + bo, id, 1);
                    tc::mma_tf32(tmem + 32 * el, alo + ao, bhi + bo, id, 1);
                }
            }
            tc::commit(&mbar);
        }
        if (has_next) fetch_x();  // the values of the next pair's nodes (indices loaded above)
        {
            bool w = true;
            if (warp == 0) w = tc::mbar_wait(&mbar, phase, ETC_WAIT_POLLS);
            ok = __syncthreads_and(w);
            phase ^= 1;
            tc::fence_after_sync();
        }
        if (!ok) break;
        // 4. D rows to shared memory (row 32 w + lane of element w / 2)
        {
            const int el = warp >> 1;
            float a[16], b[16];
            tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + 32 * el, a);
            tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + 32 * el + 16, b);
            float *yr = Yd + tid * ETC_YLD;
#pragma unroll
            for (int r = 0; r < 16; r++) yr[r] = a[r];
#pragma unroll
            for (int r = 0; r < 8; r++) yr[16 + r] = b[r];
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        // 5. node sums over the (up to 8) micro elements around each node, added to y
        if (valid) {
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const int v = u + 64 * k;
                if (v < ETC_NXE) {
                    const int vx = v % ETC_N1, vy = (v / ETC_N1) % ETC_N1, vz = v / (ETC_N1 * ETC_N1);
                    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        const int mx = vx - c8x(c), my = vy - c8y(c), mz = vz - c8z(c);
                        if ((unsigned)mx < ETC_L && (unsigned)my < ETC_L && (unsigned)mz < ETC_L) {
                            const float *yr = Yd + (e_loc * 64 + (mz * ETC_L + my) * ETC_L + mx) * ETC_YLD;
                            s0 += yr[c];
                            s1 += yr[8 + c];
                            s2 += yr[16 + c];
                        }
                    }
                    float *dst = &y[3 * (ptrdiff_t)gcur[k]];
                    atomicAdd(dst, s0);
                    atomicAdd(dst + 1, s1);
                    atomicAdd(dst + 2, s2);
                }
            }
        }
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) atomicExch(&g_etc_status, 1);
        tc::mbar_wait(&mbar, phase ^ 1, ETC_WAIT_POLLS);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, ETC_TMEM_COLS);
}

// Any level 5 <= L <= 16 (no compile-time kernel): one CTA per macro element, warp 0
// builds K, the (L+1)^3 x 3 values of u and out in dynamic shared memory (FP64 up to
// L = 12, FP32 up to L = 16 within 227 KB), micro elements over the threads (u read
// once per micro element, 24 rows, shared-memory atomics), node ids read again for
// the scatter.
constexpr int EL_MAX_L = 16;
template <typename T>
__host__ __device__ constexpr size_t el_cta_smem_bytes(int L) {
    return (576 + 96 + 6 * (size_t)(L + 1) * (L + 1) * (L + 1)) * sizeof(T);
}

// three components of a nodal vector: component d of node g at c[d][g * stride]
// (interleaved xyz: c = {u, u + 1, u + 2}, stride 3; separate arrays: stride 1)
template <typename P>
struct Comp3 {
    P c[3];
    ptrdiff_t stride;
};

template <typename T>
__global__ void __launch_bounds__(256) elasticity_apply_cta_kernel(int L, ptrdiff_t nelements,
                                                                   const idx_t *const *elements, ptrdiff_t stride,
                                                                   const float *adjugate, const float *determinant,
                                                                   T mu, T lambda, Comp3<const T *> x,
                                                                   Comp3<T *> y) {
    extern __shared__ __align__(16) unsigned char el_cta_smem[];
    const int N1 = L + 1, NXE = N1 * N1 * N1, NM = L * L * L;
    T *K = reinterpret_cast<T *>(el_cta_smem);
    T *Wsm = K + 576;
    T *xs = Wsm + 96;
    T *ys = xs + 3 * NXE;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T Ir[2][9];
    if (warp == 0) load_grad_regs<T>(lane, Ir);
    for (ptrdiff_t e = blockIdx.x; e < nelements; e += gridDim.x) {
        if (warp == 0) {
            T adj[9], AA[9], inv_det;
            load_sub_adjugate<T>(adjugate, determinant, stride, e, L, adj, AA, inv_det);
            build_K_warp_sym<T>(adj, AA, inv_det, mu, lambda, Ir, Wsm, K, 24, lane);
        }
        for (int l = threadIdx.x; l < NXE; l += blockDim.x) {
            const ptrdiff_t g = elements[l][e];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                xs[d * NXE + l] = x.c[d][g * x.stride];
                ys[d * NXE + l] = 0;
            }
        }
        __syncthreads();
        for (int m = threadIdx.x; m < NM; m += blockDim.x) {
            const int xi = m % L, yi = (m / L) % L, zi = m / (L * L);
            int v[8];
            T u[24];
#pragma unroll
            for (int c = 0; c < 8; c++) {
                v[c] = lidx(L, xi + c8x(c), yi + c8y(c), zi + c8z(c));
#pragma unroll
                for (int d = 0; d < 3; d++) u[d * 8 + c] = xs[d * NXE + v[c]];
            }
#pragma unroll 4
            for (int i = 0; i < 24; i++) {
                T acc = 0;
#pragma unroll
                for (int j = 0; j < 24; j++) acc += K[i * 24 + j] * u[j];
                atomicAdd(&ys[(i / 8) * NXE + v[i % 8]], acc);
            }
        }
        __syncthreads();
        for (int l = threadIdx.x; l < NXE; l += blockDim.x) {
            const int xi = l % N1, yi = (l / N1) % N1, zi = l / (N1 * N1);
            const bool interior = xi > 0 && xi < L && yi > 0 && yi < L && zi > 0 && zi < L;
            const ptrdiff_t g = elements[l][e];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                if (interior)
                    y.c[d][g * y.stride] += ys[d * NXE + l];
                else
                    atomicAdd(&y.c[d][g * y.stride], ys[d * NXE + l]);
            }
        }
        __syncthreads();
    }
}

// Block diagonal at any level (runtime L), warp per macro element as the compile-time kernel.
template <typename T>
__global__ void __launch_bounds__(64) elasticity_block_diag_any_kernel(int L, ptrdiff_t nelements,
                                                                       const idx_t *const *elements, ptrdiff_t stride,
                                                                       const float *adjugate, const float *determinant,
                                                                       T mu, T lambda, T *diag3, T *block6) {
    const int N1 = L + 1, NXE = N1 * N1 * N1;
    constexpr int WPB = 2;
    __shared__ T Bs[WPB][8][6];
    __shared__ T Ks[WPB][576];
    __shared__ T Is[576];
    __shared__ T Ws[WPB][81];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bi[6] = {0, 0, 0, 1, 1, 2}, bj[6] = {0, 1, 2, 1, 2, 2};
    load_grad_table<T>(Is);
    for (ptrdiff_t e = (ptrdiff_t)blockIdx.x * WPB + warp; e < nelements; e += (ptrdiff_t)gridDim.x * WPB) {
        T adj[9], AA[9], inv_det;
        load_sub_adjugate<T>(adjugate, determinant, stride, e, L, adj, AA, inv_det);
        build_K_warp<T>(adj, AA, inv_det, mu, lambda, Is, Ws[warp], Ks[warp], 24, lane);
        for (int k = lane; k < 48; k += 32) {
            const int a = k / 6, c = k % 6;
            Bs[warp][a][c] = Ks[warp][(bi[c] * 8 + a) * 24 + bj[c] * 8 + a];
        }
        __syncwarp();
        for (int l = lane; l < NXE; l += 32) {
            const int xi = l % N1, yi = (l / N1) % N1, zi = l / (N1 * N1);
            T sacc[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
            for (int a = 0; a < 8; a++) {
                const bool ok = (c8x(a) ? xi > 0 : xi < L) && (c8y(a) ? yi > 0 : yi < L) && (c8z(a) ? zi > 0 : zi < L);
                if (ok)
#pragma unroll
                    for (int c = 0; c < 6; c++) sacc[c] += Bs[warp][a][c];
            }
            const ptrdiff_t g = elements[l][e];
            const bool interior = xi > 0 && xi < L && yi > 0 && yi < L && zi > 0 && zi < L;
            if (diag3) {
                const T dv[3] = {sacc[0], sacc[3], sacc[5]};
                for (int d = 0; d < 3; d++) {
                    if (interior)
                        diag3[3 * g + d] += dv[d];
                    else
                        atomicAdd(&diag3[3 * g + d], dv[d]);
                }
            }
            if (block6) {
                for (int c = 0; c < 6; c++) {
                    if (interior)
                        block6[6 * g + c] += sacc[c];
                    else
                        atomicAdd(&block6[6 * g + c], sacc[c]);
                }
            }
        }
        __syncwarp();
    }
}

template <typename T>
static int launch_el_cta_views(int L, ptrdiff_t nelements, idx_t **elements, ptrdiff_t stride, const float *adj,
                               const float *det, T mu, T lambda, Comp3<const T *> xv, Comp3<T *> yv, cudaStream_t s) {
    const size_t smem = el_cta_smem_bytes<T>(L);
    if (smem > 227 * 1024)
        return set_error("sfem_gb300_linear_elasticity_apply: level %d needs %zu bytes of shared memory in %s", L,
                         smem, sizeof(T) == 8 ? "FP64" : "FP32");
    static std::atomic<size_t> attr{0};  // largest shared-memory opt-in so far (per T)
    if (smem > 48 * 1024 && smem > attr.load(std::memory_order_relaxed)) {
        cudaFuncSetAttribute(elasticity_apply_cta_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr.store(smem, std::memory_order_relaxed);  // a racing caller at worst repeats the opt-in
    }
    const int grid = (int)std::min<ptrdiff_t>(nelements, (ptrdiff_t)kNumSMs * 8);
    elasticity_apply_cta_kernel<T><<<grid, 256, smem, s>>>(L, nelements, elements, stride, adj, det, mu, lambda, xv, yv);
    return check_launch("sfem_gb300_linear_elasticity_apply(SSHEX8, CTA per element)");
}

template <typename T>
static int launch_el_cta(int L, ptrdiff_t nelements, idx_t **elements, ptrdiff_t stride, const float *adj,
                         const float *det, T mu, T lambda, const T *x, T *y, cudaStream_t s) {
    return launch_el_cta_views<T>(L, nelements, elements, stride, adj, det, mu, lambda,
                                  Comp3<const T *>{{x, x + 1, x + 2}, 3}, Comp3<T *>{{y, y + 1, y + 2}, 3}, s);
}

static int g_elasticity_kernel = -1;  // -1 default (tcgen05 at L = 4), 0 SIMT warp kernel, 1 tcgen05 3xTF32

static int elasticity_apply_tf32x3(ptrdiff_t nelements, idx_t **elements, ptrdiff_t stride, const float *adj,
                                   const float *det, float mu, float lambda, const float *x, float *y, cudaStream_t s) {
    static std::once_flag attr;
    std::call_once(attr, [] {
        cudaFuncSetAttribute(elasticity_apply_tf32x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ETC_SMEM);
    });
    const ptrdiff_t pairs = (nelements + 1) / 2;
    const int grid = (int)std::min<ptrdiff_t>(pairs, (ptrdiff_t)kNumSMs * ETC_CTAS_PER_SM);
    elasticity_apply_tf32x3_kernel<<<grid, 128, ETC_SMEM, s>>>(nelements, elements, stride, adj, det, mu, lambda, x, y);
    return check_launch("sfem_gb300_linear_elasticity_apply(SSHEX8 L=4, tcgen05 3xTF32)");
}

template <typename T>
static int elasticity_apply_tpl(int element_type, ptrdiff_t nelements, idx_t **elements, ptrdiff_t stride,
                                const float *adj, const float *det, T mu, T lambda, const T *x, T *y, cudaStream_t s) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    const int blocks = grid_for((nelements + 1) / 2, 1, kNumSMs * 64);
    if (element_type == SFEM_GB300_HEX8) {
        elasticity_apply_warp_kernel<T, 1, true><<<blocks, 64, 0, s>>>(nelements, elements, stride, adj, det, mu,
                                                                       lambda, x, y);
        return check_launch("sfem_gb300_linear_elasticity_apply(HEX8)");
    }
    const int L = element_type - SFEM_GB300_SSHEX8_BASE;
    if constexpr (sizeof(T) == 4) {
        if (L == 4 && g_elasticity_kernel != 0)
            return elasticity_apply_tf32x3(nelements, elements, stride, adj, det, mu, lambda, x, y, s);
    }
#define SFEM_EL_CASE(LL)                                                                                             \
    case LL:                                                                                                         \
        elasticity_apply_warp_kernel<T, LL, false><<<blocks, 64, 0, s>>>(nelements, elements, stride, adj, det, mu, \
                                                                         lambda, x, y);                              \
        return check_launch("sfem_gb300_linear_elasticity_apply(SSHEX8)");
    switch (L) {
        SFEM_EL_CASE(1)
        SFEM_EL_CASE(2)
        SFEM_EL_CASE(3)
        SFEM_EL_CASE(4)
        default:
            if (L >= 5 && L <= EL_MAX_L)
                return launch_el_cta<T>(L, nelements, elements, stride, adj, det, mu, lambda, x, y, s);
            return set_error("sfem_gb300_linear_elasticity_apply: unsupported element type %d", element_type);
    }
#undef SFEM_EL_CASE
}

template <typename T>
static int elasticity_diag_tpl(int element_type, ptrdiff_t nelements, idx_t **elements, ptrdiff_t stride,
                               const float *adj, const float *det, T mu, T lambda, T *diag3, T *block6, cudaStream_t s) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    const int blocks = grid_for((nelements + 1) / 2, 1, kNumSMs * 64);
    if (element_type == SFEM_GB300_HEX8) {
        elasticity_block_diag_kernel<T, 1, true><<<blocks, 64, 0, s>>>(nelements, elements, stride, adj, det, mu,
                                                                       lambda, diag3, block6);
        return check_launch("sfem_gb300_linear_elasticity_block_diag(HEX8)");
    }
    const int L = element_type - SFEM_GB300_SSHEX8_BASE;
#define SFEM_EL_CASE(LL)                                                                                             \
    case LL:                                                                                                         \
        elasticity_block_diag_kernel<T, LL, false><<<blocks, 64, 0, s>>>(nelements, elements, stride, adj, det, mu, \
                                                                         lambda, diag3, block6);                     \
        return check_launch("sfem_gb300_linear_elasticity_block_diag(SSHEX8)");
    switch (L) {
        SFEM_EL_CASE(1)
        SFEM_EL_CASE(2)
        SFEM_EL_CASE(3)
        SFEM_EL_CASE(4)
        default:
            if (L >= 5 && L <= EL_MAX_L) {
                elasticity_block_diag_any_kernel<T><<<blocks, 64, 0, s>>>(L, nelements, elements, stride, adj, det, mu,
                                                                          lambda, diag3, block6);
                return check_launch("sfem_gb300_linear_elasticity_block_diag(SSHEX8, any level)");
            }
            return set_error("sfem_gb300_linear_elasticity_block_diag: unsupported element type %d", element_type);
    }
#undef SFEM_EL_CASE
}

// position of column `col` in CRS row `row` (sorted columns), -1 if absent
__device__ __forceinline__ idx_t bsr_find_col(const idx_t *rowptr, const idx_t *colidx, idx_t row, idx_t col) {
    idx_t lo = rowptr[row], hi = rowptr[row + 1] - 1;
    while (lo <= hi) {
        const idx_t mid = (lo + hi) >> 1;
        const idx_t c = colidx[mid];
        if (c == col) return mid;
        if (c < col)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    return -1;
}

// Assembly of the hex8 (or one sshex8 micro level's macro) elasticity matrix into a block
// sparse row pattern with 3 x 3 row-major blocks (affine_hex8_linear_elasticity_bsr,
// operators/hex8/hex8_linear_elasticity.hpp:74-110; cu_affine_hex8_linear_elasticity_bsr,
// operators/hex8/cuda/cu_hex8_linear_elasticity.cu:265): one warp per element builds K in
// shared memory, lanes add its 8 x 8 node blocks into the pattern (values +=).
template <typename T>
__global__ void __launch_bounds__(64) elasticity_bsr_kernel(ptrdiff_t nelements, const idx_t *const *elements,
                                                            ptrdiff_t stride, const float *adjugate,
                                                            const float *determinant, T mu, T lambda,
                                                            const idx_t *rowptr, const idx_t *colidx, T *values,
                                                            int *missing) {
    __shared__ T Ws[2][81];
    __shared__ T Ks[2][576];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T Ir[2][9];
    load_grad_regs<T>(lane, Ir);
    for (ptrdiff_t e = (ptrdiff_t)blockIdx.x * 2 + warp; e < nelements; e += (ptrdiff_t)gridDim.x * 2) {
        T adj[9], AA[9], inv_det;
        load_sub_adjugate<T>(adjugate, determinant, stride, e, 1, adj, AA, inv_det);
        build_K_warp_sym<T>(adj, AA, inv_det, mu, lambda, Ir, Ws[warp], Ks[warp], 24, lane);
        for (int ab = lane; ab < 64; ab += 32) {
            const int a = ab >> 3, b = ab & 7;
            const idx_t k = bsr_find_col(rowptr, colidx, elements[a][e], elements[b][e]);
            if (k < 0) {
                atomicAdd(missing, 1);
                continue;
            }
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) atomicAdd(&values[(ptrdiff_t)k * 9 + i * 3 + j], Ks[warp][(i * 8 + a) * 24 + j * 8 + b]);
        }
        __syncwarp();
    }
}

}  // namespace sfem_gb300

using namespace sfem_gb300;

extern "C" int cu_linear_elasticity_bsr(int element_type, ptrdiff_t nelements, idx_t **elements,
                                        ptrdiff_t jacobian_stride, const void *jacobian_adjugate,
                                        const void *jacobian_determinant, double mu, double lambda, int real_type,
                                        const int32_t *rowptr, const int32_t *colidx, void *values, void *stream) {
    if (element_type != SFEM_GB300_HEX8)
        return set_error("cu_linear_elasticity_bsr: element type %d (HEX8 only, as the reference)", element_type);
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    int *missing = nullptr;
    if (cudaMallocAsync((void **)&missing, sizeof(int), s) != cudaSuccess)
        return set_error("cu_linear_elasticity_bsr: allocation failed");
    cudaMemsetAsync(missing, 0, sizeof(int), s);
    const int blocks = grid_for((nelements + 1) / 2, 1, kNumSMs * 32);
    if (real_type == SFEM_GB300_FLOAT32)
        elasticity_bsr_kernel<float><<<blocks, 64, 0, s>>>(nelements, elements, jacobian_stride,
                                                           (const float *)jacobian_adjugate,
                                                           (const float *)jacobian_determinant, (float)mu,
                                                           (float)lambda, rowptr, colidx, (float *)values, missing);
    else if (real_type == SFEM_GB300_FLOAT64 || real_type == SFEM_GB300_REAL_DEFAULT)
        elasticity_bsr_kernel<double><<<blocks, 64, 0, s>>>(nelements, elements, jacobian_stride,
                                                            (const float *)jacobian_adjugate,
                                                            (const float *)jacobian_determinant, mu, lambda, rowptr,
                                                            colidx, (double *)values, missing);
    else {
        cudaFreeAsync(missing, s);
        return set_error("cu_linear_elasticity_bsr: unsupported real type %d", real_type);
    }
    const int lerr = check_launch("cu_linear_elasticity_bsr");
    int h_missing = 0;
    cudaMemcpyAsync(&h_missing, missing, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    cudaFreeAsync(missing, s);
    if (lerr) return SFEM_GB300_FAILURE;
    if (h_missing) return set_error("cu_linear_elasticity_bsr: %d element node pairs missing from the pattern", h_missing);
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_linear_elasticity_apply(int element_type, ptrdiff_t nelements, idx_t **elements,
                                                  ptrdiff_t jacobian_stride, const float *adjugate,
                                                  const float *determinant, double mu, double lambda, int real_type,
                                                  const void *u, void *out, void *stream) {
    const cudaStream_t s = stream_of(stream);
    if (real_type == SFEM_GB300_FLOAT32)
        return elasticity_apply_tpl<float>(element_type, nelements, elements, jacobian_stride, adjugate, determinant,
                                           (float)mu, (float)lambda, (const float *)u, (float *)out, s);
    if (real_type == SFEM_GB300_FLOAT32_BF16TC) {
        if (nelements <= 0) return SFEM_GB300_SUCCESS;
        return elasticity_apply_tc(element_type, nelements, elements, jacobian_stride, adjugate, determinant,
                                   (float)mu, (float)lambda, (const float *)u, (float *)out, s);
    }
    if (real_type == SFEM_GB300_FLOAT64 || real_type == SFEM_GB300_REAL_DEFAULT)
        return elasticity_apply_tpl<double>(element_type, nelements, elements, jacobian_stride, adjugate, determinant,
                                            mu, lambda, (const double *)u, (double *)out, s);
    return set_error("sfem_gb300_linear_elasticity_apply: unsupported real type %d", real_type);
}

template <typename T>
static int elasticity_apply_em_tpl(int element_type, ptrdiff_t nelements, idx_t **elements, const T *K, const T *x,
                                   T *y, cudaStream_t s) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    const int blocks = grid_for((nelements + 1) / 2, 1, kNumSMs * 64);
    if (element_type == SFEM_GB300_HEX8) {
        elasticity_apply_warp_kernel<T, 1, true, true><<<blocks, 64, 0, s>>>(nelements, elements, 0, nullptr, nullptr,
                                                                             T(0), T(0), x, y, K);
        return check_launch("sfem_gb300_linear_elasticity_apply_em(HEX8)");
    }
    const int L = element_type - SFEM_GB300_SSHEX8_BASE;
#define SFEM_EL_EM_CASE(LL)                                                                                      \
    case LL:                                                                                                     \
        elasticity_apply_warp_kernel<T, LL, false, true><<<blocks, 64, 0, s>>>(nelements, elements, 0, nullptr, \
                                                                               nullptr, T(0), T(0), x, y, K);   \
        return check_launch("sfem_gb300_linear_elasticity_apply_em(SSHEX8)");
    switch (L) {
        SFEM_EL_EM_CASE(1)
        SFEM_EL_EM_CASE(2)
        SFEM_EL_EM_CASE(3)
        SFEM_EL_EM_CASE(4)
        default:
            return set_error("sfem_gb300_linear_elasticity_apply_em: unsupported element type %d", element_type);
    }
#undef SFEM_EL_EM_CASE
}

extern "C" int sfem_gb300_linear_elasticity_element_matrices(int element_type, ptrdiff_t nelements,
                                                             ptrdiff_t jacobian_stride, const float *adjugate,
                                                             const float *determinant, double mu, double lambda,
                                                             int real_type, void *K, void *stream) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    const int L = element_type == SFEM_GB300_HEX8 ? 1 : element_type - SFEM_GB300_SSHEX8_BASE;
    if (L < 1 || L > 16)
        return set_error("sfem_gb300_linear_elasticity_element_matrices: unsupported element type %d", element_type);
    const cudaStream_t s = stream_of(stream);
    const int blocks = grid_for((nelements + 1) / 2, 1, kNumSMs * 64);
    if (real_type == SFEM_GB300_FLOAT32)
        elasticity_element_matrices_kernel<float><<<blocks, 64, 0, s>>>(nelements, L, jacobian_stride, adjugate,
                                                                        determinant, (float)mu, (float)lambda,
                                                                        (float *)K);
    else if (real_type == SFEM_GB300_FLOAT64 || real_type == SFEM_GB300_REAL_DEFAULT)
        elasticity_element_matrices_kernel<double><<<blocks, 64, 0, s>>>(nelements, L, jacobian_stride, adjugate,
                                                                         determinant, mu, lambda, (double *)K);
    else
        return set_error("sfem_gb300_linear_elasticity_element_matrices: unsupported real type %d", real_type);
    return check_launch("sfem_gb300_linear_elasticity_element_matrices");
}

extern "C" int sfem_gb300_linear_elasticity_apply_em(int element_type, ptrdiff_t nelements, idx_t **elements,
                                                     const void *K, int real_type, const void *u, void *out,
                                                     void *stream) {
    const cudaStream_t s = stream_of(stream);
    if (real_type == SFEM_GB300_FLOAT32)
        return elasticity_apply_em_tpl<float>(element_type, nelements, elements, (const float *)K, (const float *)u,
                                              (float *)out, s);
    if (real_type == SFEM_GB300_FLOAT64 || real_type == SFEM_GB300_REAL_DEFAULT)
        return elasticity_apply_em_tpl<double>(element_type, nelements, elements, (const double *)K,
                                               (const double *)u, (double *)out, s);
    return set_error("sfem_gb300_linear_elasticity_apply_em: unsupported real type %d", real_type);
}

extern "C" int sfem_gb300_set_elasticity_kernel(int variant) {
    if (variant < -1 || variant > 1) return set_error("sfem_gb300_set_elasticity_kernel: variant %d (-1, 0 or 1)", variant);
    g_elasticity_kernel = variant;
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_elasticity_status(void) {
    int st = 0;
    if (cudaMemcpyFromSymbol(&st, g_etc_status, sizeof(int)) != cudaSuccess) return -1;
    if (st) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_etc_status, &zero, sizeof(int));
    }
    return st;
}

extern "C" int cu_affine_sshex8_linear_elasticity_apply(int level, ptrdiff_t nelements, idx_t **elements,
                                                        ptrdiff_t jacobian_stride, const void *jacobian_adjugate,
                                                        const void *jacobian_determinant, double mu, double lambda,
                                                        int real_type, ptrdiff_t u_stride, const void *ux,
                                                        const void *uy, const void *uz, ptrdiff_t out_stride,
                                                        void *outx, void *outy, void *outz, void *stream) {
    // interleaved xyz vectors (ux = u, uy = u + 1, uz = u + 2, stride 3): the tuned kernels;
    // any other layout (separate component arrays, other strides): the CTA-per-element
    // kernel reading and writing through the component pointers and strides
    const size_t es = (real_type == SFEM_GB300_FLOAT32 || real_type == SFEM_GB300_FLOAT32_BF16TC) ? 4 : 8;
    if (u_stride == 3 && out_stride == 3 && (const char *)uy == (const char *)ux + es &&
        (const char *)uz == (const char *)ux + 2 * es && (char *)outy == (char *)outx + es &&
        (char *)outz == (char *)outx + 2 * es)
        return sfem_gb300_linear_elasticity_apply(SFEM_GB300_SSHEX8(level), nelements, elements, jacobian_stride,
                                                  (const float *)jacobian_adjugate, (const float *)jacobian_determinant,
                                                  mu, lambda, real_type, ux, outx, stream);
    if (level < 1 || level > EL_MAX_L)
        return set_error("cu_affine_sshex8_linear_elasticity_apply: level %d (1..%d)", level, EL_MAX_L);
    if (u_stride < 1 || out_stride < 1)
        return set_error("cu_affine_sshex8_linear_elasticity_apply: strides must be positive");
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    const float *adj = (const float *)jacobian_adjugate, *det = (const float *)jacobian_determinant;
    if (es == 4)
        return launch_el_cta_views<float>(level, nelements, elements, jacobian_stride, adj, det, (float)mu,
                                          (float)lambda,
                                          Comp3<const float *>{{(const float *)ux, (const float *)uy, (const float *)uz},
                                                               u_stride},
                                          Comp3<float *>{{(float *)outx, (float *)outy, (float *)outz}, out_stride}, s);
    if (real_type != SFEM_GB300_FLOAT64 && real_type != SFEM_GB300_REAL_DEFAULT)
        return set_error("cu_affine_sshex8_linear_elasticity_apply: unsupported real type %d", real_type);
    return launch_el_cta_views<double>(
            level, nelements, elements, jacobian_stride, adj, det, mu, lambda,
            Comp3<const double *>{{(const double *)ux, (const double *)uy, (const double *)uz}, u_stride},
            Comp3<double *>{{(double *)outx, (double *)outy, (double *)outz}, out_stride}, s);
}

extern "C" int sfem_gb300_linear_elasticity_block_diag(int element_type, ptrdiff_t nelements, idx_t **elements,
                                                       ptrdiff_t jacobian_stride, const float *adjugate,
                                                       const float *determinant, double mu, double lambda,
                                                       int real_type, void *diag3, void *block6, void *stream) {
    const cudaStream_t s = stream_of(stream);
    if (real_type == SFEM_GB300_FLOAT32)
        return elasticity_diag_tpl<float>(element_type, nelements, elements, jacobian_stride, adjugate, determinant,
                                          (float)mu, (float)lambda, (float *)diag3, (float *)block6, s);
    if (real_type == SFEM_GB300_FLOAT64 || real_type == SFEM_GB300_REAL_DEFAULT)
        return elasticity_diag_tpl<double>(element_type, nelements, elements, jacobian_stride, adjugate, determinant,
                                           mu, lambda, (double *)diag3, (double *)block6, s);
    return set_error("sfem_gb300_linear_elasticity_block_diag: unsupported real type %d", real_type);
}

extern "C" int sfem_gb300_block3_invert(int real_type, ptrdiff_t n_nodes, void *block6, double omega,
                                        ptrdiff_t n_dirichlet, const int32_t *dirichlet_nodes, void *stream) {
    const cudaStream_t s = stream_of(stream);
    if (n_nodes <= 0) return SFEM_GB300_SUCCESS;
    if (real_type == SFEM_GB300_FLOAT32) {
        if (n_dirichlet > 0)
            block_identity_kernel<float><<<grid_for(n_dirichlet, 256), 256, 0, s>>>(n_dirichlet, dirichlet_nodes, (float *)block6);
        block_inverse_kernel<float><<<grid_for(n_nodes, 256), 256, 0, s>>>(n_nodes, (float *)block6, (float)omega);
    } else {
        if (n_dirichlet > 0)
            block_identity_kernel<double><<<grid_for(n_dirichlet, 256), 256, 0, s>>>(n_dirichlet, dirichlet_nodes, (double *)block6);
        block_inverse_kernel<double><<<grid_for(n_nodes, 256), 256, 0, s>>>(n_nodes, (double *)block6, omega);
    }
    return check_launch("sfem_gb300_block3_invert");
}

extern "C" int sfem_gb300_block3_apply(int real_type, ptrdiff_t n_nodes, const void *block6, const void *r, void *x,
                                       void *stream) {
    const cudaStream_t s = stream_of(stream);
    if (n_nodes <= 0) return SFEM_GB300_SUCCESS;
    if (real_type == SFEM_GB300_FLOAT32)
        block_apply_kernel<float><<<grid_for(n_nodes, 256), 256, 0, s>>>(n_nodes, (const float *)block6,
                                                                         (const float *)r, (float *)x);
    else
        block_apply_kernel<double><<<grid_for(n_nodes, 256), 256, 0, s>>>(n_nodes, (const double *)block6,
                                                                          (const double *)r, (double *)x);
    return check_launch("sfem_gb300_block3_apply");
}
