// Learned smoother on sshex8 micro-grid patches (no reference counterpart).
//
// A patch is the 5x5x5 node grid of one L=4 macro element (lidx order,
// x fastest).  The network is three 3x3x3 convolutions with zero padding
// (1 -> C -> C -> 1 channels, ReLU between layers), weights and activations
// stored in BF16, arithmetic in FP32.  Layout: activations channels-last
// [patch][125][C]; weights [co][ci][27] with offset index o = (dz+1)*9+(dy+1)*3+(dx+1).
//
// Kernels: gather (residual -> normalised patches), forward, backward-data,
// backward-weights (FP32 gradient accumulation), MSE gradient, Adam update,
// scatter (patch corrections -> global vector, averaged over shared nodes).
// One CTA owns a batch of patches in a grid-stride loop and keeps the layer's
// weights in shared memory.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "tcgen05.cuh"

namespace sfem_gb300 {

constexpr int PN = 5;           // patch edge (L + 1)
constexpr int PV = PN * PN * PN;  // 125 nodes
constexpr int PP = PN + 2;      // padded edge
constexpr int PPV = PP * PP * PP;  // 343 padded nodes
constexpr int KMAX_C = 16;

__device__ __forceinline__ int pad_index(int v) {
    const int x = v % PN, y = (v / PN) % PN, z = v / (PN * PN);
    return (z + 1) * PP * PP + (y + 1) * PP + (x + 1);
}
__device__ __forceinline__ int off_delta(int o) {
    const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dz = o / 9 - 1;
    return dz * PP * PP + dy * PP + dx;
}

// ---------------------------------------------------------------------------- forward
// out[p][v][co] = act(sum_{ci,o} W[co][ci][o] in[p][v+o][ci])
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) patchconv_forward_kernel(ptrdiff_t P, const __nv_bfloat16 *__restrict__ in,
                                                                const __nv_bfloat16 *__restrict__ W, int relu,
                                                                __nv_bfloat16 *__restrict__ out) {
    extern __shared__ float smem_f[];
    float *w = smem_f;                    // COUT * CIN * 27
    float *xin = smem_f + COUT * CIN * 27;  // PPV * CIN
    for (int k = threadIdx.x; k < COUT * CIN * 27; k += blockDim.x) w[k] = __bfloat162float(W[k]);
    for (ptrdiff_t p = blockIdx.x; p < P; p += gridDim.x) {
        __syncthreads();
        for (int k = threadIdx.x; k < PPV * CIN; k += blockDim.x) xin[k] = 0.f;
        __syncthreads();
        for (int k = threadIdx.x; k < PV * CIN; k += blockDim.x)
            xin[pad_index(k / CIN) * CIN + k % CIN] = __bfloat162float(in[p * PV * CIN + k]);
        __syncthreads();
        const int v = threadIdx.x;
        if (v < PV) {
            float acc[COUT];
#pragma unroll
            for (int co = 0; co < COUT; co++) acc[co] = 0.f;
            const int base = pad_index(v);
#pragma unroll 3
            for (int o = 0; o < 27; o++) {
                const float *xp = &xin[(base + off_delta(o)) * CIN];
                float xv[CIN];
#pragma unroll
                for (int ci = 0; ci < CIN; ci++) xv[ci] = xp[ci];
#pragma unroll
                for (int co = 0; co < COUT; co++)
#pragma unroll
                    for (int ci = 0; ci < CIN; ci++) acc[co] += w[(co * CIN + ci) * 27 + o] * xv[ci];
            }
#pragma unroll
            for (int co = 0; co < COUT; co++) {
                const float a = relu ? fmaxf(acc[co], 0.f) : acc[co];
                out[(p * PV + v) * COUT + co] = __float2bfloat16(a);
            }
        }
    }
}

// ---------------------------------------------------------------------------- backward data
// gin[p][v][ci] = mask(in) * sum_{co,o} W[co][ci][o] gout[p][v-o][co]
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) patchconv_backward_data_kernel(ptrdiff_t P,
                                                                      const __nv_bfloat16 *__restrict__ gout,
                                                                      const __nv_bfloat16 *__restrict__ W,
                                                                      const __nv_bfloat16 *__restrict__ in_act,
                                                                      __nv_bfloat16 *__restrict__ gin) {
    extern __shared__ float smem_f[];
    float *w = smem_f;                  // COUT * CIN * 27
    float *g = smem_f + COUT * CIN * 27;  // PPV * COUT
    for (int k = threadIdx.x; k < COUT * CIN * 27; k += blockDim.x) w[k] = __bfloat162float(W[k]);
    for (ptrdiff_t p = blockIdx.x; p < P; p += gridDim.x) {
        __syncthreads();
        for (int k = threadIdx.x; k < PPV * COUT; k += blockDim.x) g[k] = 0.f;
        __syncthreads();
        for (int k = threadIdx.x; k < PV * COUT; k += blockDim.x)
            g[pad_index(k / COUT) * COUT + k % COUT] = __bfloat162float(gout[p * PV * COUT + k]);
        __syncthreads();
        const int v = threadIdx.x;
        if (v < PV) {
            float acc[CIN];
#pragma unroll
            for (int ci = 0; ci < CIN; ci++) acc[ci] = 0.f;
            const int base = pad_index(v);
#pragma unroll 3
            for (int o = 0; o < 27; o++) {
                const float *gp = &g[(base - off_delta(o)) * COUT];
#pragma unroll
                for (int co = 0; co < COUT; co++) {
                    const float gv = gp[co];
#pragma unroll
                    for (int ci = 0; ci < CIN; ci++) acc[ci] += w[(co * CIN + ci) * 27 + o] * gv;
                }
            }
#pragma unroll
            for (int ci = 0; ci < CIN; ci++) {
                float a = acc[ci];
                if (in_act && __bfloat162float(in_act[(p * PV + v) * CIN + ci]) <= 0.f) a = 0.f;  // ReLU'
                gin[(p * PV + v) * CIN + ci] = __float2bfloat16(a);
            }
        }
    }
}

// ---------------------------------------------------------------------------- backward weights
// dW[co][ci][o] += sum_{p,v} gout[p][v][co] in[p][v+o][ci]   (FP32 accumulation, one atomic per entry per CTA)
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) patchconv_backward_weights_kernel(ptrdiff_t P,
                                                                         const __nv_bfloat16 *__restrict__ gout,
                                                                         const __nv_bfloat16 *__restrict__ in,
                                                                         float *__restrict__ dW) {
    constexpr int NW = COUT * CIN * 27;
    constexpr int PER = (NW + 127) / 128;
    __shared__ float xin[PPV * CIN];
    __shared__ float g[PV * COUT];
    float acc[PER];
#pragma unroll
    for (int j = 0; j < PER; j++) acc[j] = 0.f;
    for (ptrdiff_t p = blockIdx.x; p < P; p += gridDim.x) {
        __syncthreads();
        for (int k = threadIdx.x; k < PPV * CIN; k += blockDim.x) xin[k] = 0.f;
        __syncthreads();
        for (int k = threadIdx.x; k < PV * CIN; k += blockDim.x)
            xin[pad_index(k / CIN) * CIN + k % CIN] = __bfloat162float(in[p * PV * CIN + k]);
        for (int k = threadIdx.x; k < PV * COUT; k += blockDim.x) g[k] = __bfloat162float(gout[p * PV * COUT + k]);
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const int k = threadIdx.x + 128 * j;
            if (k < NW) {
                const int co = k / (CIN * 27), ci = (k / 27) % CIN, o = k % 27;
                const int d = off_delta(o);
                float s = 0.f;
                for (int v = 0; v < PV; v++) s += g[v * COUT + co] * xin[(pad_index(v) + d) * CIN + ci];
                acc[j] += s;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const int k = threadIdx.x + 128 * j;
        if (k < NW) atomicAdd(&dW[k], acc[j]);
    }
}

// ---------------------------------------------------------------------------- data movement

// in[p][v] = s_p^-1 * (scale . r)[elements[v][p]],  s_p = RMS of the patch (0 -> 1)
template <typename T>
__global__ void gather_patches_kernel(ptrdiff_t P, const idx_t *const *elements, const T *__restrict__ r,
                                      const T *__restrict__ scale, __nv_bfloat16 *__restrict__ out,
                                      float *__restrict__ patch_scale) {
    __shared__ float vals[PV];
    __shared__ float red[4];
    for (ptrdiff_t p = blockIdx.x; p < P; p += gridDim.x) {
        float sq = 0.f;
        for (int v = threadIdx.x; v < PV; v += blockDim.x) {
            const idx_t g = elements[v][p];
            float val = (float)r[g];
            if (scale) val *= (float)scale[g];
            vals[v] = val;
            sq += val * val;
        }
        for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
        __syncthreads();
        float tot = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
        float s = sqrtf(tot / PV);
        if (!(s > 0.f)) s = 1.f;
        for (int v = threadIdx.x; v < PV; v += blockDim.x) out[p * PV + v] = __float2bfloat16(vals[v] / s);
        if (threadIdx.x == 0 && patch_scale) patch_scale[p] = s;
        __syncthreads();
    }
}

// x[g] += alpha * s_p * out[p][v] / count[g]
template <typename T>
__global__ void scatter_patches_kernel(ptrdiff_t P, const idx_t *const *elements, const __nv_bfloat16 *__restrict__ in,
                                       const float *__restrict__ patch_scale, const uint16_t *__restrict__ count,
                                       T alpha, T *__restrict__ x) {
    const ptrdiff_t total = P * PV;
    for (ptrdiff_t t = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; t < total; t += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t p = t % P;
        const int v = (int)(t / P);
        const idx_t g = elements[v][p];
        const T val = alpha * (T)(patch_scale[p] * __bfloat162float(in[p * PV + v])) / (T)count[g];
        atomicAdd(&x[g], val);
    }
}

// gy = 2/N (y - target) (BF16 in/out), loss partial sums into *loss (FP32 atomics)
__global__ void mse_grad_kernel(ptrdiff_t n, const __nv_bfloat16 *__restrict__ y, const __nv_bfloat16 *__restrict__ t,
                                __nv_bfloat16 *__restrict__ gy, float *loss) {
    float acc = 0.f;
    const float s = 2.f / (float)n;
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * blockDim.x) {
        const float d = __bfloat162float(y[i]) - __bfloat162float(t[i]);
        gy[i] = __float2bfloat16(s * d);
        acc += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, acc / (float)n);
}

// Adam on FP32 master weights w (mirrored into BF16 wb), moments m, v; step t (1-based)
__global__ void adam_kernel(int n, float *w, const float *g, float *m, float *v, __nv_bfloat16 *wb, float lr,
                            float beta1, float beta2, float eps, int t) {
    const float c1 = 1.f - powf(beta1, (float)t), c2 = 1.f - powf(beta2, (float)t);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        m[i] = beta1 * m[i] + (1.f - beta1) * g[i];
        v[i] = beta2 * v[i] + (1.f - beta2) * g[i] * g[i];
        w[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
        wb[i] = __float2bfloat16(w[i]);
    }
}

// ---------------------------------------------------------------------------- fused inference
// The learned correction of the smoother in one kernel: gather + RMS normalise,
// the three convolutions on the tensor cores (mma.sync m16n8k16, BF16 operands,
// FP32 accumulate, BF16 activations between layers exactly as the layer kernels
// above store them), and the averaged scatter.  One warp per patch; a patch is a
// GEMM with M = 128 positions (125 used), N = 16 channels, K = 27 taps x C_in:
// conv1 K = 32 (27 taps padded), conv2 and conv3 one k-tile of 16 input channels
// per tap.  Activations live in shared memory as [padded position][channel]
// rows of 32 bytes, so a k-tile of A is one ldmatrix.x4 from 16 row addresses.
constexpr int LC_WARPS = 4;
constexpr int LC_ROWS = PPV + 1;  // padded positions + one zero row for unused GEMM rows
constexpr int LC_BF1 = 2 * 2 * 32;   // uint2 fragments: [k-tile][n-tile][lane]
constexpr int LC_BF2 = 27 * 2 * 32;  // [tap][n-tile][lane]
constexpr int LC_BF3 = 27 * 32;      // [tap][lane] (n-tile 0, column 0 only)

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat16 a = __float2bfloat16(lo), b = __float2bfloat16(hi);
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}
__device__ __forceinline__ uint32_t pack_bf16_raw(__nv_bfloat16 a, __nv_bfloat16 b) {
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

__device__ __forceinline__ void mma_bf16_16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};\n"
            : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldmatrix_x4(uint32_t (&a)[4], const void *smem_row) {
    const unsigned addr = (unsigned)__cvta_generic_to_shared(smem_row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3])
                 : "r"(addr));
}

// B fragments of the three layers from the [co][ci][27] BF16 weights.  Fragment of
// lane (g = lane/4, q = lane%4): b0 = (B[2q][g], B[2q+1][g]), b1 = (B[2q+8][g], B[2q+9][g]).
__global__ void learned_fragments_kernel(const __nv_bfloat16 *__restrict__ W1, const __nv_bfloat16 *__restrict__ W2,
                                         const __nv_bfloat16 *__restrict__ W3, uint2 *__restrict__ frag) {
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < LC_BF1 + LC_BF2 + LC_BF3; i += gridDim.x * blockDim.x) {
        const int lane = i % 32, g = lane >> 2, q = lane & 3;
        uint2 f;
        if (i < LC_BF1) {  // conv1: B[k = tap][n = co] = W1[co][0][tap]
            const int j = (i / 32) % 2, kt = i / 64;
            auto w = [&](int k) { const int tap = 16 * kt + k; return tap < 27 ? W1[(8 * j + g) * 27 + tap] : zero; };
            f.x = pack_bf16_raw(w(2 * q), w(2 * q + 1));
            f.y = pack_bf16_raw(w(2 * q + 8), w(2 * q + 9));
        } else if (i < LC_BF1 + LC_BF2) {  // conv2 tap t: B[ci][co] = W2[co][ci][t]
            const int k = i - LC_BF1, j = (k / 32) % 2, t = k / 64;
            auto w = [&](int ci) { return W2[((8 * j + g) * KMAX_C + ci) * 27 + t]; };
            f.x = pack_bf16_raw(w(2 * q), w(2 * q + 1));
            f.y = pack_bf16_raw(w(2 * q + 8), w(2 * q + 9));
        } else {  // conv3 tap t: column 0 = W3[0][ci][t], columns 1..7 zero
            const int t = (i - LC_BF1 - LC_BF2) / 32;
            auto w = [&](int ci) { return g == 0 ? W3[ci * 27 + t] : zero; };
            f.x = pack_bf16_raw(w(2 * q), w(2 * q + 1));
            f.y = pack_bf16_raw(w(2 * q + 8), w(2 * q + 9));
        }
        frag[i] = f;
    }
}

// d[g] += omega * s_p * net(patch_p)[v] / count[g] for every patch p (g = elements[v][p])
template <typename T>
__global__ void __launch_bounds__(32 * LC_WARPS, 2) learned_correction_kernel(
        ptrdiff_t P, const idx_t *const *elements, const T *__restrict__ r, const T *__restrict__ inv_diag,
        const uint2 *__restrict__ frag_g, const uint16_t *__restrict__ count, float omega, T *__restrict__ d) {
    extern __shared__ __align__(16) unsigned char lc_smem[];
    uint2 *frag = reinterpret_cast<uint2 *>(lc_smem);
    __nv_bfloat16 *act = reinterpret_cast<__nv_bfloat16 *>(frag + LC_BF1 + LC_BF2 + LC_BF3);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, q = lane & 3;
    __nv_bfloat16 *a1 = act + (size_t)warp * 2 * LC_ROWS * KMAX_C;  // [LC_ROWS][16]
    __nv_bfloat16 *a2 = a1 + LC_ROWS * KMAX_C;                      // [LC_ROWS][16]
    __nv_bfloat16 *a0 = act + (size_t)LC_WARPS * 2 * LC_ROWS * KMAX_C + warp * (PPV + 1);  // [PPV]
    float *outp = reinterpret_cast<float *>(act + (size_t)LC_WARPS * 2 * LC_ROWS * KMAX_C + LC_WARPS * (PPV + 1)) +
                  warp * 128;
    for (int i = threadIdx.x; i < LC_BF1 + LC_BF2 + LC_BF3; i += blockDim.x) frag[i] = frag_g[i];
    // zero every activation buffer once: the padding rows are never written again
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int i = lane; i < 2 * LC_ROWS * KMAX_C; i += 32) a1[i] = zero;
    for (int i = lane; i < PPV; i += 32) a0[i] = zero;
    __syncthreads();
    const uint2 *bf1 = frag, *bf2 = frag + LC_BF1, *bf3 = frag + LC_BF1 + LC_BF2;
    const ptrdiff_t nwarps = (ptrdiff_t)gridDim.x * LC_WARPS;
    // ldmatrix row of this lane in each m-tile (-1: a GEMM row past the 125 positions)
    const int mrow = (lane >> 3 & 1) * 8 + (lane & 7);
    const int mcol = (lane >> 4) * 8;
    int rowbase[8];
#pragma unroll
    for (int mt = 0; mt < 8; mt++) rowbase[mt] = 16 * mt + mrow < PV ? pad_index(16 * mt + mrow) : -1;
    for (ptrdiff_t p = (ptrdiff_t)blockIdx.x * LC_WARPS + warp; p < P; p += nwarps) {
        // gather D^-1 r, normalise by the patch RMS
        idx_t gv[4];
        float val[4];
        float ss = 0.f;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int v = lane + 32 * k;
            gv[k] = 0;
            val[k] = 0.f;
            if (v < PV) {
                gv[k] = elements[v][p];
                float x = (float)r[gv[k]];
                if (inv_diag) x *= (float)inv_diag[gv[k]];
                val[k] = x;
                ss += x * x;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
        float sc = sqrtf(ss / PV);
        if (!(sc > 0.f)) sc = 1.f;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int v = lane + 32 * k;
            if (v < PV) a0[pad_index(v)] = __float2bfloat16(val[k] / sc);
        }
        __syncwarp();
        // conv1 (1 -> 16), ReLU: A[pos][tap] = a0[pad(pos) + delta(tap)]
#pragma unroll 1
        for (int mt = 0; mt < 8; mt++) {
            float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
            const int r0 = 16 * mt + g, r1 = r0 + 8;
            const int b0 = r0 < PV ? pad_index(r0) : -1, b1 = r1 < PV ? pad_index(r1) : -1;
#pragma unroll
            for (int kt = 0; kt < 2; kt++) {
                auto av = [&](int base, int k) {
                    const int tap = 16 * kt + k;
                    return (base >= 0 && tap < 27) ? a0[base + off_delta(tap)] : zero;
                };
                uint32_t a[4];
                a[0] = pack_bf16_raw(av(b0, 2 * q), av(b0, 2 * q + 1));
                a[1] = pack_bf16_raw(av(b1, 2 * q), av(b1, 2 * q + 1));
                a[2] = pack_bf16_raw(av(b0, 2 * q + 8), av(b0, 2 * q + 9));
                a[3] = pack_bf16_raw(av(b1, 2 * q + 8), av(b1, 2 * q + 9));
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    const uint2 bb = bf1[(kt * 2 + j) * 32 + lane];
                    mma_bf16_16816(acc[j], a, bb.x, bb.y);
                }
            }
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const int co = 8 * j + 2 * q;
                if (b0 >= 0)
                    *reinterpret_cast<uint32_t *>(&a1[b0 * KMAX_C + co]) =
                            pack_bf16(fmaxf(acc[j][0], 0.f), fmaxf(acc[j][1], 0.f));
                if (b1 >= 0)
                    *reinterpret_cast<uint32_t *>(&a1[b1 * KMAX_C + co]) =
                            pack_bf16(fmaxf(acc[j][2], 0.f), fmaxf(acc[j][3], 0.f));
            }
        }
        __syncwarp();
        // conv2 (16 -> 16), ReLU: one k-tile of 16 input channels per tap, taps outer so the
        // B fragments of a tap are loaded once for the 8 m-tiles; all 16 accumulators stay
        // in registers.  Row addresses: this lane's ldmatrix row of m-tile mt is the padded
        // position rowbase[mt] (patch independent) shifted by the tap's compile-time offset.
        {
            float acc[8][2][4];
#pragma unroll
            for (int mt = 0; mt < 8; mt++)
#pragma unroll
                for (int j = 0; j < 2; j++)
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[mt][j][c] = 0.f;
#pragma unroll
            for (int t = 0; t < 27; t++) {
                const uint2 bb0 = bf2[(t * 2 + 0) * 32 + lane], bb1 = bf2[(t * 2 + 1) * 32 + lane];
#pragma unroll
                for (int mt = 0; mt < 8; mt++) {
                    const int row = rowbase[mt] >= 0 ? rowbase[mt] + off_delta(t) : PPV;
                    uint32_t a[4];
                    ldmatrix_x4(a, a1 + row * KMAX_C + mcol);
                    mma_bf16_16816(acc[mt][0], a, bb0.x, bb0.y);
                    mma_bf16_16816(acc[mt][1], a, bb1.x, bb1.y);
                }
            }
#pragma unroll
            for (int mt = 0; mt < 8; mt++) {
                const int r0 = 16 * mt + g, r1 = r0 + 8;
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    const int co = 8 * j + 2 * q;
                    if (r0 < PV)
                        *reinterpret_cast<uint32_t *>(&a2[pad_index(r0) * KMAX_C + co]) =
                                pack_bf16(fmaxf(acc[mt][j][0], 0.f), fmaxf(acc[mt][j][1], 0.f));
                    if (r1 < PV)
                        *reinterpret_cast<uint32_t *>(&a2[pad_index(r1) * KMAX_C + co]) =
                                pack_bf16(fmaxf(acc[mt][j][2], 0.f), fmaxf(acc[mt][j][3], 0.f));
                }
            }
        }
        __syncwarp();
        // conv3 (16 -> 1): output column 0 of an 8-wide n-tile
        {
            float acc[8][4];
#pragma unroll
            for (int mt = 0; mt < 8; mt++)
#pragma unroll
                for (int c = 0; c < 4; c++) acc[mt][c] = 0.f;
#pragma unroll
            for (int t = 0; t < 27; t++) {
                const uint2 bb = bf3[t * 32 + lane];
#pragma unroll
                for (int mt = 0; mt < 8; mt++) {
                    const int row = rowbase[mt] >= 0 ? rowbase[mt] + off_delta(t) : PPV;
                    uint32_t a[4];
                    ldmatrix_x4(a, a2 + row * KMAX_C + mcol);
                    mma_bf16_16816(acc[mt], a, bb.x, bb.y);
                }
            }
            if (q == 0) {  // rounded like the stored activations of the layer kernels
#pragma unroll
                for (int mt = 0; mt < 8; mt++) {
                    outp[16 * mt + g] = __bfloat162float(__float2bfloat16(acc[mt][0]));
                    outp[16 * mt + g + 8] = __bfloat162float(__float2bfloat16(acc[mt][2]));
                }
            }
        }
        __syncwarp();
        // scatter, averaged over the macro elements sharing a node
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int v = lane + 32 * k;
            if (v < PV) {
                const idx_t gg = gv[k];
                const T inc = (T)omega * (T)(sc * outp[v]) / (T)count[gg];
                atomicAdd(&d[gg], inc);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------- tcgen05 inference
// The same fused correction on the 5th-generation tensor cores.  One CTA of eight
// warps owns one patch at a time (four CTAs per SM).  tcgen05.mma (M = 128, K = 16,
// BF16 in, FP32 accumulate in tensor memory) is issued by lane 0 of warps 0..2, and
// the accumulators are read back with tcgen05.ld: warps w and w + 4 share TMEM lanes
// 32 (w % 4) .. + 31 and split the work between them by tile or by column.
//
// The tensor pipe takes about 40 cycles per M = 128, K = 16 MMA whatever N is up to
// N = 32 (measured on GB300), so the layers are arranged for few, wide MMAs:
//   conv1 (1 -> 16):  A = im2col of the padded input (K = 27 taps + 5 zero, two K
//                     steps) for rows q = 57 + i, i < 256 (two M tiles), N = 16.
//   conv2 (16 -> 16): taps grouped by dx: D[r][(dx, co)] = sum_{dy,dz,ci}
//                     act1[r + 7 dy + 49 dz][ci] W2[co][ci][(dx, dy, dz)], N = 48,
//                     nine MMAs per tile (rows r = 56 + i); the A operand of (dy, dz) is
//                     the activation buffer started 7 dy + 49 dz rows later (a descriptor
//                     start-address shift).  out[r] = sum_dx D[r + dx][dx] with warp
//                     shuffles (rows r +- 1 are the neighbouring lanes; the rows at warp
//                     boundaries go through shared memory).
//   conv3 (16 -> 1):  the same grouping with N = 16 (columns dx + 1 = 0, 1, 2 used):
//                     out[r] = D3[r - 1][0] + D3[r][1] + D3[r + 1][2].
// Activations are [channel chunk][padded position][8 BF16] rows of 16 bytes (7^3
// padded grid, zero halo); rows that are halo positions are computed and discarded.
constexpr int TC_Q0 = PP * PP + PP + 1;  // 57: padded index of patch node 0
constexpr int TC_R2 = TC_Q0 - 1;         // first conv2 row (rows r - 1 .. r + 1 of every output)
constexpr int TC_ROWS = 384;             // activation rows: max shifted row 56 + 255 + 56 = 367
constexpr int TC_ACT_CHUNK = TC_ROWS * 16;
constexpr int TC_COL_CHUNK = 256 * 16;
constexpr int TC_B1_BYTES = 2 * 2 * 16 * 16;  // [kstep][chunk][n 16][8] BF16
constexpr int TC_B2_BLOCK = 2 * 48 * 16;      // one (dy, dz): [chunk][n = (dx, co) 48][8]
constexpr int TC_B2_BYTES = 9 * TC_B2_BLOCK;
constexpr int TC_B3_BLOCK = 2 * 16 * 16;       // one (dy, dz): [chunk][n = dx + 1 (3 of 16)][8]
constexpr int TC_B3_BYTES = 9 * TC_B3_BLOCK;
constexpr int TC_OPERAND_BYTES = TC_B1_BYTES + TC_B2_BYTES + TC_B3_BYTES;
constexpr int TC_OFF_B1 = 0, TC_OFF_B2 = TC_B1_BYTES, TC_OFF_B3 = TC_B1_BYTES + TC_B2_BYTES;
constexpr int TC_OFF_ACT1 = TC_OPERAND_BYTES;
constexpr int TC_OFF_COL = TC_OFF_ACT1 + 2 * TC_ACT_CHUNK;  // im2col, then act2
constexpr int TC_OFF_A0 = TC_OFF_COL + 4 * TC_COL_CHUNK;
constexpr int TC_OFF_XB = TC_OFF_A0 + TC_ROWS * 2;  // rows at warp boundaries: [chunk 8][2][16] float
constexpr int TC_OFF_OUT = TC_OFF_XB + 8 * 2 * 16 * 4;  // network output per patch node
constexpr int TC_OFF_RED = TC_OFF_OUT + 128 * 4;
constexpr int TC_SMEM = TC_OFF_RED + 8 * 4;
constexpr int TC_THREADS = 256;
constexpr int TC_CTAS_PER_SM = 4;
constexpr uint32_t TC_TMEM_COLS = 128;  // D1 cols 0..31, D2 32..127, then D3 0..31
constexpr int TC_WAIT_POLLS = 1 << 20;
static_assert((TC_SMEM + 1024 + 1024) * TC_CTAS_PER_SM <= 228 * 1024, "shared memory of the resident CTAs");
static_assert(TC_TMEM_COLS * TC_CTAS_PER_SM <= 512, "tensor memory of the resident CTAs");
static_assert(TC_R2 + 255 + 7 + 49 < TC_ROWS && TC_Q0 + 255 + TC_Q0 < TC_ROWS, "shifted rows stay in the buffers");
static_assert(2 * TC_ACT_CHUNK <= 4 * TC_COL_CHUNK, "act2 aliases the im2col region");

__device__ int g_lc_status;  // nonzero: a tensor-core wait gave up (kernel returned early)

// B operands in the no-swizzle K-major layout from the [co][ci][27] BF16 weights
__global__ void learned_tc_operands_kernel(const __nv_bfloat16 *__restrict__ W1, const __nv_bfloat16 *__restrict__ W2,
                                           const __nv_bfloat16 *__restrict__ W3, __nv_bfloat16 *__restrict__ out) {
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    constexpr int n1 = TC_B1_BYTES / 2, n2 = TC_B2_BYTES / 2, n3 = TC_B3_BYTES / 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n1 + n2 + n3; i += gridDim.x * blockDim.x) {
        if (i < n1) {  // conv1: k = tap = 16 s + 8 c + e, n = co
            const int e = i % 8, n = (i / 8) % 16, c = (i / 128) % 2, st = i / 256;
            const int k = 16 * st + 8 * c + e;
            out[i] = k < 27 ? W1[n * 27 + k] : zero;
        } else if (i < n1 + n2) {  // conv2 (dy, dz) block g: n = 16 (dx + 1) + co, k = ci
            const int j = i - n1;
            const int e = j % 8, n = (j / 8) % 48, c = (j / 384) % 2, g = j / 768;
            const int dxi = n / 16, co = n % 16, dyi = g % 3, dzi = g / 3;
            const int t = dzi * 9 + dyi * 3 + dxi;
            out[i] = W2[(co * KMAX_C + 8 * c + e) * 27 + t];
        } else {  // conv3 (dy, dz) block g: n = dx + 1 (n < 3), k = ci
            const int j = i - n1 - n2;
            const int e = j % 8, n = (j / 8) % 16, c = (j / 128) % 2, g = j / 256;
            const int t = (g / 3) * 9 + (g % 3) * 3 + n;
            out[i] = n < 3 ? W3[(8 * c + e) * 27 + t] : zero;
        }
    }
}

__device__ __forceinline__ bool tc_interior(int q) {
    const int x = q % PP, y = (q / PP) % PP, z = q / (PP * PP);
    return q >= 0 && q < PPV && x >= 1 && x <= PN && y >= 1 && y <= PN && z >= 1 && z <= PN;
}

__device__ __forceinline__ void tc_store_row(unsigned char *act, int q, const float (&v)[16], bool keep) {
#pragma unroll
    for (int c = 0; c < 2; c++) {
        uint4 w = make_uint4(0, 0, 0, 0);
        if (keep) {
            w.x = pack_bf16(fmaxf(v[8 * c + 0], 0.f), fmaxf(v[8 * c + 1], 0.f));
            w.y = pack_bf16(fmaxf(v[8 * c + 2], 0.f), fmaxf(v[8 * c + 3], 0.f));
            w.z = pack_bf16(fmaxf(v[8 * c + 4], 0.f), fmaxf(v[8 * c + 5], 0.f));
            w.w = pack_bf16(fmaxf(v[8 * c + 6], 0.f), fmaxf(v[8 * c + 7], 0.f));
        }
        *reinterpret_cast<uint4 *>(act + c * TC_ACT_CHUNK + q * 16) = w;
    }
}

__device__ __forceinline__ void tc_sync() {
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

// d[g] += omega * s_p * net(patch_p)[v] / count[g] for every patch p (g = elements[v][p])
template <typename T>
__global__ void __launch_bounds__(TC_THREADS, TC_CTAS_PER_SM) learned_correction_tc_kernel(
        ptrdiff_t P, const idx_t *const *elements, const T *__restrict__ r, const T *__restrict__ inv_diag,
        const uint4 *__restrict__ operands, const uint16_t *__restrict__ count, float omega, T *__restrict__ d) {
    extern __shared__ __align__(16) unsigned char tcs[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_holder;
    __shared__ const idx_t *srow[PV];  // connectivity row pointers, loaded once
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wq = warp & 3, grp = warp >> 2;  // TMEM lane quarter, warp group
    __nv_bfloat16 *a0 = reinterpret_cast<__nv_bfloat16 *>(tcs + TC_OFF_A0);
    float *red = reinterpret_cast<float *>(tcs + TC_OFF_RED);
    float *xb = reinterpret_cast<float *>(tcs + TC_OFF_XB);
    float *outp = reinterpret_cast<float *>(tcs + TC_OFF_OUT);
    unsigned char *act1 = tcs + TC_OFF_ACT1, *act2 = tcs + TC_OFF_COL;
    // operands in; activation / im2col / input buffers zeroed (halo rows of act1 and a0 stay zero)
    for (int i = tid; i < TC_OPERAND_BYTES / 16; i += TC_THREADS) reinterpret_cast<uint4 *>(tcs)[i] = operands[i];
    for (int i = TC_OPERAND_BYTES / 16 + tid; i < TC_OFF_XB / 16; i += TC_THREADS)
        reinterpret_cast<uint4 *>(tcs)[i] = make_uint4(0, 0, 0, 0);
    if (tid < PV) srow[tid] = elements[tid];
    if (warp == 0) tc::tmem_alloc(&tmem_holder, TC_TMEM_COLS);
    if (tid == 0) tc::mbar_init(&mbar, 4);  // one arrival from lane 0 of warps 0..3 per layer
    tc::fence_async_smem();
    tc_sync();
    const uint32_t tmem = tmem_holder;
    const uint32_t lane_base = (uint32_t)(32 * wq) << 16;
    const bool committer = lane == 0 && warp < 4;
    constexpr uint32_t id16 = tc::idesc_bf16_f32(128, 16), id48 = tc::idesc_bf16_f32(128, 48);
    // operand descriptors (built where they are issued, to keep registers free)
    auto d_col = [&]() { return tc::sdesc(tc::smem_u32(tcs + TC_OFF_COL), TC_COL_CHUNK, 128); };
    auto d_act1 = [&]() { return tc::sdesc(tc::smem_u32(act1), TC_ACT_CHUNK, 128); };
    auto d_act2 = [&]() { return tc::sdesc(tc::smem_u32(act2), TC_ACT_CHUNK, 128); };
    auto d_b1 = [&]() { return tc::sdesc(tc::smem_u32(tcs + TC_OFF_B1), 256, 128); };
    auto d_b2 = [&]() { return tc::sdesc(tc::smem_u32(tcs + TC_OFF_B2), 48 * 16, 128); };
    auto d_b3 = [&]() { return tc::sdesc(tc::smem_u32(tcs + TC_OFF_B3), 256, 128); };
    uint32_t phase = 0;
    bool ok = true;
    // one thread polls the mbarrier; the others wait at the CTA barrier (no issue slots)
    auto wait_mma = [&]() {
        bool w = true;
        if (warp == 0) w = tc::mbar_wait(&mbar, phase, TC_WAIT_POLLS);
        const bool all = __syncthreads_and(w);
        phase ^= 1;
        tc::fence_after_sync();
        return all;
    };
    // thread v owns patch node v; the next patch's node index is loaded one patch ahead and
    // its residual value after the current patch's first tensor-core wait
    const int v = tid;
    auto load_val = [&](idx_t g) {
        float x = (float)r[g];
        if (inv_diag) x *= (float)inv_diag[g];
        return x;
    };
    idx_t gv_next = 0;
    float val_next = 0.f;
    if ((ptrdiff_t)blockIdx.x < P && v < PV) {
        gv_next = srow[v][blockIdx.x];
        val_next = load_val(gv_next);
    }
    // this thread's rows: conv1 row q1 (tile grp), conv2 row r2 (tile grp, chunk c2 = 4 grp + wq)
    const int q1 = TC_Q0 + 128 * grp + 32 * wq + lane;
    const int c2 = 4 * grp + wq;
    const int r2 = TC_R2 + 32 * c2 + lane;
    const bool in_q1 = tc_interior(q1), in_r2 = tc_interior(r2);
    for (ptrdiff_t p = blockIdx.x; p < P && ok; p += gridDim.x) {
        // D^-1 r of this patch, normalised by the patch RMS
        const idx_t gv = gv_next;
        const float val = val_next;
        const ptrdiff_t pn = p + gridDim.x;
        const bool has_next = pn < P && v < PV;
        if (has_next) gv_next = srow[v][pn];
        float ss = val * val;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
        if (lane == 0) red[warp] = ss;
        __syncthreads();
        float sc = 0.f;
#pragma unroll
        for (int k = 0; k < 8; k++) sc += red[k];
        sc = sqrtf(sc / PV);
        if (!(sc > 0.f)) sc = 1.f;
        if (v < PV) a0[pad_index(v)] = __float2bfloat16(val / sc);
        __syncthreads();
        // conv1 im2col: col[i][k] = a0[TC_Q0 + i + off_delta(k)], k < 27 (row i = tid)
        {
            const int i = tid, q = TC_Q0 + i;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                uint32_t w[4];
#pragma unroll
                for (int e2 = 0; e2 < 4; e2++) {
                    const int k0 = 8 * c + 2 * e2, k1 = k0 + 1;
                    const __nv_bfloat16 lo = k0 < 27 ? a0[q + off_delta(k0)] : __float2bfloat16(0.f);
                    const __nv_bfloat16 hi = k1 < 27 ? a0[q + off_delta(k1)] : __float2bfloat16(0.f);
                    w[e2] = pack_bf16_raw(lo, hi);
                }
                *reinterpret_cast<uint4 *>(tcs + TC_OFF_COL + c * TC_COL_CHUNK + i * 16) =
                        make_uint4(w[0], w[1], w[2], w[3]);
            }
        }
        tc::fence_async_smem();
        tc_sync();
        // conv1: warp h < 2 issues tile h (two K steps into cols 16 h)
        if (committer) {
            if (warp < 2) {
#pragma unroll
                for (int st = 0; st < 2; st++)
                    tc::mma_bf16(tmem + 16 * warp, d_col() + (uint64_t)(2 * st * TC_COL_CHUNK / 16 + warp * 128),
                                 d_b1() + (uint64_t)(32 * st), id16, st > 0);
            }
            tc::commit(&mbar);
        }
        ok = wait_mma();
        if (!ok) break;
        if (has_next) val_next = load_val(gv_next);
        {
            float a[16];
            tc::tmem_ld16(tmem + lane_base + 16 * grp, a);
            if (in_q1) tc_store_row(act1, q1, a, true);
        }
        tc::fence_async_smem();
        tc_sync();
        // conv2: warp h < 2 issues tile h: nine (dy, dz) MMAs of N = 48 into cols 32 + 48 h
        if (committer) {
            if (warp < 2) {
                const uint64_t arow = d_act1() + (uint64_t)(TC_R2 + 128 * warp), b2 = d_b2();
#pragma unroll
                for (int g = 0; g < 9; g++) {
                    const int shift = 7 * (g % 3 - 1) + 49 * (g / 3 - 1);
                    tc::mma_bf16(tmem + 32 + 48 * warp, arow + (uint64_t)(int64_t)shift,
                                 b2 + (uint64_t)(TC_B2_BLOCK / 16 * g), id48, g > 0);
                }
            }
            tc::commit(&mbar);
        }
        ok = wait_mma();
        if (!ok) break;
        {
            // out[r] = D[r - 1][dx = -1] + D[r][dx = 0] + D[r + 1][dx = +1] (16 channels)
            const uint32_t dcol = tmem + lane_base + 32 + 48 * grp;
            float acc[16], t[16];
            tc::tmem_ld16(dcol + 0, t);  // dx = -1 slice of row r2: needed by row r2 + 1
            if (lane == 31)
#pragma unroll
                for (int j = 0; j < 16; j++) xb[(c2 * 2 + 0) * 16 + j] = t[j];
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const float u = __shfl_up_sync(0xffffffffu, t[j], 1);
                acc[j] = lane == 0 ? 0.f : u;
            }
            tc::tmem_ld16(dcol + 32, t);  // dx = +1 slice of row r2: needed by row r2 - 1
            if (lane == 0)
#pragma unroll
                for (int j = 0; j < 16; j++) xb[(c2 * 2 + 1) * 16 + j] = t[j];
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const float u = __shfl_down_sync(0xffffffffu, t[j], 1);
                acc[j] += lane == 31 ? 0.f : u;
            }
            tc::tmem_ld16(dcol + 16, t);  // dx = 0 slice
#pragma unroll
            for (int j = 0; j < 16; j++) acc[j] += t[j];
            __syncthreads();
            if (lane == 0 && c2 > 0)
#pragma unroll
                for (int j = 0; j < 16; j++) acc[j] += xb[((c2 - 1) * 2 + 0) * 16 + j];
            if (lane == 31 && c2 < 7)
#pragma unroll
                for (int j = 0; j < 16; j++) acc[j] += xb[((c2 + 1) * 2 + 1) * 16 + j];
            // act2: every one of its 384 rows is rewritten (the region is shared with the
            // im2col buffer and the conv3 dump): rows 56..311 here, the rest zeroed
            tc_store_row(act2, r2, acc, in_r2);
            if (tid < 128) tc_store_row(act2, tid < TC_R2 ? tid : TC_R2 + 256 + (tid - TC_R2), acc, false);
        }
        tc::fence_async_smem();
        tc_sync();
        // conv3: warp h < 2 issues tile h: nine (dy, dz) MMAs of N = 16 into cols 16 h
        if (committer) {
            if (warp < 2) {
                const uint64_t arow = d_act2() + (uint64_t)(TC_R2 + 128 * warp), b3 = d_b3();
#pragma unroll
                for (int g = 0; g < 9; g++) {
                    const int shift = 7 * (g % 3 - 1) + 49 * (g / 3 - 1);
                    tc::mma_bf16(tmem + 16 * warp, arow + (uint64_t)(int64_t)shift,
                                 b3 + (uint64_t)(TC_B3_BLOCK / 16 * g), id16, g > 0);
                }
            }
            tc::commit(&mbar);
        }
        ok = wait_mma();
        if (!ok) break;
        {
            // out[r] = D3[r - 1][0] + D3[r][1] + D3[r + 1][2]
            float a[4];
            tc::tmem_ld4(tmem + lane_base + 16 * grp, a);
            if (lane == 31) xb[(c2 * 2 + 0) * 16] = a[0];
            if (lane == 0) xb[(c2 * 2 + 1) * 16] = a[2];
            const float um = __shfl_up_sync(0xffffffffu, a[0], 1), up = __shfl_down_sync(0xffffffffu, a[2], 1);
            float o = a[1] + (lane == 0 ? 0.f : um) + (lane == 31 ? 0.f : up);
            __syncthreads();
            if (lane == 0 && c2 > 0) o += xb[((c2 - 1) * 2 + 0) * 16];
            if (lane == 31 && c2 < 7) o += xb[((c2 + 1) * 2 + 1) * 16];
            if (in_r2) {
                const int x = r2 % PP - 1, y = (r2 / PP) % PP - 1, z = r2 / (PP * PP) - 1;
                outp[(z * PN + y) * PN + x] = __bfloat162float(__float2bfloat16(o));  // rounded like the layer kernels
            }
        }
        tc_sync();
        if (v < PV) atomicAdd(&d[gv], (T)omega * (T)(sc * outp[v]) / (T)count[gv]);
        __syncthreads();  // outp and xb are rewritten by the next patch
    }
    if (!ok) {
        if (tid == 0) atomicExch(&g_lc_status, 1);
        // let the MMAs still in flight finish (bounded) before the tensor memory is released
        tc::mbar_wait(&mbar, phase ^ 1, TC_WAIT_POLLS);
    }
    tc_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, TC_TMEM_COLS);
}

static size_t lc_smem_bytes() {
    return sizeof(uint2) * (LC_BF1 + LC_BF2 + LC_BF3) +
           sizeof(__nv_bfloat16) * ((size_t)LC_WARPS * 2 * LC_ROWS * KMAX_C + LC_WARPS * (PPV + 1)) +
           sizeof(float) * LC_WARPS * 128;
}

static int conv_grid(ptrdiff_t P) { return grid_for(P, 1, kNumSMs * 8); }

}  // namespace sfem_gb300

using namespace sfem_gb300;

// dynamic shared memory of the forward / backward-data kernels: weights + padded patch
static size_t pc_smem(int cin, int cout, int padded_channels) {
    return sizeof(float) * (size_t)(cout * cin * 27 + PPV * padded_channels);
}

template <typename F>
static void pc_set_smem(F *kernel, size_t bytes) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

#define SFEM_PC_LAUNCH(KER, CI, CO, SMEM, ...)                     \
    do {                                                           \
        const size_t _b = (SMEM);                                  \
        if (_b > 48 * 1024) pc_set_smem(KER<CI, CO>, _b);          \
        KER<CI, CO><<<conv_grid(P), 128, _b, s>>>(__VA_ARGS__);    \
    } while (0)

#define SFEM_PC_DISPATCH_SMEM(KER, SMEMFN, ...)                                                              \
    do {                                                                                                     \
        if (cin == 1 && cout == KMAX_C)                                                                      \
            SFEM_PC_LAUNCH(KER, 1, KMAX_C, SMEMFN, __VA_ARGS__);                                             \
        else if (cin == KMAX_C && cout == KMAX_C)                                                            \
            SFEM_PC_LAUNCH(KER, KMAX_C, KMAX_C, SMEMFN, __VA_ARGS__);                                        \
        else if (cin == KMAX_C && cout == 1)                                                                 \
            SFEM_PC_LAUNCH(KER, KMAX_C, 1, SMEMFN, __VA_ARGS__);                                             \
        else if (cin == 1 && cout == 1)                                                                      \
            SFEM_PC_LAUNCH(KER, 1, 1, SMEMFN, __VA_ARGS__);                                                  \
        else                                                                                                 \
            return set_error("patchconv: channel pair (%d, %d) not supported (1 or %d)", cin, cout, KMAX_C); \
    } while (0)

extern "C" int sfem_gb300_patchconv_forward(ptrdiff_t P, int cin, int cout, const void *in, const void *W, int relu,
                                            void *out, void *stream) {
    if (P <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    SFEM_PC_DISPATCH_SMEM(patchconv_forward_kernel, pc_smem(cin, cout, cin), P, (const __nv_bfloat16 *)in,
                          (const __nv_bfloat16 *)W, relu, (__nv_bfloat16 *)out);
    return check_launch("sfem_gb300_patchconv_forward");
}

extern "C" int sfem_gb300_patchconv_backward_data(ptrdiff_t P, int cin, int cout, const void *gout, const void *W,
                                                  const void *in_act, void *gin, void *stream) {
    if (P <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    SFEM_PC_DISPATCH_SMEM(patchconv_backward_data_kernel, pc_smem(cin, cout, cout), P, (const __nv_bfloat16 *)gout,
                          (const __nv_bfloat16 *)W, (const __nv_bfloat16 *)in_act, (__nv_bfloat16 *)gin);
    return check_launch("sfem_gb300_patchconv_backward_data");
}

extern "C" int sfem_gb300_patchconv_backward_weights(ptrdiff_t P, int cin, int cout, const void *gout, const void *in,
                                                     float *dW, void *stream) {
    if (P <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    SFEM_PC_DISPATCH_SMEM(patchconv_backward_weights_kernel, 0, P, (const __nv_bfloat16 *)gout,
                          (const __nv_bfloat16 *)in, dW);
    return check_launch("sfem_gb300_patchconv_backward_weights");
}

extern "C" int sfem_gb300_gather_patches(int real_type, ptrdiff_t P, idx_t **elements, const void *r,
                                         const void *scale, void *out_bf16, float *patch_scale, void *stream) {
    if (P <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    if (real_type == SFEM_GB300_FLOAT32)
        gather_patches_kernel<float><<<conv_grid(P), 128, 0, s>>>(P, elements, (const float *)r, (const float *)scale,
                                                                  (__nv_bfloat16 *)out_bf16, patch_scale);
    else
        gather_patches_kernel<double><<<conv_grid(P), 128, 0, s>>>(P, elements, (const double *)r,
                                                                   (const double *)scale, (__nv_bfloat16 *)out_bf16,
                                                                   patch_scale);
    return check_launch("sfem_gb300_gather_patches");
}

extern "C" int sfem_gb300_scatter_patches(int real_type, ptrdiff_t P, idx_t **elements, const void *in_bf16,
                                          const float *patch_scale, const uint16_t *count, double alpha, void *x,
                                          void *stream) {
    if (P <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    const ptrdiff_t total = P * PV;
    if (real_type == SFEM_GB300_FLOAT32)
        scatter_patches_kernel<float><<<grid_for(total, 256, kNumSMs * 32), 256, 0, s>>>(
                P, elements, (const __nv_bfloat16 *)in_bf16, patch_scale, count, (float)alpha, (float *)x);
    else
        scatter_patches_kernel<double><<<grid_for(total, 256, kNumSMs * 32), 256, 0, s>>>(
                P, elements, (const __nv_bfloat16 *)in_bf16, patch_scale, count, alpha, (double *)x);
    return check_launch("sfem_gb300_scatter_patches");
}

extern "C" int sfem_gb300_mse_grad(ptrdiff_t n, const void *y, const void *target, void *gy, float *loss,
                                   void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    mse_grad_kernel<<<grid_for(n, 256, kNumSMs * 8), 256, 0, stream_of(stream)>>>(
            n, (const __nv_bfloat16 *)y, (const __nv_bfloat16 *)target, (__nv_bfloat16 *)gy, loss);
    return check_launch("sfem_gb300_mse_grad");
}

extern "C" int sfem_gb300_adam_step(int n, float *w, const float *g, float *m, float *v, void *w_bf16, float lr,
                                    float beta1, float beta2, float eps, int t, void *stream) {
    if (n <= 0) return SFEM_GB300_SUCCESS;
    adam_kernel<<<grid_for(n, 256, 64), 256, 0, stream_of(stream)>>>(n, w, g, m, v, (__nv_bfloat16 *)w_bf16, lr, beta1,
                                                                      beta2, eps, t);
    return check_launch("sfem_gb300_adam_step");
}

// operand buffer: [mma.sync B fragments][tcgen05 B operands]
static constexpr size_t kLcFragBytes = sizeof(uint2) * (LC_BF1 + LC_BF2 + LC_BF3);
static_assert(kLcFragBytes % 16 == 0, "tensor-core operands start 16-byte aligned");
static int g_learned_kernel = 0;  // 0: tcgen05 (default), 1: mma.sync

extern "C" size_t sfem_gb300_learned_fragments_size(void) { return kLcFragBytes + TC_OPERAND_BYTES; }

extern "C" int sfem_gb300_learned_fragments(const void *W1, const void *W2, const void *W3, void *frag, void *stream) {
    if ((reinterpret_cast<uintptr_t>(frag) & 15) != 0)
        return set_error("sfem_gb300_learned_fragments: operand buffer must be 16-byte aligned");
    const cudaStream_t s = stream_of(stream);
    learned_fragments_kernel<<<(LC_BF1 + LC_BF2 + LC_BF3 + 255) / 256, 256, 0, s>>>(
            (const __nv_bfloat16 *)W1, (const __nv_bfloat16 *)W2, (const __nv_bfloat16 *)W3, (uint2 *)frag);
    learned_tc_operands_kernel<<<(TC_OPERAND_BYTES / 2 + 255) / 256, 256, 0, s>>>(
            (const __nv_bfloat16 *)W1, (const __nv_bfloat16 *)W2, (const __nv_bfloat16 *)W3,
            reinterpret_cast<__nv_bfloat16 *>(static_cast<unsigned char *>(frag) + kLcFragBytes));
    return check_launch("sfem_gb300_learned_fragments");
}

extern "C" int sfem_gb300_set_learned_kernel(int variant) {
    if (variant < 0 || variant > 1) return set_error("sfem_gb300_set_learned_kernel: variant %d (0 or 1)", variant);
    g_learned_kernel = variant;
    return SFEM_GB300_SUCCESS;
}

extern "C" int sfem_gb300_learned_status(void) {
    int st = 0;
    if (cudaMemcpyFromSymbol(&st, g_lc_status, sizeof(int)) != cudaSuccess) return -1;
    if (st) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_lc_status, &zero, sizeof(int));
    }
    return st;
}

extern "C" int sfem_gb300_learned_correction(int real_type, ptrdiff_t P, idx_t **elements, const void *r,
                                             const void *inv_diag, const void *frag, const uint16_t *count,
                                             double omega, void *d, void *stream) {
    if (P <= 0) return SFEM_GB300_SUCCESS;
    const cudaStream_t s = stream_of(stream);
    if (g_learned_kernel == 0) {
        static bool tc_attr[2] = {false, false};
        const int grid = (int)std::min<ptrdiff_t>(P, (ptrdiff_t)kNumSMs * TC_CTAS_PER_SM);
        const uint4 *ops = reinterpret_cast<const uint4 *>(static_cast<const unsigned char *>(frag) + kLcFragBytes);
        if (real_type == SFEM_GB300_FLOAT32) {
            if (!tc_attr[0]) {
                cudaFuncSetAttribute(learned_correction_tc_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     TC_SMEM);
                tc_attr[0] = true;
            }
            learned_correction_tc_kernel<float><<<grid, TC_THREADS, TC_SMEM, s>>>(P, elements, (const float *)r,
                                                                           (const float *)inv_diag, ops, count,
                                                                           (float)omega, (float *)d);
        } else {
            if (!tc_attr[1]) {
                cudaFuncSetAttribute(learned_correction_tc_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     TC_SMEM);
                tc_attr[1] = true;
            }
            learned_correction_tc_kernel<double><<<grid, TC_THREADS, TC_SMEM, s>>>(P, elements, (const double *)r,
                                                                            (const double *)inv_diag, ops, count,
                                                                            (float)omega, (double *)d);
        }
        return check_launch("sfem_gb300_learned_correction");
    }
    const size_t smem = lc_smem_bytes();
    static bool attr[2] = {false, false};
    const int grid = (int)std::min<ptrdiff_t>((P + LC_WARPS - 1) / LC_WARPS, (ptrdiff_t)kNumSMs * 2);
    if (real_type == SFEM_GB300_FLOAT32) {
        if (!attr[0]) {
            cudaFuncSetAttribute(learned_correction_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
            attr[0] = true;
        }
        learned_correction_kernel<float><<<grid, 32 * LC_WARPS, smem, s>>>(
                P, elements, (const float *)r, (const float *)inv_diag, (const uint2 *)frag, count, (float)omega,
                (float *)d);
    } else {
        if (!attr[1]) {
            cudaFuncSetAttribute(learned_correction_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
            attr[1] = true;
        }
        learned_correction_kernel<double><<<grid, 32 * LC_WARPS, smem, s>>>(
                P, elements, (const double *)r, (const double *)inv_diag, (const uint2 *)frag, count, (float)omega,
                (double *)d);
    }
    return check_launch("sfem_gb300_learned_correction");
}
