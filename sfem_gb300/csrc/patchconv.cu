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

#include "common.cuh"

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
