// Multigrid transfer between nested sshex8 levels (and the sshex8 -> hex8 step).
//
// Prolongation (sshex8_prolongate, operators/sshex8/sshex8_interpolate.cpp:259-558;
// sshex8_hierarchical_prolongation, :129-237): inside each macro element the
// fine-level values are the trilinear interpolation of the coarse-level values;
// the output is overwritten (shared nodes receive identical values from every
// element: the same face corners are summed in the same order).
//
// Restriction (sshex8_restrict, :633-760; sshex8_hierarchical_restriction, :12-127):
// R = P^T, with the fine input divided by the element-node incidence count
// (sshex8_element_node_incidence_count, :239-257) so that nodes shared by several
// macro elements are counted once; output accumulated with atomics.
//
// One thread per (target node of a macro element, macro element), element index
// fastest so that the SoA connectivity reads elements[v][e] are coalesced.
#include "common.cuh"

namespace sfem_gb300 {

// P: to[gid(e, fine lidx)] = sum_c w_c from[gid(e, coarse corner c)]
// No floating-point division inside the kernels (FP64 division is a long
// instruction sequence on GB300): the 1/s factor comes from the host and the
// incidence counts of nested hex meshes (1, 2, 4, 8) are inverted exactly.
template <typename T>
__device__ __forceinline__ T inv_count(unsigned c) {
    switch (c) {
        case 1:
            return T(1);
        case 2:
            return T(0.5);
        case 4:
            return T(0.25);
        case 8:
            return T(0.125);
        default:
            return T(1) / T(c);
    }
}

template <typename T>
__global__ void prolongate_kernel(ptrdiff_t nelements, int from_level, const idx_t *const *from_elements, int to_level,
                                  const idx_t *const *to_elements, int vec_size, const T *__restrict__ from,
                                  T *__restrict__ to, T inv_s) {
    const int nf = to_level + 1;
    const int s = to_level / from_level;
    const ptrdiff_t total = nelements * (ptrdiff_t)(nf * nf * nf);
    for (ptrdiff_t t = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; t < total; t += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t e = t % nelements;
        const int v = (int)(t / nelements);
        const int xi = v % nf, yi = (v / nf) % nf, zi = v / (nf * nf);
        const int cx = min(xi / s, from_level - 1), cy = min(yi / s, from_level - 1), cz = min(zi / s, from_level - 1);
        const T tx = T(xi - cx * s) * inv_s, ty = T(yi - cy * s) * inv_s, tz = T(zi - cz * s) * inv_s;
        const ptrdiff_t gid = to_elements[v][e];
        T acc[3] = {0, 0, 0};
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const T w = (c8x(c) ? tx : T(1) - tx) * (c8y(c) ? ty : T(1) - ty) * (c8z(c) ? tz : T(1) - tz);
            if (w == T(0)) continue;
            const ptrdiff_t src = from_elements[lidx(from_level, cx + c8x(c), cy + c8y(c), cz + c8z(c))][e];
            for (int d = 0; d < vec_size; d++) acc[d] += w * from[src * vec_size + d];
        }
        for (int d = 0; d < vec_size; d++) to[gid * vec_size + d] = acc[d];
    }
}

// R: to[gid(e, coarse node)] += sum over fine nodes f of this element in the coarse node's
// support of w(f) from[f] / count[f]
template <typename T>
__global__ void restrict_kernel(ptrdiff_t nelements, int from_level, const idx_t *const *from_elements,
                                const uint16_t *__restrict__ count, int to_level, const idx_t *const *to_elements,
                                int vec_size, const T *__restrict__ from, T *__restrict__ to, T inv_s) {
    const int nc = to_level + 1;
    const int s = from_level / to_level;
    const ptrdiff_t total = nelements * (ptrdiff_t)(nc * nc * nc);
    for (ptrdiff_t t = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; t < total; t += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t e = t % nelements;
        const int v = (int)(t / nelements);
        const int X = v % nc, Y = (v / nc) % nc, Z = v / (nc * nc);
        T acc[3] = {0, 0, 0};
        // fine nodes within one coarse cell of (X,Y,Z), inside the macro element.  For a
        // power-of-two ratio the weights (products of k/s and 1/count) are dyadic and exact
        // in float: they are formed in float and only the weighted sum runs in T.
        const int x0 = max(0, (X - 1) * s + 1), x1 = min(from_level, (X + 1) * s - 1);
        const int y0 = max(0, (Y - 1) * s + 1), y1 = min(from_level, (Y + 1) * s - 1);
        const int z0 = max(0, (Z - 1) * s + 1), z1 = min(from_level, (Z + 1) * s - 1);
        const bool dyadic = sizeof(T) == 8 && (s & (s - 1)) == 0;  // float vectors: plain path
        const float inv_sf = 1.0f / (float)s;
        for (int zi = z0; zi <= z1; zi++) {
            const T wz = T(1) - T(abs(zi - Z * s)) * inv_s;
            const float wzf = 1.0f - (float)abs(zi - Z * s) * inv_sf;
            for (int yi = y0; yi <= y1; yi++) {
                const T wy = T(1) - T(abs(yi - Y * s)) * inv_s;
                const float wyf = 1.0f - (float)abs(yi - Y * s) * inv_sf;
                for (int xi = x0; xi <= x1; xi++) {
                    const ptrdiff_t f = from_elements[lidx(from_level, xi, yi, zi)][e];
                    T w;
                    if (dyadic) {
                        const float wxf = 1.0f - (float)abs(xi - X * s) * inv_sf;
                        w = (T)(wxf * wyf * wzf * inv_count<float>(count[f]));
                    } else {
                        const T wx = T(1) - T(abs(xi - X * s)) * inv_s;
                        w = wx * wy * wz * inv_count<T>(count[f]);
                    }
                    for (int d = 0; d < vec_size; d++) acc[d] += w * from[f * vec_size + d];
                }
            }
        }
        const ptrdiff_t gid = to_elements[v][e];
        for (int d = 0; d < vec_size; d++) atomicAdd(&to[gid * vec_size + d], acc[d]);
    }
}

// Factor-2 prolongation (coarse level LC -> fine level 2 LC, the 1 -> 2 and 2 -> 4
// steps) with one thread per macro element: the (LC+1)^3 coarse values of the
// element are loaded once into registers and the (2LC+1)^3 fine values follow from
// compile-time weights (1, 1/2, 1/4, 1/8: each fine node is a coarse node, an edge
// midpoint, a face centre or a cell centre).  Consecutive threads own consecutive
// elements, so every connectivity row read is coalesced.  Same values and
// summation order as the per-(node, element) kernel above.  (The same structure for
// the restriction, 125 fine loads and 27 accumulators per thread, ran slower than
// the per-(coarse node, element) kernel, which keeps the restriction.)
template <int LC>
__host__ __device__ constexpr int fine_lidx2(int x, int y, int z) {
    return (z * (2 * LC + 1) + y) * (2 * LC + 1) + x;
}

template <typename T, int LC>
__global__ void __launch_bounds__(128, LC == 1 ? 4 : 2) prolongate2_kernel(ptrdiff_t nelements, const idx_t *const *from_elements,
                                                          const idx_t *const *to_elements, int vec_size,
                                                          const T *__restrict__ from, T *__restrict__ to) {
    constexpr int NC = LC + 1, NCV = NC * NC * NC;
    constexpr int NF = 2 * LC + 1, NFV = NF * NF * NF;
    __shared__ const idx_t *srow_c[NCV], *srow_f[NFV];
    for (int v = threadIdx.x; v < NCV; v += blockDim.x) srow_c[v] = from_elements[v];
    for (int v = threadIdx.x; v < NFV; v += blockDim.x) srow_f[v] = to_elements[v];
    __syncthreads();
    const ptrdiff_t e = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x;
    if (e >= nelements) return;
    idx_t cid[NCV];
#pragma unroll
    for (int v = 0; v < NCV; v++) cid[v] = __ldg(&srow_c[v][e]);
    for (int d = 0; d < vec_size; d++) {
        T cv[NCV];
#pragma unroll
        for (int v = 0; v < NCV; v++) cv[v] = __ldg(&from[(ptrdiff_t)cid[v] * vec_size + d]);
#pragma unroll
        for (int zi = 0; zi < NF; zi++)
#pragma unroll
            for (int yi = 0; yi < NF; yi++)
#pragma unroll
                for (int xi = 0; xi < NF; xi++) {
                    // the same corner order and weights as the general kernel: w_c = prod of (t or 1-t)
                    const int cx = min(xi / 2, LC - 1), cy = min(yi / 2, LC - 1), cz = min(zi / 2, LC - 1);
                    const T tx = T(xi - 2 * cx) * T(0.5), ty = T(yi - 2 * cy) * T(0.5), tz = T(zi - 2 * cz) * T(0.5);
                    T acc = 0;
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        const T w = (c8x(c) ? tx : T(1) - tx) * (c8y(c) ? ty : T(1) - ty) * (c8z(c) ? tz : T(1) - tz);
                        if (w == T(0)) continue;
                        acc += w * cv[((cz + c8z(c)) * NC + cy + c8y(c)) * NC + cx + c8x(c)];
                    }
                    const ptrdiff_t gid = __ldg(&srow_f[fine_lidx2<LC>(xi, yi, zi)][e]);
                    to[gid * vec_size + d] = acc;
                }
    }
}

__global__ void incidence_count_kernel(ptrdiff_t nelements, int level, const idx_t *const *elements, uint16_t *count) {
    const int n1 = level + 1;
    const ptrdiff_t total = nelements * (ptrdiff_t)(n1 * n1 * n1);
    for (ptrdiff_t t = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; t < total; t += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t e = t % nelements;
        const int v = (int)(t / nelements);
        // 16-bit counter: lock-free compare-and-swap increment (always progresses)
        unsigned short *c = (unsigned short *)(count + elements[v][e]);
        unsigned short old = *c, seen;
        while ((seen = atomicCAS(c, old, (unsigned short)(old + 1))) != old) old = seen;
    }
}

template <typename T>
static int prolongate_tpl(ptrdiff_t nelements, int from_level, idx_t **from_elements, int to_level,
                          idx_t **to_elements, int vec_size, const void *from, void *to, cudaStream_t s) {
    if (to_level == 2 * from_level && (from_level == 1 || from_level == 2)) {
        const int blocks = (int)((nelements + 127) / 128);
        if (from_level == 1)
            prolongate2_kernel<T, 1><<<blocks, 128, 0, s>>>(nelements, from_elements, to_elements, vec_size,
                                                              (const T *)from, (T *)to);
        else
            prolongate2_kernel<T, 2><<<blocks, 128, 0, s>>>(nelements, from_elements, to_elements, vec_size,
                                                              (const T *)from, (T *)to);
        return check_launch("sfem_gb300_sshex8_prolongate (factor 2)");
    }
    const ptrdiff_t total = nelements * (ptrdiff_t)((to_level + 1) * (to_level + 1) * (to_level + 1));
    prolongate_kernel<T><<<grid_for(total, 256, kNumSMs * 32), 256, 0, s>>>(
            nelements, from_level, from_elements, to_level, to_elements, vec_size, (const T *)from, (T *)to,
            (T)(1.0 / (double)(to_level / from_level)));
    return check_launch("sfem_gb300_sshex8_prolongate");
}

template <typename T>
static int restrict_tpl(ptrdiff_t nelements, int from_level, idx_t **from_elements, const uint16_t *count,
                        int to_level, idx_t **to_elements, int vec_size, const void *from, void *to, cudaStream_t s) {
    const ptrdiff_t total = nelements * (ptrdiff_t)((to_level + 1) * (to_level + 1) * (to_level + 1));
    restrict_kernel<T><<<grid_for(total, 256, kNumSMs * 32), 256, 0, s>>>(
            nelements, from_level, from_elements, count, to_level, to_elements, vec_size, (const T *)from, (T *)to,
            (T)(1.0 / (double)(from_level / to_level)));
    return check_launch("sfem_gb300_sshex8_restrict");
}

// y[vec*i + c] = sum_k w[k] x[vec*col[k] + c]: a nested interpolation (or its
// transpose) stored as CSR with double weights; one thread per (row, component).
template <typename T>
__global__ void crs_transfer_kernel(ptrdiff_t nrows, int vec, const idx_t *__restrict__ rowptr,
                                    const idx_t *__restrict__ colidx, const double *__restrict__ w,
                                    const T *__restrict__ x, T *__restrict__ y) {
    const ptrdiff_t total = nrows * vec;
    for (ptrdiff_t t = blockIdx.x * (ptrdiff_t)blockDim.x + threadIdx.x; t < total;
         t += (ptrdiff_t)gridDim.x * blockDim.x) {
        const ptrdiff_t i = t / vec;
        const int c = (int)(t - i * vec);
        double acc = 0;
        for (idx_t k = rowptr[i]; k < rowptr[i + 1]; k++) acc += w[k] * (double)x[(ptrdiff_t)colidx[k] * vec + c];
        y[t] = (T)acc;
    }
}

}  // namespace sfem_gb300

namespace sfem_gb300 {
}  // namespace sfem_gb300

using namespace sfem_gb300;

extern "C" int sfem_gb300_sshex8_prolongate(ptrdiff_t nelements, int from_level, idx_t **from_elements, int to_level,
                                            idx_t **to_elements, int vec_size, int real_type, const void *from,
                                            void *to, void *stream) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    if (from_level < 1 || to_level < from_level || to_level % from_level)
        return set_error("sfem_gb300_sshex8_prolongate: nested levels required (to_level %% from_level == 0), got %d -> %d",
                         from_level, to_level);
    if (vec_size < 1 || vec_size > 3) return set_error("sfem_gb300_sshex8_prolongate: vec_size must be 1..3");
    const cudaStream_t s = stream_of(stream);
    if (real_type == SFEM_GB300_FLOAT32)
        return prolongate_tpl<float>(nelements, from_level, from_elements, to_level, to_elements, vec_size, from, to, s);
    if (real_type == SFEM_GB300_FLOAT64 || real_type == SFEM_GB300_REAL_DEFAULT)
        return prolongate_tpl<double>(nelements, from_level, from_elements, to_level, to_elements, vec_size, from, to, s);
    return set_error("sfem_gb300_sshex8_prolongate: unsupported real type %d", real_type);
}

extern "C" int sfem_gb300_sshex8_restrict(ptrdiff_t nelements, int from_level, idx_t **from_elements,
                                          const uint16_t *from_element_to_node_incidence_count, int to_level,
                                          idx_t **to_elements, int vec_size, int real_type, const void *from, void *to,
                                          void *stream) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    if (to_level < 1 || from_level < to_level || from_level % to_level)
        return set_error("sfem_gb300_sshex8_restrict: nested levels required (from_level %% to_level == 0), got %d -> %d",
                         from_level, to_level);
    if (vec_size < 1 || vec_size > 3) return set_error("sfem_gb300_sshex8_restrict: vec_size must be 1..3");
    const cudaStream_t s = stream_of(stream);
    if (real_type == SFEM_GB300_FLOAT32)
        return restrict_tpl<float>(nelements, from_level, from_elements, from_element_to_node_incidence_count, to_level,
                                   to_elements, vec_size, from, to, s);
    if (real_type == SFEM_GB300_FLOAT64 || real_type == SFEM_GB300_REAL_DEFAULT)
        return restrict_tpl<double>(nelements, from_level, from_elements, from_element_to_node_incidence_count,
                                    to_level, to_elements, vec_size, from, to, s);
    return set_error("sfem_gb300_sshex8_restrict: unsupported real type %d", real_type);
}

extern "C" int sfem_gb300_sshex8_element_node_incidence_count(int level, ptrdiff_t nelements, idx_t **elements,
                                                              uint16_t *count, void *stream) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    const ptrdiff_t total = nelements * (ptrdiff_t)((level + 1) * (level + 1) * (level + 1));
    incidence_count_kernel<<<grid_for(total, 256, kNumSMs * 32), 256, 0, stream_of(stream)>>>(nelements, level,
                                                                                               elements, count);
    return check_launch("sfem_gb300_sshex8_element_node_incidence_count");
}

extern "C" int sfem_gb300_crs_transfer(int real_type, ptrdiff_t nrows, int vec_size, const idx_t *rowptr,
                                       const idx_t *colidx, const double *weights, const void *x, void *y,
                                       void *stream) {
    if (nrows <= 0) return SFEM_GB300_SUCCESS;
    if (vec_size < 1) return set_error("sfem_gb300_crs_transfer: vec_size must be >= 1");
    const cudaStream_t s = stream_of(stream);
    const int blocks = grid_for(nrows * vec_size, 256, kNumSMs * 16);
    if (real_type == SFEM_GB300_FLOAT32)
        crs_transfer_kernel<float><<<blocks, 256, 0, s>>>(nrows, vec_size, rowptr, colidx, weights, (const float *)x,
                                                          (float *)y);
    else
        crs_transfer_kernel<double><<<blocks, 256, 0, s>>>(nrows, vec_size, rowptr, colidx, weights,
                                                           (const double *)x, (double *)y);
    return check_launch("sfem_gb300_crs_transfer");
}
