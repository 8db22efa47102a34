// Reduction workspace layout shared by the vector and solver kernels.
#pragma once

#include "common.cuh"

namespace sfem_gb300 {

constexpr int kReduceBlock = 256;
constexpr int kReduceMaxBlocks = 1024;
// [ticket (unsigned, padded to 256 B)] [partials: kReduceMaxBlocks doubles]
constexpr size_t kReduceWorkspaceBytes = 256 + kReduceMaxBlocks * sizeof(double);

struct ReduceWorkspace {
    unsigned *ticket;
    double *partials;
};

inline ReduceWorkspace workspace_of(void *ws) {
    char *base = static_cast<char *>(ws);
    return ReduceWorkspace{reinterpret_cast<unsigned *>(base), reinterpret_cast<double *>(base + 256)};
}

int reduce_grid(ptrdiff_t n);

// Block-level sum of v into partials[blockIdx.x]; the last block combines the
// partials in fixed order and writes *result (optionally sqrt'ed), then resets the ticket.
__device__ __forceinline__ void reduce_epilogue(double v, ReduceWorkspace ws, double *result, int do_sqrt) {
    __shared__ double warp_sums[kReduceBlock / 32];
    __shared__ bool is_last;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_sums[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < kReduceBlock / 32; w++) s += warp_sums[w];
        ws.partials[blockIdx.x] = s;
        __threadfence();
        const unsigned ticket = atomicAdd(ws.ticket, 1u);
        is_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double s = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kReduceBlock) s += ((volatile double *)ws.partials)[b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) warp_sums[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < kReduceBlock / 32; w++) t += warp_sums[w];
        *result = do_sqrt ? sqrt(t) : t;
        *ws.ticket = 0u;
    }
}


}  // namespace sfem_gb300
