// Allocation-free variant of the deterministic dot product.
//
// Some callers cannot allocate device memory at the point where they need a
// reduction: code that runs while a CUDA graph is being built by someone else's
// capture, code inside a custom memory-pool or arena that forbids cudaMalloc,
// or plugins loaded into a host that owns every allocation.  For them this
// entry point takes only the inputs (x, y) and the output (result) and uses a
// scratch area that lives inside this library: a file-scope __device__ array
// of fixed size, created when the library is loaded onto a GPU and held until
// the process exits.
//
// Limits and sharing rules:
//  * the scratch holds one ticket word and kNoAllocPartials = 1024 partial sums
//    (8.25 KiB per GPU); the reduction grid is capped at that many blocks, and
//    vectors longer than SFEM_GB300_NOALLOC_MAX_N entries are rejected;
//  * every call on a GPU shares the one scratch array, which keeps the last
//    call's contents; the ticket must start at zero and is cleared by the
//    first call on each device and reset by every completed reduction;
//  * calls that overlap on the GPU (different streams, or different host
//    threads without ordering) race on the scratch and must be serialised by
//    the caller;
//  * every call looks up the device address of the scratch in the current
//    context with cudaGetSymbolAddress; the first call that sees an address on a
//    device (the first call there, or the first after a device reset or a change of
//    context) clears the scratch with cudaMemsetAsync; make that first call before
//    any stream capture.
#include <mutex>

#include "blas.cuh"
#include "common.cuh"

namespace sfem_gb300 {

constexpr int kNoAllocPartials = kReduceMaxBlocks;

// [ticket padded to 256 B][kNoAllocPartials doubles]
static __device__ __align__(256) unsigned char g_noalloc_scratch[256 + kNoAllocPartials * sizeof(double)];

template <typename T>
__global__ void __launch_bounds__(kReduceBlock) dot_noalloc_kernel(ptrdiff_t n, const T *__restrict__ x,
                                                                   const T *__restrict__ y, ReduceWorkspace ws,
                                                                   double *result) {
    T acc = 0;
    for (ptrdiff_t i = blockIdx.x * (ptrdiff_t)kReduceBlock + threadIdx.x; i < n; i += (ptrdiff_t)gridDim.x * kReduceBlock)
        acc += x[i] * y[i];
    reduce_epilogue((double)acc, ws, result, 0);
}

// Device address of the scratch in the current device's context, looked up on every call
// with that device current (a host-side lookup, no allocation).  The scratch is cleared
// the first time an address is seen on a device, and again whenever the address changes
// (a new context after cudaDeviceReset, or a different context made current), so a
// stale address from an earlier context is never used.
static int scratch_for_current_device(void **ptr, cudaStream_t s) {
    static std::mutex mu;
    static void *addr[64] = {nullptr};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return set_error("sfem_gb300_dot_noalloc: no current CUDA device");
    void *p = nullptr;
    const cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess || !p)
        return set_error("sfem_gb300_dot_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(err));
    std::lock_guard<std::mutex> lock(mu);
    if (addr[dev] != p) {
        if (cudaMemsetAsync(p, 0, sizeof(g_noalloc_scratch), s) != cudaSuccess)
            return set_error("sfem_gb300_dot_noalloc: clearing the scratch failed");
        addr[dev] = p;
    }
    *ptr = p;
    return SFEM_GB300_SUCCESS;
}

}  // namespace sfem_gb300

using namespace sfem_gb300;

extern "C" int sfem_gb300_dot_noalloc(int real_type, ptrdiff_t n, const void *x, const void *y, double *result,
                                      void *stream) {
    if (n < 0 || n > (ptrdiff_t)SFEM_GB300_NOALLOC_MAX_N)
        return set_error("sfem_gb300_dot_noalloc: n = %td outside [0, %lld]", n, (long long)SFEM_GB300_NOALLOC_MAX_N);
    const cudaStream_t s = stream_of(stream);
    void *scratch = nullptr;
    if (scratch_for_current_device(&scratch, s)) return SFEM_GB300_FAILURE;
    const int grid = reduce_grid(n);
    if (grid > kNoAllocPartials) return set_error("sfem_gb300_dot_noalloc: reduction grid exceeds the scratch");
    const ReduceWorkspace ws = workspace_of(scratch);
    if (real_type == SFEM_GB300_FLOAT32)
        dot_noalloc_kernel<float><<<grid, kReduceBlock, 0, s>>>(n, (const float *)x, (const float *)y, ws, result);
    else if (real_type == SFEM_GB300_FLOAT64 || real_type == SFEM_GB300_REAL_DEFAULT)
        dot_noalloc_kernel<double><<<grid, kReduceBlock, 0, s>>>(n, (const double *)x, (const double *)y, ws, result);
    else
        return set_error("sfem_gb300_dot_noalloc: unsupported real type %d", real_type);
    return check_launch("sfem_gb300_dot_noalloc");
}
