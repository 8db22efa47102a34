// Tiles of 32 consecutive macro elements: asynchronous shared-memory copies and the
// packed per-tile block layout shared by the sshex8 Laplacian kernels.
#pragma once

#include <cstdint>

namespace sfem_gb300 {

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Connectivity and metric repacked once per operator into one contiguous block per
// tile of PK_TILE = 32 consecutive macro elements: [node][el] int32 ids followed by
// [6][el] metric entries as float bits (elements past the end: node 0, metric 0), so
// a CTA fetches its tile's ids and metric with one bulk copy (cp.async.bulk,
// completion counted on an mbarrier) instead of (L+1)^3 row segments from SoA rows.
constexpr int PK_TILE = 32;
constexpr int PK_L = 4;  // the packed element-matrix kernel's level (the stencil kernel also packs L = 3)
__host__ __device__ constexpr int pk_words(int L) { return PK_TILE * ((L + 1) * (L + 1) * (L + 1) + 6); }
// polls of a tile's bulk-copy mbarrier before a kernel gives up and reports it
constexpr int LAP_WAIT_POLLS = 1 << 20;
// polls of the drain after giving up: the copy has to land before the CTA may exit
constexpr int LAP_DRAIN_POLLS = 1 << 26;

}  // namespace sfem_gb300

namespace sfem_gb300 {
// Poll bound of the FIRST wait on a tile's bulk copy: LAP_WAIT_POLLS, unless a test
// lowered it (sfem_gb300_set_tile_wait_polls) to make that wait give up on purpose.
// The drain wait that follows a give-up always keeps LAP_DRAIN_POLLS.
int first_wait_polls();
}  // namespace sfem_gb300

namespace sfem_gb300 {
typedef int32_t idx_t;
// Node-centric sshex8 Laplacian apply (stencil.cu): y += A x for the levels
// sshex8_laplacian_stencil_supported() accepts; `packed` (tile blocks, 16-byte aligned)
// or the SoA connectivity and metric.
bool sshex8_laplacian_stencil_supported(int L);
template <typename T>
int sshex8_laplacian_stencil_apply(int L, ptrdiff_t nelements, const int32_t *packed, idx_t **elements,
                                   ptrdiff_t fff_stride, const float *fff, const T *x, T *y, cudaStream_t s);
// status of the stencil kernels' bulk-copy waits since the last call (read and cleared)
int sshex8_laplacian_stencil_status();
}  // namespace sfem_gb300
