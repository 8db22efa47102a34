// Node-centric (stencil) form of the affine sshex8 Laplacian apply, sm_103a.
//
// Reference: affine_sshex8_laplacian_stencil_apply_fff (operators/sshex8/sshex8_laplacian.cpp:698-769),
// the reference's CPU default (operators/laplacian.cpp:195-205): per macro element the
// 27-point stencil of the micro element matrix at the nodes inside the macro element
// (sshex8_stencil, operators/stencil/stencil3.hpp:167) and partial stencils at its
// surface nodes (sshex8_surface_stencil, operators/stencil/sshex8_skeleton_stencil.hpp:1683).
//
// Every output value is computed once, by one thread, as a gather over its (at most 27)
// neighbours inside the macro element: no shared-memory accumulation and no element
// matrix.  At L = 4 a macro element costs 2,197 FMA (27 x 27 inside, 54 x 18 on faces,
// 36 x 12 on edges, 8 x 8 at corners) against 4,096 for the micro element-matrix form.
//
// Stencil coefficients.  With one metric G (the sub-FFF, 6 entries) per macro element the
// micro element matrix is A = sum_pq G_pq int d_p phi_i d_q phi_j, each term a product of
// one-dimensional integrals.  The coefficient coupling node i to node i + d is the sum of
// A over the micro elements of this macro element that contain both nodes, which
// factorises per axis: per axis the node is on the low face (LO), inside (MID) or on the
// high face (HI) of the macro element, and the assembled 1D integral over the micro
// intervals containing both i and i + delta is a compile-time constant of (class, delta).
// So every coefficient is sum_m g_m W_m(class, d) with compile-time weights W.
//
// Thread mapping.  A CTA takes a tile of 32 consecutive macro elements (lane = element,
// so every shared-memory access of a warp is conflict-free: [node][element] layout) and
// four warps split the (L+1)^2 node columns (ix, iy); a warp walks each of its columns in
// z with a three-plane register window and scatters every finished value with one
// atomic add (a value inside the macro element has no other contributor, so the atomic
// only serves the surface).  A warp handles columns of one class at a time, so its
// coefficients are built once per class in registers.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <mutex>

#include "common.cuh"
#include "tcgen05.cuh"
#include "tiles.cuh"

namespace sfem_gb300 {
namespace stencil {

enum : int { LO = 0, MID = 1, HI = 2 };

// int_0^1 of (test, trial) factor type t for linear basis psi_0 = 1 - s, psi_1 = s:
// t = 0 mass psi_a psi_b, 1 stiffness psi'_a psi'_b, 2 psi'_a psi_b, 3 psi_a psi'_b
__host__ __device__ constexpr double q1_1d(int t, int a, int b) {
    return t == 0 ? (a == b ? 1.0 / 3.0 : 1.0 / 6.0)
           : t == 1 ? (a == b ? 1.0 : -1.0)
           : t == 2 ? (a ? 0.5 : -0.5)
                    : (b ? 0.5 : -0.5);
}

// the same integral summed over the micro intervals of the macro element that contain
// node i (class cls) and node i + delta: the right interval [i, i+1] (node i is its
// local 0) exists unless i is on the high face, the left one [i-1, i] unless on the low face
__host__ __device__ constexpr double q1_1d_assembled(int t, int cls, int delta) {
    return delta == 1    ? (cls != HI ? q1_1d(t, 0, 1) : 0.0)
           : delta == -1 ? (cls != LO ? q1_1d(t, 1, 0) : 0.0)
                         : (cls != LO ? q1_1d(t, 1, 1) : 0.0) + (cls != HI ? q1_1d(t, 0, 0) : 0.0);
}

// factor type on `axis` of the term int d_p phi_i d_q phi_j
__host__ __device__ constexpr int factor_type(int axis, int p, int q) {
    return (axis == p && axis == q) ? 1 : axis == p ? 2 : axis == q ? 3 : 0;
}

__host__ __device__ constexpr double pq_product(int p, int q, int cx, int cy, int cz, int dx, int dy, int dz) {
    return q1_1d_assembled(factor_type(0, p, q), cx, dx) * q1_1d_assembled(factor_type(1, p, q), cy, dy) *
           q1_1d_assembled(factor_type(2, p, q), cz, dz);
}

// weight of metric entry m (00, 01, 02, 11, 12, 22) in the coefficient of offset d at a
// node of class (cx, cy, cz); off-diagonal entries stand for G_pq and G_qp
__host__ __device__ constexpr double weight(int m, int cx, int cy, int cz, int dx, int dy, int dz) {
    return m == 0   ? pq_product(0, 0, cx, cy, cz, dx, dy, dz)
           : m == 1 ? pq_product(0, 1, cx, cy, cz, dx, dy, dz) + pq_product(1, 0, cx, cy, cz, dx, dy, dz)
           : m == 2 ? pq_product(0, 2, cx, cy, cz, dx, dy, dz) + pq_product(2, 0, cx, cy, cz, dx, dy, dz)
           : m == 3 ? pq_product(1, 1, cx, cy, cz, dx, dy, dz)
           : m == 4 ? pq_product(1, 2, cx, cy, cz, dx, dy, dz) + pq_product(2, 1, cx, cy, cz, dx, dy, dz)
                    : pq_product(2, 2, cx, cy, cz, dx, dy, dz);
}

// a neighbour at offset d along an axis exists inside the macro element
__host__ __device__ constexpr bool offset_ok(int cls, int d) { return d > 0 ? cls != HI : d < 0 ? cls != LO : true; }

// What one lane holds: the value of one macro element and its node-id type.  (Two
// elements per lane with packed FP32x2 arithmetic and 8-byte shared loads was built
// and measured slower: 63.8 against 45.6 us on the 48^3 L = 4 mesh -- more
// instructions for the packed pairs, 148 registers, 12 warps per SM.)
template <typename V>
struct Lanes;
template <>
struct Lanes<float> {
    using S = float;
    using I = int32_t;
    static __device__ __forceinline__ float zero() { return 0.f; }
    static __device__ __forceinline__ float splat(double w) { return (float)w; }
    static __device__ __forceinline__ float fma(float a, float b, float c) { return fmaf(a, b, c); }
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float scale(float a, float h) { return a * h; }
    static __device__ __forceinline__ void scatter(float *y, I id, float v, unsigned valid) {
        if (valid & 1u) atomicAdd(y + id, v);
    }
};
template <>
struct Lanes<double> {
    using S = double;
    using I = int32_t;
    static __device__ __forceinline__ double zero() { return 0.0; }
    static __device__ __forceinline__ double splat(double w) { return w; }
    static __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
    static __device__ __forceinline__ double add(double a, double b) { return a + b; }
    static __device__ __forceinline__ void scatter(double *y, I id, double v, unsigned valid) {
        if (valid & 1u) atomicAdd(y + id, v);
    }
};
// The affine micro element matrix A (hex8 corner order) is symmetric and invariant
// under the point reflection xi -> 1 - xi (corner c -> pi(c) = (0 6)(1 7)(2 4)(3 5):
// A[pi k][pi j] = A[k][j]), so its 64 entries take 20 distinct values.  Each warp builds
// five of them per element from the sub-metric (compile-time Q1 weights), the CTA shares
// them in shared memory, and a stencil coefficient is the sum of the entries A[k][k+d]
// over the micro elements of this macro element containing both nodes: 530 operations
// per tile and lane for all node classes instead of 1,042 with every coefficient
// expanded in the six metric entries.
__host__ __device__ constexpr int reflect8(int c) {
    return c == 0 ? 6 : c == 1 ? 7 : c == 2 ? 4 : c == 3 ? 5 : c == 4 ? 2 : c == 5 ? 3 : c == 6 ? 0 : 1;
}
__host__ __device__ constexpr int min2(int a, int b) { return a < b ? a : b; }
__host__ __device__ constexpr int canon_key(int k, int j) {
    return min2(min2(k * 8 + j, j * 8 + k), min2(reflect8(k) * 8 + reflect8(j), reflect8(j) * 8 + reflect8(k)));
}
constexpr int kUnique = 20;
struct UniqueEntries {
    int of[64];   // unique index of entry (k, j)
    int rep[kUnique];  // key k * 8 + j of a representative of each unique index
    constexpr UniqueEntries() : of(), rep() {
        int n = 0;
        for (int key = 0; key < 64; key++) {
            if (canon_key(key / 8, key % 8) != key) continue;
            rep[n] = key;
            for (int q = 0; q < 64; q++)
                if (canon_key(q / 8, q % 8) == key) of[q] = n;
            n++;
        }
    }
};
static_assert(UniqueEntries().rep[kUnique - 1] > 0, "20 distinct entries");
static_assert(kUnique == 5 * 4, "five entries for each of the four warps");

__host__ __device__ constexpr int corner_of(int x, int y, int z) { return z * 4 + (y ? (x ? 2 : 3) : (x ? 1 : 0)); }

// unique index of A[k][k + d] for corner k, or -1 when that micro element of a node of
// class (cx, cy, cz) is outside the macro element or k + d is not one of its corners
__host__ __device__ constexpr int stencil_term(int k, int cx, int cy, int cz, int dx, int dy, int dz) {
    const int c[3] = {c8x(k), c8y(k), c8z(k)}, cl[3] = {cx, cy, cz}, d[3] = {dx, dy, dz};
    int jj[3] = {0, 0, 0};
    for (int ax = 0; ax < 3; ax++) {
        jj[ax] = c[ax] + d[ax];
        if (jj[ax] < 0 || jj[ax] > 1) return -1;
        if ((cl[ax] == LO && c[ax] != 0) || (cl[ax] == HI && c[ax] != 1)) return -1;
    }
    constexpr UniqueEntries t{};
    return t.of[k * 8 + corner_of(jj[0], jj[1], jj[2])];
}

// the coefficient from the shared entries a[u * NS] (u = unique index)
template <typename V, int NS>
__device__ __forceinline__ V coefficient(const V *__restrict__ a, int cx, int cy, int cz, int dx, int dy, int dz) {
    V c = Lanes<V>::zero();
    bool first = true;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int u = stencil_term(k, cx, cy, cz, dx, dy, dz);
        if (u < 0) continue;
        c = first ? a[u * NS] : Lanes<V>::add(c, a[u * NS]);
        first = false;
    }
    return c;
}

// unique entry U of the micro element matrix from the sub-metric g
template <typename V, int U>
__device__ __forceinline__ V unique_entry(const V (&g)[6]) {
    constexpr int key = UniqueEntries().rep[U];
    V c = Lanes<V>::zero();
#pragma unroll
    for (int m = 0; m < 6; m++) {
        const double w = lap_weight(key / 8, key % 8, m);
        if (w != 0.0) c = Lanes<V>::fma(g[m], Lanes<V>::splat(w), c);
    }
    return c;
}

// warp W's share of the entries: U = W, W + 4, ... into a[U * NS]
template <typename V, int NS, int W>
__device__ __forceinline__ void store_entries(const V (&g)[6], V *a) {
    a[W * NS] = unique_entry<V, W>(g);
    a[(W + 4) * NS] = unique_entry<V, W + 4>(g);
    a[(W + 8) * NS] = unique_entry<V, W + 8>(g);
    a[(W + 12) * NS] = unique_entry<V, W + 12>(g);
    a[(W + 16) * NS] = unique_entry<V, W + 16>(g);
}

template <typename T>
__device__ __forceinline__ void cp_async_val(T *smem, const T *gmem);
template <>
__device__ __forceinline__ void cp_async_val<float>(float *smem, const float *gmem) {
    cp_async4(smem, gmem);
}
template <>
__device__ __forceinline__ void cp_async_val<double>(double *smem, const double *gmem) {
    cp_async8(smem, gmem);
}

// the valid (dy, dx) neighbours of plane z of the column at `col` into w[dy+1][dx+1];
// consecutive nodes are NS values apart
template <typename V, int L, int NS, int CX, int CY>
__device__ __forceinline__ void load_plane(V (&w)[3][3], const V *__restrict__ col, int z) {
    constexpr int N1 = L + 1, NP = N1 * N1;
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++)
            if (offset_ok(CY, j - 1) && offset_ok(CX, i - 1)) w[j][i] = col[(z * NP + (j - 1) * N1 + (i - 1)) * NS];
}

// Columns [c0, c1) of class (CX, CY) for this lane's macro element(s).  Columns of a
// class are numbered x fastest over the MID positions 1..L-1.  sx and sidx point at the
// lane's values / ids of node 0; node v is v * NS further.
template <typename V, int L, int NS, int CX, int CY>
__device__ __forceinline__ void columns(const V *__restrict__ sx, const typename Lanes<V>::I *__restrict__ sidx,
                                        const V *__restrict__ sa, int c0, int c1, unsigned valid,
                                        typename Lanes<V>::S *__restrict__ y) {
    using Op = Lanes<V>;
    constexpr int N1 = L + 1, NP = N1 * N1;
    // coefficients of the low (dz = 0, +1) and high (dz = -1, 0) z classes; a node inside
    // in z takes dz = +1 from the low class, dz = -1 from the high class and the sum of
    // both for dz = 0 (the assembled 1D integrals add up the same way)
    V clo[3][3][2], chi[3][3][2], cmid[3][3];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
            if (!(offset_ok(CY, j - 1) && offset_ok(CX, i - 1))) continue;
            clo[j][i][0] = coefficient<V, NS>(sa, CX, CY, LO, i - 1, j - 1, 0);
            clo[j][i][1] = coefficient<V, NS>(sa, CX, CY, LO, i - 1, j - 1, 1);
            chi[j][i][0] = coefficient<V, NS>(sa, CX, CY, HI, i - 1, j - 1, -1);
            chi[j][i][1] = coefficient<V, NS>(sa, CX, CY, HI, i - 1, j - 1, 0);
            cmid[j][i] = Op::add(clo[j][i][0], chi[j][i][1]);
        }
    // kept as a loop: unrolling the columns (every shared-memory address a fixed offset)
    // raised the FP32 kernel to 80 registers and 58 us against 47 us on the 48^3 L = 4 mesh
#pragma unroll 1
    for (int c = c0; c < c1; c++) {
        const int ix = CX == LO ? 0 : CX == HI ? L : (CY == MID ? 1 + c % (L - 1) : 1 + c);
        const int iy = CY == LO ? 0 : CY == HI ? L : (CX == MID ? 1 + c / (L - 1) : 1 + c);
        const V *col = sx + (iy * N1 + ix) * NS;
        const typename Op::I *icol = sidx + (iy * N1 + ix) * NS;
        V w[3][3][3];
        load_plane<V, L, NS, CX, CY>(w[1], col, 0);
        load_plane<V, L, NS, CX, CY>(w[2], col, 1);
#pragma unroll
        for (int iz = 0; iz <= L; iz++) {
            V a0 = Op::zero(), a1 = Op::zero(), a2 = Op::zero();
#pragma unroll
            for (int j = 0; j < 3; j++)
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    if (!(offset_ok(CY, j - 1) && offset_ok(CX, i - 1))) continue;
                    if (iz > 0) a0 = Op::fma(chi[j][i][0], w[0][j][i], a0);
                    a1 = Op::fma(iz == 0 ? clo[j][i][0] : iz == L ? chi[j][i][1] : cmid[j][i], w[1][j][i], a1);
                    if (iz < L) a2 = Op::fma(clo[j][i][1], w[2][j][i], a2);
                }
            const V v = Op::add(Op::add(a0, a1), a2);
            if (valid) Op::scatter(y, icol[iz * NP * NS], v, valid);
            if (iz < L) {
#pragma unroll
                for (int j = 0; j < 3; j++)
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        w[0][j][i] = w[1][j][i];
                        w[1][j][i] = w[2][j][i];
                    }
                if (iz + 2 <= L) load_plane<V, L, NS, CX, CY>(w[2], col, iz + 2);
            }
        }
    }
}

// The four warps' column schedule: two warps split the inside columns, two take the
// face, edge and corner columns.
template <typename V, int L, int NS>
__device__ __forceinline__ void all_columns(int warp, const V *sx, const typename Lanes<V>::I *sidx, const V *sa,
                                            unsigned valid, typename Lanes<V>::S *y) {
    constexpr int NIN = (L - 1) * (L - 1);
    constexpr int HALF = (NIN + 1) / 2;
    if constexpr (L == 2) {
        // nine columns of one node class each: 2 / 2 / 2 / 3 per warp
        switch (warp) {
            case 0:
                columns<V, L, NS, MID, MID>(sx, sidx, sa, 0, 1, valid, y);
                columns<V, L, NS, LO, LO>(sx, sidx, sa, 0, 1, valid, y);
                break;
            case 1:
                columns<V, L, NS, LO, MID>(sx, sidx, sa, 0, 1, valid, y);
                columns<V, L, NS, HI, MID>(sx, sidx, sa, 0, 1, valid, y);
                break;
            case 2:
                columns<V, L, NS, MID, LO>(sx, sidx, sa, 0, 1, valid, y);
                columns<V, L, NS, MID, HI>(sx, sidx, sa, 0, 1, valid, y);
                break;
            default:
                columns<V, L, NS, HI, LO>(sx, sidx, sa, 0, 1, valid, y);
                columns<V, L, NS, LO, HI>(sx, sidx, sa, 0, 1, valid, y);
                columns<V, L, NS, HI, HI>(sx, sidx, sa, 0, 1, valid, y);
                break;
        }
        return;
    }
    switch (warp) {
        case 0:
            columns<V, L, NS, MID, MID>(sx, sidx, sa, 0, HALF, valid, y);
            break;
        case 1:
            columns<V, L, NS, MID, MID>(sx, sidx, sa, HALF, NIN, valid, y);
            break;
        case 2:
            columns<V, L, NS, LO, MID>(sx, sidx, sa, 0, L - 1, valid, y);
            columns<V, L, NS, HI, MID>(sx, sidx, sa, 0, L - 1, valid, y);
            columns<V, L, NS, LO, LO>(sx, sidx, sa, 0, 1, valid, y);
            columns<V, L, NS, HI, LO>(sx, sidx, sa, 0, 1, valid, y);
            break;
        default:
            columns<V, L, NS, MID, LO>(sx, sidx, sa, 0, L - 1, valid, y);
            columns<V, L, NS, MID, HI>(sx, sidx, sa, 0, L - 1, valid, y);
            columns<V, L, NS, LO, HI>(sx, sidx, sa, 0, 1, valid, y);
            columns<V, L, NS, HI, HI>(sx, sidx, sa, 0, 1, valid, y);
            break;
    }
}

constexpr int kWarps = 4;
constexpr int kThreads = 32 * kWarps;

// Shared memory of a tile: the ids [node][el] and metric [6][el] (the packed block
// layout), then x [node][el], then the 20 distinct element-matrix entries [u][el].
template <typename T, int L>
__host__ __device__ constexpr size_t smem_bytes() {
    return (size_t)pk_words(L) * 4 + ((size_t)(L + 1) * (L + 1) * (L + 1) + kUnique) * PK_TILE * sizeof(T);
}

__device__ int g_status;  // nonzero: a bulk-copy wait gave up (2: its drain gave up too)

// One CTA per tile of PK_TILE macro elements.  PACKED: ids and metric come as one bulk
// copy of the tile's packed block; otherwise from the SoA rows elements[v][e] and the SoA
// metric fff[m * fff_stride + e].
template <typename T, int L, bool PACKED>
__global__ void __launch_bounds__(kThreads) sshex8_laplacian_stencil_kernel(
        ptrdiff_t nelements, const int32_t *__restrict__ packed, const idx_t *const *elements, ptrdiff_t fff_stride,
        const float *__restrict__ fff, const T *__restrict__ x, T *__restrict__ y, int first_polls) {
    constexpr int TILE = PK_TILE;
    constexpr int N1 = L + 1;
    constexpr int NXE = N1 * N1 * N1;
    constexpr int WORDS = pk_words(L);
    static_assert(WORDS * 4 % 16 == 0, "a tile's bulk copy is a whole number of 16-byte units");
    extern __shared__ __align__(128) unsigned char st_smem[];
    __shared__ __align__(8) uint64_t mbar;
    int32_t *sidx = reinterpret_cast<int32_t *>(st_smem);
    const float *smet = reinterpret_cast<const float *>(sidx + NXE * TILE);
    T *sx = reinterpret_cast<T *>(st_smem + (size_t)WORDS * 4);
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const ptrdiff_t t = blockIdx.x;
    const ptrdiff_t e0 = t * TILE;
    const int nvalid = (int)((nelements - e0) < TILE ? (nelements - e0) : TILE);
    const bool valid = lane < nvalid;
    T g[6];
    const T h = T(1) / T(L);
    if (PACKED) {
        if (tid == 0) {
            tc::mbar_init(&mbar, 1);
            tc::mbar_arrive_expect_tx(&mbar, WORDS * 4);
            tc::bulk_load(st_smem, packed + t * WORDS, WORDS * 4, &mbar);
        }
        __syncthreads();
        if (!__syncthreads_and(tc::mbar_wait(&mbar, 0, first_polls))) {
            // leave no copy in flight into this CTA's shared memory
            if (tid == 0) {
                atomicExch(&g_status, 1);
                if (!tc::mbar_wait(&mbar, 0, LAP_DRAIN_POLLS)) atomicExch(&g_status, 2);
            }
            return;
        }
#pragma unroll
        for (int m = 0; m < 6; m++) g[m] = valid ? (T)smet[m * TILE + lane] * h : T(0);
    } else {
        __shared__ const idx_t *srow[NXE];
        for (int v = tid; v < NXE; v += kThreads) srow[v] = elements[v];
        __syncthreads();
        constexpr int Q = TILE / 4;  // 16-byte chunks per row segment
        for (int k = tid; k < NXE * Q; k += kThreads) {
            const int v = k / Q, q = k % Q;
            const idx_t *row = srow[v] + e0;
            if (nvalid == TILE && ((reinterpret_cast<uintptr_t>(row) & 15) == 0)) {
                cp_async16(&sidx[v * TILE + 4 * q], row + 4 * q);
            } else {
#pragma unroll
                for (int r = 0; r < 4; r++)
                    if (4 * q + r < nvalid) cp_async4(&sidx[v * TILE + 4 * q + r], row + 4 * q + r);
            }
        }
#pragma unroll
        for (int m = 0; m < 6; m++) g[m] = valid ? (T)__ldg(&fff[m * fff_stride + e0 + lane]) * h : T(0);
        cp_async_wait_all();
        __syncthreads();
    }
    // gather x of the tile's micro grids
    if (nvalid == TILE) {
#pragma unroll 4
        for (int k = tid; k < NXE * TILE; k += kThreads) cp_async_val<T>(&sx[k], x + sidx[k]);
    } else {
        for (int k = tid; k < NXE * TILE; k += kThreads)
            if (k % TILE < nvalid) cp_async_val<T>(&sx[k], x + sidx[k]);
    }
    // the distinct element-matrix entries, five per warp, while the gathers are in flight
    T *sa = sx + NXE * TILE;
    switch (warp) {
        case 0: store_entries<T, TILE, 0>(g, sa + lane); break;
        case 1: store_entries<T, TILE, 1>(g, sa + lane); break;
        case 2: store_entries<T, TILE, 2>(g, sa + lane); break;
        default: store_entries<T, TILE, 3>(g, sa + lane); break;
    }
    cp_async_wait_all();
    __syncthreads();
    all_columns<T, L, TILE>(warp, sx + lane, sidx + lane, sa + lane, valid ? 1u : 0u, y);
}

template <typename T, int L, bool PACKED>
static int launch(ptrdiff_t nelements, const int32_t *packed, idx_t **elements, ptrdiff_t fff_stride, const float *fff,
                  const T *x, T *y, cudaStream_t s) {
    const ptrdiff_t ntiles = (nelements + PK_TILE - 1) / PK_TILE;
    if (ntiles > 0x7fffffff) return set_error("sshex8 Laplacian stencil apply: too many tiles");
    constexpr size_t smem = smem_bytes<T, L>();
    static std::once_flag attr;  // shared-memory opt-in, once per instantiation
    std::call_once(attr, [] {
        cudaFuncSetAttribute(sshex8_laplacian_stencil_kernel<T, L, PACKED>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    sshex8_laplacian_stencil_kernel<T, L, PACKED><<<(unsigned)ntiles, kThreads, smem, s>>>(
            nelements, packed, elements, fff_stride, fff, x, y, first_wait_polls());
    return check_launch("sshex8 Laplacian stencil apply");
}

}  // namespace stencil

static std::atomic<int> g_first_wait_polls{LAP_WAIT_POLLS};
int first_wait_polls() { return g_first_wait_polls.load(std::memory_order_relaxed); }

// Levels served by the node-centric kernel (packed tiles: L = 4 only).
bool sshex8_laplacian_stencil_supported(int L) { return L >= 2 && L <= 4; }

template <typename T>
int sshex8_laplacian_stencil_apply(int L, ptrdiff_t nelements, const int32_t *packed, idx_t **elements,
                                   ptrdiff_t fff_stride, const float *fff, const T *x, T *y, cudaStream_t s) {
    if (nelements <= 0) return SFEM_GB300_SUCCESS;
    if (!sshex8_laplacian_stencil_supported(L)) return set_error("sshex8 Laplacian stencil apply: level %d not served", L);
    if (packed) {
        if (reinterpret_cast<uintptr_t>(packed) & 15)
            return set_error("sshex8 Laplacian stencil apply: packed block not 16-byte aligned");
        if (L == 3) return stencil::launch<T, 3, true>(nelements, packed, nullptr, 0, nullptr, x, y, s);
        if (L != PK_L) return set_error("sshex8 Laplacian stencil apply: no packed tiles at level %d", L);
        return stencil::launch<T, 4, true>(nelements, packed, nullptr, 0, nullptr, x, y, s);
    }
    switch (L) {
        case 2:
            return stencil::launch<T, 2, false>(nelements, nullptr, elements, fff_stride, fff, x, y, s);
        case 3:
            return stencil::launch<T, 3, false>(nelements, nullptr, elements, fff_stride, fff, x, y, s);
        default:
            return stencil::launch<T, 4, false>(nelements, nullptr, elements, fff_stride, fff, x, y, s);
    }
}

template int sshex8_laplacian_stencil_apply<float>(int, ptrdiff_t, const int32_t *, idx_t **, ptrdiff_t,
                                                   const float *, const float *, float *, cudaStream_t);
template int sshex8_laplacian_stencil_apply<double>(int, ptrdiff_t, const int32_t *, idx_t **, ptrdiff_t,
                                                    const float *, const double *, double *, cudaStream_t);

int sshex8_laplacian_stencil_status() {
    int st = 0;
    if (cudaMemcpyFromSymbol(&st, stencil::g_status, sizeof(int)) != cudaSuccess) return -1;
    if (st) {
        const int zero = 0;
        cudaMemcpyToSymbol(stencil::g_status, &zero, sizeof(int));
    }
    return st;
}

}  // namespace sfem_gb300

extern "C" int sfem_gb300_set_tile_wait_polls(int polls) {
    const int prev = sfem_gb300::g_first_wait_polls.load();
    sfem_gb300::g_first_wait_polls.store(polls < 0 ? sfem_gb300::LAP_WAIT_POLLS : polls);
    return prev;
}
