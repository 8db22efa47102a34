// C++ test of include/sfem_gb300_adapter.hpp: the BLAS, Operator and Op adapters
// instantiated on the reference-shaped interfaces, driven the way the reference's
// solver templates and frontend drive them (a CG loop written against BLAS<T> and
// Operator<T> only), checked against host arithmetic and operator identities.
// Exit code 0 = every check passed.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <memory>
#include <random>
#include <vector>

#include "sfem_gb300_adapter.hpp"

namespace A = sfem_gb300::adapter;
using A::idx_t;
using A::real_t;

static int failures = 0;
#define EXPECT(cond, ...)                                  \
    do {                                                   \
        if (!(cond)) {                                     \
            std::fprintf(stderr, "FAILED %s: ", #cond);    \
            std::fprintf(stderr, __VA_ARGS__);             \
            std::fprintf(stderr, "\n");                    \
            failures++;                                    \
        }                                                  \
    } while (0)

template <typename T>
static T *to_device(const std::vector<T> &h) {
    T *d = nullptr;
    A::check_cuda(cudaMalloc((void **)&d, h.size() * sizeof(T)), "malloc");
    A::check_cuda(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice), "h2d");
    return d;
}
template <typename T>
static std::vector<T> to_host(const T *d, size_t n) {
    std::vector<T> h(n);
    A::check_cuda(cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost), "d2h");
    return h;
}

// Structured semi-structured mesh: nx x ny x nz macro elements at level L on a
// lexicographic global grid; SoA rows on the device plus a device array of row pointers.
struct Mesh {
    int L, nx, ny, nz;
    ptrdiff_t E, N;
    std::vector<std::vector<idx_t>> rows;  // [(L+1)^3][E]
    std::vector<std::vector<float>> xyz;   // [3][N]
    idx_t **d_elements = nullptr, **d_corners = nullptr;
    float **d_points = nullptr;
    std::vector<void *> owned;

    Mesh(int L_, int nx_, int ny_, int nz_) : L(L_), nx(nx_), ny(ny_), nz(nz_) {
        const int N1 = L + 1, gx = nx * L + 1, gy = ny * L + 1, gz = nz * L + 1;
        E = (ptrdiff_t)nx * ny * nz;
        N = (ptrdiff_t)gx * gy * gz;
        rows.assign(N1 * N1 * N1, std::vector<idx_t>(E));
        for (int ez = 0; ez < nz; ez++)
            for (int ey = 0; ey < ny; ey++)
                for (int ex = 0; ex < nx; ex++) {
                    const ptrdiff_t e = ((ptrdiff_t)ez * ny + ey) * nx + ex;
                    for (int z = 0; z <= L; z++)
                        for (int y = 0; y <= L; y++)
                            for (int x = 0; x <= L; x++)
                                rows[(z * N1 + y) * N1 + x][e] =
                                        (idx_t)(((ptrdiff_t)(ez * L + z) * gy + ey * L + y) * gx + ex * L + x);
                }
        xyz.assign(3, std::vector<float>(N));
        std::mt19937 rng(3);
        std::uniform_real_distribution<float> u(-0.05f, 0.05f);
        for (int k = 0; k < gz; k++)
            for (int j = 0; j < gy; j++)
                for (int i = 0; i < gx; i++) {
                    const ptrdiff_t n = ((ptrdiff_t)k * gy + j) * gx + i;
                    // stretched, sheared grid (affine per macro element is what the operator assumes)
                    xyz[0][n] = (float)i / (nx * L) * 2.0f + 0.1f * (float)j / (ny * L);
                    xyz[1][n] = (float)j / (ny * L);
                    xyz[2][n] = (float)k / (nz * L) * 0.5f;
                }
        std::vector<idx_t *> rp;
        for (auto &r : rows) {
            idx_t *d = to_device(r);
            owned.push_back(d);
            rp.push_back(d);
        }
        d_elements = to_device(rp);
        owned.push_back(d_elements);
        static const int c8[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
        std::vector<idx_t *> cp;
        for (auto &c : c8) cp.push_back(rp[(c[2] * L * N1 + c[1] * L) * N1 + c[0] * L]);
        d_corners = to_device(cp);
        owned.push_back(d_corners);
        std::vector<float *> pp;
        for (auto &v : xyz) {
            float *d = to_device(v);
            owned.push_back(d);
            pp.push_back(d);
        }
        d_points = to_device(pp);
        owned.push_back(d_points);
    }
    ~Mesh() {
        for (void *p : owned) cudaFree(p);
    }
};

static double host_dot(const std::vector<double> &a, const std::vector<double> &b) {
    double s = 0;
    for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
    return s;
}

static void test_blas() {
    using BLAS = A::DeviceBLAS<double, A::interfaces::BLAS<double>>;
    std::unique_ptr<A::interfaces::BLAS<double>> blas(new BLAS());
    const ptrdiff_t n = 100003;
    std::mt19937 rng(1);
    std::normal_distribution<double> nd;
    std::vector<double> hx(n), hy(n);
    for (auto &v : hx) v = nd(rng);
    for (auto &v : hy) v = nd(rng);
    double *x = blas->allocate(n), *y = blas->allocate(n), *z = blas->allocate(n);
    A::check_cuda(cudaMemcpy(x, hx.data(), n * 8, cudaMemcpyHostToDevice), "h2d");
    A::check_cuda(cudaMemcpy(y, hy.data(), n * 8, cudaMemcpyHostToDevice), "h2d");
    const double d = blas->dot(n, x, y), dh = host_dot(hx, hy);
    EXPECT(std::fabs(d - dh) <= 1e-12 * std::sqrt(host_dot(hx, hx) * host_dot(hy, hy)), "dot %g vs %g", d, dh);
    const double nrm = blas->norm2(n, x);
    EXPECT(std::fabs(nrm - std::sqrt(host_dot(hx, hx))) <= 1e-13 * nrm, "norm2 %g", nrm);
    blas->zaxpby(n, 2.0, x, -3.0, y, z);  // z = 2x - 3y
    blas->axpby(n, 0.5, x, 2.0, y);       // y = 0.5x + 2y
    blas->axpy(n, -1.0, x, y);            // y -= x
    blas->scal(n, 4.0, y);
    blas->xypaz(n, x, x, 1.0, z);  // z = x*x + z
    std::vector<double> hz = to_host(z, n), hy2 = to_host(y, n);
    double ez = 0, ey = 0;
    for (ptrdiff_t i = 0; i < n; i++) {
        ez = std::fmax(ez, std::fabs(hz[i] - (hx[i] * hx[i] + 2 * hx[i] - 3 * hy[i])));
        ey = std::fmax(ey, std::fabs(hy2[i] - 4 * (0.5 * hx[i] + 2 * hy[i] - hx[i])));
    }
    EXPECT(ez <= 1e-13 && ey <= 1e-13, "vector updates %g %g", ez, ey);
    blas->values(n, 2.0, z);
    blas->reciprocal(n, 3.0, z);  // 3 / 2
    blas->copy(n, z, y);
    std::vector<double> hr = to_host(y, n);
    EXPECT(hr[0] == 1.5 && hr[n - 1] == 1.5, "values / reciprocal / copy %g", hr[0]);
    blas->zeros(n, y);
    EXPECT(blas->norm2(n, y) == 0.0, "zeros");
    blas->destroy(x);
    blas->destroy(y);
    blas->destroy(z);
}

// CG written against BLAS<T> and Operator<T> only, as the reference's ConjugateGradient
template <class Op, class Blas>
static int cg(Op &op, Blas &blas, const double *b, double *x, double rtol, int max_it, double *rel) {
    const ptrdiff_t n = op.rows();
    double *r = blas.allocate(n), *p = blas.allocate(n), *Ap = blas.allocate(n);
    blas.zeros(n, x);
    blas.copy(n, b, r);
    blas.copy(n, b, p);
    double rr = blas.dot(n, r, r);
    const double b2 = rr;
    int it = 0;
    for (; it < max_it && std::sqrt(rr / b2) > rtol; it++) {
        blas.zeros(n, Ap);
        op.apply(p, Ap);
        const double alpha = rr / blas.dot(n, p, Ap);
        blas.axpy(n, alpha, p, x);
        blas.axpy(n, -alpha, Ap, r);
        const double rr_new = blas.dot(n, r, r);
        blas.axpby(n, 1.0, r, rr_new / rr, p);
        rr = rr_new;
    }
    *rel = std::sqrt(rr / b2);
    blas.destroy(r);
    blas.destroy(p);
    blas.destroy(Ap);
    return it;
}

static void test_laplacian() {
    using Op = A::LaplacianOp<A::interfaces::Op, A::interfaces::EXECUTION_SPACE_DEVICE>;
    using BLAS = A::DeviceBLAS<double, A::interfaces::BLAS<double>>;
    Mesh m(4, 5, 4, 3);
    auto op = std::make_shared<Op>(SFEM_GB300_SSHEX8(4), m.E, m.d_elements, m.d_corners, m.d_points, m.N);
    std::shared_ptr<A::interfaces::Op> base = op;
    EXPECT(std::string(base->name()) == "gpu:Laplacian" && base->is_linear(), "name");
    EXPECT(base->execution_space() == A::interfaces::EXECUTION_SPACE_DEVICE, "execution space");
    EXPECT(base->initialize() == 0, "initialize");
    BLAS blas;
    const ptrdiff_t n = m.N;
    std::mt19937 rng(2);
    std::normal_distribution<double> nd;
    std::vector<double> hx(n), hy(n), ones(n, 1.0);
    for (auto &v : hx) v = nd(rng);
    for (auto &v : hy) v = nd(rng);
    double *x = to_device(hx), *y = to_device(hy), *one = to_device(ones);
    double *Ax = blas.allocate(n), *Ay = blas.allocate(n), *A1 = blas.allocate(n), *dg = blas.allocate(n);
    EXPECT(base->apply(nullptr, x, Ax) == 0 && base->apply(nullptr, y, Ay) == 0, "apply");
    EXPECT(base->gradient(one, A1) == 0, "gradient");
    EXPECT(base->hessian_diag(nullptr, dg) == 0, "diag");
    const double xAy = blas.dot(n, x, Ay), yAx = blas.dot(n, y, Ax);
    EXPECT(std::fabs(xAy - yAx) <= 1e-12 * std::fabs(xAy) + 1e-12, "symmetry %g %g", xAy, yAx);
    std::vector<double> a1 = to_host(A1, n), d = to_host(dg, n);
    double m1 = 0, md = 0;
    for (ptrdiff_t i = 0; i < n; i++) {
        m1 = std::fmax(m1, std::fabs(a1[i]));
        md = std::fmax(md, std::fabs(d[i]));
    }
    EXPECT(m1 <= 1e-12 * md, "A 1 = 0 (%g against diagonal %g)", m1, md);
    // the diagonal equals e_i . A e_i
    for (ptrdiff_t i : {ptrdiff_t(0), n / 3, n - 1}) {
        std::vector<double> e(n, 0.0);
        e[i] = 1;
        double *de = to_device(e);
        double *Ae = blas.allocate(n);
        base->apply(nullptr, de, Ae);
        const double aii = to_host(Ae + i, 1)[0];
        EXPECT(std::fabs(aii - d[i]) <= 1e-13 * md, "diag entry %td: %g vs %g", i, aii, d[i]);
        cudaFree(de);
        blas.destroy(Ae);
    }
    double v = 0;
    EXPECT(base->value(x, &v) == 0 && std::fabs(v - 0.5 * blas.dot(n, x, Ax)) <= 1e-12 * std::fabs(v), "value");
    // Operator<T> around the op (A + I: SPD without constraints) and CG on BLAS<T>
    using Operator = A::DeviceOperator<double, A::interfaces::Operator<double>, A::interfaces::EXECUTION_SPACE_DEVICE>;
    Operator shifted(n, n, [&](const double *in, double *out) {
        const int rc = base->apply(nullptr, in, out);
        blas.axpy(n, 1.0, in, out);
        return rc;
    });
    A::interfaces::Operator<double> &opref = shifted;
    double *sol = blas.allocate(n), rel = 1;
    const int its = cg(opref, blas, y, sol, 1e-10, 500, &rel);
    double *chk = blas.allocate(n);
    opref.apply(sol, chk);
    blas.axpy(n, -1.0, y, chk);
    const double true_rel = blas.norm2(n, chk) / blas.norm2(n, y);
    EXPECT(rel <= 1e-10 && true_rel <= 1e-9, "CG through the adapters: %d iterations, rel %g, true %g", its, rel,
           true_rel);
    for (double *p : {x, y, one}) cudaFree(p);
    for (double *p : {Ax, Ay, A1, dg, sol, chk}) blas.destroy(p);
}

static void test_elasticity() {
    using Op = A::LinearElasticityOp<A::interfaces::Op, A::interfaces::EXECUTION_SPACE_DEVICE>;
    using BLAS = A::DeviceBLAS<double, A::interfaces::BLAS<double>>;
    Mesh m(1, 4, 3, 2);
    auto op = std::make_shared<Op>(SFEM_GB300_HEX8, m.E, m.d_elements, m.d_corners, m.d_points, m.N, 1.0, 10.0);
    A::interfaces::Op &base = *op;
    EXPECT(std::string(base.name()) == "gpu:LinearElasticity", "name");
    EXPECT(base.initialize() == 0, "initialize");
    BLAS blas;
    const ptrdiff_t n = 3 * m.N;
    std::vector<double> hu(n), tx(n, 0.0);
    std::mt19937 rng(4);
    std::normal_distribution<double> nd;
    for (auto &v : hu) v = nd(rng);
    for (ptrdiff_t i = 0; i < m.N; i++) tx[3 * i] = 1.0;  // rigid translation in x
    double *u = to_device(hu), *t = to_device(tx);
    double *Ku = blas.allocate(n), *Kt = blas.allocate(n);
    EXPECT(base.apply(nullptr, u, Ku) == 0 && base.apply(nullptr, t, Kt) == 0, "apply");
    std::vector<double> ku = to_host(Ku, n), kt = to_host(Kt, n);
    double mku = 0, mkt = 0;
    for (ptrdiff_t i = 0; i < n; i++) {
        mku = std::fmax(mku, std::fabs(ku[i]));
        mkt = std::fmax(mkt, std::fabs(kt[i]));
    }
    EXPECT(mkt <= 1e-12 * mku, "K (rigid translation) = 0: %g", mkt);
    // BSR on the full node graph reproduces the matrix-free apply
    std::vector<std::vector<idx_t>> nbr(m.N);
    for (ptrdiff_t e = 0; e < m.E; e++)
        for (int a = 0; a < 8; a++)
            for (int b = 0; b < 8; b++) nbr[m.rows[a][e]].push_back(m.rows[b][e]);
    std::vector<A::count_t> rowptr(m.N + 1, 0);
    std::vector<idx_t> colidx;
    for (ptrdiff_t i = 0; i < m.N; i++) {
        auto &c = nbr[i];
        std::sort(c.begin(), c.end());
        c.erase(std::unique(c.begin(), c.end()), c.end());
        colidx.insert(colidx.end(), c.begin(), c.end());
        rowptr[i + 1] = (A::count_t)colidx.size();
    }
    A::count_t *d_rp = to_device(rowptr);
    idx_t *d_ci = to_device(colidx);
    double *vals = blas.allocate(colidx.size() * 9);
    EXPECT(base.hessian_bsr(nullptr, d_rp, d_ci, vals) == 0, "bsr");
    std::vector<double> hv = to_host(vals, colidx.size() * 9), y(n, 0.0);
    for (ptrdiff_t i = 0; i < m.N; i++)
        for (A::count_t k = rowptr[i]; k < rowptr[i + 1]; k++)
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) y[3 * i + r] += hv[(size_t)k * 9 + r * 3 + c] * hu[3 * colidx[k] + c];
    double eb = 0;
    for (ptrdiff_t i = 0; i < n; i++) eb = std::fmax(eb, std::fabs(y[i] - ku[i]));
    EXPECT(eb <= 1e-12 * mku, "BSR SpMV against apply: %g", eb);
    double *dg = blas.allocate(n), *bd = blas.allocate(6 * m.N);
    EXPECT(base.hessian_diag(nullptr, dg) == 0 && base.hessian_block_diag_sym(nullptr, bd) == 0, "diagonals");
    std::vector<double> hd = to_host(dg, n), hb = to_host(bd, 6 * m.N);
    double ed = 0;
    for (ptrdiff_t i = 0; i < m.N; i++) {
        ed = std::fmax(ed, std::fabs(hd[3 * i] - hb[6 * i]));
        ed = std::fmax(ed, std::fabs(hd[3 * i + 1] - hb[6 * i + 3]));
        ed = std::fmax(ed, std::fabs(hd[3 * i + 2] - hb[6 * i + 5]));
    }
    double mdiag = 0;
    for (double v : hd) mdiag = std::fmax(mdiag, std::fabs(v));
    EXPECT(ed <= 1e-14 * mdiag, "block diagonal holds the diagonal: %g", ed);
    EXPECT(base.hessian_crs(nullptr, d_rp, d_ci, vals) != 0, "scalar CRS refused for the vector operator");
    cudaFree(u);
    cudaFree(t);
    cudaFree(d_rp);
    cudaFree(d_ci);
    for (double *p : {Ku, Kt, vals, dg, bd}) blas.destroy(p);
}

int main() {
    try {
        test_blas();
        test_laplacian();
        test_elasticity();
    } catch (const std::exception &ex) {
        std::fprintf(stderr, "exception: %s\n", ex.what());
        return 2;
    }
    if (failures) {
        std::fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("adapter test: all checks passed\n");
    return 0;
}
