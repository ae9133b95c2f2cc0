// numa_oracle.cpp — CPU restatement of the reference's matrix-free nonlinear-solve path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU library is checked against
// (tests/, __graft_entry__.smoke()) and the CPU baseline that bench.py times.  Nothing in the
// product library links, loads or calls it.
//
// It restates, in plain C++20 + OpenMP, the algorithms of kapumota/chebyshev-nonlinear-lab
// (namespace numa::op), citing the reference file:line each function follows.  Parallelism
// mirrors the reference exactly (OpenMP where the reference has it, serial where it is serial:
// the multigrid V-cycle and most GMRES loops), so that its timings stand for the reference's.
// It is pinned against the reference itself: tests/golden/ holds outputs of the reference's own
// headers compiled here (oracle/build_ref.sh, oracle/ref_driver.cpp), and the reference's
// published count table (docs/research/R1_OPERATOR_INTERFACE.md:113-121).
//
// Floating-point contraction is disabled at build time (-ffp-contract=off) so that the
// element-wise arithmetic is the IEEE sequence written here.
//
// C API at the end (extern "C"), used from Python through ctypes.

#include "../include/numa_gpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <stdexcept>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

using DVec = std::vector<double>;
using Clock = std::chrono::steady_clock;

static double seconds_since(Clock::time_point t0) {
    return std::chrono::duration<double>(Clock::now() - t0).count();
}

// ---------------------------------------------------------------- BLAS-1 (operator.hpp:19-41)
static double dot(const DVec& a, const DVec& b) {
    double s = 0.0;
    const long n = static_cast<long>(a.size());
#pragma omp parallel for reduction(+ : s) schedule(static) if (n > 4096)
    for (long i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

static double norm2(const DVec& a) { return std::sqrt(dot(a, a)); }

static void axpy(double a, const DVec& x, DVec& y) {
    const long n = static_cast<long>(x.size());
#pragma omp parallel for schedule(static) if (n > 4096)
    for (long i = 0; i < n; ++i) y[i] += a * x[i];
}

// ---------------------------------------------------------------- Bratu3D (problems/bratu3d.hpp)
struct Bratu {
    std::size_t n;
    double lambda;
    double h2inv;  // (n+1)^2, bratu3d.hpp:15

    Bratu(std::size_t n_, double lam) : n(n_), lambda(lam), h2inv((n_ + 1.0) * (n_ + 1.0)) {}
    std::size_t size() const { return n * n * n; }

    // out = h^-2 (6 v - sum of the six neighbours), Dirichlet zeros skipped (bratu3d.hpp:73-95).
    void neg_laplacian(const DVec& v, DVec& out) const {
        out.resize(v.size());
        const long nl = static_cast<long>(n);
        const std::size_t plane = n * n;
#pragma omp parallel for collapse(2) schedule(static) if (nl > 16)
        for (long i = 0; i < nl; ++i)
            for (long j = 0; j < nl; ++j) {
                const std::size_t row = (static_cast<std::size_t>(i) * n + j) * n;
                for (std::size_t k = 0; k < n; ++k) {
                    const std::size_t p = row + k;
                    double acc = 6.0 * v[p];
                    if (i > 0) acc -= v[p - plane];
                    if (i + 1 < nl) acc -= v[p + plane];
                    if (j > 0) acc -= v[p - n];
                    if (j + 1 < nl) acc -= v[p + n];
                    if (k > 0) acc -= v[p - 1];
                    if (k + 1 < n) acc -= v[p + 1];
                    out[p] = h2inv * acc;
                }
            }
    }

    // F(u) = -lap u - lambda e^u (bratu3d.hpp:21-31)
    void eval(const DVec& u, DVec& out) const {
        neg_laplacian(u, out);
        const long cnt = static_cast<long>(out.size());
#pragma omp parallel for schedule(static) if (cnt > 4096)
        for (long p = 0; p < cnt; ++p) out[p] -= lambda * std::exp(u[p]);
    }

    // F'(u) v = -lap v - lambda e^u v (bratu3d.hpp:33-43)
    void jvp(const DVec& u, const DVec& v, DVec& out) const {
        neg_laplacian(v, out);
        const long cnt = static_cast<long>(out.size());
#pragma omp parallel for schedule(static) if (cnt > 4096)
        for (long p = 0; p < cnt; ++p) out[p] -= lambda * std::exp(u[p]) * v[p];
    }

    // F''(u)[v,v] = -lambda e^u v^2 (bratu3d.hpp:46-56)
    void d2(const DVec& u, const DVec& v, DVec& out) const {
        out.resize(u.size());
        const long cnt = static_cast<long>(out.size());
#pragma omp parallel for schedule(static) if (cnt > 4096)
        for (long p = 0; p < cnt; ++p) out[p] = -lambda * std::exp(u[p]) * v[p] * v[p];
    }

    // d = 6 h^-2 - lambda e^u (bratu3d.hpp:59-69)
    void jacobi_diag(const DVec& u, DVec& d) const {
        d.resize(u.size());
        const long cnt = static_cast<long>(d.size());
#pragma omp parallel for schedule(static) if (cnt > 4096)
        for (long p = 0; p < cnt; ++p) d[p] = 6.0 * h2inv - lambda * std::exp(u[p]);
    }
};

// Forward-difference J v with two F evaluations (operator.hpp:101-114).
template <class Op>
static void jvp_fd(const Op& f, const DVec& x, const DVec& v, DVec& out) {
    const std::size_t N = x.size();
    out.assign(N, 0.0);
    const double nv = norm2(v);
    if (nv == 0.0) return;
    const double h = std::sqrt(std::numeric_limits<double>::epsilon()) * (1.0 + norm2(x)) / nv;
    DVec xp = x, f0(N), f1(N);
    axpy(h, v, xp);
    f.eval(x, f0);
    f.eval(xp, f1);
    for (std::size_t p = 0; p < N; ++p) out[p] = (f1[p] - f0[p]) / h;
}

// Central second difference with three F evaluations, step eps^(1/4) (operator.hpp:118-134).
template <class Op>
static void d2_fd(const Op& f, const DVec& x, const DVec& v, DVec& out) {
    const std::size_t N = x.size();
    out.assign(N, 0.0);
    const double nv = norm2(v);
    if (nv == 0.0) return;
    const double h = std::pow(std::numeric_limits<double>::epsilon(), 0.25) * (1.0 + norm2(x)) / nv;
    DVec xp = x, xm = x, f0(N), fp(N), fm(N);
    axpy(h, v, xp);
    axpy(-h, v, xm);
    f.eval(x, f0);
    f.eval(xp, fp);
    f.eval(xm, fm);
    for (std::size_t p = 0; p < N; ++p) out[p] = (fp[p] - 2.0 * f0[p] + fm[p]) / (h * h);
}

// Operator wrapper: which derivative forms the drivers see, plus call timers (timing.hpp:37-75).
struct Timers {
    double t_F = 0, t_JVP = 0, t_D2 = 0, t_prec = 0, t_setup = 0;
};

struct BratuOp {
    const Bratu& f;
    int jvp_mode;  // 0 analytic, 1 FD
    int d2_mode;
    Timers* timers;

    std::size_t size() const { return f.size(); }
    void eval(const DVec& x, DVec& out) const {
        auto t0 = Clock::now();
        f.eval(x, out);
        timers->t_F += seconds_since(t0);
    }
    void jvp(const DVec& x, const DVec& v, DVec& out) const {
        auto t0 = Clock::now();
        if (jvp_mode == 1) jvp_fd(f, x, v, out); else f.jvp(x, v, out);
        timers->t_JVP += seconds_since(t0);
    }
    void d2(const DVec& x, const DVec& v, DVec& out) const {
        auto t0 = Clock::now();
        if (d2_mode == 1) d2_fd(f, x, v, out); else f.d2(x, v, out);
        timers->t_D2 += seconds_since(t0);
    }
};

// ---------------------------------------------------------------- PoissonMG (linalg/poisson_mg.hpp)
class PoissonMG {
public:
    struct Level {
        std::size_t n = 0;
        double h2inv = 0.0;
        DVec x, b, r;
    };

    // Levels while n is odd, halving (m-1)/2 and h2inv/4, down to n = 1 (poisson_mg.hpp:26-64).
    PoissonMG(std::size_t n, int pre = 2, int post = 2) : pre_(pre), post_(post) {
        if (n == 0) throw std::invalid_argument("PoissonMG: grid size must be positive");
        if (pre < 0 || post < 0) throw std::invalid_argument("PoissonMG: negative sweep count");
        const std::size_t maxs = std::numeric_limits<std::size_t>::max();
        if (n > maxs / n || n * n > maxs / n) throw std::overflow_error("PoissonMG: n^3 overflows");
        std::size_t m = n;
        double h2 = (static_cast<double>(n) + 1.0) * (static_cast<double>(n) + 1.0);
        for (;;) {
            Level L;
            L.n = m;
            L.h2inv = h2;
            L.x.assign(m * m * m, 0.0);
            L.b.assign(m * m * m, 0.0);
            L.r.assign(m * m * m, 0.0);
            levels_.push_back(std::move(L));
            if (m % 2 == 0 || m <= 1) break;
            m = (m - 1) / 2;
            h2 /= 4.0;
        }
    }

    std::size_t levels() const { return levels_.size(); }

    // z = V-cycle(r) (poisson_mg.hpp:69-80)
    void apply(const DVec& r, DVec& z) const {
        Level& top = levels_[0];
        if (r.size() != top.x.size()) throw std::invalid_argument("PoissonMG: residual size mismatch");
        top.b = r;
        std::fill(top.x.begin(), top.x.end(), 0.0);
        cycle(0);
        z = top.x;
    }
    void operator()(const DVec& r, DVec& z) const { apply(r, z); }

    // One red-black Gauss-Seidel sweep; order 0 = colour 0 then 1, order 1 reversed.
    // Colour of (i,j,k) is (i+j+k)&1 (poisson_mg.hpp:99-126).
    static void smooth(Level& L, int order) {
        const std::size_t n = L.n, plane = n * n;
        const double inv = 1.0 / L.h2inv;
        for (int pass = 0; pass < 2; ++pass) {
            const std::size_t colour = static_cast<std::size_t>(order == 0 ? pass : 1 - pass);
            for (std::size_t i = 0; i < n; ++i)
                for (std::size_t j = 0; j < n; ++j)
                    for (std::size_t k = (i + j + colour) & 1; k < n; k += 2) {
                        const std::size_t p = (i * n + j) * n + k;
                        double acc = L.b[p] * inv;
                        if (i > 0) acc += L.x[p - plane];
                        if (i + 1 < n) acc += L.x[p + plane];
                        if (j > 0) acc += L.x[p - n];
                        if (j + 1 < n) acc += L.x[p + n];
                        if (k > 0) acc += L.x[p - 1];
                        if (k + 1 < n) acc += L.x[p + 1];
                        L.x[p] = acc / 6.0;
                    }
        }
    }

    // r = b - h^-2 (6x - sum nbrs) (poisson_mg.hpp:128-149)
    static void residual(Level& L) {
        const std::size_t n = L.n, plane = n * n;
        for (std::size_t i = 0; i < n; ++i)
            for (std::size_t j = 0; j < n; ++j)
                for (std::size_t k = 0; k < n; ++k) {
                    const std::size_t p = (i * n + j) * n + k;
                    double acc = 6.0 * L.x[p];
                    if (i > 0) acc -= L.x[p - plane];
                    if (i + 1 < n) acc -= L.x[p + plane];
                    if (j > 0) acc -= L.x[p - n];
                    if (j + 1 < n) acc -= L.x[p + n];
                    if (k > 0) acc -= L.x[p - 1];
                    if (k + 1 < n) acc -= L.x[p + 1];
                    L.r[p] = L.b[p] - L.h2inv * acc;
                }
    }

    // 27-point full weighting, coarse I <-> fine 2I+1, weights (1/4,1/2,1/4)^3; the sum runs
    // a outer, b middle, c inner, each weight product formed as wa*wb*wc (poisson_mg.hpp:152-188).
    static void restrict_to(const Level& F, Level& C) {
        static const double w[3] = {0.25, 0.5, 0.25};
        const std::size_t nf = F.n, nc = C.n;
        for (std::size_t I = 0; I < nc; ++I)
            for (std::size_t J = 0; J < nc; ++J)
                for (std::size_t K = 0; K < nc; ++K) {
                    double acc = 0.0;
                    for (int a = 0; a < 3; ++a) {
                        const std::size_t fi = 2 * I + a;
                        if (fi >= nf) continue;
                        for (int b = 0; b < 3; ++b) {
                            const std::size_t fj = 2 * J + b;
                            if (fj >= nf) continue;
                            for (int c = 0; c < 3; ++c) {
                                const std::size_t fk = 2 * K + c;
                                if (fk >= nf) continue;
                                acc += w[a] * w[b] * w[c] * F.r[(fi * nf + fj) * nf + fk];
                            }
                        }
                    }
                    C.b[(I * nc + J) * nc + K] = acc;
                }
    }

    // 1D interpolation stencil of fine index f over a coarse grid of size nc
    // (poisson_mg.hpp:191-220): odd f -> coarse (f-1)/2 with weight 1; even f -> coarse f/2-1
    // and f/2 (those inside the grid) with weight 1/2 each.
    static int interp_1d(std::size_t f, std::size_t nc, std::size_t idx[2], double wt[2]) {
        if (f % 2 == 1) {
            idx[0] = (f - 1) / 2;
            wt[0] = 1.0;
            return 1;
        }
        int cnt = 0;
        const std::size_t right = f / 2;
        if (right >= 1) { idx[cnt] = right - 1; wt[cnt] = 0.5; ++cnt; }
        if (right < nc) { idx[cnt] = right; wt[cnt] = 0.5; ++cnt; }
        return cnt;
    }

    // Trilinear interpolation added into the fine x (poisson_mg.hpp:222-260).
    static void prolong_add(const Level& C, Level& F) {
        const std::size_t nf = F.n, nc = C.n;
        for (std::size_t i = 0; i < nf; ++i) {
            std::size_t ci[2]; double wi[2];
            const int ni = interp_1d(i, nc, ci, wi);
            for (std::size_t j = 0; j < nf; ++j) {
                std::size_t cj[2]; double wj[2];
                const int nj = interp_1d(j, nc, cj, wj);
                for (std::size_t k = 0; k < nf; ++k) {
                    std::size_t ck[2]; double wk[2];
                    const int nk = interp_1d(k, nc, ck, wk);
                    double acc = 0.0;
                    for (int a = 0; a < ni; ++a)
                        for (int b = 0; b < nj; ++b)
                            for (int c = 0; c < nk; ++c)
                                acc += wi[a] * wj[b] * wk[c] * C.x[(ci[a] * nc + cj[b]) * nc + ck[c]];
                    F.x[(i * nf + j) * nf + k] += acc;
                }
            }
        }
    }

    // V(pre, post); coarsest n == 1 solved exactly, else 30 alternating sweeps
    // (poisson_mg.hpp:262-294).
    void cycle(std::size_t l) const {
        Level& L = levels_[l];
        if (l + 1 == levels_.size()) {
            if (L.n == 1) {
                L.x[0] = L.b[0] / (6.0 * L.h2inv);
            } else {
                for (int s = 0; s < 30; ++s) smooth(L, s % 2);
            }
            return;
        }
        for (int s = 0; s < pre_; ++s) smooth(L, 0);
        residual(L);
        Level& C = levels_[l + 1];
        restrict_to(L, C);
        std::fill(C.x.begin(), C.x.end(), 0.0);
        cycle(l + 1);
        prolong_add(C, L);
        for (int s = 0; s < post_; ++s) smooth(L, 1);
    }

    mutable std::vector<Level> levels_;

private:
    int pre_, post_;
};

// ---------------------------------------------------------------- HelmholtzMG2D (linalg/helmholtz_mg2d.hpp)
// 2D V-cycle for alpha I - nu Lap_h, 5-point stencil, red-black Gauss-Seidel (colour (i+j)&1),
// 9-point full weighting, bilinear additive prolongation; levels while n is odd, s = nu h^-2
// quartered per level (helmholtz_mg2d.hpp:15-32); coarsest n = 1 exact, else 30 sweeps.
class HelmholtzMG2D {
public:
    struct Level {
        std::size_t n = 0;
        double s = 0.0;
        DVec x, b, r;
    };
    HelmholtzMG2D(std::size_t n, double alpha, double nu, int pre = 2, int post = 2)
        : alpha_(alpha), pre_(pre), post_(post) {
        std::size_t m = n;
        double s = nu * (static_cast<double>(n) + 1.0) * (static_cast<double>(n) + 1.0);
        for (;;) {
            Level L;
            L.n = m;
            L.s = s;
            L.x.assign(m * m, 0.0);
            L.b.assign(m * m, 0.0);
            L.r.assign(m * m, 0.0);
            levels_.push_back(std::move(L));
            if (m % 2 == 0 || m <= 1) break;
            m = (m - 1) / 2;
            s /= 4.0;
        }
    }
    std::size_t levels() const { return levels_.size(); }
    void apply(const DVec& r, DVec& z) const {
        Level& L0 = levels_[0];
        L0.b = r;
        std::fill(L0.x.begin(), L0.x.end(), 0.0);
        cycle(0);
        z = L0.x;
    }

    // (helmholtz_mg2d.hpp:51-70): x = (b + s * sum of the 4 neighbours) / (alpha + 4 s)
    void smooth(Level& L, int order) const {
        const std::size_t n = L.n;
        const double den = alpha_ + 4.0 * L.s;
        for (int pass = 0; pass < 2; ++pass) {
            const std::size_t colour = (order == 0) ? pass : 1 - pass;
#pragma omp parallel for schedule(static) if (n * n > 4096)
            for (long ii = 0; ii < static_cast<long>(n); ++ii) {
                const std::size_t i = static_cast<std::size_t>(ii);
                for (std::size_t j = (i + colour) & 1; j < n; j += 2) {
                    const std::size_t p = i * n + j;
                    double nb = 0.0;
                    if (i > 0) nb += L.x[p - n];
                    if (i + 1 < n) nb += L.x[p + n];
                    if (j > 0) nb += L.x[p - 1];
                    if (j + 1 < n) nb += L.x[p + 1];
                    L.x[p] = (L.b[p] + L.s * nb) / den;
                }
            }
        }
    }
    // r = b - (alpha x + s (4x - nb)) (helmholtz_mg2d.hpp:72-87)
    void residual(Level& L) const {
        const std::size_t n = L.n;
#pragma omp parallel for schedule(static) if (n * n > 4096)
        for (long ii = 0; ii < static_cast<long>(n); ++ii) {
            const std::size_t i = static_cast<std::size_t>(ii);
            for (std::size_t j = 0; j < n; ++j) {
                const std::size_t p = i * n + j;
                double nb = 0.0;
                if (i > 0) nb += L.x[p - n];
                if (i + 1 < n) nb += L.x[p + n];
                if (j > 0) nb += L.x[p - 1];
                if (j + 1 < n) nb += L.x[p + 1];
                L.r[p] = L.b[p] - (alpha_ * L.x[p] + L.s * (4.0 * L.x[p] - nb));
            }
        }
    }
    // 9-point full weighting, coarse I <-> fine 2I+1 (helmholtz_mg2d.hpp:89-108)
    static void restrict_to(const Level& F, Level& C) {
        static const double w[3] = {0.25, 0.5, 0.25};
        const std::size_t nf = F.n, nc = C.n;
#pragma omp parallel for schedule(static) if (nc * nc > 4096)
        for (long II = 0; II < static_cast<long>(nc); ++II)
            for (std::size_t J = 0; J < nc; ++J) {
                const std::size_t I = static_cast<std::size_t>(II);
                double acc = 0.0;
                for (int a = 0; a < 3; ++a) {
                    const std::size_t fi = 2 * I + a;
                    if (fi >= nf) continue;
                    for (int b = 0; b < 3; ++b) {
                        const std::size_t fj = 2 * J + b;
                        if (fj >= nf) continue;
                        acc += w[a] * w[b] * F.r[fi * nf + fj];
                    }
                }
                C.b[I * nc + J] = acc;
            }
    }
    // bilinear additive prolongation (helmholtz_mg2d.hpp:110-136)
    static void prolong_add(const Level& C, Level& F) {
        const std::size_t nf = F.n, nc = C.n;
#pragma omp parallel for schedule(static) if (nf * nf > 4096)
        for (long ii = 0; ii < static_cast<long>(nf); ++ii) {
            const std::size_t i = static_cast<std::size_t>(ii);
            std::size_t ci[2]; double wi[2];
            const int ni = PoissonMG::interp_1d(i, nc, ci, wi);
            for (std::size_t j = 0; j < nf; ++j) {
                std::size_t cj[2]; double wj[2];
                const int nj = PoissonMG::interp_1d(j, nc, cj, wj);
                double acc = 0.0;
                for (int a = 0; a < ni; ++a)
                    for (int b = 0; b < nj; ++b) acc += wi[a] * wj[b] * C.x[ci[a] * nc + cj[b]];
                F.x[i * nf + j] += acc;
            }
        }
    }
    void cycle(std::size_t l) const {
        Level& L = levels_[l];
        if (l + 1 == levels_.size()) {
            if (L.n == 1) L.x[0] = L.b[0] / (alpha_ + 4.0 * L.s);
            else
                for (int s = 0; s < 30; ++s) smooth(L, s % 2);
            return;
        }
        for (int s = 0; s < pre_; ++s) smooth(L, 0);
        residual(L);
        Level& C = levels_[l + 1];
        restrict_to(L, C);
        std::fill(C.x.begin(), C.x.end(), 0.0);
        cycle(l + 1);
        prolong_add(C, L);
        for (int s = 0; s < post_; ++s) smooth(L, 1);
    }
    mutable std::vector<Level> levels_;

private:
    double alpha_;
    int pre_, post_;
};

// ---------------------------------------------------------------- Burgers2D (problems/burgers2d.hpp)
// One implicit-Euler step of 2D viscous Burgers with a manufactured root:
// F(w) = w/dt + (u u_x + v u_y, u v_x + v v_y) - nu Lap_h w - g, w = (u, v) on n^2 interior
// points each, central differences, homogeneous Dirichlet; g makes w* = a (sin pi x sin pi y,
// sin 2 pi x sin pi y) an exact discrete root (burgers2d.hpp:25-52).
struct Burgers {
    std::size_t n;
    double nu, dt, amp;
    DVec source, exact;

    Burgers(std::size_t n_, double nu_, double dt_, double amp_) : n(n_), nu(nu_), dt(dt_), amp(amp_) {
        if (n == 0 || !(nu > 0.0) || !(dt > 0.0) || !std::isfinite(nu) || !std::isfinite(dt) || !std::isfinite(amp))
            throw std::invalid_argument("Burgers2D: invalid n, nu or dt");
        const double pi = std::acos(-1.0);
        const double h = 1.0 / (static_cast<double>(n) + 1.0);
        const std::size_t nn = n * n;
        exact.assign(2 * nn, 0.0);
        for (std::size_t i = 0; i < n; ++i)
            for (std::size_t j = 0; j < n; ++j) {
                const double y = (static_cast<double>(i) + 1.0) * h;
                const double x = (static_cast<double>(j) + 1.0) * h;
                exact[i * n + j] = amp * std::sin(pi * x) * std::sin(pi * y);
                exact[nn + i * n + j] = amp * std::sin(2.0 * pi * x) * std::sin(pi * y);
            }
        DVec g;
        eval_raw(exact, g);
        source = std::move(g);
    }
    std::size_t size() const { return 2 * n * n; }

    double at(const DVec& a, std::size_t comp, long i, long j) const {
        if (i < 0 || j < 0 || i >= static_cast<long>(n) || j >= static_cast<long>(n)) return 0.0;
        return a[comp * n * n + static_cast<std::size_t>(i) * n + static_cast<std::size_t>(j)];
    }

    // (burgers2d.hpp:169-210)
    void eval_raw(const DVec& w, DVec& out) const {
        const std::size_t nn = n * n;
        const double h = 1.0 / (static_cast<double>(n) + 1.0);
        const double inv2h = 1.0 / (2.0 * h), invh2 = 1.0 / (h * h), invdt = 1.0 / dt;
        out.assign(size(), 0.0);
#pragma omp parallel for schedule(static) if (nn > 4096)
        for (long i = 0; i < static_cast<long>(n); ++i)
            for (long j = 0; j < static_cast<long>(n); ++j) {
                const std::size_t p = static_cast<std::size_t>(i) * n + static_cast<std::size_t>(j);
                const double u = w[p], v = w[nn + p];
                const double ux = (at(w, 0, i, j + 1) - at(w, 0, i, j - 1)) * inv2h;
                const double uy = (at(w, 0, i + 1, j) - at(w, 0, i - 1, j)) * inv2h;
                const double vx = (at(w, 1, i, j + 1) - at(w, 1, i, j - 1)) * inv2h;
                const double vy = (at(w, 1, i + 1, j) - at(w, 1, i - 1, j)) * inv2h;
                const double lu = (at(w, 0, i, j + 1) + at(w, 0, i, j - 1) + at(w, 0, i + 1, j) + at(w, 0, i - 1, j) -
                                   4.0 * u) * invh2;
                const double lv = (at(w, 1, i, j + 1) + at(w, 1, i, j - 1) + at(w, 1, i + 1, j) + at(w, 1, i - 1, j) -
                                   4.0 * v) * invh2;
                out[p] = invdt * u + u * ux + v * uy - nu * lu;
                out[nn + p] = invdt * v + u * vx + v * vy - nu * lv;
            }
    }
    void eval(const DVec& w, DVec& out) const {
        eval_raw(w, out);
        for (std::size_t q = 0; q < out.size(); ++q) out[q] -= source[q];
    }
    // (burgers2d.hpp:71-123)
    void jvp(const DVec& w, const DVec& d, DVec& out) const {
        const std::size_t nn = n * n;
        const double h = 1.0 / (static_cast<double>(n) + 1.0);
        const double inv2h = 1.0 / (2.0 * h), invh2 = 1.0 / (h * h), invdt = 1.0 / dt;
        out.assign(size(), 0.0);
#pragma omp parallel for schedule(static) if (nn > 4096)
        for (long i = 0; i < static_cast<long>(n); ++i)
            for (long j = 0; j < static_cast<long>(n); ++j) {
                const std::size_t p = static_cast<std::size_t>(i) * n + static_cast<std::size_t>(j);
                const double u = w[p], v = w[nn + p], du = d[p], dv = d[nn + p];
                const double ux = (at(w, 0, i, j + 1) - at(w, 0, i, j - 1)) * inv2h;
                const double uy = (at(w, 0, i + 1, j) - at(w, 0, i - 1, j)) * inv2h;
                const double vx = (at(w, 1, i, j + 1) - at(w, 1, i, j - 1)) * inv2h;
                const double vy = (at(w, 1, i + 1, j) - at(w, 1, i - 1, j)) * inv2h;
                const double dux = (at(d, 0, i, j + 1) - at(d, 0, i, j - 1)) * inv2h;
                const double duy = (at(d, 0, i + 1, j) - at(d, 0, i - 1, j)) * inv2h;
                const double dvx = (at(d, 1, i, j + 1) - at(d, 1, i, j - 1)) * inv2h;
                const double dvy = (at(d, 1, i + 1, j) - at(d, 1, i - 1, j)) * inv2h;
                const double ldu = (at(d, 0, i, j + 1) + at(d, 0, i, j - 1) + at(d, 0, i + 1, j) + at(d, 0, i - 1, j) -
                                    4.0 * du) * invh2;
                const double ldv = (at(d, 1, i, j + 1) + at(d, 1, i, j - 1) + at(d, 1, i + 1, j) + at(d, 1, i - 1, j) -
                                    4.0 * dv) * invh2;
                out[p] = invdt * du + du * ux + u * dux + dv * uy + v * duy - nu * ldu;
                out[nn + p] = invdt * dv + du * vx + u * dvx + dv * vy + v * dvy - nu * ldv;
            }
    }
    // exact second derivative 2 (du dux + dv duy, du dvx + dv dvy) (burgers2d.hpp:125-160)
    void d2(const DVec& w, const DVec& d, DVec& out) const {
        (void)w;
        const std::size_t nn = n * n;
        const double h = 1.0 / (static_cast<double>(n) + 1.0);
        const double inv2h = 1.0 / (2.0 * h);
        out.assign(size(), 0.0);
#pragma omp parallel for schedule(static) if (nn > 4096)
        for (long i = 0; i < static_cast<long>(n); ++i)
            for (long j = 0; j < static_cast<long>(n); ++j) {
                const std::size_t p = static_cast<std::size_t>(i) * n + static_cast<std::size_t>(j);
                const double du = d[p], dv = d[nn + p];
                const double dux = (at(d, 0, i, j + 1) - at(d, 0, i, j - 1)) * inv2h;
                const double duy = (at(d, 0, i + 1, j) - at(d, 0, i - 1, j)) * inv2h;
                const double dvx = (at(d, 1, i, j + 1) - at(d, 1, i, j - 1)) * inv2h;
                const double dvy = (at(d, 1, i + 1, j) - at(d, 1, i - 1, j)) * inv2h;
                out[p] = 2.0 * (du * dux + dv * duy);
                out[nn + p] = 2.0 * (du * dvx + dv * dvy);
            }
    }
};

struct BurgersOp {
    const Burgers& f;
    int jvp_mode, d2_mode;
    Timers* timers;
    std::size_t size() const { return f.size(); }
    void eval(const DVec& x, DVec& out) const {
        auto t0 = Clock::now();
        f.eval(x, out);
        timers->t_F += seconds_since(t0);
    }
    void jvp(const DVec& x, const DVec& v, DVec& out) const {
        auto t0 = Clock::now();
        if (jvp_mode == 1) jvp_fd(f, x, v, out); else f.jvp(x, v, out);
        timers->t_JVP += seconds_since(t0);
    }
    void d2(const DVec& x, const DVec& v, DVec& out) const {
        auto t0 = Clock::now();
        if (d2_mode == 1) d2_fd(f, x, v, out); else f.d2(x, v, out);
        timers->t_D2 += seconds_since(t0);
    }
};

// ---------------------------------------------------------------- Brusselator1DStep (problems/brusselator1d.hpp)
// One implicit-Euler step of the 1D Brusselator, w = (u, v) on n interior points each, Dirichlet
// u = A = 1, v = B = 3, alpha = 1/50, previous state u = 1 + sin(2 pi x), v = 3
// (brusselator1d.hpp:22-45).  Expressions are written in the reference's order of operations.
struct Bruss1D {
    static constexpr double A = 1.0, B = 3.0, alpha = 1.0 / 50.0;
    std::size_t n;
    double dt, h, h2inv;
    DVec prev;

    Bruss1D(std::size_t n_, double dt_) : n(n_), dt(dt_), h(1.0 / (static_cast<double>(n_) + 1.0)) {
        if (n == 0 || !(dt > 0.0) || !std::isfinite(dt)) throw std::invalid_argument("Brusselator1DStep: n, dt");
        h2inv = 1.0 / (h * h);
        prev.assign(2 * n, 0.0);
        const double pi = std::acos(-1.0);
        for (std::size_t i = 0; i < n; ++i) {
            const double x = (static_cast<double>(i) + 1.0) * h;
            prev[i] = 1.0 + std::sin(2.0 * pi * x);
            prev[n + i] = 3.0;
        }
    }
    std::size_t size() const { return 2 * n; }
    // boundary values u = 1, v = 3 for the state (:144-149), zero for a direction (:151-154)
    double val(const DVec& w, std::size_t c, long i) const {
        if (i < 0 || i >= static_cast<long>(n)) return c == 0 ? 1.0 : 3.0;
        return w[c * n + static_cast<std::size_t>(i)];
    }
    double dir(const DVec& d, std::size_t c, long i) const {
        if (i < 0 || i >= static_cast<long>(n)) return 0.0;
        return d[c * n + static_cast<std::size_t>(i)];
    }
    // (:47-69)
    void eval(const DVec& w, DVec& out) const {
        out.assign(size(), 0.0);
        const double invdt = 1.0 / dt;
#pragma omp parallel for schedule(static) if (n > 4096)
        for (long i = 0; i < static_cast<long>(n); ++i) {
            const std::size_t q = static_cast<std::size_t>(i);
            const double u = w[q], v = w[n + q];
            const double lu = (val(w, 0, i - 1) - 2.0 * u + val(w, 0, i + 1)) * h2inv;
            const double lv = (val(w, 1, i - 1) - 2.0 * v + val(w, 1, i + 1)) * h2inv;
            out[q] = (u - prev[q]) * invdt - alpha * lu - A - u * u * v + (B + 1.0) * u;
            out[n + q] = (v - prev[n + q]) * invdt - alpha * lv - B * u + u * u * v;
        }
    }
    // (:71-98)
    void jvp(const DVec& w, const DVec& d, DVec& out) const {
        out.assign(size(), 0.0);
        const double invdt = 1.0 / dt;
#pragma omp parallel for schedule(static) if (n > 4096)
        for (long i = 0; i < static_cast<long>(n); ++i) {
            const std::size_t q = static_cast<std::size_t>(i);
            const double u = w[q], v = w[n + q], du = d[q], dv = d[n + q];
            const double ldu = (dir(d, 0, i - 1) - 2.0 * du + dir(d, 0, i + 1)) * h2inv;
            const double ldv = (dir(d, 1, i - 1) - 2.0 * dv + dir(d, 1, i + 1)) * h2inv;
            out[q] = invdt * du - alpha * ldu - (2.0 * u * v) * du - u * u * dv + (B + 1.0) * du;
            out[n + q] = invdt * dv - alpha * ldv - B * du + (2.0 * u * v) * du + u * u * dv;
        }
    }
    // (:100-118)
    void d2(const DVec& w, const DVec& d, DVec& out) const {
        out.assign(size(), 0.0);
        for (std::size_t i = 0; i < n; ++i) {
            const double u = w[i], v = w[n + i], du = d[i], dv = d[n + i];
            const double q = 2.0 * v * du * du + 4.0 * u * du * dv;
            out[i] = -q;
            out[n + i] = q;
        }
    }
    // 2x2 point blocks of the Jacobian without the off-diagonal diffusion (:120-141)
    void blocks(const DVec& w, DVec& a11, DVec& a12, DVec& a21, DVec& a22) const {
        a11.resize(n);
        a12.resize(n);
        a21.resize(n);
        a22.resize(n);
        const double base = 1.0 / dt + 2.0 * alpha * h2inv;
        for (std::size_t i = 0; i < n; ++i) {
            const double u = w[i], v = w[n + i];
            a11[i] = base - 2.0 * u * v + (B + 1.0);
            a12[i] = -u * u;
            a21[i] = -B + 2.0 * u * v;
            a22[i] = base + u * u;
        }
    }
};

// BrusselatorJacobi::Bound: z = block^-1 r per point, z = r where the determinant is not finite
// or below 1e-14 in magnitude (brusselator1d.hpp:194-222).
static void bruss_block_apply(const DVec& a11, const DVec& a12, const DVec& a21, const DVec& a22, const DVec& r,
                              DVec& z) {
    const std::size_t n = a11.size();
    z.assign(2 * n, 0.0);
    for (std::size_t i = 0; i < n; ++i) {
        const double det = a11[i] * a22[i] - a12[i] * a21[i];
        if (!std::isfinite(det) || std::abs(det) < 1e-14) {
            z[i] = r[i];
            z[n + i] = r[n + i];
            continue;
        }
        z[i] = (a22[i] * r[i] - a12[i] * r[n + i]) / det;
        z[n + i] = (-a21[i] * r[i] + a11[i] * r[n + i]) / det;
    }
}

// ---------------------------------------------------------------- Brusselator2D (periodic, this project's)
// Implicit-Euler step of the 2-species Brusselator on an n x n periodic grid of the unit square
// (h = 1/n): the reaction terms of brusselator1d.hpp:47-98 with parameters A, B, D_u, D_v, dt and
// the 5-point Laplacian as a sum of neighbour differences.  w = (u, v) component-major, row-major planes.
// The reference has no 2D Brusselator: this restatement is the checker of the GPU form only.
struct Bruss2DParams {
    double A, B, Du, Dv, dt;
};

struct Bruss2D {
    std::size_t n;
    Bruss2DParams P;
    double h2inv;
    DVec prev;

    Bruss2D(std::size_t n_, const Bruss2DParams& p, const double* prev_) : n(n_), P(p) {
        if (n < 3 || !(P.dt > 0.0) || !(P.Du >= 0.0) || !(P.Dv >= 0.0)) throw std::invalid_argument("Brusselator2D");
        h2inv = static_cast<double>(n) * static_cast<double>(n);
        prev.assign(prev_, prev_ + 2 * n * n);
    }
    std::size_t size() const { return 2 * n * n; }
    std::size_t up(std::size_t i) const { return i + 1 == n ? 0 : i + 1; }
    std::size_t dn(std::size_t i) const { return i == 0 ? n - 1 : i - 1; }
    // ((W - c) + (E - c)) + ((S - c) + (N - c)) (h^-2 D is applied by the caller): neighbouring values of a smooth state
    // are within a factor of two, so every difference is exact and the rounding floor of F stays far
    // below the residuals a time step asks for (the form Sum - 4c cancels values near 1 and then
    // multiplies the rounding by D h^-2).
    double lap(const double* a, std::size_t i, std::size_t j) const {
        const double c = a[i * n + j];
        return ((a[i * n + dn(j)] - c) + (a[i * n + up(j)] - c)) + ((a[dn(i) * n + j] - c) + (a[up(i) * n + j] - c));
    }
    // F_u = fma(B+1, u, fma(-u^2, v, fma(-D_u h^-2, L u, fma(u - u_prev, 1/dt, -A))))
    // F_v = fma(u^2, v, fma(-B, u, fma(-D_v h^-2, L v, (v - v_prev) / dt)))   (L: lap without h^-2)
    void eval(const DVec& w, DVec& out) const {
        const std::size_t nn = n * n;
        const double invdt = 1.0 / P.dt, Bp1 = P.B + 1.0, duh = P.Du * h2inv, dvh = P.Dv * h2inv;
        out.assign(size(), 0.0);
#pragma omp parallel for schedule(static) if (nn > 4096)
        for (long ii = 0; ii < static_cast<long>(n); ++ii)
            for (std::size_t j = 0; j < n; ++j) {
                const std::size_t i = static_cast<std::size_t>(ii), p = i * n + j;
                const double u = w[p], v = w[nn + p], uu = u * u;
                const double lu = lap(w.data(), i, j), lv = lap(w.data() + nn, i, j);
                out[p] = std::fma(Bp1, u, std::fma(-uu, v, std::fma(-duh, lu, std::fma(u - prev[p], invdt, -P.A))));
                out[nn + p] = std::fma(uu, v, std::fma(-P.B, u, std::fma(-dvh, lv, (v - prev[nn + p]) * invdt)));
            }
    }
    // J d with the point block [[c1 - 2uv, -u^2], [2uv - B, 1/dt + u^2]], c1 = 1/dt + (B + 1):
    // (J d)_u = fma(-u^2, dv, fma(-D_u h^-2, L du, a11 du)), (J d)_v = fma(a22, dv, fma(a21, du, -D_v h^-2 L dv))
    void jvp(const DVec& w, const DVec& d, DVec& out) const {
        const std::size_t nn = n * n;
        const double invdt = 1.0 / P.dt, c1 = invdt + (P.B + 1.0), duh = P.Du * h2inv, dvh = P.Dv * h2inv;
        out.assign(size(), 0.0);
#pragma omp parallel for schedule(static) if (nn > 4096)
        for (long ii = 0; ii < static_cast<long>(n); ++ii)
            for (std::size_t j = 0; j < n; ++j) {
                const std::size_t i = static_cast<std::size_t>(ii), p = i * n + j;
                const double u = w[p], v = w[nn + p], du = d[p], dv = d[nn + p];
                const double lu = lap(d.data(), i, j), lv = lap(d.data() + nn, i, j);
                const double u2 = 2.0 * u, uu = u * u;
                const double a11 = std::fma(-u2, v, c1), a21 = std::fma(u2, v, -P.B), a22 = invdt + uu;
                out[p] = std::fma(-uu, dv, std::fma(-duh, lu, a11 * du));
                out[nn + p] = std::fma(a22, dv, std::fma(a21, du, -dvh * lv));
            }
    }
    void d2(const DVec& w, const DVec& d, DVec& out) const {
        const std::size_t nn = n * n;
        out.assign(size(), 0.0);
        for (std::size_t p = 0; p < nn; ++p) {
            const double u = w[p], v = w[nn + p], du = d[p], dv = d[nn + p];
            const double q = 2.0 * v * du * du + 4.0 * u * du * dv;
            out[p] = -q;
            out[nn + p] = q;
        }
    }
};

// Periodic geometric multigrid for the coupled 2x2 block K(x) - diag(D_u, D_v) Lap_h of the
// Brusselator2D Jacobian (this project's design; the reference's only Brusselator
// preconditioner is the point-block Jacobi above).  Levels halve n while the coarse n is even
// and >= 4; K = [[1/dt + B + 1 - 2uv, -u^2], [2uv - B, 1/dt + u^2]] at the fine level from the
// Newton iterate, full-weighting restricted to the coarse levels; red-black point-block
// Gauss-Seidel (colour (i+j)&1), pre-smoothing colours 0,1, post-smoothing 1,0; residual and
// full weighting (9-point, periodic), bilinear periodic prolongation added; the coarsest level
// takes 30 sweeps from zero.
class BrussMG2D {
public:
    struct Level {
        std::size_t n;
        double su, sv;
        DVec xu, xv, bu, bv, k11, k12, k21, k22;
    };

    BrussMG2D(std::size_t n, const Bruss2DParams& p, int pre = 2, int post = 2) : P_(p), pre_(pre), post_(post) {
        if (n < 4 || n % 2 != 0) throw std::invalid_argument("BrussMG2D needs an even n >= 4");
        std::size_t m = n;
        for (;;) {
            Level L;
            L.n = m;
            L.su = P_.Du * (static_cast<double>(m) * static_cast<double>(m));
            L.sv = P_.Dv * (static_cast<double>(m) * static_cast<double>(m));
            const std::size_t mm = m * m;
            for (DVec* a : {&L.xu, &L.xv, &L.bu, &L.bv, &L.k11, &L.k12, &L.k21, &L.k22}) a->assign(mm, 0.0);
            levels_.push_back(std::move(L));
            if (m % 4 != 0 || m / 2 < 4) break;
            m /= 2;
        }
    }
    std::size_t levels() const { return levels_.size(); }

    // K at the fine level from w = (u, v), restricted to every coarser level.
    void set_state(const DVec& w) {
        Level& F = levels_[0];
        const std::size_t nn = F.n * F.n;
        const double c1 = 1.0 / P_.dt + (P_.B + 1.0), c2 = 1.0 / P_.dt;
        for (std::size_t p = 0; p < nn; ++p) {
            const double u = w[p], v = w[nn + p];
            F.k11[p] = c1 - (2.0 * u) * v;
            F.k12[p] = -(u * u);
            F.k21[p] = (2.0 * u) * v - P_.B;
            F.k22[p] = c2 + u * u;
        }
        for (std::size_t l = 0; l + 1 < levels_.size(); ++l) {
            Level& f = levels_[l];
            Level& c = levels_[l + 1];
            fw(f.n, f.k11, c.k11);
            fw(f.n, f.k12, c.k12);
            fw(f.n, f.k21, c.k21);
            fw(f.n, f.k22, c.k22);
        }
    }

    void apply(const DVec& r, DVec& z) {
        Level& F = levels_[0];
        const std::size_t nn = F.n * F.n;
        std::copy(r.begin(), r.begin() + nn, F.bu.begin());
        std::copy(r.begin() + nn, r.begin() + 2 * nn, F.bv.begin());
        cycle(0);
        z.resize(2 * nn);
        std::copy(F.xu.begin(), F.xu.end(), z.begin());
        std::copy(F.xv.begin(), F.xv.end(), z.begin() + nn);
    }

    // ((4c + 2((W + E) + (S + N))) + (((SW + SE) + NW) + NE)) / 16 at fine (2I, 2J), periodic.
    static void fw(std::size_t nf, const DVec& f, DVec& c) {
        const std::size_t nc = nf / 2;
        for (std::size_t I = 0; I < nc; ++I)
            for (std::size_t J = 0; J < nc; ++J) {
                const std::size_t i = 2 * I, j = 2 * J;
                const std::size_t im = i == 0 ? nf - 1 : i - 1, ip = i + 1, jm = j == 0 ? nf - 1 : j - 1, jp = j + 1;
                const double ctr = f[i * nf + j];
                const double edge = (f[i * nf + jm] + f[i * nf + jp]) + (f[im * nf + j] + f[ip * nf + j]);
                const double corner = ((f[im * nf + jm] + f[im * nf + jp]) + f[ip * nf + jm]) + f[ip * nf + jp];
                c[I * nc + J] = ((4.0 * ctr + 2.0 * edge) + corner) * 0.0625;
            }
    }

private:
    static double nsum(const DVec& a, std::size_t n, std::size_t i, std::size_t j) {
        const std::size_t im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
        const std::size_t jm = j == 0 ? n - 1 : j - 1, jp = j + 1 == n ? 0 : j + 1;
        return ((a[i * n + jm] + a[i * n + jp]) + a[im * n + j]) + a[ip * n + j];
    }
    void smooth(Level& L, int colour) {
        const std::size_t n = L.n;
        for (std::size_t i = 0; i < n; ++i)
            for (std::size_t j = (i + colour) & 1; j < n; j += 2) {
                const std::size_t p = i * n + j;
                const double ru = L.bu[p] + L.su * nsum(L.xu, n, i, j);
                const double rv = L.bv[p] + L.sv * nsum(L.xv, n, i, j);
                const double m11 = L.k11[p] + 4.0 * L.su, m22 = L.k22[p] + 4.0 * L.sv;
                const double det = m11 * m22 - L.k12[p] * L.k21[p];
                L.xu[p] = (m22 * ru - L.k12[p] * rv) / det;
                L.xv[p] = (m11 * rv - L.k21[p] * ru) / det;
            }
    }
    void cycle(std::size_t l) {
        Level& L = levels_[l];
        std::fill(L.xu.begin(), L.xu.end(), 0.0);
        std::fill(L.xv.begin(), L.xv.end(), 0.0);
        if (l + 1 == levels_.size()) {
            for (int s = 0; s < 30; ++s) {
                smooth(L, 0);
                smooth(L, 1);
            }
            return;
        }
        for (int s = 0; s < pre_; ++s) {
            smooth(L, 0);
            smooth(L, 1);
        }
        const std::size_t n = L.n, nn = n * n;
        DVec ru(nn), rv(nn);
        for (std::size_t i = 0; i < n; ++i)
            for (std::size_t j = 0; j < n; ++j) {
                const std::size_t p = i * n + j;
                const double u = L.xu[p], v = L.xv[p];
                ru[p] = L.bu[p] - ((L.k11[p] * u + L.k12[p] * v) + L.su * (4.0 * u - nsum(L.xu, n, i, j)));
                rv[p] = L.bv[p] - ((L.k21[p] * u + L.k22[p] * v) + L.sv * (4.0 * v - nsum(L.xv, n, i, j)));
            }
        Level& C = levels_[l + 1];
        fw(n, ru, C.bu);
        fw(n, rv, C.bv);
        cycle(l + 1);
        prolong_add(C.n, C.xu, L.xu);
        prolong_add(C.n, C.xv, L.xv);
        for (int s = 0; s < post_; ++s) {
            smooth(L, 1);
            smooth(L, 0);
        }
    }
    // fine (2I, 2J) += c; (2I+1, 2J) += (c + c_{I+1}) / 2; (2I, 2J+1) += (c + c_{J+1}) / 2;
    // (2I+1, 2J+1) += (((c + c_{I+1}) + c_{J+1}) + c_{I+1,J+1}) / 4, periodic.
    static void prolong_add(std::size_t nc, const DVec& c, DVec& f) {
        const std::size_t nf = 2 * nc;
        for (std::size_t I = 0; I < nc; ++I)
            for (std::size_t J = 0; J < nc; ++J) {
                const std::size_t I1 = I + 1 == nc ? 0 : I + 1, J1 = J + 1 == nc ? 0 : J + 1;
                const double c00 = c[I * nc + J], c10 = c[I1 * nc + J], c01 = c[I * nc + J1], c11 = c[I1 * nc + J1];
                f[(2 * I) * nf + 2 * J] += c00;
                f[(2 * I + 1) * nf + 2 * J] += 0.5 * (c00 + c10);
                f[(2 * I) * nf + 2 * J + 1] += 0.5 * (c00 + c01);
                f[(2 * I + 1) * nf + 2 * J + 1] += 0.25 * (((c00 + c10) + c01) + c11);
            }
    }

    Bruss2DParams P_;
    int pre_, post_;
    std::vector<Level> levels_;
};

template <class F>
struct GenericOp {
    const F& f;
    int jvp_mode, d2_mode;
    Timers* timers;
    std::size_t size() const { return f.size(); }
    void eval(const DVec& x, DVec& out) const {
        auto t0 = Clock::now();
        f.eval(x, out);
        timers->t_F += seconds_since(t0);
    }
    void jvp(const DVec& x, const DVec& v, DVec& out) const {
        auto t0 = Clock::now();
        if (jvp_mode == 1) jvp_fd(f, x, v, out); else f.jvp(x, v, out);
        timers->t_JVP += seconds_since(t0);
    }
    void d2(const DVec& x, const DVec& v, DVec& out) const {
        auto t0 = Clock::now();
        if (d2_mode == 1) d2_fd(f, x, v, out); else f.d2(x, v, out);
        timers->t_D2 += seconds_since(t0);
    }
};

// ---------------------------------------------------------------- preconditioner providers
constexpr int kBurgersMG = 3;

// A bound preconditioner is "z = M^-1 r"; make(x) binds it at a nonlinear iterate
// (krylov_newton.hpp:20-22, poisson_mg.hpp:303-320, bratu3d.hpp:104-120).
struct Provider {
    int kind = 0;  // numa_gpu_precond_kind, or kBurgersMG
    const Bratu* f = nullptr;
    std::shared_ptr<PoissonMG> mg;
    std::shared_ptr<HelmholtzMG2D> hmg;  // BurgersMGProvider (burgers2d.hpp:220-246)
    const Bruss1D* bf = nullptr;         // BrusselatorJacobi (brusselator1d.hpp:194-222)
    std::shared_ptr<BrussMG2D> bmg;      // Brusselator2D coupled-block multigrid
    std::size_t nn = 0;
    DVec diag, a11, a12, a21, a22;
    Timers* timers = nullptr;

    void make(const DVec& x) {
        auto t0 = Clock::now();
        if (kind == NUMA_GPU_PRECOND_JACOBI) f->jacobi_diag(x, diag);
        if (kind == NUMA_GPU_PRECOND_BRUSS_JACOBI) bf->blocks(x, a11, a12, a21, a22);
        if (kind == NUMA_GPU_PRECOND_BRUSS_MG) bmg->set_state(x);
        if (timers) timers->t_setup += seconds_since(t0);
    }
    void operator()(const DVec& r, DVec& z) const {
        auto t0 = Clock::now();
        if (kind == NUMA_GPU_PRECOND_BRUSS_JACOBI) {
            bruss_block_apply(a11, a12, a21, a22, r, z);
        } else if (kind == NUMA_GPU_PRECOND_BRUSS_MG) {
            bmg->apply(r, z);
        } else if (kind == NUMA_GPU_PRECOND_POISSON_MG) {
            mg->apply(r, z);
        } else if (kind == kBurgersMG) {
            DVec ru(r.begin(), r.begin() + nn), rv(r.begin() + nn, r.end()), zu, zv;
            hmg->apply(ru, zu);
            hmg->apply(rv, zv);
            z.resize(r.size());
            std::copy(zu.begin(), zu.end(), z.begin());
            std::copy(zv.begin(), zv.end(), z.begin() + nn);
        } else if (kind == NUMA_GPU_PRECOND_JACOBI) {
            z.resize(r.size());
            for (std::size_t p = 0; p < r.size(); ++p) z[p] = r[p] / diag[p];
        } else {
            z = r;
        }
        if (timers) timers->t_prec += seconds_since(t0);
    }
};

// ---------------------------------------------------------------- GMRES (linalg/gmres.hpp)
struct GmresResult {
    std::size_t iters = 0, matvecs = 0, precs = 0;
    double rel_res = 0.0;
    bool converged = false, breakdown = false;
};

struct KrylovSpace {
    std::vector<DVec> V;
    std::vector<std::vector<double>> Hbar;
    std::size_t k = 0;
    void clear() { V.clear(); Hbar.clear(); k = 0; }
};

// Restarted right-preconditioned GMRES(m), modified Gram-Schmidt Arnoldi, Givens rotations
// (gmres.hpp:61-223).  The matvec counter includes restart residuals; each cycle ends with one
// more preconditioner application to V y.
template <class Apply, class Precond>
static GmresResult gmres(const Apply& A, const Precond& M, const DVec& b, DVec& x, double rtol,
                         std::size_t m, std::size_t max_iters, bool zero_guess = true,
                         KrylovSpace* save = nullptr, const DVec* r_init = nullptr) {
    const std::size_t N = b.size();
    GmresResult res;
    if (save) save->clear();
    const double bnorm = norm2(b);
    if (bnorm == 0.0) { x.assign(N, 0.0); res.converged = true; return res; }
    if (m == 0) { res.rel_res = 1.0; res.breakdown = true; return res; }
    if (max_iters == 0) { res.rel_res = 1.0; return res; }
    if (r_init && r_init->size() != N) { res.rel_res = 1.0; res.breakdown = true; return res; }
    if (zero_guess) x.assign(N, 0.0);

    DVec r(N), w(N), z(N), comb(N);
    std::vector<DVec> V(m + 1, DVec(N));
    std::vector<std::vector<double>> H(m + 1, std::vector<double>(m, 0.0));
    std::vector<std::vector<double>> Hraw(m + 1, std::vector<double>(m, 0.0));
    std::vector<double> cs(m), sn(m), g(m + 1), y(m);

    bool given = r_init != nullptr;
    bool first = zero_guess;
    std::size_t k_last = 0;

    while (res.iters < max_iters) {
        if (given) { r = *r_init; given = false; first = false; }
        else if (first) { r = b; first = false; }
        else {
            A(x, w);
            ++res.matvecs;
            for (std::size_t p = 0; p < N; ++p) r[p] = b[p] - w[p];
        }
        const double beta = norm2(r);
        res.rel_res = beta / bnorm;
        if (res.rel_res <= rtol) { res.converged = true; k_last = 0; break; }

        for (auto& row : Hraw) std::fill(row.begin(), row.end(), 0.0);
        for (std::size_t p = 0; p < N; ++p) V[0][p] = r[p] / beta;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;

        std::size_t k = 0;
        k_last = 0;
        while (k < m && res.iters < max_iters) {
            const std::size_t j = k;
            M(V[j], z);
            ++res.precs;
            A(z, w);
            ++res.matvecs;
            for (std::size_t i = 0; i <= j; ++i) {
                H[i][j] = dot(w, V[i]);
                axpy(-H[i][j], V[i], w);
            }
            H[j + 1][j] = norm2(w);
            if (H[j + 1][j] > 0.0) {
                for (std::size_t p = 0; p < N; ++p) V[j + 1][p] = w[p] / H[j + 1][j];
            } else {
                std::fill(V[j + 1].begin(), V[j + 1].end(), 0.0);
            }
            for (std::size_t i = 0; i <= j + 1; ++i) Hraw[i][j] = H[i][j];
            for (std::size_t i = 0; i < j; ++i) {
                const double t = cs[i] * H[i][j] + sn[i] * H[i + 1][j];
                H[i + 1][j] = -sn[i] * H[i][j] + cs[i] * H[i + 1][j];
                H[i][j] = t;
            }
            const double den = std::hypot(H[j][j], H[j + 1][j]);
            if (!(den > 0.0) || !std::isfinite(den)) { res.breakdown = true; return res; }
            cs[j] = H[j][j] / den;
            sn[j] = H[j + 1][j] / den;
            H[j][j] = den;
            H[j + 1][j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++k;
            ++res.iters;
            k_last = k;
            res.rel_res = std::abs(g[j + 1]) / bnorm;
            if (res.rel_res <= rtol) break;
        }
        for (std::size_t ii = k; ii-- > 0;) {
            const double piv = H[ii][ii];
            if (!(std::abs(piv) > 0.0) || !std::isfinite(piv)) { res.breakdown = true; return res; }
            double s = g[ii];
            for (std::size_t jj = ii + 1; jj < k; ++jj) s -= H[ii][jj] * y[jj];
            y[ii] = s / piv;
        }
        std::fill(comb.begin(), comb.end(), 0.0);
        for (std::size_t i = 0; i < k; ++i) axpy(y[i], V[i], comb);
        M(comb, z);
        ++res.precs;
        axpy(1.0, z, x);
        if (res.rel_res <= rtol) { res.converged = true; break; }
    }
    if (save && k_last > 0) {
        save->k = k_last;
        save->V = V;
        save->Hbar.assign(k_last + 1, std::vector<double>(k_last, 0.0));
        for (std::size_t i = 0; i <= k_last; ++i)
            for (std::size_t j = 0; j < k_last; ++j) save->Hbar[i][j] = Hraw[i][j];
    }
    return res;
}

static bool space_usable(const KrylovSpace& s, std::size_t N) {
    if (s.k == 0 || s.V.size() < s.k + 1 || s.Hbar.size() < s.k + 1) return false;
    for (std::size_t i = 0; i <= s.k; ++i)
        if (s.Hbar[i].size() < s.k) return false;
    for (std::size_t i = 0; i <= s.k; ++i)
        if (s.V[i].size() != N) return false;
    return true;
}

// Second solve with the same A and M: least-squares projection of b on the saved space
// (k+1 dots, QR of Hbar by Givens), initial guess M^-1 V y, residual b - V Hbar y, then GMRES
// from that residual; falls back to a fresh GMRES if the space is unusable or singular
// (gmres.hpp:229-323).
template <class Apply, class Precond>
static GmresResult gmres_recycled(const Apply& A, const Precond& M, const DVec& b, DVec& x,
                                  double rtol, std::size_t m, std::size_t max_iters,
                                  const KrylovSpace& sp, KrylovSpace* save = nullptr) {
    const std::size_t k = sp.k, N = b.size();
    x.assign(N, 0.0);
    if (!space_usable(sp, N)) return gmres(A, M, b, x, rtol, m, max_iters, true, save);
    std::vector<double> rhs(k + 1, 0.0);
    for (std::size_t i = 0; i <= k; ++i) rhs[i] = dot(sp.V[i], b);
    auto R = sp.Hbar;
    std::vector<double> cs(k, 0.0), sn(k, 0.0);
    for (std::size_t j = 0; j < k; ++j) {
        for (std::size_t i = 0; i < j; ++i) {
            const double t = cs[i] * R[i][j] + sn[i] * R[i + 1][j];
            R[i + 1][j] = -sn[i] * R[i][j] + cs[i] * R[i + 1][j];
            R[i][j] = t;
        }
        const double den = std::hypot(R[j][j], R[j + 1][j]);
        if (!(den > 0.0) || !std::isfinite(den)) return gmres(A, M, b, x, rtol, m, max_iters, true, save);
        cs[j] = R[j][j] / den;
        sn[j] = R[j + 1][j] / den;
        R[j][j] = den;
        R[j + 1][j] = 0.0;
        const double t = cs[j] * rhs[j] + sn[j] * rhs[j + 1];
        rhs[j + 1] = -sn[j] * rhs[j] + cs[j] * rhs[j + 1];
        rhs[j] = t;
    }
    std::vector<double> y(k, 0.0);
    for (std::size_t ii = k; ii-- > 0;) {
        const double piv = R[ii][ii];
        if (!(std::abs(piv) > 0.0) || !std::isfinite(piv)) {
            x.assign(N, 0.0);
            return gmres(A, M, b, x, rtol, m, max_iters, true, save);
        }
        double s = rhs[ii];
        for (std::size_t jj = ii + 1; jj < k; ++jj) s -= R[ii][jj] * y[jj];
        y[ii] = s / piv;
    }
    DVec resid = b, comb(N, 0.0), x0(N, 0.0);
    for (std::size_t i = 0; i <= k; ++i) {
        double c = 0.0;
        for (std::size_t j = 0; j < k; ++j) c += sp.Hbar[i][j] * y[j];
        axpy(-c, sp.V[i], resid);
    }
    for (std::size_t j = 0; j < k; ++j) axpy(y[j], sp.V[j], comb);
    M(comb, x0);
    x = std::move(x0);
    GmresResult out = gmres(A, M, b, x, rtol, m, max_iters, false, save, &resid);
    ++out.precs;
    return out;
}

// ---------------------------------------------------------------- nonlinear drivers (methods/)
struct Params {
    double rtol_nl = 1e-8;
    std::size_t max_nl = 50;
    double eta_init = 0.5, eta_max = 0.9, gamma = 0.9, alpha = 2.0;
    double eta2_factor = 10.0, eta2_max = 0.5;
    std::size_t restart = 50, max_iters = 500;
    double armijo = 1e-4, min_lambda = 1e-4;
    bool recycle = false;
};

struct Result {
    DVec x;
    bool converged = false;
    std::size_t iters = 0, n_F = 0, n_JVP = 0, n_D2 = 0, n_lin_iters = 0, n_lin_failures = 0, n_prec = 0;
    double res0 = 0.0, res = 0.0;
};

// Eisenstat-Walker choice 2 with Kelley's safeguard and the oversolve floor
// 0.5 rtol_nl res0 / rnorm (krylov_newton.hpp:54-65).
static double forcing(const Params& p, std::size_t k, double rnorm, double rprev, double eta_prev,
                      double res0) {
    if (k == 0) return p.eta_init;
    double eta = p.gamma * std::pow(rnorm / rprev, p.alpha);
    const double safe = p.gamma * std::pow(eta_prev, p.alpha);
    if (safe > 0.1) eta = std::max(eta, safe);
    eta = std::min(eta, p.eta_max);
    eta = std::max(eta, 0.5 * p.rtol_nl * res0 / rnorm);
    return std::min(eta, p.eta_max);
}

// Inexact Newton with Armijo backtracking; J z = F, step x - lambda z (krylov_newton.hpp:69-114).
template <class Op>
static Result newton_krylov(const Op& f, DVec x, const Params& p, Provider& pc) {
    const std::size_t N = f.size();
    Result out;
    DVec Fx(N), Fn(N), z(N), xn(N);
    f.eval(x, Fx); ++out.n_F;
    double rnorm = norm2(Fx);
    out.res0 = rnorm;
    double rprev = rnorm, eta_prev = p.eta_init;
    for (std::size_t k = 0; k < p.max_nl; ++k) {
        if (rnorm <= p.rtol_nl * out.res0) { out.converged = true; break; }
        const double eta = forcing(p, k, rnorm, rprev, eta_prev, out.res0);
        pc.make(x);
        auto A = [&](const DVec& v, DVec& o) { f.jvp(x, v, o); };
        z.assign(N, 0.0);
        const GmresResult g = gmres(A, pc, Fx, z, eta, p.restart, p.max_iters);
        out.n_JVP += g.matvecs;
        out.n_lin_iters += g.iters;
        out.n_prec += g.precs;
        if (!g.converged) ++out.n_lin_failures;
        if (g.breakdown) break;
        double lam = 1.0;
        bool ok = false;
        while (lam >= p.min_lambda) {
            for (std::size_t q = 0; q < N; ++q) xn[q] = x[q] - lam * z[q];
            f.eval(xn, Fn); ++out.n_F;
            if (norm2(Fn) <= (1.0 - p.armijo * lam) * rnorm) { ok = true; break; }
            lam *= 0.5;
        }
        if (!ok) break;
        x = xn; Fx = Fn;
        rprev = rnorm; rnorm = norm2(Fx); eta_prev = eta;
        ++out.iters;
    }
    if (rnorm <= p.rtol_nl * out.res0) out.converged = true;
    out.x = std::move(x);
    out.res = rnorm;
    return out;
}

// Inexact Chebyshev: J z = F, J u = F''(x)[z,z], trial x - z - u/2, Newton backtracking
// fallback (krylov_newton.hpp:116-189).
template <class Op>
static Result chebyshev_inexact(const Op& f, DVec x, const Params& p, Provider& pc) {
    const std::size_t N = f.size();
    Result out;
    DVec Fx(N), Fn(N), z(N), u(N), w(N), xn(N);
    f.eval(x, Fx); ++out.n_F;
    double rnorm = norm2(Fx);
    out.res0 = rnorm;
    double rprev = rnorm, eta_prev = p.eta_init;
    for (std::size_t k = 0; k < p.max_nl; ++k) {
        if (rnorm <= p.rtol_nl * out.res0) { out.converged = true; break; }
        const double eta1 = forcing(p, k, rnorm, rprev, eta_prev, out.res0);
        const double eta2 = std::min(p.eta2_max, p.eta2_factor * eta1);
        pc.make(x);
        auto A = [&](const DVec& v, DVec& o) { f.jvp(x, v, o); };
        z.assign(N, 0.0);
        KrylovSpace space;
        const GmresResult g1 = gmres(A, pc, Fx, z, eta1, p.restart, p.max_iters, true,
                                     p.recycle ? &space : nullptr);
        out.n_JVP += g1.matvecs;
        out.n_lin_iters += g1.iters;
        out.n_prec += g1.precs;
        if (!g1.converged) ++out.n_lin_failures;
        if (g1.breakdown) break;
        f.d2(x, z, w); ++out.n_D2;
        u.assign(N, 0.0);
        const GmresResult g2 = p.recycle
            ? gmres_recycled(A, pc, w, u, eta2, p.restart, p.max_iters, space)
            : gmres(A, pc, w, u, eta2, p.restart, p.max_iters);
        out.n_JVP += g2.matvecs;
        out.n_lin_iters += g2.iters;
        out.n_prec += g2.precs;
        if (!g2.converged) ++out.n_lin_failures;
        bool ok = false;
        if (!g2.breakdown) {
            for (std::size_t q = 0; q < N; ++q) xn[q] = x[q] - z[q] - 0.5 * u[q];
            f.eval(xn, Fn); ++out.n_F;
            if (norm2(Fn) < rnorm) ok = true;
        }
        if (!ok) {
            double lam = 1.0;
            while (lam >= p.min_lambda) {
                for (std::size_t q = 0; q < N; ++q) xn[q] = x[q] - lam * z[q];
                f.eval(xn, Fn); ++out.n_F;
                if (norm2(Fn) <= (1.0 - p.armijo * lam) * rnorm) { ok = true; break; }
                lam *= 0.5;
            }
        }
        if (!ok) break;
        x = xn; Fx = Fn;
        rprev = rnorm; rnorm = norm2(Fx); eta_prev = eta1;
        ++out.iters;
    }
    if (rnorm <= p.rtol_nl * out.res0) out.converged = true;
    out.x = std::move(x);
    out.res = rnorm;
    return out;
}

// Tensor-free Chebyshev (Eustaquio-Ribeiro-Dumett 2018, alpha = 0): curvature from two JVPs at
// x and x + h d1, h = clamp(sqrt(eps) ||x|| / ||d1||, 2 eps, 0.5) (tf_chebyshev_2018.hpp:23-132).
static double tf2018_step(const DVec& x, const DVec& d1) {
    const double eps = std::numeric_limits<double>::epsilon();
    const double nd = norm2(d1);
    if (!(nd > 0.0)) return 2.0 * eps;
    const double raw = std::sqrt(eps) * norm2(x) / nd;
    return std::clamp(raw, 2.0 * eps, 0.5);
}

template <class Op>
static Result tf_chebyshev_2018(const Op& f, DVec x, const Params& p, Provider& pc) {
    const std::size_t N = f.size();
    Result out;
    DVec Fx(N), Fn(N), z(N), d1(N), d2v(N), curv(N), rhs2(N), j0(N), j1(N);
    f.eval(x, Fx); ++out.n_F;
    double rnorm = norm2(Fx);
    out.res0 = rnorm;
    const double eps = std::numeric_limits<double>::epsilon();
    for (std::size_t k = 0; k < p.max_nl; ++k) {
        if (rnorm <= p.rtol_nl * out.res0) { out.converged = true; break; }
        const double eta1 = std::clamp(std::min(1e-8, rnorm * rnorm), 2.0 * eps, 1e-8);
        const double eta2 = std::clamp(std::min(1e-8, rnorm), 2.0 * eps, 1e-8);
        pc.make(x);
        auto A = [&](const DVec& v, DVec& o) { f.jvp(x, v, o); };
        z.assign(N, 0.0);
        const GmresResult g1 = gmres(A, pc, Fx, z, eta1, p.restart, p.max_iters);
        out.n_JVP += g1.matvecs;
        out.n_lin_iters += g1.iters;
        out.n_prec += g1.precs;
        if (!g1.converged) { ++out.n_lin_failures; break; }
        if (g1.breakdown) break;
        d1 = z;
        for (double& e : d1) e = -e;
        const double h = tf2018_step(x, d1);
        DVec xh = x;
        axpy(h, d1, xh);
        f.jvp(x, d1, j0);
        f.jvp(xh, d1, j1);
        curv.resize(N);
        for (std::size_t q = 0; q < N; ++q) curv[q] = (j1[q] - j0[q]) / h;
        out.n_JVP += 2;
        for (std::size_t q = 0; q < N; ++q) rhs2[q] = -0.5 * curv[q];
        d2v.assign(N, 0.0);
        const GmresResult g2 = gmres(A, pc, rhs2, d2v, eta2, p.restart, p.max_iters);
        out.n_JVP += g2.matvecs;
        out.n_lin_iters += g2.iters;
        out.n_prec += g2.precs;
        if (!g2.converged) { ++out.n_lin_failures; break; }
        if (g2.breakdown) break;
        axpy(1.0, d1, x);
        axpy(1.0, d2v, x);
        f.eval(x, Fn); ++out.n_F;
        Fx = Fn;
        rnorm = norm2(Fx);
        ++out.iters;
        if (!std::isfinite(rnorm)) break;
    }
    if (rnorm <= p.rtol_nl * out.res0) out.converged = true;
    out.x = std::move(x);
    out.res = rnorm;
    return out;
}

static Params to_params(const numa_krylov_params* cp) {
    Params p;
    if (!cp) return p;
    p.rtol_nl = cp->rtol_nl;
    p.max_nl = cp->max_nl;
    p.eta_init = cp->eta_init;
    p.eta_max = cp->eta_max;
    p.gamma = cp->gamma;
    p.alpha = cp->alpha;
    p.eta2_factor = cp->eta2_factor;
    p.eta2_max = cp->eta2_max;
    p.restart = cp->gmres_restart;
    p.max_iters = cp->gmres_max_iters;
    p.armijo = cp->armijo;
    p.min_lambda = cp->min_lambda;
    p.recycle = cp->recycle != 0;
    return p;
}

// Runs a driver on a Brusselator operator and fills the C result (bench-style timers included).
static int bruss_solve(int method, Params p, const std::function<Result(int, Params&, Timers&)>& run,
                       double* x_out, numa_krylov_result* res) {
    auto t_start = Clock::now();
    Timers t;
    if (method == NUMA_GPU_METHOD_CHEB_REC) p.recycle = true;
    if (method < NUMA_GPU_METHOD_NK || method > NUMA_GPU_METHOD_TF2018) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    Result r = run(method, p, t);
    if (x_out) std::memcpy(x_out, r.x.data(), r.x.size() * sizeof(double));
    if (res) {
        std::memset(res, 0, sizeof(*res));
        res->converged = r.converged ? 1 : 0;
        res->iters = r.iters;
        res->n_F = r.n_F;
        res->n_JVP = r.n_JVP;
        res->n_D2 = r.n_D2;
        res->n_lin_iters = r.n_lin_iters;
        res->n_lin_failures = r.n_lin_failures;
        res->n_prec = r.n_prec;
        res->res0 = r.res0;
        res->res = r.res;
        res->t_F = t.t_F;
        res->t_JVP = t.t_JVP;
        res->t_D2 = t.t_D2;
        res->t_prec = t.t_prec;
        res->t_setup_dynamic = t.t_setup;
        res->t_total = seconds_since(t_start);
    }
    return 0;
}

template <class Op>
static Result run_method(int method, const Op& op, const DVec& x0, const Params& p, Provider& pc) {
    switch (method) {
        case NUMA_GPU_METHOD_NK: return newton_krylov(op, x0, p, pc);
        case NUMA_GPU_METHOD_TF2018: return tf_chebyshev_2018(op, x0, p, pc);
        default: return chebyshev_inexact(op, x0, p, pc);
    }
}

}  // namespace oracle

// ============================================================================ C API (ctypes)
using namespace oracle;

extern "C" {

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

double oracle_dot(size_t N, const double* a, const double* b) {
    DVec A(a, a + N), B(b, b + N);
    return dot(A, B);
}

void oracle_bratu3d_eval(size_t n, double lambda, const double* u, double* out) {
    Bratu f(n, lambda);
    DVec U(u, u + f.size()), O;
    f.eval(U, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
}

void oracle_bratu3d_jvp(size_t n, double lambda, const double* u, const double* v, double* out, int mode) {
    Bratu f(n, lambda);
    DVec U(u, u + f.size()), V(v, v + f.size()), O;
    if (mode == 1) jvp_fd(f, U, V, O); else f.jvp(U, V, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
}

void oracle_bratu3d_d2(size_t n, double lambda, const double* u, const double* v, double* out, int mode) {
    Bratu f(n, lambda);
    DVec U(u, u + f.size()), V(v, v + f.size()), O;
    if (mode == 1) d2_fd(f, U, V, O); else f.d2(U, V, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
}

void oracle_bratu3d_jacobi_diag(size_t n, double lambda, const double* u, double* d) {
    Bratu f(n, lambda);
    DVec U(u, u + f.size()), D;
    f.jacobi_diag(U, D);
    std::memcpy(d, D.data(), D.size() * sizeof(double));
}

// Returns the level count, or -1 / -2 for the reference's invalid_argument / overflow_error.
int oracle_mg_levels(size_t n, int pre, int post) {
    try {
        PoissonMG mg(n, pre, post);
        return static_cast<int>(mg.levels());
    } catch (const std::overflow_error&) {
        return -2;
    } catch (const std::invalid_argument&) {
        return -1;
    }
}

int oracle_mg_apply(size_t n, int pre, int post, const double* r, double* z) {
    try {
        PoissonMG mg(n, pre, post);
        DVec R(r, r + n * n * n), Z;
        mg.apply(R, Z);
        std::memcpy(z, Z.data(), Z.size() * sizeof(double));
        return 0;
    } catch (...) {
        return -1;
    }
}

// Single V-cycle stages on one level (for kernel-level parity).
void oracle_mg_smooth(size_t n, double h2inv, double* x, const double* b, int order) {
    PoissonMG::Level L;
    L.n = n; L.h2inv = h2inv;
    L.x.assign(x, x + n * n * n);
    L.b.assign(b, b + n * n * n);
    PoissonMG::smooth(L, order);
    std::memcpy(x, L.x.data(), L.x.size() * sizeof(double));
}

void oracle_mg_residual(size_t n, double h2inv, const double* x, const double* b, double* r) {
    PoissonMG::Level L;
    L.n = n; L.h2inv = h2inv;
    L.x.assign(x, x + n * n * n);
    L.b.assign(b, b + n * n * n);
    L.r.assign(n * n * n, 0.0);
    PoissonMG::residual(L);
    std::memcpy(r, L.r.data(), L.r.size() * sizeof(double));
}

void oracle_mg_restrict(size_t nf, const double* rf, double* bc) {
    PoissonMG::Level F, C;
    F.n = nf; F.r.assign(rf, rf + nf * nf * nf);
    C.n = (nf - 1) / 2; C.b.assign(C.n * C.n * C.n, 0.0);
    PoissonMG::restrict_to(F, C);
    std::memcpy(bc, C.b.data(), C.b.size() * sizeof(double));
}

void oracle_mg_prolong_add(size_t nc, const double* xc, double* xf) {
    PoissonMG::Level F, C;
    C.n = nc; C.x.assign(xc, xc + nc * nc * nc);
    F.n = 2 * nc + 1; F.x.assign(xf, xf + F.n * F.n * F.n);
    PoissonMG::prolong_add(C, F);
    std::memcpy(xf, F.x.data(), F.x.size() * sizeof(double));
}

static void fill_gmres_result(const GmresResult& g, numa_gmres_result* out) {
    if (!out) return;
    out->iters = g.iters;
    out->matvecs = g.matvecs;
    out->precs = g.precs;
    out->rel_res = g.rel_res;
    out->converged = g.converged ? 1 : 0;
    out->breakdown = g.breakdown ? 1 : 0;
}

static Provider make_provider(int kind, const Bratu& f, std::size_t n, Timers* t) {
    Provider pc;
    pc.kind = kind;
    pc.f = &f;
    pc.timers = t;
    if (kind == NUMA_GPU_PRECOND_POISSON_MG) pc.mg = std::make_shared<PoissonMG>(n);
    return pc;
}

// GMRES on the Bratu3D Jacobian at xpt (analytic or FD matvec) with a provider bound at xpt.
int oracle_gmres_bratu3d(size_t n, double lambda, const double* xpt, int jvp_mode, int precond_kind,
                         const double* b, double* x, double rtol, size_t restart, size_t max_iters,
                         int zero_guess, numa_gmres_result* out) {
    Bratu f(n, lambda);
    Timers t;
    BratuOp op{f, jvp_mode, 0, &t};
    const std::size_t N = f.size();
    DVec X(xpt, xpt + N), B(b, b + N), S(x, x + N);
    Provider pc = make_provider(precond_kind, f, n, &t);
    pc.make(X);
    auto A = [&](const DVec& v, DVec& o) { op.jvp(X, v, o); };
    GmresResult g = gmres(A, pc, B, S, rtol, restart, max_iters, zero_guess != 0);
    std::memcpy(x, S.data(), N * sizeof(double));
    fill_gmres_result(g, out);
    return 0;
}

// gmres with save, then gmres_recycled on a second right-hand side (the reference test
// tests/test_operators.cpp:235-275): writes both solutions and both results.
int oracle_gmres_recycle_pair(size_t n, double lambda, const double* xpt, int precond_kind,
                              const double* b1, const double* b2, double rtol, size_t restart,
                              size_t max_iters, double* z1, double* u2, size_t* k_saved,
                              numa_gmres_result* r1, numa_gmres_result* r2) {
    Bratu f(n, lambda);
    Timers t;
    const std::size_t N = f.size();
    DVec X(xpt, xpt + N), B1(b1, b1 + N), B2(b2, b2 + N), Z(N, 0.0), U;
    Provider pc = make_provider(precond_kind, f, n, &t);
    pc.make(X);
    auto A = [&](const DVec& v, DVec& o) { f.jvp(X, v, o); };
    KrylovSpace sp;
    GmresResult g1 = gmres(A, pc, B1, Z, rtol, restart, max_iters, true, &sp);
    GmresResult g2 = gmres_recycled(A, pc, B2, U, rtol, restart, max_iters, sp);
    std::memcpy(z1, Z.data(), N * sizeof(double));
    std::memcpy(u2, U.data(), N * sizeof(double));
    if (k_saved) *k_saved = sp.k;
    fill_gmres_result(g1, r1);
    fill_gmres_result(g2, r2);
    return 0;
}

// GMRES on the plain -Laplacian with the V-cycle (tests/test_operators.cpp:207-233).
int oracle_gmres_poisson_mg(size_t n, const double* b, double* x, double rtol, size_t restart,
                            size_t max_iters, numa_gmres_result* out) {
    Bratu lap(n, 0.0);
    PoissonMG mg(n);
    const std::size_t N = n * n * n;
    DVec B(b, b + N), S(N, 0.0);
    auto A = [&](const DVec& v, DVec& o) { lap.neg_laplacian(v, o); };
    auto M = [&](const DVec& r, DVec& z) { mg.apply(r, z); };
    GmresResult g = gmres(A, M, B, S, rtol, restart, max_iters);
    std::memcpy(x, S.data(), N * sizeof(double));
    fill_gmres_result(g, out);
    return 0;
}

// Full nonlinear solve of Bratu3D(n, lambda) from x0 with method / provider kind.
int oracle_solve_bratu3d(size_t n, double lambda, int method, int precond_kind,
                         const numa_krylov_params* cp, const double* x0, double* x_out,
                         numa_krylov_result* res) {
    try {
        auto t_start = Clock::now();
        Bratu f(n, lambda);
        Timers t;
        const int jm = cp ? cp->jvp_mode : 0;
        const int dm = cp ? cp->d2_mode : 0;
        BratuOp op{f, jm, dm, &t};
        Params p = to_params(cp);
        if (method == NUMA_GPU_METHOD_CHEB_REC) p.recycle = true;
        auto t_setup = Clock::now();
        Provider pc = make_provider(precond_kind, f, n, &t);
        const double setup_static = seconds_since(t_setup);
        DVec X0(x0, x0 + f.size());
        Result r;
        switch (method) {
            case NUMA_GPU_METHOD_NK: r = newton_krylov(op, X0, p, pc); break;
            case NUMA_GPU_METHOD_CHEB:
            case NUMA_GPU_METHOD_CHEB_REC: r = chebyshev_inexact(op, X0, p, pc); break;
            case NUMA_GPU_METHOD_TF2018: r = tf_chebyshev_2018(op, X0, p, pc); break;
            default: return NUMA_GPU_ERR_INVALID_ARGUMENT;
        }
        if (x_out) std::memcpy(x_out, r.x.data(), r.x.size() * sizeof(double));
        if (res) {
            std::memset(res, 0, sizeof(*res));
            res->converged = r.converged ? 1 : 0;
            res->iters = r.iters;
            res->n_F = r.n_F;
            res->n_JVP = r.n_JVP;
            res->n_D2 = r.n_D2;
            res->n_lin_iters = r.n_lin_iters;
            res->n_lin_failures = r.n_lin_failures;
            res->n_prec = r.n_prec;
            res->res0 = r.res0;
            res->res = r.res;
            res->t_F = t.t_F;
            res->t_JVP = t.t_JVP;
            res->t_D2 = t.t_D2;
            res->t_prec = t.t_prec;
            res->t_setup_dynamic = t.t_setup + setup_static;
            res->t_total = seconds_since(t_start);
        }
        return 0;
    } catch (const std::overflow_error&) {
        return NUMA_GPU_ERR_OVERFLOW;
    } catch (const std::invalid_argument&) {
        return NUMA_GPU_ERR_INVALID_ARGUMENT;
    }
}

double oracle_forcing(const numa_krylov_params* cp, size_t k, double rnorm, double rprev,
                      double eta_prev, double res0) {
    return forcing(to_params(cp), k, rnorm, rprev, eta_prev, res0);
}

// ---- Burgers2D and HelmholtzMG2D
int oracle_burgers2d_exact(size_t n, double nu, double dt, double amp, double* out) {
    try {
        Burgers f(n, nu, dt, amp);
        std::memcpy(out, f.exact.data(), f.size() * sizeof(double));
        return 0;
    } catch (...) {
        return NUMA_GPU_ERR_INVALID_ARGUMENT;
    }
}

int oracle_burgers2d_eval(size_t n, double nu, double dt, double amp, const double* w, double* out) {
    Burgers f(n, nu, dt, amp);
    DVec W(w, w + f.size()), O;
    f.eval(W, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int oracle_burgers2d_jvp(size_t n, double nu, double dt, double amp, const double* w, const double* d, double* out,
                         int mode) {
    Burgers f(n, nu, dt, amp);
    DVec W(w, w + f.size()), D(d, d + f.size()), O;
    if (mode == 1) jvp_fd(f, W, D, O); else f.jvp(W, D, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int oracle_burgers2d_d2(size_t n, double nu, double dt, double amp, const double* w, const double* d, double* out,
                        int mode) {
    Burgers f(n, nu, dt, amp);
    DVec W(w, w + f.size()), D(d, d + f.size()), O;
    if (mode == 1) d2_fd(f, W, D, O); else f.d2(W, D, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int oracle_hmg2d_levels(size_t n, double alpha, double nu) {
    HelmholtzMG2D mg(n, alpha, nu);
    return static_cast<int>(mg.levels());
}

int oracle_hmg2d_apply(size_t n, double alpha, double nu, int pre, int post, const double* r, double* z) {
    HelmholtzMG2D mg(n, alpha, nu, pre, post);
    DVec R(r, r + n * n), Z;
    mg.apply(R, Z);
    std::memcpy(z, Z.data(), Z.size() * sizeof(double));
    return 0;
}

// Burgers2D(n, nu, dt, amp) from x0 with NoPrecond (precond_kind 0) or BurgersMGProvider (1).
int oracle_solve_burgers2d(size_t n, double nu, double dt, double amp, int method, int precond_kind,
                           const numa_krylov_params* cp, const double* x0, double* x_out, numa_krylov_result* res) {
    try {
        auto t_start = Clock::now();
        Burgers f(n, nu, dt, amp);
        Timers t;
        BurgersOp op{f, cp ? cp->jvp_mode : 0, cp ? cp->d2_mode : 0, &t};
        Params p = to_params(cp);
        if (method == NUMA_GPU_METHOD_CHEB_REC) p.recycle = true;
        Provider pc;
        pc.timers = &t;
        if (precond_kind == NUMA_GPU_PRECOND_POISSON_MG) {
            pc.kind = kBurgersMG;
            pc.hmg = std::make_shared<HelmholtzMG2D>(n, 1.0 / dt, nu);
            pc.nn = n * n;
        }
        DVec X0(x0, x0 + f.size());
        Result r;
        switch (method) {
            case NUMA_GPU_METHOD_NK: r = newton_krylov(op, X0, p, pc); break;
            case NUMA_GPU_METHOD_CHEB:
            case NUMA_GPU_METHOD_CHEB_REC: r = chebyshev_inexact(op, X0, p, pc); break;
            case NUMA_GPU_METHOD_TF2018: r = tf_chebyshev_2018(op, X0, p, pc); break;
            default: return NUMA_GPU_ERR_INVALID_ARGUMENT;
        }
        if (x_out) std::memcpy(x_out, r.x.data(), r.x.size() * sizeof(double));
        if (res) {
            std::memset(res, 0, sizeof(*res));
            res->converged = r.converged ? 1 : 0;
            res->iters = r.iters;
            res->n_F = r.n_F;
            res->n_JVP = r.n_JVP;
            res->n_D2 = r.n_D2;
            res->n_lin_iters = r.n_lin_iters;
            res->n_lin_failures = r.n_lin_failures;
            res->n_prec = r.n_prec;
            res->res0 = r.res0;
            res->res = r.res;
            res->t_F = t.t_F;
            res->t_JVP = t.t_JVP;
            res->t_D2 = t.t_D2;
            res->t_prec = t.t_prec;
            res->t_total = seconds_since(t_start);
        }
        return 0;
    } catch (const std::invalid_argument&) {
        return NUMA_GPU_ERR_INVALID_ARGUMENT;
    }
}

// ---- Brusselator1DStep and Brusselator2D
int oracle_bruss1d_previous(size_t n, double dt, double* out) {
    try {
        Bruss1D f(n, dt);
        std::memcpy(out, f.prev.data(), f.size() * sizeof(double));
        return 0;
    } catch (const std::invalid_argument&) {
        return NUMA_GPU_ERR_INVALID_ARGUMENT;
    }
}

int oracle_bruss1d_eval(size_t n, double dt, const double* w, double* out) {
    Bruss1D f(n, dt);
    DVec W(w, w + f.size()), O;
    f.eval(W, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int oracle_bruss1d_jvp(size_t n, double dt, const double* w, const double* d, double* out, int mode) {
    Bruss1D f(n, dt);
    DVec W(w, w + f.size()), D(d, d + f.size()), O;
    if (mode == 1) jvp_fd(f, W, D, O); else f.jvp(W, D, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int oracle_bruss1d_d2(size_t n, double dt, const double* w, const double* d, double* out, int mode) {
    Bruss1D f(n, dt);
    DVec W(w, w + f.size()), D(d, d + f.size()), O;
    if (mode == 1) d2_fd(f, W, D, O); else f.d2(W, D, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

// BrusselatorJacobi made at w and applied to r.
int oracle_bruss1d_jacobi_apply(size_t n, double dt, const double* w, const double* r, double* z) {
    Bruss1D f(n, dt);
    DVec W(w, w + f.size()), R(r, r + f.size()), a11, a12, a21, a22, Z;
    f.blocks(W, a11, a12, a21, a22);
    bruss_block_apply(a11, a12, a21, a22, R, Z);
    std::memcpy(z, Z.data(), Z.size() * sizeof(double));
    return 0;
}

// Brusselator1DStep(n, dt) from x0 (null: the previous state, run_campaign's natural start) with
// NoPrecond or BrusselatorJacobi.
int oracle_solve_bruss1d(size_t n, double dt, int method, int precond_kind, const numa_krylov_params* cp,
                         const double* x0, double* x_out, numa_krylov_result* res) {
    try {
        Bruss1D f(n, dt);
        if (precond_kind != NUMA_GPU_PRECOND_NONE && precond_kind != NUMA_GPU_PRECOND_BRUSS_JACOBI)
            return NUMA_GPU_ERR_INVALID_ARGUMENT;
        const DVec X0 = x0 ? DVec(x0, x0 + f.size()) : f.prev;
        return bruss_solve(method, to_params(cp), [&](int m, Params& p, Timers& t) {
            GenericOp<Bruss1D> op{f, cp ? cp->jvp_mode : 0, cp ? cp->d2_mode : 0, &t};
            Provider pc;
            pc.timers = &t;
            pc.kind = precond_kind;
            pc.bf = &f;
            return run_method(m, op, X0, p, pc);
        }, x_out, res);
    } catch (const std::invalid_argument&) {
        return NUMA_GPU_ERR_INVALID_ARGUMENT;
    }
}

// prm = {A, B, D_u, D_v, dt}
static Bruss2DParams bruss2d_params(const double* prm) { return Bruss2DParams{prm[0], prm[1], prm[2], prm[3], prm[4]}; }

int oracle_bruss2d_eval(size_t n, const double* prm, const double* prev, const double* w, double* out) {
    Bruss2D f(n, bruss2d_params(prm), prev);
    DVec W(w, w + f.size()), O;
    f.eval(W, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int oracle_bruss2d_jvp(size_t n, const double* prm, const double* prev, const double* w, const double* d,
                       double* out, int mode) {
    Bruss2D f(n, bruss2d_params(prm), prev);
    DVec W(w, w + f.size()), D(d, d + f.size()), O;
    if (mode == 1) jvp_fd(f, W, D, O); else f.jvp(W, D, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int oracle_bruss2d_d2(size_t n, const double* prm, const double* prev, const double* w, const double* d,
                      double* out, int mode) {
    Bruss2D f(n, bruss2d_params(prm), prev);
    DVec W(w, w + f.size()), D(d, d + f.size()), O;
    if (mode == 1) d2_fd(f, W, D, O); else f.d2(W, D, O);
    std::memcpy(out, O.data(), O.size() * sizeof(double));
    return 0;
}

int oracle_bmg2d_levels(size_t n) {
    try {
        BrussMG2D mg(n, Bruss2DParams{1.0, 1.0, 1.0, 1.0, 1.0});
        return static_cast<int>(mg.levels());
    } catch (const std::invalid_argument&) {
        return -1;
    }
}

// One V-cycle of the coupled-block multigrid set at the state w, applied to r.
int oracle_bmg2d_apply(size_t n, const double* prm, const double* w, int pre, int post, const double* r, double* z) {
    try {
        BrussMG2D mg(n, bruss2d_params(prm), pre, post);
        DVec W(w, w + 2 * n * n), R(r, r + 2 * n * n), Z;
        mg.set_state(W);
        mg.apply(R, Z);
        std::memcpy(z, Z.data(), Z.size() * sizeof(double));
        return 0;
    } catch (const std::invalid_argument&) {
        return NUMA_GPU_ERR_INVALID_ARGUMENT;
    }
}

// One implicit-Euler step of Brusselator2D from the previous state prev, Newton start x0 (null:
// prev), with NoPrecond or the coupled-block multigrid.
int oracle_solve_bruss2d(size_t n, const double* prm, const double* prev, int method, int precond_kind,
                         const numa_krylov_params* cp, const double* x0, double* x_out, numa_krylov_result* res) {
    try {
        Bruss2D f(n, bruss2d_params(prm), prev);
        if (precond_kind != NUMA_GPU_PRECOND_NONE && precond_kind != NUMA_GPU_PRECOND_BRUSS_MG)
            return NUMA_GPU_ERR_INVALID_ARGUMENT;
        const DVec X0 = x0 ? DVec(x0, x0 + f.size()) : f.prev;
        std::shared_ptr<BrussMG2D> mg;
        if (precond_kind == NUMA_GPU_PRECOND_BRUSS_MG) mg = std::make_shared<BrussMG2D>(n, f.P);
        return bruss_solve(method, to_params(cp), [&](int m, Params& p, Timers& t) {
            GenericOp<Bruss2D> op{f, cp ? cp->jvp_mode : 0, cp ? cp->d2_mode : 0, &t};
            Provider pc;
            pc.timers = &t;
            pc.kind = precond_kind;
            pc.bmg = mg;
            return run_method(m, op, X0, p, pc);
        }, x_out, res);
    } catch (const std::invalid_argument&) {
        return NUMA_GPU_ERR_INVALID_ARGUMENT;
    }
}

}  // extern "C"
