// FP64 CPU restatement of BoundaryValueDiffEq.jl's adaptive MIRK solve.
//
// TEST INFRASTRUCTURE ONLY. This is the oracle: the parity tests, the smoke check
// and the benchmark's CPU-baseline leg compile it (together with a user problem
// source) and compare the CUDA library against it. The shipped library never links,
// loads or calls anything under oracle/.
//
// The reference (Julia) cannot run in this environment, so every step below restates
// the reference's algorithm from its source; each function cites the lines it follows.
// The nonlinear and linear solvers the reference takes from external packages
// (NonlinearSolveFirstOrder's NewtonRaphson polyalgorithm, FastAlmostBandedMatrices'
// almost-banded factorisation, ForwardDiff) are restated from their mathematics:
// Newton on ||F||_inf <= abstol, exact forward-mode Jacobian, and a stable structured
// Gaussian elimination with partial pivoting of the almost-block-diagonal system.
//
// The problem (f, bc) is a user source compiled into the same translation unit:
//   template <class T, class P> void bvp_f(T* du, const T* u, const P* p, P t);
//   standard problems:  template <class T, class P> void bvp_bc(T* res, const T* const* ua, const P* p);
//                       (ua[k] = u(bc_t[k]) as the reference's EvalSol returns it)
//   two-point problems: template <class T, class P> void bvp_bca(T* res, const T* ua, const P* p);
//                       template <class T, class P> void bvp_bcb(T* res, const T* ub, const P* p);
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef BVP_TRACE
#include <cstdio>
#endif

#include "dual.hpp"
#include "mirk_tableaus.hpp"

namespace oracle {

enum RetCode : int32_t { RET_SUCCESS = 0, RET_FAILURE = 1, RET_MAXITERS = 2 };

struct ProblemInfo {
    int32_t M;
    int32_t n_params;
    int32_t twopoint;      // 0: standard (bc over EvalSol points), 1: two-point (bca, bcb)
    int32_t n_bc_pts;      // standard: number of evaluation times
    int32_t La, Lb;        // two-point: residual counts at a and b (La + Lb == M)
    double bc_t[16];       // standard: evaluation times u(bc_t[k])
};

struct Options {
    int32_t order;             // 2..6
    int32_t adaptive;          // 1: defect-controlled mesh refinement
    int32_t max_subintervals;  // reference default 3000 (algorithms.jl:60)
    int32_t max_newton;        // Newton iteration cap per attempt
    int32_t max_rounds;        // safety cap on outer (mesh) rounds
    int32_t transfer_inplace;  // 1: reproduce the reference's in-place y0 transfer
    int32_t bc_jac_exact;      // 0: reference BC Jacobian (primal stages), 1: exact
    int32_t linesearch_fallback;
    int32_t stall_steps;
    int32_t nthreads;
    double abstol;             // reference default 1e-6 (mirk.jl:50)
    double defect_threshold;   // reference default 0.1 (calc_errors.jl:54-60)
    double divergence_factor;
    int32_t mirk6i;            // 1 with order 6: MIRK6I (mirk_tableaus.jl:154-194)
    // error controller (Core/src/calc_errors.jl:54-139): 0 DefectControl, 1 GlobalErrorControl,
    // 2 SequentialErrorControl, 3 HybridErrorControl; the global estimate's method: 0
    // HOErrorControl (MIRK(p+2) on the same mesh), 1 REErrorControl (same method, halved mesh)
    int32_t controller;
    int32_t global_method;
    double hybrid_de, hybrid_ge;   // HybridErrorControl's DE and GE weights
};

inline void fill_default_options(Options* o) {
    o->order = 4; o->adaptive = 1; o->max_subintervals = 3000; o->max_newton = 100;
    o->max_rounds = 64; o->transfer_inplace = 1; o->bc_jac_exact = 0;
    o->linesearch_fallback = 1; o->stall_steps = 32; o->nthreads = 0;
    o->abstol = 1e-6; o->defect_threshold = 0.1; o->divergence_factor = 1e3; o->mirk6i = 0;
    o->controller = 0; o->global_method = 0; o->hybrid_de = 1.0; o->hybrid_ge = 1.0;
}

enum Controller : int32_t { CTL_DEFECT = 0, CTL_GLOBAL = 1, CTL_SEQUENTIAL = 2, CTL_HYBRID = 3 };
enum GlobalMethod : int32_t { GLOBAL_HO = 0, GLOBAL_RE = 1 };

// Julia's max over values that may be NaN: NaN wins (Base.max, used by maximum).
inline double julia_max(double a, double b) { return (std::isnan(a) || std::isnan(b)) ? NAN : std::max(a, b); }

// Julia's round(Int, x): round half to even (the default rounding mode of rint).
inline long round_even(double x) { return (long)std::nearbyint(x); }

// interval(mesh, t) = clamp(searchsortedfirst(mesh, t) - 1, 1, N - 1)
// (lib/BoundaryValueDiffEqCore/src/utils.jl:119-121), 0-based.
inline int interval_of(const double* mesh, int N, double t) {
    const int lb = int(std::lower_bound(mesh, mesh + N, t) - mesh);
    int ii = lb - 1;
    if (ii < 0) ii = 0;
    if (ii > N - 2) ii = N - 2;
    return ii;
}

// Dense Gaussian elimination with partial pivoting, in place; b has nrhs columns
// stored column-major with leading dimension n. Returns false on an exact zero pivot.
inline bool dense_solve(int n, double* A /* row-major n x n */, double* b, int nrhs = 1) {
    for (int k = 0; k < n; ++k) {
        int piv = k; double best = std::fabs(A[k * n + k]);
        for (int r = k + 1; r < n; ++r) {
            const double a = std::fabs(A[r * n + k]);
            if (a > best) { best = a; piv = r; }
        }
        if (!(best > 0) || !std::isfinite(best)) return false;
        if (piv != k) {
            for (int c = 0; c < n; ++c) std::swap(A[k * n + c], A[piv * n + c]);
            for (int q = 0; q < nrhs; ++q) std::swap(b[q * n + k], b[q * n + piv]);
        }
        const double inv = 1.0 / A[k * n + k];
        for (int r = k + 1; r < n; ++r) {
            const double m = A[r * n + k] * inv;
            if (m == 0) continue;
            A[r * n + k] = 0;
            for (int c = k + 1; c < n; ++c) A[r * n + c] -= m * A[k * n + c];
            for (int q = 0; q < nrhs; ++q) b[q * n + r] -= m * b[q * n + k];
        }
    }
    for (int q = 0; q < nrhs; ++q)
        for (int k = n - 1; k >= 0; --k) {
            double s = b[q * n + k];
            for (int c = k + 1; c < n; ++c) s -= A[k * n + c] * b[q * n + c];
            b[q * n + k] = s / A[k * n + k];
        }
    return true;
}

template <int M>
struct InstanceSolver {
    static constexpr int D = 2 * M;
    using DualI = Dual<D>;  // tangents along (y_i, y_{i+1}) of one interval
    using DualU = Dual<M>;  // tangents along one BC evaluation point

    const Tableau& tb;
    const Tableau* tb_hi = nullptr;    // MIRK(p+2), for the HOErrorControl estimate
    const Options& op;
    const ProblemInfo& pi;
    const double* p;

    int N = 0;                         // mesh points
    std::vector<double> mesh, h;       // h kept separately (half_mesh! halves it, adaptivity.jl:287-301)
    std::vector<double> y;             // N x M
    std::vector<double> K;             // (N-1) x s x M
    std::vector<double> KI;            // (N-1) x (s*-s) x M
    std::vector<double> F;             // residual, M*N

    int newton_total = 0, rounds = 0, retcode = RET_FAILURE, newton_last = 0;
    double last_defect = std::numeric_limits<double>::quiet_NaN();
    double last_resid = std::numeric_limits<double>::quiet_NaN();
    double last_global = std::numeric_limits<double>::quiet_NaN();   // last global error norm

    InstanceSolver(const Tableau& t, const Options& o, const ProblemInfo& info, const double* params)
        : tb(t), op(o), pi(info), p(params) {}

    int ns() const { return tb.s_star - tb.s; }

    // --- Φ for one interval (collocation.jl:44-72), templated so the Jacobian can reuse it.
    template <class T>
    void phi_interval(int i, const T* yi, const T* yi1, T* Ki /* s x M */, T* ri) const {
        const double hi = h[i];
        T Y[M];
        for (int r = 0; r < tb.s; ++r) {
            for (int m = 0; m < M; ++m) Y[m] = (1.0 - tb.v[r]) * yi[m] + tb.v[r] * yi1[m];
            for (int j = 0; j < r; ++j) {
                if (tb.x[r][j] == 0) continue;
                for (int m = 0; m < M; ++m) Y[m] = Y[m] + hi * (Ki[j * M + m] * tb.x[r][j]);
            }
            const double tr = mesh[i] + tb.c[r] * hi;
            bvp_f<T, double>(&Ki[r * M], Y, p, tr);
#if BVP_SINGULAR
            // K_r += S Y_r / t_r for t_r > 0 (collocation.jl:60-66 via __add_singular_term!,
            // Core/src/utils.jl:936-941); only the collocation stages carry the term
            if (tr > 0.0) {
                T su[M];
                bvp_sing<T, double>(su, Y, p);
                const double it = 1.0 / tr;
                for (int m = 0; m < M; ++m) Ki[r * M + m] = Ki[r * M + m] + su[m] * it;
            }
#endif
        }
        for (int m = 0; m < M; ++m) {
            T acc = T(0.0);
            for (int r = 0; r < tb.s; ++r) acc = acc + Ki[r * M + m] * tb.b[r];
            ri[m] = (yi1[m] - yi[m]) - hi * acc;
        }
    }

    // --- extra interpolant stages of one interval (interpolation.jl:337-372).
    template <class T>
    void interp_stages_interval(int i, const T* yi, const T* yi1, const T* Ki, T* KIi) const {
        const double hi = h[i];
        const int S = tb.s;
        T Y[M];
        for (int r = 0; r < ns(); ++r) {
            for (int m = 0; m < M; ++m) Y[m] = T(0.0);
            for (int j = 0; j < S; ++j)
                for (int m = 0; m < M; ++m) Y[m] = Y[m] + Ki[j * M + m] * tb.x_star[r][j];
            for (int q = 0; q < r; ++q)
                for (int m = 0; m < M; ++m) Y[m] = Y[m] + KIi[q * M + m] * tb.x_star[r][S + q];
            for (int m = 0; m < M; ++m)
                Y[m] = Y[m] * hi + (1.0 - tb.v_star[r]) * yi[m] + tb.v_star[r] * yi1[m];
            bvp_f<T, double>(&KIi[r * M], Y, p, mesh[i] + tb.c_star[r] * hi);
        }
    }

    // z = y_i + h (Σ w_r K_r + Σ w_{s+q} KI_q)  (interpolation.jl:214-242, adaptivity.jl:645-666)
    template <class T>
    void sum_stages(int i, const double* w, const T* yi, const T* Ki, const T* KIi, T* z) const {
        for (int m = 0; m < M; ++m) {
            T acc = T(0.0);
            for (int r = 0; r < tb.s; ++r) acc = acc + Ki[r * M + m] * w[r];
            for (int q = 0; q < ns(); ++q) acc = acc + KIi[q * M + m] * w[tb.s + q];
            z[m] = acc * h[i] + yi[m];
        }
    }

    // BC evaluation point -> node for Jacobian purposes and value via EvalSol.
    // Returns node index (0 / N-1 for exact endpoints, else the interval index).
    int eval_sol(double t, double* z, bool* interior) const {
        if (t == mesh[0]) { for (int m = 0; m < M; ++m) z[m] = y[m]; *interior = false; return 0; }
        if (t == mesh[N - 1]) {
            for (int m = 0; m < M; ++m) z[m] = y[(N - 1) * M + m];
            *interior = false; return N - 1;
        }
        const int ii = interval_of(mesh.data(), N, t);
        const double tau = (t - mesh[ii]) / h[ii];
        double w[9], wp[9];
        interp_weights(tb.scheme, tau, w, wp);
        std::vector<double> kiv(std::max(1, ns() * M));
        interp_stages_interval<double>(ii, &y[ii * M], &y[(ii + 1) * M], &K[ii * tb.s * M], kiv.data());
        sum_stages<double>(ii, w, &y[ii * M], &K[ii * tb.s * M], kiv.data(), z);
        *interior = true;
        return ii;
    }

    // Full residual: standard [bc; r_1..r_{N-1}] (mirk.jl:471-494), two-point
    // [bca; r...; bcb] (mirk.jl:509-534). Returns ||F||_inf; non-finite -> +inf.
    double residual() {
        const int S = tb.s;
        K.resize(size_t(N - 1) * S * M);
        F.assign(size_t(M) * N, 0.0);
        double nrm = 0;
        bool bad = false;
        const int off = pi.twopoint ? pi.La : M;
        for (int i = 0; i < N - 1; ++i) {
            double* ri = &F[size_t(off) + size_t(i) * M];
            phi_interval<double>(i, &y[i * M], &y[(i + 1) * M], &K[size_t(i) * S * M], ri);
        }
        if (!pi.twopoint) {
            std::vector<double> ua(size_t(pi.n_bc_pts) * M);
            std::vector<const double*> ptrs(pi.n_bc_pts);
            for (int k = 0; k < pi.n_bc_pts; ++k) {
                bool interior;
                eval_sol(pi.bc_t[k], &ua[k * M], &interior);
                ptrs[k] = &ua[k * M];
            }
            bvp_bc<double, double>(&F[0], ptrs.data(), p);
        } else {
            double ra[M], rb[M];
            bvp_bca<double, double>(ra, &y[0], p);
            bvp_bcb<double, double>(rb, &y[(N - 1) * M], p);
            for (int k = 0; k < pi.La; ++k) F[k] = ra[k];
            for (int k = 0; k < pi.Lb; ++k) F[size_t(pi.La) + size_t(N - 1) * M + k] = rb[k];
        }
        for (double v : F) {
            if (!std::isfinite(v)) bad = true;
            nrm = std::max(nrm, std::fabs(v));
        }
        return bad ? std::numeric_limits<double>::infinity() : nrm;
    }

    // --- Jacobian (FP64, exact forward mode for the collocation blocks).
    struct BcBlock { int node; double J[M * M]; };  // L(=M) rows x M cols touching one node
    std::vector<double> Sb, Rb;  // (N-1) x M x M, row-major per block
    std::vector<BcBlock> bcb;    // BC row contributions

    void add_bc_block(int node, const double* J /* M x M */) {
        for (auto& b : bcb)
            if (b.node == node) { for (int q = 0; q < M * M; ++q) b.J[q] += J[q]; return; }
        BcBlock nb; nb.node = node; std::memcpy(nb.J, J, sizeof(nb.J)); bcb.push_back(nb);
    }

    void jacobian() {
        const int S = tb.s;
        Sb.assign(size_t(N - 1) * M * M, 0.0);
        Rb.assign(size_t(N - 1) * M * M, 0.0);
        std::vector<DualI> Kd(size_t(S) * M);
        for (int i = 0; i < N - 1; ++i) {
            DualI yi[M], yi1[M], ri[M];
            for (int m = 0; m < M; ++m) {
                yi[m] = DualI(y[i * M + m]); yi[m].d[m] = 1.0;
                yi1[m] = DualI(y[(i + 1) * M + m]); yi1[m].d[M + m] = 1.0;
            }
            phi_interval<DualI>(i, yi, yi1, Kd.data(), ri);
            for (int a = 0; a < M; ++a)
                for (int c = 0; c < M; ++c) {
                    Sb[size_t(i) * M * M + a * M + c] = ri[a].d[c];
                    Rb[size_t(i) * M * M + a * M + c] = ri[a].d[M + c];
                }
        }
        bcb.clear();
        if (pi.twopoint) {
            // rows 0..La-1 touch node 0, rows La..M-1 touch node N-1
            DualU ua[M], ra[M], rb[M];
            for (int m = 0; m < M; ++m) { ua[m] = DualU(y[m]); ua[m].d[m] = 1.0; }
            bvp_bca<DualU, double>(ra, ua, p);
            double J0[M * M] = {0};
            for (int a = 0; a < pi.La; ++a) for (int c = 0; c < M; ++c) J0[a * M + c] = ra[a].d[c];
            add_bc_block(0, J0);
            for (int m = 0; m < M; ++m) { ua[m] = DualU(y[(N - 1) * M + m]); ua[m].d[m] = 1.0; }
            bvp_bcb<DualU, double>(rb, ua, p);
            double J1[M * M] = {0};
            for (int a = 0; a < pi.Lb; ++a)
                for (int c = 0; c < M; ++c) J1[(pi.La + a) * M + c] = rb[a].d[c];
            add_bc_block(N - 1, J1);
            return;
        }
        // standard: bc(ua) with ua[k] = u(bc_t[k]).
        const int P = pi.n_bc_pts;
        std::vector<double> uav(size_t(P) * M);
        std::vector<int> node(P);
        std::vector<char> inter(P);
        for (int k = 0; k < P; ++k) {
            bool in; node[k] = eval_sol(pi.bc_t[k], &uav[k * M], &in); inter[k] = in;
        }
        for (int k = 0; k < P; ++k) {
            std::vector<DualU> ua(size_t(P) * M);
            std::vector<const DualU*> ptrs(P);
            for (int q = 0; q < P; ++q) {
                for (int m = 0; m < M; ++m) {
                    ua[q * M + m] = DualU(uav[q * M + m]);
                    if (q == k) ua[q * M + m].d[m] = 1.0;
                }
                ptrs[q] = &ua[q * M];
            }
            DualU res[M];
            bvp_bc<DualU, double>(res, ptrs.data(), p);
            double G[M * M];  // d bc / d u_k
            for (int a = 0; a < M; ++a) for (int c = 0; c < M; ++c) G[a * M + c] = res[a].d[c];
            if (!inter[k] || !op.bc_jac_exact) {
                // reference: the interpolant's stages are held at their primal values, so
                // d u(t)/d y = I on the interval's left node (interpolation.jl:214-242 with
                // mirk.jl:565-572).
                add_bc_block(node[k], G);
            } else {
                const int ii = node[k];
                const double tau = (pi.bc_t[k] - mesh[ii]) / h[ii];
                double w[9], wp[9];
                interp_weights(tb.scheme, tau, w, wp);
                DualI yi[M], yi1[M], ri[M], z[M];
                std::vector<DualI> Kd2(size_t(S) * M), KId(std::max(1, ns()) * M);
                for (int m = 0; m < M; ++m) {
                    yi[m] = DualI(y[ii * M + m]); yi[m].d[m] = 1.0;
                    yi1[m] = DualI(y[(ii + 1) * M + m]); yi1[m].d[M + m] = 1.0;
                }
                phi_interval<DualI>(ii, yi, yi1, Kd2.data(), ri);
                interp_stages_interval<DualI>(ii, yi, yi1, Kd2.data(), KId.data());
                sum_stages<DualI>(ii, w, yi, Kd2.data(), KId.data(), z);
                double JL[M * M], JR[M * M];
                for (int a = 0; a < M; ++a)
                    for (int c = 0; c < M; ++c) {
                        double sl = 0, sr = 0;
                        for (int q = 0; q < M; ++q) {
                            sl += G[a * M + q] * z[q].d[c];
                            sr += G[a * M + q] * z[q].d[M + c];
                        }
                        JL[a * M + c] = sl; JR[a * M + c] = sr;
                    }
                add_bc_block(ii, JL);
                add_bc_block(ii + 1, JR);
            }
        }
    }

    // --- Linear solve J δ = -F with a structured elimination (FP64).
    // Nodes touched by BC rows (plus 0 and N-1) are kept; each segment of collocation
    // equations between two kept nodes is reduced left to right by Gaussian elimination
    // with partial pivoting on the shared node's columns; the kept-node system is
    // solved densely and the eliminated nodes are recovered by back substitution.
    bool linear_solve(std::vector<double>& delta) {
        const int off = pi.twopoint ? pi.La : M;
        std::vector<int> kept;
        kept.push_back(0); kept.push_back(N - 1);
        for (auto& b : bcb) kept.push_back(b.node);
        std::sort(kept.begin(), kept.end());
        kept.erase(std::unique(kept.begin(), kept.end()), kept.end());
        const int Kn = int(kept.size());
        const int W = 3 * M + 1;
        struct Rec { double U[M * M], X[M * M], Y[M * M], g[M]; };
        std::vector<Rec> rec(N);
        std::vector<double> segA(size_t(Kn) * M * M), segB(size_t(Kn) * M * M), segg(size_t(Kn) * M);
        std::vector<double> Wm(size_t(2 * M) * W);
        for (int j = 0; j + 1 < Kn; ++j) {
            const int a = kept[j], b = kept[j + 1];
            double A[M * M], B[M * M], g[M];
            std::memcpy(A, &Sb[size_t(a) * M * M], sizeof(A));
            std::memcpy(B, &Rb[size_t(a) * M * M], sizeof(B));
            for (int m = 0; m < M; ++m) g[m] = -F[size_t(off) + size_t(a) * M + m];
            for (int c = a + 1; c < b; ++c) {
                // columns: [δ_c (M) | δ_a (M) | δ_{c+1} (M) | rhs]
                for (int r = 0; r < M; ++r) {
                    double* row = &Wm[size_t(r) * W];
                    for (int q = 0; q < M; ++q) { row[q] = B[r * M + q]; row[M + q] = A[r * M + q]; row[2 * M + q] = 0; }
                    row[3 * M] = g[r];
                    double* row2 = &Wm[size_t(M + r) * W];
                    for (int q = 0; q < M; ++q) {
                        row2[q] = Sb[size_t(c) * M * M + r * M + q];
                        row2[M + q] = 0;
                        row2[2 * M + q] = Rb[size_t(c) * M * M + r * M + q];
                    }
                    row2[3 * M] = -F[size_t(off) + size_t(c) * M + r];
                }
                for (int k = 0; k < M; ++k) {
                    int piv = k; double best = std::fabs(Wm[size_t(k) * W + k]);
                    for (int r = k + 1; r < 2 * M; ++r) {
                        const double v = std::fabs(Wm[size_t(r) * W + k]);
                        if (v > best) { best = v; piv = r; }
                    }
                    if (!(best > 0) || !std::isfinite(best)) return false;
                    if (piv != k)
                        for (int q = 0; q < W; ++q) std::swap(Wm[size_t(k) * W + q], Wm[size_t(piv) * W + q]);
                    const double inv = 1.0 / Wm[size_t(k) * W + k];
                    for (int r = k + 1; r < 2 * M; ++r) {
                        const double mlt = Wm[size_t(r) * W + k] * inv;
                        if (mlt == 0) continue;
                        for (int q = k; q < W; ++q) Wm[size_t(r) * W + q] -= mlt * Wm[size_t(k) * W + q];
                    }
                }
                Rec& R = rec[c];
                for (int r = 0; r < M; ++r) {
                    for (int q = 0; q < M; ++q) {
                        R.U[r * M + q] = Wm[size_t(r) * W + q];
                        R.X[r * M + q] = Wm[size_t(r) * W + M + q];
                        R.Y[r * M + q] = Wm[size_t(r) * W + 2 * M + q];
                        A[r * M + q] = Wm[size_t(M + r) * W + M + q];
                        B[r * M + q] = Wm[size_t(M + r) * W + 2 * M + q];
                    }
                    R.g[r] = Wm[size_t(r) * W + 3 * M];
                    g[r] = Wm[size_t(M + r) * W + 3 * M];
                }
            }
            std::memcpy(&segA[size_t(j) * M * M], A, sizeof(A));
            std::memcpy(&segB[size_t(j) * M * M], B, sizeof(B));
            std::memcpy(&segg[size_t(j) * M], g, sizeof(g));
        }
        // kept-node system
        const int n = Kn * M;
        std::vector<double> G(size_t(n) * n, 0.0), rhs(n, 0.0);
        for (int j = 0; j + 1 < Kn; ++j)
            for (int r = 0; r < M; ++r) {
                const int row = j * M + r;
                for (int q = 0; q < M; ++q) {
                    G[size_t(row) * n + j * M + q] = segA[size_t(j) * M * M + r * M + q];
                    G[size_t(row) * n + (j + 1) * M + q] = segB[size_t(j) * M * M + r * M + q];
                }
                rhs[row] = segg[size_t(j) * M + r];
            }
        {
            const int row0 = (Kn - 1) * M;
            // BC residual rows of F are at [0, off) and, for two-point, the tail.
            for (auto& b : bcb) {
                const int kj = int(std::lower_bound(kept.begin(), kept.end(), b.node) - kept.begin());
                for (int r = 0; r < M; ++r)
                    for (int q = 0; q < M; ++q) G[size_t(row0 + r) * n + kj * M + q] += b.J[r * M + q];
            }
            for (int r = 0; r < M; ++r) {
                double fr;
                if (!pi.twopoint) fr = F[r];
                else fr = (r < pi.La) ? F[r] : F[size_t(pi.La) + size_t(N - 1) * M + (r - pi.La)];
                rhs[row0 + r] = -fr;
            }
        }
        if (!dense_solve(n, G.data(), rhs.data())) return false;
        delta.assign(size_t(N) * M, 0.0);
        for (int j = 0; j < Kn; ++j)
            for (int m = 0; m < M; ++m) delta[size_t(kept[j]) * M + m] = rhs[j * M + m];
        for (int j = 0; j + 1 < Kn; ++j) {
            const int a = kept[j], b = kept[j + 1];
            for (int c = b - 1; c > a; --c) {
                const Rec& R = rec[c];
                double t[M];
                for (int r = 0; r < M; ++r) {
                    double s = R.g[r];
                    for (int q = 0; q < M; ++q)
                        s -= R.X[r * M + q] * delta[size_t(a) * M + q] + R.Y[r * M + q] * delta[size_t(c + 1) * M + q];
                    t[r] = s;
                }
                for (int r = M - 1; r >= 0; --r) {
                    double s = t[r];
                    for (int q = r + 1; q < M; ++q) s -= R.U[r * M + q] * delta[size_t(c) * M + q];
                    delta[size_t(c) * M + r] = s / R.U[r * M + r];
                }
            }
        }
        for (double v : delta) if (!std::isfinite(v)) return false;
        return true;
    }

    // --- Newton (restatement of NewtonRaphson, then NewtonRaphson + backtracking, the
    // first two members of the reference's default polyalgorithm,
    // lib/BoundaryValueDiffEqCore/src/default_internal_solve.jl:31-45; termination on
    // ||F||_inf <= abstol, mirk.jl:51).
    bool newton_attempt(bool linesearch, int& iters) {
        iters = 0;
        double nrm = residual();
        last_resid = nrm;
        if (!std::isfinite(nrm)) return false;
        if (nrm <= op.abstol) return true;
        const double nrm0 = nrm;
        double best = nrm; int stall = 0;
        std::vector<double> delta, ytry;
        for (int it = 0; it < op.max_newton; ++it) {
            jacobian();
            if (!linear_solve(delta)) return false;
            ++iters;
            if (!linesearch) {
                for (size_t q = 0; q < y.size(); ++q) y[q] += delta[q];
                nrm = residual();
            } else {
                // Armijo backtracking on ½||F||²: accept α when it decreases by (1 - 2cα)
                double f0 = 0; for (double v : F) f0 += v * v;
                const std::vector<double> ybase = y;
                double alpha = 1.0; bool ok = false;
                for (int ls = 0; ls < 20; ++ls) {
                    for (size_t q = 0; q < y.size(); ++q) y[q] = ybase[q] + alpha * delta[q];
                    nrm = residual();
                    double f1 = 0; for (double v : F) f1 += v * v;
                    if (std::isfinite(nrm) && f1 <= (1.0 - 2e-4 * alpha) * f0) { ok = true; break; }
                    alpha *= 0.5;
                }
                if (!ok) return false;
            }
            last_resid = nrm;
            if (!std::isfinite(nrm)) return false;
            if (nrm <= op.abstol) return true;
            if (nrm > op.divergence_factor * nrm0) return false;
            if (nrm < best) { best = nrm; stall = 0; }
            else if (++stall >= op.stall_steps) return false;
        }
        return false;
    }

    bool newton() {
        const std::vector<double> y0 = y;
        int it = 0;
        bool ok = newton_attempt(false, it);
        newton_total += it; newton_last = it;
        if (!ok && op.linesearch_fallback) {
            y = y0;
            ok = newton_attempt(true, it);
            newton_total += it; newton_last += it;
        }
        if (ok) {
            // stages at the accepted iterate (the last residual evaluation)
            residual();
        }
        return ok;
    }

    // --- defect estimate (adaptivity.jl:416-461): per-interval defect vector and norm.
    std::vector<double> err_max;  // per interval: max |err_i|
    double defect_estimate() {
        const int S = tb.s;
        KI.assign(size_t(N - 1) * std::max(1, ns()) * M, 0.0);
        err_max.assign(N - 1, 0.0);
        double w1[9], w1p[9], w2[9], w2p[9];
        interp_weights(tb.scheme, tb.tau_star, w1, w1p);
        interp_weights(tb.scheme, 1.0 - tb.tau_star, w2, w2p);
        double dn = 0;
        for (int i = 0; i < N - 1; ++i) {
            const double* Ki = &K[size_t(i) * S * M];
            double* KIi = &KI[size_t(i) * std::max(1, ns()) * M];
            interp_stages_interval<double>(i, &y[i * M], &y[(i + 1) * M], Ki, KIi);
            double est[2];
            const double* wv[2] = {w1, w2};
            const double* wpv[2] = {w1p, w2p};
            const double tv[2] = {tb.tau_star, 1.0 - tb.tau_star};
            for (int smp = 0; smp < 2; ++smp) {
                double z[M], zp[M], fz[M];
                sum_stages<double>(i, wv[smp], &y[i * M], Ki, KIi, z);
                for (int m = 0; m < M; ++m) {
                    double acc = 0;
                    for (int r = 0; r < S; ++r) acc += Ki[r * M + m] * wpv[smp][r];
                    for (int q = 0; q < ns(); ++q) acc += KIi[q * M + m] * wpv[smp][S + q];
                    zp[m] = acc;
                }
                bvp_f<double, double>(fz, z, p, mesh[i] + tv[smp] * h[i]);
                double e = 0;
                for (int m = 0; m < M; ++m) e = std::max(e, std::fabs((zp[m] - fz[m]) / (std::fabs(fz[m]) + 1.0)));
                est[smp] = e;
            }
            err_max[i] = est[0] > est[1] ? est[0] : est[1];
            if (!(err_max[i] <= dn)) dn = std::isnan(err_max[i]) ? INFINITY : std::max(dn, err_max[i]);
        }
        last_defect = dn;
        return dn;
    }

    // --- the interpolant's extra stages at the current solution (interp_setup!,
    // interpolation.jl:337-372)
    void interp_setup() {
        const int S = tb.s, NS = std::max(1, ns());
        KI.assign(size_t(N - 1) * NS * M, 0.0);
        for (int i = 0; i < N - 1; ++i)
            interp_stages_interval<double>(i, &y[i * M], &y[(i + 1) * M], &K[size_t(i) * S * M],
                                           &KI[size_t(i) * NS * M]);
    }

    // Stages of the final solution for dense output (interpolation.jl:17-204 reads the
    // cache's K and extra stages of the last residual / defect evaluation).
    void finalize_stages() {
        residual();
        interp_setup();
    }

    // --- global error estimate (adaptivity.jl:508-567). A second, non-adaptive solve starts
    // from the current solution: REErrorControl on the halved mesh with the same method
    // (halve_sol, adaptivity.jl:310-332: the old nodes at the even 0-based positions, each new
    // midpoint node the mean of its neighbours), HOErrorControl with MIRK(p+2) on the same mesh
    // (__high_order_method, adaptivity.jl:552-555). The new cache takes mesh_dt = diff(mesh)
    // (mirk.jl:75-76), and the outcome of its Newton solve is not consulted. At each current
    // node err_j = max_m |(y_high - y) / (1 + |y|)|, each interval keeps the larger of its two
    // end nodes' errors (GE_subinterval!, adaptivity.jl:557-567), the norm is their maximum,
    // times 2^p / (2^p - 1) for Richardson extrapolation (adaptivity.jl:534). The estimate is
    // taken against the low-order solution as it stands before the second solve (the
    // estimators' documented formulas, calc_errors.jl:99-128).
    std::vector<double> gerr;   // per interval
    double global_estimate() {
        const bool re = op.global_method == GLOBAL_RE;
        InstanceSolver<M> hs(re ? tb : *tb_hi, op, pi, p);
        const int n = N - 1;
        if (re) {
            hs.N = 2 * n + 1;
            hs.mesh.assign(hs.N, 0.0);
            hs.y.assign(size_t(hs.N) * M, 0.0);
            for (int i = 0; i <= n; ++i) {
                hs.mesh[2 * i] = mesh[i];
                for (int m = 0; m < M; ++m) hs.y[size_t(2 * i) * M + m] = y[size_t(i) * M + m];
            }
            for (int i = 0; i < n; ++i) {
                hs.mesh[2 * i + 1] = (hs.mesh[2 * i + 2] + hs.mesh[2 * i]) / 2.0;
                for (int m = 0; m < M; ++m)
                    hs.y[size_t(2 * i + 1) * M + m] =
                        (hs.y[size_t(2 * i + 2) * M + m] + hs.y[size_t(2 * i) * M + m]) / 2.0;
            }
        } else {
            hs.N = N;
            hs.mesh = mesh;
            hs.y = y;
        }
        hs.h.resize(hs.N - 1);
        for (int q = 0; q + 1 < hs.N; ++q) hs.h[q] = hs.mesh[q + 1] - hs.mesh[q];
        hs.newton();
        const int stride = re ? 2 : 1;
        std::vector<double> en(N);
        for (int j = 0; j < N; ++j) {
            double e = 0.0;
            for (int m = 0; m < M; ++m) {
                const double lo = y[size_t(j) * M + m];
                e = julia_max(e, std::fabs((hs.y[size_t(stride * j) * M + m] - lo) / (1.0 + std::fabs(lo))));
            }
            en[j] = e;
        }
        gerr.assign(n, 0.0);
        double g = 0.0;
        for (int i = 0; i < n; ++i) {
            gerr[i] = en[i] >= en[i + 1] ? en[i] : en[i + 1];
            g = julia_max(g, gerr[i]);
        }
        if (re) {
            const double p2 = double(1 << tb.order);
            g = g * p2 / (p2 - 1.0);
        }
        last_global = g;
        return g;
    }

    // --- half_mesh! (adaptivity.jl:287-301)
    void half_mesh() {
        const int n = N - 1;
        std::vector<double> nm(2 * n + 1), nh(2 * n);
        for (int i = 0; i <= n; ++i) nm[2 * i] = mesh[i];
        for (int i = 0; i < n; ++i) {
            nm[2 * i + 1] = (nm[2 * i + 2] + nm[2 * i]) / 2.0;
            nh[2 * i] = h[i] / 2.0; nh[2 * i + 1] = h[i] / 2.0;
        }
        mesh.swap(nm); h.swap(nh); N = 2 * n + 1;
    }

    // --- redistribute! (adaptivity.jl:250-278): equidistribute the piecewise-constant
    // density s_hat over Nsub subintervals.
    void redistribute(int Nsub, const std::vector<double>& s_hat,
                      const std::vector<double>& old_mesh, const std::vector<double>& old_h) {
        const int n = int(old_mesh.size()) - 1;
        double tot = 0;
        for (int k = 0; k < n; ++k) tot += s_hat[k] * old_h[k];
        const double zeta = tot / Nsub;
        std::vector<double> nm(Nsub + 1);
        nm[0] = old_mesh[0];
        double t = old_mesh[0], integral = 0;
        int k = 0, i = 0;
        while (k < n) {
            const double next_piece = s_hat[k] * (old_mesh[k + 1] - t);
            const double int_next = integral + next_piece;
            if (int_next > zeta) {
                const double pt = (zeta - integral) / s_hat[k] + t;
                if (i + 1 < Nsub) nm[i + 1] = pt;  // the reference would index past the end here
                t = pt; ++i; integral = 0;
            } else {
                integral = int_next; t = old_mesh[k + 1]; ++k;
            }
        }
        nm[Nsub] = old_mesh[n];
        mesh.swap(nm);
        h.resize(Nsub);
        for (int q = 0; q < Nsub; ++q) h[q] = mesh[q + 1] - mesh[q];
        N = Nsub + 1;
    }

    // --- mesh_selector! (adaptivity.jl:23-243); returns false on Failure. ŝ per interval from
    // the controller's errors: DefectControl (defect / abstol)^(1/(p+1)) with ρ = 1 (23-75);
    // GlobalErrorControl (global / abstol)^(1/p), ρ = 2 (77-125); SequentialErrorControl the
    // errors of this round's estimate (the global ones when the defect passed) to 1/(p+1),
    // ρ = 2 (127-177); HybridErrorControl the sum of the defect and global terms, each to
    // 1/(p+1), ρ = 2 (179-243).
    // `order` overrides the method order (the FIRK solver's, whose tableau is not a MIRK one).
    bool mesh_selector(std::vector<double>& old_mesh, std::vector<double>& old_h,
                       int ctl = CTL_DEFECT, bool seq_global = false, int order = 0) {
        const int n = N - 1;
        const double safety = 1.3, rho = ctl == CTL_DEFECT ? 1.0 : 2.0;
        const int ub = 4 * (N - 1), lb = N / 2;
        std::vector<double> s_hat(n);
        const int p = order > 0 ? order : tb.order;
        const double e1 = 1.0 / (p + 1);
        for (int i = 0; i < n; ++i) {
            if (ctl == CTL_DEFECT) s_hat[i] = std::pow(err_max[i] / op.abstol, e1);
            else if (ctl == CTL_GLOBAL) s_hat[i] = std::pow(gerr[i] / op.abstol, 1.0 / p);
            else if (ctl == CTL_SEQUENTIAL) s_hat[i] = std::pow((seq_global ? gerr : err_max)[i] / op.abstol, e1);
            else s_hat[i] = std::pow(err_max[i] / op.abstol, e1) + std::pow(gerr[i] / op.abstol, e1);
        }
        double r1 = -INFINITY, r2 = 0;
        for (int i = 0; i < n; ++i) { r1 = std::max(r1, s_hat[i]); r2 += s_hat[i]; }
        const double r3 = r2 / (N - 1);
        long n_pred = round_even(safety * r2 + 1);
        const double n_ = 0.1 * n;
        if (std::fabs(double(n_pred - n)) < n_) n_pred = round_even(n + n_);
        old_mesh = mesh; old_h = h;
        if (r1 <= rho * r3) {
            if (2L * n > op.max_subintervals) return false;
            half_mesh();
        } else {
            long Nsub = std::min<long>(std::max<long>(n_pred, lb), ub);
            if (Nsub > op.max_subintervals) return false;
            for (int i = 0; i < n; ++i) s_hat[i] /= old_h[i];
            redistribute(int(Nsub), s_hat, old_mesh, old_h);
        }
        return true;
    }

    // --- solution transfer to the new mesh through the old interpolant
    // (interp_eval!, adaptivity.jl:6-13, called from mirk.jl:366-371).
    void transfer(const std::vector<double>& old_mesh, const std::vector<double>& old_h) {
        const int On = int(old_mesh.size());
        const int S = tb.s, NS = std::max(1, ns());
        std::vector<double> old_y = y;           // clean copy
        std::vector<double> ny(size_t(N) * M);
        for (int j = 0; j < N; ++j) {
            const double m_t = mesh[j];
            const int i = interval_of(old_mesh.data(), On, m_t);
            const double dt = old_h[i];
            const double tau = (m_t - old_mesh[i]) / dt;
            double w[9], wp[9];
            interp_weights(tb.scheme, tau, w, wp);
            // The reference overwrites y0 in place while reading y0[old interval]
            // (mirk.jl:366-371): node j's base is the new value of node i when i < j, else the
            // old one (y0 keeps its old length when the mesh shrinks, so an old interval past
            // the new node count still holds its old value).
            const std::vector<double>& src = (op.transfer_inplace && i < j) ? ny : old_y;
            double z[M];
            for (int m = 0; m < M; ++m) {
                double acc = 0;
                for (int r = 0; r < S; ++r) acc += K[(size_t(i) * S + r) * M + m] * w[r];
                for (int q = 0; q < ns(); ++q) acc += KI[(size_t(i) * NS + q) * M + m] * w[S + q];
                z[m] = acc * dt + src[size_t(i) * M + m];
            }
            for (int m = 0; m < M; ++m) ny[size_t(j) * M + m] = z[m];
        }
        y.swap(ny);
    }

    // --- outer loop (solve!, mirk.jl:286-332 with __perform_mirk_iteration 334-388)
    void solve() {
        int info_ok = 1;
        double error_norm = 2 * op.abstol;
        rounds = 0;
        retcode = RET_FAILURE;
        while (true) {
            ++rounds;
            error_norm = 2 * op.abstol;
            const bool nl_ok = newton();
#ifdef BVP_TRACE
            fprintf(stderr, "round %d N=%d newton_ok=%d iters=%d resid=%.3e\n", rounds, N, int(nl_ok), newton_last, last_resid);
#endif
            if (!op.adaptive) { retcode = nl_ok ? RET_SUCCESS : RET_FAILURE; return; }
            bool ok = nl_ok;
            bool seq_global = false;
            if (ok) {
                // error_estimate! for the controller (adaptivity.jl:361-503). A norm that is not
                // finite counts as a failed round, for every controller.
                if (op.controller == CTL_DEFECT) {
                    error_norm = defect_estimate();
                    ok = !(error_norm > op.defect_threshold);
                } else if (op.controller == CTL_GLOBAL) {
                    // the global estimate alone (361-368); the transfer below reads the
                    // interpolant's extra stages at this solution
                    error_norm = global_estimate();
                    interp_setup();
                } else if (op.controller == CTL_SEQUENTIAL) {
                    // the defect first, the global estimate once the defect is within abstol
                    // (464-482)
                    error_norm = defect_estimate();
                    ok = !(error_norm > op.defect_threshold);
                    if (ok && error_norm <= op.abstol) {
                        seq_global = true;
                        error_norm = global_estimate();
                    }
                } else {
                    // DE * defect + GE * global; the defect threshold does not apply (485-503)
                    const double dn = defect_estimate();
                    const double gn = global_estimate();
                    error_norm = op.hybrid_de * dn + op.hybrid_ge * gn;
                }
#ifdef BVP_TRACE
                fprintf(stderr, "   error=%.3e\n", error_norm);
#endif
                if (!std::isfinite(error_norm)) ok = false;
            }
            if (ok) {
                if (error_norm > op.abstol) {
                    std::vector<double> om, oh;
                    if (mesh_selector(om, oh, op.controller, seq_global)) {
                        transfer(om, oh);
                        info_ok = 1;
                    } else {
                        info_ok = 0;
                    }
                } else {
                    info_ok = 1;
                }
            } else {
                if (2L * (N - 1) > op.max_subintervals) {
                    info_ok = 0;
                } else {
                    half_mesh();
                    y.assign(size_t(N) * M, 0.0);
                    info_ok = 1;
                }
            }
            if (!(info_ok && error_norm > op.abstol)) break;
            if (rounds >= op.max_rounds) { retcode = RET_MAXITERS; return; }
        }
        retcode = info_ok ? RET_SUCCESS : RET_FAILURE;
    }
};

}  // namespace oracle
