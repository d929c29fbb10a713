// FP64 CPU restatement of BoundaryValueDiffEq.jl's FIRK solve in the expanded form
// (nested_nlsolve = false, the default: lib/BoundaryValueDiffEqFIRK/src/algorithms.jl:9-110).
//
// TEST INFRASTRUCTURE ONLY: the parity tests compile it with a problem source and compare the
// CUDA library's FIRK path against it; the shipped library never links or calls it.
//
// Unknowns per interval: the node y_i and the stage derivatives K_1..K_s (extend_y,
// firk.jl:76-83); residual rows (collocation.jl:44-120): the continuity
// y_{i+1} - y_i - h sum_j b_j K_j and the stage equations f(y_i + h sum_j a_rj K_j, t_i + c_r h)
// - K_r, with the BC rows of the problem type. The Newton iteration is NewtonRaphson (the FIRK
// algorithms' default nlsolve, algorithms.jl:9) on ||F||_inf <= abstol with the exact Jacobian;
// its linear system is solved by eliminating each interval's stage unknowns from its own
// stage equations (an s·M dense solve) and solving the remaining almost-block-diagonal system
// in the nodes with the MIRK solver's structured elimination, then recovering the stages:
// the same Newton step as a direct solve of the expanded system, up to rounding.
//
// Adaptivity (adaptivity.jl:246-606, firk.jl:572-622): the defect of the continuous extension
// q at τ* and 1 - τ*, the defect-controlled mesh selection, halving and restart. Two points
// where the restatement takes the documented intent: (1) the new mesh's initial guess takes the
// interpolated node values at the node positions, and each interval's stage slots the value of
// its right node, as extend_y lays out a first guess; the reference writes the interpolated
// values to the first N entries of the expanded vector (firk.jl:598-601), which places them in
// stage slots and leaves the rest of the vector as it was; (2) the interpolant uses each old
// interval's own length; the reference scales it by the ratio of the expanded vectors' lengths
// whenever the mesh grows (adaptivity.jl:13-17). Boundary conditions at interior times are not
// covered: standard BCs are evaluated at the mesh endpoints only.
#pragma once
#include "firk_tableaus.hpp"
#include "mirk_oracle.hpp"

namespace oracle {

template <int M>
struct FirkSolver : InstanceSolver<M> {
    using Base = InstanceSolver<M>;
    using Base::N; using Base::mesh; using Base::h; using Base::y; using Base::F; using Base::p;
    using Base::op; using Base::pi; using Base::Sb; using Base::Rb; using Base::bcb;
    using Base::newton_total; using Base::newton_last; using Base::rounds; using Base::retcode;
    using Base::last_defect; using Base::last_resid; using Base::err_max;
    using DualU = Dual<M>;

    const FirkTableau& ft;
    std::vector<double> K;    // (N-1) x s x M stage derivatives
    std::vector<double> Fs;   // (N-1) x s x M stage residuals
    std::vector<double> X;    // (N-1) x (s M) x (M+1): J_K^-1 [J_y | R] of the last linearisation

    FirkSolver(const Tableau& dummy, const FirkTableau& t, const Options& o, const ProblemInfo& info,
               const double* params)
        : Base(dummy, o, info, params), ft(t) {}

    int S() const { return ft.s; }

    // extend_y (firk.jl:76-83): each interval's stage slots take its right node's value
    void extend() {
        K.assign(size_t(N - 1) * S() * M, 0.0);
        for (int i = 0; i + 1 < N; ++i)
            for (int r = 0; r < S(); ++r)
                for (int m = 0; m < M; ++m) K[(size_t(i) * S() + r) * M + m] = y[size_t(i + 1) * M + m];
    }

    // Φ (collocation.jl:44-120) and the BC rows; ||F||_inf over all rows (+inf if not finite)
    double residual() {
        const int s = S();
        F.assign(size_t(M) * N, 0.0);
        Fs.assign(size_t(N - 1) * s * M, 0.0);
        const int off = pi.twopoint ? pi.La : M;
        for (int i = 0; i + 1 < N; ++i) {
            const double hi = h[i];
            const double* Ki = &K[size_t(i) * s * M];
            for (int r = 0; r < s; ++r) {
                double Y[M], fy[M];
                for (int m = 0; m < M; ++m) {
                    double acc = y[size_t(i) * M + m];
                    for (int j = 0; j < s; ++j) acc += hi * (Ki[j * M + m] * ft.a[r][j]);
                    Y[m] = acc;
                }
                bvp_f<double, double>(fy, Y, p, mesh[i] + ft.c[r] * hi);
                for (int m = 0; m < M; ++m) Fs[(size_t(i) * s + r) * M + m] = fy[m] - Ki[r * M + m];
            }
            for (int m = 0; m < M; ++m) {
                double acc = 0.0;
                for (int j = 0; j < s; ++j) acc += Ki[j * M + m] * ft.b[j];
                F[size_t(off) + size_t(i) * M + m] = (y[size_t(i + 1) * M + m] - y[size_t(i) * M + m]) - hi * acc;
            }
        }
        if (!pi.twopoint) {
            std::vector<const double*> ptrs(pi.n_bc_pts);
            for (int k = 0; k < pi.n_bc_pts; ++k) ptrs[k] = pi.bc_t[k] == mesh[0] ? &y[0] : &y[size_t(N - 1) * M];
            bvp_bc<double, double>(&F[0], ptrs.data(), p);
        } else {
            double ra[M], rb[M];
            bvp_bca<double, double>(ra, &y[0], p);
            bvp_bcb<double, double>(rb, &y[size_t(N - 1) * M], p);
            for (int k = 0; k < pi.La; ++k) F[k] = ra[k];
            for (int k = 0; k < pi.Lb; ++k) F[size_t(pi.La) + size_t(N - 1) * M + k] = rb[k];
        }
        double nrm = 0.0;
        bool bad = false;
        for (double v : F) { if (!std::isfinite(v)) bad = true; nrm = std::max(nrm, std::fabs(v)); }
        for (double v : Fs) { if (!std::isfinite(v)) bad = true; nrm = std::max(nrm, std::fabs(v)); }
        return bad ? INFINITY : nrm;
    }

    // BC Jacobian blocks on the end nodes (both problem types)
    void bc_blocks() {
        bcb.clear();
        if (pi.twopoint) {
            DualU ua[M], ra[M], rb[M];
            for (int m = 0; m < M; ++m) { ua[m] = DualU(y[m]); ua[m].d[m] = 1.0; }
            bvp_bca<DualU, double>(ra, ua, p);
            double J0[M * M] = {0};
            for (int r = 0; r < pi.La; ++r) for (int c = 0; c < M; ++c) J0[r * M + c] = ra[r].d[c];
            this->add_bc_block(0, J0);
            for (int m = 0; m < M; ++m) { ua[m] = DualU(y[size_t(N - 1) * M + m]); ua[m].d[m] = 1.0; }
            bvp_bcb<DualU, double>(rb, ua, p);
            double J1[M * M] = {0};
            for (int r = 0; r < pi.Lb; ++r) for (int c = 0; c < M; ++c) J1[(pi.La + r) * M + c] = rb[r].d[c];
            this->add_bc_block(N - 1, J1);
            return;
        }
        const int P = pi.n_bc_pts;
        for (int k = 0; k < P; ++k) {
            std::vector<DualU> ua(size_t(P) * M);
            std::vector<const DualU*> ptrs(P);
            for (int q = 0; q < P; ++q) {
                const double* src = pi.bc_t[q] == mesh[0] ? &y[0] : &y[size_t(N - 1) * M];
                for (int m = 0; m < M; ++m) {
                    ua[q * M + m] = DualU(src[m]);
                    if (q == k) ua[q * M + m].d[m] = 1.0;
                }
                ptrs[q] = &ua[q * M];
            }
            DualU res[M];
            bvp_bc<DualU, double>(res, ptrs.data(), p);
            double G[M * M];
            for (int r = 0; r < M; ++r) for (int c = 0; c < M; ++c) G[r * M + c] = res[r].d[c];
            this->add_bc_block(pi.bc_t[k] == mesh[0] ? 0 : N - 1, G);
        }
    }

    // Linearisation and the condensed node system: per interval J_K (s M x s M) =
    // h a_rj J_f(Y_r) - δ_rj I, J_y = J_f(Y_r); X = J_K^-1 [J_y | R_stage]; the node equation
    // δy_{i+1} + (h sum_j b_j X_y,j - I) δy_i = -(C_i + h sum_j b_j X_r,j).
    bool condense() {
        const int s = S(), n = s * M, w = M + 1;
        Sb.assign(size_t(N - 1) * M * M, 0.0);
        Rb.assign(size_t(N - 1) * M * M, 0.0);
        X.assign(size_t(N - 1) * n * w, 0.0);
        const int off = pi.twopoint ? pi.La : M;
        std::vector<double> JK(size_t(n) * n);
        for (int i = 0; i + 1 < N; ++i) {
            const double hi = h[i];
            const double* Ki = &K[size_t(i) * s * M];
            double* Xi = &X[size_t(i) * n * w];
            std::fill(JK.begin(), JK.end(), 0.0);
            for (int r = 0; r < s; ++r) {
                DualU Y[M], fy[M];
                for (int m = 0; m < M; ++m) {
                    double acc = y[size_t(i) * M + m];
                    for (int j = 0; j < s; ++j) acc += hi * (Ki[j * M + m] * ft.a[r][j]);
                    Y[m] = DualU(acc);
                    Y[m].d[m] = 1.0;
                }
                bvp_f<DualU, double>(fy, Y, p, mesh[i] + ft.c[r] * hi);
                for (int q = 0; q < M; ++q) {
                    const int row = r * M + q;
                    for (int c = 0; c < M; ++c) {
                        const double J = fy[q].d[c];
                        Xi[row * w + c] = J;                               // J_y
                        for (int j = 0; j < s; ++j) JK[size_t(row) * n + j * M + c] = hi * ft.a[r][j] * J;
                    }
                    JK[size_t(row) * n + row] -= 1.0;
                    Xi[row * w + M] = Fs[(size_t(i) * s + r) * M + q];   // R
                }
            }
            if (!firk_dense(n, JK.data(), Xi, w)) return false;
            double* Si = &Sb[size_t(i) * M * M];
            double* Ri = &Rb[size_t(i) * M * M];
            for (int q = 0; q < M; ++q) {
                for (int c = 0; c < M; ++c) {
                    double acc = 0.0;
                    for (int j = 0; j < s; ++j) acc += ft.b[j] * Xi[(j * M + q) * w + c];
                    Si[q * M + c] = hi * acc - (q == c ? 1.0 : 0.0);
                    Ri[q * M + c] = q == c ? 1.0 : 0.0;
                }
                double acc = 0.0;
                for (int j = 0; j < s; ++j) acc += ft.b[j] * Xi[(j * M + q) * w + M];
                F[size_t(off) + size_t(i) * M + q] += hi * acc;
            }
        }
        bc_blocks();
        return true;
    }

    // NewtonRaphson on the expanded system; returns true on ||F||_inf <= abstol
    bool newton() {
        int it = 0;
        double nrm = residual();
        last_resid = nrm;
        newton_last = 0;
        if (!std::isfinite(nrm)) return false;
        if (nrm <= op.abstol) return true;
        const double nrm0 = nrm;
        double best = nrm;
        int stall = 0;
        std::vector<double> delta;
        bool ok = false;
        for (; it < op.max_newton; ++it) {
            if (!condense() || !this->linear_solve(delta)) break;
            const int s = S(), n = s * M, w = M + 1;
            for (int i = 0; i + 1 < N; ++i) {
                const double* Xi = &X[size_t(i) * n * w];
                for (int row = 0; row < n; ++row) {
                    double v = Xi[row * w + M];
                    for (int c = 0; c < M; ++c) v += Xi[row * w + c] * delta[size_t(i) * M + c];
                    K[size_t(i) * n + row] -= v;
                }
            }
            for (size_t q = 0; q < y.size(); ++q) y[q] += delta[q];
            nrm = residual();
            last_resid = nrm;
            if (!std::isfinite(nrm)) break;
            if (nrm <= op.abstol) { ok = true; ++it; break; }
            if (nrm > op.divergence_factor * nrm0) { ++it; break; }
            if (nrm < best) { best = nrm; stall = 0; }
            else if (++stall >= op.stall_steps) { ++it; break; }
        }
        newton_total += it;
        newton_last = it;
        return ok;
    }

    // continuous extension q (adaptivity.jl:579-606) of interval i at τ: value and derivative
    void eval_q(int i, double tau, double* z, double* zp) const {
        const int s = S();
        const double hi = h[i];
        const double* Ki = &K[size_t(i) * s * M];
        q_of(&y[size_t(i) * M], Ki, hi, tau, z, zp);
    }

    // q = y_i + sum_k c_k (τ h)^(k+1), c_k = (q_coeff K)_k / h^k, powers by repeated products
    void q_of(const double* yi, const double* Ki, double hi, double tau, double* z, double* zp) const {
        const int s = S();
        for (int m = 0; m < M; ++m) {
            double v = yi[m], d = 0.0, hk = 1.0, th = 1.0;
            const double tauh = tau * hi;
            for (int k = 0; k < s; ++k) {
                double ck = 0.0;
                for (int j = 0; j < s; ++j) ck += ft.q[k][j] * Ki[j * M + m];
                ck /= hk;
                d += (k + 1) * ck * th;
                th *= tauh;
                v += ck * th;
                hk *= hi;
            }
            z[m] = v;
            zp[m] = d;
        }
    }

    // defect_estimate! (adaptivity.jl:375-420)
    double defect_estimate() {
        err_max.assign(N - 1, 0.0);
        double dn = 0.0;
        for (int i = 0; i + 1 < N; ++i) {
            double est[2];
            for (int smp = 0; smp < 2; ++smp) {
                const double tau = smp ? 1.0 - ft.tau_star : ft.tau_star;
                double z[M], zp[M], fz[M];
                eval_q(i, tau, z, zp);
                bvp_f<double, double>(fz, z, p, mesh[i] + tau * h[i]);
                double e = 0.0;
                for (int m = 0; m < M; ++m) e = std::max(e, std::fabs((zp[m] - fz[m]) / (std::fabs(fz[m]) + 1.0)));
                est[smp] = e;
            }
            err_max[i] = est[0] > est[1] ? est[0] : est[1];
            if (!(err_max[i] <= dn)) dn = std::isnan(err_max[i]) ? INFINITY : std::max(dn, err_max[i]);
        }
        last_defect = dn;
        return dn;
    }

    // interp_eval! (adaptivity.jl:7-50, 191-245): the quintic S through y_j, y_{j+1}, their f,
    // and q and q' at the interval's midpoint, evaluated at t - t_j
    void transfer(const std::vector<double>& old_mesh, const std::vector<double>& old_h) {
        const int On = int(old_mesh.size());
        std::vector<double> ny(size_t(N) * M);
        const std::vector<double> oy = y;
        for (int q = 0; q < N; ++q) {
            const double tq = mesh[q];
            const int j = interval_of(old_mesh.data(), On, tq);
            const double hj = old_h[j];
            double fa[M], fb[M], zm[M], zpm[M];
            bvp_f<double, double>(fa, &oy[size_t(j) * M], p, old_mesh[j]);
            bvp_f<double, double>(fb, &oy[size_t(j + 1) * M], p, old_mesh[j + 1]);
            // q at the old interval's midpoint
            q_of(&oy[size_t(j) * M], &K[size_t(j) * S() * M], hj, 0.5, zm, zpm);
            const double tt[3] = {0.0, hj, hj / 2.0};
            const double tau = tq - old_mesh[j];
            for (int m = 0; m < M; ++m) {
                // rows: value at 0, h, h/2; derivative at 0, h, h/2 (s_constraints_block)
                double A[36], x[6];
                for (int r = 0; r < 3; ++r) {
                    double pw = 1.0, dp = 0.0;
                    for (int k = 0; k < 6; ++k) {
                        A[r * 6 + k] = pw;
                        A[(r + 3) * 6 + k] = dp;
                        dp = (k + 1) * pw;
                        pw *= tt[r];
                    }
                }
                x[0] = oy[size_t(j) * M + m]; x[1] = oy[size_t(j + 1) * M + m]; x[2] = zm[m];
                x[3] = fa[m]; x[4] = fb[m]; x[5] = zpm[m];
                firk_dense(6, A, x, 1);
                double v = 0.0, tk = 1.0;
                for (int k = 0; k < 6; ++k) { v += x[k] * tk; tk *= tau; }
                ny[size_t(q) * M + m] = v;
            }
        }
        y.swap(ny);
        extend();
    }

    void solve() {
        int info_ok = 1;
        double error_norm = 2 * op.abstol;
        rounds = 0;
        retcode = RET_FAILURE;
        while (true) {
            ++rounds;
            error_norm = 2 * op.abstol;
            const bool nl_ok = newton();
            if (!op.adaptive) { retcode = nl_ok ? RET_SUCCESS : RET_FAILURE; return; }
            bool ok = nl_ok;
            if (ok) {
                error_norm = defect_estimate();
                ok = !(error_norm > op.defect_threshold) && std::isfinite(error_norm);
            }
            if (ok) {
                if (error_norm > op.abstol) {
                    std::vector<double> om, oh;
                    if (this->mesh_selector(om, oh, CTL_DEFECT, false, ft.order)) {
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
                    this->half_mesh();
                    y.assign(size_t(N) * M, 0.0);
                    K.assign(size_t(N - 1) * S() * M, 0.0);
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
