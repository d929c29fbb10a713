// FIRK collocation in the expanded form (Radau IIA, Lobatto IIIA/IIIB/IIIC), one warp per
// instance: lib/BoundaryValueDiffEqFIRK/src/firk.jl:290-622 (the expanded cache, its Newton
// solve and adaptive rounds), collocation.jl:44-120 (the residual), adaptivity.jl:7-606 (the
// continuous extension q, the defect, mesh selection and the solution transfer).
//
// Unknowns per interval: the node y_i and the stage derivatives K_1..K_s (a.K, FS x M per
// interval). Each Newton step linearises every interval's stage equations, eliminates its
// stage unknowns (firk_block, in the structured solve's interval loop) and solves the node
// system with the same elimination, shuffle tree and separator solve as the MIRK path; the
// stages follow from the kept condensation records (firk_update). Everything is FP64 and the
// iteration is NewtonRaphson, the FIRK algorithms' default (algorithms.jl:9). The mesh
// selection and halving are the MIRK path's; the transfer evaluates the quintic interpolant
// through the nodes, their f and q at the old interval's midpoint, writes the new nodes and
// lays the stage slots out as a first guess (each interval's slots its right node's value,
// firk.jl:76-83). Boundary conditions at interior times are not covered: an instance whose
// standard BCs name a time other than its tspan's ends fails with flag bit 2.
#pragma once

namespace bvp {

// extend_y (firk.jl:76-83) on the current buffer
BVP_DEV void firk_extend(const Args& a, const Inst& I) {
    const double* y = y_of(a, I, I.cur);
    double* K = a.K + I.nb * FN;
    for (int k = lane_id(); k < (I.N - 1) * FN; k += 32) K[k] = y[(k / FN + 1) * M + k % M];
    __syncwarp();
}

// Φ (collocation.jl:44-120): stage rows f(Y_r, t_r) - K_r and continuity rows, with the BC
// rows on lane 0; ||F||_inf over all of them (+inf if any is not finite).
BVP_DEV double firk_residual(const Args& a, const Inst& I) {
    const int lane = lane_id();
    const double* mesh = mesh_of(a, I, I.cur);
    const double* h = h_of(a, I, I.cur);
    const double* y = y_of(a, I, I.cur);
    const double* K = a.K + I.nb * FN;
    double mx = 0.0;
    bool bad = false;
    for (int i = lane; i < I.N - 1; i += 32) {
        const double hi = h[i];
        const double* Ki = K + i * FN;
#pragma unroll 1
        for (int r = 0; r < FS; ++r) {
            double Y[M], fy[M];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                double acc = y[i * M + m];
#pragma unroll
                for (int j = 0; j < FS; ++j) acc += hi * (Ki[j * M + m] * FA[r][j]);
                Y[m] = acc;
            }
            call_f<double, double>(fy, Y, I.p, mesh[i] + FC[r] * hi);
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const double v = fy[m] - Ki[r * M + m];
                bad |= !isfinite(v);
                mx = fmax(mx, fabs(v));
            }
        }
#pragma unroll
        for (int m = 0; m < M; ++m) {
            double acc = 0.0;
#pragma unroll
            for (int j = 0; j < FS; ++j) acc += Ki[j * M + m] * FB[j];
            const double v = (y[(i + 1) * M + m] - y[i * M + m]) - hi * acc;
            bad |= !isfinite(v);
            mx = fmax(mx, fabs(v));
        }
    }
    __syncwarp();
    if (lane == 0) mx = fmax(mx, bc_rows_lane0<double>(a, I, I.p, bad));
    __syncwarp();
    mx = warp_max(mx);
    return warp_any(bad) ? dinf() : mx;
}

// After the structured solve: K -= X_r + X_y δy_i per interval, y += δy.
BVP_DEV void firk_update(const Args& a, const Inst& I) {
    const int lane = lane_id();
    double* y = y_of(a, I, I.cur);
    double* K = a.K + I.nb * FN;
    const JT* dl = a.delta + I.nb * M;
    for (int i = lane; i < I.N - 1; i += 32) {
        const double* X = a.fx + (I.nb + i) * FXW;
#pragma unroll 1
        for (int row = 0; row < FN; ++row) {
            double v = X[row * (M + 1) + M];
#pragma unroll
            for (int c = 0; c < M; ++c) v += X[row * (M + 1) + c] * double(dl[i * M + c]);
            K[i * FN + row] -= v;
        }
    }
    for (int k = lane; k < I.N * M; k += 32) y[k] += double(dl[k]);
    __syncwarp();
}

// NewtonRaphson on the expanded system (termination on ||F||_inf <= abstol, with the stall and
// divergence tests of the MIRK path's Newton and no line-search retry).
BVP_DEV bool firk_newton(const Args& a, Inst& I, InstState& s) {
    int it = 0;
    double nrm = firk_residual(a, I);
    s.resid = nrm;
    if (!isfinite(nrm)) return false;
    if (nrm <= a.abstol) return true;
    const double nrm0 = nrm;
    double best = nrm;
    int stall = 0;
    bool ok = false;
#pragma unroll 1
    for (; it < a.max_newton; ++it) {
        bc_jacobian(a, I);
        if (!linear_solve(a, I)) break;
        firk_update(a, I);
        nrm = firk_residual(a, I);
        s.resid = nrm;
        if (!isfinite(nrm)) break;
        if (nrm <= a.abstol) { ok = true; ++it; break; }
        if (nrm > a.divergence_factor * nrm0) { ++it; break; }
        if (nrm < best) { best = nrm; stall = 0; }
        else if (++stall >= a.stall_steps) { ++it; break; }
    }
    s.newton_iters += it;
    return ok;
}

// q (adaptivity.jl:579-606) of interval i at τ from node y_i and stages K_i: value z and
// derivative zp; coefficients c_k = (q_coeff K)_k / h^k, q = y_i + sum_k c_k (τ h)^(k+1)
BVP_DEV void firk_q(const double* yi, const double* Ki, double hi, double tau, double* z, double* zp) {
#pragma unroll
    for (int m = 0; m < M; ++m) {
        double v = yi[m], d = 0.0, hk = 1.0, th = 1.0;
        const double tauh = tau * hi;
#pragma unroll
        for (int k = 0; k < FS; ++k) {
            double ck = 0.0;
#pragma unroll
            for (int j = 0; j < FS; ++j) ck += FQ[k][j] * Ki[j * M + m];
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

// defect_estimate! (adaptivity.jl:375-420): at τ* and 1 - τ*, (q' - f(q)) / (|f(q)| + 1)
BVP_DEV double firk_defect(const Args& a, const Inst& I) {
    const int lane = lane_id();
    const double* mesh = mesh_of(a, I, I.cur);
    const double* h = h_of(a, I, I.cur);
    const double* y = y_of(a, I, I.cur);
    const double* K = a.K + I.nb * FN;
    double dn = 0.0;
    bool bad = false;
    for (int i = lane; i < I.N - 1; i += 32) {
        double est[2];
#pragma unroll 1
        for (int smp = 0; smp < 2; ++smp) {
            const double tau = smp ? 1.0 - FTAU : FTAU;
            double z[M], zp[M], fz[M];
            firk_q(y + i * M, K + i * FN, h[i], tau, z, zp);
            call_f<double, double>(fz, z, I.p, mesh[i] + tau * h[i]);
            double e = 0.0;
#pragma unroll
            for (int m = 0; m < M; ++m) e = fmax(e, fabs((zp[m] - fz[m]) / (fabs(fz[m]) + 1.0)));
            est[smp] = e;
        }
        const double ei = est[0] > est[1] ? est[0] : est[1];
        a.err[I.nb + i] = ei;
        bad |= isnan(ei);
        dn = fmax(dn, ei);
    }
    __syncwarp();
    dn = warp_max(dn);
    return warp_any(bad) ? dinf() : dn;
}

// interp_eval! (adaptivity.jl:7-50, 191-245) onto the new mesh in buffer cur^1: the quintic
// S(τ) on [0, h] with S = y_i, y_{i+1} and S' = f(y_i), f(y_{i+1}) at the ends, S = q and S' = q'
// at the midpoint, evaluated at τ = t - t_i.
BVP_DEV void firk_transfer(const Args& a, const Inst& I, int newN) {
    const int lane = lane_id();
    const int No = I.N;
    const double* om = mesh_of(a, I, I.cur);
    const double* oh = h_of(a, I, I.cur);
    const double* oy = y_of(a, I, I.cur);
    const double* nm = mesh_of(a, I, I.cur ^ 1);
    double* ny = y_of(a, I, I.cur ^ 1);
    const double* K = a.K + I.nb * FN;
    for (int j = lane; j < newN; j += 32) {
        const double t = nm[j];
        const int i = interval_of(om, No, t);
        const double hj = oh[i];
        double fa[M], fb[M], zm[M], zpm[M];
        call_f<double, double>(fa, oy + i * M, I.p, om[i]);
        call_f<double, double>(fb, oy + (i + 1) * M, I.p, om[i + 1]);
        firk_q(oy + i * M, K + i * FN, hj, 0.5, zm, zpm);
        // rows: value at 0, h, h/2; derivative at 0, h, h/2 (s_constraints_block)
        double A[36], X[6 * M];
        const double tt[3] = {0.0, hj, hj / 2.0};
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            double pw = 1.0, dp = 0.0;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                A[r * 6 + k] = pw;
                A[(r + 3) * 6 + k] = dp;
                dp = (k + 1) * pw;
                pw *= tt[r];
            }
        }
#pragma unroll
        for (int m = 0; m < M; ++m) {
            X[0 * M + m] = oy[i * M + m];
            X[1 * M + m] = oy[(i + 1) * M + m];
            X[2 * M + m] = zm[m];
            X[3 * M + m] = fa[m];
            X[4 * M + m] = fb[m];
            X[5 * M + m] = zpm[m];
        }
#pragma unroll 1
        for (int k = 0; k < 6; ++k) {
            int p = k;
            for (int r = k + 1; r < 6; ++r)
                if (fabs(A[r * 6 + k]) > fabs(A[p * 6 + k])) p = r;
            if (p != k) {
                for (int q = 0; q < 6; ++q) { const double tq = A[k * 6 + q]; A[k * 6 + q] = A[p * 6 + q]; A[p * 6 + q] = tq; }
                for (int q = 0; q < M; ++q) { const double tq = X[k * M + q]; X[k * M + q] = X[p * M + q]; X[p * M + q] = tq; }
            }
            for (int r = k + 1; r < 6; ++r) {
                const double mlt = A[r * 6 + k] / A[k * 6 + k];
                for (int q = k; q < 6; ++q) A[r * 6 + q] -= mlt * A[k * 6 + q];
                for (int q = 0; q < M; ++q) X[r * M + q] -= mlt * X[k * M + q];
            }
        }
#pragma unroll 1
        for (int k = 5; k >= 0; --k)
            for (int q = 0; q < M; ++q) {
                double v = X[k * M + q];
                for (int c = k + 1; c < 6; ++c) v -= A[k * 6 + c] * X[c * M + q];
                X[k * M + q] = v / A[k * 6 + k];
            }
        const double tau = t - om[i];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            double v = 0.0, tk = 1.0;
#pragma unroll
            for (int k = 0; k < 6; ++k) { v += X[k * M + m] * tk; tk *= tau; }
            ny[j * M + m] = v;
        }
    }
    __syncwarp();
}

// One instance's adaptive FIRK solve (firk.jl:527-622): Newton, defect, mesh selection and
// transfer, or halving and a zero restart when Newton fails or the defect exceeds the threshold.
BVP_DEV void firk_solve_instance(const Args& a, Inst& I) {
    InstState s;
    s.retcode = RET_FAILURE; s.newton_iters = 0; s.rounds = 0; s.flags = 0;
    s.defect = __longlong_as_double(0x7ff8000000000000LL);
    s.resid = s.defect;
    s.global_err = s.defect;
    init_instance(a, I);
    firk_extend(a, I);
    if (!TWOPOINT) {
        const double* mesh = mesh_of(a, I, I.cur);
        bool interior = false;
#pragma unroll
        for (int k = 0; k < NBC; ++k) interior |= !(a.bc_t[k] == mesh[0] || a.bc_t[k] == mesh[I.N - 1]);
        if (interior) {
            s.flags |= 4;
            finish_instance(a, I, s);
            return;
        }
    }
    int info_ok = 1;
    bool maxed = false;
    while (true) {
        ++s.rounds;
        mesh_setup(a, I);
        double error_norm = 2 * a.abstol;
        const bool nl_ok = firk_newton(a, I, s);
        if (!a.adaptive) { s.retcode = nl_ok ? RET_SUCCESS : RET_FAILURE; info_ok = nl_ok; break; }
        bool ok = nl_ok;
        if (ok) {
            error_norm = firk_defect(a, I);
            s.defect = error_norm;
            ok = !(error_norm > a.defect_threshold) && isfinite(error_norm);
        }
        if (ok) {
            if (error_norm > a.abstol) {
                int newN = 0;
                info_ok = mesh_selector(a, I, newN);
                if (info_ok) {
                    firk_transfer(a, I, newN);
                    I.cur ^= 1;
                    I.N = newN;
                    firk_extend(a, I);
                }
            } else {
                info_ok = 1;
            }
        } else {
            if (2L * (I.N - 1) > a.max_sub || 2 * (I.N - 1) + 1 > I.cap) {
                info_ok = 0;
                if (2 * (I.N - 1) + 1 > I.cap) s.flags |= 2;
            } else {
                half_mesh(a, I, I.cur, I.cur ^ 1);
                I.cur ^= 1;
                I.N = 2 * (I.N - 1) + 1;
                double* y = y_of(a, I, I.cur);
                for (int k = lane_id(); k < I.N * M; k += 32) y[k] = 0.0;
                double* K = a.K + I.nb * FN;
                for (int k = lane_id(); k < (I.N - 1) * FN; k += 32) K[k] = 0.0;
                __syncwarp();
                info_ok = 1;
            }
        }
        if (!(info_ok && error_norm > a.abstol)) break;
        if (s.rounds >= a.max_rounds) { maxed = true; break; }
    }
    if (a.adaptive) s.retcode = maxed ? RET_MAXITERS : (info_ok ? RET_SUCCESS : RET_FAILURE);
    finish_instance(a, I, s);
}

}  // namespace bvp
