// FIRK coefficients for the device code, computed on the host from their defining conditions
// and handed to NVRTC as constants (bvp_firk_constants).
//
// Schemes (lib/BoundaryValueDiffEqFIRK/src/radau_tableaus.jl, lobatto_tableaus.jl; orders from
// alg_utils.jl:1-22): Radau IIA with s = 1, 2, 3, 5, 7 stages (order 2s - 1) and Lobatto IIIA,
// IIIB, IIIC with s = 2..5 (order 2s - 2).
//   nodes       Radau IIA: the right Radau points (closed forms up to s = 3; the published roots
//               for s = 5, 7); Lobatto: 0, 1 and the interior Lobatto points
//   A           Radau IIA and Lobatto IIIA by collocation, sum_j a_ij c_j^(k-1) = c_i^k / k;
//               IIIB a_ij = b_j (1 - a^IIIA_ji / b_i); IIIC a_i1 = b_1 with collocation for
//               k = 1..s-1 on the other columns
//   b           the collocation A's last row (c_s = 1)
//   q_coeff     W^-1, W_jk = k c_j^(k-1): the continuous extension whose derivative takes the
//               stage values at the nodes
//   τ*          the defect sample point as the reference sets it for each scheme
#pragma once
#include <cmath>
#include <cstdio>
#include <string>

struct BvpFirkTab {
    int family = 0, s = 0, order = 0;   // order 0: no such scheme
    double c[7] = {0}, b[7] = {0}, a[7][7] = {{0}}, q[7][7] = {{0}}, tau = 0.0;
};

// in-place Gaussian elimination with partial pivoting, n x n, nr right-hand sides (row-major)
inline bool bvp_firk_solve(int n, double* A, double* X, int nr) {
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int r = k + 1; r < n; ++r)
            if (std::fabs(A[r * n + k]) > std::fabs(A[p * n + k])) p = r;
        if (A[p * n + k] == 0.0) return false;
        if (p != k) {
            for (int j = 0; j < n; ++j) { const double t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
            for (int j = 0; j < nr; ++j) { const double t = X[k * nr + j]; X[k * nr + j] = X[p * nr + j]; X[p * nr + j] = t; }
        }
        for (int r = k + 1; r < n; ++r) {
            const double f = A[r * n + k] / A[k * n + k];
            for (int j = k; j < n; ++j) A[r * n + j] -= f * A[k * n + j];
            for (int j = 0; j < nr; ++j) X[r * nr + j] -= f * X[k * nr + j];
        }
    }
    for (int k = n - 1; k >= 0; --k)
        for (int j = 0; j < nr; ++j) {
            double v = X[k * nr + j];
            for (int i = k + 1; i < n; ++i) v -= A[k * n + i] * X[i * nr + j];
            X[k * nr + j] = v / A[k * n + k];
        }
    return true;
}

// family: 1 Radau IIA, 2 Lobatto IIIA, 3 Lobatto IIIB, 4 Lobatto IIIC (the bvp_options.firk codes)
inline BvpFirkTab bvp_firk_tableau(int family, int s) {
    BvpFirkTab t;
    t.family = family;
    t.s = s;
    const bool radau = family == 1;
    const bool ok = radau ? (s == 1 || s == 2 || s == 3 || s == 5 || s == 7) : (family >= 2 && family <= 4 && s >= 2 && s <= 5);
    if (!ok) return t;
    if (radau) {
        static const double r5[5] = {0.5710419611451768219312e-1, 0.27684301363812382768e+0,
                                     0.5835904323689168200567e+0, 0.8602401356562194478479e+0, 1.0};
        static const double r7[7] = {0.2931642715978489197205e-1, 0.14807859966848429185e+0,
                                     0.3369846902811542990971e+0, 0.5586715187715501320814e+0,
                                     0.7692338620300545009169e+0, 0.9269456713197411148519e+0, 1.0};
        if (s == 1) t.c[0] = 1.0;
        if (s == 2) { t.c[0] = 1.0 / 3.0; t.c[1] = 1.0; }
        if (s == 3) { const double q6 = std::sqrt(6.0); t.c[0] = (4.0 - q6) / 10.0; t.c[1] = (4.0 + q6) / 10.0; t.c[2] = 1.0; }
        if (s == 5) for (int i = 0; i < 5; ++i) t.c[i] = r5[i];
        if (s == 7) for (int i = 0; i < 7; ++i) t.c[i] = r7[i];
        t.order = 2 * s - 1;
        t.tau = 0.0;
    } else {
        t.c[0] = 0.0;
        t.c[s - 1] = 1.0;
        if (s == 3) t.c[1] = 0.5;
        if (s == 4) { const double q5 = std::sqrt(5.0); t.c[1] = 0.5 - q5 / 10.0; t.c[2] = 0.5 + q5 / 10.0; }
        if (s == 5) { const double q21 = std::sqrt(21.0); t.c[1] = 0.5 - q21 / 14.0; t.c[2] = 0.5; t.c[3] = 0.5 + q21 / 14.0; }
        t.order = 2 * s - 2;
        static const double tau_ab[6] = {0, 0, 0.5, 0.21132486540518713, 0.5, 0.33000947820757126};
        static const double tau_c[6] = {0, 0, 0.5, 0.7886751345948129, 0.5, 0.6699905217924309};
        t.tau = family == 4 ? tau_c[s] : tau_ab[s];
    }
    double coll[7][7] = {{0}};
    for (int i = 0; i < s; ++i) {
        double V[49], x[7];
        for (int k = 0; k < s; ++k) {
            for (int j = 0; j < s; ++j) V[k * s + j] = std::pow(t.c[j], k);
            x[k] = std::pow(t.c[i], k + 1) / (k + 1);
        }
        bvp_firk_solve(s, V, x, 1);
        for (int j = 0; j < s; ++j) coll[i][j] = x[j];
    }
    for (int j = 0; j < s; ++j) t.b[j] = coll[s - 1][j];
    if (family == 1 || family == 2) {
        for (int i = 0; i < s; ++i)
            for (int j = 0; j < s; ++j) t.a[i][j] = coll[i][j];
    } else if (family == 3) {
        for (int i = 0; i < s; ++i)
            for (int j = 0; j < s; ++j) t.a[i][j] = t.b[j] * (1.0 - coll[j][i] / t.b[i]);
    } else {
        for (int i = 0; i < s; ++i) {
            t.a[i][0] = t.b[0];
            const int n = s - 1;
            double V[49], x[7];
            for (int k = 0; k < n; ++k) {
                for (int j = 0; j < n; ++j) V[k * n + j] = std::pow(t.c[j + 1], k);
                x[k] = std::pow(t.c[i], k + 1) / (k + 1) - (k == 0 ? t.b[0] : 0.0);
            }
            bvp_firk_solve(n, V, x, 1);
            for (int j = 0; j < n; ++j) t.a[i][j + 1] = x[j];
        }
    }
    double W[49], X[49];
    for (int j = 0; j < s; ++j)
        for (int k = 0; k < s; ++k) {
            W[j * s + k] = (k + 1) * std::pow(t.c[j], k);
            X[j * s + k] = j == k ? 1.0 : 0.0;
        }
    bvp_firk_solve(s, W, X, s);
    for (int k = 0; k < s; ++k)
        for (int j = 0; j < s; ++j) t.q[k][j] = X[k * s + j];
    return t;
}

// The scheme as device constants (namespace bvp): FS, FORDER, FTAU, FC, FB, FA, FQ, with every
// double printed to round-trip exactly.
inline std::string bvp_firk_constants(const BvpFirkTab& t) {
    char buf[64];
    auto num = [&](double v) { std::snprintf(buf, sizeof(buf), "%.17g", v); return std::string(buf); };
    const int s = t.s;
    std::string o = "#define BVP_FIRK 1\nnamespace bvp {\nconstexpr int FS = " + std::to_string(s) +
                    ", FORDER = " + std::to_string(t.order) + ";\nconstexpr double FTAU = " + num(t.tau) + ";\n";
    auto vec = [&](const char* name, const double* v) {
        o += std::string("constexpr double ") + name + "[" + std::to_string(s) + "] = {";
        for (int i = 0; i < s; ++i) o += (i ? ", " : "") + num(v[i]);
        o += "};\n";
    };
    auto mat = [&](const char* name, const double (*m)[7]) {
        o += std::string("constexpr double ") + name + "[" + std::to_string(s) + "][" + std::to_string(s) + "] = {";
        for (int i = 0; i < s; ++i) {
            o += i ? ", {" : "{";
            for (int j = 0; j < s; ++j) o += (j ? ", " : "") + num(m[i][j]);
            o += "}";
        }
        o += "};\n";
    };
    vec("FC", t.c);
    vec("FB", t.b);
    mat("FA", t.a);
    mat("FQ", t.q);
    o += "}  // namespace bvp\n";
    return o;
}
