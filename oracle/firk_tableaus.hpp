// FIRK (Radau IIA, Lobatto IIIA/IIIB/IIIC) coefficients, FP64, from their defining conditions.
//
// TEST INFRASTRUCTURE ONLY: part of the CPU oracle the parity tests compare the CUDA library
// against; nothing in the shipped library includes it.
//
// The reference tabulates these schemes in lib/BoundaryValueDiffEqFIRK/src/radau_tableaus.jl
// and lobatto_tableaus.jl (stage counts and orders: alg_utils.jl:1-22, Radau IIA order 2s-1,
// Lobatto order 2s-2). Here every coefficient is computed from what defines it:
//   nodes c     Radau IIA: the right Radau points on (0, 1] (1/3, (4 -+ sqrt 6)/10 in closed form,
//               s = 5 and 7 as the published roots); Lobatto: 0, 1 and the interior Lobatto
//               points (1/2, 1/2 -+ sqrt5/10, 1/2 -+ sqrt21/14)
//   A (Radau IIA, Lobatto IIIA)  collocation: sum_j a_ij c_j^(k-1) = c_i^k / k, k = 1..s
//   b           the last row of the collocation A (c_s = 1)
//   Lobatto IIIB a_ij = b_j (1 - a^IIIA_ji / b_i)
//   Lobatto IIIC a_i1 = b_1 and the collocation conditions for k = 1..s-1 on the other columns
//   q_coeff     the continuous extension q(τ) = y_i + h sum_k (q K)_k τ^k whose derivative
//               takes the stage values K_j at τ = c_j: q = W^-1 with W_jk = k c_j^(k-1)
//               (the reference's q_coeff tables, radau_tableaus.jl:16-149)
//   τ*          the defect sample point of each scheme as the reference sets it
#pragma once
#include <cmath>

namespace oracle {

enum FirkFamily : int { FIRK_RADAU_IIA = 0, FIRK_LOBATTO_IIIA = 1, FIRK_LOBATTO_IIIB = 2, FIRK_LOBATTO_IIIC = 3 };

struct FirkTableau {
    int family = 0, s = 0, order = 0;   // order 0: no such scheme
    double c[7] = {0}, b[7] = {0};
    double a[7][7] = {{0}};             // a[i][j]: stage i's weight on K_j
    double q[7][7] = {{0}};             // q_coeff[k][j]
    double tau_star = 0;
};

// Gaussian elimination with partial pivoting on an n x n row-major system with nr right-hand
// sides (columns of X, row-major n x nr), in place.
inline bool firk_dense(int n, double* A, double* X, int nr) {
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int r = k + 1; r < n; ++r)
            if (std::fabs(A[r * n + k]) > std::fabs(A[p * n + k])) p = r;
        if (A[p * n + k] == 0.0) return false;
        if (p != k) {
            for (int c = 0; c < n; ++c) { const double t = A[k * n + c]; A[k * n + c] = A[p * n + c]; A[p * n + c] = t; }
            for (int c = 0; c < nr; ++c) { const double t = X[k * nr + c]; X[k * nr + c] = X[p * nr + c]; X[p * nr + c] = t; }
        }
        for (int r = k + 1; r < n; ++r) {
            const double m = A[r * n + k] / A[k * n + k];
            for (int c = k; c < n; ++c) A[r * n + c] -= m * A[k * n + c];
            for (int c = 0; c < nr; ++c) X[r * nr + c] -= m * X[k * nr + c];
        }
    }
    for (int k = n - 1; k >= 0; --k)
        for (int c = 0; c < nr; ++c) {
            double v = X[k * nr + c];
            for (int j = k + 1; j < n; ++j) v -= A[k * n + j] * X[j * nr + c];
            X[k * nr + c] = v / A[k * n + k];
        }
    return true;
}

inline FirkTableau make_firk_tableau(int family, int s) {
    FirkTableau t;
    t.family = family;
    t.s = s;
    const bool radau = family == FIRK_RADAU_IIA;
    if (radau ? !(s == 1 || s == 2 || s == 3 || s == 5 || s == 7) : !(s >= 2 && s <= 5) || family > 3 || family < 0)
        return t;
    double* c = t.c;
    if (radau) {
        if (s == 1) c[0] = 1.0;
        if (s == 2) { c[0] = 1.0 / 3.0; c[1] = 1.0; }
        if (s == 3) { const double r6 = std::sqrt(6.0); c[0] = (4.0 - r6) / 10.0; c[1] = (4.0 + r6) / 10.0; c[2] = 1.0; }
        if (s == 5) {
            const double v[5] = {0.5710419611451768219312e-1, 0.27684301363812382768e+0, 0.5835904323689168200567e+0,
                                 0.8602401356562194478479e+0, 1.0};
            for (int i = 0; i < 5; ++i) c[i] = v[i];
        }
        if (s == 7) {
            const double v[7] = {0.2931642715978489197205e-1, 0.14807859966848429185e+0, 0.3369846902811542990971e+0,
                                 0.5586715187715501320814e+0, 0.7692338620300545009169e+0, 0.9269456713197411148519e+0,
                                 1.0};
            for (int i = 0; i < 7; ++i) c[i] = v[i];
        }
        t.order = 2 * s - 1;
        t.tau_star = 0.0;
    } else {
        c[0] = 0.0;
        c[s - 1] = 1.0;
        if (s == 3) c[1] = 0.5;
        if (s == 4) { const double r5 = std::sqrt(5.0); c[1] = 0.5 - r5 / 10.0; c[2] = 0.5 + r5 / 10.0; }
        if (s == 5) { const double r21 = std::sqrt(21.0); c[1] = 0.5 - r21 / 14.0; c[2] = 0.5; c[3] = 0.5 + r21 / 14.0; }
        t.order = 2 * s - 2;
        const double ts_ab[6] = {0, 0, 0.5, 0.21132486540518713, 0.5, 0.33000947820757126};
        const double ts_c[6] = {0, 0, 0.5, 0.7886751345948129, 0.5, 0.6699905217924309};
        t.tau_star = family == FIRK_LOBATTO_IIIC ? ts_c[s] : ts_ab[s];
    }
    // collocation A: for each stage i, sum_j a_ij c_j^(k-1) = c_i^k / k
    double coll[7][7] = {{0}};
    for (int i = 0; i < s; ++i) {
        double V[49], x[7];
        for (int k = 0; k < s; ++k) {
            for (int j = 0; j < s; ++j) V[k * s + j] = std::pow(c[j], k);
            x[k] = std::pow(c[i], k + 1) / (k + 1);
        }
        firk_dense(s, V, x, 1);
        for (int j = 0; j < s; ++j) coll[i][j] = x[j];
    }
    for (int j = 0; j < s; ++j) t.b[j] = coll[s - 1][j];
    if (family == FIRK_RADAU_IIA || family == FIRK_LOBATTO_IIIA) {
        for (int i = 0; i < s; ++i)
            for (int j = 0; j < s; ++j) t.a[i][j] = coll[i][j];
    } else if (family == FIRK_LOBATTO_IIIB) {
        for (int i = 0; i < s; ++i)
            for (int j = 0; j < s; ++j) t.a[i][j] = t.b[j] * (1.0 - coll[j][i] / t.b[i]);
    } else {
        for (int i = 0; i < s; ++i) {
            t.a[i][0] = t.b[0];
            const int n = s - 1;
            double V[49], x[7];
            for (int k = 0; k < n; ++k) {
                for (int j = 0; j < n; ++j) V[k * n + j] = std::pow(c[j + 1], k);
                x[k] = std::pow(c[i], k + 1) / (k + 1) - (k == 0 ? t.b[0] : 0.0);
            }
            firk_dense(n, V, x, 1);
            for (int j = 0; j < n; ++j) t.a[i][j + 1] = x[j];
        }
    }
    // q = W^-1, W_jk = k c_j^(k-1)
    {
        double W[49], X[49];
        for (int j = 0; j < s; ++j)
            for (int k = 0; k < s; ++k) {
                W[j * s + k] = (k + 1) * std::pow(c[j], k);
                X[j * s + k] = j == k ? 1.0 : 0.0;
            }
        firk_dense(s, W, X, s);
        for (int k = 0; k < s; ++k)
            for (int j = 0; j < s; ++j) t.q[k][j] = X[k * s + j];
    }
    return t;
}

}  // namespace oracle
