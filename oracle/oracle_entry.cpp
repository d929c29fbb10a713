// C ABI of the CPU oracle, compiled once per problem source (BVP_PROBLEM_HEADER) and
// state dimension (BVP_M) by oracle/oracle.py.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, the smoke check and the benchmark's CPU
// baseline leg to check the CUDA library; never part of the shipped path.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "dual.hpp"

using std::sin; using std::cos; using std::tan; using std::exp; using std::log;
using std::sqrt; using std::tanh; using std::sinh; using std::cosh; using std::atan;
using std::pow; using std::fabs; using std::abs;
using oracle::Dual;

#define BVP_F template <class T, class P> inline void bvp_f(T* du, const T* u, const P* p, P t)
#define BVP_BC template <class T, class P> inline void bvp_bc(T* res, const T* const* ua, const P* p)
#define BVP_BCA template <class T, class P> inline void bvp_bca(T* res, const T* ua, const P* p)
#define BVP_BCB template <class T, class P> inline void bvp_bcb(T* res, const T* ub, const P* p)
// optional singular term S u of y' = S y / t + f(t, y) (the problem's singular_term)
#define BVP_SING template <class T, class P> inline void bvp_sing(T* su, const T* u, const P* p)

#ifndef BVP_M
#error "BVP_M must be defined"
#endif
#ifndef BVP_TWOPOINT
#define BVP_TWOPOINT 0
#endif

#include BVP_PROBLEM_HEADER

#if BVP_TWOPOINT
template <class T, class P> inline void bvp_bc(T*, const T* const*, const P*) {}
#else
template <class T, class P> inline void bvp_bca(T*, const T*, const P*) {}
template <class T, class P> inline void bvp_bcb(T*, const T*, const P*) {}
#endif

#include "mirk_oracle.hpp"
#include "firk_oracle.hpp"

using namespace oracle;
static constexpr int MM = BVP_M;

extern "C" {

int oracle_state_dim() { return MM; }

void oracle_default_options(Options* o) { fill_default_options(o); }

// Uniform mesh of n intervals on [t0, t1]: t0 + i*(t1-t0)/n via fma (the reference's
// range(t0; stop = t1, length = n + 1), Core/utils.jl:694-700), endpoints exact.
static void uniform_mesh(double t0, double t1, int n, double* mesh) {
    const double hh = (t1 - t0) / n;
    for (int i = 0; i <= n; ++i) mesh[i] = std::fma(double(i), hh, t0);
    mesh[n] = t1;
}

void oracle_uniform_mesh(double t0, double t1, int n, double* mesh) { uniform_mesh(t0, t1, n, mesh); }

// Full adaptive solve of a batch of independent instances (the reference's
// EnsembleProblem analogue; each instance follows solve! exactly).
//   y0_mode 0: y0 holds M values per instance, copied to every mesh point
//   y0_mode 1: y0 holds (n_intervals[i]+1)*M values per instance, packed
// Outputs are per instance with capacity cap_nodes; K_out/KI_out may be null.
int oracle_solve_batch(const ProblemInfo* info, const Options* opt, int n_inst,
                       const double* params, const int32_t* n_intervals, const double* tspans,
                       int y0_mode, const double* y0, int cap_nodes, int32_t* retcode,
                       int32_t* n_nodes, double* mesh_out, double* y_out, int32_t* newton_iters,
                       int32_t* rounds, double* defect, double* resid, double* K_out,
                       double* KI_out, double* global_err) {
    if (info->M != MM) return -1;
    const Tableau tb = make_tableau(opt->order, opt->mirk6i);
    if (tb.order == 0) return -2;
    // HOErrorControl solves with MIRK(p+2) (adaptivity.jl:552-555): MIRK4, MIRK5, MIRK6 exist
    const bool ho = opt->adaptive && opt->controller != CTL_DEFECT && opt->global_method == GLOBAL_HO;
    const Tableau tb_hi = ho ? make_tableau(opt->order + 2) : Tableau();
    if (ho && (opt->mirk6i || opt->order + 2 > 6)) return -3;
    std::vector<int64_t> y0_off(n_inst + 1, 0);
    for (int i = 0; i < n_inst; ++i)
        y0_off[i + 1] = y0_off[i] + (y0_mode == 1 ? int64_t(n_intervals[i] + 1) * MM : MM);
    const int NS = std::max(1, tb.s_star - tb.s);
    int nt = opt->nthreads;
#ifdef _OPENMP
    if (nt <= 0) nt = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
#endif
    for (int q = 0; q < n_inst; ++q) {
        InstanceSolver<MM> sv(tb, *opt, *info, params + size_t(q) * info->n_params);
        if (ho) sv.tb_hi = &tb_hi;
        const int n = n_intervals[q];
        sv.N = n + 1;
        sv.mesh.resize(n + 1);
        uniform_mesh(tspans[2 * q], tspans[2 * q + 1], n, sv.mesh.data());
        sv.h.resize(n);
        for (int i = 0; i < n; ++i) sv.h[i] = sv.mesh[i + 1] - sv.mesh[i];
        sv.y.resize(size_t(n + 1) * MM);
        const double* src = y0 + y0_off[q];
        for (int i = 0; i <= n; ++i)
            for (int m = 0; m < MM; ++m) sv.y[size_t(i) * MM + m] = (y0_mode == 1) ? src[size_t(i) * MM + m] : src[m];
        sv.solve();
        if (K_out || KI_out) {
            const double keep = sv.last_resid;
            sv.finalize_stages();
            sv.last_resid = keep;
        }
        retcode[q] = sv.retcode;
        n_nodes[q] = sv.N;
        newton_iters[q] = sv.newton_total;
        rounds[q] = sv.rounds;
        defect[q] = sv.last_defect;
        resid[q] = sv.last_resid;
        if (global_err) global_err[q] = sv.last_global;
        const int nc = std::min(sv.N, cap_nodes);
        if (sv.N > cap_nodes) retcode[q] = 3;
        for (int i = 0; i < nc; ++i) {
            mesh_out[size_t(q) * cap_nodes + i] = sv.mesh[i];
            for (int m = 0; m < MM; ++m) y_out[(size_t(q) * cap_nodes + i) * MM + m] = sv.y[size_t(i) * MM + m];
        }
        if (K_out && sv.K.size() >= size_t(nc - 1) * tb.s * MM)
            std::memcpy(K_out + size_t(q) * (cap_nodes - 1) * tb.s * MM, sv.K.data(),
                        sizeof(double) * size_t(nc - 1) * tb.s * MM);
        if (KI_out && sv.KI.size() >= size_t(nc - 1) * NS * MM)
            std::memcpy(KI_out + size_t(q) * (cap_nodes - 1) * NS * MM, sv.KI.data(),
                        sizeof(double) * size_t(nc - 1) * NS * MM);
    }
    return 0;
}

// One residual evaluation on a given mesh / solution: F (M*N) in the reference's
// ordering, K ((N-1) x s x M). Returns ||F||_inf.
double oracle_residual(const ProblemInfo* info, const Options* opt, const double* params, int N,
                       const double* mesh, const double* y, double* F_out, double* K_out) {
    const Tableau tb = make_tableau(opt->order, opt->mirk6i);
    InstanceSolver<MM> sv(tb, *opt, *info, params);
    sv.N = N;
    sv.mesh.assign(mesh, mesh + N);
    sv.h.resize(N - 1);
    for (int i = 0; i < N - 1; ++i) sv.h[i] = mesh[i + 1] - mesh[i];
    sv.y.assign(y, y + size_t(N) * MM);
    const double nrm = sv.residual();
    if (F_out) std::memcpy(F_out, sv.F.data(), sizeof(double) * sv.F.size());
    if (K_out) std::memcpy(K_out, sv.K.data(), sizeof(double) * sv.K.size());
    return nrm;
}

// Collocation Jacobian blocks S_i = dr_i/dy_i, R_i = dr_i/dy_{i+1} ((N-1) x M x M each,
// row-major) and the BC rows as (node, M x M) pairs. Returns the number of BC blocks.
int oracle_jacobian(const ProblemInfo* info, const Options* opt, const double* params, int N,
                    const double* mesh, const double* y, double* S_out, double* R_out,
                    int32_t* bc_nodes, double* bc_blocks) {
    const Tableau tb = make_tableau(opt->order, opt->mirk6i);
    InstanceSolver<MM> sv(tb, *opt, *info, params);
    sv.N = N;
    sv.mesh.assign(mesh, mesh + N);
    sv.h.resize(N - 1);
    for (int i = 0; i < N - 1; ++i) sv.h[i] = mesh[i + 1] - mesh[i];
    sv.y.assign(y, y + size_t(N) * MM);
    sv.residual();
    sv.jacobian();
    std::memcpy(S_out, sv.Sb.data(), sizeof(double) * sv.Sb.size());
    std::memcpy(R_out, sv.Rb.data(), sizeof(double) * sv.Rb.size());
    for (size_t k = 0; k < sv.bcb.size(); ++k) {
        bc_nodes[k] = sv.bcb[k].node;
        std::memcpy(bc_blocks + k * MM * MM, sv.bcb[k].J, sizeof(double) * MM * MM);
    }
    return int(sv.bcb.size());
}

// One Newton step direction: solves J delta = -F at (mesh, y). Returns 0 on success.
int oracle_newton_step(const ProblemInfo* info, const Options* opt, const double* params, int N,
                       const double* mesh, const double* y, double* delta_out) {
    const Tableau tb = make_tableau(opt->order, opt->mirk6i);
    InstanceSolver<MM> sv(tb, *opt, *info, params);
    sv.N = N;
    sv.mesh.assign(mesh, mesh + N);
    sv.h.resize(N - 1);
    for (int i = 0; i < N - 1; ++i) sv.h[i] = mesh[i + 1] - mesh[i];
    sv.y.assign(y, y + size_t(N) * MM);
    sv.residual();
    sv.jacobian();
    std::vector<double> d;
    if (!sv.linear_solve(d)) return 1;
    std::memcpy(delta_out, d.data(), sizeof(double) * d.size());
    return 0;
}

// Defect estimate on (mesh, y): per-interval max |defect| and the norm.
double oracle_defect(const ProblemInfo* info, const Options* opt, const double* params, int N,
                     const double* mesh, const double* y, double* err_out) {
    const Tableau tb = make_tableau(opt->order, opt->mirk6i);
    InstanceSolver<MM> sv(tb, *opt, *info, params);
    sv.N = N;
    sv.mesh.assign(mesh, mesh + N);
    sv.h.resize(N - 1);
    for (int i = 0; i < N - 1; ++i) sv.h[i] = mesh[i + 1] - mesh[i];
    sv.y.assign(y, y + size_t(N) * MM);
    sv.residual();
    const double dn = sv.defect_estimate();
    if (err_out) std::memcpy(err_out, sv.err_max.data(), sizeof(double) * (N - 1));
    return dn;
}

// Interpolant u(t) (deriv 0) or u'(t) (deriv 1) of a solved instance given its mesh,
// solution and stages (interpolation.jl:17-204). order: 2..6, or 7 for MIRK6I.
void oracle_interpolate(int order, int N, const double* mesh, const double* y, const double* K,
                        const double* KI, int n_t, const double* ts, int deriv, double* out) {
    const Tableau tb = order == 7 ? make_tableau(6, 1) : make_tableau(order);
    const int S = tb.s, NS = std::max(1, tb.s_star - tb.s), ns = tb.s_star - tb.s;
    for (int k = 0; k < n_t; ++k) {
        const int i = interval_of(mesh, N, ts[k]);
        const double dt = mesh[i + 1] - mesh[i];
        const double tau = (ts[k] - mesh[i]) / dt;
        double w[9], wp[9];
        interp_weights(tb.scheme, tau, w, wp);
        const double* wv = deriv ? wp : w;
        for (int m = 0; m < MM; ++m) {
            double acc = 0;
            for (int r = 0; r < S; ++r) acc += K[(size_t(i) * S + r) * MM + m] * wv[r];
            for (int q = 0; q < ns; ++q) acc += KI[(size_t(i) * NS + q) * MM + m] * wv[S + q];
            out[size_t(k) * MM + m] = deriv ? acc : acc * dt + y[size_t(i) * MM + m];
        }
    }
}


// FIRK coefficients of one scheme (family: 0 Radau IIA, 1 Lobatto IIIA, 2 IIIB, 3 IIIC):
// out = [order, s, tau*, c(7), b(7), a(7x7), q(7x7)]; returns 0, or -1 for no such scheme.
int oracle_firk_tableau(int family, int stages, double* out) {
    const FirkTableau t = make_firk_tableau(family, stages);
    if (t.order == 0) return -1;
    out[0] = t.order; out[1] = t.s; out[2] = t.tau_star;
    for (int i = 0; i < 7; ++i) { out[3 + i] = t.c[i]; out[10 + i] = t.b[i]; }
    for (int i = 0; i < 7; ++i)
        for (int j = 0; j < 7; ++j) { out[17 + i * 7 + j] = t.a[i][j]; out[66 + i * 7 + j] = t.q[i][j]; }
    return 0;
}

// Expanded FIRK solve of a batch (firk.jl:290-622); arguments as oracle_solve_batch, with
// the scheme given by family and stages (opt->order is not used). K_out (may be null):
// the final stage derivatives, (cap_nodes - 1) x stages x M per instance.
int oracle_firk_solve_batch(const ProblemInfo* info, const Options* opt, int family, int stages, int n_inst,
                            const double* params, const int32_t* n_intervals, const double* tspans, int y0_mode,
                            const double* y0, int cap_nodes, int32_t* retcode, int32_t* n_nodes, double* mesh_out,
                            double* y_out, int32_t* newton_iters, int32_t* rounds, double* defect, double* resid,
                            double* K_out) {
    if (info->M != MM) return -1;
    const FirkTableau ft = make_firk_tableau(family, stages);
    if (ft.order == 0) return -2;
    if (!info->twopoint)
        for (int k = 0; k < info->n_bc_pts; ++k)
            for (int q = 0; q < n_inst; ++q)
                if (info->bc_t[k] != tspans[2 * q] && info->bc_t[k] != tspans[2 * q + 1]) return -3;
    const Tableau dummy = make_tableau(4);
    std::vector<int64_t> y0_off(n_inst + 1, 0);
    for (int i = 0; i < n_inst; ++i)
        y0_off[i + 1] = y0_off[i] + (y0_mode == 1 ? int64_t(n_intervals[i] + 1) * MM : MM);
    int nt = opt->nthreads;
#ifdef _OPENMP
    if (nt <= 0) nt = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
#endif
    for (int q = 0; q < n_inst; ++q) {
        FirkSolver<MM> sv(dummy, ft, *opt, *info, params + size_t(q) * info->n_params);
        const int n = n_intervals[q];
        sv.N = n + 1;
        sv.mesh.resize(n + 1);
        uniform_mesh(tspans[2 * q], tspans[2 * q + 1], n, sv.mesh.data());
        sv.h.resize(n);
        for (int i = 0; i < n; ++i) sv.h[i] = sv.mesh[i + 1] - sv.mesh[i];
        sv.y.resize(size_t(n + 1) * MM);
        const double* src = y0 + y0_off[q];
        for (int i = 0; i <= n; ++i)
            for (int m = 0; m < MM; ++m) sv.y[size_t(i) * MM + m] = (y0_mode == 1) ? src[size_t(i) * MM + m] : src[m];
        sv.extend();
        sv.solve();
        retcode[q] = sv.retcode;
        n_nodes[q] = sv.N;
        newton_iters[q] = sv.newton_total;
        rounds[q] = sv.rounds;
        defect[q] = sv.last_defect;
        resid[q] = sv.last_resid;
        const int nc = std::min(sv.N, cap_nodes);
        if (sv.N > cap_nodes) retcode[q] = 3;
        for (int i = 0; i < nc; ++i) {
            mesh_out[size_t(q) * cap_nodes + i] = sv.mesh[i];
            for (int m = 0; m < MM; ++m) y_out[(size_t(q) * cap_nodes + i) * MM + m] = sv.y[size_t(i) * MM + m];
        }
        if (K_out)
            std::memcpy(K_out + size_t(q) * (cap_nodes - 1) * stages * MM, sv.K.data(),
                        sizeof(double) * size_t(std::max(nc - 1, 0)) * stages * MM);
    }
    return 0;
}

// The FIRK residual (stage and continuity rows, BC rows) and its norm on a given mesh, nodes
// and stages: F as oracle_residual lays it out, Fs (N-1) x stages x M.
double oracle_firk_residual(const ProblemInfo* info, const Options* opt, int family, int stages,
                            const double* params, int N, const double* mesh, const double* y, const double* K,
                            double* F_out, double* Fs_out) {
    const FirkTableau ft = make_firk_tableau(family, stages);
    const Tableau dummy = make_tableau(4);
    FirkSolver<MM> sv(dummy, ft, *opt, *info, params);
    sv.N = N;
    sv.mesh.assign(mesh, mesh + N);
    sv.h.resize(N - 1);
    for (int i = 0; i + 1 < N; ++i) sv.h[i] = mesh[i + 1] - mesh[i];
    sv.y.assign(y, y + size_t(N) * MM);
    sv.K.assign(K, K + size_t(N - 1) * stages * MM);
    const double nrm = sv.residual();
    if (F_out) std::memcpy(F_out, sv.F.data(), sizeof(double) * sv.F.size());
    if (Fs_out) std::memcpy(Fs_out, sv.Fs.data(), sizeof(double) * sv.Fs.size());
    return nrm;
}

}  // extern "C"
