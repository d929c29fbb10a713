// Batched adaptive MIRK solve on sm_103a: device code.
//
// NVRTC compiles this file once per (problem source, M, method, Jacobian precision)
// after bvp_prelude.cuh and the user's problem source. Compile-time configuration:
//   BVP_M          state dimension                 BVP_ORDER    MIRK order (2..6)
//   BVP_TWOPOINT   1 for two-point BCs (bca, bcb)  BVP_NBC      BC evaluation points
//   BVP_JT         Jacobian / factorisation scalar (float by default)
//
// One warp owns one BVP instance for its whole adaptive solve; a persistent grid of
// warps pulls instances from an atomic work counter (coarsest initial meshes first). The warp's
// lanes split the mesh intervals for the per-interval work (residual, Jacobian blocks,
// defect) and the block pairs of each cyclic-reduction level.
//
// Precision: the residual that decides Newton convergence, the defect, the mesh selection
// and the solution transfer are FP64. The Jacobian blocks and the factorisation run in
// BVP_JT. With JT = float the first Newton iterations also use an FP32 residual (GB300's
// FP32 pipe is far wider than its FP64 pipe); convergence is always decided in FP64.
//
// Reference functions restated here (paths relative to the reference project):
//   Φ residual             lib/BoundaryValueDiffEqMIRK/src/collocation.jl:44-72
//   residual layout        lib/BoundaryValueDiffEqMIRK/src/mirk.jl:471-534
//   EvalSol BC access      lib/BoundaryValueDiffEqMIRK/src/interpolation.jl:214-242
//   extra stages           lib/BoundaryValueDiffEqMIRK/src/interpolation.jl:337-372
//   Jacobian blocks        lib/BoundaryValueDiffEqMIRK/src/mirk.jl:697-838 (exact block pattern)
//   Newton driver          lib/BoundaryValueDiffEqCore/src/default_internal_solve.jl:31-45
//   defect                 lib/BoundaryValueDiffEqMIRK/src/adaptivity.jl:416-461
//   mesh selection         lib/BoundaryValueDiffEqMIRK/src/adaptivity.jl:23-75, 250-304
//   solution transfer      lib/BoundaryValueDiffEqMIRK/src/adaptivity.jl:6-13 (mirk.jl:361-373)
//   outer loop             lib/BoundaryValueDiffEqMIRK/src/mirk.jl:286-388
#pragma once

#ifndef BVP_JT
#define BVP_JT float
#endif
#define BVP_JT_PTR BVP_JT
#include "bvp_shared.h"
#ifndef BVP_TWOPOINT
#define BVP_TWOPOINT 0
#endif
#ifndef BVP_NBC
#define BVP_NBC 2
#endif
#ifndef BVP_LA
#define BVP_LA 0
#endif
#include "bvp_tableau.cuh"

#if BVP_TWOPOINT
template <class T, class P> BVP_DEV void bvp_bc(T*, const T* const*, const P*) {}
#else
template <class T, class P> BVP_DEV void bvp_bca(T*, const T*, const P*) {}
template <class T, class P> BVP_DEV void bvp_bcb(T*, const T*, const P*) {}
#endif

namespace bvp {

constexpr unsigned FULL = 0xffffffffu;
constexpr int M = BVP_M;
constexpr int D = 2 * M;              // tangent directions of one interval
constexpr int NBC = BVP_NBC;
constexpr int TWOPOINT = BVP_TWOPOINT;
constexpr int NBCP = TWOPOINT ? 2 : NBC;  // BC evaluation points
constexpr int LA = BVP_LA;
using JT = BVP_JT;
constexpr bool F32_PHASE_OK = sizeof(JT) == 4;
constexpr int EQW = 2 * M * M + M;    // reduced equation: A (MxM), B (MxM), g (M)
constexpr int RECW = 3 * M * M + M;   // elimination record: U, X, Y (MxM), g (M)
constexpr int NBCB = TWOPOINT ? 2 : 2 * NBC;   // BC Jacobian blocks (node, MxM)
constexpr int KMAX = 2 + NBCB;                 // kept (separator) nodes
constexpr int NDENSE = KMAX * M;

enum : int { RET_SUCCESS = 0, RET_FAILURE = 1, RET_MAXITERS = 2 };

// error controllers (Core/src/calc_errors.jl:54-139); the paths other than DefectControl are
// compiled in only with BVP_GLOBAL_CTL, so the defect-controlled kernel stays as it is
#ifndef BVP_GLOBAL_CTL
#define BVP_GLOBAL_CTL 0
#endif
constexpr bool GLOBAL_CTL = BVP_GLOBAL_CTL != 0;
enum : int { CTL_DEFECT = 0, CTL_GLOBAL = 1, CTL_SEQUENTIAL = 2, CTL_HYBRID = 3 };
enum : int { GLOBAL_HO = 0, GLOBAL_RE = 1 };

// FIRK (expanded Radau IIA / Lobatto collocation, bvp_firk.cuh): the host prepends the scheme's
// coefficients (FS stages, order FORDER, c, b, a, q_coeff and τ*) and defines BVP_FIRK
#ifndef BVP_FIRK
#define BVP_FIRK 0
constexpr int FS = 1, FORDER = 1;
constexpr double FTAU = 0.0, FC[1] = {1.0}, FB[1] = {1.0}, FA[1][1] = {{1.0}}, FQ[1][1] = {{1.0}};
#endif
constexpr bool FIRK = BVP_FIRK != 0;
#ifndef BVP_POLISH_ONLY
#define BVP_POLISH_ONLY 0
#endif
#ifndef BVP_BLOCK_MODE
#define BVP_BLOCK_MODE 0
#endif
constexpr int GROUP_WARPS = 4;   // warps of a fused block (block mode: all of them on one instance)
// block mode: compiled into a module of its own (BVP_BLOCK_MODE), which the host loads for
// batches with long meshes, so that the warp-only kernels keep their code; defect control only
constexpr bool GROUP_OK = BVP_BLOCK_MODE && !GLOBAL_CTL && !FIRK && !BVP_POLISH_ONLY;
constexpr int FN = FS * M;          // stage unknowns of an interval
constexpr int FXW = FN * (M + 1);   // its condensation record: J_K^-1 [J_y | R]

// ---- launch arguments (shared with the host runtime) ------------------------------------
using InstState = BvpInstState;
using Args = BvpArgs;

// per-instance scratch layout (doubles), the same formulas as bvp_make_layout()
constexpr int SCR_BCRES = 0;                           // M        BC residual (FP64)
constexpr int SCR_BCBLK = SCR_BCRES + M;               // NBCB x M x M  BC Jacobian blocks
constexpr int SCR_SEG = SCR_BCBLK + NBCB * M * M;      // (KMAX-1) x EQW segment relations (JT)
constexpr int SCR_UA = SCR_SEG + (KMAX - 1) * EQW;     // NBCP x M  u at the BC points (FP64)
constexpr int SCR_BCW = SCR_UA + NBCP * M;             // NBCP x SS interpolant weights at the BC points
constexpr int SCRW = SCR_BCW + NBCP * SS;
// int scratch
constexpr int ISCR_NK = 0;                   // kept count
constexpr int ISCR_KEPT = 1;                 // KMAX kept nodes
constexpr int ISCR_NB = ISCR_KEPT + KMAX;    // number of BC blocks
constexpr int ISCR_BNODE = ISCR_NB + 1;      // NBCB block nodes
constexpr int ISCR_UNODE = ISCR_BNODE + NBCB;  // NBCP: node each BC point maps to
constexpr int ISCR_UIN = ISCR_UNODE + NBCP;    // NBCP: 1 if the point is interior
constexpr int ISCR_LOFF = ISCR_UIN + NBCP;     // KMAX+1: first lane of each segment
constexpr int ISCRW = ISCR_LOFF + KMAX + 1;
static_assert(KMAX - 1 <= 32, "one lane at least per separator segment");

// ---- warp helpers ------------------------------------------------------------------------
BVP_DEV int lane_id() { return threadIdx.x & 31; }
BVP_DEV double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
BVP_DEV double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}
BVP_DEV bool warp_any(bool b) { return __any_sync(FULL, b) != 0; }
// a / b for 1 <= b <= 1e30 (the defect's |f| + 1 scaling): an FP32 reciprocal and one FP64
// correction step, relative error ~1e-14 (the square of the reciprocal's), in a few FP64
// operations instead of a full division; other b divide exactly.
BVP_DEV double div_scaled(double a, double b) {
    if (!(b >= 1.0 && b <= 1e30)) return a / b;
    const double r = double(__frcp_rn(float(b)));
    const double q = a * r;
    return fma(fma(-b, q, a), r, q);
}
BVP_DEV double dinf() { return __longlong_as_double(0x7ff0000000000000LL); }

// lower_bound(mesh, t) - 1 clamped to [0, N-2]: the reference's interval()
// (lib/BoundaryValueDiffEqCore/src/utils.jl:119-121)
BVP_DEV int interval_of(const double* mesh, int N, double t) {
    int lo = 0, hi = N;  // first index with mesh[idx] >= t
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (mesh[mid] < t) lo = mid + 1; else hi = mid;
    }
    int ii = lo - 1;
    ii = ii < 0 ? 0 : ii;
    ii = ii > N - 2 ? N - 2 : ii;
    return ii;
}

// ---- per-instance view -----------------------------------------------------------------
struct GroupShared;
struct Inst {
    int q, cap, N, cur;
    long long nb;          // node offset
    const double* p;
    const JT* pj;
    double* scr;
    int* iscr;
    JT* dns;               // per-warp shared memory for the separator system
    JT* trec;              // per-warp shared memory for the shuffle tree's elimination records (or null)
    GroupShared* grp;      // block mode: the block's command area (null: the warp solves alone)
};

BVP_DEV double* mesh_of(const Args& a, const Inst& I, int b) { return a.mesh + b * a.tot + I.nb; }
BVP_DEV double* h_of(const Args& a, const Inst& I, int b) { return a.h + b * a.tot + I.nb; }
BVP_DEV double* y_of(const Args& a, const Inst& I, int b) { return a.y + (b * a.tot + I.nb) * M; }
BVP_DEV JT* yj_of(const Args& a, const Inst& I) { return a.yj + I.nb * M; }

// parameters and iterate in the residual's precision R (R = float only when JT = float)
template <class R> BVP_DEV const R* params_as(const Inst& I) {
    if constexpr (sizeof(R) == 8) return reinterpret_cast<const R*>(I.p);
    else return reinterpret_cast<const R*>(I.pj);
}
template <class R> BVP_DEV R y_at(const Args& a, const Inst& I, int k) {
    if constexpr (sizeof(R) == 8) return y_of(a, I, I.cur)[k];
    else return R(yj_of(a, I)[k]);
}

// Every evaluation of the problem's f goes through call_f. The evaluations of one scalar
// type can share one out-of-line copy (the user's f and its math library calls, e.g. sin
// with its large-argument path, are then in the kernel once instead of at every call site),
// which keeps the fused kernel's hot code, and its instruction-cache misses, smaller.
#ifndef BVP_F64_NOINLINE
#define BVP_F64_NOINLINE 1
#endif
#ifndef BVP_F32_NOINLINE
#define BVP_F32_NOINLINE 0
#endif
#ifndef BVP_DUAL_NOINLINE
#define BVP_DUAL_NOINLINE 0
#endif
#if BVP_F64_NOINLINE
__device__ __noinline__ void call_f64(double* du, const double* u, const double* p, double t) {
    bvp_f<double, double>(du, u, p, t);
}
#endif
#if BVP_F32_NOINLINE
__device__ __noinline__ void call_f32(float* du, const float* u, const float* p, float t) {
    bvp_f<float, float>(du, u, p, t);
}
#endif
#if BVP_DUAL_NOINLINE
__device__ __noinline__ void call_fdual(Dual<JT, D>* du, const Dual<JT, D>* u, const JT* p, JT t) {
    bvp_f<Dual<JT, D>, JT>(du, u, p, t);
}
#endif
template <class A, class B> struct same_t { static constexpr bool value = false; };
template <class A> struct same_t<A, A> { static constexpr bool value = true; };
template <class T, class PT> BVP_DEV void call_f(T* du, const T* u, const PT* p, PT t) {
#if BVP_F64_NOINLINE
    if constexpr (same_t<T, double>::value && same_t<PT, double>::value) { call_f64(du, u, p, t); return; }
#endif
#if BVP_F32_NOINLINE
    if constexpr (same_t<T, float>::value && same_t<PT, float>::value) { call_f32(du, u, p, t); return; }
#endif
#if BVP_DUAL_NOINLINE
    if constexpr (same_t<T, Dual<JT, D>>::value && same_t<PT, JT>::value) { call_fdual(du, u, p, t); return; }
#endif
    bvp_f<T, PT>(du, u, p, t);
}
#ifndef BVP_SINGULAR
#define BVP_SINGULAR 0
#endif
// A collocation stage: f plus the singular term S u / t for t > 0 (collocation.jl:60-66 with
// __add_singular_term!, Core/src/utils.jl:936-941). The interpolant's extra stages and the
// defect evaluate f alone, as the reference does (interpolation.jl:337-372,
// adaptivity.jl:416-461).
template <class T, class PT> BVP_DEV void call_stage_f(T* du, const T* u, const PT* p, PT t) {
    call_f<T, PT>(du, u, p, t);
#if BVP_SINGULAR
    if (t > PT(0)) {
        T su[M];
        bvp_sing<T, PT>(su, u, p);
        const PT it = PT(1) / t;
#pragma unroll
        for (int m = 0; m < M; ++m) du[m] = du[m] + su[m] * it;
    }
#endif
}

// MIRK4/5/6 put their first two stages on the mesh nodes (c = v = 0 and c = v = 1, no x
// terms): K_1 of interval i is f(y_i, t_i) and K_2 is f(y_{i+1}, t_{i+1}), which is K_1 of
// interval i+1. The residual evaluates each node once and shares it between neighbours
// (the reference evaluates it twice, collocation.jl:60-66).
constexpr bool NODE_SHARE = !FIRK && S >= 2 && ORD >= 4;

// ---- Φ for one interval (collocation.jl:44-72) ------------------------------------------
// With `node` non-null and NODE_SHARE, stage 0 is taken from node[] (f at the left node)
// and stage 1 is evaluated at the right node with t = t_{i+1} and written back to node[].
// With `dy` non-null the residual uses the FP64 difference y_{i+1} - y_i instead of the
// one formed from yi, yi1 (the FP32 residual keeps its roundoff near h|K| eps32).
template <class T, class PT, class TT>
BVP_DEV void phi_interval(const T* yi, const T* yi1, T* Ki, T* ri, const PT* p, TT ti, TT hi_d,
                          T* node = nullptr, TT ti1 = TT(0), const double* dy = nullptr) {
    const PT hi = PT(hi_d);
    T Y[M];
#pragma unroll
    for (int r = 0; r < S; ++r) {
        if (NODE_SHARE && r == 0 && node) {
#pragma unroll
            for (int m = 0; m < M; ++m) Ki[m] = node[m];
            continue;
        }
        if (NODE_SHARE && r == 1 && node) {
            call_stage_f<T, PT>(&Ki[M], yi1, p, PT(ti1));
#pragma unroll
            for (int m = 0; m < M; ++m) node[m] = Ki[M + m];
            continue;
        }
#pragma unroll
        for (int m = 0; m < M; ++m) Y[m] = PT(1.0 - tab_v(r)) * yi[m] + PT(tab_v(r)) * yi1[m];
#pragma unroll
        for (int j = 0; j < r; ++j) {
            if (tab_x(r, j) != 0.0) {
#pragma unroll
                for (int m = 0; m < M; ++m) Y[m] = Y[m] + hi * (Ki[j * M + m] * PT(tab_x(r, j)));
            }
        }
        call_stage_f<T, PT>(&Ki[r * M], Y, p, PT(ti + TT(tab_c(r)) * hi_d));
    }
#pragma unroll
    for (int m = 0; m < M; ++m) {
        T acc = Ki[m] * PT(tab_b(0));
#pragma unroll
        for (int r = 1; r < S; ++r) acc = acc + Ki[r * M + m] * PT(tab_b(r));
        if (dy) ri[m] = T(PT(dy[m])) - hi * acc;
        else ri[m] = (yi1[m] - yi[m]) - hi * acc;
    }
}

// extra interpolant stages of one interval (interpolation.jl:337-372)
template <class T, class PT>
BVP_DEV void interp_stages(const T* yi, const T* yi1, const T* Ki, T* KIi, const PT* p, double ti, double hi_d) {
    const PT hi = PT(hi_d);
    T Y[M];
#pragma unroll
    for (int r = 0; r < NSX; ++r) {
#pragma unroll
        for (int m = 0; m < M; ++m) {
            T acc = Ki[m] * PT(tab_xs(r, 0));
#pragma unroll
            for (int j = 1; j < S; ++j) acc = acc + Ki[j * M + m] * PT(tab_xs(r, j));
#pragma unroll
            for (int qq = 0; qq < r; ++qq) acc = acc + KIi[qq * M + m] * PT(tab_xs(r, S + qq));
            Y[m] = acc * hi + PT(1.0 - tab_vs(r)) * yi[m] + PT(tab_vs(r)) * yi1[m];
        }
        call_f<T, PT>(&KIi[r * M], Y, p, PT(ti + tab_cs(r) * hi_d));
    }
}

// z = y_i + h (Σ w_r K_r + Σ w_{s+q} KI_q)
template <class T, class W>
BVP_DEV void sum_stages(const W* w, const T* yi, const T* Ki, const T* KIi, W hi, T* z) {
#pragma unroll
    for (int m = 0; m < M; ++m) {
        T acc = Ki[m] * w[0];
#pragma unroll
        for (int r = 1; r < S; ++r) acc = acc + Ki[r * M + m] * w[r];
#pragma unroll
        for (int qq = 0; qq < NSX; ++qq) acc = acc + KIi[qq * M + m] * w[S + qq];
        z[m] = acc * hi + yi[m];
    }
}

// Per-mesh setup (lane 0), redone whenever the mesh changes:
//  * each BC evaluation time t_k is located as the reference's EvalSol does
//    (interpolation.jl:214-242): the exact endpoints give y_1 / y_N, any other t the
//    interval ii = interval(mesh, t) with the interpolant weights at τ = (t - t_ii)/h_ii;
//    the node the BC Jacobian row is attributed to is the endpoint or ii (the reference
//    differentiates the BCs with the interpolant's stages held fixed, mirk.jl:565-572);
//  * the separator nodes of the partition solve: 0, N-1 and every node a BC row touches;
//  * the lanes per separator segment: a power of two no larger than the segment,
//    proportional to its share of the mesh, at least one, 32 in all.
// interpolant weights at a run-time τ: one out-of-line copy for the mesh setup, the
// transfer and dense output (the defect's constant τ* fold at compile time)
__device__ __noinline__ void interp_weights_rt(double t, double* w, double* wp) { interp_weights<double>(t, w, wp); }

// the lane-0 part of mesh_setup, out of line: it runs once per mesh round and its straight
// code is better kept out of the hot loop's instruction stream
__device__ __noinline__ void mesh_setup_lane0(const double* mesh, const double* h, int N, const double* bc_t,
                                              int bc_jac_exact, double* scr, int* iscr) {
    int kept[KMAX];
    int nk = 0;
    kept[nk++] = 0;
    kept[nk++] = N - 1;
    if (TWOPOINT) {
        iscr[ISCR_UNODE] = 0; iscr[ISCR_UNODE + 1] = N - 1;
        iscr[ISCR_UIN] = 0; iscr[ISCR_UIN + 1] = 0;
    } else {
        for (int k = 0; k < NBC; ++k) {
            const double t = bc_t[k];
            int node, in = 0;
            if (t == mesh[0]) node = 0;
            else if (t == mesh[N - 1]) node = N - 1;
            else {
                node = interval_of(mesh, N, t);
                in = 1;
                double w[SS], wp[SS];
                interp_weights_rt((t - mesh[node]) / h[node], w, wp);
                for (int s2 = 0; s2 < SS; ++s2) scr[SCR_BCW + k * SS + s2] = w[s2];
            }
            iscr[ISCR_UNODE + k] = node;
            iscr[ISCR_UIN + k] = in;
            kept[nk++] = node;
            if (in && bc_jac_exact) kept[nk++] = node + 1;
        }
    }
    for (int u = 1; u < nk; ++u) {
        const int v = kept[u];
        int w2 = u - 1;
        while (w2 >= 0 && kept[w2] > v) { kept[w2 + 1] = kept[w2]; --w2; }
        kept[w2 + 1] = v;
    }
    int nu = 0;
    for (int u = 0; u < nk; ++u)
        if (nu == 0 || kept[u] != kept[nu - 1]) kept[nu++] = kept[u];
    iscr[ISCR_NK] = nu;
    for (int u = 0; u < nu; ++u) iscr[ISCR_KEPT + u] = kept[u];
    const int ns = nu - 1, m = N - 1;
    int o = 0;
    for (int j = 0; j < ns; ++j) {
        const int len = kept[j + 1] - kept[j];
        int want = 1 + ((32 - ns) * len) / m;
        want = want < len ? want : len;
        int L = 1;
        while (2 * L <= want) L *= 2;
        iscr[ISCR_LOFF + j] = o;
        o += L;
    }
    iscr[ISCR_LOFF + ns] = o;
}

BVP_DEV void mesh_setup(const Args& a, const Inst& I) {
    if (lane_id() == 0) {
        double bt[NBC];
#pragma unroll
        for (int k = 0; k < NBC; ++k) bt[k] = a.bc_t[k];
        mesh_setup_lane0(mesh_of(a, I, I.cur), h_of(a, I, I.cur), I.N, bt, a.bc_jac_exact, I.scr, I.iscr);
    }
    {
        // the mesh in the Jacobian precision (FP32 stage times without FP64 conversions)
        const double* mesh = mesh_of(a, I, I.cur);
        const double* h = h_of(a, I, I.cur);
        JT* tj = a.tj + I.nb;
        JT* hj = a.hj + I.nb;
        for (int i = lane_id(); i < I.N; i += 32) {
            tj[i] = JT(mesh[i]);
            if (i < I.N - 1) hj[i] = JT(h[i]);
        }
    }
    __syncwarp();
}

// ---- K1: residual and stages (warp). Returns ||F||_inf (+inf if non-finite). -----------
// R is the precision of the stage evaluations and the residual assembly: double for the
// Newton residual that decides convergence (writes K and F in FP64), float for the early
// Newton iterations of the mixed-precision path (writes only the FP32 right-hand side).
// Each lane owns a contiguous block of intervals so node stages pass between neighbours
// in registers. Lane 0 then evaluates the BCs and caches u at the BC points.
// The BC rows on lane 0: u at the BC points (interior ones as the interval loop cached them,
// endpoints from the nodes) cached for the Jacobian, the BC residual into the scratch; returns
// its largest magnitude and flags a non-finite entry in bad.
template <class R>
BVP_DEV double bc_rows_lane0(const Args& a, const Inst& I, const R* pr, bool& bad) {
    double mx = 0.0;
    R res[M];
#pragma unroll
    for (int m = 0; m < M; ++m) res[m] = R(0);
    double* ua_c = I.scr + SCR_UA;
    if (TWOPOINT) {
        R ya[M], yb[M], ra[M], rb[M];
#pragma unroll
        for (int m = 0; m < M; ++m) { ya[m] = y_at<R>(a, I, m); yb[m] = y_at<R>(a, I, (I.N - 1) * M + m); }
        bvp_bca<R, R>(ra, ya, pr);
        bvp_bcb<R, R>(rb, yb, pr);
        for (int k = 0; k < LA; ++k) res[k] = ra[k];
        for (int k = LA; k < M; ++k) res[k] = rb[k - LA];
        for (int m = 0; m < M; ++m) { ua_c[m] = double(ya[m]); ua_c[M + m] = double(yb[m]); }
    } else {
        R ua[NBC * M];
        const R* ptrs[NBC];
#pragma unroll
        for (int k = 0; k < NBC; ++k) {
            if (I.iscr[ISCR_UIN + k]) {
#pragma unroll
                for (int m = 0; m < M; ++m) ua[k * M + m] = R(ua_c[k * M + m]);
            } else {
                // exact endpoints: EvalSol returns y_1 / y_N
                const int nd = I.iscr[ISCR_UNODE + k];
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    ua[k * M + m] = y_at<R>(a, I, nd * M + m);
                    ua_c[k * M + m] = double(ua[k * M + m]);
                }
            }
            ptrs[k] = &ua[k * M];
        }
        bvp_bc<R, R>(res, ptrs, pr);
    }
#pragma unroll
    for (int m = 0; m < M; ++m) {
        I.scr[SCR_BCRES + m] = double(res[m]);
        bad |= !isfinite(res[m]);
        mx = fmax(mx, fabs(double(res[m])));
    }
    return mx;
}

// The intervals of group lane gl of GL (a warp's lanes, or a block's in block mode): its
// largest |F| entry; a non-finite entry sets bad.
template <class R, int GL>
BVP_DEV double residual_part(const Args& a, const Inst& I, int gl, bool& bad) {
    const double* mesh = mesh_of(a, I, I.cur);
    const double* h = h_of(a, I, I.cur);
    const R* pr = params_as<R>(I);
    R mxr = R(0);
    const int nI = I.N - 1;
    const int per = (nI + GL - 1) / GL;
    const int i0 = gl * per;
    const int i1 = min(i0 + per, nI);
    R node[M];
    if (NODE_SHARE && i0 < i1) {
        R y0v[M];
#pragma unroll
        for (int m = 0; m < M; ++m) y0v[m] = y_at<R>(a, I, i0 * M + m);
        call_stage_f<R, R>(node, y0v, pr, sizeof(R) == 8 ? R(mesh[i0]) : R(a.tj[I.nb + i0]));
    }
    const double* y64 = y_of(a, I, I.cur);
    // interior BC points: the lane whose block holds the interval evaluates the
    // interpolant there from its registers (the stages it just computed)
    int bc_iv[NBCP];
#pragma unroll
    for (int k = 0; k < NBCP; ++k) bc_iv[k] = (!TWOPOINT && I.iscr[ISCR_UIN + k]) ? I.iscr[ISCR_UNODE + k] : -1;
    for (int i = i0; i < i1; ++i) {
        R yi[M], yi1[M], Ki[S * M], ri[M];
#pragma unroll
        for (int m = 0; m < M; ++m) { yi[m] = y_at<R>(a, I, i * M + m); yi1[m] = y_at<R>(a, I, (i + 1) * M + m); }
        if constexpr (sizeof(R) == 8) {
            phi_interval<R, R, double>(yi, yi1, Ki, ri, pr, mesh[i], h[i], NODE_SHARE ? node : nullptr, mesh[i + 1]);
        } else {
            double dy[M];
#pragma unroll
            for (int m = 0; m < M; ++m) dy[m] = y64[(i + 1) * M + m] - y64[i * M + m];
            const JT* tj = a.tj + I.nb;
            const JT* hj = a.hj + I.nb;
            phi_interval<R, R, R>(yi, yi1, Ki, ri, pr, R(tj[i]), R(hj[i]), NODE_SHARE ? node : nullptr, R(tj[i + 1]),
                                  dy);
        }
#pragma unroll 1
        for (int k = 0; k < NBCP; ++k) {
            if (bc_iv[k] == i) {
                R KIi[NSXA * M], w[SS], z[M];
                interp_stages<R, R>(yi, yi1, Ki, KIi, pr, mesh[i], h[i]);
#pragma unroll
                for (int s = 0; s < SS; ++s) w[s] = R(I.scr[SCR_BCW + k * SS + s]);
                sum_stages<R, R>(w, yi, Ki, KIi, R(h[i]), z);
#pragma unroll
                for (int m = 0; m < M; ++m) I.scr[SCR_UA + k * M + m] = double(z[m]);
            }
        }
        JT* Fj = a.Fj + (I.nb + i) * M;
        if constexpr (sizeof(R) == 8) {
            double* Kg = a.K + (I.nb + i) * (S * M);
#pragma unroll
            for (int k = 0; k < S * M; ++k) Kg[k] = Ki[k];
            double* Fg = a.F + (I.nb + i) * M;
#pragma unroll
            for (int m = 0; m < M; ++m) Fg[m] = ri[m];
        }
#pragma unroll
        for (int m = 0; m < M; ++m) {
            Fj[m] = JT(ri[m]);
            bad |= !isfinite(ri[m]);
            mxr = fmax(mxr, fabs(ri[m]));
        }
    }
    return double(mxr);
}

BVP_DEV double group_phase(const Args& a, const Inst& I, int cmd, bool& bad);
constexpr int CMD_EXIT = 0, CMD_RES32 = 1, CMD_RES64 = 2, CMD_DEFECT = 3;

template <class R = double>
BVP_DEV double residual(const Args& a, const Inst& I) {
    const int lane = lane_id();
    bool bad = false;
    double mx;
    if (GROUP_OK && I.grp) mx = group_phase(a, I, sizeof(R) == 8 ? CMD_RES64 : CMD_RES32, bad);
    else mx = residual_part<R, 32>(a, I, lane, bad);
    __syncwarp();
    if (lane == 0) mx = fmax(mx, bc_rows_lane0<R>(a, I, params_as<R>(I), bad));
    __syncwarp();
    mx = warp_max(mx);
    bad = warp_any(bad);
    return bad ? dinf() : mx;
}

// Σ F² over the full FP64 residual (for the line search)
BVP_DEV double residual_sq(const Args& a, const Inst& I) {
    const int lane = lane_id();
    double s = 0.0;
    for (int i = lane; i < I.N - 1; i += 32) {
        const double* Fg = a.F + (I.nb + i) * M;
#pragma unroll
        for (int m = 0; m < M; ++m) s += Fg[m] * Fg[m];
    }
    if (lane == 0) {
#pragma unroll
        for (int m = 0; m < M; ++m) s += I.scr[SCR_BCRES + m] * I.scr[SCR_BCRES + m];
    }
    return warp_sum(s);
}

// ---- K2: Jacobian blocks (warp) ------------------------------------------------------------
// S_i = ∂r_i/∂y_i and R_i = ∂r_i/∂y_{i+1} by forward mode with 2M tangents in JT, from the
// JT copy of the iterate. BC rows use u at the BC points cached by the last residual.
// BC Jacobian blocks: one (node, L x M) block per slot of the scratch; lane k evaluates the
// BCs' derivative with respect to u at BC point k (two-point: lane 0 bca, lane 1 bcb). With
// the exact BC Jacobian an interior point gives two blocks (its interval's nodes), so each
// point owns two slots, the second one zero for an endpoint. The separator solve adds the
// blocks that share a node.
BVP_DEV void write_bc_block(const Inst& I, int slot, int node, const double* G) {
    I.iscr[ISCR_BNODE + slot] = node;
    double* dst = I.scr + SCR_BCBLK + slot * M * M;
#pragma unroll
    for (int q = 0; q < M * M; ++q) dst[q] = G[q];
}

// the collocation blocks of every interval into Sb / Rb (the Newton solve computes them inside
// its block elimination instead; this pass serves the per-kernel tests)
BVP_DEV void jacobian_blocks(const Args& a, const Inst& I) {
    using DI = Dual<JT, D>;
    const int lane = lane_id();
    const JT* yj = yj_of(a, I);
    const JT* tj = a.tj + I.nb;
    const JT* hj = a.hj + I.nb;
    for (int i = lane; i < I.N - 1; i += 32) {
        DI yi[M], yi1[M], Ki[S * M], ri[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            yi[m] = DI(yj[i * M + m]); yi[m].d[m] = JT(1);
            yi1[m] = DI(yj[(i + 1) * M + m]); yi1[m].d[M + m] = JT(1);
        }
        phi_interval<DI, JT, JT>(yi, yi1, Ki, ri, I.pj, tj[i], hj[i]);
        JT* Sg = a.Sb + (I.nb + i) * (M * M);
        JT* Rg = a.Rb + (I.nb + i) * (M * M);
#pragma unroll
        for (int r = 0; r < M; ++r)
#pragma unroll
            for (int c = 0; c < M; ++c) {
                Sg[r * M + c] = ri[r].d[c];
                Rg[r * M + c] = ri[r].d[M + c];
            }
    }
    __syncwarp();
}

// the BC rows' Jacobian blocks (scratch), from u at the BC points cached by the last residual
BVP_DEV void bc_jacobian(const Args& a, const Inst& I) {
    using DI = Dual<JT, D>;
    const int lane = lane_id();
    const double* mesh = mesh_of(a, I, I.cur);
    const double* h = h_of(a, I, I.cur);
    const JT* yj = yj_of(a, I);
    using DU = Dual<JT, M>;
    const double* ua_c = I.scr + SCR_UA;
    double G[M * M];
    if (TWOPOINT) {
        if (lane < 2) {
            DU ua[M], ra[M];
#pragma unroll
            for (int m = 0; m < M; ++m) { ua[m] = DU(JT(ua_c[lane * M + m])); ua[m].d[m] = JT(1); }
#pragma unroll
            for (int q = 0; q < M * M; ++q) G[q] = 0.0;
            if (lane == 0) {
                bvp_bca<DU, JT>(ra, ua, I.pj);
                for (int r = 0; r < LA; ++r) for (int c = 0; c < M; ++c) G[r * M + c] = double(ra[r].d[c]);
            } else {
                bvp_bcb<DU, JT>(ra, ua, I.pj);
                for (int r = LA; r < M; ++r) for (int c = 0; c < M; ++c) G[r * M + c] = double(ra[r - LA].d[c]);
            }
            write_bc_block(I, lane, lane == 0 ? 0 : I.N - 1, G);
        }
        if (lane == 0) I.iscr[ISCR_NB] = 2;
    } else {
        const int k = lane;
        if (k < NBC) {
            DU ua[NBC * M];
            const DU* ptrs[NBC];
#pragma unroll
            for (int qq = 0; qq < NBC; ++qq) {
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    ua[qq * M + m] = DU(JT(ua_c[qq * M + m]));
                    if (qq == k) ua[qq * M + m].d[m] = JT(1);
                }
                ptrs[qq] = &ua[qq * M];
            }
            DU res[M];
            bvp_bc<DU, JT>(res, ptrs, I.pj);
#pragma unroll
            for (int r = 0; r < M; ++r)
#pragma unroll
                for (int c = 0; c < M; ++c) G[r * M + c] = double(res[r].d[c]);
            const int node = I.iscr[ISCR_UNODE + k];
            const int slot = a.bc_jac_exact ? 2 * k : k;
            if (!I.iscr[ISCR_UIN + k] || !a.bc_jac_exact) {
                // the interpolant's stages are held at their primal values: du(t)/dy = I
                // on the interval's left node (interpolation.jl:214-242, mirk.jl:565-572)
                write_bc_block(I, slot, node, G);
                if (a.bc_jac_exact) {
                    double Z[M * M];
#pragma unroll
                    for (int q = 0; q < M * M; ++q) Z[q] = 0.0;
                    write_bc_block(I, slot + 1, node, Z);
                }
            } else {
                // exact: chain through the interval's stages and extra stages
                const int ii = node;
                JT w[SS];
#pragma unroll
                for (int s2 = 0; s2 < SS; ++s2) w[s2] = JT(I.scr[SCR_BCW + k * SS + s2]);
                DI yi[M], yi1[M], Ki[S * M], KIi[NSXA * M], ri[M], z[M];
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    yi[m] = DI(yj[ii * M + m]); yi[m].d[m] = JT(1);
                    yi1[m] = DI(yj[(ii + 1) * M + m]); yi1[m].d[M + m] = JT(1);
                }
                phi_interval<DI, JT, double>(yi, yi1, Ki, ri, I.pj, mesh[ii], h[ii]);
                interp_stages<DI, JT>(yi, yi1, Ki, KIi, I.pj, mesh[ii], h[ii]);
                sum_stages<DI, JT>(w, yi, Ki, KIi, JT(h[ii]), z);
                double JL[M * M], JR[M * M];
                for (int r = 0; r < M; ++r)
                    for (int c = 0; c < M; ++c) {
                        double sl = 0.0, sr = 0.0;
                        for (int qq = 0; qq < M; ++qq) {
                            sl += G[r * M + qq] * double(z[qq].d[c]);
                            sr += G[r * M + qq] * double(z[qq].d[M + c]);
                        }
                        JL[r * M + c] = sl; JR[r * M + c] = sr;
                    }
                write_bc_block(I, slot, ii, JL);
                write_bc_block(I, slot + 1, ii + 1, JR);
            }
        }
        if (lane == 0) I.iscr[ISCR_NB] = a.bc_jac_exact ? 2 * NBC : NBC;
    }
    __syncwarp();
}

BVP_DEV void jacobian(const Args& a, const Inst& I) {
    jacobian_blocks(a, I);
    bc_jacobian(a, I);
}

// ---- K3: structured factorisation + solve (warp) -----------------------------------------
// Partition method over the almost-block-diagonal system. The separator nodes (0, N-1 and
// every node a BC row touches) split the collocation chain into segments; each segment gets
// a power-of-two group of lanes and each lane a contiguous block of its intervals.
//   1. every lane eliminates its block's interior nodes in turn (registers), leaving one
//      relation A δ_a + B δ_b = g between its block ends;
//   2. a shuffle tree inside each lane group eliminates the block-end nodes pairwise until
//      the group's root holds the segment relation;
//   3. the segment relations and the BC rows form a small dense system in the separator
//      values, solved on one lane;
//   4. the tree is unwound (block-end values), then each lane back-substitutes its block.
// Every elimination is Gaussian elimination with row pivoting on the shared node's 2M x M
// column block (the reference factors the same matrix with an almost-banded QR/LU,
// mirk.jl:721-777).
BVP_DEV void load_eq0(const Args& a, const Inst& I, int i, JT* A, JT* B, JT* g) {
    const JT* Sg = a.Sb + (I.nb + i) * (M * M);
    const JT* Rg = a.Rb + (I.nb + i) * (M * M);
    const JT* Fg = a.Fj + (I.nb + i) * M;
#pragma unroll
    for (int q = 0; q < M * M; ++q) { A[q] = Sg[q]; B[q] = Rg[q]; }
#pragma unroll
    for (int m = 0; m < M; ++m) g[m] = -Fg[m];
}
BVP_DEV void load_eq(const JT* src, JT* A, JT* B, JT* g) {
#pragma unroll
    for (int q = 0; q < M * M; ++q) { A[q] = src[q]; B[q] = src[M * M + q]; }
#pragma unroll
    for (int m = 0; m < M; ++m) g[m] = src[2 * M * M + m];
}
BVP_DEV void store_eq(JT* dst, const JT* A, const JT* B, const JT* g) {
#pragma unroll
    for (int q = 0; q < M * M; ++q) { dst[q] = A[q]; dst[M * M + q] = B[q]; }
#pragma unroll
    for (int m = 0; m < M; ++m) dst[2 * M * M + m] = g[m];
}

// left: Al δ_lo + Bl δ_mid = gl;  right: Ar δ_mid + Br δ_hi = gr.
// Eliminates δ_mid; writes the pivot rows (U δ_mid + X δ_lo + Y δ_hi = gu) to rec and
// the reduced equation (An δ_lo + Bn δ_hi = gn). Returns false on a zero pivot.
BVP_DEV bool eliminate_pair(const JT* Al, const JT* Bl, const JT* gl, const JT* Ar, const JT* Br,
                            const JT* gr, JT* rec, JT* An, JT* Bn, JT* gn) {
    constexpr int W = 3 * M + 1;
    JT Wm[2 * M][W];
#pragma unroll
    for (int r = 0; r < M; ++r) {
#pragma unroll
        for (int c = 0; c < M; ++c) {
            Wm[r][c] = Bl[r * M + c];     Wm[r][M + c] = Al[r * M + c];     Wm[r][2 * M + c] = JT(0);
            Wm[M + r][c] = Ar[r * M + c]; Wm[M + r][M + c] = JT(0);         Wm[M + r][2 * M + c] = Br[r * M + c];
        }
        Wm[r][3 * M] = gl[r];
        Wm[M + r][3 * M] = gr[r];
    }
    bool ok = true;
#pragma unroll
    for (int k = 0; k < M; ++k) {
        int piv = k;
        JT best = fabs(Wm[k][k]);
#pragma unroll
        for (int r = k + 1; r < 2 * M; ++r) {
            const JT v = fabs(Wm[r][k]);
            if (v > best) { best = v; piv = r; }
        }
        ok = ok && (best > JT(0)) && isfinite(best);
#pragma unroll
        for (int r = k + 1; r < 2 * M; ++r) {
            if (r == piv) {
#pragma unroll
                for (int c = 0; c < W; ++c) { const JT t = Wm[k][c]; Wm[k][c] = Wm[r][c]; Wm[r][c] = t; }
            }
        }
        const JT inv = JT(1) / Wm[k][k];
#pragma unroll
        for (int r = k + 1; r < 2 * M; ++r) {
            const JT mlt = Wm[r][k] * inv;
#pragma unroll
            for (int c = k; c < W; ++c) Wm[r][c] -= mlt * Wm[k][c];
        }
    }
#pragma unroll
    for (int r = 0; r < M; ++r) {
#pragma unroll
        for (int c = 0; c < M; ++c) {
            rec[r * M + c] = Wm[r][c];
            rec[M * M + r * M + c] = Wm[r][M + c];
            rec[2 * M * M + r * M + c] = Wm[r][2 * M + c];
            An[r * M + c] = Wm[M + r][M + c];
            Bn[r * M + c] = Wm[M + r][2 * M + c];
        }
        rec[3 * M * M + r] = Wm[r][3 * M];
        gn[r] = Wm[M + r][3 * M];
    }
    return ok;
}

BVP_DEV JT* seg_of(const Inst& I, int j) { return reinterpret_cast<JT*>(I.scr + SCR_SEG) + j * EQW; }

// δ_x from an elimination record: U δ_x = g - X δ_lo - Y δ_hi (U upper triangular)
BVP_DEV void back_solve(const JT* rg, const JT* dlo, const JT* dhi, JT* dx) {
    JT t[M];
#pragma unroll
    for (int r = 0; r < M; ++r) {
        JT s = rg[3 * M * M + r];
#pragma unroll
        for (int c = 0; c < M; ++c) s -= rg[M * M + r * M + c] * dlo[c] + rg[2 * M * M + r * M + c] * dhi[c];
        t[r] = s;
    }
#pragma unroll
    for (int r = M - 1; r >= 0; --r) {
        JT s = t[r];
#pragma unroll
        for (int c = r + 1; c < M; ++c) s -= rg[r * M + c] * t[c];
        t[r] = s / rg[r * M + r];
    }
#pragma unroll
    for (int r = 0; r < M; ++r) dx[r] = t[r];
}

// dense Gaussian elimination with partial pivoting, one lane
template <class R>
BVP_DEV bool dense_solve(int n, R* A, R* b) {
    for (int k = 0; k < n; ++k) {
        int piv = k;
        R best = fabs(A[k * n + k]);
        for (int r = k + 1; r < n; ++r) {
            const R v = fabs(A[r * n + k]);
            if (v > best) { best = v; piv = r; }
        }
        if (!(best > R(0)) || !isfinite(best)) return false;
        if (piv != k) {
            for (int c = 0; c < n; ++c) { const R t = A[k * n + c]; A[k * n + c] = A[piv * n + c]; A[piv * n + c] = t; }
            const R t = b[k]; b[k] = b[piv]; b[piv] = t;
        }
        const R inv = R(1) / A[k * n + k];
        for (int r = k + 1; r < n; ++r) {
            const R mlt = A[r * n + k] * inv;
            if (mlt == R(0)) continue;
            for (int c = k + 1; c < n; ++c) A[r * n + c] -= mlt * A[k * n + c];
            b[r] -= mlt * b[k];
        }
    }
    for (int k = n - 1; k >= 0; --k) {
        R s = b[k];
        for (int c = k + 1; c < n; ++c) s -= A[k * n + c] * b[c];
        b[k] = s / A[k * n + k];
    }
    return true;
}

// The separator system on the whole warp, in shared memory (n = nk M <= NDENSE <= 32 rows
// of DLD entries, the right-hand side in column n): lane r assembles and updates row r.
// Gaussian elimination with partial pivoting (the pivot row, largest |a_rk| and the first
// on ties as dense_solve picks it, found by a warp reduction; the exchange done across the
// columns), then back substitution by columns. Loops rather than unrolled code: the solve
// runs once per Newton step and stays small in the instruction cache. Writes δ at the
// separator nodes.
constexpr bool SMEM_DENSE = NDENSE <= 32;
constexpr int DLD = NDENSE + 1 + ((NDENSE + 1) % 2 == 0 ? 1 : 0);   // odd row stride
BVP_DEV bool separator_solve_warp(const Args& a, const Inst& I, int nk) {
    const int lane = lane_id();
    const int n = nk * M;
    const int row0 = (nk - 1) * M;
    JT* A = I.dns;
    if (lane < n) {
        JT* ar = A + lane * DLD;
#pragma unroll 1
        for (int c = 0; c <= n; ++c) ar[c] = JT(0);
        if (lane < row0) {
            // segment relation j: A δ_{kept j} + B δ_{kept j+1} = g
            const int j = lane / M, r = lane - j * M;
            const JT* seg = seg_of(I, j);
            for (int c = 0; c < M; ++c) {
                ar[j * M + c] = seg[r * M + c];
                ar[(j + 1) * M + c] = seg[M * M + r * M + c];
            }
            ar[n] = seg[2 * M * M + r];
        } else {
            // BC row r: every BC contribution's block, added at its separator's columns
            const int r = lane - row0;
            const int nb = I.iscr[ISCR_NB];
#pragma unroll 1
            for (int k = 0; k < nb; ++k) {
                const int node = I.iscr[ISCR_BNODE + k];
                int kj = 0;
                while (kj < nk - 1 && I.iscr[ISCR_KEPT + kj] != node) ++kj;
                const double* G = I.scr + SCR_BCBLK + k * M * M + r * M;
                for (int c = 0; c < M; ++c) ar[kj * M + c] += JT(G[c]);
            }
            ar[n] = JT(-I.scr[SCR_BCRES + r]);
        }
    }
    __syncwarp();
#pragma unroll 1
    for (int k = 0; k < n; ++k) {
        const bool cand = lane >= k && lane < n;
        JT v;
        int pr;
        if constexpr (sizeof(JT) == 4) {
            // largest |a| by one warp reduction on the bit patterns (non-negative floats order as
            // their bits), the lowest such row by a ballot
            const unsigned key = cand ? __float_as_uint(fabsf(float(A[lane * DLD + k]))) : 0u;
            const unsigned mk = __reduce_max_sync(FULL, key);
            pr = __ffs(__ballot_sync(FULL, cand && key == mk)) - 1;
            v = JT(__uint_as_float(mk));
        } else {
            v = cand ? fabs(A[lane * DLD + k]) : JT(-1);
            pr = lane;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const JT v2 = __shfl_xor_sync(FULL, v, o);
                const int p2 = __shfl_xor_sync(FULL, pr, o);
                if (v2 > v || (v2 == v && p2 < pr)) { v = v2; pr = p2; }
            }
        }
        if (!(v > JT(0)) || !isfinite(v)) return false;   // uniform across the warp
        if (pr != k) {
#pragma unroll 1
            for (int c = lane; c <= n; c += 32) {
                const JT t = A[k * DLD + c];
                A[k * DLD + c] = A[pr * DLD + c];
                A[pr * DLD + c] = t;
            }
            __syncwarp();
        }
        if (lane > k && lane < n) {
            JT* ar = A + lane * DLD;
            const JT* ak = A + k * DLD;
            const JT mlt = ar[k] * (JT(1) / ak[k]);
            // four columns' loads in flight at a time
#pragma unroll 4
            for (int c = k + 1; c <= n; ++c) ar[c] -= mlt * ak[c];
        }
        __syncwarp();
    }
#pragma unroll 1
    for (int k = n - 1; k >= 0; --k) {
        if (lane == k) A[k * DLD + n] = A[k * DLD + n] / A[k * DLD + k];
        __syncwarp();
        if (lane < k) A[lane * DLD + n] -= A[lane * DLD + k] * A[k * DLD + n];
        __syncwarp();
    }
    if (lane < n) a.delta[(I.nb + I.iscr[ISCR_KEPT + lane / M]) * M + lane % M] = A[lane * DLD + n];
    __syncwarp();
    return true;
}

#ifndef BVP_TREE_UNROLL
#define BVP_TREE_UNROLL 1
#endif
constexpr int TREE_UNROLL = BVP_TREE_UNROLL;  // shuffle-tree levels unrolled (1: one copy of each step)
// The shuffle tree's elimination records stay in shared memory when they fit: at level s the
// combining lanes of a group are 2^(s+1) apart, so lane >> (s+1) numbers them without
// collisions across groups, and the five levels need 16 + 8 + 4 + 2 + 1 = 31 slots. The lane
// that writes a record at level s is the one that reads it back in the unwind.
constexpr int TREE_SLOTS = 31;
BVP_DEV int tree_slot(int s, int lane) { return (32 - (32 >> s)) + (lane >> (s + 1)); }

// S_c = ∂r_c/∂y_c and R_c = ∂r_c/∂y_{c+1} of interval c by forward mode (2M tangents), the same
// blocks jacobian_blocks writes. With NODE_SHARE, node holds f at y_c with its tangents in the
// y_c slots on entry, and f at y_{c+1} with its tangents moved to the y_{c+1}-as-left-node
// slots on return (the next interval's first stage).
BVP_DEV void block_jacobian(const JT* yj, const JT* tj, const JT* hj, const JT* pj, int c, Dual<JT, D>* node,
                            JT* Sr, JT* Rr) {
    using DI = Dual<JT, D>;
    DI yi[M], yi1[M], Ki[S * M], ri[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
        yi[m] = DI(yj[c * M + m]); yi[m].d[m] = JT(1);
        yi1[m] = DI(yj[(c + 1) * M + m]); yi1[m].d[M + m] = JT(1);
    }
    phi_interval<DI, JT, JT>(yi, yi1, Ki, ri, pj, tj[c], hj[c], NODE_SHARE ? node : nullptr, tj[c + 1]);
    if (NODE_SHARE) {
#pragma unroll
        for (int m = 0; m < M; ++m)
#pragma unroll
            for (int k = 0; k < M; ++k) { node[m].d[k] = node[m].d[M + k]; node[m].d[M + k] = JT(0); }
    }
#pragma unroll
    for (int r = 0; r < M; ++r)
#pragma unroll
        for (int cc = 0; cc < M; ++cc) {
            Sr[r * M + cc] = ri[r].d[cc];
            Rr[r * M + cc] = ri[r].d[M + cc];
        }
}

#if BVP_FIRK
// FIRK interval c, linearised at the current nodes and stages: the stage equations
// R_r = f(Y_r, t_r) - K_r with Y_r = y_c + h sum_j a_rj K_j have J_K = h a_rj J_f(Y_r) - δ_rj I
// and J_y = J_f(Y_r); X = J_K^-1 [J_y | R] (an FN x FN elimination with partial pivoting, kept
// in a.fx for the stage update) eliminates the stage unknowns from the continuity row
// C = y_{c+1} - y_c - h sum_j b_j K_j, leaving the node relation of the structured solve:
// S = h sum_j b_j X_y,j - I, R = I, right-hand side -(C + h sum_j b_j X_r,j).
BVP_DEV bool firk_block(const Args& a, const Inst& I, int c, double* Sr, double* Rr, double* gr) {
    using DU = Dual<double, M>;
    const double* mesh = mesh_of(a, I, I.cur);
    const double* hv = h_of(a, I, I.cur);
    const double* y = y_of(a, I, I.cur);
    const double* Kc = a.K + (I.nb + c) * FN;
    const double hc = hv[c];
    double JK[FN * FN];
    double X[FXW];
#pragma unroll
    for (int q = 0; q < FN * FN; ++q) JK[q] = 0.0;
#pragma unroll 1
    for (int r = 0; r < FS; ++r) {
        DU Y[M], fy[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            double acc = y[c * M + m];
#pragma unroll
            for (int j = 0; j < FS; ++j) acc += hc * (Kc[j * M + m] * FA[r][j]);
            Y[m] = DU(acc);
            Y[m].d[m] = 1.0;
        }
        bvp_f<DU, double>(fy, Y, I.p, mesh[c] + FC[r] * hc);
#pragma unroll
        for (int q = 0; q < M; ++q) {
            const int row = r * M + q;
#pragma unroll
            for (int cc = 0; cc < M; ++cc) {
                const double J = fy[q].d[cc];
                X[row * (M + 1) + cc] = J;
#pragma unroll
                for (int j = 0; j < FS; ++j) JK[row * FN + j * M + cc] = hc * FA[r][j] * J;
            }
            JK[row * FN + row] -= 1.0;
            X[row * (M + 1) + M] = fy[q].v - Kc[r * M + q];
        }
    }
    // elimination with partial pivoting on JK, applied to the M + 1 columns of X
    bool ok = true;
#pragma unroll 1
    for (int k = 0; k < FN; ++k) {
        int p = k;
        for (int r = k + 1; r < FN; ++r)
            if (fabs(JK[r * FN + k]) > fabs(JK[p * FN + k])) p = r;
        if (JK[p * FN + k] == 0.0) { ok = false; break; }
        if (p != k) {
            for (int q = 0; q < FN; ++q) { const double t = JK[k * FN + q]; JK[k * FN + q] = JK[p * FN + q]; JK[p * FN + q] = t; }
            for (int q = 0; q <= M; ++q) { const double t = X[k * (M + 1) + q]; X[k * (M + 1) + q] = X[p * (M + 1) + q]; X[p * (M + 1) + q] = t; }
        }
        for (int r = k + 1; r < FN; ++r) {
            const double mlt = JK[r * FN + k] / JK[k * FN + k];
            for (int q = k; q < FN; ++q) JK[r * FN + q] -= mlt * JK[k * FN + q];
            for (int q = 0; q <= M; ++q) X[r * (M + 1) + q] -= mlt * X[k * (M + 1) + q];
        }
    }
    if (ok) {
#pragma unroll 1
        for (int k = FN - 1; k >= 0; --k)
            for (int q = 0; q <= M; ++q) {
                double v = X[k * (M + 1) + q];
                for (int j = k + 1; j < FN; ++j) v -= JK[k * FN + j] * X[j * (M + 1) + q];
                X[k * (M + 1) + q] = v / JK[k * FN + k];
            }
    }
    double* fx = a.fx + (I.nb + c) * FXW;
#pragma unroll
    for (int q = 0; q < FXW; ++q) fx[q] = X[q];
#pragma unroll
    for (int q = 0; q < M; ++q) {
#pragma unroll
        for (int cc = 0; cc < M; ++cc) {
            double acc = 0.0;
#pragma unroll
            for (int j = 0; j < FS; ++j) acc += FB[j] * X[(j * M + q) * (M + 1) + cc];
            Sr[q * M + cc] = hc * acc - (q == cc ? 1.0 : 0.0);
            Rr[q * M + cc] = q == cc ? 1.0 : 0.0;
        }
        double kb = 0.0, xb = 0.0;
#pragma unroll
        for (int j = 0; j < FS; ++j) {
            kb += Kc[j * M + q] * FB[j];
            xb += FB[j] * X[(j * M + q) * (M + 1) + M];
        }
        const double C = (y[(c + 1) * M + q] - y[c * M + q]) - hc * kb;
        gr[q] = -(C + hc * xb);
    }
    return ok;
}
#endif

// Newton direction δ (in a.delta) for J δ = -F. Returns false if singular.
BVP_DEV bool linear_solve(const Args& a, const Inst& I) {
    const int lane = lane_id();
    const int nk = I.iscr[ISCR_NK];
    const int ns = nk - 1;
    // this lane's segment, position in its lane group and interval block
    int seg = -1, t = 0, L = 1, na = 0, nbk = 0;
    for (int j = 0; j < ns; ++j) {
        const int o0 = I.iscr[ISCR_LOFF + j], o1 = I.iscr[ISCR_LOFF + j + 1];
        if (lane >= o0 && lane < o1) { seg = j; t = lane - o0; L = o1 - o0; }
    }
    const bool active = seg >= 0;
    if (active) { na = I.iscr[ISCR_KEPT + seg]; nbk = I.iscr[ISCR_KEPT + seg + 1]; }
    const int len = nbk - na;
    const int blo = na + (t * len) / L;            // block [blo, bhi)
    const int bhi = na + ((t + 1) * len) / L;
    bool bad = false;
    // 1. sequential elimination inside the block, each interval's Jacobian blocks computed
    //    where they are used (block_jacobian) instead of read back from memory
    JT A[M * M], B[M * M], g[M];
    if (active) {
        using DI = Dual<JT, D>;
        const JT* yj = yj_of(a, I);
        const JT* tj = a.tj + I.nb;
        const JT* hj = a.hj + I.nb;
        const JT* Fj = a.Fj + I.nb * M;
        DI node[M];
        {
            DI y0v[M];
#pragma unroll
            for (int m = 0; m < M; ++m) { y0v[m] = DI(yj[blo * M + m]); y0v[m].d[m] = JT(1); }
            if (NODE_SHARE) call_stage_f<DI, JT>(node, y0v, I.pj, tj[blo]);
        }
#pragma unroll 1
        for (int c = blo; c < bhi; ++c) {
            JT Sr[M * M], Rr[M * M], gr[M];
#if BVP_FIRK
            bad |= !firk_block(a, I, c, Sr, Rr, gr);
#else
            block_jacobian(yj, tj, hj, I.pj, c, node, Sr, Rr);
#pragma unroll
            for (int m = 0; m < M; ++m) gr[m] = -Fj[c * M + m];
#endif
            if (c == blo) {
#pragma unroll
                for (int q = 0; q < M * M; ++q) { A[q] = Sr[q]; B[q] = Rr[q]; }
#pragma unroll
                for (int m = 0; m < M; ++m) g[m] = gr[m];
            } else {
                bad |= !eliminate_pair(A, B, g, Sr, Rr, gr, a.rec + (I.nb + c) * RECW, A, B, g);
            }
        }
    }
    // 2. shuffle tree over the block relations of each lane group
    int bnode = bhi;
    int xs[5];
#pragma unroll TREE_UNROLL
    for (int s = 0; s < 5; ++s) {
        const int step = 1 << s;
        JT Ap[M * M], Bp[M * M], gp[M];
#pragma unroll
        for (int q = 0; q < M * M; ++q) {
            Ap[q] = __shfl_down_sync(FULL, A[q], step);
            Bp[q] = __shfl_down_sync(FULL, B[q], step);
        }
#pragma unroll
        for (int q = 0; q < M; ++q) gp[q] = __shfl_down_sync(FULL, g[q], step);
        const int bp = __shfl_down_sync(FULL, bnode, step);
        xs[s] = bnode;
        if (active && (t % (2 * step)) == 0 && t + step < L) {
            JT* rdst = I.trec ? I.trec + tree_slot(s, lane) * RECW : a.rec + (I.nb + bnode) * RECW;
            bad |= !eliminate_pair(A, B, g, Ap, Bp, gp, rdst, A, B, g);
            bnode = bp;
        }
    }
    if (active && t == 0) store_eq(seg_of(I, seg), A, B, g);
    __syncwarp();
    // 3. separator system
    int dense_ok = 1;
    if constexpr (SMEM_DENSE) {
        dense_ok = separator_solve_warp(a, I, nk) ? 1 : 0;
    } else if (lane == 0) {
        // in thread-local storage (L1-resident), not the global scratch: the elimination
        // reads back what it just wrote
        const int n = nk * M;
        JT G[NDENSE * NDENSE];
        JT rhs[NDENSE];
        for (int q = 0; q < n * n; ++q) G[q] = JT(0);
        for (int j = 0; j + 1 < nk; ++j) {
            const JT* seg = seg_of(I, j);
            for (int r = 0; r < M; ++r) {
                const int row = j * M + r;
                for (int c = 0; c < M; ++c) {
                    G[row * n + j * M + c] = seg[r * M + c];
                    G[row * n + (j + 1) * M + c] = seg[M * M + r * M + c];
                }
                rhs[row] = seg[2 * M * M + r];
            }
        }
        const int row0 = (nk - 1) * M;
        const int nb = I.iscr[ISCR_NB];
        for (int k = 0; k < nb; ++k) {
            const int node = I.iscr[ISCR_BNODE + k];
            int kj = 0;
            while (I.iscr[ISCR_KEPT + kj] != node) ++kj;
            for (int r = 0; r < M; ++r)
                for (int c = 0; c < M; ++c)
                    G[(row0 + r) * n + kj * M + c] += JT(I.scr[SCR_BCBLK + k * M * M + r * M + c]);
        }
        for (int r = 0; r < M; ++r) rhs[row0 + r] = JT(-I.scr[SCR_BCRES + r]);
        dense_ok = dense_solve<JT>(n, G, rhs) ? 1 : 0;
        for (int j = 0; j < nk; ++j) {
            JT* d = a.delta + (I.nb + I.iscr[ISCR_KEPT + j]) * M;
            for (int r = 0; r < M; ++r) d[r] = rhs[j * M + r];
        }
    }
    dense_ok = __shfl_sync(FULL, dense_ok, 0);
    __syncwarp();
    if (warp_any(bad) || !dense_ok) return false;
    // 4a. unwind the tree: every lane gets δ at its block ends (the group roots read them from
    //     the separator solve's shared-memory rows, else from δ)
    JT da[M], db[M];
    if (active && t == 0) {
        if constexpr (SMEM_DENSE) {
            const int n = nk * M;
#pragma unroll
            for (int m = 0; m < M; ++m) {
                da[m] = I.dns[(seg * M + m) * DLD + n];
                db[m] = I.dns[((seg + 1) * M + m) * DLD + n];
            }
        } else {
#pragma unroll
            for (int m = 0; m < M; ++m) {
                da[m] = a.delta[(I.nb + na) * M + m];
                db[m] = a.delta[(I.nb + nbk) * M + m];
            }
        }
    }
#pragma unroll TREE_UNROLL
    for (int s = 4; s >= 0; --s) {
        const int step = 1 << s;
        const bool comb = active && (t % (2 * step)) == 0 && t + step < L;
        JT dx[M];
        if (comb) {
            back_solve(I.trec ? I.trec + tree_slot(s, lane) * RECW : a.rec + (I.nb + xs[s]) * RECW, da, db, dx);
            JT* dg = a.delta + (I.nb + xs[s]) * M;
#pragma unroll
            for (int m = 0; m < M; ++m) dg[m] = dx[m];
        }
        JT r1[M], r2[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            r1[m] = __shfl_up_sync(FULL, comb ? dx[m] : JT(0), step);
            r2[m] = __shfl_up_sync(FULL, db[m], step);
        }
        const bool recv = active && (t % (2 * step)) == step;
        if (recv) {
#pragma unroll
            for (int m = 0; m < M; ++m) { da[m] = r1[m]; db[m] = r2[m]; }
        }
        if (comb) {
#pragma unroll
            for (int m = 0; m < M; ++m) db[m] = dx[m];
        }
    }
    // 4b. back substitution inside the block
    if (active) {
        JT* dgl = a.delta + (I.nb + blo) * M;
#pragma unroll
        for (int m = 0; m < M; ++m) dgl[m] = da[m];
        JT dn[M];
#pragma unroll
        for (int m = 0; m < M; ++m) dn[m] = db[m];
        if constexpr (RECW <= 32) {
            // records in registers, the next one loaded while this one is applied
            const JT* rbase = a.rec + I.nb * RECW;
            JT rc[RECW], rn[RECW];
            if (bhi - 1 > blo) {
#pragma unroll
                for (int q = 0; q < RECW; ++q) rc[q] = rbase[(bhi - 1) * RECW + q];
            }
#pragma unroll 1
            for (int c = bhi - 1; c > blo; --c) {
                if (c - 1 > blo) {
#pragma unroll
                    for (int q = 0; q < RECW; ++q) rn[q] = rbase[(c - 1) * RECW + q];
                }
                JT dc[M];
                back_solve(rc, da, dn, dc);
                JT* dg = a.delta + (I.nb + c) * M;
#pragma unroll
                for (int m = 0; m < M; ++m) { dg[m] = dc[m]; dn[m] = dc[m]; bad |= !isfinite(dc[m]); }
#pragma unroll
                for (int q = 0; q < RECW; ++q) rc[q] = rn[q];
            }
        } else {
            for (int c = bhi - 1; c > blo; --c) {
                JT dc[M];
                back_solve(a.rec + (I.nb + c) * RECW, da, dn, dc);
                JT* dg = a.delta + (I.nb + c) * M;
#pragma unroll
                for (int m = 0; m < M; ++m) { dg[m] = dc[m]; dn[m] = dc[m]; bad |= !isfinite(dc[m]); }
            }
        }
#pragma unroll
        for (int m = 0; m < M; ++m) bad |= !isfinite(da[m]) || !isfinite(db[m]);
    }
    __syncwarp();
    return !warp_any(bad);
}

// ---- Newton (default_internal_solve.jl:31-45; ||F||_inf <= abstol, mirk.jl:51) ------------
BVP_DEV void copy_y(double* dst, const double* src, int n) {
    for (int k = lane_id(); k < n; k += 32) dst[k] = src[k];
    __syncwarp();
}

// JT copy of the current iterate
BVP_DEV void refresh_yj(const Args& a, const Inst& I) {
    const double* y = y_of(a, I, I.cur);
    JT* yj = yj_of(a, I);
    for (int k = lane_id(); k < I.N * M; k += 32) yj[k] = JT(y[k]);
    __syncwarp();
}

#ifndef BVP_FP32_SWITCH
#define BVP_FP32_SWITCH 100.0   // the FP32 phase ends when the FP32 residual falls to this times abstol
#endif
// Mixed-precision Newton: the iterations run on the FP32 residual (stages in FP32, node
// differences in FP64, roundoff about h|K| eps32) until it falls to 100 abstol or stops
// improving near that level; the last steps then take the FP64 residual as right-hand side,
// so the accepted iterate is the one an FP64 Newton reaches (an FP32 right-hand side would
// move it by cond(J) times its roundoff). Every convergence decision is made in FP64.
BVP_DEV bool newton_attempt(const Args& a, Inst& I, bool linesearch, int& iters, double& nrm_out) {
    const int lane = lane_id();
    double* y = y_of(a, I, I.cur);
    JT* yj = yj_of(a, I);
    double* yb = a.ybase + I.nb * M;
    const JT* dl = a.delta + I.nb * M;
    const int nM = I.N * M;
    iters = 0;
    refresh_yj(a, I);
    bool f32 = F32_PHASE_OK && a.fp32_phase && !linesearch;
    const double switch_tol = BVP_FP32_SWITCH * a.abstol;
    // One residual evaluation per pass of this loop (a single inlined copy of each residual
    // kernel); `why` says what the evaluation is for.
    enum { R_START, R_SWITCH, R_STEP, R_TRIAL };
    int why = R_START;
    double nrm0 = 0.0, best = 0.0, f0 = 0.0, alpha = 1.0;
    int stall = 0, ls = 0;
#pragma unroll 1
    while (true) {
        double nrm;
        if constexpr (F32_PHASE_OK) nrm = f32 ? residual<float>(a, I) : residual<double>(a, I);
        else nrm = residual<double>(a, I);
        if (why == R_TRIAL) {
            // backtracking line search: accept when ||F||^2 decreased enough (Armijo)
            const double f1 = residual_sq(a, I);
            if (!(isfinite(nrm) && f1 <= (1.0 - 2e-4 * alpha) * f0)) {
                alpha *= 0.5;
                if (++ls >= 20) { nrm_out = nrm; return false; }
                for (int k = lane; k < nM; k += 32) {
                    const double v = yb[k] + alpha * double(dl[k]);
                    y[k] = v;
                    yj[k] = JT(v);
                }
                __syncwarp();
                continue;
            }
            why = R_STEP;
        }
        nrm_out = nrm;
        if (why == R_START) {
            if (f32 && !(nrm > switch_tol)) { f32 = false; continue; }
            if (!isfinite(nrm)) return false;
            if (nrm <= a.abstol) return true;
            nrm0 = nrm; best = nrm; stall = 0;
        } else if (why == R_SWITCH) {
            if (!isfinite(nrm)) return false;
            if (nrm <= a.abstol) return true;
            nrm0 = fmax(nrm0, nrm); best = nrm; stall = 0;
        } else {
            if (f32 && (!(nrm > switch_tol) || (!(nrm < best) && best < 10.0 * switch_tol))) {
                // close enough, or the FP32 residual stopped improving near its roundoff floor
                // (far from it a non-decreasing step is ordinary Newton behaviour): continue on
                // the FP64 residual, which restarts the stall bookkeeping
                f32 = false;
                why = R_SWITCH;
                continue;
            }
            if (!isfinite(nrm)) return false;
            if (nrm <= a.abstol) return true;
            if (nrm > a.divergence_factor * nrm0) return false;
            if (nrm < best) { best = nrm; stall = 0; }
            else if (++stall >= a.stall_steps) return false;
        }
        if (iters >= a.max_newton) return false;
        bc_jacobian(a, I);
        if (!linear_solve(a, I)) return false;
        ++iters;
        if (!linesearch) {
            for (int k = lane; k < nM; k += 32) {
                const double v = y[k] + double(dl[k]);
                y[k] = v;
                yj[k] = JT(v);
            }
            __syncwarp();
            why = R_STEP;
        } else {
            f0 = residual_sq(a, I);
            copy_y(yb, y, nM);
            alpha = 1.0; ls = 0;
            for (int k = lane; k < nM; k += 32) {
                const double v = yb[k] + double(dl[k]);
                y[k] = v;
                yj[k] = JT(v);
            }
            __syncwarp();
            why = R_TRIAL;
        }
    }
}

// Newton, then Newton with backtracking from the same start when the first fails
// (default_internal_solve.jl:31-45): one inlined copy of the attempt.
BVP_DEV bool newton(const Args& a, Inst& I, InstState& s) {
    double* y = y_of(a, I, I.cur);
    const int nM = I.N * M;
    copy_y(a.ybak + I.nb * M, y, nM);
    bool ok = false;
    double nrm = 0.0;
#pragma unroll 1
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (attempt == 1) {
            if (!a.linesearch) break;
            copy_y(y, a.ybak + I.nb * M, nM);
            s.flags |= 1;
        }
        int it = 0;
        ok = newton_attempt(a, I, attempt == 1, it, nrm);
        s.newton_iters += it;
        if (ok) break;
    }
    s.resid = nrm;
    return ok;
}

// ---- K4: defect estimate (adaptivity.jl:416-461) -------------------------------------------
template <int GL>
BVP_DEV double defect_part(const Args& a, const Inst& I, int gl, bool& bad) {
    const double* mesh = mesh_of(a, I, I.cur);
    const double* h = h_of(a, I, I.cur);
    const double* y = y_of(a, I, I.cur);
    double w1[SS], w1p[SS], w2[SS], w2p[SS];
    interp_weights<double>(tau_star(), w1, w1p);
    interp_weights<double>(1.0 - tau_star(), w2, w2p);
    double dn = 0.0;
    for (int i = gl; i < I.N - 1; i += GL) {
        double yi[M], yi1[M], Ki[S * M], KIi[NSXA * M];
#pragma unroll
        for (int m = 0; m < M; ++m) { yi[m] = y[i * M + m]; yi1[m] = y[(i + 1) * M + m]; }
        const double* Kg = a.K + (I.nb + i) * (S * M);
#pragma unroll
        for (int k = 0; k < S * M; ++k) Ki[k] = Kg[k];
        interp_stages<double, double>(yi, yi1, Ki, KIi, I.p, mesh[i], h[i]);
        double* KIg = a.KI + (I.nb + i) * (NSXA * M);
#pragma unroll
        for (int k = 0; k < NSX * M; ++k) KIg[k] = KIi[k];
        double est[2];
#pragma unroll
        for (int smp = 0; smp < 2; ++smp) {
            const double* w = smp ? w2 : w1;
            const double* wp = smp ? w2p : w1p;
            double z[M], zp[M], fz[M];
            sum_stages<double, double>(w, yi, Ki, KIi, h[i], z);
#pragma unroll
            for (int m = 0; m < M; ++m) {
                double acc = Ki[m] * wp[0];
#pragma unroll
                for (int r = 1; r < S; ++r) acc += Ki[r * M + m] * wp[r];
#pragma unroll
                for (int qq = 0; qq < NSX; ++qq) acc += KIi[qq * M + m] * wp[S + qq];
                zp[m] = acc;
            }
            call_f<double, double>(fz, z, I.p, mesh[i] + (smp ? 1.0 - tau_star() : tau_star()) * h[i]);
            double e = 0.0;
#pragma unroll
            for (int m = 0; m < M; ++m) e = fmax(e, fabs(div_scaled(zp[m] - fz[m], fabs(fz[m]) + 1.0)));
            est[smp] = e;
        }
        const double ei = est[0] > est[1] ? est[0] : est[1];
        a.err[I.nb + i] = ei;
        bad |= isnan(ei);
        dn = fmax(dn, ei);
    }
    return dn;
}

BVP_DEV double defect(const Args& a, const Inst& I) {
    bool bad = false;
    double dn;
    if (GROUP_OK && I.grp) dn = group_phase(a, I, CMD_DEFECT, bad);
    else dn = defect_part<32>(a, I, lane_id(), bad);
    __syncwarp();
    dn = warp_max(dn);
    return warp_any(bad) ? dinf() : dn;
}

// ---- block mode ------------------------------------------------------------------------------
// A long mesh is solved by a whole block: its first warp runs the solve and the other warps
// join it for the phases that are independent per interval (the residuals and the defect,
// most of a long mesh's time), each lane of the block taking its share of the intervals. The
// warps meet at a named barrier of the block's 128 threads; the leader posts a command and
// the instance, every warp runs its part and leaves its largest value, and the leader
// combines them. The parts are the warp code's with 128 lanes instead of 32, and each
// interval's values do not depend on which lane computes them, so the results are the same
// as the warp's.
struct GroupShared {
    Inst inst;
    int cmd;
    int bad[GROUP_WARPS];
    double red[GROUP_WARPS];
};
// bar.sync is warp-aligned: a warp that reached it in pieces (after a lane-0 store) could
// count twice, so the warp reconverges first
BVP_DEV void group_bar() {
    __syncwarp();
    asm volatile("bar.sync 1, 128;" ::: "memory");
}

__device__ __noinline__ double group_part(const Args& a, const Inst& I, int cmd, int gl, int* bad_out) {
    bool bad = false;
    double v = 0.0;
    if (cmd == CMD_RES64) {
        v = residual_part<double, 32 * GROUP_WARPS>(a, I, gl, bad);
    } else if (cmd == CMD_RES32) {
        if constexpr (F32_PHASE_OK) v = residual_part<float, 32 * GROUP_WARPS>(a, I, gl, bad);
    } else {
        v = defect_part<32 * GROUP_WARPS>(a, I, gl, bad);
    }
    *bad_out = bad ? 1 : 0;
    return v;
}

// the leader's side: post, run its own part, collect (every lane gets the block's result)
BVP_DEV double group_phase(const Args& a, const Inst& I, int cmd, bool& bad) {
    GroupShared* g = I.grp;
    const int lane = lane_id();
    if (lane == 0) { g->inst = I; g->cmd = cmd; }
    group_bar();
    int b = 0;
    double v = warp_max(group_part(a, I, cmd, lane, &b));
    const bool wb = warp_any(b != 0);
    if (lane == 0) { g->red[0] = v; g->bad[0] = wb ? 1 : 0; }
    group_bar();
#pragma unroll
    for (int w = 1; w < GROUP_WARPS; ++w) { v = fmax(v, g->red[w]); bad |= g->bad[w] != 0; }
    bad |= wb;
    return v;
}

// the other warps' side, until the leader posts CMD_EXIT
BVP_DEV void group_helper(const Args& a, GroupShared* g, int w) {
    const int lane = lane_id();
    while (true) {
        group_bar();
        const int cmd = g->cmd;
        if (cmd == CMD_EXIT) break;
        const Inst I = g->inst;
        int b = 0;
        const double v = warp_max(group_part(a, I, cmd, w * 32 + lane, &b));
        const bool wb = warp_any(b != 0);
        if (lane == 0) { g->red[w] = v; g->bad[w] = wb ? 1 : 0; }
        group_bar();
    }
}

// ---- mesh selection (adaptivity.jl:23-75, 250-304) -------------------------------------------
// half_mesh! of buffer src into buffer dst. Each new node's old interval (the one the
// reference's interval() finds for it, lower_bound - 1 clamped) goes to iold as a hint for
// the solution transfer.
BVP_DEV void half_mesh(const Args& a, Inst& I, int src, int dst) {
    const double* m0 = mesh_of(a, I, src);
    const double* h0 = h_of(a, I, src);
    double* m1 = mesh_of(a, I, dst);
    double* h1 = h_of(a, I, dst);
    int* io = a.iold + I.nb;
    const int n = I.N - 1;
    for (int i = lane_id(); i <= n; i += 32) {
        m1[2 * i] = m0[i];
        io[2 * i] = i > 0 ? i - 1 : 0;
        if (i < n) {
            m1[2 * i + 1] = (m0[i + 1] + m0[i]) / 2.0;
            h1[2 * i] = h0[i] / 2.0;
            h1[2 * i + 1] = h0[i] / 2.0;
            io[2 * i + 1] = i;
        }
    }
    __syncwarp();
}

BVP_DEV long round_even(double x) { return (long)rint(x); }

// x^(1/P), the selector's ŝ = (err/abstol)^(1/(p+1)) (adaptivity.jl:43; 1/p for the global
// error, adaptivity.jl:96): an FP32 seed refined by two Newton steps on y^P = x in FP64 (the
// derivative's reciprocal taken in FP32: the first step leaves ~1e-14, the second the FP64
// roundoff of y^P), a dozen FP64 operations instead of a double-precision pow. Zero, extreme
// and non-finite arguments go to pow.
template <int P>
BVP_DEV double root_n(double x) {
    if (!(x >= 1e-30 && x <= 1e30)) return pow(x, 1.0 / P);
    double y = double(powf(float(x), 1.0f / float(P)));
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        double ypm1 = y;
#pragma unroll
        for (int k = 2; k < P; ++k) ypm1 *= y;                 // y^(P-1)
        const double r = fma(ypm1, y, -x);                     // y^P - x
        const float c = 1.0f / (float(P) * float(ypm1));
        y = fma(-r, double(c), y);
    }
    return y;
}
BVP_DEV double root_p1(double x) { return root_n<(FIRK ? FORDER : ORD) + 1>(x); }

// which errors make the selector's ŝ: the defect's (DefectControl, and SequentialErrorControl
// before its defect passes), the global estimate's to 1/(p+1) (SequentialErrorControl after),
// to 1/p (GlobalErrorControl), or the sum of both terms (HybridErrorControl, 207-209)
enum : int { SEL_DEFECT = 0, SEL_GLOBAL_P1 = 1, SEL_GLOBAL_P = 2, SEL_HYBRID = 3 };

// Returns 1 on success (new mesh in buffer cur^1, newN set, iold hints written), 0 on Failure.
//
// redistribute! (adaptivity.jl:250-278) places Nsub - 1 interior points so that each
// subinterval holds the same share ζ = Σ ŝ / Nsub of the piecewise-constant density ŝ_k / h_k.
// The reference walks the mesh sequentially; here the cumulative density is a warp scan
// (each lane a contiguous block of old intervals, running sums inside the block), point j
// lies in the old interval k whose cumulative range (C_k, C_k+1] holds j ζ, at
// t_k + (j ζ - C_k) h_k / ŝ_k. The point indices per interval come from floor(C / ζ) with a
// running maximum across the warp, so every point 1..Nsub-1 is placed exactly once even
// where the block sums round differently from the running sums. The positions agree with
// the sequential walk to rounding (same formula, different association).
// The selectors of the global-error controllers (adaptivity.jl:77-243) differ from the
// defect's only in ŝ (sel) and in ρ = 2.
BVP_DEV int mesh_selector(const Args& a, Inst& I, int& newN, int sel = SEL_DEFECT, double rho = 1.0) {
    const int lane = lane_id();
    const int n = I.N - 1;
    const double* h0 = h_of(a, I, I.cur);
    double* e = a.err + I.nb;
    const double* g = a.gerr + I.nb;
    const double inv_tol = 1.0 / a.abstol;
    double r1 = -dinf(), r2p = 0.0;
    for (int i = lane; i < n; i += 32) {
        double sh;
        if constexpr (GLOBAL_CTL) {
            if (sel == SEL_DEFECT) sh = root_p1(e[i] * inv_tol);
            else if (sel == SEL_GLOBAL_P1) sh = root_p1(g[i] * inv_tol);
            else if (sel == SEL_GLOBAL_P) sh = root_n<ORD>(g[i] * inv_tol);
            else sh = root_p1(e[i] * inv_tol) + root_p1(g[i] * inv_tol);
        } else {
            sh = root_p1(e[i] * inv_tol);
        }
        e[i] = sh;
        r1 = fmax(r1, sh);
        r2p += sh;
    }
    __syncwarp();   // the block sums below read other lanes' ŝ
    r1 = warp_max(r1);
    const double r2 = warp_sum(r2p);
    const double r3 = r2 / (I.N - 1);
    long n_pred = round_even(1.3 * r2 + 1);
    const double n_ = 0.1 * n;
    if (fabs(double(n_pred - n)) < n_) n_pred = round_even(n + n_);
    const int dst = I.cur ^ 1;
    if (r1 <= rho * r3) {
        if (2L * n > a.max_sub || 2 * n + 1 > I.cap) return 0;
        half_mesh(a, I, I.cur, dst);
        newN = 2 * n + 1;
        return 1;
    }
    const long lb = I.N / 2, ub = 4L * (I.N - 1);
    long Nl = n_pred < lb ? lb : n_pred;
    Nl = Nl > ub ? ub : Nl;
    if (Nl > a.max_sub || Nl + 1 > I.cap) return 0;
    const int Nsub = int(Nl);
    const double* om = mesh_of(a, I, I.cur);
    double* nm = mesh_of(a, I, dst);
    double* nh = h_of(a, I, dst);
    int* io = a.iold + I.nb;
    double* cbeg = a.F + I.nb * M;         // C_k per old interval (the residual is recomputed next round)
    // 1. block sums of ŝ and their exclusive scan
    const int per = (n + 31) >> 5;
    const int k0 = min(lane * per, n), k1 = min(k0 + per, n);
    double bsum = 0.0;
    for (int k = k0; k < k1; ++k) bsum += e[k];
    double incl = bsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
    }
    const double tot = __shfl_sync(FULL, incl, 31);
    const double zeta = tot / double(Nsub);
    const double izeta = double(Nsub) / tot;
    double base = __shfl_up_sync(FULL, incl, 1);
    if (lane == 0) base = 0.0;
    auto jof = [&](double c) {
        const double q = floor(c * izeta);
        return q >= double(Nsub - 1) ? Nsub - 1 : (q > 0.0 ? int(q) : 0);
    };
    // 2. first point index of each lane's block: running maximum of the block ends' indices
    double cend = base;
    for (int k = k0; k < k1; ++k) cend += e[k];
    int jm = k1 > k0 ? jof(cend) : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(FULL, jm, o);
        if (lane >= o) jm = max(jm, t);
    }
    int jlo = __shfl_up_sync(FULL, jm, 1);
    if (lane == 0) jlo = 0;
    // 3. each old interval's points: their interval in iold, C_k and h_k / ŝ_k for the positions
    double c = base;
    for (int k = k0; k < k1; ++k) {
        const double P = e[k];
        const double cn = c + P;
        const int jhi = max(jlo, jof(cn));
        if (jhi > jlo) {
            cbeg[k * M] = c;
            e[k] = P > 0.0 ? h0[k] / P : 0.0;
            for (int j = jlo + 1; j <= jhi; ++j) io[j] = k;
        }
        jlo = jhi;
        c = cn;
    }
    if (lane == 0) { io[0] = 0; io[Nsub] = n - 1; }
    __syncwarp();
    // 4. the points
    for (int j = lane; j <= Nsub; j += 32) {
        double pt;
        if (j == 0) pt = om[0];
        else if (j == Nsub) pt = om[n];
        else {
            const int k = io[j];
            pt = fma(fma(double(j), zeta, -cbeg[k * M]), e[k], om[k]);
            pt = fmin(fmax(pt, om[k]), om[k + 1]);
        }
        nm[j] = pt;
    }
    __syncwarp();
    for (int q = lane; q < Nsub; q += 32) nh[q] = nm[q + 1] - nm[q];
    __syncwarp();
    newN = Nsub + 1;
    return 1;
}

// New solution on mesh buffer cur^1 from the old interpolant (adaptivity.jl:6-13 as called in
// mirk.jl:366-371). With transfer_inplace the reference's in-place update is reproduced:
// node j reads y[i_old] after nodes < j were already overwritten, so its base is the new value
// of node i_old when i_old < j and the old one otherwise. Lanes take 32 consecutive nodes at a
// time; a base inside the same 32 comes from that lane by shuffles, in dependency order (each
// node depends on an earlier one, so the chain ends), which reproduces the sequential values
// exactly. The old interval of each node is the mesh selector's hint, checked against the
// interval() rule (lower_bound - 1, clamped) and searched for when it does not hold.
BVP_DEV void transfer(const Args& a, Inst& I, int newN) {
    const int lane = lane_id();
    const int src = I.cur, dst = I.cur ^ 1;
    const int No = I.N;
    const double* om = mesh_of(a, I, src);
    const double* oh = h_of(a, I, src);
    const double* nm = mesh_of(a, I, dst);
    const double* oy = y_of(a, I, src);
    double* ny = y_of(a, I, dst);
    const int* io = a.iold + I.nb;
    const bool inplace = a.transfer_inplace != 0;
    for (int c0 = 0; c0 < newN; c0 += 32) {
        const int j = c0 + lane;
        const bool act = j < newN;
        double v[M];
        int i = 0;
        if (act) {
            const double t = nm[j];
            i = io[j];
            const bool hint = i >= 0 && i <= No - 2 && (i == 0 || om[i] < t) && (i == No - 2 || t <= om[i + 1]);
            if (!hint) i = interval_of(om, No, t);
            const double dt = oh[i];
            const double tau = (t - om[i]) / dt;
            double w[SS], wp[SS];
            interp_weights_rt(tau, w, wp);
            const double* Kg = a.K + (I.nb + i) * (S * M);
            const double* KIg = a.KI + (I.nb + i) * (NSXA * M);
#pragma unroll
            for (int m = 0; m < M; ++m) {
                double acc = Kg[m] * w[0];
#pragma unroll
                for (int r = 1; r < S; ++r) acc += Kg[r * M + m] * w[r];
#pragma unroll
                for (int qq = 0; qq < NSX; ++qq) acc += KIg[qq * M + m] * w[S + qq];
                v[m] = acc * dt;
            }
        }
        if (!inplace) {
            if (act) {
#pragma unroll
                for (int m = 0; m < M; ++m) ny[j * M + m] = v[m] + oy[i * M + m];
            }
        } else {
            double val[M];
            bool done = !act || i >= j || i < c0;
            if (act) {
                const double* b = i >= j ? oy + i * M : ny + i * M;
#pragma unroll
                for (int m = 0; m < M; ++m) val[m] = done ? v[m] + b[m] : 0.0;
            }
            const int from = (i - c0) & 31;
            while (__any_sync(FULL, !done)) {
                const int sd = __shfl_sync(FULL, int(done), from);
                double sv[M];
#pragma unroll
                for (int m = 0; m < M; ++m) sv[m] = __shfl_sync(FULL, act ? val[m] : 0.0, from);
                if (!done && sd) {
#pragma unroll
                    for (int m = 0; m < M; ++m) val[m] = v[m] + sv[m];
                    done = true;
                }
            }
            if (act) {
#pragma unroll
                for (int m = 0; m < M; ++m) ny[j * M + m] = val[m];
            }
        }
        __syncwarp();
    }
}

// ---- one instance, whole adaptive solve (solve!, mirk.jl:286-388) -----------------------------
BVP_DEV void init_instance(const Args& a, Inst& I) {
    const int lane = lane_id();
    const int n = a.n_init[I.q];
    const double t0 = a.tspans[2 * I.q], t1 = a.tspans[2 * I.q + 1];
    double* mesh = mesh_of(a, I, 0);
    double* h = h_of(a, I, 0);
    double* y = y_of(a, I, 0);
    const double hh = (t1 - t0) / n;   // range(t0; stop = t1, length = n + 1) (Core/utils.jl:694-700)
    for (int i = lane; i <= n; i += 32) mesh[i] = (i == n) ? t1 : fma(double(i), hh, t0);
    __syncwarp();
    for (int i = lane; i < n; i += 32) h[i] = mesh[i + 1] - mesh[i];
    if (a.y0_mode == 0) {
        const double* src = a.y0 + I.q * M;
        for (int k = lane; k < (n + 1) * M; k += 32) y[k] = src[k % M];
    } else if (a.y0_mode == 1) {
        const double* src = a.y0 + a.y0_off[I.q] * M;
        for (int k = lane; k < (n + 1) * M; k += 32) y[k] = src[k];
    } else {
        // guess on a uniform grid of n_grid points over the tspan, resampled linearly onto
        // the initial mesh (separately rounded products and sum, as the host resampling does)
        const int G = a.n_grid;
        const float* gq = a.y0_grid + (long long)I.q * G * M;
        const double inv_n = 1.0 / double(n);
        for (int j = lane; j <= n; j += 32) {
            const double sg = __dmul_rn(__dmul_rn(double(j), inv_n), double(G - 1));
            int i0 = int(floor(sg));
            i0 = i0 < 0 ? 0 : (i0 > G - 2 ? G - 2 : i0);
            const double f = sg - i0;
#pragma unroll
            for (int m = 0; m < M; ++m)
                y[j * M + m] = __dadd_rn(__dmul_rn(1.0 - f, double(gq[i0 * M + m])),
                                         __dmul_rn(f, double(gq[(i0 + 1) * M + m])));
        }
    }
    __syncwarp();
    I.N = n + 1;
    I.cur = 0;
}

BVP_DEV void finalize_stages(const Args& a, Inst& I) {
    mesh_setup(a, I);
    refresh_yj(a, I);
    residual<double>(a, I);
    const double* mesh = mesh_of(a, I, I.cur);
    const double* h = h_of(a, I, I.cur);
    const double* y = y_of(a, I, I.cur);
    for (int i = lane_id(); i < I.N - 1; i += 32) {
        double yi[M], yi1[M], Ki[S * M], KIi[NSXA * M];
#pragma unroll
        for (int m = 0; m < M; ++m) { yi[m] = y[i * M + m]; yi1[m] = y[(i + 1) * M + m]; }
        const double* Kg = a.K + (I.nb + i) * (S * M);
#pragma unroll
        for (int k = 0; k < S * M; ++k) Ki[k] = Kg[k];
        interp_stages<double, double>(yi, yi1, Ki, KIi, I.p, mesh[i], h[i]);
        double* KIg = a.KI + (I.nb + i) * (NSXA * M);
#pragma unroll
        for (int k = 0; k < NSX * M; ++k) KIg[k] = KIi[k];
    }
    __syncwarp();
}

// ---- global error estimates (adaptivity.jl:463-567) ------------------------------------------
// The second solve of a global estimate, on buffer cur^1 from the current solution:
// REErrorControl on the halved mesh (halve_sol, adaptivity.jl:310-332: the old nodes at the
// even 0-based positions, each midpoint node the mean of its neighbours), HOErrorControl on
// the same mesh in the module compiled for MIRK(p+2) (phase 2). The new cache takes
// mesh_dt = diff(mesh) (mirk.jl:75-76); the Newton outcome is not consulted (adaptivity.jl:
// 530-531, 547-549) and its iterations are not the instance's. Returns false when the halved
// mesh does not fit the instance's capacity.
BVP_DEV bool second_solve(const Args& a, Inst& I, bool halve) {
    const int lane = lane_id();
    const int n = I.N - 1;
    const int Nn = halve ? 2 * n + 1 : I.N;
    if (Nn > I.cap) return false;
    const double* m0 = mesh_of(a, I, I.cur);
    const double* y0 = y_of(a, I, I.cur);
    double* m1 = mesh_of(a, I, I.cur ^ 1);
    double* h1 = h_of(a, I, I.cur ^ 1);
    double* y1 = y_of(a, I, I.cur ^ 1);
    const int st = halve ? 2 : 1;
    for (int i = lane; i <= n; i += 32) {
        m1[st * i] = m0[i];
#pragma unroll
        for (int m = 0; m < M; ++m) y1[st * i * M + m] = y0[i * M + m];
        if (halve && i < n) {
            m1[2 * i + 1] = (m0[i + 1] + m0[i]) / 2.0;
#pragma unroll
            for (int m = 0; m < M; ++m) y1[(2 * i + 1) * M + m] = (y0[(i + 1) * M + m] + y0[i * M + m]) / 2.0;
        }
    }
    __syncwarp();
    for (int q = lane; q < Nn - 1; q += 32) h1[q] = m1[q + 1] - m1[q];
    __syncwarp();
    const int c0 = I.cur, N0 = I.N;
    I.cur ^= 1;
    I.N = Nn;
    mesh_setup(a, I);
    InstState t;
    t.N = Nn; t.cur = I.cur; t.retcode = RET_FAILURE; t.newton_iters = 0; t.rounds = 0; t.flags = 0;
    t.defect = 0.0; t.resid = 0.0; t.global_err = 0.0;
    newton(a, I, t);
    I.cur = c0;
    I.N = N0;
    return true;
}

// The estimate from the second solve's nodes (buffer cur^1, every st-th of them at the current
// nodes): err_j = max_m |(y_high - y) / (1 + |y|)| at each current node, each interval keeps
// the larger of its end nodes' errors (GE_subinterval!, adaptivity.jl:557-567), the norm is
// their maximum (NaN when any is), times 2^p / (2^p - 1) for Richardson extrapolation
// (adaptivity.jl:534). The current solution's stages are then evaluated again for the
// transfer: the second solve overwrote K, and GlobalErrorControl has no defect pass to
// leave the extra stages.
BVP_DEV double global_finish(const Args& a, Inst& I, int st) {
    const int lane = lane_id();
    const double* yl = y_of(a, I, I.cur);
    const double* yh = y_of(a, I, I.cur ^ 1);
    double* g = a.gerr + I.nb;
    auto node_err = [&](int j) {
        double e = 0.0;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            const double lo = yl[j * M + m];
            const double v = fabs((yh[st * j * M + m] - lo) / (1.0 + fabs(lo)));
            e = (isnan(v) || v > e) ? v : e;
        }
        return e;
    };
    double gn = 0.0;
    bool bad = false;
    for (int i = lane; i < I.N - 1; i += 32) {
        const double e0 = node_err(i), e1 = node_err(i + 1);
        const double gi = e0 >= e1 ? e0 : e1;
        g[i] = gi;
        bad |= isnan(gi);
        gn = fmax(gn, gi);
    }
    __syncwarp();
    gn = warp_max(gn);
    if (warp_any(bad)) gn = __longlong_as_double(0x7ff8000000000000LL);
    if (a.global_method == GLOBAL_RE) {
        const double p2 = double(1 << ORD);
        gn = gn * p2 / (p2 - 1.0);
    }
    finalize_stages(a, I);
    return gn;
}

// An instance stops for its MIRK(p+2) solve: its state goes to st[q], its id to the pause list.
BVP_DEV void pause_instance(const Args& a, const Inst& I, InstState& s) {
    s.N = I.N;
    s.cur = I.cur;
    if (lane_id() == 0) {
        a.st[I.q] = s;
        a.pause_list[atomicAdd(a.pause_count, 1)] = I.q;
    }
    __syncwarp();
}

// Phase 2 (the module of order p+2): the second solve of the HOErrorControl estimate.
BVP_DEV void polish_instance(const Args& a, Inst& I) {
    const InstState s = a.st[I.q];
    I.N = s.N;
    I.cur = s.cur;
    second_solve(a, I, false);
}

BVP_DEV void finish_instance(const Args& a, Inst& I, InstState& s);

BVP_DEV void solve_instance(const Args& a, Inst& I) {
    InstState s;
    // phase 1: the instance stopped after its Newton solve (and defect) of this round for the
    // MIRK(p+2) solve, which left its nodes in buffer cur^1
    bool resumed = GLOBAL_CTL && a.phase == 1;
    if (resumed) {
        s = a.st[I.q];
        I.N = s.N;
        I.cur = s.cur;
    } else {
        s.retcode = RET_FAILURE; s.newton_iters = 0; s.rounds = 0; s.flags = 0;
        s.defect = __longlong_as_double(0x7ff8000000000000LL);
        s.resid = s.defect;
        s.global_err = s.defect;
        init_instance(a, I);
    }
    int info_ok = 1;
    bool maxed = false;
    while (true) {
        double error_norm = 2 * a.abstol;
        bool ok = true;
        int sel = SEL_DEFECT;
        if (!resumed) {
            ++s.rounds;
            mesh_setup(a, I);
            const bool nl_ok = newton(a, I, s);
            if (!a.adaptive) { s.retcode = nl_ok ? RET_SUCCESS : RET_FAILURE; info_ok = nl_ok; break; }
            ok = nl_ok;
            if constexpr (!GLOBAL_CTL) {
                if (ok) {
                    error_norm = defect(a, I);
                    s.defect = error_norm;
                    ok = !(error_norm > a.defect_threshold) && !isnan(error_norm);
                }
            } else if (ok) {
                // error_estimate! for the controller (adaptivity.jl:361-503)
                const int ctl = a.controller;
                if (ctl != CTL_GLOBAL) {
                    error_norm = defect(a, I);
                    s.defect = error_norm;
                    if (ctl != CTL_HYBRID) ok = !(error_norm > a.defect_threshold);
                }
                // SequentialErrorControl takes the global estimate once the defect is within
                // abstol (464-482); HybridErrorControl ignores the defect threshold (485-503)
                const bool glob = ok && (ctl == CTL_GLOBAL || ctl == CTL_HYBRID ||
                                         (ctl == CTL_SEQUENTIAL && error_norm <= a.abstol));
                if (glob) {
                    if (a.global_method == GLOBAL_HO) {
                        pause_instance(a, I, s);
                        return;
                    }
                    if (!second_solve(a, I, true)) {
                        s.flags |= 2;
                        error_norm = __longlong_as_double(0x7ff8000000000000LL);
                    } else {
                        const double gn = global_finish(a, I, 2);
                        s.global_err = gn;
                        error_norm = ctl == CTL_HYBRID ? a.hybrid_de * error_norm + a.hybrid_ge * gn : gn;
                        sel = ctl == CTL_GLOBAL ? SEL_GLOBAL_P : (ctl == CTL_HYBRID ? SEL_HYBRID : SEL_GLOBAL_P1);
                    }
                }
                // a norm that is not finite counts as a failed round, for every controller
                if (!isfinite(error_norm)) ok = false;
            }
        } else {
            resumed = false;
            const int ctl = a.controller;
            const double gn = global_finish(a, I, 1);
            s.global_err = gn;
            error_norm = ctl == CTL_HYBRID ? a.hybrid_de * s.defect + a.hybrid_ge * gn : gn;
            sel = ctl == CTL_GLOBAL ? SEL_GLOBAL_P : (ctl == CTL_HYBRID ? SEL_HYBRID : SEL_GLOBAL_P1);
            ok = isfinite(error_norm);
        }
        if (ok) {
            if (error_norm > a.abstol) {
                int newN = 0;
                const double rho = (GLOBAL_CTL && a.controller != CTL_DEFECT) ? 2.0 : 1.0;
                info_ok = mesh_selector(a, I, newN, sel, rho);
                if (info_ok) {
                    transfer(a, I, newN);
                    I.cur ^= 1;
                    I.N = newN;
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
                __syncwarp();
                info_ok = 1;
            }
        }
        if (!(info_ok && error_norm > a.abstol)) break;
        if (s.rounds >= a.max_rounds) { maxed = true; break; }
    }
    if (a.adaptive) s.retcode = maxed ? RET_MAXITERS : (info_ok ? RET_SUCCESS : RET_FAILURE);
    if (a.want_stages) finalize_stages(a, I);
    finish_instance(a, I, s);
}

// An instance's results: the final mesh and solution to buffer 0, its state record, and with
// host outputs its mesh, solution (and stages) to the pinned host arrays.
BVP_DEV void finish_instance(const Args& a, Inst& I, InstState& s) {
    // results live in buffer 0
    if (I.cur == 1) {
        double* m0 = mesh_of(a, I, 0); const double* m1 = mesh_of(a, I, 1);
        double* h0 = h_of(a, I, 0); const double* h1 = h_of(a, I, 1);
        double* y0 = y_of(a, I, 0); const double* y1 = y_of(a, I, 1);
        for (int k = lane_id(); k < I.N; k += 32) { m0[k] = m1[k]; if (k < I.N - 1) h0[k] = h1[k]; }
        for (int k = lane_id(); k < I.N * M; k += 32) y0[k] = y1[k];
        __syncwarp();
        I.cur = 0;
    }
    s.N = I.N;
    s.cur = 0;
    if (lane_id() == 0) a.st[I.q] = s;
    if (a.host_mesh) {
        // results to the host while the rest of the batch still runs: room from the cursor,
        // so the host's packed arrays hold instances in completion order
        unsigned long long start = 0;
        if (lane_id() == 0) start = atomicAdd(a.out_cursor, (unsigned long long)I.N);
        start = __shfl_sync(FULL, start, 0);
        const bool fits = (long long)start + I.N <= a.host_cap;
        if (fits) {
            const double* m0 = mesh_of(a, I, 0);
            const double* y0 = y_of(a, I, 0);
            for (int k = lane_id(); k < I.N; k += 32) a.host_mesh[start + k] = m0[k];
            for (int k = lane_id(); k < I.N * M; k += 32) a.host_y[start * M + k] = y0[k];
            if (a.want_stages && a.host_K) {
                for (int k = lane_id(); k < (I.N - 1) * S * M; k += 32)
                    a.host_K[start * S * M + k] = a.K[I.nb * S * M + k];
                for (int k = lane_id(); k < (I.N - 1) * NSXA * M; k += 32)
                    a.host_KI[start * NSXA * M + k] = a.KI[I.nb * NSXA * M + k];
            }
        }
        if (lane_id() == 0) {
            a.host_start[I.q] = fits ? (long long)start : -1;
            a.host_st[I.q] = s;
        }
    }
    __syncwarp();
}

#if BVP_FIRK
}  // namespace bvp
#include "bvp_firk.cuh"
namespace bvp {
#endif

BVP_DEV Inst make_inst(const Args& a, int q) {
    Inst I;
    I.q = q;
    I.nb = a.node_off[q];
    I.cap = a.cap[q];
    I.p = a.params + (long long)q * a.n_params;
    I.pj = a.params_j + (long long)q * a.n_params;
    I.scr = a.scr + (long long)q * SCRW;
    I.iscr = a.iscr + (long long)q * ISCRW;
    I.dns = nullptr;
    I.trec = nullptr;
    I.grp = nullptr;
    I.N = 0;
    I.cur = 0;
    return I;
}

}  // namespace bvp

// ---- kernels ---------------------------------------------------------------------------------
// Persistent fused solve: each warp repeatedly takes the next instance from the work
// counter and runs its complete adaptive solve.
// Per-warp scratch in shared memory when it fits (it is read back right after being
// written, by other lanes of the warp); otherwise the global scratch arrays.
namespace bvp {
constexpr int WARPS_PER_BLOCK = GROUP_WARPS;
constexpr bool SCR_SMEM = WARPS_PER_BLOCK * (SCRW * 8 + ISCRW * 4) <= 40 * 1024;
constexpr int SM_SCRW = SCR_SMEM ? SCRW : 1;
constexpr int SM_ISCRW = SCR_SMEM ? ISCRW : 1;
constexpr int SM_DNS = SMEM_DENSE ? NDENSE * DLD : 1;
constexpr bool TREC_SMEM = WARPS_PER_BLOCK * TREE_SLOTS * RECW * int(sizeof(JT)) <= 16 * 1024;
constexpr int SM_TREC = TREC_SMEM ? TREE_SLOTS * RECW : 1;

BVP_DEV void fused_body(const Args& a) {
    __shared__ double s_scr[WARPS_PER_BLOCK][SM_SCRW];
    __shared__ int s_iscr[WARPS_PER_BLOCK][SM_ISCRW];
    __shared__ JT s_dns[WARPS_PER_BLOCK][SM_DNS];
    __shared__ JT s_trec[WARPS_PER_BLOCK][SM_TREC];
    __shared__ GroupShared s_grp;
    __shared__ int s_item;
    const int lane = lane_id();
    const int w = threadIdx.x >> 5;
    // block mode first: the first n_group positions of the order (the long meshes, as bvp_prep
    // placed them), one per block at a time from the second counter
    const int n_group = GROUP_OK ? a.work_counter[5] : 0;
    bool block_mode = GROUP_OK && n_group > 0;
    // warp mode. The static deal (blocks b and b + S share an SM when the grid fills S SMs a
    // block at a time) only when every warp starts together, without block-mode work
    const bool deal = a.deal_sms > 0 && n_group == 0;
    int k_first = -1;
    if (deal) {
        const int S = a.deal_sms, sm = int(blockIdx.x) % S, j = (int(blockIdx.x) / S) * WARPS_PER_BLOCK + w;
        k_first = j * S + ((j & 1) ? S - 1 - sm : sm);
    }
    while (true) {
        int k = -1;
        if (GROUP_OK && block_mode) {
            if (threadIdx.x == 0) s_item = atomicAdd(a.work_counter + 4, 1);
            group_bar();
            const int gi = s_item;
            if (gi >= n_group) {
                block_mode = false;
            } else if (w != 0) {
                group_helper(a, &s_grp, w);
                continue;
            } else {
                k = gi;
            }
        }
        const bool grp = k >= 0;
        if (!grp) {
            k = k_first;
            k_first = -1;
            if (k < 0) {
                if (lane == 0)
                    k = n_group + atomicAdd(a.work_counter, 1) + (deal ? WARPS_PER_BLOCK * int(gridDim.x) : 0);
                k = __shfl_sync(FULL, k, 0);
            }
            if (k >= a.n_inst) break;
        }
        Inst I = make_inst(a, a.order[k]);
        if (SCR_SMEM) { I.scr = s_scr[w]; I.iscr = s_iscr[w]; }
        I.dns = s_dns[w];
        if (TREC_SMEM) I.trec = s_trec[w];
        if (GROUP_OK && grp) I.grp = &s_grp;
        if (GLOBAL_CTL && a.phase == 2) {
            polish_instance(a, I);
            continue;
        }
        const long long c0 = a.inst_cost ? clock64() : 0;
#if BVP_FIRK
        firk_solve_instance(a, I);
#else
        solve_instance(a, I);
#endif
        if (a.inst_cost && lane == 0) a.inst_cost[I.q] = float(clock64() - c0) * (1.0f / 2000.0f);
        if (GROUP_OK && grp) {
            // release the helpers
            if (lane == 0) s_grp.cmd = CMD_EXIT;
            group_bar();
        }
    }
}
}  // namespace bvp

// The same kernel for three register budgets: 4, 3 or 2 resident blocks of 4 warps per SM
// (128, 168 and 255 registers per thread at most). More resident warps hide more latency;
// fewer leave each warp the registers its solve needs without spilling (the pendulum's MIRK4
// solve takes 156: 198 bytes of spills per thread at 4 blocks, none at 3). The handle's
// autotuner picks one by timing them on its own batches.
// The builds with the error controllers and the FIRK schemes are not tuned: one kernel each, at
// 3 blocks per SM (which keeps the MIRK4 pendulum solve's registers without spills), and the
// module that only runs HOErrorControl's MIRK(p+2) solves (BVP_POLISH_ONLY) has nothing else.
#if BVP_GLOBAL_CTL || BVP_FIRK
extern "C" __global__ void __launch_bounds__(128, 3) bvp_solve_fused(const bvp::Args a) { bvp::fused_body(a); }
#elif BVP_BLOCK_MODE
// the block-mode module: one launch shape, 2 blocks per SM (the fastest of the three on the
// long meshes it is for)
extern "C" __global__ void __launch_bounds__(128, 2) bvp_solve_fused(const bvp::Args a) { bvp::fused_body(a); }
#else
extern "C" __global__ void __launch_bounds__(128, 4) bvp_solve_fused(const bvp::Args a) { bvp::fused_body(a); }
extern "C" __global__ void __launch_bounds__(128, 3) bvp_solve_fused_b3(const bvp::Args a) { bvp::fused_body(a); }
extern "C" __global__ void __launch_bounds__(128, 2) bvp_solve_fused_b2(const bvp::Args a) { bvp::fused_body(a); }
#endif
#if !BVP_POLISH_ONLY && !BVP_FIRK && !BVP_BLOCK_MODE

// Stage kernels on caller-provided (mesh, y) in buffer 0 with N = st[q].N. Used by the
// per-kernel parity tests; stage: 0 residual (F, K, BC residual), 1 Jacobian blocks,
// 2 Newton direction (residual + Jacobian + factor/solve), 3 defect (residual + defect).
// The scratch ends in the global arrays for the host to read.
extern "C" __global__ void __launch_bounds__(128) bvp_stage(const bvp::Args a, int stage, double* out_norm) {
    __shared__ double s_scr[bvp::WARPS_PER_BLOCK][bvp::SM_SCRW];
    __shared__ int s_iscr[bvp::WARPS_PER_BLOCK][bvp::SM_ISCRW];
    __shared__ bvp::JT s_dns[bvp::WARPS_PER_BLOCK][bvp::SM_DNS];
    __shared__ bvp::JT s_trec[bvp::WARPS_PER_BLOCK][bvp::SM_TREC];
    const int lane = bvp::lane_id();
    const int w = threadIdx.x >> 5;
    while (true) {
        int k = 0;
        if (lane == 0) k = atomicAdd(a.work_counter, 1);
        k = __shfl_sync(bvp::FULL, k, 0);
        if (k >= a.n_inst) break;
        bvp::Inst I = bvp::make_inst(a, a.order[k]);
        if (bvp::TREC_SMEM) I.trec = s_trec[w];
        double* g_scr = I.scr;
        int* g_iscr = I.iscr;
        if (bvp::SCR_SMEM) { I.scr = s_scr[w]; I.iscr = s_iscr[w]; }
        I.dns = s_dns[w];
        I.N = a.st[I.q].N;
        I.cur = 0;
        bvp::mesh_setup(a, I);
        bvp::refresh_yj(a, I);
        double v = bvp::residual<double>(a, I);
        if (stage >= 1 && stage <= 2) bvp::jacobian(a, I);  // stage 2's solve recomputes the same blocks
        if (stage == 2) v = bvp::linear_solve(a, I) ? 0.0 : 1.0;
        if (stage == 3) v = bvp::defect(a, I);
        if (lane == 0) out_norm[I.q] = v;
        __syncwarp();
        if (bvp::SCR_SMEM) {
            for (int q = lane; q < bvp::SCRW; q += 32) g_scr[q] = I.scr[q];
            for (int q = lane; q < bvp::ISCRW; q += 32) g_iscr[q] = I.iscr[q];
        }
        __syncwarp();
    }
}
#endif  // !BVP_POLISH_ONLY && !BVP_FIRK && !BVP_BLOCK_MODE

// Copy the results of every instance (buffer 0) into packed host-bound arrays.
// out_off has n_inst + 1 entries (bvp_out_offsets); the outputs hold cap points: a batch
// whose packed size exceeds cap writes nothing (the host grows the outputs and packs again).
extern "C" __global__ void bvp_pack(const bvp::Args a, const long long* out_off, long long cap, double* mesh_out,
                                    double* y_out, int want_stages, double* K_out, double* KI_out) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = bvp::lane_id();
    if (warp >= a.n_inst || out_off[a.n_inst] > cap) return;
    const int q = warp;
    const long long nb = a.node_off[q];
    const int N = a.st[q].N;
    const long long o = out_off[q];
    for (int k = lane; k < N; k += 32) mesh_out[o + k] = a.mesh[nb + k];
    for (int k = lane; k < N * bvp::M; k += 32) y_out[o * bvp::M + k] = a.y[nb * bvp::M + k];
    if (want_stages) {
        // stages are per interval; packed at the instance's node offset (N-1 used)
        for (int k = lane; k < (N - 1) * bvp::S * bvp::M; k += 32)
            K_out[o * bvp::S * bvp::M + k] = a.K[nb * bvp::S * bvp::M + k];
        for (int k = lane; k < (N - 1) * bvp::NSXA * bvp::M; k += 32)
            KI_out[o * bvp::NSXA * bvp::M + k] = a.KI[nb * bvp::NSXA * bvp::M + k];
    }
}

// Packed-output offsets of the last solve: the exclusive prefix sum of every instance's final
// point count (n + 1 entries, into d_off and the host-mapped h_off) and a copy of the
// per-instance states into host-mapped h_st. One block.
extern "C" __global__ void __launch_bounds__(1024) bvp_out_offsets(int n, const BvpInstState* st, long long* d_off,
                                                                   long long* h_off, BvpInstState* h_st) {
    __shared__ long long wsum[32];
    __shared__ long long carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += blockDim.x) {
        const int q = base + tid;
        long long c = 0;
        if (q < n) {
            const BvpInstState sq = st[q];
            h_st[q] = sq;
            c = sq.N;
        }
        long long v = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(bvp::FULL, v, o);
            if (lane >= o) v += t;
        }
        if (lane == 31) wsum[warp] = v;
        __syncthreads();
        if (warp == 0) {
            long long w = (lane < int(blockDim.x >> 5)) ? wsum[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long t = __shfl_up_sync(bvp::FULL, w, o);
                if (lane >= o) w += t;
            }
            wsum[lane] = w;
        }
        __syncthreads();
        const long long excl = carry + (warp > 0 ? wsum[warp - 1] : 0) + v - c;
        if (q < n) { d_off[q] = excl; h_off[q] = excl; }
        __syncthreads();
        if (tid == 0) carry += wsum[31];
        __syncthreads();
    }
    if (tid == 0) { d_off[n] = carry; h_off[n] = carry; }
}

#if !BVP_POLISH_ONLY && !BVP_FIRK && !BVP_BLOCK_MODE

// Dense output of the last solve (needs want_stages): u(t) or u'(t) at nq query times per
// instance through the MIRK interpolant (interpolation.jl:17-204: interval(mesh, t),
// τ = (t - t_i)/h_i, u = y_i + h Σ w_r(τ) K_r, u' = Σ w'_r(τ) K_r). One warp per instance,
// lanes over queries.
extern "C" __global__ void bvp_dense(const bvp::Args a, int nq, const double* tq, int deriv, double* out) {
    using namespace bvp;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = lane_id();
    if (warp >= a.n_inst) return;
    const int q = warp;
    const long long nb = a.node_off[q];
    const int N = a.st[q].N;
    const double* mesh = a.mesh + nb;
    const double* y = a.y + nb * M;
    for (int j = lane; j < nq; j += 32) {
        const double t = tq[(long long)q * nq + j];
        const int i = interval_of(mesh, N, t);
        const double dt = a.h[nb + i];
        double w[SS], wp[SS];
        interp_weights_rt((t - mesh[i]) / dt, w, wp);
        const double* wv = deriv ? wp : w;
        const double* Kg = a.K + (nb + i) * (S * M);
        const double* KIg = a.KI + (nb + i) * (NSXA * M);
        double* o = out + ((long long)q * nq + j) * M;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            double acc = Kg[m] * wv[0];
#pragma unroll
            for (int r = 1; r < S; ++r) acc += Kg[r * M + m] * wv[r];
#pragma unroll
            for (int qq = 0; qq < NSX; ++qq) acc += KIg[qq * M + m] * wv[S + qq];
            o[m] = deriv ? acc : acc * dt + y[i * M + m];
        }
    }
}

// Device-side layout constants, checked against the host's at handle creation.
#endif  // !BVP_POLISH_ONLY && !BVP_FIRK && !BVP_BLOCK_MODE

extern "C" __global__ void bvp_layout_probe(int* out) {
    out[0] = bvp::SCRW;
    out[1] = bvp::ISCRW;
    out[2] = bvp::EQW;
    out[3] = bvp::RECW;
    out[4] = int(sizeof(BvpArgs));
    out[5] = int(sizeof(BvpInstState));
    out[6] = bvp::NSXA;
    out[7] = bvp::S;
}

// Parameters in the Jacobian precision.
extern "C" __global__ void bvp_convert_params(const double* p, bvp::JT* pj, long long n) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        pj[k] = bvp::JT(p[k]);
}

// One block: node capacities (cap_scale max(n, max_sub) + 1; cap_scale 2 leaves room for the
// halved mesh of REErrorControl's second solve), their exclusive prefix sum (arena offsets),
// and the work order: coarsest initial mesh first. A coarse initial mesh is the
// likeliest to need further mesh rounds, each a new Newton solve, so those instances carry
// the longest chains of dependent work and start first; the single-round fine meshes fill in
// behind them and finish while the machine drains (measured on the 4096-instance pendulum
// batch: about 11% less time than largest-first).
extern "C" __global__ void __launch_bounds__(1024) bvp_prep(int n, const int* n_init, int max_sub, int cap_scale,
                                                            int* cap, long long* node_off, int* order, int* counter,
                                                            const float* cost_tab, int group_min) {
    constexpr int NB = 4096;            // sort keys of one class
    constexpr int NB2 = 2 * NB;         // block-mode instances' keys first, then the others'
    __shared__ int hist[NB2];
    __shared__ long long wsum[32];
    __shared__ long long carry;
    __shared__ int n_group;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k = tid; k < NB2; k += blockDim.x) hist[k] = 0;
    if (tid == 0) { carry = 0; n_group = 0; counter[0] = 0; counter[4] = 0; }
    __syncthreads();
    for (int base = 0; base < n; base += blockDim.x) {
        const int q = base + tid;
        long long c = 0;
        if (q < n) {
            const int ni = n_init[q];
            c = (long long)cap_scale * (ni > max_sub ? ni : max_sub) + 1;
            cap[q] = int(c);
        }
        long long v = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(bvp::FULL, v, o);
            if (lane >= o) v += t;
        }
        if (lane == 31) wsum[warp] = v;
        __syncthreads();
        if (warp == 0) {
            long long w = (lane < int(blockDim.x >> 5)) ? wsum[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long t = __shfl_up_sync(bvp::FULL, w, o);
                if (lane >= o) w += t;
            }
            wsum[lane] = w;
        }
        __syncthreads();
        const long long excl = carry + (warp > 0 ? wsum[warp - 1] : 0) + v - c;
        if (q < n) node_off[q] = excl;
        __syncthreads();
        if (tid == 0) carry += wsum[31];
        __syncthreads();
    }
    // sort key: the learned cost (longest first) when the handle has a cost table, else the
    // initial interval count (coarsest first)
    const float cmax = cost_tab ? cost_tab[BVP_COST_BUCKETS] : 0.0f;
    auto key_of = [&](int q) {
        const int ni = n_init[q];
        if (cmax > 0.0f) {
            const float c = cost_tab[min(ni >> 3, BVP_COST_BUCKETS - 1)];
            const int kq = int(fminf(fmaxf(c / cmax, 0.0f), 1.0f) * float(NB - 1));
            return NB - 1 - kq;
        }
        return ni < NB - 1 ? ni : NB - 1;
    };
    // block mode (group_min > 0): meshes of at least group_min intervals, sorted among
    // themselves the same way, ahead of the others; their count goes to counter[5]
    auto key2_of = [&](int q) {
        const bool grp = group_min > 0 && n_init[q] >= group_min;
        return (grp ? 0 : NB) + key_of(q);
    };
    for (int q = tid; q < n; q += blockDim.x) {
        const int k2 = key2_of(q);
        atomicAdd(&hist[k2], 1);
        if (k2 < NB) atomicAdd(&n_group, 1);
    }
    __syncthreads();
    if (tid == 0) counter[5] = n_group;
    {
        // exclusive scan of the histogram by the whole block: each thread a run of NB2 / 1024
        // bins, a warp scan of the run sums, then the warps' totals
        constexpr int PER = NB2 / 1024;
        int v[PER];
        int s = 0;
#pragma unroll
        for (int k = 0; k < PER; ++k) { v[k] = hist[tid * PER + k]; s += v[k]; }
        int incl = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(bvp::FULL, incl, o);
            if (lane >= o) incl += t;
        }
        __shared__ int wtot[32];
        if (lane == 31) wtot[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            int w = wtot[lane], wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(bvp::FULL, wi, o);
                if (lane >= o) wi += t;
            }
            wtot[lane] = wi - w;
        }
        __syncthreads();
        int run = wtot[warp] + incl - s;
#pragma unroll
        for (int k = 0; k < PER; ++k) { hist[tid * PER + k] = run; run += v[k]; }
    }
    __syncthreads();
    for (int q = tid; q < n; q += blockDim.x) {
        const int pos = atomicAdd(&hist[key2_of(q)], 1);
        order[pos] = q;
    }
}

// The work-order autotuner's update after a solve that recorded its instances' times: the
// longest time per initial-size bucket, blended half and half with the table's earlier value
// where the table has one; a bucket without instances takes the value of the nearest measured
// bucket below it (above it, before the first); the largest value goes to
// tab[BVP_COST_BUCKETS]. The longest, not the mean: a bucket whose instances mostly need one
// mesh round but a few need two holds those few among the batch's longest solves, and
// longest-first scheduling must start them early (on the pendulum batch, 7% of the
// 64-80-interval meshes take a second round; ordered by the mean they started last and
// ended 60 us after everything else). One block.
extern "C" __global__ void __launch_bounds__(1024) bvp_learn_costs(int n, const int* n_init, const float* cost,
                                                                   float* tab, int blend) {
    __shared__ float s_sum[BVP_COST_BUCKETS];
    __shared__ int s_cnt[BVP_COST_BUCKETS];
    const int tid = threadIdx.x;
    for (int b = tid; b < BVP_COST_BUCKETS; b += blockDim.x) { s_sum[b] = 0.0f; s_cnt[b] = 0; }
    __syncthreads();
    for (int q = tid; q < n; q += blockDim.x) {
        const int b = min(n_init[q] >> 3, BVP_COST_BUCKETS - 1);
        // non-negative floats order as their bit patterns
        atomicMax(reinterpret_cast<int*>(&s_sum[b]), __float_as_int(fmaxf(cost[q], 0.0f)));
        atomicAdd(&s_cnt[b], 1);
    }
    __syncthreads();
    for (int b = tid; b < BVP_COST_BUCKETS; b += blockDim.x) {
        if (s_cnt[b] > 0) {
            const float m = s_sum[b];
            s_sum[b] = (blend && tab[b] > 0.0f) ? 0.5f * (tab[b] + m) : m;
        } else {
            s_sum[b] = blend ? tab[b] : 0.0f;
            s_cnt[b] = s_sum[b] > 0.0f ? 1 : 0;
        }
    }
    __syncthreads();
    if (tid == 0) {
        float last = 0.0f, mx = 0.0f;
        int seen = -1;
        for (int b = 0; b < BVP_COST_BUCKETS; ++b) {
            if (s_cnt[b] > 0) {
                if (seen < 0) for (int c = 0; c < b; ++c) s_sum[c] = s_sum[b];   // leading gap
                last = s_sum[b];
                seen = b;
                mx = fmaxf(mx, last);
            } else if (seen >= 0) {
                s_sum[b] = last;                                              // trailing and inner gaps
            }
        }
        tab[BVP_COST_BUCKETS] = mx;
    }
    __syncthreads();
    for (int b = tid; b < BVP_COST_BUCKETS; b += blockDim.x) tab[b] = s_sum[b];
}
