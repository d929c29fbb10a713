// Structures shared by the host runtime and the JIT-compiled device code: the kernel
// argument block, the per-instance state record, and the scratch layout formulas.
// Both sides include this file so the launch ABI cannot drift. The device build defines
// BVP_JT_PTR as the Jacobian scalar type; the host sees those arrays as void*.
#pragma once

#ifndef BVP_JT_PTR
#define BVP_JT_PTR void
#endif

#ifdef __CUDACC_RTC__
typedef long long bvp_i64;
#else
#include <cstdint>
typedef long long bvp_i64;
#endif

struct BvpInstState {
    int N;              // current mesh points
    int cur;            // active ping-pong buffer
    int retcode;        // 0 success, 1 failure, 2 max rounds
    int newton_iters;
    int rounds;
    int flags;          // bit0: line-search fallback used, bit1: capacity guard hit
    double defect;
    double resid;
    double global_err;  // last global error estimate (global, sequential and hybrid controllers)
};

struct BvpArgs {
    int n_inst, n_params;
    int adaptive, max_sub, max_newton, max_rounds, stall_steps;
    int transfer_inplace, bc_jac_exact, linesearch, want_stages, y0_mode, fp32_phase;
    double abstol, defect_threshold, divergence_factor;
    double bc_t[16];
    bvp_i64 tot;                   // total node capacity (sum over instances)
    const int* order;              // work order (instance ids, coarsest initial mesh first)
    int* work_counter;
    int deal_sms;                  // > 0: the grid is that many SMs times the resident blocks per
                                   // SM, and each warp's first position of the order is dealt
                                   // statically, round j (the warp's index among its SM's warps)
                                   // taking positions j S .. j S + S - 1 over the SMs in a snake,
                                   // so the longest solves start spread over the SMs; the counter
                                   // deals the positions from 4 * gridDim.x on. 0: every position
                                   // comes from the counter
    const double* params;          // n_inst x n_params
    const BVP_JT_PTR* params_j;    // same, in the Jacobian precision
    const int* n_init;             // initial interval counts
    const double* tspans;          // n_inst x 2
    const double* y0;              // y0_mode 0: n_inst x M; 1: packed per-node guesses (2: y0_grid)
    const bvp_i64* y0_off;         // y0_mode 1: per-instance offsets (in M-vectors)
    const float* y0_grid;          // y0_mode 2: n_inst x n_grid x M guesses on uniform grids
    int n_grid;
    const bvp_i64* node_off;       // per-instance node offset into the arena
    const int* cap;                // per-instance node capacity
    double* mesh;                  // [2][tot]
    double* h;                     // [2][tot]
    double* y;                     // [2][tot][M]
    double* ybak;                  // [tot][M]
    double* ybase;                 // [tot][M]
    double* K;                     // [tot][S][M]
    double* KI;                    // [tot][NSXA][M]
    double* F;                     // [tot][M]  collocation residual of interval i
    double* err;                   // [tot]
    double* inc;                   // [tot][M]
    int* iold;                     // [tot]
    BVP_JT_PTR* Sb;                // [tot][M][M]
    BVP_JT_PTR* Rb;                // [tot][M][M]
    BVP_JT_PTR* rec;               // [tot][RECW]
    BVP_JT_PTR* delta;             // [tot][M]
    BVP_JT_PTR* yj;                // [tot][M]  current iterate in the Jacobian precision
    BVP_JT_PTR* Fj;                // [tot][M]  collocation residual in the Jacobian precision
    BVP_JT_PTR* tj;                // [tot]     mesh of the current round in the Jacobian precision
    BVP_JT_PTR* hj;                // [tot]     its spacings in the Jacobian precision
    double* scr;                   // per-instance scratch, SCRW doubles each
    int* iscr;                     // per-instance int scratch, ISCRW ints each
    BvpInstState* st;
    // results straight to pinned host memory the device maps (null: results stay on the device):
    // each instance takes host_cap-bounded room from out_cursor when it finishes
    double* host_mesh;
    double* host_y;
    double* host_K;
    double* host_KI;
    bvp_i64* host_start;           // per instance: first point of its results, -1 when it did not fit
    BvpInstState* host_st;
    unsigned long long* out_cursor;
    bvp_i64 host_cap;              // points the host arrays hold
    float* inst_cost;              // per instance: solve time (SM cycles / 2000), recorded while
                                   // the handle learns its work order (null: not recorded)
    // error control (compiled in with BVP_GLOBAL_CTL): 0 DefectControl, 1 GlobalErrorControl,
    // 2 SequentialErrorControl, 3 HybridErrorControl; the global estimate by 0 HOErrorControl
    // (a MIRK(p+2) solve on the same mesh, in the module compiled for that order) or
    // 1 REErrorControl (the same method on the halved mesh)
    int controller, global_method;
    double hybrid_de, hybrid_ge;
    double* gerr;                  // [tot] per-interval global error estimates
    int phase;                     // 0 new solves; 1 resume after the MIRK(p+2) solve; 2 that solve
    int* pause_list;               // phase 0/1: instances stopping for the MIRK(p+2) solve, appended
    int* pause_count;              //   at *pause_count
    double* fx;                    // FIRK: [tot][FS M (M+1)] each interval's condensation record
};

// Work-order cost table of the fused solve: the longest solve time of the instances whose
// initial interval count falls in each bucket (n_init >> 3), learned from a handle's first solves.
#define BVP_COST_BUCKETS 512

// Launch arguments of the larger-state kernels (M > 8, bvp_large.cuh): one instance per CTA or
// per grid row, the Newton and mesh rounds driven from the host.
struct BvpLargeArgs {
    int n_inst, n_params, n_active;
    double alpha;                  // bl_update: y = ybase + alpha delta (alpha 0: y += delta)
    const int* active;             // instance ids taking part in this launch
    const double* params;
    const BVP_JT_PTR* params_j;
    const bvp_i64* node_off;
    const int* N;                  // current point count per instance
    double* mesh;                  // [2][tot]: current mesh in buffer 0, a new one in buffer 1
    double* h;                     // [2][tot]
    double* y;                     // [2][tot][M]
    double* ybase;                 // [tot][M]
    double* ybak;                  // [tot][M]
    double* K;                     // [tot][S][M]
    double* KI;                    // [tot][NSXA][M]
    double* F;                     // [tot][M]
    double* err;                   // [tot]
    double* inc;                   // [tot][M]
    int* iold;                     // [tot]
    double* bcres;                 // [n_inst][M]: La rows at t0, then Lb rows at t1
    BVP_JT_PTR* yj;                // [tot][M]
    BVP_JT_PTR* Sb;                // [tot][M][M]
    BVP_JT_PTR* Rb;                // [tot][M][M]
    BVP_JT_PTR* G;                 // [n_inst][2][M][M]: dbca/dy0 (rows 0..La-1), dbcb/dyN (rows La..M-1)
    BVP_JT_PTR* rec;               // [tot][3M^2 + M]
    BVP_JT_PTR* delta;             // [tot][M]
    unsigned long long* norm;      // [n_inst]: max |F| as the bits of a non-negative double
    double* sq;                    // [n_inst]: sum of F^2
    unsigned long long* dnorm;     // [n_inst]: defect norm bits
    int* bad;                      // [n_inst]: singular block in the last solve
    bvp_i64 tot;
    int transfer_inplace;
    const int* newN;               // bl_transfer: point count of the new mesh (buffer 1)
};

// Scratch layout as a function of (M, order, BC evaluation points, two-point, MIRK6I).
struct BvpLayout {
    int M, S, SS, NSX, NSXA, EQW, RECW, NBCB, KMAX, NDENSE;
    int SCR_BCRES, SCR_BCBLK, SCR_SEG, SCR_UA, SCR_BCW, SCRW;
    int ISCR_NK, ISCR_KEPT, ISCR_NB, ISCR_BNODE, ISCR_UNODE, ISCR_UIN, ISCR_LOFF, ISCRW;
};

#ifdef __CUDACC_RTC__
#define BVP_LAYOUT_FN __host__ __device__ inline
#else
#define BVP_LAYOUT_FN inline
#endif

BVP_LAYOUT_FN BvpLayout bvp_make_layout(int M, int order, int nbc, int twopoint, int mirk6i = 0) {
    BvpLayout L;
    L.M = M;
    L.S = order - 1;
    L.SS = (order == 2 || order == 3) ? 3 : (order == 4 ? 4 : (order == 5 ? 6 : (mirk6i ? 8 : 9)));
    L.NSX = L.SS - L.S;
    L.NSXA = L.NSX > 0 ? L.NSX : 1;
    L.EQW = 2 * M * M + M;
    L.RECW = 3 * M * M + M;
    L.NBCB = twopoint ? 2 : 2 * nbc;
    L.KMAX = 2 + L.NBCB;
    L.NDENSE = L.KMAX * M;
    L.SCR_BCRES = 0;
    L.SCR_BCBLK = L.SCR_BCRES + M;
    L.SCR_SEG = L.SCR_BCBLK + L.NBCB * M * M;
    L.SCR_UA = L.SCR_SEG + (L.KMAX - 1) * L.EQW;
    L.SCR_BCW = L.SCR_UA + (twopoint ? 2 : nbc) * M;
    L.SCRW = L.SCR_BCW + (twopoint ? 2 : nbc) * L.SS;
    L.ISCR_NK = 0;
    L.ISCR_KEPT = 1;
    L.ISCR_NB = L.ISCR_KEPT + L.KMAX;
    L.ISCR_BNODE = L.ISCR_NB + 1;
    L.ISCR_UNODE = L.ISCR_BNODE + L.NBCB;
    L.ISCR_UIN = L.ISCR_UNODE + (twopoint ? 2 : nbc);
    L.ISCR_LOFF = L.ISCR_UIN + (twopoint ? 2 : nbc);
    L.ISCRW = L.ISCR_LOFF + L.KMAX + 1;
    return L;
}
