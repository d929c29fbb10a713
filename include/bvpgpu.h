/* bvpgpu.h — C ABI of the GB300 batched MIRK boundary-value solver (libbvpgpu.so).
 *
 * Plain C types only: pointers, sizes and enums. The library owns all device memory,
 * the JIT-compiled kernels and the CUDA stream; the caller owns every host buffer it
 * passes in. One handle per host thread; calls on a handle are stream-ordered and
 * return after their results are on the host (except bvp_solve_batch_device).
 *
 * Each entry point names the reference interface it stands in for (paths relative to
 * the SciML/BoundaryValueDiffEq.jl project).
 */
#ifndef BVPGPU_H
#define BVPGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    BVP_OK = 0,
    BVP_ERR_INVALID = 1,   /* bad argument: the reference raises ArgumentError (e.g. dt <= 0, Core/src/utils.jl:354) */
    BVP_ERR_COMPILE = 2,   /* the problem source did not compile (NVRTC log in bvp_last_error) */
    BVP_ERR_CUDA = 3,      /* a CUDA runtime call failed */
    BVP_ERR_NOMEM = 4,     /* device or pinned host allocation failed */
    BVP_ERR_STATE = 5,     /* no results available yet / handle misuse */
    BVP_ERR_TOO_LARGE = 6  /* the call's work does not fit its fixed static scratch (bvp_mlp_forward_noalloc) */
} bvp_status;

/* Per-instance return codes, the reference's ReturnCode values of solve! (mirk.jl:293-331). */
typedef enum {
    BVP_RET_SUCCESS = 0,
    BVP_RET_FAILURE = 1,   /* Newton failed beyond the mesh cap, or mesh selection exceeded max_subintervals */
    BVP_RET_MAXITERS = 2   /* outer (mesh) round cap reached */
} bvp_retcode;

/* Problem description (the shape part of a BVProblem / TwoPointBVProblem).
 * Standard problems evaluate the BC on u(bc_t[k]) as the reference's EvalSol does
 * (lib/BoundaryValueDiffEqMIRK/src/interpolation.jl:214-242); two-point problems give La
 * residuals at t0 and Lb at t1 (lib/BoundaryValueDiffEqCore/src/utils.jl:157-181). */
typedef struct {
    int32_t M;            /* state dimension 1..32: up to 8 one warp solves an instance; above 8
                             the larger-state kernels run (two-point BCs, bvp_solve_batch only) */
    int32_t n_params;     /* parameters per instance */
    int32_t twopoint;     /* 0 standard, 1 two-point */
    int32_t n_bc_pts;     /* standard: number of evaluation times (1..16) */
    int32_t La, Lb;       /* two-point: residual counts, La + Lb == M */
    double bc_t[16];      /* standard: evaluation times */
} bvp_problem_desc;

/* Solver options; defaults (bvp_default_options) are the reference's:
 * abstol 1e-6, adaptive, DefectControl(defect_threshold = 0.1), max_num_subintervals 3000
 * (lib/BoundaryValueDiffEqMIRK/src/mirk.jl:49-53, algorithms.jl:55-61,
 *  lib/BoundaryValueDiffEqCore/src/calc_errors.jl:54-60). */
typedef struct {
    int32_t order;                /* MIRK order: 2, 3, 4, 5 or 6 (see mirk6i) */
    int32_t adaptive;             /* 1: defect-controlled mesh refinement */
    int32_t max_subintervals;     /* mesh cap (reference default 3000) */
    int32_t max_newton;           /* Newton iterations per attempt */
    int32_t max_rounds;           /* cap on outer mesh rounds (the reference has none) */
    int32_t transfer_inplace;     /* 1: the reference's in-place solution transfer (default) */
    int32_t bc_jac_exact;         /* 0: the reference's BC Jacobian (stages held fixed), 1: exact */
    int32_t linesearch_fallback;  /* 1: retry a failed Newton with backtracking */
    int32_t stall_steps;          /* Newton stops after this many non-improving steps */
    int32_t jac_precision;        /* 32: FP32 Jacobian blocks and factorisation, 64: FP64 */
    int32_t want_stages;          /* 1: keep K and the interpolant stages for dense output */
    int32_t fp32_phase;           /* 1: Newton iterates on an FP32 residual down to 100 abstol
                                     (jac_precision 32 only); the final steps and every
                                     convergence decision use the FP64 residual */
    double abstol;
    double defect_threshold;
    double divergence_factor;     /* Newton stops when ||F|| exceeds this times its start */
    int32_t mirk6i;               /* 1 with order 6: MIRK6I, the order-6 scheme with Lobatto-point
                                     stages and its own interpolant (mirk_tableaus.jl:154-194,
                                     interpolation.jl:583-693; BoundaryValueDiffEqMIRK.jl:179) */
    int32_t controller;           /* bvp_controller: the __init kwarg `controller`
                                     (Core/src/calc_errors.jl:54-139); M <= 8 */
    int32_t global_method;        /* bvp_global_method of the global estimate (the controller's
                                     GlobalErrorControl(method = ...)) */
    double hybrid_de, hybrid_ge;  /* HybridErrorControl(DE, GE) */
    int32_t firk;                 /* 0: MIRK (order, mirk6i). A FIRK scheme in the expanded form
                                     (lib/BoundaryValueDiffEqFIRK): 1 RadauIIa, 2 LobattoIIIa,
                                     3 LobattoIIIb, 4 LobattoIIIc, with firk_stages stages (RadauIIa
                                     1, 2, 3, 5, 7; Lobatto 2..5). FP64 throughout, DefectControl,
                                     M <= 8, standard BCs at the tspan's ends or two-point BCs, no
                                     singular term and no stage output */
    int32_t firk_stages;
    int32_t block_min;            /* meshes of at least this many initial intervals are solved by a
                                     whole 128-thread block instead of one warp: the residuals and
                                     the defect spread over 128 lanes, the rest of the solve on the
                                     block's first warp; the results are the same. 0: the library's
                                     threshold (512 intervals); -1: never. The defect-controlled
                                     MIRK path only (M <= 8) */
} bvp_options;

/* Error controllers (lib/BoundaryValueDiffEqCore/src/calc_errors.jl:54-139, the error
 * estimates of lib/BoundaryValueDiffEqMIRK/src/adaptivity.jl:361-567). With HOErrorControl the
 * solve synchronises with the host once per mesh round (the MIRK(p+2) solves run between
 * launches), also in bvp_solve_batch_device. */
typedef enum {
    BVP_CTL_DEFECT = 0,      /* DefectControl: the defect of the continuous extension (default) */
    BVP_CTL_GLOBAL = 1,      /* GlobalErrorControl: the global error estimate alone */
    BVP_CTL_SEQUENTIAL = 2,  /* SequentialErrorControl: the defect, then the global estimate
                                once the defect is within abstol */
    BVP_CTL_HYBRID = 3       /* HybridErrorControl: DE * defect + GE * global */
} bvp_controller;

typedef enum {
    BVP_GLOBAL_HO = 0,       /* HOErrorControl: MIRK(p+2) on the same mesh (orders 2, 3, 4) */
    BVP_GLOBAL_RE = 1        /* REErrorControl: Richardson extrapolation from the halved mesh */
} bvp_global_method;

/* Per-instance outputs of a batch (caller-owned arrays of n_inst entries; any may be NULL). */
typedef struct {
    int32_t* retcode;
    int32_t* n_nodes;       /* final mesh points */
    int32_t* newton_iters;  /* Newton iterations over all rounds */
    int32_t* rounds;        /* outer mesh rounds */
    double* defect;         /* last defect norm */
    double* resid;          /* last ||F||_inf */
    double* global_err;     /* last global error estimate (controllers other than DefectControl) */
} bvp_results;

typedef struct bvp_handle_s bvp_handle;

/* Defaults of MIRKn() + __init kwargs (algorithms.jl:55-61, mirk.jl:49-53). */
void bvp_default_options(bvp_options* opt);

/* Setup: replaces SciMLBase.__init(prob::BVProblem, alg::AbstractMIRK; ...)
 * (lib/BoundaryValueDiffEqMIRK/src/mirk.jl:49-265). The problem source (f and bc as
 * BVP_F / BVP_BC or BVP_BCA + BVP_BCB bodies) is JIT-compiled once for sm_103a. */
bvp_status bvp_create(const bvp_problem_desc* desc, const char* source, const bvp_options* opt,
                      bvp_handle** out);

/* Batched solve: replaces SciMLBase.solve!(cache::MIRKCache) (mirk.jl:286-332) applied to
 * every trajectory of an EnsembleProblem (test/Core/ensemble_tests.jl:20-38).
 *   params      n_inst x n_params (row-major)
 *   n_intervals initial uniform mesh sizes, cld(t1 - t0, dt) (Core/src/utils.jl:349-363)
 *   tspans      n_inst x 2 (t0 < t1)
 *   y0_mode 0:  y0 is n_inst x M, copied to every mesh point (Core/src/utils.jl:766-769)
 *   y0_mode 1:  y0 holds (n_intervals[i]+1) x M guesses per instance, packed in order
 *               (the vector-of-arrays initial guess, Core/src/utils.jl:750-765)
 * Results stay in the handle until the next solve (bvp_get_solution / bvp_get_packed). */
bvp_status bvp_solve_batch(bvp_handle* h, int32_t n_inst, const double* params,
                           const int32_t* n_intervals, const double* tspans, int32_t y0_mode,
                           const double* y0, bvp_results* out);

/* Same solve with inputs already in device memory (device pointers; y0_off is the
 * per-instance offset, in M-vectors, for y0_mode 1, else NULL). max_intervals bounds
 * n_intervals. Runs on the handle's stream and returns without synchronising; results
 * stay on the device (read them with bvp_fetch_results). For state dimensions above 8 (the
 * host-driven path) the inputs are read back on the handle's stream and the call returns
 * after the solve; bvp_fetch_results reads the results the same way. */
bvp_status bvp_solve_batch_device(bvp_handle* h, int32_t n_inst, const double* d_params,
                                  const int32_t* d_n_intervals, const double* d_tspans,
                                  int32_t y0_mode, const double* d_y0, const int64_t* d_y0_off,
                                  int32_t max_intervals);

/* bvp_solve_batch_device with the initial guess given on a uniform grid of n_grid points
 * over each instance's tspan (d_grid: n_inst x n_grid x M, FP32, e.g. a surrogate's output),
 * resampled linearly onto the initial mesh inside the solve: the vector-of-arrays guess
 * form of __initial_guess_on_mesh (Core/src/utils.jl:750-765) without a separate pass. */
bvp_status bvp_solve_batch_device_grid(bvp_handle* h, int32_t n_inst, const double* d_params,
                                       const int32_t* d_n_intervals, const double* d_tspans,
                                       const float* d_grid, int32_t n_grid, int32_t max_intervals);

/* Synchronise and bring the results of the last solve to the host. */
bvp_status bvp_fetch_results(bvp_handle* h, bvp_results* out);

/* Final mesh and solution of instance `inst` of the last batch: the ODESolution the
 * reference builds (mirk.jl:324-331; Core/src/utils.jl:798-805). cap is the capacity of
 * mesh (points) and y (points x M). */
bvp_status bvp_get_solution(bvp_handle* h, int32_t inst, double* mesh, double* y, int32_t cap,
                            int32_t* n_nodes);

/* Pointers to the packed results of the last batch (valid until the next solve):
 * instance i occupies points offsets[i] .. offsets[i] + n_nodes[i] - 1 of mesh / y (x M),
 * offsets[n_inst] is the total; with want_stages, K (s x M per interval) and KI (extra
 * stages x M per interval) use the same offsets (interval k of instance q at offsets[q] + k).
 * The host calls write each instance's results as it finishes, so the instances' ranges
 * are in completion order, not instance order. */
bvp_status bvp_get_packed(bvp_handle* h, const int64_t** offsets, const double** mesh,
                          const double** y, const double** K, const double** KI);

/* One kernel stage on caller-given meshes and solutions (packed as bvp_get_packed):
 * stage 0 residual (__mirk_loss!, mirk.jl:471-494), 1 Jacobian blocks
 * (__mirk_mpoint_jacobian!, mirk.jl:824-838), 2 Newton direction (the linear solve of
 * NewtonRaphson), 3 defect (error_estimate!, adaptivity.jl:416-461). Outputs (any may be
 * NULL, packed by node offsets): norm (n_inst), F (collocation residual per interval,
 * x M), bc_res (n_inst x M), K (per interval, s x M), S and R (per interval, M x M),
 * delta (per point, x M), err (per interval). */
bvp_status bvp_eval_stage(bvp_handle* h, int32_t stage, int32_t n_inst, const double* params,
                          const int32_t* n_nodes, const double* mesh, const double* y,
                          double* norm, double* F, double* bc_res, double* K, double* S,
                          double* R, double* delta, double* err);

/* Dense output of the last solve (needs options.want_stages = 1): u(t) (deriv 0) or u'(t)
 * (deriv 1) at nq times per instance; tq is n_inst x nq, out n_inst x nq x M. Replaces
 * evaluating the returned solution, sol(t) / sol(t, Val{1})
 * (lib/BoundaryValueDiffEqMIRK/src/interpolation.jl:17-204). */
bvp_status bvp_dense_output(bvp_handle* h, int32_t nq, const double* tq, int32_t deriv, double* out);

/* ---- surrogate warm start --------------------------------------------------------------
 * A multilayer perceptron (GELU hidden layers, linear output) with BF16 weights and
 * activations and FP32 accumulation, trained and evaluated by the library's own tensor-core
 * kernels. It maps instance parameters to a solution guess on a fixed grid; the reference
 * has no counterpart: the guess stands in for the constant initial guess that __init copies
 * to every node (lib/BoundaryValueDiffEqCore/src/utils.jl:766-769) and enters the solve as
 * the reference's vector-of-arrays initial guess (utils.jl:750-765, y0_mode 1 above).
 * Parameters are packed as W_1 (w_0 x w_1, row-major), b_1, W_2, b_2, ... in FP32. */
typedef struct bvp_mlp_s bvp_mlp;

bvp_status bvp_mlp_create(int32_t n_layers, const int32_t* widths, bvp_mlp** out);
int64_t bvp_mlp_num_params(bvp_mlp* net);
bvp_status bvp_mlp_set_params(bvp_mlp* net, const float* params);
bvp_status bvp_mlp_get_params(bvp_mlp* net, float* params);
/* Input and output scaling applied inside the network: x_n = (x - in_mu) / in_sd on entry,
 * y = z out_sd + out_mu on exit; the training loss is the MSE of z against the scaled targets. */
bvp_status bvp_mlp_set_normalization(bvp_mlp* net, const float* in_mu, const float* in_sd,
                                     const float* out_mu, const float* out_sd);
/* y = net(x) for a batch (host arrays, batch x w_0 in, batch x w_L out). */
bvp_status bvp_mlp_forward(bvp_mlp* net, int32_t batch, const float* x, float* y);
/* Mean-squared-error loss of one batch and its gradient (packed like the parameters). */
bvp_status bvp_mlp_loss_grad(bvp_mlp* net, int32_t batch, const float* x, const float* t, float* loss,
                             float* grad);
/* Adam on minibatches drawn from (x, t) (n samples, host arrays); returns the mean loss of
 * the last epoch. */
bvp_status bvp_mlp_train(bvp_mlp* net, int32_t n, const float* x, const float* t, int32_t epochs,
                         int32_t batch, float lr, uint64_t seed, float* last_loss);
/* Device-pointer forward on the given stream (cudaStream_t as void*); no synchronisation. */
bvp_status bvp_mlp_forward_device(bvp_mlp* net, int32_t batch, const float* d_x, float* d_y, void* stream);
/* The forward of bvp_mlp_forward_device, with the same results, for callers that must not
 * allocate device memory during the call: a serving loop that runs under a fixed memory
 * budget, or code that enqueues work where cudaMalloc would synchronise the device. It has
 * no counterpart in the reference. A network every one of whose widths is at most 256 (and,
 * past the input, a multiple of 8) runs the single fused kernel bvp_mlp_forward_device runs
 * for it, which needs no scratch, for any batch. Any other network runs the layer-by-layer
 * kernels bvp_mlp_forward_device runs for it, on scratch (two BF16 activation buffers and
 * one FP32 pre-activation buffer of batch x widest-layer elements, each rounded up to 256
 * bytes) carved from one static device array of BVP_MLP_NOALLOC_SCRATCH_BYTES; a batch that
 * does not fit returns BVP_ERR_TOO_LARGE before any work (8 MiB holds 4096 rows of a
 * 256-wide network, 2048 of a 512-wide one). Nothing in the scratch needs to start at zero:
 * every element the call reads is written earlier in the same call. A null stream means the
 * network's own stream, as for bvp_mlp_forward_device. The first call on a device looks up
 * the array's address with that device current (module set-up) and caches it for the
 * process; make that first call before any stream capture. The cached address does not
 * survive cudaDeviceReset (the library does not see the reset; use a new process). The
 * scratch is shared by every call on a device: calls that overlap in time (different
 * streams or threads) race; calls on one stream are ordered and safe. Devices 0..63. */
#define BVP_MLP_NOALLOC_SCRATCH_BYTES (8u << 20)
bvp_status bvp_mlp_forward_noalloc(bvp_mlp* net, int32_t batch, const float* d_x, float* d_y, void* stream);
/* Resample guesses given on a uniform grid of n_grid points over each instance's tspan
 * (grid: n_inst x n_grid x M) onto each instance's uniform initial mesh of n_intervals[i]
 * intervals by linear interpolation, packed as y0_mode 1 expects. Device pointers; y0_off
 * (n_inst + 1 offsets, in M-vectors) is the packing. */
bvp_status bvp_resample_guess_device(int32_t n_inst, int32_t n_grid, int32_t M, const float* d_grid,
                                     const double* d_tspans, const int32_t* d_n_intervals,
                                     const int64_t* d_y0_off, double* d_y0, void* stream);
void bvp_mlp_destroy(bvp_mlp* net);

/* Surrogate-warm batched solve: the network maps each instance's n_features features to a
 * guess on n_grid uniform points of its tspan (output width n_grid x M), the guess is
 * resampled onto the instance's initial mesh and the batch is solved from it; instances that
 * do not converge are solved again from y0_plain (n_inst x M, the constant guess) and
 * their results replace the warm attempt's. The plain MIRK Newton judges every result.
 * *n_fallback receives the number of re-solved instances. Results as bvp_solve_batch (the
 * stages are kept only when no instance needed the fallback). */
bvp_status bvp_solve_batch_warm(bvp_handle* h, bvp_mlp* net, int32_t n_inst, int32_t n_features,
                                const float* features, int32_t n_grid, const double* params,
                                const int32_t* n_intervals, const double* tspans,
                                const double* y0_plain, bvp_results* out, int32_t* n_fallback);

/* bvp_solve_batch_warm's solve on inputs already in device memory (d_features: n_inst x the
 * network's input width, FP32): the network's forward writes the grid guesses on a second
 * stream beside the solve's per-batch setup, and the solve waits for it. No plain-guess
 * fallback (the caller reads the retcodes with bvp_fetch_results and re-solves with
 * bvp_solve_batch_device); returns without synchronising. */
bvp_status bvp_solve_batch_device_warm(bvp_handle* h, bvp_mlp* net, int32_t n_inst, const float* d_features,
                                       int32_t n_grid, const double* d_params, const int32_t* d_n_intervals,
                                       const double* d_tspans, int32_t max_intervals);

/* Device time of the last solve's kernels in milliseconds (CUDA events on the handle's
 * stream): [0] whole solve, [1] fused solve kernel. */
bvp_status bvp_last_timing(bvp_handle* h, double* ms2);

/* Launch shapes the handle's autotuner picked (no reference counterpart: the reference runs
 * on the CPU). threads[0]: block size of the larger-state linear solve (0 until the first
 * Newton step of a state dimension above 8 has run). */
bvp_status bvp_get_tuning(bvp_handle* h, int32_t* threads);

/* The fused solve's launch shape (no reference counterpart): bvp_solve_fused is built for 4, 3
 * and 2 resident blocks of 4 warps per SM (register budgets of 128, 168 and 255 per thread).
 * The handle starts with 3; once its work order is learned, its next solves of one batch
 * shape (instance count, guess form; at least 256 instances) rotate through the three (a first,
 * untimed launch of each, then two timed solves each), and it keeps the fastest. *blocks_per_sm: the current choice (0 for
 * state dimensions above 8); *tuned (if not NULL): 1 once chosen; ms (if not NULL, 3 entries):
 * the candidates' mean kernel times so far. */
bvp_status bvp_get_fused_tuning(bvp_handle* h, int32_t* blocks_per_sm, int32_t* tuned, float* ms);

/* Block mode (bvp_options.block_min): *block_min the threshold in effect (0: block mode off,
 * also after its module failed to build, the reason then in bvp_last_error),
 * *last (if not NULL) 1 when the last solve ran the block-mode module (its largest initial mesh
 * reached the threshold; 2 resident blocks per SM, not tuned), else 0. No reference
 * counterpart: a performance report of this library, like bvp_get_fused_tuning. */
bvp_status bvp_get_block_mode(bvp_handle* h, int32_t* block_min, int32_t* last);

/* The fused solve's work order (no reference counterpart: the reference solves one problem at
 * a time). One warp carries one instance, so a batch ends when its slowest instances end; the
 * handle's first three solves of at least 256 instances record every instance's solve time
 * and fold it into a table of the longest time per initial-size bucket (initial intervals / 8, 512
 * buckets), and later solves start the instances the table predicts to be longest first
 * (before any table: coarsest initial mesh first). The order changes no result. *learned: 1
 * once the table exists; costs (if not NULL): the first n_costs of the 512 bucket costs and,
 * at index 512, their maximum (relative units). */
bvp_status bvp_get_work_order(bvp_handle* h, int32_t* learned, float* costs, int32_t n_costs);

/* The handle's CUDA stream (cudaStream_t as void*). */
void* bvp_stream(bvp_handle* h);

const char* bvp_last_error(bvp_handle* h);
void bvp_destroy(bvp_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* BVPGPU_H */
