"""Parity of the benchmark's own form against the oracle: the first 1024 instances of the
timed pendulum batch (pendulum_family(4096, seed=2024)), solved the way the benchmark solves
them (FP32 Jacobian and factorisation, FP32 Newton phase, surrogate-warm through
bvp_solve_batch_warm with the plain-guess fallback), and solved by the oracle from the same
initial guesses (the network's grid resampled onto each initial mesh, the reference's
vector-of-arrays guess).

The reference accepts the first Newton iterate with ||F||_inf <= abstol (mirk.jl:51), and with
its BC Jacobian that holds the interpolant's stages fixed (mirk.jl:565-572) the iteration
converges linearly at an interior BC point, so that iterate is not the discrete solution:
measured on this batch, the oracle's accepted iterates lie up to ~1e-5 from the exact root of
the collocation equations on their own meshes. A solver whose Newton path differs in its
rounding (the FP32 Jacobian) stops at a point that differs by about as much, and the defect
of that point, which picks the next mesh, differs with it. So in this form the contract is
accuracy plus agreement where the mesh sequences agree (the FP64 mode, which follows the
oracle's path, is held to identity in test_gpu_solve.py):
  * identical retcodes;
  * every GPU result passes the reference's acceptance tests evaluated in FP64 by the oracle
    (||F||_inf <= abstol, defect <= abstol) on its own mesh;
  * the errors against a tight solution of the same problem (the oracle at abstol 1e-10,
    MIRK6) are the oracle's own: at least 99% of instances within the oracle's error plus
    abstol, the largest and the median no larger than the oracle's (plus abstol, plus 10%);
  * the final mesh is the oracle's for at least 85% of instances (measured: 88%), and on those
    at least 98% agree within max(abstol, 1e-9 |u|) at every node (measured: 99%, median
    difference 4e-9).
The report printed (and written to $BVP_PARITY_REPORT) gives the measured figures.
"""
import json
import os

import numpy as np
import pytest

from oracle.oracle import Oracle, RET_SUCCESS

pytestmark = pytest.mark.gpu

GRID = 64


def test_timed_form_matches_oracle(pkg, problems):
    p = problems.PENDULUM
    sv_tr = pkg.BatchSolver(p, order=4, want_stages=1)
    tr_p, tr_n, tr_t, tr_y = problems.pendulum_family(16384, seed=2024 + 10000)
    sur = pkg.Surrogate(p, n_params_in=3, grid=GRID)
    X, T = sur.training_data(sv_tr, tr_p, tr_p, tr_n, tr_t, tr_y)
    sur.fit(X, T, epochs=40, batch=512, lr=2e-3)
    params, nint, tsp, y0 = problems.pendulum_family(4096, seed=2024)
    n = 1024
    params, nint, tsp, y0 = params[:n], nint[:n], tsp[:n], y0[:n]
    sv = pkg.BatchSolver(p, order=4)                   # the benchmark's options
    res, nfb = sv.solve_warm(sur.net, params, GRID, params, nint, tsp, y0)
    o = Oracle(p.source, p.M, p.n_params, bc_t=p.bc_t)
    guess = sur.guess(params, nint)
    ref = o.solve_batch(params, nint, tsp, guess, y0_mode=1)
    if nfb:
        # instances the warm attempt did not converge were solved again from the plain guess
        bad = np.nonzero(ref["retcode"] != RET_SUCCESS)[0]
        plain = o.solve_batch(params[bad], nint[bad], tsp[bad], y0[bad])
        for k, q in enumerate(bad):
            for key in ("retcode", "n_nodes", "newton_iters", "rounds"):
                ref[key][q] = plain[key][k]
            ref["mesh"][q] = plain["mesh"][k]
            ref["y"][q] = plain["y"][k]
    tight = o.solve_batch(params, nint, tsp, y0, order=6, abstol=1e-10, want_stages=True)
    assert (tight["retcode"] == RET_SUCCESS).all()
    assert (res.retcode == ref["retcode"]).all()
    same = np.zeros(n, bool)
    stats = {k: [] for k in ("err_gpu", "err_ref", "diff", "d_ref", "d_gpu", "excess")}
    for i in range(n):
        m, y = res.solution(i)
        nrm = o.residual(params[i], m, y)[2]
        assert nrm <= 1e-6 * (1 + 1e-6), (i, nrm)
        assert o.defect(params[i], m, y)[1] <= 1e-6 * (1 + 1e-3), i
        Nt = int(tight["n_nodes"][i])
        mt = tight["mesh"][i, :Nt]
        N = int(ref["n_nodes"][i])
        mr, yr = ref["mesh"][i, :N], ref["y"][i, :N]
        err_gpu = np.abs(y - o.interpolate(6, mt, tight["y"][i], tight["K"][i], tight["KI"][i], m)).max()
        err_ref = np.abs(yr - o.interpolate(6, mt, tight["y"][i], tight["K"][i], tight["KI"][i], mr)).max()
        stats["err_gpu"].append(err_gpu)
        stats["err_ref"].append(err_ref)
        if len(m) != N or np.abs(m - mr).max() > 1e-9:
            continue
        same[i] = True
        ystar = o.collocation_root(params[i], m, yr)
        d_ref, d_gpu = np.abs(yr - ystar).max(), np.abs(y - ystar).max()
        tol = max(1e-6, 1e-9 * np.abs(yr).max())
        diff = np.abs(y - yr).max()
        stats["diff"].append(diff)
        stats["d_ref"].append(d_ref)
        stats["d_gpu"].append(d_gpu)
        stats["excess"].append(diff - tol)
    q = {k: np.quantile(np.array(v), [0.5, 0.9, 0.99, 1.0]).tolist() for k, v in stats.items() if v}
    eg, er = np.array(stats["err_gpu"]), np.array(stats["err_ref"])
    summary = {"same_mesh": float(same.mean()), "within_tol_on_same_mesh": float((np.array(stats["excess"]) <= 0).mean()),
               "err_gpu_le_err_ref_plus_tol": float((eg <= er + 1e-6).mean()),
               "quantiles_50_90_99_100": q, "fallback": int(nfb)}
    print(json.dumps(summary))
    out = os.environ.get("BVP_PARITY_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(summary, f, indent=1)
    assert same.mean() >= 0.85, summary
    assert summary["within_tol_on_same_mesh"] >= 0.98, summary
    assert summary["err_gpu_le_err_ref_plus_tol"] >= 0.99, summary
    assert eg.max() <= er.max() + 1e-6, summary
    assert np.median(eg) <= 1.1 * np.median(er), summary
