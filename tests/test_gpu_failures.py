"""Failure paths of the batched solve against the oracle, made on the host side of the input
(no GPU fault is involved): the reference's outer loop halves the mesh and restarts from a
zero guess whenever Newton fails or the defect exceeds its threshold, and returns Failure once
the mesh would pass max_num_subintervals (mirk.jl:361-385, adaptivity.jl:49-73).

* an f that returns NaN for flagged instances (a NaN parameter) fails those instances only:
  their neighbours in the same batch are bit-identical to a batch without the flags;
* max_newton = 1 leaves Newton unconverged, so every instance halves to the mesh cap;
* max_rounds = 1 stops instances that need a second mesh round with MaxIters;
* a small max_subintervals turns refinements past the cap into Failure.
Retcodes, Newton counts, rounds and final meshes follow the oracle's in FP64 mode."""
import dataclasses

import numpy as np
import pytest

from oracle.oracle import Oracle, RET_SUCCESS, RET_FAILURE, RET_MAXITERS

pytestmark = pytest.mark.gpu


def _nanflag(problems):
    # the pendulum with a fourth parameter added to du[1]: 0 leaves it unchanged, NaN poisons f
    p = problems.PENDULUM
    src = p.source.replace("du[1] = -p[0] * sin(u[0]);", "du[1] = -p[0] * sin(u[0]) + p[3];")
    assert src != p.source
    return dataclasses.replace(p, name="pendulum_nanflag", n_params=4, source=src)


def _oracle(p):
    return Oracle(p.source, p.M, p.n_params, twopoint=p.twopoint, bc_t=p.bc_t, La=p.La, Lb=p.Lb)


def _batch(problems, n, seed):
    params, nint, tsp, y0 = problems.pendulum_family(n, seed=seed)
    return np.concatenate([params, np.zeros((n, 1))], axis=1), nint, tsp, y0


def _same_results(a, b, idx_a, idx_b):
    for ia, ib in zip(idx_a, idx_b):
        assert a.retcode[ia] == b.retcode[ib] and a.n_nodes[ia] == b.n_nodes[ib]
        assert a.newton_iters[ia] == b.newton_iters[ib] and a.rounds[ia] == b.rounds[ib]
        ma, ya = a.solution(ia)
        mb, yb = b.solution(ib)
        assert np.array_equal(ma, mb) and np.array_equal(ya, yb)


@pytest.mark.parametrize("jac_precision", [32, 64])
def test_nan_instances_fail_alone(pkg, problems, jac_precision):
    p = _nanflag(problems)
    params, nint, tsp, y0 = _batch(problems, 96, seed=31)
    flagged = np.arange(3, 96, 7)
    bad = params.copy()
    bad[flagged, 3] = np.nan
    sv = pkg.BatchSolver(p, order=4, jac_precision=jac_precision)
    res_bad = sv.solve(bad, nint, tsp, y0)
    res_ok = sv.solve(params, nint, tsp, y0)
    assert (res_bad.retcode[flagged] == RET_FAILURE).all()
    keep = np.setdiff1d(np.arange(96), flagged)
    assert (res_ok.retcode == RET_SUCCESS).all()
    _same_results(res_bad, res_ok, keep, keep)
    # the flagged instances ended at the mesh cap, as the oracle's do
    ref = _oracle(p).solve_batch(bad[flagged], nint[flagged], tsp[flagged], y0[flagged])
    assert (ref["retcode"] == RET_FAILURE).all()
    assert (res_bad.n_nodes[flagged] == ref["n_nodes"]).all()
    assert (res_bad.rounds[flagged] == ref["rounds"]).all()


def test_newton_cap_matches_oracle(pkg, problems):
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(64, seed=32)
    sv = pkg.BatchSolver(p, order=4, jac_precision=64, max_newton=1)
    res = sv.solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0, max_newton=1)
    assert (ref["retcode"] != RET_SUCCESS).any()
    assert (res.retcode == ref["retcode"]).all()
    assert (res.rounds == ref["rounds"]).all()
    assert (res.n_nodes == ref["n_nodes"]).all()
    assert (res.newton_iters == ref["newton_iters"]).mean() >= 0.95


def test_round_cap_gives_maxiters(pkg, problems):
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(128, seed=33)
    sv = pkg.BatchSolver(p, order=4, jac_precision=64, max_rounds=1)
    res = sv.solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0, max_rounds=1)
    assert (ref["retcode"] == RET_MAXITERS).any() and (ref["retcode"] == RET_SUCCESS).any()
    assert (res.retcode == ref["retcode"]).all()
    assert (res.rounds == 1).all()
    # instances that converged in one round carry the oracle's solution
    ok = ref["retcode"] == RET_SUCCESS
    for i in np.nonzero(ok)[0]:
        N = int(ref["n_nodes"][i])
        m, y = res.solution(i)
        assert len(m) == N and np.abs(y - ref["y"][i, :N]).max() <= 1e-6


def test_mesh_cap_failure_matches_oracle(pkg, problems):
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(128, seed=34, n_min=32, n_max=60)
    sv = pkg.BatchSolver(p, order=4, jac_precision=64, max_subintervals=64)
    res = sv.solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0, max_subintervals=64)
    assert (ref["retcode"] == RET_FAILURE).any() and (ref["retcode"] == RET_SUCCESS).any()
    assert (res.retcode == ref["retcode"]).mean() >= 0.99
    assert (res.n_nodes <= 65).all()
