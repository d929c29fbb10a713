"""The larger-state path (M > 8: csrc/bvp_large.cuh and the host-driven rounds) against the
oracle, on the coupled nonlinear n = 32 family u' = A u + tanh(B u) + c with separated
boundary conditions (16 components fixed at each end)."""
import numpy as np
import pytest

from oracle.oracle import Oracle, RET_SUCCESS

pytestmark = pytest.mark.gpu


def _oracle(p):
    return Oracle(p.source, p.M, p.n_params, twopoint=p.twopoint, bc_t=p.bc_t, La=p.La, Lb=p.Lb)


def _compare(res, ref, tol_rel, frac_tight=1.0):
    n = len(res.n_nodes)
    assert (res.retcode == ref["retcode"]).all(), (res.retcode, ref["retcode"])
    assert (res.n_nodes == ref["n_nodes"]).all(), (res.n_nodes, ref["n_nodes"])
    tight = []
    for i in range(n):
        N = int(ref["n_nodes"][i])
        m, y = res.solution(i)
        # FP64 sums in another order (FMA contraction) move redistributed points at 1e-11
        assert np.abs(m - ref["mesh"][i, :N]).max() <= 1e-9
        u = np.abs(ref["y"][i, :N]).max()
        err = np.abs(y - ref["y"][i, :N]).max()
        assert err <= tol_rel * max(1.0, u), (i, err)
        tight.append(err <= max(1e-6, 1e-9 * u))
    assert np.mean(tight) >= frac_tight


@pytest.mark.parametrize("jac_precision", [64, 32])
def test_nonlinear32_matches_oracle(pkg, problems, jac_precision):
    # FP64 blocks: the Newton iterates follow the oracle's, solutions within max(abstol, 1e-9|u|);
    # FP32 blocks (FP64 residual as right-hand side): the same root, within 1e-5 relative
    p = problems.NONLINEAR32
    params, nint, tsp, y0 = problems.nonlinear32_family(6, n_intervals=64)
    sv = pkg.BatchSolver(p, order=4, jac_precision=jac_precision)
    res = sv.solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0)
    assert (res.retcode == RET_SUCCESS).all()
    # the autotuner picked a linear-solve block of 3..8 warps on the first Newton step
    t = sv.tuning()["linsolve_threads"]
    assert t % 32 == 0 and 96 <= t <= 256, t
    if jac_precision == 64:
        assert (res.newton_iters == ref["newton_iters"]).all(), (res.newton_iters, ref["newton_iters"])
        _compare(res, ref, 1e-6)
    else:
        _compare(res, ref, 1e-5)


def test_nonlinear32_refines_like_the_oracle(pkg, problems):
    # a coarse initial mesh forces mesh selection, redistribution and the in-place transfer
    p = problems.NONLINEAR32
    params, nint, tsp, y0 = problems.nonlinear32_family(4, seed=77, n_intervals=6)
    sv = pkg.BatchSolver(p, order=4, jac_precision=64)
    res = sv.solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0)
    assert (ref["rounds"] > 1).any()
    assert (res.rounds == ref["rounds"]).all(), (res.rounds, ref["rounds"])
    _compare(res, ref, 1e-6)


def test_nonlinear32_mirk6_and_reference_size(pkg, problems):
    # the benchmark configuration's mesh (1024 intervals) on a few instances, and MIRK6: every
    # result passes the reference's acceptance tests evaluated by the oracle
    p = problems.NONLINEAR32
    o = _oracle(p)
    for order, nI, count in ((4, 1024, 8), (6, 64, 4)):
        params, nint, tsp, y0 = problems.nonlinear32_family(count, seed=5, n_intervals=nI)
        sv = pkg.BatchSolver(p, order=order)
        res = sv.solve(params, nint, tsp, y0)
        assert (res.retcode == RET_SUCCESS).all()
        for i in range(count):
            m, y = res.solution(i)
            F, K, nrm = o.residual(params[i], m, y, order=order)
            assert nrm <= 1e-6 * (1 + 1e-6), (order, i, nrm)
            err, dn = o.defect(params[i], m, y, order=order)
            assert dn <= 1e-6 * (1 + 1e-3), (order, i, dn)


def test_nonlinear32_dense_output(pkg, problems):
    # sol(t) and sol(t, Val{1}) of the larger-state path (interpolation.jl:17-206): the stages the
    # library returns are the oracle's at the GPU's solution, and the dense output is the MIRK
    # interpolant of those stages
    p = problems.NONLINEAR32
    o = _oracle(p)
    params, nint, tsp, y0 = problems.nonlinear32_family(3, seed=11, n_intervals=64)
    sv = pkg.BatchSolver(p, order=4, jac_precision=64, want_stages=1)
    res = sv.solve(params, nint, tsp, y0)
    assert (res.retcode == RET_SUCCESS).all()
    rng = np.random.default_rng(3)
    tq = np.sort(rng.uniform(0.0, 1.0, (3, 21)), axis=1)
    tq[:, 0], tq[:, -1] = 0.0, 1.0
    u = sv.dense(tq)
    du = sv.dense(tq, deriv=1)
    checked_ki = 0
    for i in range(3):
        m, y = res.solution(i)
        K, KI = res.stages(i)
        n = len(m)
        F, Kref, nrm = o.residual(params[i], m, y)
        scale = max(1.0, np.abs(Kref).max())
        assert np.abs(K - Kref.reshape(K.shape)).max() <= 1e-10 * scale
        if res.rounds[i] == 1:
            # uniform mesh: the oracle started from the GPU's (converged) solution returns its
            # own interpolant stages there
            ref = o.solve_batch(params[i:i + 1], [n - 1], tsp[i:i + 1], y, y0_mode=1, adaptive=0,
                                want_stages=True)
            assert np.abs(KI - ref["KI"][0, :n - 1]).max() <= 1e-10 * scale
            checked_ki += 1
        assert np.abs(u[i] - o.interpolate(4, m, y, K, KI, tq[i])).max() < 1e-12
        assert np.abs(du[i] - o.interpolate(4, m, y, K, KI, tq[i], deriv=1)).max() < 1e-11
        # at t0 the interpolant is the first node; at t1 it meets the last node up to the last
        # interval's collocation residual, which the accepted solution keeps within abstol
        assert np.abs(u[i][0] - y[0]).max() == 0.0
        assert np.abs(u[i][-1] - y[-1]).max() <= 1e-6 * (1 + 1e-6)
    assert checked_ki >= 1


@pytest.mark.parametrize("y0_mode", [0, 1])
def test_nonlinear32_device_inputs(pkg, problems, y0_mode):
    # the device-input entry point on the host-driven path: inputs read back on the handle's
    # stream, the same solve as from host buffers (same handle, so the same tuned block size)
    import torch
    p = problems.NONLINEAR32
    params, nint, tsp, y0 = problems.nonlinear32_family(4, seed=5, n_intervals=64)
    if y0_mode == 1:
        y0 = np.concatenate([np.tile(y0[q], (int(nint[q]) + 1, 1)) for q in range(len(nint))])
    sv = pkg.BatchSolver(p, order=4, jac_precision=64)
    sv.solve(params, nint, tsp, y0, y0_mode=y0_mode)          # tunes the linear solve
    ref = sv.solve(params, nint, tsp, y0, y0_mode=y0_mode)

    def dev(x, dt):
        return torch.tensor(np.ascontiguousarray(x), dtype=dt, device="cuda")

    off = None
    if y0_mode == 1:
        off = dev(np.concatenate([[0], np.cumsum(nint[:-1] + 1)]), torch.int64)
    sv.solve_device(dev(params, torch.float64), dev(nint, torch.int32), dev(tsp, torch.float64),
                    dev(y0, torch.float64), int(nint.max()), y0_mode=y0_mode, d_y0_off=off)
    res = sv.fetch()
    for f in ("retcode", "n_nodes", "newton_iters", "rounds"):
        assert np.array_equal(getattr(res, f), getattr(ref, f)), f
    for i in range(len(nint)):
        for a, b in zip(res.solution(i), ref.solution(i)):
            assert np.array_equal(a, b), i
