"""End-to-end parity of the batched GPU solve with the CPU oracle (the reference algorithm
restated), through the C ABI, plus the reference's golden problems run on the GPU."""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle, RET_SUCCESS

pytestmark = pytest.mark.gpu


def _oracle(p):
    return Oracle(p.source, p.M, p.n_params, twopoint=p.twopoint, bc_t=p.bc_t, La=p.La, Lb=p.Lb)


def _parity_report(res, ref, abstol=1e-6):
    """Per-instance comparison. Returns (same_mesh_mask, max_err_same_mesh, interp_err)."""
    n = len(res.n_nodes)
    same = np.zeros(n, bool)
    errs = np.zeros(n)
    for i in range(n):
        N = int(ref["n_nodes"][i])
        if int(res.n_nodes[i]) != N:
            continue
        m_g, y_g = res.solution(i)
        if np.abs(m_g - ref["mesh"][i, :N]).max() > 1e-9:
            continue
        same[i] = True
        errs[i] = np.abs(y_g - ref["y"][i, :N]).max()
    return same, errs


def test_pendulum_reference_config(pkg, problems):
    # benchmark/simple_pendulum.jl: g = 9.81, dt = 0.05 -> 32 intervals, MIRK4
    p = problems.PENDULUM
    sv = pkg.BatchSolver(p, order=4)
    params = np.array([[9.81, 0.0, 0.0]])
    y0 = np.array([[math.pi / 2, math.pi / 2]])
    res = sv.solve(params, [32], [[0, math.pi / 2]], y0)
    ref = _oracle(p).solve_batch(params, [32], [[0, math.pi / 2]], y0)
    assert res.retcode[0] == RET_SUCCESS == ref["retcode"][0]
    assert res.n_nodes[0] == ref["n_nodes"][0]
    same, errs = _parity_report(res, ref)
    assert same[0]
    u = np.abs(ref["y"][0, :ref["n_nodes"][0]]).max()
    assert errs[0] <= max(1e-6, 1e-9 * u)


@pytest.mark.parametrize("jac_precision", [32, 64])
def test_pendulum_family_parity(pkg, problems, jac_precision):
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(512, seed=77)
    sv = pkg.BatchSolver(p, order=4, jac_precision=jac_precision)
    res = sv.solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0)
    assert (res.retcode == ref["retcode"]).all()
    same, errs = _parity_report(res, ref)
    # discrete mesh decisions may flip on a handful of instances whose Newton iterates
    # differ below abstol; everything else must match point by point
    assert same.mean() >= 0.97, same.mean()
    u = np.array([np.abs(ref["y"][i, :ref["n_nodes"][i]]).max() for i in range(len(nint))])
    tol = np.maximum(1e-6, 1e-9 * u)
    assert (errs[same] <= tol[same]).all(), errs[same].max()


def test_pendulum_family_newton_residual(pkg, problems):
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(256, seed=78)
    res = pkg.BatchSolver(p, order=4).solve(params, nint, tsp, y0)
    ok = res.retcode == RET_SUCCESS
    assert ok.all()
    assert (res.resid[ok] <= 1e-6).all()
    assert (res.defect[ok] <= 1e-6).all()
    # the FP64 CPU residual of every returned solution is within abstol
    o = _oracle(p)
    for i in range(0, 256, 17):
        m, y = res.solution(i)
        F, K, nrm = o.residual(params[i], m, y)
        assert nrm <= 1e-6


def test_singular_perturbation_mirk6_parity(pkg, problems):
    p = problems.SINGULAR_PERTURBATION
    params, nint, tsp, y0 = problems.singular_perturbation_family(24, seed=5, n_min=64, n_max=512)
    sv = pkg.BatchSolver(p, order=6)
    res = sv.solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0, order=6)
    assert (res.retcode == ref["retcode"]).mean() >= 0.9
    same, errs = _parity_report(res, ref)
    both_ok = (res.retcode == RET_SUCCESS) & (ref["retcode"] == RET_SUCCESS) & same
    assert both_ok.sum() >= 12
    assert (errs[both_ok] <= 1e-6).all(), errs[both_ok].max()


@pytest.mark.parametrize("order", [2, 3, 4, 5, 6])
def test_affineness_gpu(pkg, problems, order):
    # mirk_basic_tests.jl:103-118
    for name in ("affine", "affine_twopoint"):
        p = problems.ALL[name]
        res = pkg.BatchSolver(p, order=order).solve(np.zeros((1, 0)), [25], [[0, 5.0]], [p.u0])
        assert res.retcode[0] == RET_SUCCESS
        m, y = res.solution(0)
        assert np.abs(np.diff(y[:, 0]) + 0.2).max() + abs(y[0, 0] - 5) < 1e-2


@pytest.mark.parametrize("order", [2, 3, 4, 5, 6])
def test_convergence_order_gpu(pkg, problems, order):
    # mirk_basic_tests.jl:122-139, non-adaptive, FP64 Jacobian so the order is visible
    p = problems.LINEAR
    sv = pkg.BatchSolver(p, order=order, adaptive=0, jac_precision=64, max_newton=20)
    errs = []
    for n in (40, 20, 10):
        res = sv.solve(np.zeros((1, 0)), [n], [[0, 5.0]], [p.u0])
        m, y = res.solution(0)
        errs.append(np.abs(y - problems.linear_analytic(m)).max())
    est = np.log2(np.array(errs[1:]) / np.array(errs[:-1])).mean()
    assert abs(est - order) < 0.4, (errs, est)


def test_torus_geodesic_gpu(pkg, problems):
    # mirk_basic_tests.jl:726-756
    p = problems.TORUS
    a1, a2 = (0.5, -1.2), (-0.5, 0.3)
    res = pkg.BatchSolver(p, order=4).solve(np.array([a1 + a2]), [20], [[0, 1.0]], [p.u0])
    assert res.retcode[0] == RET_SUCCESS
    m, y = res.solution(0)
    assert np.abs(y[0, :2] - a1).max() < 1e-8
    assert np.abs(y[-1, :2] - a2).max() < 1e-8


def test_multipoint_dense_output_gpu(pkg, problems):
    # mirk_basic_tests.jl:271-312 through the GPU's returned stages + the oracle interpolant
    p = problems.MULTIPOINT
    res = pkg.BatchSolver(p, order=4, want_stages=1).solve(np.zeros((1, 0)), [1571], [[0, math.pi / 2]], [p.u0])
    assert res.retcode[0] == RET_SUCCESS
    m, y = res.solution(0)
    K, KI = res.stages(0)
    o = _oracle(p)
    for t in (math.pi / 6, math.pi / 3):
        got = o.interpolate(4, m, y, K, KI, [t])[0]
        assert np.abs(got - [math.sin(t), math.cos(t)]).max() < 1e-6


def test_ragged_batch_and_edges(pkg, problems):
    # a batch mixing a single-interval mesh, tiny and large meshes; every instance is
    # solved independently, so a batch result equals per-instance results
    p = problems.PENDULUM
    sv = pkg.BatchSolver(p, order=4)
    nint = np.array([1, 2, 3, 33, 256, 1000, 7], np.int32)
    n = len(nint)
    params = np.tile([9.81, 0.0, 0.0], (n, 1))
    tsp = np.tile([0, math.pi / 2], (n, 1))
    y0 = np.tile([math.pi / 2, math.pi / 2], (n, 1))
    res = sv.solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0)
    assert (res.retcode == ref["retcode"]).all()
    for i in range(n):
        one = sv.solve(params[i:i + 1], nint[i:i + 1], tsp[i:i + 1], y0[i:i + 1])
        assert one.n_nodes[0] == res.n_nodes[i]
        assert np.array_equal(one.solution(0)[1], res.solution(i)[1])


def test_invalid_arguments_rejected(pkg, problems):
    p = problems.PENDULUM
    sv = pkg.BatchSolver(p, order=4)
    with pytest.raises(pkg.BVPError):
        sv.solve(np.zeros((1, 3)), [0], [[0, 1.0]], [[0, 0]])     # no intervals
    with pytest.raises(pkg.BVPError):
        sv.solve(np.zeros((1, 3)), [8], [[1.0, 1.0]], [[0, 0]])   # empty tspan
