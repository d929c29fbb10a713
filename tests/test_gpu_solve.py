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


def test_pendulum_family_parity_fp64(pkg, problems):
    # FP64 Jacobian and factorisation: the Newton iterates follow the oracle's, so the
    # meshes match and the solutions agree within max(abstol, 1e-9 |u|) point by point
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(512, seed=77)
    sv = pkg.BatchSolver(p, order=4, jac_precision=64)
    res = sv.solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0)
    assert (res.retcode == ref["retcode"]).all()
    assert (res.newton_iters == ref["newton_iters"]).mean() >= 0.99
    same, errs = _parity_report(res, ref)
    assert same.mean() >= 0.99, same.mean()
    u = np.array([np.abs(ref["y"][i, :ref["n_nodes"][i]]).max() for i in range(len(nint))])
    tol = np.maximum(1e-6, 1e-9 * u)
    assert (errs[same] <= tol[same]).all(), errs[same].max()


def test_pendulum_family_fp32_same_accuracy(pkg, problems):
    # FP32 Jacobian/factorisation with the FP32 Newton phase: every accepted solution
    # passes the reference's own acceptance tests evaluated in FP64 by the oracle
    # (||F||_inf <= abstol, defect <= abstol); where the mesh sequence matches the
    # oracle's, the solutions agree within max(abstol, 1e-9 |u|) for nearly all instances
    # (the rest differ by the FP32 path's distinct Newton iterates, bounded by cond * abstol)
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(512, seed=77)
    sv = pkg.BatchSolver(p, order=4, jac_precision=32)
    res = sv.solve(params, nint, tsp, y0)
    o = _oracle(p)
    ref = o.solve_batch(params, nint, tsp, y0)
    assert (res.retcode == ref["retcode"]).mean() >= 0.99
    same, errs = _parity_report(res, ref)
    assert same.mean() >= 0.8, same.mean()
    u = np.array([np.abs(ref["y"][i, :ref["n_nodes"][i]]).max() for i in range(len(nint))])
    tol = np.maximum(1e-6, 1e-9 * u)
    assert (errs[same] <= tol[same]).mean() >= 0.95
    assert (errs[same] <= 1e-3 * np.maximum(1, u[same])).all(), errs[same].max()
    for i in range(len(nint)):
        if res.retcode[i] != RET_SUCCESS:
            continue
        m, y = res.solution(i)
        F, K, nrm = o.residual(params[i], m, y)
        assert nrm <= 1e-6 * (1 + 1e-6), (i, nrm)
        err, dn = o.defect(params[i], m, y)
        assert dn <= 1e-6 * (1 + 1e-3), (i, dn)


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
    o = _oracle(p)
    ref = o.solve_batch(params, nint, tsp, y0, order=6)
    for jp in (64, 32):
        sv = pkg.BatchSolver(p, order=6, jac_precision=jp)
        res = sv.solve(params, nint, tsp, y0)
        same, errs = _parity_report(res, ref)
        print(f"jac{jp}: retcode match {(res.retcode == ref['retcode']).mean():.3f} same mesh {same.mean():.3f} "
              f"max err same {errs[same].max() if same.any() else 0:.3e}")
        # ε down to 1e-3 makes the systems so ill-conditioned that roundoff alone (the
        # cyclic reduction's elimination order against the oracle's sequential one)
        # moves the defect enough to flip discrete mesh decisions; where the mesh
        # sequence matches, FP64 agrees to roundoff
        assert (res.retcode == ref["retcode"]).mean() >= 0.9
        ok = same & (res.retcode == RET_SUCCESS)
        if jp == 64:
            assert (errs[ok] <= 1e-6).all(), errs[ok].max()
        for i in range(len(nint)):
            if res.retcode[i] != RET_SUCCESS:
                continue
            m, y = res.solution(i)
            F, K, nrm = o.residual(params[i], m, y, order=6)
            assert nrm <= 1e-6 * (1 + 1e-6), (jp, i, nrm)
            err, dn = o.defect(params[i], m, y, order=6)
            assert dn <= 1e-6 * (1 + 1e-3), (jp, i, dn)


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


@pytest.mark.parametrize("jac_precision", [64, 32])
def test_torus_geodesic_gpu(pkg, problems, jac_precision):
    # mirk_basic_tests.jl:726-756. The reference's 1e-8 on the BCs comes from its FP64
    # Newton overshooting abstol quadratically; the FP64 mode reproduces that, the FP32
    # mode meets the solve's own tolerance (||F||_inf <= abstol = 1e-6)
    p = problems.TORUS
    a1, a2 = (0.5, -1.2), (-0.5, 0.3)
    res = pkg.BatchSolver(p, order=4, jac_precision=jac_precision).solve(
        np.array([a1 + a2]), [20], [[0, 1.0]], [p.u0])
    assert res.retcode[0] == RET_SUCCESS
    m, y = res.solution(0)
    tol = 1e-8 if jac_precision == 64 else 1e-6
    assert np.abs(y[0, :2] - a1).max() < tol
    assert np.abs(y[-1, :2] - a2).max() < tol


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


@pytest.mark.parametrize("jac_precision", [64, 32])
def test_singular_term_matches_oracle(pkg, problems, jac_precision):
    # Lane-Emden with its singular term (MIRK4, MIRK6, fixed and adaptive meshes): the GPU
    # reproduces the oracle's retcode, rounds and final mesh; FP64 mode agrees point by point
    # within max(abstol, 1e-9 |u|), FP32 mode passes the reference's acceptance test (the FP64
    # residual of the returned solution, evaluated by the oracle, within abstol)
    p = problems.LANE_EMDEN
    o = _oracle(p)
    params = np.zeros((1, 0))
    y0 = np.array([p.u0])
    for order in (4, 6):
        for adaptive in (0, 1):
            sv = pkg.BatchSolver(p, order=order, jac_precision=jac_precision, adaptive=adaptive)
            res = sv.solve(params, [100], [[0.0, 1.0]], y0)
            ref = o.solve_batch(params, [100], [[0.0, 1.0]], y0, order=order, adaptive=adaptive)
            assert res.retcode[0] == ref["retcode"][0]
            assert res.n_nodes[0] == ref["n_nodes"][0]
            assert res.rounds[0] == ref["rounds"][0]
            same, errs = _parity_report(res, ref)
            assert same[0]
            if jac_precision == 64:
                assert errs[0] <= 1e-6, (order, adaptive, errs[0])
            elif res.retcode[0] == RET_SUCCESS:
                m, y = res.solution(0)
                assert o.residual(params[0], m, y, order=order)[2] <= 1e-6 * (1 + 1e-6)


@pytest.mark.parametrize("jac_precision", [64, 32])
def test_mathieu_eigenvalue_gpu(pkg, problems, jac_precision):
    # the reference's parameter-estimation golden value (mirk_basic_tests.jl:485-507):
    # lambda = 17.09658 within 1e-4, from the test's guess, MIRK4, dt = 0.05
    p = problems.MATHIEU
    n = int(math.ceil(math.pi / 0.05 - 1e-12))
    guess = problems.mathieu_guess(n)
    sv = pkg.BatchSolver(p, order=4, jac_precision=jac_precision)
    res = sv.solve(np.zeros((1, 0)), [n], [[0.0, math.pi]], guess, y0_mode=1)
    assert res.retcode[0] == RET_SUCCESS
    m, y = res.solution(0)
    assert np.abs(y[:, 2] - 17.09658).max() < 1e-4
    o = _oracle(p)
    if jac_precision == 64:
        # FP64 blocks follow the oracle's iterates: same rounds and final mesh
        ref = o.solve_batch(np.zeros((1, 0)), [n], [[0.0, math.pi]], guess, y0_mode=1, order=4)
        assert res.n_nodes[0] == ref["n_nodes"][0] and res.rounds[0] == ref["rounds"][0]
    else:
        # FP32 blocks: the reference's acceptance tests, evaluated in FP64 by the oracle
        assert o.residual(np.zeros(0), m, y)[2] <= 1e-6 * (1 + 1e-6)
        assert o.defect(np.zeros(0), m, y)[1] <= 1e-6 * (1 + 1e-3)


def test_reference_style_solve(pkg, problems):
    # the reference's own call, solve(prob, MIRK4(), dt = 0.05) on the pendulum
    # (benchmark/simple_pendulum.jl), through the reference-style front end, and an ensemble
    sciml = pkg.sciml
    p = problems.PENDULUM
    sol = sciml.solve(p, sciml.MIRK4(jac_precision=64), dt=0.05, p=[9.81, 0.0, 0.0],
                      u0=[math.pi / 2, math.pi / 2])
    o = _oracle(p)
    ref = o.solve_batch(np.array([[9.81, 0.0, 0.0]]), [32], [[0.0, math.pi / 2]],
                        np.array([[math.pi / 2, math.pi / 2]]))
    assert sol.successful and ref["retcode"][0] == RET_SUCCESS
    N = int(ref["n_nodes"][0])
    assert len(sol.t) == N
    assert np.abs(sol.u - ref["y"][0, :N]).max() <= 1e-6
    # sol(t): the interpolant meets the nodes within the collocation residual
    assert np.abs(sol(sol.t[:6]) - sol.u[:6]).max() <= 1e-6
    assert sol(0.0).shape == (2,)
    params, nint, tsp, y0 = problems.pendulum_family(8, seed=12)
    sols = sciml.solve(sciml.EnsembleProblem(p, params=params, tspans=tsp), sciml.MIRK4(jac_precision=64), dt=0.05)
    refs = o.solve_batch(params, [32] * 8, tsp, np.tile([math.pi / 2, math.pi / 2], (8, 1)))
    for i, s in enumerate(sols):
        n = int(refs["n_nodes"][i])
        assert s.successful and len(s.t) == n
        assert np.abs(s.u - refs["y"][i, :n]).max() <= 1e-6


def test_mirk6i_golden_gpu(pkg, problems):
    # MIRK6I through the reference's golden tests on the GPU: affineness
    # (mirk_basic_tests.jl:113-116) and the observed order 6 (:134-137)
    for name in ("affine", "affine_twopoint"):
        p = problems.ALL[name]
        res = pkg.BatchSolver(p, order=6, mirk6i=1).solve(np.zeros((1, 0)), [25], [[0, 5.0]], [p.u0])
        assert res.retcode[0] == RET_SUCCESS
        m, y = res.solution(0)
        assert np.abs(np.diff(y[:, 0]) + 0.2).max() + abs(y[0, 0] - 5) < 1e-2
    p = problems.LINEAR
    sv = pkg.BatchSolver(p, order=6, mirk6i=1, adaptive=0, jac_precision=64, max_newton=20)
    errs = []
    for n in (40, 20, 10):
        res = sv.solve(np.zeros((1, 0)), [n], [[0, 5.0]], [p.u0])
        m, y = res.solution(0)
        errs.append(np.abs(y - problems.linear_analytic(m)).max())
    est = np.log2(np.array(errs[1:]) / np.array(errs[:-1])).mean()
    assert abs(est - 6) < 0.4, (errs, est)


def test_mirk6i_pendulum_parity_fp64(pkg, problems):
    # MIRK6I adaptive solves of the pendulum family against the oracle: same retcodes, the
    # oracle's final meshes, solutions within max(abstol, 1e-9 |u|), dense output equal to
    # the oracle's interpolant of the same stages
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(128, seed=91)
    sv = pkg.BatchSolver(p, order=6, mirk6i=1, jac_precision=64, want_stages=1)
    res = sv.solve(params, nint, tsp, y0)
    o = _oracle(p)
    ref = o.solve_batch(params, nint, tsp, y0, order=6, mirk6i=1)
    assert (res.retcode == ref["retcode"]).all()
    same, errs = _parity_report(res, ref)
    assert same.mean() >= 0.99, same.mean()
    u = np.array([np.abs(ref["y"][i, :ref["n_nodes"][i]]).max() for i in range(len(nint))])
    assert (errs[same] <= np.maximum(1e-6, 1e-9 * u[same])).all(), errs[same].max()
    tq = tsp[:, :1] + (tsp[:, 1:] - tsp[:, :1]) * np.linspace(0.013, 0.987, 7)[None, :]
    for deriv in (0, 1):
        d = sv.dense(tq, deriv=deriv)
        for i in range(0, len(nint), 9):
            m, y = res.solution(i)
            K, KI = res.stages(i)
            want = o.interpolate(6, m, y, K, KI, tq[i], deriv=deriv, mirk6i=1)
            assert np.abs(d[i] - want).max() <= 1e-10 * max(1.0, np.abs(want).max())


def test_learned_work_order_changes_no_result(pkg, problems):
    # the work-order autotuner: after the handle's first solves of >= 256 instances the fused
    # solve starts the instances its cost table predicts to be longest first; every instance's
    # result is the same bit for bit as under the initial (coarsest-first) order
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(1024, seed=97)
    fresh = pkg.BatchSolver(p, order=4)
    assert fresh.work_order()[0] is False
    ref = fresh.solve(params, nint, tsp, y0)
    tuned = pkg.BatchSolver(p, order=4)
    for _ in range(3):
        tuned.solve(params, nint, tsp, y0)
    learned, costs = tuned.work_order()
    assert learned and costs[512] > 0 and (costs[:512] > 0).all()
    # coarse initial meshes (several mesh rounds) cost more than the single-round middle sizes
    assert costs[32 // 8] > costs[96 // 8]
    res = tuned.solve(params, nint, tsp, y0)
    for f in ("retcode", "n_nodes", "newton_iters", "rounds"):
        assert np.array_equal(getattr(res, f), getattr(ref, f))
    for i in range(len(nint)):
        assert np.array_equal(res.solution(i)[1], ref.solution(i)[1])


def test_launch_shape_tuner_changes_no_result(pkg, problems):
    # the launch-shape autotuner: after the work order is learned, the next nine solves of the
    # same batch shape run the fused kernel built for 4, 3 and 2 resident blocks per SM (an
    # untimed first launch and two timed ones each) and the handle keeps the fastest; the three
    # builds differ only in their register budgets, so every solve's results are the same bit
    # for bit
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(512, seed=98)
    sv = pkg.BatchSolver(p, order=4)
    t0 = sv.tuning()
    assert t0["fused_blocks_per_sm"] == 3 and not t0["fused_tuned"]
    ref = sv.solve(params, nint, tsp, y0)
    for _ in range(13):
        res = sv.solve(params, nint, tsp, y0)
        for f in ("retcode", "n_nodes", "newton_iters", "rounds"):
            assert np.array_equal(getattr(res, f), getattr(ref, f))
        assert res.y_packed.shape == ref.y_packed.shape
        for i in range(0, 512, 17):
            assert np.array_equal(res.solution(i)[1], ref.solution(i)[1])
    t = sv.tuning()
    assert t["fused_tuned"] and t["fused_blocks_per_sm"] in (4, 3, 2)
    ms = t["fused_ms_by_blocks"]
    assert all(v > 0 for v in ms.values())
    assert ms[t["fused_blocks_per_sm"]] == min(ms.values())
