"""The error controllers other than DefectControl on the GPU against the oracle
(Core/src/calc_errors.jl:54-139; the estimates of adaptivity.jl:361-567 and the selectors of
adaptivity.jl:77-243): GlobalErrorControl, SequentialErrorControl and HybridErrorControl, each
with the HOErrorControl estimate (a MIRK(p+2) solve on the same mesh, run by the module of that
order between launches) and the REErrorControl one (the same method on the halved mesh, inside
the fused kernel).

On the linear problem and the torus geodesics, in FP64 mode (which follows the oracle's Newton
path): the same retcodes, mesh rounds, Newton iterations and final meshes, solutions within
max(abstol, 1e-9 |u|), global estimates within 1e-3 relative. In the FP32 mode the solutions
pass the reference's acceptance on their own meshes and their error against the exact
solution (the linear problem) is the oracle's. The reference's own error-control test
(mirk_basic_tests.jl:414-434) runs under every controller."""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle, RET_SUCCESS

pytestmark = pytest.mark.gpu

GLOBAL_CASES = [("global", "HO"), ("global", "RE"), ("sequential", "HO"), ("sequential", "RE"),
                ("hybrid", "HO"), ("hybrid", "RE")]


def _oracle(p):
    return Oracle(p.source, p.M, p.n_params, twopoint=p.twopoint, bc_t=p.bc_t, La=p.La, Lb=p.Lb)


def _linear_batch():
    nint = np.array([4, 6, 9, 10, 13, 17, 24, 40], np.int32)
    n = len(nint)
    return np.zeros((n, 0)), nint, np.tile([0.0, 5.0], (n, 1)), np.tile([5.0, -3.5], (n, 1))


def _torus_batch(n=12, seed=41):
    rng = np.random.default_rng(seed)
    a1 = rng.uniform(-0.8, 0.8, (n, 2))
    a2 = rng.uniform(-0.8, 0.8, (n, 2))
    nint = rng.integers(8, 40, n).astype(np.int32)
    return np.concatenate([a1, a2], 1), nint, np.tile([0.0, 1.0], (n, 1)), np.tile([0.5, -1.2, 0.0, 0.0], (n, 1))


def _match(res, ref, abstol=1e-6):
    n = len(res.n_nodes)
    assert (res.retcode == ref["retcode"]).all(), (res.retcode, ref["retcode"])
    assert (res.rounds == ref["rounds"]).all(), (res.rounds, ref["rounds"])
    assert (res.newton_iters == ref["newton_iters"]).all(), (res.newton_iters, ref["newton_iters"])
    assert (res.n_nodes == ref["n_nodes"]).all()
    for i in range(n):
        N = int(ref["n_nodes"][i])
        m, y = res.solution(i)
        assert np.abs(m - ref["mesh"][i, :N]).max() <= 1e-9 * max(1.0, np.abs(m).max()), i
        yr = ref["y"][i, :N]
        assert np.abs(y - yr).max() <= max(abstol, 1e-9 * np.abs(yr).max()), i
        g, gr = res.global_err[i], ref["global_err"][i]
        assert (math.isnan(g) and math.isnan(gr)) or abs(g - gr) <= 1e-3 * abs(gr) + 1e-12, (i, g, gr)


@pytest.mark.parametrize("ctl,gm", GLOBAL_CASES)
@pytest.mark.parametrize("order", [2, 3, 4])
def test_linear_fp64_matches_oracle(pkg, problems, ctl, gm, order):
    p = problems.LINEAR
    params, nint, tsp, y0 = _linear_batch()
    res = pkg.BatchSolver(p, order=order, jac_precision=64, controller=ctl, global_method=gm).solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0, order=order, controller=ctl, global_method=gm)
    _match(res, ref)


@pytest.mark.parametrize("ctl", ["global", "sequential", "hybrid"])
@pytest.mark.parametrize("order,mirk6i", [(5, 0), (6, 0), (6, 1)])
def test_richardson_higher_orders_fp64(pkg, problems, ctl, order, mirk6i):
    p = problems.LINEAR
    params, nint, tsp, y0 = _linear_batch()
    res = pkg.BatchSolver(p, order=order, jac_precision=64, controller=ctl, global_method="RE",
                          mirk6i=mirk6i).solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0, order=order, mirk6i=mirk6i, controller=ctl,
                                 global_method="RE")
    _match(res, ref)


@pytest.mark.parametrize("ctl,gm", GLOBAL_CASES)
def test_torus_fp64_matches_oracle(pkg, problems, ctl, gm):
    p = problems.TORUS
    params, nint, tsp, y0 = _torus_batch()
    res = pkg.BatchSolver(p, order=4, jac_precision=64, controller=ctl, global_method=gm).solve(params, nint, tsp, y0)
    ref = _oracle(p).solve_batch(params, nint, tsp, y0, order=4, controller=ctl, global_method=gm)
    assert (ref["retcode"] == RET_SUCCESS).all()
    _match(res, ref)


@pytest.mark.parametrize("ctl,gm", GLOBAL_CASES)
def test_fp32_mode_meets_the_reference_acceptance(pkg, problems, ctl, gm):
    # the benchmark's precision: FP32 Jacobian and Newton phase, every decision in FP64
    p = problems.LINEAR
    params, nint, tsp, y0 = _linear_batch()
    res = pkg.BatchSolver(p, order=4, controller=ctl, global_method=gm).solve(params, nint, tsp, y0)
    o = _oracle(p)
    ref = o.solve_batch(params, nint, tsp, y0, order=4, controller=ctl, global_method=gm)
    assert (res.retcode == ref["retcode"]).all() and (res.retcode == RET_SUCCESS).all()
    for i in range(len(nint)):
        m, y = res.solution(i)
        assert o.residual((), m, y)[2] <= 1e-6 * (1 + 1e-6)
        N = int(ref["n_nodes"][i])
        err = np.abs(y - problems.linear_analytic(m)).max()
        err_ref = np.abs(ref["y"][i, :N] - problems.linear_analytic(ref["mesh"][i, :N])).max()
        assert err <= 1.1 * err_ref + 1e-6, (i, err, err_ref)


@pytest.mark.parametrize("ctl,gm", [("defect", "HO")] + GLOBAL_CASES)
def test_reference_error_control_testset(pkg, problems, ctl, gm):
    # mirk_basic_tests.jl:414-434: the pendulum, MIRK4, dt = 0.05, abstol = 1e-5, each controller,
    # through the reference-style API
    sc = pkg.sciml
    c = {"defect": sc.DefectControl(), "global": sc.GlobalErrorControl(),
         "sequential": sc.SequentialErrorControl(), "hybrid": sc.HybridErrorControl()}[ctl]
    if gm == "RE" and ctl != "defect":
        ge = sc.GlobalErrorControl(method=sc.REErrorControl())
        c = {"global": ge, "sequential": sc.SequentialErrorControl(global_error=ge),
             "hybrid": sc.HybridErrorControl(global_error=ge)}[ctl]
    p = problems.PENDULUM
    sol = sc.solve(p, sc.MIRK4(jac_precision=64), dt=0.05, abstol=1e-5, p=(9.81, 0.0, 0.0), controller=c)
    assert sol.successful
    o = _oracle(p)
    ref = o.solve_batch([[9.81, 0.0, 0.0]], [32], [[0.0, math.pi / 2]], [p.u0], order=4, abstol=1e-5,
                        controller=ctl, global_method=gm)
    N = int(ref["n_nodes"][0])
    assert len(sol.t) == N and np.abs(sol.t - ref["mesh"][0, :N]).max() <= 1e-9
    assert np.abs(sol.u - ref["y"][0, :N]).max() <= 1e-5
    assert abs(sol(math.pi / 4)[0] + math.pi / 2) <= 1e-5


def test_ho_needs_mirk_p_plus_2(pkg, problems):
    with pytest.raises(pkg.BVPError):
        pkg.BatchSolver(problems.LINEAR, order=5, controller="global", global_method="HO")
