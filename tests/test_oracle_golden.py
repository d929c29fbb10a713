"""The CPU oracle against the golden values the reference's own tests pin for the MIRK
path (lib/BoundaryValueDiffEqMIRK/test/Core/mirk_basic_tests.jl and ensemble_tests.jl).
These run on the CPU only; they establish that the oracle restates the reference before
it is used to judge the CUDA library."""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle, RET_SUCCESS

ORDERS = (2, 3, 4, 5, 6)


def _oracle(p):
    return Oracle(p.source, p.M, p.n_params, twopoint=p.twopoint, bc_t=p.bc_t, La=p.La, Lb=p.Lb)


def _solve1(p, dt=None, n=None, params=(), y0=None, **kw):
    o = _oracle(p)
    t0, t1 = p.tspan
    if n is None:
        n = int(math.ceil((t1 - t0) / dt - 1e-12))  # cld(t1 - t0, dt) (Core/utils.jl:354)
    pa = np.asarray(params, dtype=np.float64).reshape(1, -1) if len(params) else np.zeros((1, 1))
    y0 = p.u0 if y0 is None else y0
    r = o.solve_batch(pa, [n], [[t0, t1]], np.asarray(y0, dtype=np.float64), want_stages=True, **kw)
    N = int(r["n_nodes"][0])
    return o, r, N


@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("name", ["affine", "affine_twopoint"])
def test_affineness(problems, name, order):
    # mirk_basic_tests.jl:103-118: exact solution u1 = 5 - t; dt = 0.2
    p = problems.ALL[name]
    o, r, N = _solve1(p, dt=0.2, order=order)
    assert r["retcode"][0] == RET_SUCCESS
    u1 = r["y"][0, :N, 0]
    assert np.abs(np.diff(u1) + 0.2).max() + abs(u1[0] - 5) < 1e-2


@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("name", ["linear", "linear_twopoint"])
def test_convergence_order_linear(problems, name, order):
    # mirk_basic_tests.jl:122-139: observed order ~ p within 0.4 on dts = 1/8, 1/4, 1/2.
    p = problems.ALL[name]
    errs = []
    for dt in (1 / 8, 1 / 4, 1 / 2):
        o, r, N = _solve1(p, dt=dt, order=order, adaptive=0, max_newton=20)
        assert r["retcode"][0] == RET_SUCCESS
        t = r["mesh"][0, :N]
        errs.append(np.abs(r["y"][0, :N] - problems.linear_analytic(t)).max())
    errs = np.array(errs)
    est = np.log2(errs[1:] / errs[:-1]).mean()
    assert abs(est - order) < 0.4, (errs, est)


@pytest.mark.parametrize("order", ORDERS)
def test_interpolation_twopoint(problems, order):
    # mirk_basic_tests.jl:181-223 and 235-244: sol(0.001) and sol(0.04, Val{1}), atol 1e-6
    p = problems.TWOPOINT_INTERP
    o, r, N = _solve1(p, dt=0.001, params=(1.0,), order=order)
    assert r["retcode"][0] == RET_SUCCESS
    mesh, y, K, KI = r["mesh"][0, :N], r["y"][0], r["K"][0], r["KI"][0]
    u, du = problems.twopoint_interp_analytic(np.array([0.001]))
    got = o.interpolate(order, mesh, y, K, KI, [0.001])
    assert np.abs(got - u).max() < 1e-6
    u4, du4 = problems.twopoint_interp_analytic(np.array([0.04]))
    assert np.abs(o.interpolate(order, mesh, y, K, KI, [0.04]) - u4).max() < 1e-6
    assert np.abs(o.interpolate(order, mesh, y, K, KI, [0.04], deriv=1) - du4).max() < 1e-6


@pytest.mark.parametrize("adaptive", [1, 0])
@pytest.mark.parametrize("order", ORDERS)
def test_interpolation_multipoint(problems, order, adaptive):
    # mirk_basic_tests.jl:271-312: sol(pi/6) and sol(pi/3) vs (sin, cos), atol 1e-6
    p = problems.MULTIPOINT
    o, r, N = _solve1(p, dt=0.001, order=order, adaptive=adaptive)
    assert r["retcode"][0] == RET_SUCCESS
    mesh, y, K, KI = r["mesh"][0, :N], r["y"][0], r["K"][0], r["KI"][0]
    for t in (math.pi / 6, math.pi / 3):
        got = o.interpolate(order, mesh, y, K, KI, [t])[0]
        assert np.abs(got - [math.sin(t), math.cos(t)]).max() < 1e-6


def test_torus_geodesic_refines(problems):
    # mirk_basic_tests.jl:726-756: adaptive refinement, BCs satisfied to 1e-8
    p = problems.TORUS
    a1, a2 = (0.5, -1.2), (-0.5, 0.3)
    o, r, N = _solve1(p, dt=0.05, params=a1 + a2, order=4)
    assert r["retcode"][0] == RET_SUCCESS
    y = r["y"][0, :N]
    assert np.abs(y[0, :2] - a1).max() < 1e-8
    assert np.abs(y[-1, :2] - a2).max() < 1e-8


def test_initial_guess_passthrough(problems):
    # mirk_basic_tests.jl:678-720: maxiters = 0, non-adaptive -> the guess comes back exactly
    p = problems.LINEAR_TWOPOINT
    o = _oracle(p)
    n = 10
    rng = np.random.default_rng(7)
    guess = rng.normal(size=(n + 1, 2))
    r = o.solve_batch(np.zeros((1, 1)), [n], [[0.0, 1.0]], guess, y0_mode=1, adaptive=0,
                      max_newton=0, linesearch_fallback=0)
    assert np.array_equal(r["y"][0, :n + 1], guess)


@pytest.mark.parametrize("order", ORDERS)
def test_ensemble_converges(problems, order):
    # ensemble_tests.jl:7-41: random p per trajectory, every trajectory converged
    p = problems.ENSEMBLE
    o = _oracle(p)
    rng = np.random.default_rng(11)
    n = 10
    params = rng.uniform(0, 1, (n, 1))
    r = o.solve_batch(params, [16] * n, np.tile(p.tspan, (n, 1)), np.tile(p.u0, (n, 1)),
                      order=order)
    assert (r["retcode"] == RET_SUCCESS).all()


def test_pendulum_reference_config(problems):
    # benchmark/simple_pendulum.jl:5-32 with dt = 0.05 (the reference test only checks that
    # it runs); cross-checked against scipy's independent collocation solver.
    scipy_integrate = pytest.importorskip("scipy.integrate")
    p = problems.PENDULUM
    o, r, N = _solve1(p, dt=0.05, params=(9.81, 0.0, 0.0), order=4)
    assert r["retcode"][0] == RET_SUCCESS
    mesh, y = r["mesh"][0, :N], r["y"][0, :N]
    u_mid = o.interpolate(4, mesh, r["y"][0], r["K"][0], r["KI"][0], [math.pi / 4])[0]
    assert abs(u_mid[0] + math.pi / 2) < 1e-6
    assert abs(y[-1, 0] - math.pi / 2) < 1e-6

    # scipy solve_bvp on the same problem: interior condition handled by splitting at pi/4
    def fun(t, u):
        return np.vstack([u[1], -9.81 * np.sin(u[0])])

    # solve on [pi/4, pi/2] and [0, pi/4] as a two-piece problem with continuity
    def fun2(t, w):
        # w = (u on [0,pi/4] mapped to s in [0,1], u on [pi/4,pi/2] mapped to s in [0,1])
        h = math.pi / 4
        return np.vstack([h * w[1], -h * 9.81 * np.sin(w[0]), h * w[3], -h * 9.81 * np.sin(w[2])])

    def bc2(wa, wb):
        return np.array([wb[0] + math.pi / 2, wa[2] + math.pi / 2, wb[2] - math.pi / 2,
                         wb[1] - wa[3]])

    s = np.linspace(0, 1, 50)
    w0 = np.zeros((4, s.size))
    w0[0] = np.interp(s * math.pi / 4, mesh, y[:, 0]); w0[1] = np.interp(s * math.pi / 4, mesh, y[:, 1])
    w0[2] = np.interp(math.pi / 4 + s * math.pi / 4, mesh, y[:, 0])
    w0[3] = np.interp(math.pi / 4 + s * math.pi / 4, mesh, y[:, 1])
    sol = scipy_integrate.solve_bvp(fun2, bc2, s, w0, tol=1e-8, max_nodes=100000)
    assert sol.success
    assert abs(sol.sol(0.0)[0] - y[0, 0]) < 1e-4
    assert abs(sol.sol(0.0)[1] - y[0, 1]) < 1e-4


@pytest.mark.parametrize("order", (3, 4, 5, 6))
def test_singular_term_lane_emden(problems, order):
    # the singular term S y / t (Core/src/utils.jl:925-941) enters the collocation stages for
    # t > 0 (collocation.jl:60-66). Lane-Emden y'' + (2/t) y' + y = 0 (singular_bvp_tests.jl:14-50)
    # on fixed meshes converges to y = sin(t)/t; the stage at t = 0 lacks the term's limit, so the
    # order is one. (The reference test builds its problem without passing singular_term, so it
    # pins no value for this path.)
    p = problems.LANE_EMDEN
    errs = []
    for n in (100, 200, 400):
        o, r, N = _solve1(p, n=n, order=order, adaptive=0)
        assert r["retcode"][0] == RET_SUCCESS
        m, y = r["mesh"][0, :N], r["y"][0, :N]
        errs.append(np.abs(y - problems.lane_emden_analytic(m)).max())
    assert errs[0] < 1e-3
    for e0, e1 in zip(errs, errs[1:]):
        assert 1.6 < e0 / e1 < 2.5, errs
    # adaptive: the defect (adaptivity.jl:416-461) evaluates f without the singular term, so the
    # estimate stays above the 10% threshold and the mesh halves until it exceeds the cap
    o, r, N = _solve1(p, n=100, order=order)
    assert r["retcode"][0] != RET_SUCCESS and N > 1000


def test_mathieu_eigenvalue(problems):
    # mirk_basic_tests.jl:485-507: unknown-parameter estimation, lambda = 17.09658 (atol 1e-4);
    # the parameter is carried as a state with zero derivative, MIRK4, dt = 0.05 on (0, pi)
    p = problems.MATHIEU
    n = int(math.ceil(math.pi / 0.05 - 1e-12))
    o = _oracle(p)
    r = o.solve_batch(np.zeros((1, 0)), [n], [[0.0, math.pi]], problems.mathieu_guess(n), y0_mode=1, order=4)
    assert r["retcode"][0] == RET_SUCCESS
    N = int(r["n_nodes"][0])
    lam = r["y"][0, :N, 2]
    assert np.abs(lam - 17.09658).max() < 1e-4


# MIRK6I (mirk_tableaus.jl:154-194, interpolation.jl:583-693): the reference runs it through
# the same golden tests as MIRK2-6 (mirk_basic_tests.jl:113-116, 134-137, 241-266).
@pytest.mark.parametrize("name", ["affine", "affine_twopoint"])
def test_affineness_mirk6i(problems, name):
    p = problems.ALL[name]
    o, r, N = _solve1(p, dt=0.2, order=6, mirk6i=1)
    assert r["retcode"][0] == RET_SUCCESS
    u1 = r["y"][0, :N, 0]
    assert np.abs(np.diff(u1) + 0.2).max() + abs(u1[0] - 5) < 1e-2


@pytest.mark.parametrize("name", ["linear", "linear_twopoint"])
def test_convergence_order_mirk6i(problems, name):
    p = problems.ALL[name]
    errs = []
    for dt in (1 / 8, 1 / 4, 1 / 2):
        o, r, N = _solve1(p, dt=dt, order=6, mirk6i=1, adaptive=0, max_newton=20)
        assert r["retcode"][0] == RET_SUCCESS
        t = r["mesh"][0, :N]
        errs.append(np.abs(r["y"][0, :N] - problems.linear_analytic(t)).max())
    errs = np.array(errs)
    est = np.log2(errs[1:] / errs[:-1]).mean()
    assert abs(est - 6) < 0.4, (errs, est)


def test_interpolation_twopoint_mirk6i(problems):
    p = problems.TWOPOINT_INTERP
    o, r, N = _solve1(p, dt=0.001, params=(1.0,), order=6, mirk6i=1)
    assert r["retcode"][0] == RET_SUCCESS
    mesh, y, K, KI = r["mesh"][0, :N], r["y"][0], r["K"][0], r["KI"][0]
    assert KI.shape[1] == 3
    u, du = problems.twopoint_interp_analytic(np.array([0.001]))
    assert np.abs(o.interpolate(6, mesh, y, K, KI, [0.001], mirk6i=1) - u).max() < 1e-6
    u4, du4 = problems.twopoint_interp_analytic(np.array([0.04]))
    assert np.abs(o.interpolate(6, mesh, y, K, KI, [0.04], mirk6i=1) - u4).max() < 1e-6
    assert np.abs(o.interpolate(6, mesh, y, K, KI, [0.04], deriv=1, mirk6i=1) - du4).max() < 1e-6


def test_mirk6i_interpolant_consistency(problems):
    # the continuous extension reproduces the discrete step: at τ = 1 it equals y_{i+1} and its
    # derivative at τ = 0, 1 equals f at the nodes (the weights satisfy w(1) = b, w'(0) = e1, w'(1) = e2)
    p = problems.LINEAR
    o, r, N = _solve1(p, dt=0.1, order=6, mirk6i=1, adaptive=0)
    mesh, y, K, KI = r["mesh"][0, :N], r["y"][0], r["K"][0], r["KI"][0]
    for i in (0, 3, N - 2):
        h = mesh[i + 1] - mesh[i]
        ends = o.interpolate(6, mesh, y, K, KI, [mesh[i] + 0.999999999 * h], mirk6i=1)[0]
        assert np.abs(ends - y[i + 1]).max() < 1e-8
        d0 = o.interpolate(6, mesh, y, K, KI, [mesh[i] + 1e-12 * h], deriv=1, mirk6i=1)[0]
        assert np.abs(d0 - K[i, 0]).max() < 1e-8


# ---- error controllers (Core/src/calc_errors.jl:54-139; adaptivity.jl:77-243, 361-567) ------
GLOBAL_CASES = [("global", "HO"), ("global", "RE"), ("sequential", "HO"), ("sequential", "RE"),
                ("hybrid", "HO"), ("hybrid", "RE")]


@pytest.mark.parametrize("ctl,gm", [("defect", "HO")] + GLOBAL_CASES)
def test_error_control_adaptivity(problems, ctl, gm):
    # mirk_basic_tests.jl:414-434: the pendulum with its BCs at pi/4 and pi/2, MIRK4, dt = 0.05,
    # abstol 1e-5, under each controller (GlobalErrorControl() defaults to HOErrorControl)
    p = problems.PENDULUM
    o, r, N = _solve1(p, dt=0.05, params=(9.81, 0.0, 0.0), order=4, abstol=1e-5, controller=ctl, global_method=gm)
    assert r["retcode"][0] == RET_SUCCESS
    m, y = r["mesh"][0, :N], r["y"][0, :N]
    assert o.residual((9.81, 0.0, 0.0), m, y)[2] <= 1e-5
    assert np.abs(y[:, 0]).max() < 3.0


@pytest.mark.parametrize("order", [3, 4, 5, 6])
def test_richardson_estimate_controls_the_error(problems, order):
    # GlobalErrorControl(method = REErrorControl()) on the linear problem (exact solution known):
    # the accepted estimate is within abstol, and so is the error it estimates, in the
    # estimator's measure |y - u| / (1 + |y|) (calc_errors.jl:113-127)
    p = problems.LINEAR
    o, r, N = _solve1(p, n=10, order=order, controller="global", global_method="RE")
    assert r["retcode"][0] == RET_SUCCESS
    m, y = r["mesh"][0, :N], r["y"][0, :N]
    rel = np.abs((y - problems.linear_analytic(m)) / (1 + np.abs(y))).max()
    assert r["global_err"][0] <= 1e-6 and rel <= 2e-6, (r["global_err"][0], rel)
    assert math.isnan(r["defect"][0])            # no defect pass under GlobalErrorControl


@pytest.mark.parametrize("ctl,gm", GLOBAL_CASES)
def test_global_controllers_converge_on_the_torus(problems, ctl, gm):
    # mirk_basic_tests.jl:726-756's geodesic under the other controllers
    p = problems.TORUS
    a1, a2 = (0.5, -1.2), (-0.5, 0.3)
    o, r, N = _solve1(p, dt=0.05, params=a1 + a2, order=4, controller=ctl, global_method=gm)
    assert r["retcode"][0] == RET_SUCCESS
    y = r["y"][0, :N]
    assert np.abs(y[0, :2] - a1).max() < 1e-6 and np.abs(y[-1, :2] - a2).max() < 1e-6
    assert r["global_err"][0] <= 1e-6 or (ctl == "hybrid" and r["global_err"][0] <= 2e-6)


def test_ho_error_control_needs_mirk_p_plus_2(problems):
    # __high_order_method (adaptivity.jl:552-555) names MIRK(p+2): no MIRK7 or MIRK8 exists
    p = problems.LINEAR
    with pytest.raises(ValueError, match="order"):
        _solve1(p, n=10, order=5, controller="global", global_method="HO")


# ---- FIRK, expanded form (lib/BoundaryValueDiffEqFIRK/test/expanded) ----------------------
FIRK_SCHEMES = [("LobattoIIIa", s) for s in (2, 3, 4, 5)] + [("LobattoIIIb", s) for s in (2, 3, 4, 5)] + \
               [("LobattoIIIc", s) for s in (2, 3, 4, 5)] + [("RadauIIa", s) for s in (2, 3, 5, 7)]


@pytest.mark.parametrize("family,stages", FIRK_SCHEMES)
@pytest.mark.parametrize("name", ["affine", "affine_twopoint"])
def test_firk_affineness(problems, name, family, stages):
    # firk_affineness_tests.jl:6-29: u1 = 5 - t exactly, dt = 0.2, non-adaptive, affineTol 1e-2
    p = problems.ALL[name]
    o = _oracle(p)
    r = o.firk_solve_batch(family, stages, np.zeros((1, 1)), [25], [p.tspan], [p.u0], adaptive=0)
    assert r["retcode"][0] == RET_SUCCESS
    u1 = r["y"][0, :26, 0]
    assert np.abs(np.diff(u1) + 0.2).max() + abs(u1[0] - 5) < 1e-2


@pytest.mark.parametrize("family,stages", FIRK_SCHEMES)
@pytest.mark.parametrize("name", ["linear", "linear_twopoint"])
def test_firk_convergence_order(problems, name, family, stages):
    # firk_convergence_tests.jl:6-57: the error at the nodes falls at order 2s - 2 (Lobatto) or
    # 2s - 1 (Radau IIA), testTol 0.3, on dt = 1/8, 1/16, 1/32 (1/4 .. 1/16 for four stages);
    # estimates where the error is already at roundoff are not judged (the reference marks them
    # broken)
    p = problems.ALL[name]
    o = _oracle(p)
    dts = (1 / 4, 1 / 8, 1 / 16) if stages == 4 else (1 / 8, 1 / 16, 1 / 32)
    errs = []
    for dt in dts:
        n = int(round(5.0 / dt))
        r = o.firk_solve_batch(family, stages, np.zeros((1, 1)), [n], [p.tspan], [p.u0], adaptive=0, abstol=1e-8)
        assert r["retcode"][0] == RET_SUCCESS
        m, y = r["mesh"][0, :n + 1], r["y"][0, :n + 1]
        errs.append(np.abs(y - problems.linear_analytic(m)).max())
    order = 2 * stages - 1 if family == "RadauIIa" else 2 * stages - 2
    if errs[-1] < 1e-12:
        return
    est = np.log2(errs[-2] / errs[-1])
    assert abs(est - order) < 0.3, (errs, est)


def test_firk_tableaus_match_the_reference_tables(problems):
    # the coefficients, computed from their defining conditions, against entries the reference
    # tabulates (radau_tableaus.jl:47-69, lobatto_tableaus.jl:136-160, 244-266)
    o = _oracle(problems.LINEAR)
    order, s, tau, c, b, a, q = o.firk_tableau("RadauIIa", 3)
    assert order == 5 and tau == 0.0
    assert np.allclose(q, [[1.5580782047249224, -0.8914115380582555, 0.33333333333333315],
                           [-1.9869472213484427, 3.320280554681775, -1.3333333333333326],
                           [0.8052720793239877, -1.9163831904350983, 1.1111111111111107]], rtol=0, atol=1e-13)
    assert np.allclose(b, [4 / 9 - math.sqrt(6) / 36, 4 / 9 + math.sqrt(6) / 36, 1 / 9], atol=1e-15)
    assert np.allclose(a[0], [11 / 45 - 7 * math.sqrt(6) / 360, 37 / 225 - 169 * math.sqrt(6) / 1800,
                              -2 / 225 + math.sqrt(6) / 75], atol=1e-15)
    _, _, tau_b, _, _, ab, _ = o.firk_tableau("LobattoIIIb", 3)
    assert np.allclose(ab, [[1 / 6, -1 / 6, 0], [1 / 6, 1 / 3, 0], [1 / 6, 5 / 6, 0]], atol=1e-15)
    _, _, tau_c, _, _, ac, _ = o.firk_tableau("LobattoIIIc", 3)
    assert np.allclose(ac, [[1 / 6, -1 / 3, 1 / 6], [1 / 6, 5 / 12, -1 / 12], [1 / 6, 2 / 3, 1 / 6]], atol=1e-15)
    assert tau_b == 0.21132486540518713 and tau_c == 0.7886751345948129
    _, _, _, _, _, _, q5 = o.firk_tableau("RadauIIa", 5)
    assert np.allclose(q5[0], [1.5864079001863276, -1.0081178814983707, 0.7309748661597844,
                               -0.5092648848477398, 0.19999999999999882], atol=1e-10)


@pytest.mark.parametrize("family,stages", [("RadauIIa", 2), ("RadauIIa", 3), ("RadauIIa", 5), ("RadauIIa", 7),
                                           ("LobattoIIIa", 3), ("LobattoIIIb", 4), ("LobattoIIIc", 5)])
def test_firk_ensemble_converges(problems, family, stages):
    # ensemble_tests.jl:4-95: u'' = -p u on (0, pi/2) over random p, every trajectory converges
    # (adaptive); the second BC at the tspan's end (the FIRK path evaluates BCs at the ends, the
    # reference's test at t = 1)
    import dataclasses
    p = dataclasses.replace(problems.ENSEMBLE, bc_t=(0.0, math.pi / 2))
    o = _oracle(p)
    rng = np.random.default_rng(3)
    params = rng.uniform(0.5, 1.5, (16, 1))
    n = int(math.ceil((math.pi / 2) / 0.1 - 1e-12))
    r = o.firk_solve_batch(family, stages, params, [n] * 16, [p.tspan] * 16, [p.u0] * 16)
    assert (r["retcode"] == RET_SUCCESS).all()
