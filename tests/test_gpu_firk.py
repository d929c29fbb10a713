"""The FIRK path (Radau IIA and Lobatto IIIA/IIIB/IIIC in the expanded form,
lib/BoundaryValueDiffEqFIRK) on the GPU against the oracle.

Both solve in FP64 with NewtonRaphson and the same step (the GPU eliminates each interval's
stage unknowns inside the structured node solve, as the oracle does), so the retcodes, Newton
iterations, mesh rounds and meshes agree, and the nodes agree to 1e-9 relative. The
reference's own FIRK tests run on the GPU as well: affineness (firk_affineness_tests.jl),
convergence orders 2s - 1 / 2s - 2 (firk_convergence_tests.jl) and the adaptive ensemble
(ensemble_tests.jl, its second BC moved to the tspan's end)."""
import dataclasses
import math

import numpy as np
import pytest

from oracle.oracle import Oracle, RET_SUCCESS, RET_FAILURE

pytestmark = pytest.mark.gpu

SCHEMES = [("LobattoIIIa", s) for s in (2, 3, 4, 5)] + [("LobattoIIIb", s) for s in (2, 3, 4, 5)] + \
          [("LobattoIIIc", s) for s in (2, 3, 4, 5)] + [("RadauIIa", s) for s in (1, 2, 3, 5, 7)]
ADAPTIVE = [sc for sc in SCHEMES if sc not in (("RadauIIa", 1), ("LobattoIIIb", 2), ("LobattoIIIc", 2))]


def _oracle(p):
    return Oracle(p.source, p.M, p.n_params, twopoint=p.twopoint, bc_t=p.bc_t, La=p.La, Lb=p.Lb)


def _match(res, ref, rtol=1e-9):
    assert (res.retcode == ref["retcode"]).all(), (res.retcode, ref["retcode"])
    assert (res.newton_iters == ref["newton_iters"]).all(), (res.newton_iters, ref["newton_iters"])
    assert (res.rounds == ref["rounds"]).all(), (res.rounds, ref["rounds"])
    assert (res.n_nodes == ref["n_nodes"]).all(), (res.n_nodes, ref["n_nodes"])
    for i in range(len(res.n_nodes)):
        N = int(ref["n_nodes"][i])
        m, y = res.solution(i)
        assert np.abs(m - ref["mesh"][i, :N]).max() <= 1e-9 * max(1.0, np.abs(m).max()), i
        yr = ref["y"][i, :N]
        assert np.abs(y - yr).max() <= rtol * max(1.0, np.abs(yr).max()), (i, np.abs(y - yr).max())


def _linear_batch():
    nint = np.array([5, 8, 10, 13, 20, 32], np.int32)
    n = len(nint)
    return np.zeros((n, 0)), nint, np.tile([0.0, 5.0], (n, 1)), np.tile([5.0, -3.5], (n, 1))


@pytest.mark.parametrize("family,stages", SCHEMES)
@pytest.mark.parametrize("name", ["linear", "linear_twopoint"])
def test_firk_nonadaptive_matches_oracle(pkg, problems, name, family, stages):
    p = problems.ALL[name]
    params, nint, tsp, y0 = _linear_batch()
    sv = pkg.BatchSolver(p, abstol=1e-8, adaptive=0, firk=family, firk_stages=stages)
    res = sv.solve(params, nint, tsp, y0)
    ref = _oracle(p).firk_solve_batch(family, stages, params, nint, tsp, y0, adaptive=0, abstol=1e-8)
    _match(res, ref)


@pytest.mark.parametrize("family,stages", ADAPTIVE)
def test_firk_adaptive_matches_oracle(pkg, problems, family, stages):
    p = problems.LINEAR
    params, nint, tsp, y0 = _linear_batch()
    res = pkg.BatchSolver(p, firk=family, firk_stages=stages).solve(params, nint, tsp, y0)
    ref = _oracle(p).firk_solve_batch(family, stages, params, nint, tsp, y0)
    _match(res, ref)
    assert (res.retcode == RET_SUCCESS).all()


@pytest.mark.parametrize("family,stages", [("RadauIIa", 3), ("RadauIIa", 5), ("LobattoIIIa", 4), ("LobattoIIIc", 3)])
def test_firk_torus_matches_oracle(pkg, problems, family, stages):
    # a nonlinear four-state problem: several Newton iterations and mesh rounds
    p = problems.TORUS
    rng = np.random.default_rng(61)
    n = 8
    params = np.concatenate([rng.uniform(-0.8, 0.8, (n, 2)), rng.uniform(-0.8, 0.8, (n, 2))], 1)
    nint = rng.integers(8, 30, n).astype(np.int32)
    tsp = np.tile([0.0, 1.0], (n, 1))
    y0 = np.tile([0.5, -1.2, 0.0, 0.0], (n, 1))
    res = pkg.BatchSolver(p, firk=family, firk_stages=stages).solve(params, nint, tsp, y0)
    ref = _oracle(p).firk_solve_batch(family, stages, params, nint, tsp, y0)
    assert (ref["retcode"] == RET_SUCCESS).all()
    _match(res, ref, rtol=1e-8)


@pytest.mark.parametrize("family,stages", [("LobattoIIIa", 2), ("LobattoIIIb", 3), ("LobattoIIIc", 4), ("RadauIIa", 7)])
@pytest.mark.parametrize("name", ["affine", "affine_twopoint"])
def test_firk_affineness_gpu(pkg, problems, name, family, stages):
    # firk_affineness_tests.jl:6-29
    p = problems.ALL[name]
    res = pkg.BatchSolver(p, adaptive=0, firk=family, firk_stages=stages).solve(
        np.zeros((1, 0)), [25], [p.tspan], [p.u0])
    assert res.retcode[0] == RET_SUCCESS
    u1 = res.solution(0)[1][:, 0]
    assert np.abs(np.diff(u1) + 0.2).max() + abs(u1[0] - 5) < 1e-2


@pytest.mark.parametrize("family,stages", [("LobattoIIIa", 3), ("LobattoIIIb", 3), ("LobattoIIIc", 3), ("RadauIIa", 2),
                                           ("RadauIIa", 3)])
def test_firk_convergence_order_gpu(pkg, problems, family, stages):
    # firk_convergence_tests.jl:6-57 on the linear problem
    p = problems.LINEAR
    sv = pkg.BatchSolver(p, abstol=1e-8, adaptive=0, firk=family, firk_stages=stages)
    errs = []
    for dt in (1 / 8, 1 / 16, 1 / 32):
        n = int(round(5.0 / dt))
        res = sv.solve(np.zeros((1, 0)), [n], [[0.0, 5.0]], [[5.0, -3.5]])
        m, y = res.solution(0)
        errs.append(np.abs(y - problems.linear_analytic(m)).max())
    order = 2 * stages - 1 if family == "RadauIIa" else 2 * stages - 2
    assert abs(np.log2(errs[-2] / errs[-1]) - order) < 0.3, errs


def test_firk_ensemble_gpu(pkg, problems):
    # ensemble_tests.jl:4-95 (second BC at the tspan's end), through the SciML-style API
    sc = pkg.sciml
    p = dataclasses.replace(problems.ENSEMBLE, name="ensemble_end", bc_t=(0.0, math.pi / 2))
    rng = np.random.default_rng(5)
    for alg in (sc.RadauIIa2(), sc.RadauIIa5(), sc.LobattoIIIa4(), sc.LobattoIIIb3(), sc.LobattoIIIc5()):
        sols = sc.solve(sc.EnsembleProblem(p, params=rng.uniform(0.2, 1.0, (10, 1))), alg, dt=0.1)
        assert all(s.successful for s in sols)


def test_firk_interior_bc_fails_alone(pkg, problems):
    # standard BCs at a time inside the tspan are not covered on the FIRK path: those
    # instances fail with flag bit 2, the others in the batch solve
    p = problems.ENSEMBLE                       # BC at t = 1 inside (0, pi/2)
    sv = pkg.BatchSolver(p, firk="RadauIIa", firk_stages=3)
    tsp = np.array([[0.0, math.pi / 2], [0.0, 1.0]])
    res = sv.solve(np.array([[0.5], [0.5]]), [16, 10], tsp, [p.u0, p.u0])
    assert res.retcode[0] == RET_FAILURE and res.retcode[1] == RET_SUCCESS


def test_firk_options_are_validated(pkg, problems):
    with pytest.raises(pkg.BVPError):
        pkg.BatchSolver(problems.LINEAR, firk="RadauIIa", firk_stages=4)
    with pytest.raises(pkg.BVPError):
        pkg.BatchSolver(problems.LINEAR, firk="RadauIIa", firk_stages=1)       # no adaptivity
    with pytest.raises(pkg.BVPError):
        pkg.BatchSolver(problems.LINEAR, firk="LobattoIIIa", firk_stages=3, want_stages=1)
