"""The reference-style front end (``sciml.solve``): argument handling, the dt -> interval
count rule, return codes, ensembles and the dense-output contract, checked on the CPU with a
stand-in for the GPU solver (the GPU path itself is covered by tests/test_gpu_solve.py)."""
import math

import numpy as np
import pytest


class FakeResult:
    def __init__(self, nint, tsp, M, retcode):
        self.n_nodes = np.asarray(nint, np.int32) + 1
        self.retcode = np.asarray(retcode, np.int32)
        self.newton_iters = np.full(len(nint), 3, np.int32)
        self.rounds = np.ones(len(nint), np.int32)
        self._tsp, self._M = tsp, M

    def solution(self, i):
        n = int(self.n_nodes[i])
        m = np.linspace(self._tsp[i][0], self._tsp[i][1], n)
        return m, np.tile(np.arange(self._M, dtype=float), (n, 1)) + i


class FakeSolver:
    created = []

    def __init__(self, problem, **kw):
        self.problem, self.kw, self.calls = problem, kw, []
        FakeSolver.created.append(self)

    def solve(self, params, nint, tsp, y0, y0_mode=None):
        self.calls.append((np.array(params), np.array(nint), np.array(tsp), np.array(y0), y0_mode))
        rc = [0] * len(nint)
        if len(nint) > 1:
            rc[1] = 2
        return FakeResult(nint, tsp, self.problem.M, rc)

    def dense(self, tq, deriv=0):
        n, nq = tq.shape
        return np.stack([np.repeat((tq[i] + 100 * i + 1000 * deriv)[:, None], self.problem.M, 1) for i in range(n)])


@pytest.fixture
def sciml(pkg):
    pkg.sciml._CACHE.clear()
    FakeSolver.created.clear()
    return pkg.sciml


def test_dt_rule_and_single_problem(sciml, problems):
    p = problems.PENDULUM
    sol = sciml.solve(p, sciml.MIRK4(), dt=0.05, p=[9.81, 0.0, 0.0], _solver_cls=FakeSolver)
    sv = FakeSolver.created[0]
    params, nint, tsp, y0, mode = sv.calls[0]
    assert nint.tolist() == [32]                      # cld(pi/2, 0.05), Core/src/utils.jl:349-363
    assert mode == 0 and y0.shape == (1, 2) and params.shape == (1, 3)
    assert sv.kw["order"] == 4 and sv.kw["want_stages"] == 1 and sv.kw["adaptive"] == 1
    assert sol.retcode == "Success" and sol.successful and len(sol.t) == 33
    # the same handle is reused for the same problem, algorithm and options
    sciml.solve(p, sciml.MIRK4(), dt=0.05, p=[9.81, 0.0, 0.0], _solver_cls=FakeSolver)
    assert len(FakeSolver.created) == 1 and len(sv.calls) == 2


def test_argument_errors(sciml, problems):
    p = problems.PENDULUM
    for dt in (0.0, -0.1):
        with pytest.raises(ValueError, match="dt must be positive"):   # ArgumentError, utils.jl:354
            sciml.solve(p, sciml.MIRK4(), dt=dt, p=[9.81, 0, 0], _solver_cls=FakeSolver)
    with pytest.raises(ValueError, match="parameters"):
        sciml.solve(p, sciml.MIRK4(), dt=0.05, _solver_cls=FakeSolver)
    with pytest.raises(ValueError, match="u0"):
        sciml.solve(p, sciml.MIRK4(), dt=0.05, p=[9.81, 0, 0], u0=np.zeros((5, 2)), _solver_cls=FakeSolver)
    with pytest.raises(ValueError, match="order"):
        sciml.MIRK(7)
    assert FakeSolver.created == []


def test_per_node_guess(sciml, problems):
    p = problems.MATHIEU
    n = int(math.ceil(math.pi / 0.05 - 1e-12))
    sciml.solve(p, sciml.MIRK4(), dt=0.05, u0=problems.mathieu_guess(n), _solver_cls=FakeSolver)
    params, nint, tsp, y0, mode = FakeSolver.created[0].calls[0]
    assert mode == 1 and y0.shape == (n + 1, 3) and nint.tolist() == [n]


def test_ensemble_and_dense_output(sciml, problems):
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(3, seed=1)
    sols = sciml.solve(sciml.EnsembleProblem(p, params=params, tspans=tsp), sciml.MIRK6(), dt=0.1,
                       _solver_cls=FakeSolver)
    assert [s.retcode for s in sols] == ["Success", "MaxIters", "Success"]
    sv = FakeSolver.created[0]
    assert sv.calls[0][1].tolist() == [16, 16, 16] and sv.kw["order"] == 6
    # sol(t) is the handle's dense output for this trajectory
    assert sols[2](0.5)[0] == pytest.approx(200.5)
    assert sols[1]([0.1, 0.2], deriv=1)[:, 0] == pytest.approx([1100.1, 1100.2])
    # after the handle solves another batch the old solutions' dense output is refused
    sciml.solve(sciml.EnsembleProblem(p, params=params, tspans=tsp), sciml.MIRK6(), dt=0.1, _solver_cls=FakeSolver)
    with pytest.raises(ValueError, match="another batch"):
        sols[0](0.3)


def test_mirk6i_algorithm_reaches_the_solver(sciml, problems):
    # MIRK6I() (exported by the reference, BoundaryValueDiffEqMIRK.jl:179) selects the order-6
    # scheme with its own tableau and interpolant
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(3, seed=1)
    sciml.solve(sciml.EnsembleProblem(p, params=params, tspans=tsp), sciml.MIRK6I(), dt=0.1, _solver_cls=FakeSolver)
    kw = FakeSolver.created[-1].kw
    assert kw["order"] == 6 and kw["mirk6i"] == 1
    with pytest.raises(ValueError):
        sciml.MIRK(4, mirk6i=True)
