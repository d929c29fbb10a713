"""The reference's calling convention on top of the batched library.

    sol = solve(problem, MIRK4(), dt=0.05, abstol=1e-6)          # one problem
    sol.t, sol.u, sol.retcode, sol(0.3), sol(0.3, deriv=1)
    sols = solve(EnsembleProblem(problem, params=P), MIRK4(), dt=0.05)   # one batched call

mirrors ``solve(prob::BVProblem, MIRK4(); dt, abstol)`` (lib/BoundaryValueDiffEqMIRK/src/
mirk.jl:49-53, 286-332) and ``solve(EnsembleProblem(prob, ...), MIRK4(), ...; trajectories)``
(test/Core/ensemble_tests.jl:7-41): the same argument meanings, ``dt`` turned into
``cld(t1 - t0, dt)`` uniform intervals (lib/BoundaryValueDiffEqCore/src/utils.jl:349-363),
the same argument error for ``dt <= 0`` (utils.jl:354), the same return codes and the
interpolant as ``sol(t)`` (interpolation.jl:17-206, evaluated on the GPU). A
``problems.Problem`` plays the role of the BVProblem / TwoPointBVProblem: its CUDA C source
holds f and the BCs. Every solve runs on the GPU through ``BatchSolver``; handles are cached
per (problem, algorithm, options).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .solver import BatchSolver, RET_SUCCESS, RET_MAXITERS

RETCODES = {0: "Success", 1: "Failure", 2: "MaxIters"}


@dataclass(frozen=True)
class MIRK:
    """MIRKn() (lib/BoundaryValueDiffEqMIRK/src/algorithms.jl): the order plus the solver options
    this library exposes (Jacobian precision, mesh cap, defect threshold)."""
    order: int
    jac_precision: int = 32
    max_num_subintervals: int = 3000
    defect_threshold: float = 0.1
    mirk6i: bool = False          # MIRK6I() (mirk_tableaus.jl:154-194): order 6, own interpolant

    def __post_init__(self):
        if self.order not in (2, 3, 4, 5, 6):
            raise ValueError(f"MIRK order must be 2..6, got {self.order}")
        if self.mirk6i and self.order != 6:
            raise ValueError("MIRK6I is an order-6 scheme")
        if self.jac_precision not in (32, 64):
            raise ValueError("jac_precision must be 32 or 64")


@dataclass(frozen=True)
class HOErrorControl:
    """The global error from a MIRK(p+2) solve on the same mesh (calc_errors.jl:99-110)."""


@dataclass(frozen=True)
class REErrorControl:
    """The global error by Richardson extrapolation from the halved mesh (calc_errors.jl:113-127)."""


@dataclass(frozen=True)
class DefectControl:
    """DefectControl(; defect_threshold = 0.1) (calc_errors.jl:54-60): the default controller."""
    defect_threshold: float = 0.1


@dataclass(frozen=True)
class GlobalErrorControl:
    """GlobalErrorControl(; method = HOErrorControl()) (calc_errors.jl:67-73)."""
    method: object = HOErrorControl()


@dataclass(frozen=True)
class SequentialErrorControl:
    """SequentialErrorControl(; defect, global_error) (calc_errors.jl:80-87): the defect first,
    the global error once the defect is within abstol."""
    defect: DefectControl = DefectControl()
    global_error: GlobalErrorControl = GlobalErrorControl()


@dataclass(frozen=True)
class HybridErrorControl:
    """HybridErrorControl(; DE = 1.0, GE = 1.0, defect, global_error) (calc_errors.jl:93-107):
    the norm DE * defect + GE * global error."""
    DE: float = 1.0
    GE: float = 1.0
    defect: DefectControl = DefectControl()
    global_error: GlobalErrorControl = GlobalErrorControl()


def _controller_options(c) -> dict:
    """The C ABI's controller fields for a controller object."""
    def method(g):
        if isinstance(g.method, HOErrorControl):
            return 0
        if isinstance(g.method, REErrorControl):
            return 1
        raise TypeError(f"unknown global error method {g.method!r}")
    if isinstance(c, DefectControl):
        return dict(controller=0, defect_threshold=c.defect_threshold)
    if isinstance(c, GlobalErrorControl):
        return dict(controller=1, global_method=method(c))
    if isinstance(c, SequentialErrorControl):
        return dict(controller=2, global_method=method(c.global_error), defect_threshold=c.defect.defect_threshold)
    if isinstance(c, HybridErrorControl):
        return dict(controller=3, global_method=method(c.global_error), hybrid_de=float(c.DE),
                    hybrid_ge=float(c.GE), defect_threshold=c.defect.defect_threshold)
    raise TypeError(f"unknown error controller {c!r}")


@dataclass(frozen=True)
class FIRK:
    """A FIRK algorithm in the expanded form (lib/BoundaryValueDiffEqFIRK/src/algorithms.jl):
    family "RadauIIa", "LobattoIIIa", "LobattoIIIb" or "LobattoIIIc" with `stages` stages,
    solved in FP64 throughout."""
    family: str
    stages: int
    max_num_subintervals: int = 3000
    defect_threshold: float = 0.1

    def __post_init__(self):
        ok = {"RadauIIa": (1, 2, 3, 5, 7), "LobattoIIIa": (2, 3, 4, 5), "LobattoIIIb": (2, 3, 4, 5),
              "LobattoIIIc": (2, 3, 4, 5)}
        if self.stages not in ok.get(self.family, ()):
            raise ValueError(f"no FIRK scheme {self.family}{self.stages}")


def RadauIIa1(**kw): return FIRK("RadauIIa", 1, **kw)  # noqa: E704
def RadauIIa2(**kw): return FIRK("RadauIIa", 2, **kw)  # noqa: E704
def RadauIIa3(**kw): return FIRK("RadauIIa", 3, **kw)  # noqa: E704
def RadauIIa5(**kw): return FIRK("RadauIIa", 5, **kw)  # noqa: E704
def RadauIIa7(**kw): return FIRK("RadauIIa", 7, **kw)  # noqa: E704
def LobattoIIIa2(**kw): return FIRK("LobattoIIIa", 2, **kw)  # noqa: E704
def LobattoIIIa3(**kw): return FIRK("LobattoIIIa", 3, **kw)  # noqa: E704
def LobattoIIIa4(**kw): return FIRK("LobattoIIIa", 4, **kw)  # noqa: E704
def LobattoIIIa5(**kw): return FIRK("LobattoIIIa", 5, **kw)  # noqa: E704
def LobattoIIIb2(**kw): return FIRK("LobattoIIIb", 2, **kw)  # noqa: E704
def LobattoIIIb3(**kw): return FIRK("LobattoIIIb", 3, **kw)  # noqa: E704
def LobattoIIIb4(**kw): return FIRK("LobattoIIIb", 4, **kw)  # noqa: E704
def LobattoIIIb5(**kw): return FIRK("LobattoIIIb", 5, **kw)  # noqa: E704
def LobattoIIIc2(**kw): return FIRK("LobattoIIIc", 2, **kw)  # noqa: E704
def LobattoIIIc3(**kw): return FIRK("LobattoIIIc", 3, **kw)  # noqa: E704
def LobattoIIIc4(**kw): return FIRK("LobattoIIIc", 4, **kw)  # noqa: E704
def LobattoIIIc5(**kw): return FIRK("LobattoIIIc", 5, **kw)  # noqa: E704


def MIRK2(**kw): return MIRK(2, **kw)  # noqa: E704
def MIRK3(**kw): return MIRK(3, **kw)  # noqa: E704
def MIRK4(**kw): return MIRK(4, **kw)  # noqa: E704
def MIRK5(**kw): return MIRK(5, **kw)  # noqa: E704
def MIRK6(**kw): return MIRK(6, **kw)  # noqa: E704
def MIRK6I(**kw): return MIRK(6, mirk6i=True, **kw)  # noqa: E704


@dataclass
class EnsembleProblem:
    """A batch of trajectories of one problem: per-trajectory parameters (n x n_params), and
    optionally per-trajectory time spans (n x 2) and constant initial guesses (n x M)."""
    problem: object
    params: np.ndarray | None = None
    tspans: np.ndarray | None = None
    u0: np.ndarray | None = None
    trajectories: int | None = None


class _Batch:
    """The handle and the batch a solution came from; the handle's dense output stays valid
    until it solves another batch."""

    def __init__(self, solver, n_inst):
        self.solver = solver
        self.n_inst = n_inst
        self.generation = _GEN.get(id(solver), 0) + 1
        _GEN[id(solver)] = self.generation

    def current(self) -> bool:
        return _GEN.get(id(self.solver)) == self.generation


_GEN: dict = {}


@dataclass
class BVPSolution:
    """The ODESolution of a solve (mirk.jl:324-331): nodes ``t``, values ``u`` (N x M), the
    return code, and the MIRK interpolant as ``sol(t)`` / ``sol(t, deriv=1)``, evaluated on the
    GPU by the library's dense output (``bvp_dense_output``)."""
    t: np.ndarray
    u: np.ndarray
    retcode: str
    newton_iters: int
    rounds: int
    _batch: _Batch | None = field(default=None, repr=False)
    _index: int = 0

    @property
    def successful(self) -> bool:
        return self.retcode == "Success"

    def __call__(self, tq, deriv: int = 0):
        """u(t) or u'(t) at a scalar or an array of times."""
        b = self._batch
        if b is None:
            raise ValueError("no dense output: solve with dense=True")
        if not b.current():
            raise ValueError("the solver handle has solved another batch since this solution; "
                             "evaluate sol(t) before the next solve on the same problem and algorithm")
        tq_arr = np.atleast_1d(np.asarray(tq, dtype=np.float64))
        out = b.solver.dense(np.tile(tq_arr, (b.n_inst, 1)), deriv=deriv)[self._index]
        return out[0] if np.ndim(tq) == 0 else out


def _n_intervals(tspan, dt) -> int:
    if not dt > 0:
        raise ValueError("dt must be positive")           # ArgumentError, Core/src/utils.jl:354
    t0, t1 = float(tspan[0]), float(tspan[1])
    if not t1 > t0:
        raise ValueError("tspan must satisfy t0 < t1")
    return int(math.ceil((t1 - t0) / dt - 1e-12))         # cld(t1 - t0, dt)


_CACHE: dict = {}


def _solver(problem, alg: MIRK, abstol, adaptive, dense, solver_cls, controller=None):
    key = (problem.name, problem.source, alg, float(abstol), int(adaptive), int(dense), solver_cls, controller)
    sv = _CACHE.get(key)
    if sv is None:
        opts = dict(defect_threshold=alg.defect_threshold)
        if controller is not None:
            opts.update(_controller_options(controller))
        if isinstance(alg, FIRK):
            # no stage output on the FIRK path: sol(t) is not available there
            sv = solver_cls(problem, order=4, abstol=abstol, jac_precision=64, adaptive=int(adaptive),
                            max_subintervals=alg.max_num_subintervals, firk=alg.family, firk_stages=alg.stages,
                            **opts)
        else:
            sv = solver_cls(problem, order=alg.order, abstol=abstol, jac_precision=alg.jac_precision,
                            adaptive=int(adaptive), want_stages=int(dense),
                            max_subintervals=alg.max_num_subintervals, mirk6i=int(alg.mirk6i), **opts)
        _CACHE[key] = sv
    return sv


def _to_solutions(res, solver, dense):
    n = len(res.n_nodes)
    batch = _Batch(solver, n) if dense and not getattr(getattr(solver, "options", None), "firk", 0) else None
    out = []
    for i in range(n):
        m, y = res.solution(i)
        out.append(BVPSolution(t=np.array(m), u=np.array(y), retcode=RETCODES.get(int(res.retcode[i]), "Failure"),
                               newton_iters=int(res.newton_iters[i]), rounds=int(res.rounds[i]),
                               _batch=batch, _index=i))
    return out


def solve(prob, alg, *, dt: float, abstol: float = 1e-6, adaptive: bool = True, p=None, u0=None,
          dense: bool = True, controller=None, _solver_cls=BatchSolver):
    """solve(prob, MIRKn(); dt, abstol, controller) for one problem, or for an EnsembleProblem
    (one batched call over its trajectories). ``u0`` is a constant guess (M values) or per-node
    guesses on the initial uniform mesh ((n + 1) x M); ``p`` the parameters; ``controller`` one
    of DefectControl() (the default), GlobalErrorControl(), SequentialErrorControl(),
    HybridErrorControl() (mirk.jl:50-51)."""
    if isinstance(prob, EnsembleProblem):
        base = prob.problem
        n = prob.trajectories or (len(prob.params) if prob.params is not None else 1)
        params = (np.zeros((n, 0)) if prob.params is None
                  else np.asarray(prob.params, dtype=np.float64).reshape(n, -1))
        tsp = (np.tile(np.asarray(base.tspan, dtype=np.float64), (n, 1)) if prob.tspans is None
               else np.asarray(prob.tspans, dtype=np.float64).reshape(n, 2))
        y0 = (np.tile(np.asarray(base.u0, dtype=np.float64), (n, 1)) if prob.u0 is None
              else np.asarray(prob.u0, dtype=np.float64).reshape(n, base.M))
        nint = np.array([_n_intervals(ts, dt) for ts in tsp], np.int32)
        sv = _solver(base, alg, abstol, adaptive, dense, _solver_cls, controller)
        res = sv.solve(params, nint, tsp, y0, y0_mode=0)
        return _to_solutions(res, sv, dense)
    n = _n_intervals(prob.tspan, dt)
    params = np.asarray(() if p is None else p, dtype=np.float64).reshape(1, -1)
    if params.shape[1] != prob.n_params:
        raise ValueError(f"the problem takes {prob.n_params} parameters, got {params.shape[1]}")
    guess = np.asarray(prob.u0 if u0 is None else u0, dtype=np.float64)
    if guess.size == prob.M:
        y0, mode = guess.reshape(1, prob.M), 0
    elif guess.shape == (n + 1, prob.M):
        y0, mode = guess, 1
    else:
        raise ValueError(f"u0 must hold {prob.M} values or ({n + 1}, {prob.M}) per-node values")
    sv = _solver(prob, alg, abstol, adaptive, dense, _solver_cls, controller)
    res = sv.solve(params, np.array([n], np.int32), np.asarray([prob.tspan], dtype=np.float64), y0, y0_mode=mode)
    return _to_solutions(res, sv, dense)[0]


__all__ = ["solve", "MIRK", "MIRK2", "MIRK3", "MIRK4", "MIRK5", "MIRK6", "MIRK6I", "EnsembleProblem", "BVPSolution",
           "FIRK", "RadauIIa1", "RadauIIa2", "RadauIIa3", "RadauIIa5", "RadauIIa7", "LobattoIIIa2", "LobattoIIIa3",
           "LobattoIIIa4", "LobattoIIIa5", "LobattoIIIb2", "LobattoIIIb3", "LobattoIIIb4", "LobattoIIIb5",
           "LobattoIIIc2", "LobattoIIIc3", "LobattoIIIc4", "LobattoIIIc5",
           "DefectControl", "GlobalErrorControl", "SequentialErrorControl", "HybridErrorControl",
           "HOErrorControl", "REErrorControl", "RET_SUCCESS", "RET_MAXITERS"]
