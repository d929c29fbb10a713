"""Block mode (bvp_options.block_min): a long mesh solved by a whole 128-thread block, its
residuals and defect spread over the block's four warps, gives exactly the results of the
same instance solved by one warp. Each interval's residual, stages and defect do not depend on
which lane computes them and the norms are maxima, so the comparison is bitwise: retcodes,
iteration and round counts, meshes, solutions, stages, norms."""
import numpy as np
import pytest

from oracle.oracle import RET_SUCCESS

pytestmark = pytest.mark.gpu

_FIELDS = ("retcode", "n_nodes", "newton_iters", "rounds", "defect", "resid")


def _same(a, b, stages=False):
    # per instance: the packed layout follows the order in which instances finish
    for f in _FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    for i in range(len(a.n_nodes)):
        for x, y in zip(a.solution(i), b.solution(i)):
            assert np.array_equal(x, y), i
        if stages:
            for x, y in zip(a.stages(i), b.stages(i)):
                assert np.array_equal(x, y), i


def _solve(pkg, prob, order, batch, block_min, **kw):
    return pkg.BatchSolver(prob, order=order, block_min=block_min, **kw).solve(*batch)


@pytest.mark.parametrize("jac_precision", [32, 64])
def test_long_meshes_block_equals_warp(pkg, problems, jac_precision):
    # 48 singularly perturbed instances, 512-4096 intervals, MIRK6: all of them in block mode
    # (block_min 1), none (-1), and the longer ones only (2048)
    p = problems.SINGULAR_PERTURBATION
    params, nint, tsp, y0 = problems.singular_perturbation_family(48, seed=7)
    assert (nint >= 2048).any() and (nint < 2048).any()
    batch = (params, nint, tsp, y0)
    ref = _solve(pkg, p, 6, batch, -1, jac_precision=jac_precision, want_stages=1)
    assert (ref.retcode == RET_SUCCESS).all()
    for bm in (1, 2048):
        _same(_solve(pkg, p, 6, batch, bm, jac_precision=jac_precision, want_stages=1), ref, stages=True)


def test_interior_bc_block_equals_warp(pkg, problems):
    # the pendulum's BC at t = pi/4 is evaluated from the interpolant by the lane whose
    # intervals hold it, which in block mode can be any of the 128 lanes; refinement rounds
    p = problems.PENDULUM
    batch = problems.pendulum_family(96, seed=11)
    ref = _solve(pkg, p, 4, batch, -1)
    assert (ref.rounds > 1).any()
    _same(_solve(pkg, p, 4, batch, 1), ref)
    _same(_solve(pkg, p, 4, batch, 128), ref)


def test_block_mode_failures_and_line_search(pkg, problems):
    # instances that end in Failure (mesh cap below the refined size) and the FP64 Newton's
    # line search: the control flow stays on the leader warp, the helpers follow its commands
    p = problems.SINGULAR_PERTURBATION
    params, nint, tsp, y0 = problems.singular_perturbation_family(32, seed=8, n_min=128, n_max=1024)
    batch = (params, nint, tsp, y0)
    ref = _solve(pkg, p, 6, batch, -1, max_subintervals=600)
    assert (ref.retcode != RET_SUCCESS).any()
    _same(_solve(pkg, p, 6, batch, 1, max_subintervals=600), ref)


def test_block_mode_selection(pkg, problems):
    # the library's threshold (512 initial intervals): a batch whose largest mesh reaches it runs
    # the block-mode module, others the warp kernels; block_min -1 turns it off
    sp = problems.SINGULAR_PERTURBATION
    batch = problems.singular_perturbation_family(8, seed=9)
    sv = pkg.BatchSolver(sp, order=6)
    sv.solve(*batch)
    t = sv.tuning()
    assert t["block_min"] == 512 and t["last_solve_block_mode"]
    short = problems.singular_perturbation_family(8, seed=9, n_min=64, n_max=256)
    sv.solve(*short)
    assert not sv.tuning()["last_solve_block_mode"]
    off = pkg.BatchSolver(sp, order=6, block_min=-1)
    off.solve(*batch)
    t = off.tuning()
    assert t["block_min"] == 0 and not t["last_solve_block_mode"]
