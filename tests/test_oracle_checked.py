"""The oracle under bounds-checked containers (BVP_ORACLE_CHECKED: an out-of-range index
aborts), on batches whose meshes shrink and grow, and its results repeat bitwise. An in-place
solution transfer that read past a shrunken mesh's array once made its results depend on heap
contents; this is the regression test for it."""
import numpy as np
import pytest

from oracle.oracle import Oracle

_FIELDS = ("retcode", "n_nodes", "newton_iters", "rounds", "defect", "resid")


def _oracle(p):
    return Oracle(p.source, p.M, p.n_params, twopoint=p.twopoint, bc_t=p.bc_t, La=p.La, Lb=p.Lb)


@pytest.mark.parametrize("max_sub", [600, 3000])
def test_checked_oracle_repeats(problems, monkeypatch, max_sub):
    monkeypatch.setenv("BVP_ORACLE_CHECKED", "1")
    p = problems.SINGULAR_PERTURBATION
    params, nint, tsp, y0 = problems.singular_perturbation_family(1024, seed=2025)
    batch = (params[:64], nint[:64], tsp[:64], y0[:64])
    o = _oracle(p)
    runs = [o.solve_batch(*batch, order=6, max_subintervals=max_sub, nthreads=nt) for nt in (1, 0, 1, 0)]
    # meshes shrank somewhere (the case the in-place transfer got wrong)
    assert (runs[0]["n_nodes"] < nint[:64] + 1).any()
    for r in runs[1:]:
        for f in _FIELDS:
            assert np.array_equal(r[f], runs[0][f]), f
        for i in range(64):
            N = int(r["n_nodes"][i])
            assert np.array_equal(r["y"][i, :N], runs[0]["y"][i, :N]), i


def test_checked_oracle_pendulum(problems, monkeypatch):
    monkeypatch.setenv("BVP_ORACLE_CHECKED", "1")
    o = _oracle(problems.PENDULUM)
    batch = problems.pendulum_family(256, seed=5)
    a = o.solve_batch(*batch, order=4)
    b = o.solve_batch(*batch, order=4, nthreads=1)
    assert (a["retcode"] == 0).all() and (a["rounds"] > 1).any()
    for f in _FIELDS:
        assert np.array_equal(a[f], b[f]), f
