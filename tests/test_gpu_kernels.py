"""Kernel-level parity of the four sm_103a kernels against the CPU oracle, through the
C ABI (bvp_eval_stage): K1 residual (FP64), K2 Jacobian blocks (FP32), K3 Newton
direction (FP32 structured factorisation), K4 defect (FP64)."""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _oracle(p):
    return Oracle(p.source, p.M, p.n_params, twopoint=p.twopoint, bc_t=p.bc_t, La=p.La, Lb=p.Lb)


def _cases(problems, name, n_inst=6, seed=3, order=4):
    p = problems.ALL[name]
    rng = np.random.default_rng(seed)
    meshes, ys, params = [], [], []
    t0, t1 = p.tspan
    for k in range(n_inst):
        n = int(rng.integers(5, 70))
        # a non-uniform mesh keeps every interval length different
        w = rng.uniform(0.5, 1.5, n)
        mesh = t0 + (t1 - t0) * np.concatenate([[0], np.cumsum(w) / w.sum()])
        mesh[-1] = t1
        meshes.append(mesh)
        ys.append(rng.normal(0, 1, (n + 1, p.M)))
        if name == "pendulum":
            params.append([rng.uniform(5, 15), rng.uniform(-.2, .2), rng.uniform(-.2, .2)])
        elif name == "singular_perturbation":
            params.append([math.exp(rng.uniform(math.log(1e-3), math.log(1e-1)))])
        elif name == "torus":
            params.append([0.5, -1.2, -0.5, 0.3])
        else:
            params.append([1.0] * max(p.n_params, 1))
    return p, np.array(params)[:, :max(p.n_params, 1)], meshes, ys


CASES = [("pendulum", 4), ("pendulum", 6), ("singular_perturbation", 6), ("multipoint", 4),
         ("torus", 4), ("pendulum", 2), ("pendulum", 3), ("pendulum", 5),
         ("pendulum", "6I"), ("singular_perturbation", "6I")]


def _kw(order):
    """Solver / oracle keywords of a case's scheme: MIRK2-6, or "6I" for MIRK6I."""
    return dict(order=6, mirk6i=1) if order == "6I" else dict(order=order)


@pytest.mark.parametrize("name,order", CASES)
def test_k1_residual_matches_oracle(pkg, problems, name, order):
    p, params, meshes, ys = _cases(problems, name, order=order)
    sv = pkg.BatchSolver(p, **_kw(order))
    out = sv.eval_stage(0, params, meshes, ys)
    o = _oracle(p)
    off = out["offsets"]
    for q in range(len(meshes)):
        F, K, nrm = o.residual(params[q], meshes[q], ys[q], **_kw(order))
        N, M = len(meshes[q]), p.M
        La = p.La if p.twopoint else M
        colloc = F[La:La + (N - 1) * M].reshape(N - 1, M)
        got = out["F"][off[q]:off[q] + N - 1]
        scale = max(1.0, np.abs(colloc).max())
        assert np.abs(got - colloc).max() <= 1e-12 * scale
        gotK = out["K"][off[q]:off[q] + N - 1]
        assert np.abs(gotK - K).max() <= 1e-12 * max(1.0, np.abs(K).max())
        bc = np.concatenate([F[:La], F[La + (N - 1) * M:]]) if p.twopoint else F[:M]
        assert np.abs(out["bc_res"][q] - bc).max() <= 1e-12 * max(1.0, np.abs(bc).max())
        assert abs(out["norm"][q] - nrm) <= 1e-12 * max(1.0, nrm)


@pytest.mark.parametrize("name,order", CASES)
def test_k2_jacobian_blocks_match_oracle(pkg, problems, name, order):
    # FP32 forward-mode blocks against the FP64 oracle: relative 2e-5 of the block scale
    p, params, meshes, ys = _cases(problems, name, order=order)
    sv = pkg.BatchSolver(p, **_kw(order))
    out = sv.eval_stage(1, params, meshes, ys)
    o = _oracle(p)
    off = out["offsets"]
    for q in range(len(meshes)):
        S, R, nodes, blocks = o.jacobian(params[q], meshes[q], ys[q], **_kw(order))
        N = len(meshes[q])
        gS = out["S"][off[q]:off[q] + N - 1]
        gR = out["R"][off[q]:off[q] + N - 1]
        sc = max(1.0, np.abs(S).max(), np.abs(R).max())
        assert np.abs(gS - S).max() <= 2e-5 * sc
        assert np.abs(gR - R).max() <= 2e-5 * sc


def _apply_jacobian(p, S, R, nodes, blocks, delta):
    """J δ in the reference's row order: BC rows, then collocation rows."""
    N, M = delta.shape
    colloc = np.einsum("iab,ib->ia", S, delta[:-1]) + np.einsum("iab,ib->ia", R, delta[1:])
    bc = np.zeros(M)
    for nd, B in zip(nodes, blocks):
        bc += B @ delta[nd]
    return bc, colloc


def _backward_error(p, o, params, mesh, y, delta, order):
    F, K, _ = o.residual(params, mesh, y, **_kw(order))
    S, R, nodes, blocks = o.jacobian(params, mesh, y, **_kw(order))
    N, M = len(mesh), p.M
    La = p.La if p.twopoint else M
    Fc = F[La:La + (N - 1) * M].reshape(N - 1, M)
    Fb = np.concatenate([F[:La], F[La + (N - 1) * M:]]) if p.twopoint else F[:M]
    bc, colloc = _apply_jacobian(p, S, R, nodes, blocks, delta)
    r = max(np.abs(bc + Fb).max(), np.abs(colloc + Fc).max())
    Jn = max(np.abs(S).sum(2).max() + np.abs(R).sum(2).max(), np.abs(blocks).sum(2).max() * len(blocks))
    return r / (Jn * np.abs(delta).max() + np.abs(F).max())


@pytest.mark.parametrize("name,order", CASES)
def test_k3_newton_direction_fp64_matches_oracle(pkg, problems, name, order):
    # FP64 factorisation: the structured cyclic reduction agrees with the oracle's
    # sequential elimination to roundoff times the systems' conditioning
    p, params, meshes, ys = _cases(problems, name, order=order)
    sv = pkg.BatchSolver(p, jac_precision=64, **_kw(order))
    out = sv.eval_stage(2, params, meshes, ys)
    assert (out["norm"] == 0).all(), "singular system reported"
    o = _oracle(p)
    off = out["offsets"]
    for q in range(len(meshes)):
        d = o.newton_step(params[q], meshes[q], ys[q], **_kw(order))
        N = len(meshes[q])
        got = out["delta"][off[q]:off[q] + N]
        assert np.abs(got - d).max() <= 1e-8 * max(1.0, np.abs(d).max()), (q, np.abs(got - d).max())
        assert _backward_error(p, o, params[q], meshes[q], ys[q], got, order) <= 1e-13


@pytest.mark.parametrize("name,order", CASES)
def test_k3_newton_direction_fp32_backward_stable(pkg, problems, name, order):
    # FP32 factorisation: a backward-stable solve of the FP32-rounded system, i.e. the
    # residual of J δ = -F (evaluated in FP64 with the oracle's Jacobian) is at FP32
    # roundoff relative to |J||δ| + |F|; the forward error then follows the conditioning
    p, params, meshes, ys = _cases(problems, name, order=order)
    sv = pkg.BatchSolver(p, jac_precision=32, **_kw(order))
    out = sv.eval_stage(2, params, meshes, ys)
    assert (out["norm"] == 0).all(), "singular system reported"
    o = _oracle(p)
    off = out["offsets"]
    for q in range(len(meshes)):
        N = len(meshes[q])
        got = out["delta"][off[q]:off[q] + N]
        eta = _backward_error(p, o, params[q], meshes[q], ys[q], got, order)
        assert eta <= 2e-5, (q, eta)


@pytest.mark.parametrize("name,order", CASES)
def test_k4_defect_matches_oracle(pkg, problems, name, order):
    p, params, meshes, ys = _cases(problems, name, order=order)
    sv = pkg.BatchSolver(p, **_kw(order))
    out = sv.eval_stage(3, params, meshes, ys)
    o = _oracle(p)
    off = out["offsets"]
    for q in range(len(meshes)):
        err, dn = o.defect(params[q], meshes[q], ys[q], **_kw(order))
        N = len(meshes[q])
        got = out["err"][off[q]:off[q] + N - 1]
        assert np.abs(got - err).max() <= 1e-10 * max(1.0, np.abs(err).max())
        assert abs(out["norm"][q] - dn) <= 1e-10 * max(1.0, dn)
