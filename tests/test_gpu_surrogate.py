"""The surrogate warm start: its BF16 tensor-core forward/backward kernels against the CPU
restatement (oracle/mlp_ref.py), dense output against the oracle's interpolant, and what the
trained network gains over the plain constant guess."""
import math

import numpy as np
import pytest

from oracle import mlp_ref
from oracle.oracle import Oracle, RET_SUCCESS

pytestmark = pytest.mark.gpu


def _norm(widths, rng):
    return (rng.normal(0, 1, widths[0]).astype(np.float32), rng.uniform(0.5, 2, widths[0]).astype(np.float32),
            rng.normal(0, 1, widths[-1]).astype(np.float32), rng.uniform(0.5, 2, widths[-1]).astype(np.float32))


@pytest.mark.parametrize("widths,batch", [([3, 256, 256, 256, 128], 37), ([5, 64, 33, 7], 130)])
def test_mlp_forward_and_gradient_match_cpu(pkg, widths, batch):
    # GPU: BF16 operands, FP32 accumulation. CPU: the same BF16 roundings, FP64 sums.
    # Tolerance 2e-2 in relative 2-norm per layer (FP32 summation order can move a value
    # across a BF16 rounding boundary; a wrong index or transpose gives O(1))
    rng = np.random.default_rng(3)
    net = pkg.MLP(widths, seed=4)
    p = net.get_params()
    p += rng.normal(0, 0.05, p.size).astype(np.float32)  # nonzero biases
    net.set_params(p)
    norm = _norm(widths, rng)
    net.set_normalization(*norm)
    x = rng.normal(0, 1, (batch, widths[0])).astype(np.float32)
    t = rng.normal(0, 1, (batch, widths[-1])).astype(np.float32)
    y_ref, _, _ = mlp_ref.forward(p, widths, x, norm)
    y = net.forward(x)
    assert np.linalg.norm(y - y_ref) <= 2e-2 * np.linalg.norm(y_ref)
    loss, g = net.loss_grad(x, t)
    loss_ref, g_ref = mlp_ref.loss_grad(p, widths, x, t, norm)
    assert abs(loss - loss_ref) <= 2e-2 * loss_ref
    for ow, ob in net.layout():
        pass
    lay = net.layout() + [(net.n_params, net.n_params)]
    for (ow, ob), (nxt, _) in zip(lay[:-1], lay[1:]):
        for a, b in ((ow, ob), (ob, nxt)):
            ref = g_ref[a:b]
            assert np.linalg.norm(g[a:b] - ref) <= 2e-2 * np.linalg.norm(ref) + 1e-12, (a, b)


def test_mlp_training_reduces_loss(pkg):
    # a smooth map learned by the library's Adam loop
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (4096, 3)).astype(np.float32)
    t = np.stack([np.sin(x[:, 0] + x[:, 1]), x[:, 2] ** 2, np.cos(2 * x[:, 0])], 1).astype(np.float32)
    net = pkg.MLP([3, 64, 64, 3], seed=1)
    net.set_normalization(np.zeros(3), np.ones(3), np.zeros(3), np.ones(3))
    l0, _ = net.loss_grad(x[:512], t[:512])
    last = net.train(x, t, epochs=60, batch=256, lr=3e-3, seed=2)
    assert last < 0.02 * l0, (l0, last)


def test_dense_output_matches_oracle_interpolant(pkg, problems):
    p = problems.PENDULUM
    params, nint, tsp, y0 = problems.pendulum_family(64, seed=9)
    sv = pkg.BatchSolver(p, order=4, want_stages=1, jac_precision=64)
    res = sv.solve(params, nint, tsp, y0)
    rng = np.random.default_rng(1)
    tq = np.sort(rng.uniform(0, math.pi / 2, (64, 17)), axis=1)
    u = sv.dense(tq)
    du = sv.dense(tq, deriv=1)
    o = Oracle(p.source, p.M, p.n_params, bc_t=p.bc_t)
    for i in range(64):
        m, y = res.solution(i)
        K, KI = res.stages(i)
        assert np.abs(u[i] - o.interpolate(4, m, y, K, KI, tq[i])).max() < 1e-12
        assert np.abs(du[i] - o.interpolate(4, m, y, K, KI, tq[i], deriv=1)).max() < 1e-11


def test_surrogate_warm_start_cuts_newton_iterations(pkg, problems):
    # train on plain-solver solutions of the pendulum family (disjoint seed), then solve a
    # fresh batch from the surrogate's guesses: fewer Newton iterations, every instance
    # converged, the same solutions as the plain solve at the solver's accuracy
    p = problems.PENDULUM
    sv = pkg.BatchSolver(p, order=4, want_stages=1)
    params, nint, tsp, y0 = problems.pendulum_family(8192, seed=101)
    sur = pkg.Surrogate(p, n_params_in=3)
    X, T = sur.training_data(sv, params, params, nint, tsp, y0)
    assert len(X) >= 8000
    sur.fit(X, T, epochs=80, batch=512, lr=2e-3)
    tp, tn, tt, ty = problems.pendulum_family(1024, seed=202)
    plain = sv.solve(tp, tn, tt, ty)
    warm = sur.warm_solve(sv, tp, tp, tn, tt, ty)
    assert (warm.result.retcode == RET_SUCCESS).all()
    assert (plain.retcode == RET_SUCCESS).all()
    print("newton plain", plain.newton_iters.mean(), "warm", warm.newton_warm.mean(), "fallback", len(warm.fallback))
    assert warm.newton_warm.mean() <= 0.7 * plain.newton_iters.mean()
    # the same warm start through the one C-ABI call (guess, resampling, solve and fallback
    # on the device): the device resampling rounds like the host one, so the guesses and
    # therefore the solves are identical
    dev, nfb = sv.solve_warm(sur.net, tp, sur.grid, tp, tn, tt, ty)
    assert nfb == len(warm.fallback)
    assert (dev.retcode == warm.result.retcode).all()
    assert (dev.n_nodes == warm.result.n_nodes).all()
    assert (dev.newton_iters == warm.result.newton_iters).all()
    for i in range(len(tn)):
        assert np.array_equal(dev.solution(i)[1], warm.result.solution(i)[1])
    # and on device inputs (bvp_solve_batch_device_warm: the forward on the handle's second
    # stream beside the solve's setup): the same warm results before any fallback
    import torch
    sv2 = pkg.BatchSolver(p, order=4)
    sv2.solve_device_warm(sur.net, torch.tensor(tp.astype(np.float32), device="cuda"), sur.grid,
                          torch.tensor(tp, device="cuda"), torch.tensor(tn, device="cuda"),
                          torch.tensor(tt, device="cuda"), int(tn.max()))
    dw = sv2.fetch()
    ok = dw.retcode == RET_SUCCESS
    assert ok.sum() == len(tn) - nfb
    for i in np.nonzero(ok)[0][::7]:
        assert np.array_equal(dw.solution(i)[1], dev.solution(i)[1])
    # both are solutions of the same discretisation to the same tolerance
    o = Oracle(p.source, p.M, p.n_params, bc_t=p.bc_t)
    for i in range(0, 1024, 37):
        m, y = warm.result.solution(i)
        F, K, nrm = o.residual(tp[i], m, y)
        assert nrm <= 1e-6 * (1 + 1e-6)
        err, dn = o.defect(tp[i], m, y)
        assert dn <= 1e-6 * (1 + 1e-3)


@pytest.mark.parametrize("batch", [37, 4096, 9000])
def test_tcgen05_forward_matches_the_mma_forward(pkg, batch, monkeypatch):
    # the inference kernel on the 5th-generation tensor cores (tcgen05.mma into TMEM; widths
    # multiples of 16; selected with BVPGPU_MLP_TC=1) against the default mma.sync kernel on the
    # same network and inputs: the same BF16 operands, FP32 sums in another order (a hidden
    # activation may round to the neighbouring BF16 value), and against the CPU restatement as
    # the other forward tests are
    import torch
    widths = [3, 256, 256, 256, 128]
    rng = np.random.default_rng(8)
    net_mma = pkg.MLP(widths, seed=9)
    monkeypatch.setenv("BVPGPU_MLP_TC", "1")
    net_tc = pkg.MLP(widths, seed=9)
    monkeypatch.delenv("BVPGPU_MLP_TC")
    p = net_tc.get_params()
    p += rng.normal(0, 0.05, p.size).astype(np.float32)
    norm = _norm(widths, rng)
    for net in (net_tc, net_mma):
        net.set_params(p)
        net.set_normalization(*norm)
    x = rng.normal(0, 1, (batch, 3)).astype(np.float32)
    dx = torch.tensor(x, device="cuda")
    outs = []
    for net in (net_tc, net_mma):
        dy = torch.full((batch, 128), float("nan"), device="cuda")
        net.forward_device(dx, dy, batch)
        torch.cuda.synchronize()
        outs.append(dy.cpu().numpy())
    y_tc, y_mma = outs
    assert np.isfinite(y_tc).all()
    assert np.linalg.norm(y_tc - y_mma) <= 1e-2 * np.linalg.norm(y_mma)
    y_ref, _, _ = mlp_ref.forward(p, widths, x, norm)
    assert np.linalg.norm(y_tc - y_ref) <= 2e-2 * np.linalg.norm(y_ref)
