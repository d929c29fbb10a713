"""Surrogate warm start for batched MIRK solves.

A GELU multilayer perceptron (BF16 weights and activations, FP32 accumulation, trained and
evaluated by the library's own tensor-core kernels, ``bvp_mlp_*`` in include/bvpgpu.h) maps
an instance's parameters to its solution on a uniform grid of ``GRID`` points over its
tspan. The grid guess is resampled onto the instance's initial mesh and passed to the solve
as a per-node initial guess (the reference's vector-of-arrays guess,
lib/BoundaryValueDiffEqCore/src/utils.jl:750-765). The plain MIRK Newton stays in charge:
an instance that does not converge from its warm start is solved again from the plain guess,
and the solution it returns is always judged by the solver's own defect and residual tests.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .solver import BatchSolver, BVPError, RET_SUCCESS


def _f32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


class MLP:
    """Handle on a bvp_mlp network: widths[0] inputs, widths[-1] outputs, GELU between."""

    def __init__(self, widths, seed: int = 0, lib_path=None):
        self.lib = _lib.load_library(lib_path)
        self.widths = [int(w) for w in widths]
        w = (C.c_int32 * len(self.widths))(*self.widths)
        h = C.c_void_p()
        st = self.lib.bvp_mlp_create(len(self.widths) - 1, w, C.byref(h))
        if st != 0:
            raise BVPError(f"bvp_mlp_create failed ({st})")
        self.h = h
        self.n_params = int(self.lib.bvp_mlp_num_params(h))
        self.set_params(self.init_params(seed))

    def __del__(self):
        try:
            if self.h and self.h.value:
                self.lib.bvp_mlp_destroy(self.h)
                self.h = C.c_void_p()
        except Exception:
            pass

    def layout(self):
        """(offset_W, offset_b) of every layer in the packed parameter vector."""
        out, o = [], 0
        for a, b in zip(self.widths[:-1], self.widths[1:]):
            out.append((o, o + a * b))
            o += a * b + b
        return out

    def init_params(self, seed):
        rng = np.random.default_rng(seed)
        p = np.zeros(self.n_params, np.float32)
        for (ow, ob), a, b in zip(self.layout(), self.widths[:-1], self.widths[1:]):
            p[ow:ow + a * b] = rng.normal(0, np.sqrt(2.0 / a), a * b)
        return p

    def _check(self, st, what):
        if st != 0:
            raise BVPError(f"{what} failed ({st})")

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        self._check(self.lib.bvp_mlp_set_params(self.h, _f32p(p)), "bvp_mlp_set_params")

    def get_params(self):
        p = np.zeros(self.n_params, np.float32)
        self._check(self.lib.bvp_mlp_get_params(self.h, _f32p(p)), "bvp_mlp_get_params")
        return p

    def set_normalization(self, in_mu, in_sd, out_mu, out_sd):
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (in_mu, in_sd, out_mu, out_sd)]
        self.norm = arrs
        self._check(self.lib.bvp_mlp_set_normalization(self.h, *[_f32p(a) for a in arrs]),
                    "bvp_mlp_set_normalization")

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros((x.shape[0], self.widths[-1]), np.float32)
        self._check(self.lib.bvp_mlp_forward(self.h, x.shape[0], _f32p(x), _f32p(y)), "bvp_mlp_forward")
        return y

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = np.zeros(1, np.float32)
        g = np.zeros(self.n_params, np.float32)
        self._check(self.lib.bvp_mlp_loss_grad(self.h, x.shape[0], _f32p(x), _f32p(t), _f32p(loss), _f32p(g)),
                    "bvp_mlp_loss_grad")
        return float(loss[0]), g

    def train(self, x, t, epochs=100, batch=512, lr=2e-3, seed=0):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = np.zeros(1, np.float32)
        self._check(self.lib.bvp_mlp_train(self.h, x.shape[0], _f32p(x), _f32p(t), epochs, batch, lr, seed,
                                           _f32p(loss)), "bvp_mlp_train")
        return float(loss[0])

    def forward_device(self, d_x, d_y, batch, stream=None):
        def ptr(v):
            return C.c_void_p(v.data_ptr() if hasattr(v, "data_ptr") else int(v))
        st = self.lib.bvp_mlp_forward_device(self.h, batch, ptr(d_x), ptr(d_y),
                                             C.c_void_p(stream) if stream else None)
        self._check(st, "bvp_mlp_forward_device")

    def forward_noalloc(self, d_x, d_y, batch, stream=None):
        """forward_device without any device allocation (bvp_mlp_forward_noalloc): the fused
        kernel when the network fits it, else the layer-by-layer kernels on the library's static
        scratch, where batch x widest layer is bounded by BVP_MLP_NOALLOC_SCRATCH_BYTES."""
        def ptr(v):
            return C.c_void_p(v.data_ptr() if hasattr(v, "data_ptr") else int(v))
        st = self.lib.bvp_mlp_forward_noalloc(self.h, batch, ptr(d_x), ptr(d_y), C.c_void_p(stream) if stream else None)
        if st == 6:
            raise BVPError(f"bvp_mlp_forward_noalloc: batch {batch} x widest layer {max(self.widths)} does not fit "
                           "the static scratch")
        self._check(st, "bvp_mlp_forward_noalloc")


def resample_host(grid, n_intervals):
    """Linear resampling of uniform-grid guesses (n x G x M) onto uniform meshes with
    n_intervals[i] intervals, packed for y0_mode 1 (the host twin of the device kernel)."""
    out = []
    G = grid.shape[1]
    for g, n in zip(grid, n_intervals):
        s = np.arange(n + 1) * (1.0 / n) * (G - 1)    # j (1/n) (G-1), rounded as the device rounds it
        i0 = np.clip(np.floor(s).astype(int), 0, G - 2)
        f = (s - i0)[:, None]
        out.append((1 - f) * g[i0] + f * g[i0 + 1])
    return np.concatenate(out)


@dataclass
class WarmResult:
    result: object            # BatchResult of the warm-started solve (failures replaced)
    fallback: np.ndarray      # instances solved again from the plain guess
    newton_warm: np.ndarray   # Newton iterations of the warm attempt per instance


class Surrogate:
    """Parameters -> solution on a GRID-point uniform grid, for one problem family."""

    def __init__(self, problem, n_params_in: int, grid: int = 64, hidden: int = 256, n_hidden: int = 3,
                 seed: int = 0):
        self.problem = problem
        self.grid = grid
        self.M = problem.M
        self.net = MLP([n_params_in] + [hidden] * n_hidden + [grid * problem.M], seed=seed)

    def grid_times(self, tspans):
        tspans = np.asarray(tspans, dtype=np.float64)
        u = np.linspace(0.0, 1.0, self.grid)
        return tspans[:, :1] + (tspans[:, 1:] - tspans[:, :1]) * u[None, :]

    def training_data(self, solver: BatchSolver, features, params, n_intervals, tspans, y0, chunk=8192):
        """Solve the instances with the plain solver (want_stages=1) and sample every
        converged solution on the grid: returns (features, targets) of the converged ones."""
        X, T = [], []
        for a in range(0, len(n_intervals), chunk):
            b = min(a + chunk, len(n_intervals))
            res = solver.solve(params[a:b], n_intervals[a:b], tspans[a:b], y0[a:b])
            u = solver.dense(self.grid_times(tspans[a:b]))
            ok = res.retcode == RET_SUCCESS
            X.append(np.asarray(features[a:b])[ok])
            T.append(u[ok].reshape(int(ok.sum()), -1))
        X, T = np.concatenate(X).astype(np.float32), np.concatenate(T).astype(np.float32)
        return X, T

    def fit(self, X, T, epochs=200, batch=512, lr=2e-3, seed=0):
        mu_x, sd_x = X.mean(0), X.std(0) + 1e-6
        mu_t, sd_t = T.mean(0), T.std(0) + 1e-6
        self.net.set_normalization(mu_x, sd_x, mu_t, sd_t)
        return self.net.train(X, T, epochs=epochs, batch=batch, lr=lr, seed=seed)

    def predict_grid(self, features):
        y = self.net.forward(np.asarray(features, dtype=np.float32))
        return y.reshape(len(y), self.grid, self.M)

    def guess(self, features, n_intervals):
        return resample_host(self.predict_grid(features).astype(np.float64), n_intervals)

    def warm_solve(self, solver: BatchSolver, features, params, n_intervals, tspans, y0_plain) -> WarmResult:
        """Solve from the surrogate's guesses; instances that fail are solved again from
        the plain guess and their results replace the warm attempt's."""
        res = solver.solve(params, n_intervals, tspans, self.guess(features, n_intervals), y0_mode=1)
        warm_iters = res.newton_iters.copy()
        bad = np.nonzero(res.retcode != RET_SUCCESS)[0]
        if len(bad):
            sub = solver.solve(params[bad], np.asarray(n_intervals)[bad], np.asarray(tspans)[bad],
                               np.asarray(y0_plain)[bad])
            res = merge_results(res, sub, bad, self.M)
        return WarmResult(res, bad, warm_iters)


def merge_results(base, sub, idx, M):
    """Replace instances idx of a BatchResult with the instances of another."""
    from .solver import BatchResult
    n = len(base.n_nodes)
    sols_m, sols_y = [], []
    j = {int(q): k for k, q in enumerate(idx)}
    fields = {}
    for name in ("retcode", "n_nodes", "newton_iters", "rounds", "defect", "resid", "global_err"):
        if getattr(base, name) is None or getattr(sub, name) is None:
            continue
        arr = getattr(base, name).copy()
        arr[idx] = getattr(sub, name)
        fields[name] = arr
    for q in range(n):
        if q in j:
            m, y = sub.solution(j[q])
        else:
            m, y = base.solution(q)
        sols_m.append(m)
        sols_y.append(y)
    off = np.concatenate([[0], np.cumsum([len(m) for m in sols_m])]).astype(np.int64)
    return BatchResult(offsets=off, mesh_packed=np.concatenate(sols_m), y_packed=np.concatenate(sols_y),
                       order=base.order, **fields)
