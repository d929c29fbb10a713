"""Batched MIRK solve through libbvpgpu.so.

``BatchSolver`` holds one library handle (one JIT-compiled kernel set) per
(problem, MIRK order, Jacobian precision) and solves batches of instances of that
problem; it is the Python face of the C ABI in include/bvpgpu.h. There is no CPU path:
if the CUDA library cannot be created the constructor raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import f64, i32

STATUS = {0: "OK", 1: "INVALID", 2: "COMPILE", 3: "CUDA", 4: "NOMEM", 5: "STATE", 6: "TOO_LARGE"}
RET_SUCCESS, RET_FAILURE, RET_MAXITERS = 0, 1, 2
S_OF = {2: 1, 3: 2, 4: 3, 5: 4, 6: 5}
NSX_OF = {2: 2, 3: 1, 4: 1, 5: 2, 6: 4}
NSX_MIRK6I = 3      # MIRK6I: 8 interpolant stages over its 5 discrete ones


def n_extra_stages(order: int, mirk6i: int = 0) -> int:
    """Extra interpolant stages of MIRKn (or MIRK6I), at least one slot."""
    return NSX_MIRK6I if mirk6i else max(1, NSX_OF[order])


class BVPError(RuntimeError):
    pass


@dataclass
class BatchResult:
    retcode: np.ndarray
    n_nodes: np.ndarray
    newton_iters: np.ndarray
    rounds: np.ndarray
    defect: np.ndarray
    resid: np.ndarray
    offsets: np.ndarray          # packed layout: instance i at [offsets[i], offsets[i] + n_nodes[i])
    mesh_packed: np.ndarray
    y_packed: np.ndarray         # (total, M)
    K_packed: np.ndarray | None = None
    KI_packed: np.ndarray | None = None
    order: int = 4
    global_err: np.ndarray | None = None    # last global error estimate (NaN under DefectControl)

    @property
    def mesh(self):
        """Final meshes padded to (n, max N) with NaN."""
        return self._pad(self.mesh_packed)

    @property
    def y(self):
        return self._pad(self.y_packed)

    def _pad(self, packed):
        n = len(self.n_nodes)
        nmax = int(self.n_nodes.max())
        out = np.full((n, nmax) + packed.shape[1:], np.nan)
        for i in range(n):
            a = self.offsets[i]
            k = int(self.n_nodes[i])
            out[i, :k] = packed[a:a + k]
        return out

    def solution(self, i):
        a = self.offsets[i]
        b = a + int(self.n_nodes[i])
        return self.mesh_packed[a:b], self.y_packed[a:b]

    def stages(self, i):
        a = self.offsets[i]
        b = a + int(self.n_nodes[i])
        return self.K_packed[a:b - 1], self.KI_packed[a:b - 1]


class BatchSolver:
    def __init__(self, problem, order: int = 4, abstol: float = 1e-6, *, jac_precision: int = 32,
                 lib_path: str | None = None, **opts):
        self.lib = _lib.load_library(lib_path)
        self.problem = problem
        self.order = order
        self.M = problem.M
        d = _lib.ProblemDesc()
        d.M, d.n_params, d.twopoint = problem.M, problem.n_params, int(problem.twopoint)
        d.n_bc_pts = len(problem.bc_t)
        d.La, d.Lb = problem.La, problem.Lb
        for k, t in enumerate(problem.bc_t):
            d.bc_t[k] = float(t)
        o = _lib.Options()
        self.lib.bvp_default_options(C.byref(o))
        o.order, o.abstol, o.jac_precision = order, abstol, jac_precision
        # controller="defect" | "global" | "sequential" | "hybrid", global_method="HO" | "RE"
        if isinstance(opts.get("controller"), str):
            opts["controller"] = _lib.CONTROLLERS[opts["controller"]]
        if isinstance(opts.get("global_method"), str):
            opts["global_method"] = _lib.GLOBAL_METHODS[opts["global_method"]]
        # firk="RadauIIa" | "LobattoIIIa" | "LobattoIIIb" | "LobattoIIIc" with firk_stages=s
        if isinstance(opts.get("firk"), str):
            opts["firk"] = _lib.FIRK_FAMILIES[opts["firk"]]
        for k, v in opts.items():
            if not hasattr(o, k):
                raise KeyError(k)
            setattr(o, k, v)
        self.options = o
        self.desc = d
        h = C.c_void_p()
        st = self.lib.bvp_create(C.byref(d), problem.source.encode(), C.byref(o), C.byref(h))
        self.h = h
        if st != 0:
            msg = self.lib.bvp_last_error(h).decode() if h.value else ""
            if h.value:
                self.lib.bvp_destroy(h)
                self.h = C.c_void_p()
            raise BVPError(f"bvp_create failed ({STATUS.get(st, st)}): {msg}")

    def __del__(self):
        try:
            if self.h and self.h.value:
                self.lib.bvp_destroy(self.h)
                self.h = C.c_void_p()
        except Exception:
            pass

    def _check(self, st, what):
        if st != 0:
            raise BVPError(f"{what} failed ({STATUS.get(st, st)}): {self.lib.bvp_last_error(self.h).decode()}")

    def _results(self, n):
        r = dict(retcode=np.zeros(n, np.int32), n_nodes=np.zeros(n, np.int32),
                 newton_iters=np.zeros(n, np.int32), rounds=np.zeros(n, np.int32),
                 defect=np.zeros(n), resid=np.zeros(n), global_err=np.zeros(n))
        cr = _lib.Results(i32(r["retcode"]), i32(r["n_nodes"]), i32(r["newton_iters"]),
                          i32(r["rounds"]), f64(r["defect"]), f64(r["resid"]), f64(r["global_err"]))
        return r, cr

    def _collect(self, r):
        n = len(r["retcode"])
        off = C.POINTER(C.c_int64)()
        mesh = C.POINTER(C.c_double)()
        y = C.POINTER(C.c_double)()
        K = C.POINTER(C.c_double)()
        KI = C.POINTER(C.c_double)()
        self._check(self.lib.bvp_get_packed(self.h, C.byref(off), C.byref(mesh), C.byref(y),
                                            C.byref(K), C.byref(KI)), "bvp_get_packed")
        offsets = np.ctypeslib.as_array(off, shape=(n + 1,)).copy()
        tot = int(offsets[-1])
        M = self.M
        res = BatchResult(offsets=offsets,
                          mesh_packed=np.ctypeslib.as_array(mesh, shape=(tot,)).copy(),
                          y_packed=np.ctypeslib.as_array(y, shape=(tot * M,)).copy().reshape(tot, M),
                          order=self.order, **r)
        if self.options.want_stages and bool(K) and bool(KI):
            s, nsx = S_OF[self.order], n_extra_stages(self.order, self.options.mirk6i)
            res.K_packed = np.ctypeslib.as_array(K, shape=(tot * s * M,)).copy().reshape(tot, s, M)
            res.KI_packed = np.ctypeslib.as_array(KI, shape=(tot * nsx * M,)).copy().reshape(tot, nsx, M)
        return res

    def solve(self, params, n_intervals, tspans, y0, *, y0_mode: int | None = None) -> BatchResult:
        """Solve a batch from host arrays (host -> device -> host through the C ABI)."""
        n_int = np.ascontiguousarray(n_intervals, dtype=np.int32).ravel()
        n = len(n_int)
        params = np.ascontiguousarray(params, dtype=np.float64).reshape(n, -1) if self.problem.n_params else None
        tsp = np.ascontiguousarray(tspans, dtype=np.float64).reshape(n, 2)
        y0a = np.ascontiguousarray(y0, dtype=np.float64)
        if y0_mode is None:
            y0_mode = 0 if y0a.size == n * self.M else 1
        y0a = y0a.ravel()
        r, cr = self._results(n)
        st = self.lib.bvp_solve_batch(self.h, n, f64(params), i32(n_int), f64(tsp), y0_mode, f64(y0a), C.byref(cr))
        self._check(st, "bvp_solve_batch")
        return self._collect(r)

    def solve_warm(self, net, features, n_grid, params, n_intervals, tspans, y0_plain):
        """Surrogate-warm solve through the C ABI (bvp_solve_batch_warm): network guess,
        resampling, solve and plain-guess fallback on the device. Returns
        (BatchResult, number of instances that needed the fallback)."""
        feats = np.ascontiguousarray(features, dtype=np.float32)
        n_int = np.ascontiguousarray(n_intervals, dtype=np.int32).ravel()
        n = len(n_int)
        params = np.ascontiguousarray(params, dtype=np.float64).reshape(n, -1) if self.problem.n_params else None
        tsp = np.ascontiguousarray(tspans, dtype=np.float64).reshape(n, 2)
        y0p = np.ascontiguousarray(y0_plain, dtype=np.float64).reshape(n, self.M)
        r, cr = self._results(n)
        nfb = np.zeros(1, np.int32)
        st = self.lib.bvp_solve_batch_warm(self.h, net.h, n, feats.shape[1],
                                           feats.ctypes.data_as(C.POINTER(C.c_float)), int(n_grid),
                                           f64(params), i32(n_int), f64(tsp), f64(y0p), C.byref(cr), i32(nfb))
        self._check(st, "bvp_solve_batch_warm")
        return self._collect(r), int(nfb[0])

    def solve_device(self, d_params, d_n_intervals, d_tspans, d_y0, max_intervals, *, y0_mode=0, d_y0_off=None):
        """Launch a solve on inputs already in device memory (integer device pointers or
        objects with data_ptr()); returns without synchronising."""
        def ptr(x):
            if x is None:
                return None
            return C.c_void_p(x.data_ptr() if hasattr(x, "data_ptr") else int(x))
        n = int(d_n_intervals.numel() if hasattr(d_n_intervals, "numel") else len(d_n_intervals))
        st = self.lib.bvp_solve_batch_device(self.h, n, ptr(d_params), ptr(d_n_intervals), ptr(d_tspans),
                                             y0_mode, ptr(d_y0), ptr(d_y0_off), int(max_intervals))
        self._check(st, "bvp_solve_batch_device")
        self._pending_n = n

    def solve_device_warm(self, net, d_features, n_grid, d_params, d_n_intervals, d_tspans, max_intervals):
        """Surrogate-warm solve on device inputs (bvp_solve_batch_device_warm): the network's
        forward on a second stream beside the solve's setup; returns without synchronising and
        without the plain-guess fallback."""
        def ptr(x):
            if x is None:
                return None
            return C.c_void_p(x.data_ptr() if hasattr(x, "data_ptr") else int(x))
        n = int(d_n_intervals.numel() if hasattr(d_n_intervals, "numel") else len(d_n_intervals))
        st = self.lib.bvp_solve_batch_device_warm(self.h, net.h, n, ptr(d_features), int(n_grid), ptr(d_params),
                                                  ptr(d_n_intervals), ptr(d_tspans), int(max_intervals))
        self._check(st, "bvp_solve_batch_device_warm")
        self._pending_n = n

    def solve_device_grid(self, d_params, d_n_intervals, d_tspans, d_grid, n_grid, max_intervals):
        """solve_device with the initial guesses on uniform n_grid-point grids (FP32 device
        array n_inst x n_grid x M), resampled onto the initial meshes inside the solve."""
        def ptr(x):
            return C.c_void_p(x.data_ptr() if hasattr(x, "data_ptr") else int(x))
        n = int(d_n_intervals.numel() if hasattr(d_n_intervals, "numel") else len(d_n_intervals))
        st = self.lib.bvp_solve_batch_device_grid(self.h, n, ptr(d_params) if d_params is not None else None,
                                                  ptr(d_n_intervals), ptr(d_tspans), ptr(d_grid), int(n_grid),
                                                  int(max_intervals))
        self._check(st, "bvp_solve_batch_device_grid")
        self._pending_n = n

    def fetch(self) -> BatchResult:
        r, cr = self._results(self._pending_n)
        self._check(self.lib.bvp_fetch_results(self.h, C.byref(cr)), "bvp_fetch_results")
        return self._collect(r)

    def dense(self, tq, deriv: int = 0):
        """u(t) (deriv 0) or u'(t) (deriv 1) of every instance of the last solve at the
        query times tq (n_inst x nq); needs want_stages=1."""
        tq = np.ascontiguousarray(tq, dtype=np.float64)
        n, nq = tq.shape
        out = np.zeros((n, nq, self.M))
        self._check(self.lib.bvp_dense_output(self.h, nq, f64(tq), deriv, f64(out)), "bvp_dense_output")
        return out

    def timing_ms(self):
        t = np.zeros(2)
        self._check(self.lib.bvp_last_timing(self.h, f64(t)), "bvp_last_timing")
        return float(t[0]), float(t[1])

    def tuning(self) -> dict:
        """Launch shapes the library's autotuner picked for this handle."""
        t = np.zeros(1, np.int32)
        self._check(self.lib.bvp_get_tuning(self.h, i32(t)), "bvp_get_tuning")
        b, done = np.zeros(1, np.int32), np.zeros(1, np.int32)
        ms = np.zeros(3, np.float32)
        self._check(self.lib.bvp_get_fused_tuning(self.h, i32(b), i32(done), ms.ctypes.data_as(C.POINTER(C.c_float))),
                    "bvp_get_fused_tuning")
        bm, last = np.zeros(1, np.int32), np.zeros(1, np.int32)
        self._check(self.lib.bvp_get_block_mode(self.h, i32(bm), i32(last)), "bvp_get_block_mode")
        return {"linsolve_threads": int(t[0]), "fused_blocks_per_sm": int(b[0]), "fused_tuned": bool(done[0]),
                "fused_ms_by_blocks": {4: float(ms[0]), 3: float(ms[1]), 2: float(ms[2])},
                "block_min": int(bm[0]), "last_solve_block_mode": bool(last[0])}

    def work_order(self):
        """(learned, costs): whether the fused solve's work order comes from the handle's learned
        cost table, and the table (longest solve time per initial-size bucket of 8 intervals, the
        maximum last)."""
        learned = np.zeros(1, np.int32)
        costs = np.zeros(513, np.float32)
        self._check(self.lib.bvp_get_work_order(self.h, i32(learned), costs.ctypes.data_as(C.POINTER(C.c_float)),
                                                len(costs)), "bvp_get_work_order")
        return bool(learned[0]), costs

    def stream_ptr(self) -> int:
        return int(self.lib.bvp_stream(self.h) or 0)

    def eval_stage(self, stage, params, meshes, ys):
        """Run one kernel stage on given meshes/solutions (lists per instance)."""
        n = len(meshes)
        n_nodes = np.array([len(m) for m in meshes], np.int32)
        off = np.concatenate([[0], np.cumsum(n_nodes)]).astype(np.int64)
        tot = int(off[-1])
        M, s = self.M, S_OF[self.order]
        mesh = np.ascontiguousarray(np.concatenate(meshes), dtype=np.float64)
        y = np.ascontiguousarray(np.concatenate([np.asarray(v, dtype=np.float64).reshape(-1, M) for v in ys]))
        params = np.ascontiguousarray(params, dtype=np.float64).reshape(n, -1) if self.problem.n_params else None
        out = dict(norm=np.zeros(n), F=np.zeros((tot, M)), bc_res=np.zeros((n, M)), K=np.zeros((tot, s, M)),
                   S=np.zeros((tot, M, M)), R=np.zeros((tot, M, M)), delta=np.zeros((tot, M)), err=np.zeros(tot))
        st = self.lib.bvp_eval_stage(self.h, stage, n, f64(params), i32(n_nodes), f64(mesh), f64(y),
                                     f64(out["norm"]), f64(out["F"]), f64(out["bc_res"]), f64(out["K"]),
                                     f64(out["S"]), f64(out["R"]), f64(out["delta"]), f64(out["err"]))
        self._check(st, "bvp_eval_stage")
        out["offsets"] = off
        return out
