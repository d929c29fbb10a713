"""CPU oracle loader: compiles the FP64 C++ restatement of the reference MIRK solve for a
given problem source and exposes it through ctypes.

TEST INFRASTRUCTURE ONLY. tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` use this module to check or time the CUDA library against the
reference algorithm; the shipped library never imports it.

The compiled objects go to ``oracle/_build/`` (git-ignored), keyed by a hash of the
sources and flags, so each (problem, M) pair is compiled once per machine.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SOURCES = ("oracle_entry.cpp", "mirk_oracle.hpp", "mirk_tableaus.hpp", "dual.hpp", "firk_oracle.hpp",
            "firk_tableaus.hpp")
_lock = threading.Lock()

RET_SUCCESS, RET_FAILURE, RET_MAXITERS, RET_TRUNCATED = 0, 1, 2, 3


class ProblemInfo(C.Structure):
    _fields_ = [
        ("M", C.c_int32), ("n_params", C.c_int32), ("twopoint", C.c_int32),
        ("n_bc_pts", C.c_int32), ("La", C.c_int32), ("Lb", C.c_int32),
        ("bc_t", C.c_double * 16),
    ]


class Options(C.Structure):
    _fields_ = [
        ("order", C.c_int32), ("adaptive", C.c_int32), ("max_subintervals", C.c_int32),
        ("max_newton", C.c_int32), ("max_rounds", C.c_int32), ("transfer_inplace", C.c_int32),
        ("bc_jac_exact", C.c_int32), ("linesearch_fallback", C.c_int32),
        ("stall_steps", C.c_int32), ("nthreads", C.c_int32),
        ("abstol", C.c_double), ("defect_threshold", C.c_double),
        ("divergence_factor", C.c_double), ("mirk6i", C.c_int32),
        ("controller", C.c_int32), ("global_method", C.c_int32),
        ("hybrid_de", C.c_double), ("hybrid_ge", C.c_double),
    ]


CONTROLLERS = {"defect": 0, "global": 1, "sequential": 2, "hybrid": 3}
FIRK_FAMILIES = {"RadauIIa": 0, "LobattoIIIa": 1, "LobattoIIIb": 2, "LobattoIIIc": 3}
GLOBAL_METHODS = {"HO": 0, "RE": 1}


def stage_counts(order: int, mirk6i: int = 0):
    """(discrete stages, extra interpolant stages >= 1) of MIRKn, or of MIRK6I."""
    if mirk6i:
        return 5, 3
    return {2: 1, 3: 2, 4: 3, 5: 4, 6: 5}[order], max(1, {2: 2, 3: 1, 4: 1, 5: 2, 6: 4}[order])


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


def _compile(source: str, M: int, twopoint: bool) -> str:
    h = hashlib.sha256()
    for fn in _SOURCES:
        with open(os.path.join(_HERE, fn), "rb") as f:
            h.update(f.read())
    h.update(source.encode())
    trace = bool(os.environ.get("BVP_ORACLE_TRACE"))
    # BVP_ORACLE_CHECKED: bounds-checked containers (an out-of-range index aborts)
    checked = bool(os.environ.get("BVP_ORACLE_CHECKED"))
    sing = "BVP_SING" in source
    h.update(f"M={M};tp={int(twopoint)};trace={int(trace)};sing={int(sing)};checked={int(checked)}".encode())
    key = h.hexdigest()[:20]
    os.makedirs(_BUILD, exist_ok=True)
    so = os.path.join(_BUILD, f"oracle_{key}.so")
    if os.path.exists(so):
        return so
    hdr = os.path.join(_BUILD, f"problem_{key}.h")
    with open(hdr, "w") as f:
        f.write(source)
    tmp = so + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           f"-DBVP_M={M}", f"-DBVP_TWOPOINT={int(twopoint)}",
           f"-DBVP_SINGULAR={int(sing)}", f'-DBVP_PROBLEM_HEADER="{hdr}"', "-I", _HERE,
           os.path.join(_HERE, "oracle_entry.cpp"), "-o", tmp] + (["-DBVP_TRACE"] if trace else []) + \
        (["-D_GLIBCXX_ASSERTIONS"] if checked else [])
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    os.replace(tmp, so)
    return so


class Oracle:
    """FP64 CPU restatement of the reference's adaptive MIRK solve for one problem."""

    def __init__(self, source: str, M: int, n_params: int, *, twopoint: bool = False,
                 bc_t=(), La: int = 0, Lb: int = 0):
        with _lock:
            self.so_path = _compile(source, M, twopoint)
        self.lib = C.CDLL(self.so_path)
        self.M, self.n_params, self.twopoint = M, n_params, twopoint
        info = ProblemInfo()
        info.M, info.n_params, info.twopoint = M, n_params, int(twopoint)
        info.n_bc_pts = len(bc_t)
        info.La, info.Lb = La, Lb
        for k, t in enumerate(bc_t):
            info.bc_t[k] = float(t)
        self.info = info
        L = self.lib
        L.oracle_solve_batch.restype = C.c_int
        L.oracle_residual.restype = C.c_double
        L.oracle_defect.restype = C.c_double
        L.oracle_jacobian.restype = C.c_int
        L.oracle_newton_step.restype = C.c_int
        L.oracle_firk_solve_batch.restype = C.c_int
        L.oracle_firk_residual.restype = C.c_double
        L.oracle_firk_tableau.restype = C.c_int

    def options(self, **kw) -> Options:
        o = Options()
        self.lib.oracle_default_options(C.byref(o))
        if isinstance(kw.get("controller"), str):
            kw["controller"] = CONTROLLERS[kw["controller"]]
        if isinstance(kw.get("global_method"), str):
            kw["global_method"] = GLOBAL_METHODS[kw["global_method"]]
        for k, v in kw.items():
            if not hasattr(o, k):
                raise KeyError(k)
            setattr(o, k, v)
        return o

    def solve_batch(self, params, n_intervals, tspans, y0, *, y0_mode=0, cap_nodes=None,
                    want_stages=False, **opts):
        """Solve n independent instances. Returns a dict of numpy arrays."""
        o = self.options(**opts)
        params = np.ascontiguousarray(params, dtype=np.float64).reshape(len(n_intervals), -1)
        n_int = np.ascontiguousarray(n_intervals, dtype=np.int32)
        n = len(n_int)
        tsp = np.ascontiguousarray(tspans, dtype=np.float64).reshape(n, 2)
        y0a = np.ascontiguousarray(y0, dtype=np.float64).ravel()
        if cap_nodes is None:
            cap_nodes = int(max(int(n_int.max()) + 1, 4 * int(n_int.max()) + 1,
                                o.max_subintervals + 1))
        M = self.M
        s, ns = stage_counts(o.order, o.mirk6i)
        out = dict(
            retcode=np.zeros(n, np.int32), n_nodes=np.zeros(n, np.int32),
            mesh=np.zeros((n, cap_nodes)), y=np.zeros((n, cap_nodes, M)),
            newton_iters=np.zeros(n, np.int32), rounds=np.zeros(n, np.int32),
            defect=np.zeros(n), resid=np.zeros(n), global_err=np.zeros(n),
        )
        K = KI = None
        if want_stages:
            K = np.zeros((n, cap_nodes - 1, s, M))
            KI = np.zeros((n, cap_nodes - 1, ns, M))
        rc = self.lib.oracle_solve_batch(
            C.byref(self.info), C.byref(o), C.c_int(n), _p(params, C.c_double),
            _p(n_int, C.c_int32), _p(tsp, C.c_double), C.c_int(y0_mode), _p(y0a, C.c_double),
            C.c_int(cap_nodes), _p(out["retcode"], C.c_int32), _p(out["n_nodes"], C.c_int32),
            _p(out["mesh"], C.c_double), _p(out["y"], C.c_double),
            _p(out["newton_iters"], C.c_int32), _p(out["rounds"], C.c_int32),
            _p(out["defect"], C.c_double), _p(out["resid"], C.c_double),
            _p(K, C.c_double), _p(KI, C.c_double), _p(out["global_err"], C.c_double))
        if rc == -3:
            raise ValueError("HOErrorControl needs MIRK(order + 2): orders 2, 3 and 4 only")
        if rc != 0:
            raise RuntimeError(f"oracle_solve_batch failed: {rc}")
        if want_stages:
            out["K"], out["KI"] = K, KI
        return out

    def firk_solve_batch(self, family, stages, params, n_intervals, tspans, y0, *, y0_mode=0, cap_nodes=None,
                         want_stages=False, **opts):
        """Expanded FIRK solve of n instances (family: FIRK_FAMILIES key or index)."""
        fam = FIRK_FAMILIES[family] if isinstance(family, str) else int(family)
        o = self.options(**opts)
        params = np.ascontiguousarray(params, dtype=np.float64).reshape(len(n_intervals), -1)
        n_int = np.ascontiguousarray(n_intervals, dtype=np.int32)
        n = len(n_int)
        tsp = np.ascontiguousarray(tspans, dtype=np.float64).reshape(n, 2)
        y0a = np.ascontiguousarray(y0, dtype=np.float64).ravel()
        if cap_nodes is None:
            cap_nodes = int(max(int(n_int.max()) + 1, 4 * int(n_int.max()) + 1, o.max_subintervals + 1))
        M = self.M
        out = dict(retcode=np.zeros(n, np.int32), n_nodes=np.zeros(n, np.int32),
                   mesh=np.zeros((n, cap_nodes)), y=np.zeros((n, cap_nodes, M)),
                   newton_iters=np.zeros(n, np.int32), rounds=np.zeros(n, np.int32),
                   defect=np.zeros(n), resid=np.zeros(n))
        K = np.zeros((n, cap_nodes - 1, stages, M)) if want_stages else None
        rc = self.lib.oracle_firk_solve_batch(
            C.byref(self.info), C.byref(o), C.c_int(fam), C.c_int(stages), C.c_int(n), _p(params, C.c_double),
            _p(n_int, C.c_int32), _p(tsp, C.c_double), C.c_int(y0_mode), _p(y0a, C.c_double), C.c_int(cap_nodes),
            _p(out["retcode"], C.c_int32), _p(out["n_nodes"], C.c_int32), _p(out["mesh"], C.c_double),
            _p(out["y"], C.c_double), _p(out["newton_iters"], C.c_int32), _p(out["rounds"], C.c_int32),
            _p(out["defect"], C.c_double), _p(out["resid"], C.c_double), _p(K, C.c_double))
        if rc == -2:
            raise ValueError(f"no FIRK scheme {family} with {stages} stages")
        if rc == -3:
            raise ValueError("the FIRK path evaluates standard BCs at the tspan's ends only")
        if rc != 0:
            raise RuntimeError(f"oracle_firk_solve_batch failed: {rc}")
        if want_stages:
            out["K"] = K
        return out

    def firk_tableau(self, family, stages):
        """(order, s, tau*, c, b, a, q) of a FIRK scheme as the oracle computes them."""
        fam = FIRK_FAMILIES[family] if isinstance(family, str) else int(family)
        buf = np.zeros(115)
        if self.lib.oracle_firk_tableau(C.c_int(fam), C.c_int(stages), _p(buf, C.c_double)) != 0:
            raise ValueError("no such scheme")
        s = int(buf[1])
        return (int(buf[0]), s, float(buf[2]), buf[3:3 + s].copy(), buf[10:10 + s].copy(),
                buf[17:66].reshape(7, 7)[:s, :s].copy(), buf[66:115].reshape(7, 7)[:s, :s].copy())

    def firk_residual(self, family, stages, params, mesh, y, K):
        fam = FIRK_FAMILIES[family] if isinstance(family, str) else int(family)
        params, mesh, y = self._prep(params, mesh, y)
        N, M = len(mesh), self.M
        K = np.ascontiguousarray(K, dtype=np.float64).reshape(N - 1, stages, M)
        F = np.zeros(N * M)
        Fs = np.zeros((N - 1, stages, M))
        o = self.options()
        nrm = self.lib.oracle_firk_residual(C.byref(self.info), C.byref(o), C.c_int(fam), C.c_int(stages),
                                            _p(params, C.c_double), C.c_int(N), _p(mesh, C.c_double),
                                            _p(y, C.c_double), _p(K, C.c_double), _p(F, C.c_double),
                                            _p(Fs, C.c_double))
        return F, Fs, nrm

    def _prep(self, params, mesh, y):
        params = np.ascontiguousarray(params, dtype=np.float64).ravel()
        mesh = np.ascontiguousarray(mesh, dtype=np.float64).ravel()
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(len(mesh), self.M)
        return params, mesh, y

    def residual(self, params, mesh, y, order=4, mirk6i=0):
        params, mesh, y = self._prep(params, mesh, y)
        N, M = len(mesh), self.M
        s = stage_counts(order, mirk6i)[0]
        F = np.zeros(N * M)
        K = np.zeros((N - 1, s, M))
        o = self.options(order=order, mirk6i=mirk6i)
        nrm = self.lib.oracle_residual(C.byref(self.info), C.byref(o), _p(params, C.c_double),
                                       C.c_int(N), _p(mesh, C.c_double), _p(y, C.c_double),
                                       _p(F, C.c_double), _p(K, C.c_double))
        return F, K, nrm

    def jacobian(self, params, mesh, y, order=4, bc_jac_exact=0, mirk6i=0):
        params, mesh, y = self._prep(params, mesh, y)
        N, M = len(mesh), self.M
        S = np.zeros((N - 1, M, M)); R = np.zeros((N - 1, M, M))
        nodes = np.zeros(64, np.int32); blocks = np.zeros((64, M, M))
        o = self.options(order=order, bc_jac_exact=bc_jac_exact, mirk6i=mirk6i)
        nb = self.lib.oracle_jacobian(C.byref(self.info), C.byref(o), _p(params, C.c_double),
                                      C.c_int(N), _p(mesh, C.c_double), _p(y, C.c_double),
                                      _p(S, C.c_double), _p(R, C.c_double),
                                      _p(nodes, C.c_int32), _p(blocks, C.c_double))
        return S, R, nodes[:nb].copy(), blocks[:nb].copy()

    def newton_step(self, params, mesh, y, order=4, bc_jac_exact=0, mirk6i=0):
        params, mesh, y = self._prep(params, mesh, y)
        N, M = len(mesh), self.M
        d = np.zeros(N * M)
        o = self.options(order=order, bc_jac_exact=bc_jac_exact, mirk6i=mirk6i)
        rc = self.lib.oracle_newton_step(C.byref(self.info), C.byref(o), _p(params, C.c_double),
                                         C.c_int(N), _p(mesh, C.c_double), _p(y, C.c_double),
                                         _p(d, C.c_double))
        if rc != 0:
            raise RuntimeError("singular system")
        return d.reshape(N, M)

    def collocation_root(self, params, mesh, y, order=4, mirk6i=0, max_steps=8):
        """The exact root of the collocation equations on a fixed mesh, reached from y by
        Newton steps with the exact Jacobian (the BC rows chained through the interpolant's
        stages); used to measure how far an accepted iterate (||F||_inf <= abstol) lies from
        the discrete solution it approximates."""
        params, mesh, y = self._prep(params, mesh, y)
        y = y.copy()
        for _ in range(max_steps):
            d = self.newton_step(params, mesh, y, order=order, bc_jac_exact=1, mirk6i=mirk6i)
            y += d
            if np.abs(d).max() <= 1e-14 * max(1.0, np.abs(y).max()):
                break
        return y

    def defect(self, params, mesh, y, order=4, mirk6i=0):
        params, mesh, y = self._prep(params, mesh, y)
        N = len(mesh)
        err = np.zeros(N - 1)
        o = self.options(order=order, mirk6i=mirk6i)
        dn = self.lib.oracle_defect(C.byref(self.info), C.byref(o), _p(params, C.c_double),
                                    C.c_int(N), _p(mesh, C.c_double), _p(y, C.c_double),
                                    _p(err, C.c_double))
        return err, dn

    def interpolate(self, order, mesh, y, K, KI, ts, deriv=0, mirk6i=0):
        mesh = np.ascontiguousarray(mesh, dtype=np.float64)
        N = len(mesh)
        y = np.ascontiguousarray(y[:N], dtype=np.float64)
        K = np.ascontiguousarray(K[:N - 1], dtype=np.float64)
        KI = np.ascontiguousarray(KI[:N - 1], dtype=np.float64)
        ts = np.ascontiguousarray(np.atleast_1d(ts), dtype=np.float64)
        out = np.zeros((len(ts), self.M))
        self.lib.oracle_interpolate(C.c_int(7 if mirk6i else order), C.c_int(N), _p(mesh, C.c_double),
                                    _p(y, C.c_double), _p(K, C.c_double), _p(KI, C.c_double),
                                    C.c_int(len(ts)), _p(ts, C.c_double), C.c_int(deriv),
                                    _p(out, C.c_double))
        return out

    def uniform_mesh(self, t0, t1, n):
        m = np.zeros(n + 1)
        self.lib.oracle_uniform_mesh(C.c_double(t0), C.c_double(t1), C.c_int(n), _p(m, C.c_double))
        return m
