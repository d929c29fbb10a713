"""Problem sources for the MIRK path: the benchmark families and the reference's golden
test problems, written in the library's problem-source format.

A problem source defines the right-hand side and the boundary conditions as C++
templates; the library JIT-compiles the same text for the GPU (NVRTC) and the oracle
compiles it for the CPU:

    BVP_F  { du[k] = ...(u, p, t) ... }          f(u, p, t)
    BVP_BC { res[k] = ...(ua[j][m], p) ... }     standard BVP, ua[j] = u(bc_t[j])
    BVP_BCA / BVP_BCB { res[k] = ... }           two-point BVP, residuals at a and b

``T`` is the state scalar type (double, float or a dual number) and ``P`` the parameter
type; write constants as ``P(...)`` to stay in the caller's precision.

Each problem mirrors one used by the reference: the pendulum of
``benchmark/simple_pendulum.jl:5-32``; the golden problems of
``lib/BoundaryValueDiffEqMIRK/test/Core/mirk_basic_tests.jl`` (affine f1 and linear f2,
lines 16-33 and 69-94; the two-point and multipoint interpolation problems, lines 181-312;
the torus geodesic, lines 726-756) and the ensemble problem of
``lib/BoundaryValueDiffEqMIRK/test/Core/ensemble_tests.jl:7-41``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass(frozen=True)
class Problem:
    name: str
    M: int
    n_params: int
    source: str
    twopoint: bool = False
    bc_t: tuple = ()
    La: int = 0
    Lb: int = 0
    tspan: tuple = (0.0, 1.0)
    u0: tuple = field(default=())


HALF_PI = "P(1.5707963267948966)"

# Simple pendulum family: p = (g, delta_a, delta_b); BCs theta(pi/4) = -pi/2 + delta_a,
# theta(pi/2) = pi/2 + delta_b. With p = (9.81, 0, 0) this is the reference benchmark.
PENDULUM = Problem(
    name="pendulum", M=2, n_params=3,
    source=f"""
BVP_F {{
    du[0] = u[1];
    du[1] = -p[0] * sin(u[0]);
}}
BVP_BC {{
    res[0] = ua[0][0] + {HALF_PI} - p[1];
    res[1] = ua[1][0] - {HALF_PI} - p[2];
}}
""",
    bc_t=(math.pi / 4, math.pi / 2), tspan=(0.0, math.pi / 2), u0=(math.pi / 2, math.pi / 2))

# Singularly perturbed eps*y'' + y' + y = 0, y(0) = 1, y(1) = 0 as a two-point system;
# p = (eps,).
SINGULAR_PERTURBATION = Problem(
    name="singular_perturbation", M=2, n_params=1,
    source="""
BVP_F {
    du[0] = u[1];
    du[1] = -(u[1] + u[0]) / p[0];
}
BVP_BCA { res[0] = ua[0] - P(1.0); }
BVP_BCB { res[0] = ub[0]; }
""",
    twopoint=True, La=1, Lb=1, tspan=(0.0, 1.0), u0=(0.0, 0.0))


def nonlinear32_source(n: int = 32) -> str:
    """u' = A u + tanh(B u) + c, first n/2 components fixed at t=0 and the rest at t=1.
    p = (A (n*n, row-major), B (n*n), c (n), a (n/2), b (n/2))."""
    h = n // 2
    return f"""
BVP_F {{
    const P* A = p;
    const P* B = p + {n * n};
    const P* c = p + {2 * n * n};
    for (int k = 0; k < {n}; ++k) {{
        T s1 = T(P(0.0)), s2 = T(P(0.0));
        for (int j = 0; j < {n}; ++j) {{
            s1 = s1 + A[k * {n} + j] * u[j];
            s2 = s2 + B[k * {n} + j] * u[j];
        }}
        du[k] = s1 + tanh(s2) + c[k];
    }}
}}
BVP_BCA {{
    for (int k = 0; k < {h}; ++k) res[k] = ua[k] - p[{2 * n * n + n} + k];
}}
BVP_BCB {{
    for (int k = 0; k < {h}; ++k) res[k] = ub[{h} + k] - p[{2 * n * n + n + h} + k];
}}
"""


NONLINEAR32 = Problem(
    name="nonlinear32", M=32, n_params=2 * 32 * 32 + 32 + 32,
    source=nonlinear32_source(32), twopoint=True, La=16, Lb=16, tspan=(0.0, 1.0),
    u0=tuple([0.0] * 32))

# --- golden problems of the reference's test suite -------------------------------------
AFFINE = Problem(
    name="affine", M=2, n_params=0,
    source="""
BVP_F { du[0] = u[1]; du[1] = T(P(0.0)); }
BVP_BC { res[0] = ua[0][0] - P(5.0); res[1] = ua[1][0]; }
""",
    bc_t=(0.0, 5.0), tspan=(0.0, 5.0), u0=(5.0, -3.5))

AFFINE_TWOPOINT = Problem(
    name="affine_twopoint", M=2, n_params=0,
    source="""
BVP_F { du[0] = u[1]; du[1] = T(P(0.0)); }
BVP_BCA { res[0] = ua[0] - P(5.0); }
BVP_BCB { res[0] = ub[0]; }
""",
    twopoint=True, La=1, Lb=1, tspan=(0.0, 5.0), u0=(5.0, -3.5))

LINEAR = Problem(
    name="linear", M=2, n_params=0,
    source="""
BVP_F { du[0] = u[1]; du[1] = -u[0]; }
BVP_BC { res[0] = ua[0][0] - P(5.0); res[1] = ua[1][0]; }
""",
    bc_t=(0.0, 5.0), tspan=(0.0, 5.0), u0=(5.0, -3.5))

LINEAR_TWOPOINT = Problem(
    name="linear_twopoint", M=2, n_params=0,
    source="""
BVP_F { du[0] = u[1]; du[1] = -u[0]; }
BVP_BCA { res[0] = ua[0] - P(5.0); }
BVP_BCB { res[0] = ub[0]; }
""",
    twopoint=True, La=1, Lb=1, tspan=(0.0, 5.0), u0=(5.0, -3.5))


# Lane-Emden equation of index 1, y'' + (2/t) y' + y = 0, y(0) = 1, y(1) = sin(1), written as
# u' = S u / t + f(t, u) with u = (y, y'), f = (u2, -u1), S = [[0, 0], [0, -2]] (the problem the
# reference's singular-BVP test describes, lib/BoundaryValueDiffEqMIRK/test/Core/
# singular_bvp_tests.jl:14-50); exact solution y = sin(t)/t
LANE_EMDEN = Problem(
    name="lane_emden", M=2, n_params=0,
    source="""
BVP_F { du[0] = u[1]; du[1] = -u[0]; }
BVP_SING { su[0] = T(P(0.0)); su[1] = u[1] * P(-2.0); }
BVP_BCA { res[0] = ua[0] - P(1.0); }
BVP_BCB { res[0] = ub[0] - P(0.8414709848078965); }
""",
    twopoint=True, La=1, Lb=1, tspan=(0.0, 1.0), u0=(1.0, 0.0))


def lane_emden_analytic(t):
    t = np.asarray(t, dtype=np.float64)
    ts = np.where(t == 0, 1.0, t)
    y = np.where(t == 0, 1.0, np.sin(ts) / ts)
    yp = np.where(t == 0, 0.0, (ts * np.cos(ts) - np.sin(ts)) / ts ** 2)
    return np.stack([y, yp], -1)


# Mathieu eigenvalue: y'' + (lambda - 10 cos 2t) y = 0 on (0, pi), y'(0) = 0, y(0) = 1, y'(pi) = 0,
# with the unknown lambda carried as a third state (lambda' = 0), which is how the reference's
# tune_parameters solves it (lib/BoundaryValueDiffEqMIRK/test/Core/mirk_basic_tests.jl:485-507:
# guess (cos 4t, -4 sin 4t), lambda = 15, MIRK4, dt = 0.05; lambda = 17.09658 within 1e-4)
MATHIEU = Problem(
    name="mathieu", M=3, n_params=0,
    source="""
BVP_F { du[0] = u[1]; du[1] = -(u[2] - P(10.0) * cos(P(2.0) * t)) * u[0]; du[2] = T(P(0.0)); }
BVP_BCA { res[0] = ua[1]; res[1] = ua[0] - P(1.0); }
BVP_BCB { res[0] = ub[1]; }
""",
    twopoint=True, La=2, Lb=1, tspan=(0.0, math.pi), u0=(1.0, 0.0, 15.0))


def mathieu_guess(n_intervals: int):
    """The reference test's guess (cos 4t, -4 sin 4t) and lambda = 15 on the uniform initial mesh."""
    t = np.array([math.pi if i == n_intervals else i * (math.pi / n_intervals) for i in range(n_intervals + 1)])
    return np.stack([np.cos(4 * t), -4 * np.sin(4 * t), np.full_like(t, 15.0)], -1)


def linear_analytic(t):
    t = np.asarray(t, dtype=np.float64)
    cot5 = math.cos(5.0) / math.sin(5.0)
    return np.stack([5 * (np.cos(t) - cot5 * np.sin(t)), 5 * (-np.cos(t) * cot5 - np.sin(t))], -1)


# u'' = u / lambda, u(0) = 1, u(1) = 0; p = (lambda,)
TWOPOINT_INTERP = Problem(
    name="twopoint_interp", M=2, n_params=1,
    source="""
BVP_F { du[0] = u[1]; du[1] = (P(1.0) / p[0]) * u[0]; }
BVP_BC { res[0] = ua[0][0] - P(1.0); res[1] = ua[1][0]; }
""",
    bc_t=(0.0, 1.0), tspan=(0.0, 1.0), u0=(1.0, 0.0))


def twopoint_interp_analytic(t, lam=1.0):
    a = 1 / math.sqrt(lam)
    t = np.asarray(t, dtype=np.float64)
    den = 1 - math.exp(-2 * a)
    u = (np.exp(-a * t) - np.exp((t - 2) * a)) / den
    du = (-a * np.exp(-t * a) - a * np.exp((t - 2) * a)) / den
    ddu = (a * a * np.exp(-a * t) - a * a * np.exp((t - 2) * a)) / den
    return np.stack([u, du], -1), np.stack([du, ddu], -1)


# u'' = -u with independent multipoint BCs u1(pi/6) = 1/2, u2(pi/3) = 1/2 -> (sin, cos)
MULTIPOINT = Problem(
    name="multipoint", M=2, n_params=0,
    source="""
BVP_F { du[0] = u[1]; du[1] = -u[0]; }
BVP_BC { res[0] = ua[0][0] - P(0.5); res[1] = ua[1][1] - P(0.5); }
""",
    bc_t=(math.pi / 6, math.pi / 3), tspan=(0.0, math.pi / 2), u0=(0.0, 1.0))

# geodesics on a torus (R=3, r=2), M=4; p = (a1_0, a1_1, a2_0, a2_1)
TORUS = Problem(
    name="torus", M=4, n_params=4,
    source="""
BVP_F {
    const T sth = sin(u[0]);
    const T cth = cos(u[0]);
    const T Rt = P(3.0) + P(2.0) * cth;
    du[0] = u[2];
    du[1] = u[3];
    du[2] = -(u[3] * u[3]) * Rt * sth / P(2.0);
    du[3] = P(2.0) * P(2.0) * sth / Rt * u[2] * u[3];
}
BVP_BC {
    res[0] = ua[0][0] - p[0]; res[1] = ua[0][1] - p[1];
    res[2] = ua[1][0] - p[2]; res[3] = ua[1][1] - p[3];
}
""",
    bc_t=(0.0, 1.0), tspan=(0.0, 1.0), u0=(0.5, -1.2, 0.0, 0.0))

# u'' = -p u, u(0) = 1, u(1) = 0 on (0, pi/2): the reference's ensemble problem
ENSEMBLE = Problem(
    name="ensemble", M=2, n_params=1,
    source="""
BVP_F { du[0] = u[1]; du[1] = -p[0] * u[0]; }
BVP_BC { res[0] = ua[0][0] - P(1.0); res[1] = ua[1][0]; }
""",
    bc_t=(0.0, 1.0), tspan=(0.0, math.pi / 2), u0=(0.0, 1.0))


# --- seeded instance families of the benchmark workloads --------------------------------

def pendulum_family(n: int, seed: int = 2024, n_min: int = 32, n_max: int = 256):
    """4096-instance pendulum batch: g ~ U[5,15], BC targets perturbed by U[-0.2,0.2],
    interval counts uniform on {n_min..n_max}, guess (pi/2, pi/2) at every node."""
    rng = np.random.default_rng(seed)
    g = rng.uniform(5.0, 15.0, n)
    da = rng.uniform(-0.2, 0.2, n)
    db = rng.uniform(-0.2, 0.2, n)
    nint = rng.integers(n_min, n_max + 1, n).astype(np.int32)
    params = np.stack([g, da, db], 1)
    tspans = np.tile([0.0, math.pi / 2], (n, 1))
    y0 = np.tile([math.pi / 2, math.pi / 2], (n, 1))
    return params, nint, tspans, y0


def singular_perturbation_family(n: int, seed: int = 2025, n_min: int = 512, n_max: int = 4096):
    """eps log-uniform in [1e-3, 1e-1], interval counts log-uniform integers in
    [n_min, n_max], zero guess."""
    rng = np.random.default_rng(seed)
    eps = np.exp(rng.uniform(math.log(1e-3), math.log(1e-1), n))
    nint = np.exp(rng.uniform(math.log(n_min), math.log(n_max), n)).round().astype(np.int32)
    nint = np.clip(nint, n_min, n_max)
    params = eps[:, None]
    tspans = np.tile([0.0, 1.0], (n, 1))
    y0 = np.zeros((n, 2))
    return params, nint, tspans, y0


def nonlinear32_family(n: int, seed: int = 2026, n_intervals: int = 1024, dim: int = 32):
    """A, B ~ N(0, 1/dim), c ~ N(0, 0.1^2), BC values ~ U[-1, 1]; per-instance seeds."""
    params = np.zeros((n, 2 * dim * dim + 2 * dim))
    for i in range(n):
        rng = np.random.default_rng([seed, i])
        A = rng.normal(0, 1 / math.sqrt(dim), (dim, dim))
        B = rng.normal(0, 1 / math.sqrt(dim), (dim, dim))
        c = rng.normal(0, 0.1, dim)
        ab = rng.uniform(-1, 1, dim)
        params[i] = np.concatenate([A.ravel(), B.ravel(), c, ab])
    nint = np.full(n, n_intervals, np.int32)
    tspans = np.tile([0.0, 1.0], (n, 1))
    y0 = np.zeros((n, dim))
    return params, nint, tspans, y0


ALL = {p.name: p for p in (PENDULUM, SINGULAR_PERTURBATION, NONLINEAR32, LANE_EMDEN, MATHIEU, AFFINE, AFFINE_TWOPOINT,
                           LINEAR, LINEAR_TWOPOINT, TWOPOINT_INTERP, MULTIPOINT, TORUS, ENSEMBLE)}
