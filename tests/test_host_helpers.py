"""CPU checks of the host-side helpers around the library: the guess resampling onto initial
meshes (the host twin of the device kernel), the merge of fallback results into a batch, and
the surrogate's grid times."""
import numpy as np


def test_resample_host_is_exact_for_linear_guesses(pkg):
    from bvdiffeq_gb300.surrogate import resample_host
    G, M = 64, 2
    u = np.linspace(0.0, 1.0, G)
    grid = np.stack([np.stack([3.0 * u - 1.0, -2.0 * u + 0.5], -1), np.stack([u, u], -1)])   # (2, G, M)
    nint = [7, 130]
    out = resample_host(grid, nint)
    assert out.shape == (8 + 131, M)
    for k, (g, n) in enumerate(zip(grid, nint)):
        o = sum(m + 1 for m in nint[:k])
        s = np.arange(n + 1) / n
        seg = out[o:o + n + 1]
        if k == 0:
            assert np.allclose(seg[:, 0], 3.0 * s - 1.0, atol=1e-14) and np.allclose(seg[:, 1], -2.0 * s + 0.5, atol=1e-14)
        else:
            assert np.allclose(seg[:, 0], s, atol=1e-14)
        assert np.array_equal(seg[0], g[0]) and np.allclose(seg[-1], g[-1], atol=1e-14)


def test_merge_results_replaces_the_fallback_instances(pkg):
    from bvdiffeq_gb300.solver import BatchResult
    from bvdiffeq_gb300.surrogate import merge_results

    def result(ns, base):
        off = np.concatenate([[0], np.cumsum(ns)]).astype(np.int64)
        mesh = np.concatenate([np.linspace(0, 1, n) for n in ns])
        y = np.concatenate([np.full((n, 2), base + i) for i, n in enumerate(ns)])
        k = len(ns)
        return BatchResult(retcode=np.full(k, 1 if base == 0 else 0, np.int32), n_nodes=np.array(ns, np.int32),
                           newton_iters=np.full(k, base + 1, np.int32), rounds=np.ones(k, np.int32),
                           defect=np.zeros(k), resid=np.zeros(k), offsets=off, mesh_packed=mesh, y_packed=y)

    base = result([5, 6, 7, 8], 0)
    sub = result([9, 10], 100)
    idx = np.array([1, 3])
    m = merge_results(base, sub, idx, 2)
    assert m.n_nodes.tolist() == [5, 9, 7, 10]
    assert m.retcode.tolist() == [1, 0, 1, 0] and m.newton_iters.tolist() == [1, 101, 1, 101]
    assert m.offsets.tolist() == [0, 5, 14, 21, 31]
    assert np.all(m.solution(1)[1] == 100) and np.all(m.solution(3)[1] == 101)
    assert np.all(m.solution(2)[1] == 2) and len(m.solution(2)[0]) == 7


def test_surrogate_grid_times(pkg):
    # (the network itself lives on the GPU; only the grid layout is checked here)
    from types import SimpleNamespace
    t = pkg.Surrogate.grid_times(SimpleNamespace(grid=5), [[0.0, 2.0], [1.0, 1.5]])
    assert np.allclose(t, [[0.0, 0.5, 1.0, 1.5, 2.0], [1.0, 1.125, 1.25, 1.375, 1.5]])
