"""bvp_mlp_forward_noalloc: the surrogate forward for callers that cannot allocate device
memory during the call (a serving loop under a fixed memory budget, or work enqueued where a
cudaMalloc would synchronise the device).

Checked against bvp_mlp_forward_device on two calls in a row, for a network the fused kernel
takes (no scratch at all) and for one that runs layer by layer on the library's static
scratch; the calls must leave the device's free memory unchanged, and a batch that does not
fit the static scratch is refused before any work. The file name puts it last in collection
so that it also runs after every other GPU test in the same process."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FUSED = [3, 256, 256, 256, 128]      # every width <= 256: the fused kernel, no scratch
LAYERED = [3, 512, 256, 128]         # a 512-wide layer: layer-by-layer kernels on the static scratch
SCRATCH = 8 << 20                    # BVP_MLP_NOALLOC_SCRATCH_BYTES


def _net(pkg, rng, widths):
    net = pkg.MLP(widths, seed=7)
    p = net.get_params()
    p += rng.normal(0, 0.05, p.size).astype(np.float32)
    net.set_params(p)
    w0, wl = widths[0], widths[-1]
    net.set_normalization(rng.normal(0, 1, w0), rng.uniform(0.5, 2, w0), rng.normal(0, 1, wl),
                          rng.uniform(0.5, 2, wl))
    return net


def _fits(widths, batch):
    r256 = lambda b: (b + 255) // 256 * 256
    w = max(widths)
    return 2 * r256(batch * w * 2) + r256(batch * w * 4) <= SCRATCH


@pytest.mark.parametrize("widths,batch", [(FUSED, 37), (FUSED, 4096), (FUSED, 9000), (LAYERED, 37), (LAYERED, 2048)])
def test_noalloc_forward_matches_forward_device(pkg, widths, batch):
    import torch
    rng = np.random.default_rng(11)
    net = _net(pkg, rng, widths)
    w0, wl = widths[0], widths[-1]
    x = torch.tensor(rng.normal(0, 1, (batch, w0)).astype(np.float32), device="cuda")
    y_ref = torch.empty(batch, wl, device="cuda")
    net.forward_device(x, y_ref, batch)
    torch.cuda.synchronize()
    s = torch.cuda.current_stream().cuda_stream
    y1 = torch.zeros(batch, wl, device="cuda")
    y2 = torch.full((batch, wl), float("nan"), device="cuda")
    net.forward_noalloc(x, y1, batch, s)           # first call on the device: scratch look-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    net.forward_noalloc(x, y1, batch, s)
    net.forward_noalloc(x, y2, batch)              # null stream: the network's own stream
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    # the kernels forward_device runs for this network on the same operands: 1e-6 relative
    scale = float(y_ref.abs().max())
    for y in (y1, y2):
        assert torch.isfinite(y).all()
        assert float((y - y_ref).abs().max()) <= 1e-6 * scale


def test_noalloc_forward_refuses_a_batch_larger_than_its_scratch(pkg):
    import torch
    rng = np.random.default_rng(12)
    net = _net(pkg, rng, LAYERED)
    B = 2049                                        # one row more than fits a 512-wide network
    assert _fits(LAYERED, B - 1) and not _fits(LAYERED, B)
    x = torch.zeros(B, 3, device="cuda")
    y = torch.zeros(B, 128, device="cuda")
    st = net.lib.bvp_mlp_forward_noalloc(net.h, B, x.data_ptr(), y.data_ptr(), None)
    assert st == 6                                   # BVP_ERR_TOO_LARGE
    with pytest.raises(pkg.BVPError, match="does not fit"):
        net.forward_noalloc(x, y, B)
    torch.cuda.synchronize()
    assert float(y.abs().max()) == 0.0               # refused before any work
