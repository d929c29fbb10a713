"""bvp_mlp_forward_noalloc: the surrogate forward on the library's static device scratch.

Checked against bvp_mlp_forward_device (the same kernels on the network's own buffers) on
two calls in a row; the calls must leave the device's free memory unchanged; a batch that
does not fit the static scratch is refused before any work. The file name puts it last in
collection so that it also runs after every other GPU test in the same process."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WIDTHS = [3, 256, 256, 256, 128]
SCRATCH = 8 << 20   # BVP_MLP_NOALLOC_SCRATCH_BYTES


def _net(pkg, rng):
    net = pkg.MLP(WIDTHS, seed=7)
    p = net.get_params()
    p += rng.normal(0, 0.05, p.size).astype(np.float32)
    net.set_params(p)
    net.set_normalization(rng.normal(0, 1, 3), rng.uniform(0.5, 2, 3), rng.normal(0, 1, 128),
                          rng.uniform(0.5, 2, 128))
    return net


@pytest.mark.parametrize("batch", [37, 4096])
def test_noalloc_forward_matches_forward_device(pkg, batch):
    import torch
    rng = np.random.default_rng(11)
    net = _net(pkg, rng)
    x = torch.tensor(rng.normal(0, 1, (batch, 3)).astype(np.float32), device="cuda")
    y_ref = torch.empty(batch, 128, device="cuda")
    net.forward_device(x, y_ref, batch)
    torch.cuda.synchronize()
    s = torch.cuda.current_stream().cuda_stream
    y1 = torch.zeros(batch, 128, device="cuda")
    y2 = torch.full((batch, 128), float("nan"), device="cuda")
    net.forward_noalloc(x, y1, batch, s)           # first call on the device: scratch look-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    net.forward_noalloc(x, y1, batch, s)
    net.forward_noalloc(x, y2, batch, s)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    # same kernels on the same operands: tolerance 1e-6 relative (expected bit-identical)
    scale = float(y_ref.abs().max())
    for y in (y1, y2):
        assert torch.isfinite(y).all()
        assert float((y - y_ref).abs().max()) <= 1e-6 * scale


def test_noalloc_forward_refuses_a_batch_larger_than_its_scratch(pkg):
    import torch
    rng = np.random.default_rng(12)
    net = _net(pkg, rng)
    wmax = max(WIDTHS)
    r256 = lambda b: (b + 255) // 256 * 256
    B = 4097                                        # one row more than fits a 256-wide network
    assert 2 * r256(B * wmax * 2) + r256(B * wmax * 4) > SCRATCH
    x = torch.zeros(B, 3, device="cuda")
    y = torch.zeros(B, 128, device="cuda")
    st = net.lib.bvp_mlp_forward_noalloc(net.h, B, x.data_ptr(), y.data_ptr(), None)
    assert st == 6                                   # BVP_ERR_TOO_LARGE
    with pytest.raises(pkg.BVPError, match="does not fit"):
        net.forward_noalloc(x, y, B)
    assert float(y.abs().max()) == 0.0               # refused before any work
