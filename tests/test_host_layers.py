"""Host logic of the layer mirrors that runs without a GPU: argument checks
that mirror the reference's error behaviour, the coarse-to-fine step's
gradient branch (pure tensor arithmetic) and the interpolation formula its
kernel evaluates, and the ops' refusal of host tensors (no CPU fallback)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from bpl_gb300 import ops  # noqa: E402
from bpl_gb300.layers.matching import FlowMpSadFunction  # noqa: E402
from bpl_gb300.layers.stereo import BP, MessagePassing, coarse_to_fine  # noqa: E402


def test_flow_layer_rejects_unsupported_windows_like_the_reference():
    f = torch.zeros((1, 2, 4, 4))
    for sws in (109, 150, 432):
        with pytest.raises(ValueError):
            FlowMpSadFunction.apply(f, f, sws)


def test_message_passing_and_bp_argument_checks():
    dev = torch.device("cpu")
    with pytest.raises(ValueError):
        MessagePassing(dev, 1, 8, 3, mode="sum-product")
    with pytest.raises(ValueError):
        MessagePassing(dev, 1, 8, 3, storage="fp8")
    with pytest.raises(ValueError):
        MessagePassing(dev, 1, 8, 3, storage="fp16", adjoint="exact")
    with pytest.raises(ValueError):
        BP(dev, None, 1, 8, 3, mode_inference="median")
    mp = MessagePassing(dev, 1, 8, 3)
    with pytest.raises(ValueError):
        mp.setL1L2(0.5, 0.1)


def test_coarse_to_fine_gradient_branch_normalises_like_the_reference():
    b = torch.rand((1, 3, 4, 5), requires_grad=True)
    pv = torch.rand((1, 6, 8, 10))
    out = coarse_to_fine(b, pv)
    torch.testing.assert_close(out, pv / pv.sum(dim=-1, keepdim=True))
    assert coarse_to_fine(None, pv) is pv


@pytest.mark.parametrize("call", [
    lambda t: ops.upsample_add_beliefs(t, torch.zeros((1, 4, 4, 4))),
    lambda t: ops.broadcast_slots(t),
    lambda t: ops.flow_forward(t, t, 4),
])
def test_ops_refuse_host_tensors(call):
    with pytest.raises(ops.BplError):
        call(torch.zeros((1, 2, 2, 2)))


def _lin2(o, n):
    src = max(np.float32(0.5) * (np.float32(o) + np.float32(0.5)) - np.float32(0.5), np.float32(0.0))
    i0 = int(src)
    i1 = i0 + (1 if i0 < n - 1 else 0)
    l1 = np.float32(src - np.float32(i0))
    return i0, i1, np.float32(1.0) - l1, l1


@pytest.mark.parametrize("shape", [(1, 3, 4, 5), (2, 1, 6, 2), (1, 5, 1, 7)])
def test_upsample_formula_of_the_glue_kernel_matches_torch(shape):
    """The trilinear x2 formula that csrc/pyramid.cu evaluates (source index
    0.5 (o + 0.5) - 0.5 clamped at 0, weights in quarters, rows outside and
    labels inside) against torch's own interpolation on the CPU."""
    import torch.nn.functional as F
    N, h, w, d = shape
    b = np.random.default_rng(7).random(shape, dtype=np.float32)
    ref = F.interpolate(torch.from_numpy(b).unsqueeze(1), scale_factor=2.0, mode="trilinear")[:, 0].numpy()
    out = np.empty((N, 2 * h, 2 * w, 2 * d), np.float32)
    for n in range(N):
        for y in range(2 * h):
            y0, y1, a0, a1 = _lin2(y, h)
            for x in range(2 * w):
                x0, x1, c0, c1 = _lin2(x, w)
                for z in range(2 * d):
                    z0, z1, e0, e1 = _lin2(z, d)
                    row = lambda yy, xx: e0 * b[n, yy, xx, z0] + e1 * b[n, yy, xx, z1]
                    p0 = c0 * row(y0, x0) + c1 * row(y0, x1)
                    p1 = c0 * row(y1, x0) + c1 * row(y1, x1)
                    out[n, y, x, z] = a0 * p0 + a1 * p1
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-6)
