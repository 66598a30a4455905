"""Host logic of the layer mirrors that runs without a GPU: argument checks
that mirror the reference's error behaviour, the coarse-to-fine step's
gradient branch (pure tensor arithmetic), and the ops' refusal of host
tensors (no CPU fallback)."""
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
