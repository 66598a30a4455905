"""The host-side layer mirrors (MessagePassing, LBPMinSumFunction, Inference,
the semantic variants) on the GPU, against the oracle.

The stereo layer is checked end to end: beliefs from 3 iterations, and the
autograd gradients of the cost volume and of L1/L2, which the reference
computes from the final (in-place) messages with every iteration's argmin and
scale, and in_grad passed through unchanged as the message gradient
(ops/lbp_stereo/message_passing_op_cuda.py:62-93, lbp_min_sum_kernel.cu:534-536).
"""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _softmin(x, T=1.0):
    x = -x.astype(np.float64) / T
    x -= x.max(-1, keepdims=True)
    e = np.exp(x)
    return e / e.sum(-1, keepdims=True)


def test_stereo_message_passing_forward_backward():
    from bpl_gb300.layers.stereo import MessagePassing
    dev = torch.device("cuda:0")
    g = cases.rng(3)
    B, H, W, L, iters = 1, 14, 22, 48, 3
    prob = cases.softmax_np(g.normal(0, 2, size=(B, H, W, L)).astype(np.float32))
    edge = cases.edge_weights(g, B, H, W)
    up = g.normal(0, 1, size=(B, H, W, L)).astype(np.float32)
    mp = MessagePassing(dev, iters, L, 3)
    with torch.no_grad():
        mp._L1.fill_(0.1)
        mp._L2.fill_(0.5)
    p = torch.from_numpy(prob).to(dev).requires_grad_(True)
    m0 = torch.zeros((B, 4, H, W, L), device=dev, requires_grad=True)
    beliefs, msgs = mp(p, torch.from_numpy(edge).to(dev), None, None, m0)
    beliefs.backward(torch.from_numpy(up).to(dev))

    # oracle: same iterations, in place
    cost = -prob
    jump = cases.stereo_taps(B, H, W, 0.1, 0.5)
    m = np.zeros((B, 4, H, W, L), np.float32)
    per_it = []
    for _ in range(iters):
        m, am, sc = oracle.lbp_forward(0, cost, jump, edge, m, 3)
        per_it.append((am.copy(), sc.copy()))
    np.testing.assert_array_equal(msgs.detach().cpu().numpy(), m)
    b_ref = _softmin(m.sum(1) + cost)
    np.testing.assert_allclose(beliefs.detach().cpu().numpy(), b_ref, atol=2e-6)

    # gradient: softmin backward, then every iteration's reference adjoint
    # with the final messages and in_grad = d(loss)/d(sum of messages)
    bz = b_ref
    g_sum = -(bz * (up - (up * bz).sum(-1, keepdims=True)))  # d/dz of softmin(z) with z = sum
    gin = np.broadcast_to(g_sum[:, None], (B, 4, H, W, L)).astype(np.float32)
    gcost = g_sum.copy()
    gL1 = gL2 = 0.0
    for am, sc in per_it:
        gc, gj, ge, gm = oracle.lbp_backward_ref(0, jump, edge, gin, m, am, sc)
        gcost += gc
        gL1 += gj[:, :, 2].sum() + gj[:, :, 4].sum()
        gL2 += gj[:, :, 1].sum() + gj[:, :, 5].sum()
    got = p.grad.detach().cpu().numpy()
    np.testing.assert_allclose(got, -gcost, atol=2e-4 * np.abs(gcost).max())
    assert abs(mp._L1.grad.item() - gL1) <= 2e-4 * max(abs(gL1), 1.0)
    assert abs(mp._L2.grad.item() - gL2) <= 2e-4 * max(abs(gL2), 1.0)
    # the initial messages' gradient: in_grad passed through every pass, i.e.
    # the beliefs' gradient in each slot, written out as a dense tensor
    assert m0.grad.is_contiguous() and m0.grad.stride(1) != 0
    np.testing.assert_allclose(m0.grad.cpu().numpy(), gin, atol=2e-6 * max(np.abs(gin).max(), 1.0))


@pytest.mark.parametrize("dtype,shape", [("float32", (2, 5, 7, 48)), ("float16", (1, 3, 5, 24)),
                                         ("float32", (1, 3, 5, 7)), ("float16", (2, 1, 3, 5))])
def test_broadcast_slots(dtype, shape):
    from bpl_gb300 import ops
    dev = torch.device("cuda:0")
    src = torch.randn(shape, device=dev).to(getattr(torch, dtype))
    out = ops.broadcast_slots(src)
    ref = src.unsqueeze(1).expand(shape[0], 4, *shape[1:])
    assert torch.equal(out, ref)
    # leaf_message_grad: a slot-broadcast view is written out, others pass through
    assert torch.equal(ops.leaf_message_grad(ref), ref) and ops.leaf_message_grad(ref).stride(1) != 0
    dense = ref.contiguous()
    assert ops.leaf_message_grad(dense) is dense


def test_inference_modes():
    from bpl_gb300.layers.stereo import Inference
    dev = torch.device("cuda:0")
    g = cases.rng(4)
    b = torch.from_numpy(cases.softmax_np(g.normal(0, 2, size=(2, 5, 7, 16)).astype(np.float32))).to(dev)
    bn = b.cpu().numpy()
    wta = Inference(dev, "wta")(b).cpu().numpy()
    np.testing.assert_array_equal(wta[..., 0], bn.argmax(-1))
    exp_ = Inference(dev, "expectation")(b).cpu().numpy()[..., 0]
    np.testing.assert_allclose(exp_, (bn / bn.sum(-1, keepdims=True) * np.arange(16)).sum(-1), rtol=1e-5)
    sub = Inference(dev, "sub-exp")(b).cpu().numpy()[..., 0]
    d = bn.argmax(-1)
    win = np.clip(d[..., None] + np.arange(-3, 4), 0, 15)
    bw = np.take_along_axis(bn, win, -1)
    np.testing.assert_allclose(sub, (bw / bw.sum(-1, keepdims=True) * win).sum(-1), rtol=1e-5)


@pytest.mark.parametrize("kind", ["global", "global_single", "pixel"])
def test_semantic_message_passing(kind):
    from bpl_gb300.layers.semantic import MessagePassingGlobal, MessagePassingPixel
    dev = torch.device("cuda:0")
    g = cases.rng(5)
    B, H, W, L = 1, 9, 12, 19
    prob = cases.softmax_np(g.normal(0, 2, size=(B, H, W, L)).astype(np.float32))
    edge = cases.edge_weights(g, B, H, W)
    if kind == "pixel":
        j4, jp = cases.semantic_pixel_jump(g, H, W, L)
        mp = MessagePassingPixel(dev, 2, L, L)
        jin = torch.from_numpy(jp).to(dev).requires_grad_(True)
        variant, jref = 2, j4
    else:
        j4, pg = cases.semantic_global_jump(g, L)
        mp = MessagePassingGlobal(dev, 2, L, L)
        if kind == "global_single":
            pg = pg[:, :1]
            j4 = np.ascontiguousarray(np.broadcast_to(pg[:, :1], (1, 4, L, L)))
        jin = torch.from_numpy(pg).to(dev).requires_grad_(True)
        variant, jref = 1, j4
    p = torch.from_numpy(prob).to(dev).requires_grad_(True)
    m0 = torch.zeros((B, 4, H, W, L), device=dev, requires_grad=True)
    if kind == "pixel":
        beliefs = mp(p, torch.from_numpy(edge).to(dev), m0, jin)
    else:
        beliefs = mp(p, torch.from_numpy(edge).to(dev), m0, jin, single_pw=(kind == "global_single"))
    m, _, _ = oracle.lbp_forward(variant, -prob, jref, edge, np.zeros((B, 4, H, W, L), np.float32), L, iters=2)
    np.testing.assert_allclose(beliefs.detach().cpu().numpy(), _softmin(m.sum(1) - prob), atol=2e-6)
    beliefs.sum().backward()
    assert p.grad is not None and torch.isfinite(p.grad).all()
    assert jin.grad is not None and jin.grad.shape == jin.shape and torch.isfinite(jin.grad).all()


@pytest.mark.parametrize("half", [False, True], ids=["fp32", "fp16"])
def test_fused_belief_epilogue_matches_torch(half):
    """BeliefsSoftmin (one kernel each way) against torch's
    softmin((messages.sum(1) + cost) / T): values and the gradients of the
    messages, the cost and the temperature."""
    from bpl_gb300 import ops
    from bpl_gb300.layers.stereo import BeliefsSoftmin
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev).manual_seed(7)
    B, H, W, L = 2, 9, 13, 70
    Ls = ops.padded_labels(L) if half else L
    m = torch.randn((B, 4, H, W, Ls), device=dev, generator=g)
    if half:
        m = m.half()
    cost = torch.randn((B, H, W, L), device=dev, generator=g)
    T = torch.tensor([0.7], device=dev)
    up = torch.randn((B, H, W, L), device=dev, generator=g)

    m1, c1, T1 = m.clone().requires_grad_(True), cost.clone().requires_grad_(True), T.clone().requires_grad_(True)
    y1 = BeliefsSoftmin.apply(m1, c1, T1)
    y1.backward(up)
    m2, c2, T2 = m.clone().requires_grad_(True), cost.clone().requires_grad_(True), T.clone().requires_grad_(True)
    z = (((m2[:, 0, ..., :L].float() + m2[:, 1, ..., :L].float()) + m2[:, 2, ..., :L].float())
         + m2[:, 3, ..., :L].float()) + c2
    y2 = torch.nn.functional.softmin(z / T2, dim=3)
    y2.backward(up)
    assert (y1 - y2).abs().max().item() <= 2e-6
    assert (c1.grad - c2.grad).abs().max().item() <= 1e-5 * max(1.0, c2.grad.abs().max().item())
    gm1, gm2 = m1.grad.float(), m2.grad.float()
    assert (gm1 - gm2).abs().max().item() <= 2e-3 * max(1.0, gm2.abs().max().item())
    assert abs(T1.grad.item() - T2.grad.item()) <= 1e-4 * max(1.0, abs(T2.grad.item()))
