"""MessagePassing's fused node (BPLayerFn: the passes and the belief
epilogue as one autograd node) against the composition it replaces
(LBPMinSumLoop + BeliefsSoftmin, fused=False), FP32 and FP16 storage.

The forward is the same arithmetic on the same inputs (the beliefs read the
probability volume with the sign folded in, which is exact), so beliefs and
messages are bit-identical.  The gradients differ only in the order of the
float additions of the cost's two gradients (and of the adjoint's atomics,
unordered in both): within a few ulps of the gradient's scale."""
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _inputs(seed, B, H, W, L):
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev).manual_seed(seed)
    d0 = torch.randint(0, L, (B, H, W, 1), device=dev, generator=g).float()
    lab = torch.arange(L, device=dev).float().view(1, 1, 1, L)
    sad = 4.0 * (lab - d0).abs().clamp(max=5) + torch.rand((B, H, W, L), device=dev, generator=g)
    prob = torch.softmax(-sad, -1).contiguous()
    edge = torch.exp(0.3 * torch.randn((B, 4, H, W), device=dev, generator=g)).contiguous()
    up = torch.randn((B, H, W, L), device=dev, generator=g)
    upm = torch.randn((B, 4, H, W, L), device=dev, generator=g)
    return prob, edge, up, upm


def _run(storage, fused, prob, edge, up, upm, use_messages):
    from bpl_gb300.layers.stereo import MessagePassing
    dev = prob.device
    B, H, W, L = prob.shape
    mp = MessagePassing(dev, 3, L, 3, storage=storage, fused=fused)
    with torch.no_grad():
        mp._L1.fill_(0.1)
        mp._L2.fill_(0.5)
        mp.softmin.T.fill_(0.7)
    p = prob.clone().requires_grad_(True)
    e = edge.clone().requires_grad_(True)
    m0 = torch.zeros((B, 4, H, W, L), device=dev, requires_grad=True) if storage == "fp32" else None
    beliefs, messages = mp(p, e, None, None, m0)
    loss = (beliefs * up).sum()
    if use_messages:
        loss = loss + (messages[..., :L].float() * upm).sum()
    loss.backward()
    grads = {"prob": p.grad, "edge": e.grad, "L1": mp._L1.grad, "L2": mp._L2.grad, "T": mp.softmin.T.grad}
    if m0 is not None:
        grads["messages"] = m0.grad
    return beliefs.detach(), messages.detach(), grads


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
@pytest.mark.parametrize("L,use_messages", [(40, False), (192, False), (40, True)])
def test_fused_node_matches_the_composition(storage, L, use_messages):
    prob, edge, up, upm = _inputs(L + (7 if use_messages else 0), 2, 24, 36, L)
    b1, m1, g1 = _run(storage, True, prob, edge, up, upm, use_messages)
    b0, m0, g0 = _run(storage, False, prob, edge, up, upm, use_messages)
    assert torch.equal(b1, b0), "beliefs differ"
    assert torch.equal(m1, m0), "messages differ"
    assert set(g1) == set(g0)
    for k in g0:
        a, b = g1[k], g0[k]
        assert a is not None and b is not None, k
        scale = b.abs().max().item()
        err = (a - b).abs().max().item()
        # the temperature's gradient is one sum over every (pixel, label),
        # reduced by unordered float atomics on either path
        rtol = 1e-4 if k == "T" else 1e-5
        assert err <= rtol * max(scale, 1e-30) + 1e-7, f"{storage} L={L} {k}: max err {err:.3e}, scale {scale:.3e}"
    if storage == "fp32" and not use_messages:
        # the leaf message gradient is the beliefs' gradient in every slot,
        # written by the beliefs' backward itself: bit-identical
        assert torch.equal(g1["messages"], g0["messages"])


def test_half_padded_matches_torch():
    from bpl_gb300 import ops
    dev = torch.device("cuda:0")
    for L in (192, 61, 5):
        x = torch.randn((3, 7, 11, L), device=dev)
        got = ops.half_padded(x, -1.0)
        want = ops.to_half_padded(-x, L)
        assert got.shape == want.shape and torch.equal(got, want)


@pytest.mark.parametrize("half", [False, True])
def test_layer_taps_adjoint_matches_the_plain_taps(half):
    """bpl_lbp_backward_passes_into with layer_taps: the layer's packed taps
    [offset, L2, L1, 0, L1, L2] binned three ways.  Against the plain
    adjoint: tap 1 = taps 1 + 5, taps 2 and 4 and the edge and cost
    gradients equal up to float order, taps 3 and 5 none."""
    from bpl_gb300 import ops
    from bpl_gb300.layers.stereo import pack_affinities
    prob, edge, up, _ = _inputs(5, 2, 20, 44, 70)
    dev = prob.device
    B, H, W, L = prob.shape
    aff = 0.05 + 0.5 * torch.rand((B, 4, 3, H, W), device=dev, generator=torch.Generator(device=dev).manual_seed(3))
    taps = pack_affinities(aff, torch.zeros((B, 4, H, W), device=dev))
    Ls = ops.padded_labels(L) if half else L
    P = 2
    am = torch.empty((P, B, 4, H, W, Ls), dtype=torch.uint8, device=dev)
    if half:
        cost = ops.half_padded(prob, -1.0)
        m = torch.zeros((B, 4, H, W, Ls), dtype=torch.float16, device=dev)
        for k in range(P):
            ops.lbp_forward_f16(ops.LBP_STEREO, cost, taps, edge, m, 3, L, argmin_dtype=torch.uint8, argmin=am[k])
        sc = None
        gin = ops.half_padded(up).unsqueeze(1).expand(B, 4, H, W, Ls)
    else:
        cost = (-prob).contiguous()
        m = torch.zeros((B, 4, H, W, L), device=dev)
        sc = torch.empty((P, B, 4, H, W), device=dev)
        for k in range(P):
            ops.lbp_forward(ops.LBP_STEREO, cost, taps, edge, m, 3, argmin_dtype=torch.uint8, argmin=am[k],
                            scale=sc[k])
        gin = up.unsqueeze(1).expand(B, 4, H, W, L)
    g0 = torch.zeros((B, H, W, L), device=dev)
    g1 = torch.zeros((B, H, W, L), device=dev)
    c0, j0, e0 = ops.lbp_backward_passes(ops.LBP_STEREO, taps, edge, gin, m, am, sc, L=L, grad_cost_into=g0)
    c1, j1, e1 = ops.lbp_backward_passes(ops.LBP_STEREO, taps, edge, gin, m, am, sc, L=L, grad_cost_into=g1,
                                         layer_taps=True)

    def close(a, b, name):
        scale = b.abs().max().item()
        err = (a - b).abs().max().item()
        assert err <= 1e-5 * max(scale, 1e-30) + 1e-7, f"{name}: {err:.3e} of {scale:.3e}"
    close(c1, c0, "grad_cost")
    close(e1, e0, "grad_edge")
    close(j1[:, :, 1], j0[:, :, 1] + j0[:, :, 5], "tap 1 + 5")
    close(j1[:, :, 2], j0[:, :, 2], "tap 2")
    close(j1[:, :, 4], j0[:, :, 4], "tap 4")
    assert bool((j1[:, :, 3] == 0).all()) and bool((j1[:, :, 5] == 0).all())
