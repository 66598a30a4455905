"""Exact adjoint on the GPU (bpl_lbp_backward_exact) against the oracle's
exact adjoint (whose derivative is checked against FP64 central finite
differences in test_exact_adjoint.py), for one pass and through the
MessagePassing layer with adjoint="exact"."""
import gc

import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("shape", [(2, 12, 20, 16), (1, 17, 23, 64)], ids=["b2_l16", "b1_l64"])
def test_exact_backward_single_pass(shape):
    from bpl_gb300 import ops
    dev = torch.device("cuda:0")
    B, H, W, L = shape
    g = cases.rng(31)
    cost = cases.random_cost(g, B, H, W, L)
    edge = cases.edge_weights(g, B, H, W)
    jump = cases.stereo_taps(B, H, W, 0.1, 0.5)
    m_in = g.normal(0, 0.3, size=(B, 4, H, W, L)).astype(np.float32)
    G = g.normal(0, 1, size=(B, 4, H, W, L)).astype(np.float32)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    m, am, sc = ops.lbp_forward(0, t(cost), t(jump), t(edge), t(m_in), 3, argmin_dtype=torch.uint8)
    gc, gj, ge, gm = ops.lbp_backward(0, t(jump), t(edge), t(G), m, am, sc, mode="exact")
    ref = oracle.lbp_backward_exact(0, jump, edge, G, m.cpu().numpy(), am.cpu().numpy().astype(np.float32),
                                    sc.cpu().numpy())
    for name, got, want in zip(("cost", "jump", "edge", "messages"), (gc, gj, ge, gm), ref):
        got = got.cpu().numpy()
        err = np.abs(got - want).max()
        assert err <= 2e-4 * max(1.0, np.abs(want).max()), (name, err, np.abs(want).max())


def _softmin(x):
    x = -x.astype(np.float64)
    x -= x.max(-1, keepdims=True)
    e = np.exp(x)
    return e / e.sum(-1, keepdims=True)


def test_message_passing_exact_adjoint_through_iterations():
    from bpl_gb300.layers.stereo import MessagePassing
    dev = torch.device("cuda:0")
    g = cases.rng(13)
    B, H, W, L, iters = 1, 14, 22, 32, 3
    prob = cases.softmax_np(g.normal(0, 2, size=(B, H, W, L)).astype(np.float32))
    edge = cases.edge_weights(g, B, H, W)
    up = g.normal(0, 1, size=(B, H, W, L)).astype(np.float32)
    mp = MessagePassing(dev, iters, L, 3, adjoint="exact")
    with torch.no_grad():
        mp._L1.fill_(0.1)
        mp._L2.fill_(0.5)
    p = torch.from_numpy(prob).to(dev).requires_grad_(True)
    m0 = torch.zeros((B, 4, H, W, L), device=dev, requires_grad=True)
    beliefs, _ = mp(p, torch.from_numpy(edge).to(dev), None, None, m0)
    beliefs.backward(torch.from_numpy(up).to(dev))

    # oracle: the same passes, then the exact adjoint chained backwards
    cost = -prob
    jump = cases.stereo_taps(B, H, W, 0.1, 0.5)
    m = np.zeros((B, 4, H, W, L), np.float32)
    per_it = []
    for _ in range(iters):
        m, am, sc = oracle.lbp_forward(0, cost, jump, edge, m, 3)
        per_it.append((m.copy(), am.copy(), sc.copy()))
    bz = _softmin(m.sum(1) + cost)
    g_sum = -(bz * (up - (up * bz).sum(-1, keepdims=True)))
    G = np.broadcast_to(g_sum[:, None], (B, 4, H, W, L)).astype(np.float64)
    gcost = g_sum.copy()
    gL1 = gL2 = 0.0
    for mk, amk, sck in reversed(per_it):
        gc, gj, _, gm = oracle.lbp_backward_exact(0, jump, edge, G, mk, amk, sck)
        gcost += gc
        gL1 += gj[:, :, 2].sum() + gj[:, :, 4].sum()
        gL2 += gj[:, :, 1].sum() + gj[:, :, 5].sum()
        G = gm
    got = p.grad.detach().cpu().numpy()
    np.testing.assert_allclose(got, -gcost, atol=2e-4 * np.abs(gcost).max())
    assert abs(mp._L1.grad.item() - gL1) <= 2e-4 * max(abs(gL1), 1.0)
    assert abs(mp._L2.grad.item() - gL2) <= 2e-4 * max(abs(gL2), 1.0)
    # the initial messages' gradient is the first pass's input-message gradient
    np.testing.assert_allclose(m0.grad.detach().cpu().numpy(), G, atol=2e-4 * max(1.0, np.abs(G).max()))


@pytest.mark.parametrize("adjoint,storage,size", [("reference", "fp32", "full"), ("exact", "fp32", "small"),
                                                  ("reference", "fp16", "small")])
def test_recompute_argmin_variant_matches_stored(adjoint, storage, size):
    """MessagePassing(recompute_argmin=True) stores no indices: its forward
    keeps the initial vertical message slots only, its backward re-runs the
    passes (regenerating every scanline's indices) and runs their adjoints.
    Gradients equal those of the index-storing variant, and the memory the
    forward leaves for the backward is below the stored indices.  Config:
    B=4, 256x512x96, per-pixel edge weights U[0.5,2], 3 iterations (the
    exact adjoint and FP16 storage on a 32x64 crop)."""
    from bpl_gb300.layers.stereo import MessagePassing
    dev = torch.device("cuda:0")
    g = cases.rng(23)
    B, H, W, L, iters = (4, 256, 512, 96, 3) if size == "full" else (4, 32, 64, 96, 3)
    gen = torch.Generator(device=dev).manual_seed(2)
    prob = torch.softmax(2.0 * torch.randn((B, H, W, L), device=dev, generator=gen), dim=-1)
    edge = (0.5 + 1.5 * torch.rand((B, 4, H, W), device=dev, generator=gen)).contiguous()
    up = torch.randn((B, H, W, L), device=dev, generator=gen)
    grads, held = [], []
    # stored indices as the composition (like for like: it holds the cost
    # volume for the epilogue, as the recomputing variant does), recompute,
    # and stored indices in the fused node (which holds no cost volume)
    for rec, fused in ((False, False), (True, False), (False, True)):
        mp = MessagePassing(dev, iters, L, 3, storage=storage, adjoint=adjoint, recompute_argmin=rec, fused=fused)
        with torch.no_grad():
            mp._L1.fill_(0.1)
            mp._L2.fill_(0.5)
        p = prob.clone().requires_grad_(True)
        e = edge.clone().requires_grad_(True)
        m0 = None if storage == "fp16" else torch.zeros((B, 4, H, W, L), device=dev, requires_grad=True)
        gc.collect()
        torch.cuda.synchronize()
        before = torch.cuda.memory_allocated(dev)
        beliefs, msgs = mp(p, e, None, None, m0)
        # temporaries of the forward that only a reference cycle still holds
        # (the default affinity and offset tensors) go before the count
        gc.collect()
        torch.cuda.synchronize()
        # what the forward leaves for the backward, beyond its outputs
        held.append(torch.cuda.memory_allocated(dev) - before - beliefs.numel() * 4
                    - (msgs.numel() * msgs.element_size() if m0 is None else 0))
        beliefs.backward(up)
        grads.append((beliefs.detach(), p.grad, e.grad, mp._L1.grad.item(), mp._L2.grad.item()))
        del beliefs, msgs, m0
    if adjoint == "reference":
        # both variants hold the cost volume (for the belief epilogue) and the
        # pairwise taps; beyond those, the storing variant holds the indices
        # (and the FP32 scales), the recomputing one the two initial slots
        # (and, FP16, the half copy of the cost that its re-run reads)
        Ls = ops_padded(L) if storage == "fp16" else L
        argmin_bytes = iters * B * 4 * H * W * Ls
        vert_bytes = 2 * B * H * W * Ls * (2 if storage == "fp16" else 4)
        if storage == "fp16":
            vert_bytes += B * H * W * Ls * 2
        print(f"{storage} held by the forward: stored indices {held[0] / 2**20:.1f} MiB, "
              f"recompute {held[1] / 2**20:.1f} MiB (indices {argmin_bytes / 2**20:.1f} MiB, "
              f"kept for the re-run {vert_bytes / 2**20:.1f} MiB)")
        assert vert_bytes < argmin_bytes
        # slack: the layer's default affinity and offset tensors (4 floats per
        # pixel and direction), which one variant's graph may still reference
        slack = B * 4 * 4 * H * W * 4
        assert held[0] - held[1] >= argmin_bytes - vert_bytes - slack
    assert held[2] <= held[0], "the fused node holds more than the composition"
    (b0, gp0, ge0, l10, l20), (b1, gp1, ge1, l11, l21), (b2, gp2, ge2, l12, l22) = grads
    assert torch.equal(b0, b2)
    assert (gp0 - gp2).abs().max().item() <= 1e-5 * max(1.0, gp0.abs().max().item())
    assert (ge0 - ge2).abs().max().item() <= 1e-5 * max(1.0, ge0.abs().max().item())
    assert torch.equal(b0, b1)
    assert (gp0 - gp1).abs().max().item() <= 1e-5 * max(1.0, gp0.abs().max().item())
    assert (ge0 - ge1).abs().max().item() <= 1e-5 * max(1.0, ge0.abs().max().item())
    assert abs(l10 - l11) <= 1e-5 * max(1.0, abs(l10))
    assert abs(l20 - l21) <= 1e-5 * max(1.0, abs(l20))


def ops_padded(L):
    from bpl_gb300 import ops
    return ops.padded_labels(L)
