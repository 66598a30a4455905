"""The pixel-pairwise variant fed the layer's two pairwise planes
(LBP_SEM_PIXEL_LAYER): the kernels' shift and transpose against the
materialised (4,H,W,L,L) tensor of message_passing_op_pw_pixel.py:27-38
(forward bit-equal) and the fold of the jump gradient (:47-51, within the
float-atomic tolerance).  The pairwise matrices are not symmetric, so a
missing or extra transpose shows."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _shift4(jp):
    """The reference layer's packing of the (2,H,W,L,L) planes."""
    j = torch.zeros((4,) + tuple(jp.shape[1:]), dtype=jp.dtype, device=jp.device)
    j[0] = jp[0]
    j[1, :, 1:] = jp[0, :, :-1].permute(0, 1, 3, 2)
    j[2] = jp[1]
    j[3, 1:] = jp[1, :-1].permute(0, 1, 3, 2)
    return j.contiguous()


def _fold2(gj):
    """The reference layer's fold of the (4,H,W,L,L) jump gradient."""
    gj = gj.clone()
    gj[0, :, :-1] += gj[1, :, 1:].permute(0, 1, 3, 2)
    gj[1] = gj[2]
    gj[1, :-1] += gj[3, 1:].permute(0, 1, 3, 2)
    return gj[:2]


@pytest.mark.parametrize("shape", [(1, 7, 9, 19), (2, 5, 6, 5), (1, 4, 40, 33)])
def test_two_planes_equal_the_materialised_shift(shape):
    from bpl_gb300 import ops
    dev = torch.device("cuda:0")
    g = cases.rng(51)
    B, H, W, L = shape
    cost = torch.from_numpy(cases.random_cost(g, B, H, W, L)).to(dev)
    jp = torch.from_numpy(g.uniform(0.0, 1.5, size=(2, H, W, L, L)).astype(np.float32)).to(dev)
    edge = torch.from_numpy(cases.edge_weights(g, B, H, W)).to(dev)
    j4 = _shift4(jp)
    m4 = torch.zeros((B, 4, H, W, L), device=dev)
    m2 = torch.zeros((B, 4, H, W, L), device=dev)
    for _ in range(2):
        m4, a4, s4 = ops.lbp_forward(ops.LBP_SEM_PIXEL, cost, j4, edge, m4, L, argmin_dtype=torch.uint8)
        m2, a2, s2 = ops.lbp_forward(ops.LBP_SEM_PIXEL_LAYER, cost, jp, edge, m2, L, argmin_dtype=torch.uint8)
    assert torch.equal(m4, m2) and torch.equal(a4, a2) and torch.equal(s4, s2)
    gin = torch.randn((B, 4, H, W, L), device=dev)
    _, gj4, _, _ = ops.lbp_backward(ops.LBP_SEM_PIXEL, None, edge, gin, m4, a4, s4, copy_grad_messages=False)
    gc2, gj2, _, _ = ops.lbp_backward(ops.LBP_SEM_PIXEL_LAYER, None, edge, gin, m2, a2, s2, copy_grad_messages=False)
    ref = _fold2(gj4)
    assert gj2.shape == (2, H, W, L, L)
    tol = 1e-5 * max(float(ref.abs().max()), 1.0)
    assert float((gj2 - ref).abs().max()) <= tol


def test_two_planes_fp16_storage():
    from bpl_gb300 import ops
    dev = torch.device("cuda:0")
    g = cases.rng(52)
    B, H, W, L = 1, 6, 11, 19
    cost = torch.from_numpy(cases.random_cost(g, B, H, W, L)).to(dev)
    jp = torch.from_numpy(g.uniform(0.0, 1.5, size=(2, H, W, L, L)).astype(np.float32)).to(dev)
    edge = torch.ones((B, 4, H, W), device=dev)
    ch = ops.to_half_padded(cost, L)
    Lp = ops.padded_labels(L)
    m4 = torch.zeros((B, 4, H, W, Lp), dtype=torch.float16, device=dev)
    m2 = torch.zeros_like(m4)
    j4h = ops.to_half_padded(_shift4(jp), L)
    j2h = ops.to_half_padded(jp, L)
    ops.lbp_forward_f16(ops.LBP_SEM_PIXEL, ch, j4h, edge, m4, L, L)
    ops.lbp_forward_f16(ops.LBP_SEM_PIXEL_LAYER, ch, j2h, edge, m2, L, L)
    assert torch.equal(m4, m2)


def test_semantic_pixel_layer_gradient_matches_materialised():
    """MessagePassingPixel (two planes in the kernels) against the same
    layer computed with the reference's packing and fold."""
    from bpl_gb300 import ops
    from bpl_gb300.layers.semantic import MessagePassingPixel
    dev = torch.device("cuda:0")
    g = cases.rng(53)
    B, H, W, L = 1, 8, 10, 19
    prob = torch.from_numpy(cases.softmax_np(g.normal(0, 2, size=(B, H, W, L)).astype(np.float32))).to(dev)
    edge = torch.from_numpy(cases.edge_weights(g, B, H, W)).to(dev)
    jp = torch.from_numpy(g.uniform(0.0, 1.5, size=(2, H, W, L, L)).astype(np.float32)).to(dev).requires_grad_(True)
    mp = MessagePassingPixel(dev, 2, L, L)
    b = mp(prob, edge, torch.zeros((B, 4, H, W, L), device=dev), jp)
    up = torch.randn_like(b)
    b.backward(up)
    # the same two iterations with the materialised tensor
    cost = -prob
    j4 = _shift4(jp.detach())
    m = torch.zeros((B, 4, H, W, L), device=dev)
    saved = []
    for _ in range(2):
        m, am, sc = ops.lbp_forward(ops.LBP_SEM_PIXEL, cost, j4, edge, m, L, argmin_dtype=torch.uint8)
        saved.append((am.clone(), sc.clone()))
    T = mp.softmin.T.detach()
    bref = ops.beliefs_forward(m, cost, T)
    assert torch.equal(b.detach(), bref)
    gz, _ = ops.beliefs_backward(m, cost, T, bref, up, want_temperature=False)
    gin = gz.unsqueeze(1).expand(B, 4, H, W, L).contiguous()
    gref = torch.zeros((4, H, W, L, L), device=dev)
    for am, sc in saved:
        _, gj4, _, _ = ops.lbp_backward(ops.LBP_SEM_PIXEL, None, edge, gin, m, am, sc, copy_grad_messages=False)
        gref += gj4
    ref = _fold2(gref)
    tol = 1e-5 * max(float(ref.abs().max()), 1.0)
    assert float((jp.grad - ref).abs().max()) <= tol


def test_wide_batch_shallow_ring_matches_oracle():
    """2 x 1024 columns: the vertical phase runs more scanlines than one
    wave holds with a 4-step ring, so it runs a shallower one; results are
    those of the oracle."""
    import oracle
    from bpl_gb300 import ops
    dev = torch.device("cuda:0")
    g = cases.rng(54)
    B, H, W, L = 2, 5, 1024, 19
    cost = cases.random_cost(g, B, H, W, L)
    jp = g.uniform(0.0, 1.5, size=(2, H, W, L, L)).astype(np.float32)
    edge = cases.edge_weights(g, B, H, W)
    j4 = _shift4(torch.from_numpy(jp)).numpy()
    m, am, sc = ops.lbp_forward(ops.LBP_SEM_PIXEL_LAYER, torch.from_numpy(cost).to(dev), torch.from_numpy(jp).to(dev),
                                torch.from_numpy(edge).to(dev), torch.zeros((B, 4, H, W, L), device=dev), L,
                                argmin_dtype=torch.float32)
    rm, ram, rsc = oracle.lbp_forward(2, cost, j4, edge, np.zeros((B, 4, H, W, L), np.float32), L)
    np.testing.assert_array_equal(m.cpu().numpy(), rm)
    np.testing.assert_array_equal(am.cpu().numpy(), ram)
    np.testing.assert_array_equal(sc.cpu().numpy(), rsc)
