"""FP16 storage (bpl_lbp_forward_f16): cost and messages stored as half,
FP32 arithmetic.  Not bit-exact by design; measured against the FP64 oracle:
per-pixel label disagreement (argmin of the beliefs) <= 1 %, message error
stated."""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _labels(msgs, cost):
    # per-pixel argmin of ((((M0+M1)+M2)+M3)+cost), first index
    b = (((msgs[:, 0] + msgs[:, 1]) + msgs[:, 2]) + msgs[:, 3]) + cost
    return b.argmin(-1)


@pytest.mark.parametrize("case", [("stereo_l96", 0, 1, 40, 64, 96, 3), ("stereo_l64_b2", 0, 2, 24, 40, 64, 2),
                                  ("pixel_l19", 2, 1, 32, 48, 19, 2), ("global_l19", 1, 2, 32, 48, 19, 2)],
                         ids=lambda c: c[0])
def test_fp16_forward_against_fp64_oracle(case):
    from bpl_gb300 import ops
    name, variant, B, H, W, L, iters = case
    dev = torch.device("cuda:0")
    g = cases.rng(7)
    if variant == 0:
        cost, *_ = cases.stereo_cost_from_scene(g, B, H, W, 16, L)
        jump = cases.stereo_taps(1, H, W, 0.1, 0.5)
        jt = torch.from_numpy(jump).to(dev)
    elif variant == 1:
        cost = cases.random_cost(g, B, H, W, L)
        jump, _ = cases.semantic_global_jump(g, L)
        jt = torch.from_numpy(jump).to(dev)
    else:
        cost = cases.random_cost(g, B, H, W, L)
        jump, _ = cases.semantic_pixel_jump(g, H, W, L)
        jt = ops.to_half_padded(torch.from_numpy(jump).to(dev), L)
    edge = cases.edge_weights(g, B, H, W)
    delta = 3 if variant == 0 else L
    ch = ops.to_half_padded(torch.from_numpy(cost).to(dev), L)
    mh = torch.zeros((B, 4, H, W, ops.padded_labels(L)), dtype=torch.float16, device=dev)
    for _ in range(iters):
        mh, am, sc = ops.lbp_forward_f16(variant, ch, jt, torch.from_numpy(edge).to(dev), mh, delta, L,
                                         want_scale=True)
    torch.cuda.synchronize()
    m16 = ops.normalised_f16_messages(mh, L).cpu().numpy()
    # the scale the kernel computed on request is the rows' sum of exp
    written = sc > 0
    lse = torch.logsumexp(mh[..., :L].float(), dim=-1)
    assert torch.allclose(torch.log(sc[written]), lse[written], rtol=0, atol=1e-3)
    # FP64 oracle on the same (half-rounded) inputs
    cost_r = ch[..., :L].float().cpu().numpy().astype(np.float64)
    jump_r = jump if variant in (0, 1) else jt[..., :L].float().cpu().numpy()
    m64, _, _ = oracle.lbp_forward(variant, cost_r, jump_r, edge, np.zeros((B, 4, H, W, L)), delta, fp64=True,
                                   iters=iters)
    lab16 = _labels(m16.astype(np.float64), cost_r)
    lab64 = _labels(m64, cost_r)
    disagree = float((lab16 != lab64).mean())
    err = float(np.abs(m16 - m64).max())
    print(f"{name}: label disagreement {disagree:.4%}, max message error {err:.3e}")
    assert disagree <= 0.01
    assert err <= 0.05


def test_fp16_layer_forward_backward_close_to_fp32():
    """MessagePassing(storage="fp16") against the FP32 layer on the same
    (half-rounded) cost: same labels on >= 99 % of pixels, and a cost
    gradient no farther from the FP32 one than twice the distance the FP32
    gradient itself moves when its input is rounded to half (the gradient
    follows argmin routes, so it is only as stable as the forward's ties)."""
    from bpl_gb300.layers.stereo import MessagePassing
    dev = torch.device("cuda:0")
    g = cases.rng(11)
    B, H, W, L = 1, 32, 56, 64
    cost, *_ = cases.stereo_cost_from_scene(g, B, H, W, 16, L)
    prob = torch.from_numpy(-cost).to(dev)
    edge = torch.from_numpy(cases.edge_weights(g, B, H, W)).to(dev)
    up = torch.randn((B, H, W, L), device=dev, generator=torch.Generator(device=dev).manual_seed(1))

    def run(storage, prob_in):
        mp = MessagePassing(dev, 3, L, 3, storage=storage)
        with torch.no_grad():
            mp._L1.fill_(0.1)
            mp._L2.fill_(0.5)
        p = prob_in.clone().requires_grad_(True)
        beliefs, _ = mp(p, edge, None, None, None if storage == "fp16" else
                        torch.zeros((B, 4, H, W, L), device=dev, requires_grad=True))
        beliefs.backward(up)
        return beliefs.detach().argmax(-1), p.grad.detach()

    def rel(a, b):
        return ((a - b).norm() / a.norm()).item()

    prob_h = prob.half().float()
    lab32, g32 = run("fp32", prob)
    lab32h, g32h = run("fp32", prob_h)
    lab16, g16 = run("fp16", prob_h)
    agree = (lab32h == lab16).float().mean().item()
    sens = rel(g32, g32h)
    r16 = rel(g32h, g16)
    print(f"fp16 layer: label agreement {agree:.4f}, cost-gradient relative L2 {r16:.3e} "
          f"(FP32 gradient under half rounding of its input: {sens:.3e})")
    assert agree >= 0.99
    assert r16 <= 2.0 * sens


def test_fp16_adjoint_normalises_with_the_final_rows():
    """The FP16 reference adjoint of several in-place passes against the
    oracle's adjoint in double precision, given the same final messages
    (log-normalised from the half rows), the same per-pass argmins and the
    same half-rounded upstream gradient.  The reference's Jacobian uses
    exp(m) of the final normalised message for every pass (its m_raw = m +
    log S_k and the division by S_k cancel), i.e. the softmax of the final
    row: a per-pass scale would leave every pass but the last unnormalised."""
    from bpl_gb300 import ops
    dev = torch.device("cuda:0")
    g = cases.rng(19)
    B, H, W, L, P = 1, 14, 22, 40, 3
    cost, *_ = cases.stereo_cost_from_scene(g, B, H, W, 16, L)
    jump = cases.stereo_taps(1, H, W, 0.1, 0.5)
    edge = cases.edge_weights(g, B, H, W)
    jt, et = torch.from_numpy(jump).to(dev), torch.from_numpy(edge).to(dev)
    ch = ops.to_half_padded(torch.from_numpy(cost).to(dev), L)
    Lp = ops.padded_labels(L)
    m = torch.zeros((B, 4, H, W, Lp), dtype=torch.float16, device=dev)
    ams = torch.zeros((P, B, 4, H, W, Lp), dtype=torch.uint8, device=dev)
    for k in range(P):
        ops.lbp_forward_f16(0, ch, jt, et, m, 3, L, argmin=ams[k])
    gin = ops.to_half_padded(torch.randn((B, 4, H, W, L), device=dev,
                                         generator=torch.Generator(device=dev).manual_seed(5)), L)
    gc, gj, ge = ops.lbp_backward_passes(0, jt, et, gin, m, ams, None, L=L)
    torch.cuda.synchronize()
    m_lse = ops.normalised_f16_messages(m, L).cpu().numpy()
    gin_f = gin[..., :L].float().cpu().numpy()
    ones = np.ones((B, 4, H, W), np.float32)
    rc, rj, re_ = 0.0, 0.0, 0.0
    for k in range(P):
        a = ams[k][..., :L].float().cpu().numpy()
        c_, j_, e_, _ = oracle.lbp_backward_ref(0, jump, edge, gin_f, m_lse, a, ones)
        rc, rj, re_ = rc + c_, rj + j_, re_ + e_
    for name, got, want in (("grad_cost", gc[..., :L], rc), ("grad_jump", gj, rj), ("grad_edge", ge, re_)):
        got = got.double().cpu().numpy()
        err = np.abs(got - want).max() / max(np.abs(want).max(), 1e-12)
        print(f"fp16 adjoint {name}: max error {err:.2e} of scale")
        assert err <= 1e-3, f"{name}: {err:.2e} of scale"


@pytest.mark.parametrize("case", [
    # name, B, H, W, L, taps, delta, iters
    ("l20_full_branch", 1, 9, 12, 20, "scalar", 20, 2),
    ("l70_taps8_offsets", 1, 10, 15, 70, "taps8_off", 3, 2),
    ("l48_taps8_d3", 2, 11, 17, 48, "taps8", 3, 2),
    ("l40_d6_generic", 1, 8, 14, 40, "scalar", 6, 2),
    ("l33_d0", 1, 7, 9, 33, "scalar", 0, 1),
    ("l5_one_row", 1, 1, 30, 5, "scalar", 3, 1),
    ("l5_one_column", 1, 30, 1, 5, "scalar", 3, 1),
    ("l1", 1, 4, 5, 1, "scalar", 3, 1),
    ("l256_max_lean", 1, 5, 16, 256, "scalar", 3, 1),
], ids=lambda c: c[0])
def test_fp16_lean_forward_window_forms(case):
    """The lean FP16 stereo kernel's window forms (full minimisation, zero-offset
    fast windows, the generic window with offsets, single rows and columns,
    one and 256 labels) against the FP64 oracle on the same half-rounded
    inputs: label disagreement <= 1 %, normalised messages within 0.05."""
    from bpl_gb300 import ops
    name, B, H, W, L, taps, delta, iters = case
    dev = torch.device("cuda:0")
    g = cases.rng(23)
    cost = cases.random_cost(g, B, H, W, L)
    if taps == "scalar":
        jump = cases.stereo_taps(1, H, W, 0.1, 0.5)
    else:
        jump = cases.random_taps8(g, 1, H, W, offset_scale=1.5 if taps == "taps8_off" else 0.0)
    edge = cases.edge_weights(g, B, H, W)
    ch = ops.to_half_padded(torch.from_numpy(cost).to(dev), L)
    mh = torch.zeros((B, 4, H, W, ops.padded_labels(L)), dtype=torch.float16, device=dev)
    for _ in range(iters):
        ops.lbp_forward_f16(0, ch, torch.from_numpy(jump).to(dev), torch.from_numpy(edge).to(dev), mh, delta, L)
    torch.cuda.synchronize()
    m16 = ops.normalised_f16_messages(mh, L).cpu().numpy().astype(np.float64)
    cost_r = ch[..., :L].float().cpu().numpy().astype(np.float64)
    m64, _, _ = oracle.lbp_forward(0, cost_r, jump, edge, np.zeros((B, 4, H, W, L)), delta, fp64=True, iters=iters)
    disagree = float((_labels(m16, cost_r) != _labels(m64, cost_r)).mean())
    err = float(np.abs(m16 - m64).max())
    print(f"{name}: label disagreement {disagree:.4%}, max message error {err:.3e}")
    assert disagree <= 0.01
    assert err <= 0.05
