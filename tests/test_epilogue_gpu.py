"""The epilogue kernels (bpl_cost_from_sad, bpl_messages_argmin,
bpl_beliefs_infer, through the C ABI) against the torch statements they
replace: the matching step's cost = -softmax(-SAD/T) (matching.py:22-25,
message_passing_op_cuda.py:162), the beliefs' argmax of the message sum
(message_passing_op_cuda.py:170-173, inference_op.py:23-27) and the
inference modes wta / sub-exp (inference_op.py:22-97)."""
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev():
    return torch.device("cuda:0")


def gen(seed):
    return torch.Generator(device=dev()).manual_seed(seed)


@pytest.mark.parametrize("D,T", [(192, 1.0), (61, 0.5), (7, 2.0), (1, 1.0)])
def test_cost_from_sad_matches_torch(D, T):
    from bpl_gb300 import ops
    sad = 30.0 * torch.rand((2, 9, 23, D), device=dev(), generator=gen(D))
    want = -torch.softmax(-sad / T, dim=-1)
    got = ops.cost_from_sad(sad, T)
    assert (got - want).abs().max().item() <= 1e-6
    got_h = ops.cost_from_sad(sad, T, half=True)
    Lp = ops.padded_labels(D)
    assert got_h.shape[-1] == Lp and got_h.dtype == torch.float16
    assert bool((got_h[..., D:] == 0).all())
    # within one half rounding step of the float result
    ref_h = want.half().float()
    step = torch.where(ref_h == 0, torch.full_like(ref_h, 2 ** -24), ref_h.abs() * 2 ** -10)
    assert bool(((got_h[..., :D].float() - ref_h).abs() <= step).all())


@pytest.mark.parametrize("half_m,half_c", [(False, False), (True, True), (True, False), (False, True)])
def test_messages_argmin_matches_torch(half_m, half_c):
    from bpl_gb300 import ops
    B, H, W, L = 2, 17, 29, 70
    Ls = ops.padded_labels(L) if half_m else L
    Lc = ops.padded_labels(L) if half_c else L
    g = gen(3)
    # coarse values: many exact ties, so the first-index rule is exercised
    m = (torch.randint(0, 6, (B, 4, H, W, Ls), device=dev(), generator=g).float() * 0.25)
    c = (torch.randint(0, 6, (B, H, W, Lc), device=dev(), generator=g).float() * 0.25)
    m = m.half() if half_m else m
    c = c.half() if half_c else c
    mf, cf = m[..., :L].float(), c[..., :L].float()
    z = (((mf[:, 0] + mf[:, 1]) + mf[:, 2]) + mf[:, 3]) + cf
    want = torch.argmin(z, dim=-1)
    got = ops.messages_argmin(m.contiguous(), c.contiguous(), L)
    assert torch.equal(got, want)
    got32 = ops.messages_argmin(m.contiguous(), c.contiguous(), L, out_dtype=torch.int32)
    assert torch.equal(got32.long(), want)


@pytest.mark.parametrize("L", [192, 33, 5])
def test_beliefs_infer_matches_the_reference_modes(L):
    from bpl_gb300 import ops
    from bpl_gb300.layers.stereo import Inference
    g = gen(L)
    raw = torch.randn((2, 11, 19, L), device=dev(), generator=g)
    raw[0, 0, 0] = 1.0  # a row of exact ties
    beliefs = torch.softmax(raw, dim=-1)
    got = ops.beliefs_infer(beliefs, "wta")
    assert torch.equal(got, torch.argmax(beliefs, dim=3, keepdim=True))
    # sub-exp: the reference's torch statement (inference_op.py:53-97)
    support = 3
    disp = beliefs.argmax(dim=-1).unsqueeze(-1)
    win = (torch.arange(-support, support + 1, device=dev()) + disp).clamp(0, L - 1)
    bw = torch.gather(beliefs, 3, win)
    want = torch.sum((bw / bw.sum(dim=-1, keepdim=True)) * win, dim=-1, keepdim=True)
    got = ops.beliefs_infer(beliefs, "sub-exp", support)
    assert (got - want).abs().max().item() <= 1e-5 * max(1.0, L)
    # the layer routes both modes through the kernel without a gradient
    assert torch.equal(Inference(dev(), "wta")(beliefs), torch.argmax(beliefs, dim=3, keepdim=True))
    assert (Inference(dev(), "sub-exp")(beliefs) - want).abs().max().item() <= 1e-5 * max(1.0, L)


def _pack_torch(aff, off):
    # the reference's packing statement (message_passing_op_cuda.py:35-60)
    N, D, K, H, W = aff.shape
    out = torch.zeros((N, D, K + 3, H, W), device=aff.device)
    out[:, :, 0] = off
    out[:, :, 1] = aff[:, :, -1]
    out[:, :, -1] = aff[:, :, -1]
    ic = 0
    for i in range(2, (K + 3) // 2):
        out[:, 0::2, i] = aff[:, 0::2, ic]
        out[:, 0::2, -i] = aff[:, 0::2, ic + 1]
        out[:, 1::2, i] = aff[:, 1::2, ic + 1]
        out[:, 1::2, -i] = aff[:, 1::2, ic]
        ic += 2
    return out


def _unpack_torch(gt):
    # the reference's fold (message_passing_op_cuda.py:75-93)
    N, D, Kp, H, W = gt.shape
    g = torch.zeros((N, D, Kp - 3, H, W), device=gt.device)
    g[:, :, -1] += gt[:, :, 1]
    g[:, :, -1] += gt[:, :, -1]
    ic = 0
    for i in range(2, Kp // 2):
        g[:, 0::2, ic] = gt[:, 0::2, i]
        g[:, 0::2, ic + 1] = gt[:, 0::2, -i]
        g[:, 1::2, ic + 1] = gt[:, 1::2, i]
        g[:, 1::2, ic] = gt[:, 1::2, -i]
        ic += 2
    return g, gt[:, :, 0]


@pytest.mark.parametrize("K", [3, 5])
def test_tap_packing_kernels_match_the_reference_statements(K):
    """bpl_pack_taps / bpl_unpack_tap_grad against the reference's packing and
    fold statements: bit-identical (copies, and the L3 fold's two adds in the
    same order)."""
    from bpl_gb300 import ops
    g = gen(K)
    N, H, W = 2, 13, 21
    aff = torch.rand((N, 4, K, H, W), device=dev(), generator=g)
    off = torch.randn((N, 4, H, W), device=dev(), generator=g)
    assert torch.equal(ops.pack_taps(aff, off), _pack_torch(aff, off))
    gt = torch.randn((N, 4, K + 3, H, W), device=dev(), generator=g)
    ga, go = ops.unpack_tap_grad(gt)
    ra, ro = _unpack_torch(gt)
    assert torch.equal(ga, ra) and torch.equal(go, ro)
