"""GPU parity of the flow max-projected SAD (bpl_flow_forward /
bpl_flow_backward through the C ABI) against the oracle: cost volumes and
argmins bit-exact, df0 bit-exact, df1 (float atomics, as in the reference)
within float tolerance."""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CASES = [
    # name, seed, B, C, H, W, sws, off_u, off_v, blk_u, blk_v
    ("sws6", 1, 1, 4, 10, 12, 6, 0, 0, 0, 0),
    ("sws8_off", 2, 1, 4, 9, 11, 8, -4, 4, 1, 0),
    ("sws5_odd", 3, 1, 3, 7, 9, 5, 0, 0, 0, 0),
    ("sws16_c32_batch", 4, 2, 32, 14, 40, 16, 0, 0, 0, 0),
    ("sws64_c32", 5, 1, 32, 20, 24, 64, 0, 0, 0, 0),
    ("sws12_c80", 6, 1, 80, 9, 13, 12, 0, 0, 0, 0),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_flow_forward_backward(case):
    from bpl_gb300 import ops
    name, seed, B, C, H, W, sws, ou, ov, bu, bv = case
    g = cases.rng(seed)
    f0 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    f1 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    dev = torch.device("cuda:0")
    t0, t1 = torch.from_numpy(f0).to(dev), torch.from_numpy(f1).to(dev)
    outs = ops.flow_forward(t0, t1, sws, ou, ov, bu, bv)
    ref = oracle.flow_forward(f0, f1, sws, ou, ov, bu, bv)
    for nm, a, b in zip(("cv_u", "cv_v", "u_star", "v_star"), outs, ref):
        np.testing.assert_array_equal(a.cpu().numpy(), b, err_msg=f"{name} {nm}")
    K = sws + 1
    gu = g.normal(0, 1, size=(B, H, W, K)).astype(np.float32)
    gv = g.normal(0, 1, size=(B, H, W, K)).astype(np.float32)
    df0, df1 = ops.flow_backward(t0, t1, sws, torch.from_numpy(gu).to(dev), torch.from_numpy(gv).to(dev),
                                 outs[2], outs[3])
    r0, r1 = oracle.flow_backward(f0, f1, sws, gu, gv, ref[2], ref[3])
    np.testing.assert_array_equal(df0.cpu().numpy(), r0)
    d1 = df1.cpu().numpy()
    assert np.abs(d1 - r1).max() <= 1e-5 * max(np.abs(r1).max(), 1.0)


def test_flow_matches_reference_golden():
    from conftest import load_golden
    import pytorch_cuda_flow_mp_sad_op as flow
    dev = torch.device("cuda:0")
    for name in ("flow_sws6", "flow_sws8_off", "flow_sws5_odd"):
        g = load_golden(name)
        f0, f1 = torch.from_numpy(g["f0"]).to(dev), torch.from_numpy(g["f1"]).to(dev)
        args = [int(g[k]) for k in ("sws", "offset_u", "offset_v", "block_u", "block_v")]
        outs = flow.forward(f0, f1, *args)
        for nm, a in zip(("cv_u", "cv_v", "u_star", "v_star"), outs):
            np.testing.assert_array_equal(a.cpu().numpy(), g[nm], err_msg=f"{name} {nm}")
        df0, df1 = flow.backward(f0, f1, args[0], torch.from_numpy(g["in_grad_u"]).to(dev),
                                 torch.from_numpy(g["in_grad_v"]).to(dev), torch.from_numpy(g["u_star"]).to(dev),
                                 torch.from_numpy(g["v_star"]).to(dev))
        np.testing.assert_array_equal(df0.cpu().numpy(), g["df0"])
        assert np.abs(df1.cpu().numpy() - g["df1"]).max() <= 1e-5 * max(np.abs(g["df1"]).max(), 1.0)


def test_flow_tiled_window_216_equals_single_window():
    """The reference merges four 108-windows for sws=216; the merged result
    equals one 217x217 window (same minima, indices and tie order)."""
    from bpl_gb300 import ops
    from bpl_gb300.layers.matching import FlowMpSadFunction
    g = cases.rng(9)
    B, C, H, W = 1, 4, 6, 230
    dev = torch.device("cuda:0")
    f0 = torch.from_numpy(g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)).to(dev)
    f1 = torch.from_numpy(g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)).to(dev)
    tiled = FlowMpSadFunction.apply(f0, f1, 216)
    single = ops.flow_forward(f0, f1, 216)
    for a, b in zip(tiled, single):
        np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
