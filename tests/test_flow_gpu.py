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
    ("sws10_c17_w70", 7, 1, 17, 6, 70, 10, 3, -2, 0, 1),
    ("sws4_h1_w5", 8, 1, 5, 1, 5, 4, 0, 0, 0, 0),
    ("sws6_off_outside", 10, 1, 4, 8, 9, 6, 40, 0, 0, 0),
    ("sws216", 11, 1, 3, 4, 230, 216, 0, 0, 0, 0),
    ("sws255_max", 12, 1, 2, 3, 260, 255, 0, 0, 0, 0),
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


@pytest.mark.parametrize("sws", [7, 16, 64])
def test_flow_forward_ties_bit_exact(sws):
    """Features on a coarse grid: many window entries tie, so the first-index
    rules of both minima are exercised."""
    from bpl_gb300 import ops
    g = cases.rng(20 + sws)
    B, C, H, W = 1, 5, 9, 45
    f0 = np.round(g.normal(0, 1, size=(B, C, H, W)) * 2).astype(np.float32) / 2
    f1 = np.round(g.normal(0, 1, size=(B, C, H, W)) * 2).astype(np.float32) / 2
    dev = torch.device("cuda:0")
    outs = ops.flow_forward(torch.from_numpy(f0).to(dev), torch.from_numpy(f1).to(dev), sws)
    ref = oracle.flow_forward(f0, f1, sws)
    for nm, a, b in zip(("cv_u", "cv_v", "u_star", "v_star"), outs, ref):
        np.testing.assert_array_equal(a.cpu().numpy(), b, err_msg=f"sws{sws} {nm}")


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


def _merged_216(f0, f1):
    """The reference layer's sws == 216 path (ops/flow_mp_sad/flow_mp_sad.py:
    14-44): four 108-windows with offsets -+54 and block indices, merged by
    concatenation and strict-< selection."""
    from bpl_gb300 import ops
    s = 108
    cv00_u, cv00_v, u00, v00 = ops.flow_forward(f0, f1, s, -s // 2, -s // 2, 0, 0)
    cv01_u, cv01_v, u01, v01 = ops.flow_forward(f0, f1, s, -s // 2, s // 2, 0, 1)
    cv10_u, cv10_v, u10, v10 = ops.flow_forward(f0, f1, s, s // 2, -s // 2, 1, 0)
    cv11_u, cv11_v, u11, v11 = ops.flow_forward(f0, f1, s, s // 2, s // 2, 1, 1)
    u0 = torch.cat((cv00_u, cv10_u[..., 1:]), -1)
    u1 = torch.cat((cv01_u, cv11_u[..., 1:]), -1)
    au0 = torch.cat((u00, u10[..., 1:]), -1)
    au1 = torch.cat((u01, u11[..., 1:]), -1)
    idx = u1 < u0
    u0[idx] = u1[idx]
    au0[idx] = au1[idx]
    v0 = torch.cat((cv00_v, cv01_v[..., 1:]), -1)
    v1 = torch.cat((cv10_v, cv11_v[..., 1:]), -1)
    av0 = torch.cat((v00, v01[..., 1:]), -1)
    av1 = torch.cat((v10, v11[..., 1:]), -1)
    idx = v1 < v0
    v0[idx] = v1[idx]
    av0[idx] = av1[idx]
    return u0, v0, au0, av0


def test_flow_tiled_window_216_equals_single_window():
    """The reference merges four 108-windows for sws=216; the merged result
    equals one 217x217 window (same minima, indices and tie order), which is
    what the layer computes."""
    from bpl_gb300.layers.matching import FlowMpSadFunction
    g = cases.rng(9)
    B, C, H, W = 1, 4, 6, 230
    dev = torch.device("cuda:0")
    f0 = torch.from_numpy(g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)).to(dev)
    f1 = torch.from_numpy(g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)).to(dev)
    # quantised features make exact ties between window entries common
    f0q, f1q = torch.round(f0 * 2) / 2, torch.round(f1 * 2) / 2
    for a0, a1 in ((f0, f1), (f0q, f1q)):
        single = FlowMpSadFunction.apply(a0, a1, 216)
        for a, b in zip(_merged_216(a0, a1), single):
            np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
    with pytest.raises(ValueError):
        FlowMpSadFunction.apply(f0, f1, 150)


def test_flow_window_limit_raises():
    from bpl_gb300 import ops
    dev = torch.device("cuda:0")
    f = torch.zeros((1, 2, 4, 4), device=dev)
    with pytest.raises(ops.BplError):
        ops.flow_forward(f, f, 256)


def test_flow_backward_entry_allocating_its_scratch():
    """bpl_flow_backward (scratch allocated stream-ordered inside the call)
    gives the results of bpl_flow_backward_ws."""
    import ctypes
    from bpl_gb300 import ops, _lib
    g = cases.rng(61)
    B, C, H, W, sws = 1, 8, 9, 14, 6
    dev = torch.device("cuda:0")
    f0 = torch.from_numpy(g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)).to(dev)
    f1 = torch.from_numpy(g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)).to(dev)
    cu, cv, us, vs = ops.flow_forward(f0, f1, sws)
    gu, gv = torch.randn_like(cu), torch.randn_like(cv)
    d0, d1 = ops.flow_backward(f0, f1, sws, gu, gv, us, vs)
    e0, e1 = torch.empty_like(f0), torch.empty_like(f1)
    P = ctypes.c_void_p
    st = _lib.lib().bpl_flow_backward(P(f0.data_ptr()), P(f1.data_ptr()), P(gu.data_ptr()), P(gv.data_ptr()),
                                      P(us.data_ptr()), P(vs.data_ptr()), P(e0.data_ptr()), P(e1.data_ptr()),
                                      B, C, H, W, sws, P(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    assert torch.equal(e0, d0)
    assert float((e1 - d1).abs().max()) <= 1e-5 * max(float(d1.abs().max()), 1.0)
