"""The BP module (ops/lbp_stereo/bp_op_cuda.py:80-127) on the GPU: the
disparity path, the reference's flow path (v starts from u's final
messages, bp_op_cuda.py:110) against the oracle, and the joint flow path
(u and v as one batch) against two independent calls."""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _softmin(x):
    x = -x.astype(np.float64)
    x -= x.max(-1, keepdims=True)
    e = np.exp(x)
    return e / e.sum(-1, keepdims=True)


def _bp(dev, iters, L, **kw):
    from bpl_gb300.layers.stereo import BP
    bp = BP(dev, None, iters, L, 3, mode_inference="wta", **kw)
    with torch.no_grad():
        bp.message_passing._L1.fill_(0.1)
        bp.message_passing._L2.fill_(0.5)
    return bp


def _run_oracle(cost, jump, edge, m, iters):
    for _ in range(iters):
        m, _, _ = oracle.lbp_forward(0, cost, jump, edge, m, 3)
    return m


def test_bp_disparity_path():
    dev = torch.device("cuda:0")
    g = cases.rng(31)
    B, H, W, L, iters = 1, 9, 13, 20, 2
    prob = cases.softmax_np(g.normal(0, 2, size=(B, H, W, L)).astype(np.float32))
    edge = cases.edge_weights(g, B, H, W)
    bp = _bp(dev, iters, L)
    disps, beliefs, messages = bp(torch.from_numpy(prob).to(dev), torch.from_numpy(edge).to(dev))
    m = _run_oracle(-prob, cases.stereo_taps(B, H, W, 0.1, 0.5), edge, np.zeros((B, 4, H, W, L), np.float32), iters)
    np.testing.assert_array_equal(messages.detach().cpu().numpy(), m)
    np.testing.assert_allclose(beliefs.detach().cpu().numpy(), _softmin(m.sum(1) - prob), atol=2e-6)
    assert disps.shape == (B, 1, H, W)
    assert torch.equal(disps[:, 0], beliefs.argmax(-1))


def test_bp_flow_path_follows_the_reference():
    dev = torch.device("cuda:0")
    g = cases.rng(32)
    N, H, W, K, iters = 1, 8, 11, 17, 2
    pu = cases.softmax_np(g.normal(0, 2, size=(N, H, W, K)).astype(np.float32))
    pv = cases.softmax_np(g.normal(0, 2, size=(N, H, W, K)).astype(np.float32))
    edge = cases.edge_weights(g, N, H, W)
    prob = torch.from_numpy(np.stack((pu, pv), 1)).to(dev).requires_grad_(True)
    bp = _bp(dev, iters, K)
    flow, beliefs, messages = bp(prob, torch.from_numpy(edge).to(dev))
    jump = cases.stereo_taps(N, H, W, 0.1, 0.5)
    mu = _run_oracle(-pu, jump, edge, np.zeros((N, 4, H, W, K), np.float32), iters)
    mv = _run_oracle(-pv, jump, edge, mu.copy(), iters)  # v starts from u's final messages
    np.testing.assert_allclose(beliefs[:, 0].detach().cpu().numpy(), _softmin(mu.sum(1) - pu), atol=2e-6)
    np.testing.assert_allclose(beliefs[:, 1].detach().cpu().numpy(), _softmin(mv.sum(1) - pv), atol=2e-6)
    for k in range(2):  # both entries are the one tensor, after the v pass
        np.testing.assert_array_equal(messages[:, k].detach().cpu().numpy(), mv)
    assert flow.shape == (N, 2, H, W)
    (beliefs * torch.randn_like(beliefs)).sum().backward()
    assert prob.grad is not None and torch.isfinite(prob.grad).all()


def test_bp_joint_flow_equals_independent_calls():
    dev = torch.device("cuda:0")
    g = cases.rng(33)
    N, H, W, K, iters = 2, 10, 12, 24, 3
    prob = torch.from_numpy(cases.softmax_np(g.normal(0, 2, size=(N, 2, H, W, K)).astype(np.float32))).to(dev)
    edge = torch.from_numpy(cases.edge_weights(g, N, H, W)).to(dev)
    joint = _bp(dev, iters, K, joint_flow=True)
    flow, beliefs, messages = joint(prob, edge)
    single = _bp(dev, iters, K)
    for k in range(2):
        d, b, m = single(prob[:, k].contiguous(), edge)
        assert torch.equal(beliefs[:, k], b)
        assert torch.equal(messages[:, k], m)
        assert torch.equal(flow[:, k], d[:, 0])
