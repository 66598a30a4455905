"""Exact adjoint of the LBP pass against FP64 central finite differences
(eps = 1e-6), on the oracle (CPU): cost volume, edge weights, L1/L2 (through
the tap packing) and the input messages.  The forward is piecewise linear
in these inputs (min selections fixed away from ties), so central
differences match the adjoint to rounding.

Also checks that the exact and the reference adjoint agree where the
reference's simplifications do not apply (a single vertical pass, B = 1).
"""
import numpy as np
import pytest

import cases
import oracle

EPS = 1e-6


def _taps(L1, L2, B, H, W, Lv=6):
    """[off, L2, L1, 0, L1, L2] per pixel and direction (the scalar L1/L2 packing)."""
    t = np.zeros((1, 4, Lv, H, W))
    t[:, :, 1] = L2
    t[:, :, -1] = L2
    t[:, :, 2] = L1
    t[:, :, 4] = L1
    return t


def _loss(cost, L1, L2, edge, m_in, G, delta):
    B, H, W, L = cost.shape
    m, _, _ = oracle.lbp_forward(0, cost, _taps(L1, L2, B, H, W), edge, m_in, delta, fp64=True)
    return float((G * m).sum())


@pytest.mark.parametrize("delta", [3, 8])
def test_exact_adjoint_matches_central_differences(delta):
    g = np.random.default_rng(21)
    B, H, W, L = 1, 16, 24, 8
    cost = g.normal(0, 1, size=(B, H, W, L))
    edge = g.uniform(0.5, 2.0, size=(B, 4, H, W))
    m_in = g.normal(0, 0.3, size=(B, 4, H, W, L))
    L1, L2 = 0.1, 0.5
    G = g.normal(0, 1, size=(B, 4, H, W, L))
    jump = _taps(L1, L2, B, H, W)
    m, am, sc = oracle.lbp_forward(0, cost, jump, edge, m_in, delta, fp64=True)
    gc, gj, ge, gm = oracle.lbp_backward_exact(0, jump, edge, G, m, am, sc, fp64=True)
    gL1 = gj[:, :, 2].sum() + gj[:, :, 4].sum()
    gL2 = gj[:, :, 1].sum() + gj[:, :, 5].sum()

    def fd(fn):
        return (fn(EPS) - fn(-EPS)) / (2 * EPS)

    # scalars
    d1 = fd(lambda e: _loss(cost, L1 + e, L2, edge, m_in, G, delta))
    d2 = fd(lambda e: _loss(cost, L1, L2 + e, edge, m_in, G, delta))
    assert abs(d1 - gL1) <= 1e-5 * max(1.0, abs(d1)), (d1, gL1)
    assert abs(d2 - gL2) <= 1e-5 * max(1.0, abs(d2)), (d2, gL2)
    # sampled coordinates of the cost, the edge weights and the input messages
    for _ in range(12):
        i = tuple(int(g.integers(s)) for s in cost.shape)

        def fc(e, i=i):
            c = cost.copy()
            c[i] += e
            return _loss(c, L1, L2, edge, m_in, G, delta)
        v = fd(fc)
        assert abs(v - gc[i]) <= 1e-5 * max(1.0, abs(v)), ("cost", i, v, gc[i])
    for _ in range(8):
        i = tuple(int(g.integers(s)) for s in edge.shape)

        def fe(e, i=i):
            ed = edge.copy()
            ed[i] += e
            return _loss(cost, L1, L2, ed, m_in, G, delta)
        v = fd(fe)
        assert abs(v - ge[i]) <= 1e-5 * max(1.0, abs(v)), ("edge", i, v, ge[i])
    # input messages: vertical slots (read by the horizontal sweeps), and the
    # boundary entries of every slot (chain inputs and pass-through values)
    picks = [(0, 2, 5, 7), (0, 3, 9, 11), (0, 0, 4, 0), (0, 1, 6, W - 1), (0, 2, 0, 5), (0, 3, H - 1, 3),
             (0, 0, 7, 5), (0, 1, 3, 12)]
    for (n, k, y, x) in picks:
        t = int(g.integers(L))

        def fm(e, i=(n, k, y, x, t)):
            mm = m_in.copy()
            mm[i] += e
            return _loss(cost, L1, L2, edge, mm, G, delta)
        v = fd(fm)
        assert abs(v - gm[n, k, y, x, t]) <= 1e-5 * max(1.0, abs(v)), ("messages", (n, k, y, x, t), v,
                                                                       gm[n, k, y, x, t])


def test_reference_adjoint_equals_exact_except_message_gradient():
    """Every vector J^T = I - p 1^T produces sums to zero, so the scattered
    accumulators the reference carries without J^T (its vertical parts) are
    unchanged by it: the reference adjoint's cost, tap and edge gradients
    are the exact ones.  Its message gradient (in_grad passed through) is
    not, which is what makes multi-iteration gradients differ."""
    g = np.random.default_rng(3)
    B, H, W, L = 1, 10, 14, 12
    cost = cases.random_cost(g, B, H, W, L)
    edge = cases.edge_weights(g, B, H, W)
    jump = cases.stereo_taps(1, H, W, 0.1, 0.5)
    m, am, sc = oracle.lbp_forward(0, cost, jump, edge, np.zeros((B, 4, H, W, L), np.float32), 3)
    G = g.normal(0, 1, size=(B, 4, H, W, L)).astype(np.float32)
    e = oracle.lbp_backward_exact(0, jump, edge, G, m, am, sc)
    r = oracle.lbp_backward_ref(0, jump, edge, G, m, am, sc)
    for a, b in zip(e[:3], r[:3]):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-5 * np.abs(b).max())
    assert np.abs(e[3] - r[3]).max() > 0.1 * np.abs(e[3]).max()


def test_exact_adjoint_through_iterations_matches_central_differences():
    """Two passes with messages carried between them: the exact message
    gradient chains the passes (iteration 2's input-message gradient is
    iteration 1's upstream gradient)."""
    g = np.random.default_rng(8)
    B, H, W, L = 1, 12, 16, 8
    cost = g.normal(0, 1, size=(B, H, W, L))
    edge = g.uniform(0.5, 2.0, size=(B, 4, H, W))
    G = g.normal(0, 1, size=(B, 4, H, W, L))
    L1, L2, delta = 0.1, 0.5, 3

    def loss(c, l1, l2, ed):
        m = np.zeros((B, 4, H, W, L))
        for _ in range(2):
            m, _, _ = oracle.lbp_forward(0, c, _taps(l1, l2, B, H, W), ed, m, delta, fp64=True)
        return float((G * m).sum())

    jump = _taps(L1, L2, B, H, W)
    m0 = np.zeros((B, 4, H, W, L))
    m1, am1, sc1 = oracle.lbp_forward(0, cost, jump, edge, m0, delta, fp64=True)
    m2, am2, sc2 = oracle.lbp_forward(0, cost, jump, edge, m1, delta, fp64=True)
    gc2, gj2, ge2, gm2 = oracle.lbp_backward_exact(0, jump, edge, G, m2, am2, sc2, fp64=True)
    gc1, gj1, ge1, _ = oracle.lbp_backward_exact(0, jump, edge, gm2, m1, am1, sc1, fp64=True)
    gc, gj, ge = gc1 + gc2, gj1 + gj2, ge1 + ge2
    fd = lambda fn: (fn(EPS) - fn(-EPS)) / (2 * EPS)  # noqa: E731
    for _ in range(10):
        i = tuple(int(g.integers(s)) for s in cost.shape)

        def fc(e, i=i):
            c = cost.copy()
            c[i] += e
            return loss(c, L1, L2, edge)
        v = fd(fc)
        assert abs(v - gc[i]) <= 1e-5 * max(1.0, abs(v)), (i, v, gc[i])
    v = fd(lambda e: loss(cost, L1, L2 + e, edge))
    gL2 = gj[:, :, 1].sum() + gj[:, :, 5].sum()
    assert abs(v - gL2) <= 1e-5 * max(1.0, abs(v))
    i = (0, 2, 5, 7)

    def fe(e):
        ed = edge.copy()
        ed[i] += e
        return loss(cost, L1, L2, ed)
    v = fd(fe)
    assert abs(v - ge[i]) <= 1e-5 * max(1.0, abs(v))
