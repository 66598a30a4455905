"""The timeout path of the kernels' bounded waits, on the GPU.

The TMA-staged kernels (the pixel-pairwise LBP forward's per-warp ring and
the flow SAD forward's row stages) wait on mbarriers with a poll limit.  When
a wait runs out the kernel raises the library's device error word, waits for
the copies it still has in flight and returns with its outputs incomplete.
These tests make every wait run out at once (a poll limit of 0, set through
bpl_set_wait_limit), check that the error word reports it and that the ops
layer raises, then restore the limit and check that the same launch on the
same context gives the oracle's results: the context stays usable.  No wait
here is left without a bound and nothing faults: the copies are real and
in bounds, only the waiting for them is cut short.
"""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture
def ops():
    from bpl_gb300 import ops as o
    o.read_device_error()  # start from a clear error word
    yield o
    o.set_wait_limit(None)
    o.read_device_error()


def test_pixel_forward_wait_timeout_reports_and_context_survives(ops):
    from bpl_gb300 import _lib
    dev = torch.device("cuda:0")
    g = cases.rng(71)
    B, H, W, L = 1, 6, 9, 8  # L % 4 == 0: rows and matrices come by bulk copies
    cost = cases.random_cost(g, B, H, W, L)
    jump, _ = cases.semantic_pixel_jump(g, H, W, L)
    edge = cases.edge_weights(g, B, H, W)
    msgs = cases.random_messages(g, B, H, W, L)
    c, j, e = (torch.from_numpy(a).to(dev) for a in (cost, jump, edge))

    ops.set_wait_limit(0)
    m = torch.from_numpy(msgs).to(dev)
    ops.lbp_forward(ops.LBP_SEM_PIXEL, c, j, e, m, L)
    assert ops.read_device_error() == 1, "the wait that ran out was not reported"
    assert ops.read_device_error() == 0, "reading the error word clears it"

    # the ops layer turns a reported error into an exception at its check
    ops.lbp_forward(ops.LBP_SEM_PIXEL, c, j, e, torch.from_numpy(msgs).to(dev), L)
    with pytest.raises(_lib.BplError, match="device wait timeout"):
        ops.check_device_error()

    ops.set_wait_limit(None)
    m = torch.from_numpy(msgs).to(dev)
    m, am, sc = ops.lbp_forward(ops.LBP_SEM_PIXEL, c, j, e, m, L)
    torch.cuda.synchronize()
    assert ops.read_device_error() == 0
    rm, ra, rs = oracle.lbp_forward(2, cost, jump, edge, msgs, L)
    np.testing.assert_array_equal(am.cpu().numpy(), ra)
    assert np.abs(m.cpu().numpy() - rm).max() <= 1e-5


def test_flow_forward_wait_timeout_reports_and_context_survives(ops):
    dev = torch.device("cuda:0")
    g = cases.rng(72)
    B, C, H, W, sws = 1, 20, 7, 32, 8  # W and offset_u - sws/2 multiples of 4: bulk row copies
    f0 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    f1 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    t0, t1 = torch.from_numpy(f0).to(dev), torch.from_numpy(f1).to(dev)

    ops.set_wait_limit(0)
    ops.flow_forward(t0, t1, sws)
    assert ops.read_device_error() == 1, "the wait that ran out was not reported"

    ops.set_wait_limit(None)
    outs = ops.flow_forward(t0, t1, sws)
    torch.cuda.synchronize()
    assert ops.read_device_error() == 0
    ref = oracle.flow_forward(f0, f1, sws)
    for nm, a, b in zip(("cv_u", "cv_v", "u_star", "v_star"), outs, ref):
        np.testing.assert_array_equal(a.cpu().numpy(), b, err_msg=nm)
