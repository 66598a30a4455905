"""GPU parity of the reference adjoint (bpl_lbp_backward through the C ABI)
against the oracle's double-precision restatement of the reference backward
(ops/lbp_stereo/src/lbp_min_sum_kernel.cu:215-417, :513-621).

The reference itself accumulates with float atomics in arbitrary order, so the
bar is a tolerance, per element: |gpu - oracle| <= ATOL * max|oracle| +
RTOL * |oracle| for every element of each tensor (float32 accumulation over
chains of up to W steps: an entry whose terms cancel keeps an absolute error
on the scale of the tensor), and max |gpu - oracle| <= 2e-4 * max |oracle|;
grad_messages exact.  (At the full size this library's adjoint is measured
against the reference op itself in test_reference_ops_gpu.py: its largest
error against the double-precision adjoint is about 2e-6 of the tensor's
scale, the reference op's about 3e-5.)
"""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 2e-4
ATOL = 1e-5
RTOL = 1e-4


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-12))


def assert_elementwise(a, b, what):
    lim = ATOL * max(np.abs(b).max(), 1e-30) + RTOL * np.abs(b)
    bad = np.abs(a - b) > lim
    assert not bad.any(), f"{what}: {int(bad.sum())} of {b.size} elements outside atol+rtol*|ref|"


def run_case(variant, cost, jump, edge, msgs, delta, gin, argmin_dtype=torch.float32):
    from bpl_gb300 import ops
    dev = torch.device("cuda:0")
    c, j, e = (torch.from_numpy(x).to(dev) for x in (cost, jump, edge))
    m = torch.from_numpy(msgs).to(dev)
    m, am, sc = ops.lbp_forward(variant, c, j, e, m, delta, argmin_dtype=argmin_dtype)
    g = torch.from_numpy(gin).to(dev)
    gc, gj, ge, gm = ops.lbp_backward(variant, j, e, g, m, am, sc)
    torch.cuda.synchronize()
    fwd = (m.cpu().numpy(), am.cpu().numpy().astype(np.float32), sc.cpu().numpy())
    bwd = [None if t is None else t.cpu().numpy() for t in (gc, gj, ge, gm)]
    return fwd, bwd


def check(variant, fwd, bwd, jump, edge, gin, name):
    m, am, sc = fwd
    rc, rj, re_, rm = oracle.lbp_backward_ref(variant, jump, edge, gin, m, am, sc)
    # broadcast jump/edge batches receive the sum over batch items
    if variant == 0 and jump.shape[0] == 1 and rj.shape[0] > 1:
        rj = rj.sum(0, keepdims=True)
    if edge.shape[0] == 1 and re_.shape[0] > 1:
        re_ = re_.sum(0, keepdims=True)
    assert rel_err(bwd[0], rc) <= TOL, f"{name} grad_cost {rel_err(bwd[0], rc):.2e}"
    assert rel_err(bwd[1], rj) <= TOL, f"{name} grad_jump {rel_err(bwd[1], rj):.2e}"
    assert_elementwise(bwd[0], rc, f"{name} grad_cost")
    assert_elementwise(bwd[1], rj, f"{name} grad_jump")
    if variant != 2:
        assert rel_err(bwd[2], re_) <= TOL, f"{name} grad_edge {rel_err(bwd[2], re_):.2e}"
        assert_elementwise(bwd[2], re_, f"{name} grad_edge")
    np.testing.assert_array_equal(bwd[3], gin)


CASES = [
    # name, seed, B, H, W, L, taps, delta, jb, eb
    ("l32", 1, 1, 10, 14, 32, "scalar", 3, 1, 1),
    ("l70_off", 2, 1, 9, 13, 70, "taps8_off", 3, 1, 1),
    ("l33", 3, 1, 11, 7, 33, "taps8", 2, 1, 1),
    ("l19_full", 4, 1, 8, 10, 19, "scalar", 19, 1, 1),
    ("l96_batch", 5, 2, 12, 20, 96, "taps8_off", 3, 2, 2),
    ("l192", 6, 1, 6, 40, 192, "scalar", 3, 1, 1),
    ("l64_bcast", 7, 3, 7, 9, 64, "scalar", 3, 1, 1),
    ("row", 8, 1, 1, 9, 8, "scalar", 3, 1, 1),
    ("col", 9, 1, 9, 1, 8, "scalar", 3, 1, 1),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_stereo_backward_matches_oracle(case):
    name, seed, B, H, W, L, taps, delta, jb, eb = case
    g = cases.rng(seed)
    cost = cases.random_cost(g, B, H, W, L)
    jump = cases.stereo_taps(jb, H, W, 0.1, 0.5) if taps == "scalar" else \
        cases.random_taps8(g, jb, H, W, offset_scale=1.5 if taps == "taps8_off" else 0.0)
    edge = cases.edge_weights(g, eb, H, W)
    msgs = cases.random_messages(g, B, H, W, L)
    gin = g.normal(0, 1, size=(B, 4, H, W, L)).astype(np.float32)
    fwd, bwd = run_case(0, cost, jump, edge, msgs, delta, gin)
    check(0, fwd, bwd, jump, edge, gin, name)


@pytest.mark.parametrize("dtype", ["uint8", "int16"])
def test_backward_compact_argmin(dtype):
    g = cases.rng(11)
    B, H, W, L = 1, 9, 17, 48
    cost = cases.random_cost(g, B, H, W, L)
    jump = cases.stereo_taps(1, H, W, 0.1, 0.5)
    edge = cases.edge_weights(g, 1, H, W)
    msgs = cases.random_messages(g, B, H, W, L)
    gin = g.normal(0, 1, size=(B, 4, H, W, L)).astype(np.float32)
    fwd, bwd = run_case(0, cost, jump, edge, msgs, 3, gin, argmin_dtype=getattr(torch, dtype))
    check(0, fwd, bwd, jump, edge, gin, dtype)


SEM = [("global_l19", 1, 31, 1, 10, 12, 19, 19), ("global_l19_b2", 1, 32, 2, 8, 11, 19, 3),
       ("global_l40", 1, 33, 1, 6, 9, 40, 40), ("pixel_l7", 2, 41, 1, 8, 10, 7, 7),
       ("pixel_l19_b2", 2, 42, 2, 9, 13, 19, 19), ("pixel_l8", 2, 43, 1, 6, 7, 8, 8),
       ("global_l150_k8", 1, 34, 1, 5, 7, 150, 150), ("pixel_l100_global_reads", 2, 44, 1, 5, 6, 100, 100),
       ("pixel_l130_trunc", 2, 45, 1, 4, 5, 130, 4)]


@pytest.mark.parametrize("case", SEM, ids=[c[0] for c in SEM])
def test_semantic_backward_matches_oracle(case):
    name, variant, seed, B, H, W, L, delta = case
    g = cases.rng(seed)
    cost = cases.random_cost(g, B, H, W, L)
    jump = cases.semantic_global_jump(g, L)[0] if variant == 1 else cases.semantic_pixel_jump(g, H, W, L)[0]
    edge = cases.edge_weights(g, B, H, W)
    msgs = cases.random_messages(g, B, H, W, L)
    gin = g.normal(0, 1, size=(B, 4, H, W, L)).astype(np.float32)
    fwd, bwd = run_case(variant, cost, jump, edge, msgs, delta, gin)
    check(variant, fwd, bwd, jump, edge, gin, name)


def test_backward_full_size():
    """376x1240x192 reference adjoint against the oracle."""
    g = cases.rng(12)
    B, H, W, L = 1, 376, 1240, 192
    cost = cases.random_cost(g, B, H, W, L)
    jump = cases.stereo_taps(1, H, W, 0.1, 0.5)
    edge = cases.edge_weights(g, 1, H, W)
    msgs = np.zeros((B, 4, H, W, L), np.float32)
    gin = g.normal(0, 1, size=(B, 4, H, W, L)).astype(np.float32)
    fwd, bwd = run_case(0, cost, jump, edge, msgs, 3, gin, argmin_dtype=torch.uint8)
    check(0, fwd, bwd, jump, edge, gin, "c1")


@pytest.mark.parametrize("half", [False, True], ids=["fp32", "fp16"])
def test_backward_passes_equals_sum_of_single_passes(half):
    """bpl_lbp_backward_passes (the passes' reference adjoints in one launch)
    equals the sum of one bpl_lbp_backward per pass."""
    from bpl_gb300 import ops
    dev = torch.device("cuda:0")
    g = cases.rng(17)
    B, H, W, L, P = 2, 13, 21, 40, 3
    cost = torch.from_numpy(cases.random_cost(g, B, H, W, L)).to(dev)
    edge = torch.from_numpy(cases.edge_weights(g, B, H, W)).to(dev)
    jump = torch.from_numpy(cases.stereo_taps(1, H, W, 0.1, 0.5)).to(dev)
    Ls = ops.padded_labels(L) if half else L
    gin = torch.randn((B, 4, H, W, L), device=dev, generator=torch.Generator(device=dev).manual_seed(3))
    if half:
        ch = ops.to_half_padded(cost, L)
        m = torch.zeros((B, 4, H, W, Ls), dtype=torch.float16, device=dev)
        gin = ops.to_half_padded(gin, L)
    else:
        m = torch.zeros((B, 4, H, W, L), device=dev)
    ams = torch.empty((P, B, 4, H, W, Ls), dtype=torch.uint8, device=dev)
    scs = torch.empty((P, B, 4, H, W), device=dev)
    for k in range(P):
        if half:
            ops.lbp_forward_f16(0, ch, jump, edge, m, 3, L, argmin=ams[k], scale=scs[k])
        else:
            ops.lbp_forward(0, cost, jump, edge, m, 3, argmin_dtype=torch.uint8, argmin=ams[k], scale=scs[k])
    gc, gj, ge = ops.lbp_backward_passes(0, jump, edge, gin, m, ams, scs, L=L)
    sc_, sj, se = 0, 0, 0
    for k in range(P):
        if half:
            a, b, c = ops.lbp_backward_f16(0, jump, edge, gin, m, ams[k], scs[k], L)
        else:
            a, b, c, _ = ops.lbp_backward(0, jump, edge, gin, m, ams[k], scs[k])
        sc_, sj, se = sc_ + a, sj + b, se + c
    for got, want in ((gc, sc_), (gj, sj), (ge, se)):
        assert (got - want).abs().max().item() <= 1e-4 * max(1.0, want.abs().max().item())
