"""GPU parity of the LBP forward (bpl_lbp_forward through the C ABI) against
the oracle's float emulation of the reference kernels.

Bar: argmin bit-exact; messages and scales bit-exact except where the host's
double exp/log (glibc) and the GPU's differ in the last bit after rounding to
float (the reference evaluates exp/log in double,
ops/lbp_stereo/src/lbp_min_sum_kernel.cu:167, :180-181); such elements are
counted and must stay below 1e-4 of the volume with |diff| <= 4 ulp.
"""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _run_gpu(variant, cost, jump, edge, msgs, delta, iters, argmin_dtype=None):
    from bpl_gb300 import ops
    argmin_dtype = argmin_dtype or torch.float32
    dev = torch.device("cuda:0")
    c = torch.from_numpy(cost).to(dev)
    j = torch.from_numpy(jump).to(dev)
    e = torch.from_numpy(edge).to(dev)
    m = torch.from_numpy(msgs).to(dev).contiguous()
    for _ in range(iters):
        m, am, sc = ops.lbp_forward(variant, c, j, e, m, delta, argmin_dtype=argmin_dtype)
    torch.cuda.synchronize()
    return m.cpu().numpy(), am.cpu().numpy(), sc.cpu().numpy()


def _ulps(a, b):
    ai = a.astype(np.float32).view(np.int32).astype(np.int64)
    bi = b.astype(np.float32).view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, -(ai & 0x7FFFFFFF), ai)
    bi = np.where(bi < 0, -(bi & 0x7FFFFFFF), bi)
    return np.abs(ai - bi)


def assert_parity(gpu, ref, what=""):
    m_g, a_g, s_g = gpu
    m_r, a_r, s_r = ref
    assert a_g.shape == a_r.shape
    bad = np.count_nonzero(a_g != a_r)
    assert bad == 0, f"{what}: {bad} argmin mismatches"
    for name, g, r in (("messages", m_g, m_r), ("scale", s_g, s_r)):
        u = _ulps(g, r)
        frac = np.count_nonzero(u) / max(u.size, 1)
        assert u.max() <= 4, f"{what}: {name} max ulp diff {u.max()}"
        assert frac <= 1e-4, f"{what}: {name} {frac:.2e} of elements differ"


STEREO_CASES = [
    # name, seed, B, H, W, L, taps, delta, iters, quantise, jb, eb
    ("l32", 1, 1, 12, 16, 32, "scalar", 3, 2, None, 1, 1),
    ("l32_ties", 2, 1, 12, 16, 32, "scalar", 3, 2, 8, 1, 1),
    ("l70_off", 3, 1, 9, 13, 70, "taps8_off", 3, 2, None, 1, 1),
    ("l33_ties", 4, 1, 7, 9, 33, "taps8", 2, 2, 4, 1, 1),
    ("l20_full", 5, 1, 8, 10, 20, "scalar", 20, 2, 4, 1, 1),
    ("l5_row", 6, 1, 1, 7, 5, "scalar", 3, 1, None, 1, 1),
    ("l5_col", 7, 1, 9, 1, 5, "scalar", 3, 1, None, 1, 1),
    ("l1", 8, 1, 4, 5, 1, "scalar", 3, 1, None, 1, 1),
    ("l192", 9, 1, 6, 40, 192, "scalar", 3, 2, None, 1, 1),
    ("l96_batch", 10, 3, 11, 37, 96, "taps8_off", 3, 2, None, 3, 1),
    ("l256_wide", 11, 1, 3, 70, 256, "scalar", 3, 1, None, 1, 1),
    ("l300_k12", 12, 1, 4, 9, 300, "scalar", 3, 1, None, 1, 1),
    ("l19_odd", 13, 2, 7, 8, 19, "scalar", 3, 2, None, 1, 2),
    # window forms: delta 0 (own label only), 4 (predicated 9-tap window),
    # 6 (generic scan), 8-tap affinities at delta 3 (beating offsets |jd| <= 2
    # plus tie-only L3 offsets), and the largest label count
    ("l48_d0", 16, 1, 6, 11, 48, "scalar", 0, 2, None, 1, 1),
    ("l40_d4_ties", 17, 1, 7, 12, 40, "scalar", 4, 2, 8, 1, 1),
    ("l40_d6", 18, 1, 7, 12, 40, "scalar", 6, 2, None, 1, 1),
    ("l48_taps8_d3_ties", 19, 1, 9, 14, 48, "taps8", 3, 2, 8, 1, 1),
    ("l1024_max", 20, 1, 3, 5, 1024, "scalar", 3, 1, None, 1, 1),
    # enough scanlines per phase for one warp per scanline (the small cases
    # above split each scanline's labels over several warps)
    ("l64_many_chains", 14, 8, 64, 72, 64, "taps8_off", 3, 1, None, 8, 8),
    ("l192_many_chains", 15, 2, 240, 260, 192, "scalar", 3, 1, None, 1, 2),
]


def _stereo_inputs(seed, B, H, W, L, taps, q, jb, eb):
    g = cases.rng(seed)
    cost = cases.random_cost(g, B, H, W, L, quantise=q)
    if taps == "scalar":
        jump = cases.stereo_taps(jb, H, W, 0.1, 0.5)
    else:
        jump = cases.random_taps8(g, jb, H, W, offset_scale=1.5 if taps == "taps8_off" else 0.0)
        if q:
            jump = (np.round(jump * q) / q).astype(np.float32)
    edge = cases.edge_weights(g, eb, H, W, quantise=q)
    msgs = cases.random_messages(g, B, H, W, L, quantise=q)
    return cost, jump, edge, msgs


@pytest.mark.parametrize("case", STEREO_CASES, ids=[c[0] for c in STEREO_CASES])
def test_stereo_forward_matches_oracle(case):
    name, seed, B, H, W, L, taps, delta, iters, q, jb, eb = case
    cost, jump, edge, msgs = _stereo_inputs(seed, B, H, W, L, taps, q, jb, eb)
    gpu = _run_gpu(0, cost, jump, edge, msgs, delta, iters)
    ref = oracle.lbp_forward(0, cost, jump, edge, msgs, delta, iters=iters)
    assert_parity(gpu, ref, name)


@pytest.mark.parametrize("dtype", ["uint8", "int16"])
def test_compact_argmin_matches_float(dtype):
    cost, jump, edge, msgs = _stereo_inputs(21, 2, 10, 23, 64, "taps8_off", None, 2, 2)
    f = _run_gpu(0, cost, jump, edge, msgs, 3, 1)
    c = _run_gpu(0, cost, jump, edge, msgs, 3, 1, argmin_dtype=getattr(torch, dtype))
    np.testing.assert_array_equal(f[0], c[0])
    np.testing.assert_array_equal(f[1], c[1].astype(np.float32))


SEM_CASES = [("global_l19", 1, 31, 2, 10, 12, 19, 19), ("global_l19_trunc", 1, 32, 1, 8, 11, 19, 3),
             ("global_l40", 1, 33, 1, 6, 9, 40, 40), ("global_l32_regs", 1, 34, 1, 7, 9, 32, 32),
             ("global_l1", 1, 35, 1, 5, 6, 1, 1), ("global_l31_many_chains", 1, 36, 2, 96, 128, 31, 31),
             ("global_l150_k8", 1, 37, 1, 5, 7, 150, 150), ("pixel_l100_global_reads", 2, 44, 1, 5, 6, 100, 100),
             ("pixel_l130_trunc", 2, 45, 1, 4, 5, 130, 4), ("pixel_l300_k32", 2, 46, 1, 3, 4, 300, 300), ("pixel_l7", 2, 41, 1, 8, 10, 7, 7),
             ("pixel_l19", 2, 42, 2, 9, 13, 19, 19), ("pixel_l8_trunc", 2, 43, 1, 6, 7, 8, 2)]


@pytest.mark.parametrize("case", SEM_CASES, ids=[c[0] for c in SEM_CASES])
def test_semantic_forward_matches_oracle(case):
    name, variant, seed, B, H, W, L, delta = case
    g = cases.rng(seed)
    cost = cases.random_cost(g, B, H, W, L)
    if variant == 1:
        jump, _ = cases.semantic_global_jump(g, L)
    else:
        jump, _ = cases.semantic_pixel_jump(g, H, W, L)
    edge = cases.edge_weights(g, B, H, W)
    msgs = cases.random_messages(g, B, H, W, L)
    gpu = _run_gpu(variant, cost, jump, edge, msgs, delta, 2)
    ref = oracle.lbp_forward(variant, cost, jump, edge, msgs, delta, iters=2)
    assert_parity(gpu, ref, name)


# The global variant with one label per lane (L <= 32) minimises over the
# senders as four chains over [8c, 8c+8), combined in sender order;
# quantised costs, messages, matrix and weights put exact ties (and negative
# zeros) on both sides of the chain boundaries.
GLOBAL_TIE_LS = [1, 7, 8, 9, 15, 16, 17, 24, 25, 31, 32]


@pytest.mark.parametrize("L", GLOBAL_TIE_LS)
def test_semantic_global_register_column_ties(L):
    g = cases.rng(500 + L)
    B, H, W = 2, 9, 40
    cost = cases.random_cost(g, B, H, W, L, quantise=4)
    jump, _ = cases.semantic_global_jump(g, L, quantise=2)
    edge = cases.edge_weights(g, B, H, W, quantise=2)
    msgs = cases.random_messages(g, B, H, W, L, quantise=4)
    gpu = _run_gpu(1, cost, jump, edge, msgs, L, 2)
    ref = oracle.lbp_forward(1, cost, jump, edge, msgs, L, iters=2)
    assert_parity(gpu, ref, f"global_ties_l{L}")


def test_small_config_forward():
    """96x128, 32 labels, one pass, as the small stereo workload."""
    g = cases.rng(0)
    cost, *_ = cases.stereo_cost_from_scene(g, 1, 96, 128, 32, 32)
    jump = cases.stereo_taps(1, 96, 128, 0.1, 0.5)
    edge = np.ones((1, 4, 96, 128), np.float32)
    msgs = np.zeros((1, 4, 96, 128, 32), np.float32)
    gpu = _run_gpu(0, cost, jump, edge, msgs, 3, 1)
    ref = oracle.lbp_forward(0, cost, jump, edge, msgs, 3)
    assert_parity(gpu, ref, "c0")


def test_full_size_one_pass():
    """376x1240, 192 labels, one pass against the oracle (multi-threaded)."""
    g = cases.rng(1)
    H, W, L = 376, 1240, 192
    cost = cases.random_cost(g, 1, H, W, L)
    jump = cases.stereo_taps(1, H, W, 0.1, 0.5)
    edge = cases.edge_weights(g, 1, H, W)
    msgs = np.zeros((1, 4, H, W, L), np.float32)
    gpu = _run_gpu(0, cost, jump, edge, msgs, 3, 1, argmin_dtype=torch.uint8)
    ref = oracle.lbp_forward(0, cost, jump, edge, msgs, 3)
    assert_parity((gpu[0], gpu[1].astype(np.float32), gpu[2]), ref, "c1")
