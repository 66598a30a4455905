"""GPU parity of the stereo SAD volume and its gradient (bpl_sad_forward /
bpl_sad_backward through the C ABI) against the oracle: bit-exact."""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CASES = [
    # name, seed, B, C, H, W, min, max, step, quantise
    ("c8_d12", 1, 1, 8, 10, 24, 0, 11, 1.0, None),
    ("c8_neg", 2, 1, 8, 9, 20, -3, 5, 1.0, None),
    ("c8_d4_q", 3, 1, 8, 6, 16, 0, 3, 1.0, 2),
    ("c32_d32_batch", 4, 2, 32, 20, 70, 0, 31, 1.0, None),
    ("c64_d192_wide", 5, 1, 64, 3, 300, 0, 191, 1.0, None),
    ("c5_d7_odd", 6, 1, 5, 7, 33, 2, 8, 1.0, 4),
    ("step_half", 7, 1, 6, 5, 40, 0, 9, 0.5, None),
    ("c16_d256", 8, 1, 16, 2, 520, 0, 255, 1.0, None),
    ("c40_d20_min1", 9, 1, 40, 4, 50, 1, 20, 1.0, 2),
    ("c33_dneg_wide", 10, 1, 33, 3, 37, -40, 45, 1.0, None),
]


def _inputs(seed, B, C, H, W, q):
    g = cases.rng(seed)
    f0 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    f1 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    if q:
        f0 = (np.round(f0 * q) / q).astype(np.float32)
        f1 = (np.round(f1 * q) / q).astype(np.float32)
    return f0, f1


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_sad_forward_bit_exact(case):
    from bpl_gb300 import ops
    name, seed, B, C, H, W, lo, hi, step, q = case
    f0, f1 = _inputs(seed, B, C, H, W, q)
    dev = torch.device("cuda:0")
    vol = ops.sad_forward(torch.from_numpy(f0).to(dev), torch.from_numpy(f1).to(dev), lo, hi, step)
    ref = oracle.sad_forward(f0, f1, lo, hi, step)
    np.testing.assert_array_equal(vol.cpu().numpy(), ref)


@pytest.mark.parametrize("case", [c for c in CASES if c[8] == 1.0], ids=[c[0] for c in CASES if c[8] == 1.0])
@pytest.mark.parametrize("limit", [False, True])
def test_sad_backward_bit_exact(case, limit):
    from bpl_gb300 import ops
    name, seed, B, C, H, W, lo, hi, step, q = case
    f0, f1 = _inputs(seed, B, C, H, W, q)
    D = hi - lo + 1
    gin = cases.rng(seed + 100).normal(0, 1, size=(B, H, W, D)).astype(np.float32)
    dev = torch.device("cuda:0")
    df0, df1 = ops.sad_backward(torch.from_numpy(f0).to(dev), torch.from_numpy(f1).to(dev), lo, hi,
                                torch.from_numpy(gin).to(dev), reference_channel_limit=limit)
    cl = min(C, 4 * ((D + 3) // 4)) if limit else C
    r0, r1 = oracle.sad_backward(f0, f1, gin, lo, hi, channel_limit=cl)
    np.testing.assert_array_equal(df0.cpu().numpy(), r0)
    np.testing.assert_array_equal(df1.cpu().numpy(), r1)


def test_sad_matches_reference_golden():
    """The drop-in module against the reference's own outputs."""
    from conftest import load_golden
    import pytorch_cuda_stereo_sad_op as sad
    dev = torch.device("cuda:0")
    for name in ("sad_c8_d12", "sad_c8_neg", "sad_c8_d4_q"):
        g = load_golden(name)
        f0, f1 = torch.from_numpy(g["f0"]).to(dev), torch.from_numpy(g["f1"]).to(dev)
        lo, hi = int(g["min_disp"]), int(g["max_disp"])
        np.testing.assert_array_equal(sad.forward(f0, f1, lo, hi, 1.0).cpu().numpy(), g["volume"])
        df0, df1 = sad.backward(f0, f1, lo, hi, torch.from_numpy(g["in_grad"]).to(dev))
        np.testing.assert_array_equal(df0.cpu().numpy(), g["df0"])
        np.testing.assert_array_equal(df1.cpu().numpy(), g["df1"])
