"""Pins the CPU oracle to the reference ops themselves.

The fixtures in tests/golden/*.npz were written by tests/golden/make_golden.py,
which compiles the unmodified reference kernels (namespace rename only) and
runs them on a GB300 on seeded inputs.  These tests run on the CPU.

Bars:
  * LBP forward: argmin bit-exact; messages/scales bit-exact except where
    glibc's double exp/log and CUDA's differ in the last bit after rounding
    to float (counted, <= 4 ulp, rare);
  * LBP backward: the reference accumulates with float atomics in arbitrary
    order, the oracle in double: relative tolerance 2e-4 of the tensor's
    scale;
  * SAD forward and the flow cost volumes/argmins: bit-exact;
  * SAD backward: bit-exact (gather form, fixed order); flow backward df0
    bit-exact, df1 (atomics in the reference) within float tolerance.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import load_golden

GOLD = os.path.dirname(os.path.abspath(__file__)) + "/golden"


def ulps(a, b):
    ai = a.astype(np.float32).view(np.int32).astype(np.int64)
    bi = b.astype(np.float32).view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, -(ai & 0x7FFFFFFF), ai)
    bi = np.where(bi < 0, -(bi & 0x7FFFFFFF), bi)
    return np.abs(ai - bi)


def assert_close_bits(got, ref, what, max_ulp=4, max_frac=1e-3):
    u = ulps(got, ref)
    frac = np.count_nonzero(u) / max(u.size, 1)
    assert u.max() <= max_ulp, f"{what}: max ulp {u.max()}"
    assert frac <= max_frac, f"{what}: {frac:.2e} differ"


def names(prefix):
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLD, prefix + "*.npz")))


def test_fixtures_present():
    assert len(names("lbp_stereo_fwd")) >= 8
    assert names("lbp_sem") and names("sad_") and names("flow_")


@pytest.mark.parametrize("name", [n for n in names("lbp_stereo_fwd") if n != "lbp_stereo_fwd_c0"])
def test_stereo_forward_oracle_matches_reference(name):
    g = load_golden(name)
    iters = int(g["iters"])
    m = g["messages_in"]
    for it in range(iters):
        m, am, sc = oracle.lbp_forward(0, g["cost"], g["jump"], g["edge"], m, int(g["delta"]))
        np.testing.assert_array_equal(am, g[f"argmin_{it}"], err_msg=f"{name} argmin it{it}")
        assert_close_bits(m, g[f"messages_{it}"], f"{name} messages it{it}")
        assert_close_bits(sc, g[f"scale_{it}"], f"{name} scale it{it}")


def test_small_config_forward_oracle_matches_reference():
    g = load_golden("lbp_stereo_fwd_c0")
    cost = g["cost"]
    _, H, W, L = cost.shape
    jump = np.zeros((1, 4, 6, H, W), np.float32)
    jump[:, :, 1] = 0.5
    jump[:, :, 2] = 0.1
    jump[:, :, 4] = 0.1
    jump[:, :, 5] = 0.5
    edge = np.ones((1, 4, H, W), np.float32)
    m, am, sc = oracle.lbp_forward(0, cost, jump, edge, np.zeros((1, 4, H, W, L), np.float32), int(g["delta"]))
    np.testing.assert_array_equal(am.astype(np.uint8), g["argmin_u8"])
    assert_close_bits(m.reshape(-1)[g["msg_idx"]], g["msg_sample"], "c0 message sample")
    assert_close_bits(sc, g["scale"], "c0 scale")


@pytest.mark.parametrize("name,variant", [("lbp_sem_global_l19", 1), ("lbp_sem_global_l19_trunc", 1),
                                          ("lbp_sem_pixel_l7", 2)])
def test_semantic_forward_oracle_matches_reference(name, variant):
    g = load_golden(name)
    m = g["messages_in"]
    for it in range(int(g["iters"])):
        m, am, sc = oracle.lbp_forward(variant, g["cost"], g["jump"], g["edge"], m, int(g["delta"]))
        np.testing.assert_array_equal(am, g[f"argmin_{it}"], err_msg=f"{name} argmin it{it}")
        assert_close_bits(m, g[f"messages_{it}"], f"{name} messages it{it}")


def _rel_close(got, ref, tol, what):
    scale = max(np.abs(ref).max(), 1e-12)
    err = np.abs(got - ref).max() / scale
    assert err <= tol, f"{what}: relative error {err:.2e}"


@pytest.mark.parametrize("name", names("lbp_stereo_bwd"))
def test_stereo_backward_oracle_matches_reference(name):
    g = load_golden(name)
    gc, gj, ge, gm = oracle.lbp_backward_ref(0, g["jump"], g["edge"], g["in_grad"], g["messages"],
                                             g["argmin"], g["scale"])
    _rel_close(gc, g["grad_cost"], 2e-4, name + " grad_cost")
    _rel_close(gj, g["grad_jump"], 2e-4, name + " grad_jump")
    _rel_close(ge, g["grad_edge"], 2e-4, name + " grad_edge")
    np.testing.assert_array_equal(gm.astype(np.float32), g["grad_messages"])


@pytest.mark.parametrize("name,variant", [("lbp_sem_global_l19", 1), ("lbp_sem_global_l19_trunc", 1),
                                          ("lbp_sem_pixel_l7", 2)])
def test_semantic_backward_oracle_matches_reference(name, variant):
    g = load_golden(name)
    gc, gj, ge, gm = oracle.lbp_backward_ref(variant, g["jump"], g["edge"], g["in_grad"], g["messages_1"],
                                             g["argmin_1"], g["scale_1"])
    _rel_close(gc, g["grad_cost"], 2e-4, name + " grad_cost")
    _rel_close(gj, g["grad_jump"], 2e-4, name + " grad_jump")
    _rel_close(ge, g["grad_edge"], 2e-4, name + " grad_edge")


@pytest.mark.parametrize("name", names("sad_"))
def test_sad_oracle_matches_reference(name):
    g = load_golden(name)
    lo, hi = int(g["min_disp"]), int(g["max_disp"])
    vol = oracle.sad_forward(g["f0"], g["f1"], lo, hi)
    np.testing.assert_array_equal(vol, g["volume"])
    D = hi - lo + 1
    C = g["f0"].shape[1]
    df0, df1 = oracle.sad_backward(g["f0"], g["f1"], g["in_grad"], lo, hi,
                                   channel_limit=min(C, 4 * ((D + 3) // 4)))
    np.testing.assert_array_equal(df0, g["df0"])
    np.testing.assert_array_equal(df1, g["df1"])


@pytest.mark.parametrize("name", names("flow_"))
def test_flow_oracle_matches_reference(name):
    g = load_golden(name)
    args = [int(g[k]) for k in ("sws", "offset_u", "offset_v", "block_u", "block_v")]
    cu, cv, us, vs = oracle.flow_forward(g["f0"], g["f1"], *args)
    for k, v in (("cv_u", cu), ("cv_v", cv), ("u_star", us), ("v_star", vs)):
        np.testing.assert_array_equal(v, g[k], err_msg=f"{name} {k}")
    df0, df1 = oracle.flow_backward(g["f0"], g["f1"], args[0], g["in_grad_u"], g["in_grad_v"], g["u_star"],
                                    g["v_star"])
    np.testing.assert_array_equal(df0, g["df0"])
    _rel_close(df1, g["df1"], 1e-5, name + " df1")
