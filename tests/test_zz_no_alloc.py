"""The allocation-free backward entry point (bpl_lbp_backward_noalloc).

It serves hosts that cannot call cudaMalloc when they run the backward (device
memory owned by another runtime's pool, a fixed start-up budget, or loops that
must not synchronise on an allocation): its scratch is a fixed device array
inside the library.  These tests call it through the C ABI and compare it
with the workspace-taking entry point, bpl_lbp_backward, on two calls in a row:
a larger problem first, then a smaller one, so that the second call finds the
array holding the first call's data at and beyond every offset it uses.  Both
entry points accumulate with float atomics, so results agree to float
rounding, not bit for bit.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import cases

TOL = 1e-5


def test_noalloc_rejects_oversized_problems_on_the_host(bpl_lib):
    # 1 x 512 x 512 x 64 labels needs 128 MiB of scratch: rejected before any
    # device work (null pointers are never touched)
    st = bpl_lib.bpl_lbp_backward_noalloc(0, None, None, None, None, None, 1, None, None, None, None,
                                          1, 512, 512, 64, 6, 1, 1, None)
    assert st == 1
    assert b"exceeds the fixed" in bpl_lib.bpl_last_error()


@pytest.mark.gpu
def test_noalloc_backward_matches_workspace_backward_twice():
    torch = pytest.importorskip("torch")
    from bpl_gb300 import _lib, ops
    dev = torch.device("cuda:0")
    lib = _lib.lib()
    # the first call's scratch (2*2*48*80*96 floats, 5.6 MiB) covers the second's
    shapes = ((5, (2, 48, 80, 96)), (6, (1, 24, 40, 64)))
    for call, (seed, (B, H, W, L)) in enumerate(shapes):
        g = cases.rng(seed)
        cost = torch.from_numpy(cases.random_cost(g, B, H, W, L)).to(dev)
        jump = torch.from_numpy(cases.random_taps8(g, B, H, W, offset_scale=1.0)).to(dev)
        edge = torch.from_numpy(cases.edge_weights(g, B, H, W)).to(dev)
        m = torch.from_numpy(cases.random_messages(g, B, H, W, L)).to(dev)
        m, am, sc = ops.lbp_forward(ops.LBP_STEREO, cost, jump, edge, m, 3, argmin_dtype=torch.uint8)
        gin = torch.randn((B, 4, H, W, L), device=dev, generator=torch.Generator(device=dev).manual_seed(seed))
        ref_gc, ref_gj, ref_ge, _ = ops.lbp_backward(ops.LBP_STEREO, jump, edge, gin, m, am, sc)
        gc = torch.empty_like(ref_gc)
        gj = torch.empty_like(ref_gj)
        ge = torch.empty_like(ref_ge)
        st = lib.bpl_lbp_backward_noalloc(
            ops.LBP_STEREO, jump.data_ptr(), edge.data_ptr(), gin.data_ptr(), m.data_ptr(), am.data_ptr(),
            ops.ARGMIN_U8, sc.data_ptr(), gc.data_ptr(), gj.data_ptr(), ge.data_ptr(),
            B, H, W, L, jump.shape[2], jump.shape[0], edge.shape[0], torch.cuda.current_stream().cuda_stream)
        assert st == 0, lib.bpl_last_error()
        torch.cuda.synchronize()
        for name, a, b in (("grad_cost", gc, ref_gc), ("grad_jump", gj, ref_gj), ("grad_edge", ge, ref_ge)):
            a, b = a.cpu().numpy(), b.cpu().numpy()
            err = np.abs(a - b).max() / max(np.abs(b).max(), 1e-12)
            assert err <= TOL, f"call {call}: {name} relative difference {err:.2e}"
