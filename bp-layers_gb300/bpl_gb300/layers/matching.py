"""Host-side mirror of the reference's matching layers on the GB300 kernels:
StereoMatchingSadFunction (ops/sad/stereo_sad.py:5-19) and the score-volume
step of StereoMatchingSad (matching.py:35-43)."""
from __future__ import annotations

import torch

from .. import ops


class StereoMatchingSadFunction(torch.autograd.Function):
    """forward(f0, f1, min_disp, max_disp, step=1.0) -> SAD volume (B,H,W,D)."""

    @staticmethod
    def forward(ctx, f0, f1, min_disp, max_disp, step=1.0):
        ctx.save_for_backward(f0, f1)
        ctx.min_disp, ctx.max_disp, ctx.step = int(min_disp), int(max_disp), float(step)
        return ops.sad_forward(f0.contiguous(), f1.contiguous(), ctx.min_disp, ctx.max_disp, ctx.step)

    @staticmethod
    def backward(ctx, in_grad):
        f0, f1 = ctx.saved_tensors
        if ctx.step != 1.0:
            raise ValueError("Error: Backward for step != 1 is not implemented!")
        df0, df1 = ops.sad_backward(f0.contiguous(), f1.contiguous(), ctx.min_disp, ctx.max_disp,
                                    in_grad.contiguous())
        return df0, df1, None, None, None


def sad_score_volume(f0, f1, min_disp, max_disp, step=1.0):
    """-SAD, as StereoMatchingSad.compute_score_volume returns (matching.py:42-43)."""
    return -StereoMatchingSadFunction.apply(f0, f1, min_disp, max_disp, step)


class FlowMpSadFunction(torch.autograd.Function):
    """ops/flow_mp_sad/flow_mp_sad.py:5-119: forward(f0, f1, sws) ->
    (cv_u, cv_v, u_star, v_star).  The reference runs sws <= 108 as one
    window and sws == 216 as four 108-windows merged in Python (its kernel
    keeps the K x K window in shared memory); the merge equals one 217-window
    (same minima, indices and tie order), which the kernel here computes in
    one call.  Other window sizes raise ValueError as in the reference (its
    sws == 432 branch is unfinished: it returns undefined names)."""

    @staticmethod
    def forward(ctx, f0, f1, sws):
        f0c, f1c = f0.contiguous(), f1.contiguous()
        if not (sws <= 108 or sws == 2 * 108):
            raise ValueError("Unsupported sws: %s only allowd: <= 108 or 216" % sws)
        cv_u, cv_v, u_star, v_star = ops.flow_forward(f0c, f1c, sws, 0, 0, 0, 0)
        ctx.save_for_backward(f0c, f1c, u_star, v_star)
        ctx.sws = int(sws)
        return cv_u, cv_v, u_star, v_star

    @staticmethod
    def backward(ctx, in_grad_u, in_grad_v, u_star_grad, v_star_grad):
        f0, f1, u_star, v_star = ctx.saved_tensors
        df0, df1 = ops.flow_backward(f0, f1, ctx.sws, in_grad_u.contiguous(), in_grad_v.contiguous(), u_star,
                                     v_star)
        return df0, df1, None


def flow_score_volume(f0, f1, sws):
    """(-cv_u, -cv_v), as FlowMatchingSad.compute_score_volume (flow_matching.py:50-52)."""
    cv_u, cv_v, _, _ = FlowMpSadFunction.apply(f0, f1, sws)
    return -cv_u, -cv_v
