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
    (cv_u, cv_v, u_star, v_star).  sws <= 108 is one window; sws == 216 is
    four 108-windows merged exactly as the reference merges them (the kernel
    here could take the whole window at once, but the merge fixes the
    reference's index arithmetic and tie order).  The reference's sws == 432
    branch is unfinished (it returns undefined names); it raises here."""

    @staticmethod
    def forward(ctx, f0, f1, sws):
        f0c, f1c = f0.contiguous(), f1.contiguous()
        if sws <= 108:
            cv_u, cv_v, u_star, v_star = ops.flow_forward(f0c, f1c, sws, 0, 0, 0, 0)
        elif sws == 2 * 108:
            s = sws // 2
            cv00_u, cv00_v, u00, v00 = ops.flow_forward(f0c, f1c, s, -s // 2, -s // 2, 0, 0)
            cv01_u, cv01_v, u01, v01 = ops.flow_forward(f0c, f1c, s, -s // 2, s // 2, 0, 1)
            cv10_u, cv10_v, u10, v10 = ops.flow_forward(f0c, f1c, s, s // 2, -s // 2, 1, 0)
            cv11_u, cv11_v, u11, v11 = ops.flow_forward(f0c, f1c, s, s // 2, s // 2, 1, 1)
            u0 = torch.cat((cv00_u, cv10_u[:, :, :, 1:]), dim=-1)
            u1 = torch.cat((cv01_u, cv11_u[:, :, :, 1:]), dim=-1)
            au0 = torch.cat((u00, u10[:, :, :, 1:]), dim=-1)
            au1 = torch.cat((u01, u11[:, :, :, 1:]), dim=-1)
            idx = u1 < u0
            u0[idx] = u1[idx]
            au0[idx] = au1[idx]
            v0 = torch.cat((cv00_v, cv01_v[:, :, :, 1:]), dim=-1)
            v1 = torch.cat((cv10_v, cv11_v[:, :, :, 1:]), dim=-1)
            av0 = torch.cat((v00, v01[:, :, :, 1:]), dim=-1)
            av1 = torch.cat((v10, v11[:, :, :, 1:]), dim=-1)
            idx = v1 < v0
            v0[idx] = v1[idx]
            av0[idx] = av1[idx]
            cv_u, u_star, cv_v, v_star = u0, au0, v0, av0
        else:
            raise ValueError("Unsupported sws: %s only allowd: <= 108 or 216" % sws)
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
