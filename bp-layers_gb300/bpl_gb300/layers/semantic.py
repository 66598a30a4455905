"""Host-side mirrors of the reference's semantic BP layers on the GB300
kernels:
  global pairwise  ops/lbp_semantic_pw/message_passing_op_cuda.py:23-120
  pixel pairwise   ops/lbp_semantic_pw_pixel/message_passing_op_pw_pixel.py:143-229
Same classes, arguments and results; argmin indices are kept as uint8/int16
inside the autograd functions.
"""
from __future__ import annotations

import torch
import torch.nn as nn

from .. import ops
from .stereo import BeliefsSoftmin, Inference, TemperatureSoftmin  # noqa: F401  (Inference is shared)


def _argmin_dtype(L):
    return torch.uint8 if L <= 256 else torch.int16


class LBPMinSumFunctionGlobal(torch.autograd.Function):
    """forward(cost, L1, L2, edge, messages, delta, jump, single_pw) with jump
    (1,2,L,L) (or (1,1,L,L) when single_pw): builds the four directional
    matrices [P_x, P_x^T, P_y, P_y^T] (message_passing_op_cuda.py:27-40)."""

    @staticmethod
    def forward(ctx, cost, L1, L2, edge, messages, delta, jump, single_pw):
        single = bool(single_pw.item()) if torch.is_tensor(single_pw) else bool(single_pw)
        L = cost.shape[-1]
        j = torch.zeros((jump.shape[0], 4, jump.shape[2], jump.shape[3]), dtype=torch.float32, device=cost.device)
        if not single:
            j[0, 0] = jump[0, 0]
            j[0, 2] = jump[0, 1]
            j[0, 1] = jump[0, 0].permute((1, 0))
            j[0, 3] = jump[0, 1].permute((1, 0))
        else:
            j[0, :] = jump[0, 0]
        j = j.contiguous()
        messages, argmin, scale = ops.lbp_forward(ops.LBP_SEM_GLOBAL, cost, j, edge, messages, int(delta),
                                                  argmin_dtype=_argmin_dtype(L))
        ctx.save_for_backward(j, edge, messages, argmin, scale)
        ctx.single = single
        return messages

    @staticmethod
    def backward(ctx, in_grad):
        j, edge, messages, argmin, scale = ctx.saved_tensors
        gc, gj, ge, gm = ops.lbp_backward(ops.LBP_SEM_GLOBAL, j, edge, in_grad.contiguous(), messages, argmin, scale,
                                          copy_grad_messages=False)
        if not ctx.single:
            gout = torch.zeros((gj.shape[0], 2, gj.shape[2], gj.shape[3]), device=gj.device)
            gout[0, 0] += gj[0, 0]
            gout[0, 1] += gj[0, 2]
            gout[0, 0] += gj[0, 1].permute((1, 0))
            gout[0, 1] += gj[0, 3].permute((1, 0))
        else:
            gout = torch.zeros((gj.shape[0], 1, gj.shape[2], gj.shape[3]), device=gj.device)
            gout[0, 0] += gj[0, 0] + gj[0, 1] + gj[0, 2] + gj[0, 3]
        return gc, None, None, ge, gm, None, gout, None


class MessagePassingGlobal(nn.Module):
    """ops/lbp_semantic_pw/message_passing_op_cuda.py:75-120."""

    def __init__(self, device, max_iter, num_labels, delta, mode="min-sum"):
        super().__init__()
        self.device = device
        self.max_iter = max_iter
        if mode != "min-sum":
            raise ValueError("Unknown message parsing mode " + mode)
        self.mode = mode
        self.L1 = nn.Parameter(torch.tensor(0.1, device=device), requires_grad=True)
        self.L2 = nn.Parameter(torch.tensor(2.5, device=device), requires_grad=True)
        self.softmin = TemperatureSoftmin(dim=3, init_temp=1.0, device=device)
        self.delta = delta
        self.rescaleT = None

    def projectL1L2(self):
        self.L2.data = torch.max(self.L1.data, self.L2.data)

    def forward(self, prob_vol, edge_weights, messages, jump, single_pw=False):
        N, H, W, C = prob_vol.shape
        if edge_weights is None:
            edge_weights = torch.ones((N, 4, H, W), device=prob_vol.device)
        cost = -prob_vol
        for _ in range(self.max_iter):
            messages = LBPMinSumFunctionGlobal.apply(cost, self.L1, self.L2, edge_weights, messages, self.delta,
                                                     jump, torch.tensor(single_pw))
        return BeliefsSoftmin.apply(messages, cost, self.softmin.T)


class LBPMinSumFunctionPixel(torch.autograd.Function):
    """forward(cost, L1, L2, edge, messages, delta, jump) with jump
    (2,H,W,L,L), the LR and UD pairwise planes.  The reference layer builds
    a shifted and transposed (4,H,W,L,L) copy on every pass
    (message_passing_op_pw_pixel.py:27-38) and folds the (4,H,W,L,L) jump
    gradient back to two planes (:47-51); here the kernels read the two
    planes with that shift and transpose and accumulate the gradient in the
    two-plane layout (variant LBP_SEM_PIXEL_LAYER), so neither copy exists."""

    @staticmethod
    def forward(ctx, cost, L1, L2, edge, messages, delta, jump):
        L = cost.shape[-1]
        messages, argmin, scale = ops.lbp_forward(ops.LBP_SEM_PIXEL_LAYER, cost, jump.contiguous(), edge, messages,
                                                  int(delta), argmin_dtype=_argmin_dtype(L))
        ctx.save_for_backward(edge, messages, argmin, scale)
        return messages

    @staticmethod
    def backward(ctx, in_grad):
        edge, messages, argmin, scale = ctx.saved_tensors
        gc, gj, _, gm = ops.lbp_backward(ops.LBP_SEM_PIXEL_LAYER, None, edge, in_grad.contiguous(), messages, argmin,
                                         scale, copy_grad_messages=False)
        # no edge gradient in the reference's pixel variant
        ge = torch.zeros_like(edge)
        return gc, None, None, ge, gm, None, gj


class MessagePassingPixel(nn.Module):
    """ops/lbp_semantic_pw_pixel/message_passing_op_pw_pixel.py:182-229."""

    def __init__(self, device, max_iter, num_labels, delta, mode="min-sum"):
        super().__init__()
        self.device = device
        self.max_iter = max_iter
        if mode != "min-sum":
            raise ValueError("Unknown message parsing mode " + mode)
        self.mode = mode
        self.L1 = nn.Parameter(torch.tensor(0.1, device=device), requires_grad=True)
        self.L2 = nn.Parameter(torch.tensor(2.5, device=device), requires_grad=True)
        self.softmin = TemperatureSoftmin(dim=3, init_temp=1.0, device=device)
        self.delta = delta
        self.rescaleT = None

    def projectL1L2(self):
        self.L2.data = torch.max(self.L1.data, self.L2.data)

    def forward(self, prob_vol, edge_weights, messages, jump):
        N, H, W, C = prob_vol.shape
        if edge_weights is None:
            edge_weights = torch.ones((N, 4, H, W), device=prob_vol.device)
        cost = -prob_vol
        for _ in range(self.max_iter):
            messages = LBPMinSumFunctionPixel.apply(cost, self.L1, self.L2, edge_weights, messages, self.delta, jump)
        return BeliefsSoftmin.apply(messages, cost, self.softmin.T)
