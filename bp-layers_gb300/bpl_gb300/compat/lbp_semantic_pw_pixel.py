"""Drop-in for the reference's `pytorch_cuda_lbp_op` (semantic
pixel-pairwise variant, ops/lbp_semantic_pw_pixel/src/lbp.cpp:15-54).

jump is (4,H,W,L,L); backward_minsum takes no jump argument and returns no
edge gradient (the reference returns a zero tensor, kept here).
"""
from __future__ import annotations

import torch

from .. import ops

VARIANT = ops.LBP_SEM_PIXEL


def forward_minsum(cost, jump, edge, messages, delta):
    m, am, sc = ops.lbp_forward(VARIANT, cost, jump, edge, messages, int(delta), argmin_dtype=torch.float32)
    return [m, am, sc]


def backward_minsum(cost, edge, in_grad, messages, messages_argmin, message_scale):
    gc, gj, _, gm = ops.lbp_backward(VARIANT, None, edge, in_grad, messages, messages_argmin, message_scale)
    ge = torch.zeros(tuple(edge.shape), dtype=torch.float32, device=edge.device)
    return [gc, gj, ge, gm]
