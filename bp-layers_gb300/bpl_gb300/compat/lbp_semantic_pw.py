"""Drop-in for the reference's `pytorch_cuda_lbp_op` (semantic
global-pairwise variant, ops/lbp_semantic_pw/src/lbp.cpp:16-55).

jump is (1,4,L,L) with jump[0,d,s,t] the cost of receiver label t given
sender label s; grad_jump is (N,4,L,L) with the gradient of the shared
matrix in item 0, like the reference.
"""
from __future__ import annotations

import torch

from .. import ops

VARIANT = ops.LBP_SEM_GLOBAL


def forward_minsum(cost, jump, edge, messages, delta):
    m, am, sc = ops.lbp_forward(VARIANT, cost, jump, edge, messages, int(delta), argmin_dtype=torch.float32)
    return [m, am, sc]


def backward_minsum(cost, jump, edge, in_grad, messages, messages_argmin, message_scale):
    gc, gj, ge, gm = ops.lbp_backward(VARIANT, jump, edge, in_grad, messages, messages_argmin, message_scale)
    return [gc, gj, ge, gm]
