"""Drop-in for the reference's `pytorch_cuda_lbp_op` (stereo variant).

Signatures follow ops/lbp_stereo/src/lbp.cpp:16-55:
  forward_minsum(cost, jump, edge, messages, delta) -> [messages, messages_argmin, message_scale]
  backward_minsum(cost, jump, edge, in_grad, messages, messages_argmin, message_scale)
      -> [grad_cost, grad_jump, grad_edge, grad_messages]
`messages` is updated in place and returned as the same tensor; argmin is a
float32 tensor like the reference's.  Every batch item is processed (the
reference forward processes item 0 only).
"""
from __future__ import annotations

import torch

from .. import ops

VARIANT = ops.LBP_STEREO


def forward_minsum(cost, jump, edge, messages, delta):
    m, am, sc = ops.lbp_forward(VARIANT, cost, jump, edge, messages, int(delta), argmin_dtype=torch.float32)
    return [m, am, sc]


def backward_minsum(cost, jump, edge, in_grad, messages, messages_argmin, message_scale):
    gc, gj, ge, gm = ops.lbp_backward(VARIANT, jump, edge, in_grad, messages, messages_argmin, message_scale)
    return [gc, gj, ge, gm]
