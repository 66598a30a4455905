"""Drop-in for the reference's `pytorch_cuda_flow_mp_sad_op`
(ops/flow_mp_sad/src/flow_mp_sad.cpp:10-35):
  forward(f0, f1, sws, offset_u, offset_v, blockIdx_u, blockIdx_v) -> [cv_u, cv_v, u_star, v_star]
  backward(f0, f1, sws, in_grad_u, in_grad_v, u_star, v_star) -> [df0, df1]
"""
from __future__ import annotations

from .. import ops


def forward(f0, f1, sws, offset_u, offset_v, blockIdx_u, blockIdx_v):
    return list(ops.flow_forward(f0, f1, int(sws), int(offset_u), int(offset_v), int(blockIdx_u), int(blockIdx_v)))


def backward(f0, f1, sws, in_grad_u, in_grad_v, u_star, v_star):
    return list(ops.flow_backward(f0, f1, int(sws), in_grad_u.contiguous(), in_grad_v.contiguous(),
                                  u_star.contiguous(), v_star.contiguous()))
