"""Drop-in for the reference's `pytorch_cuda_stereo_sad_op`
(ops/sad/src/stereo_sad.cpp:10-29):
  forward(f0, f1, min_disp, max_disp, step) -> cost volume (B,H,W,D)
  backward(f0, f1, min_disp, max_disp, in_grad) -> [df0, df1]
Results are bit-identical to the reference's for batch item 0 (the
reference leaves items > 0 at 40 / zero); the backward reproduces the
reference's channel coverage (only the first 4*ceil(D/4) channels)."""
from __future__ import annotations

from .. import ops


def forward(f0, f1, min_disp, max_disp, step=1.0):
    return ops.sad_forward(f0, f1, int(min_disp), int(max_disp), float(step))


def backward(f0, f1, min_disp, max_disp, in_grad):
    df0, df1 = ops.sad_backward(f0, f1, int(min_disp), int(max_disp), in_grad, reference_channel_limit=True)
    return [df0, df1]
