"""Reference import name `pytorch_cuda_stereo_sad_op` (ops/setup.py:13-16)."""
from bpl_gb300.compat.stereo_sad import backward, forward  # noqa: F401
