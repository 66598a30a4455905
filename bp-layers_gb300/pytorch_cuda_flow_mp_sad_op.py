"""Reference import name `pytorch_cuda_flow_mp_sad_op` (ops/setup.py:17-20)."""
from bpl_gb300.compat.flow_mp_sad import backward, forward  # noqa: F401
