"""GB300-native BP-Layers hot path: min-sum LBP and SAD cost-volume ops.

Layout of the package:
  _build.py     nvcc build of libbpl_gb300.so (csrc/*.cu)
  _lib.py       ctypes binding of the C ABI (include/bpl_gb300.h)
  ops.py        torch-tensor wrappers of the C ABI (allocation, checks, stream)
  compat/       drop-in replacements of the reference's extension modules
"""
from ._lib import BplError, check_device_error, lib, read_device_error  # noqa: F401

__all__ = ["BplError", "check_device_error", "lib", "read_device_error"]
