"""Reference import name `pytorch_cuda_lbp_op`.

The reference builds three different extensions under this one name
(ops/lbp_stereo/setup.py:13, ops/lbp_semantic_pw/setup.py:13,
ops/lbp_semantic_pw_pixel/setup.py:13) and reinstalls the one a script needs.
Here all three exist side by side (bpl_gb300.compat.*); this module exposes
the one named by the BPL_LBP_VARIANT environment variable: "stereo"
(default), "semantic_pw" or "semantic_pw_pixel".
"""
import importlib
import os

_VARIANT = os.environ.get("BPL_LBP_VARIANT", "stereo")
_MODULES = {"stereo": "lbp_stereo", "semantic_pw": "lbp_semantic_pw", "semantic_pw_pixel": "lbp_semantic_pw_pixel"}
if _VARIANT not in _MODULES:
    raise ImportError("BPL_LBP_VARIANT must be one of %s, got %r" % (sorted(_MODULES), _VARIANT))
_impl = importlib.import_module("bpl_gb300.compat." + _MODULES[_VARIANT])

forward_minsum = _impl.forward_minsum
backward_minsum = _impl.backward_minsum
