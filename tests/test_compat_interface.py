"""The drop-in boundary on the CPU: the reference's extension import names
resolve, expose the reference's functions with its parameter lists
(ops/lbp_stereo/src/lbp.cpp:16-55, ops/lbp_semantic_pw_pixel/src/lbp.cpp:
15-54, ops/sad/src/stereo_sad.cpp:10-29, ops/flow_mp_sad/src/
flow_mp_sad.cpp:10-35), and `pytorch_cuda_lbp_op` selects its variant from
BPL_LBP_VARIANT as the reference's reinstall-per-script does."""
import importlib
import inspect
import sys

import pytest

pytest.importorskip("torch")

LBP_FWD = ["cost", "jump", "edge", "messages", "delta"]
LBP_BWD = ["cost", "jump", "edge", "in_grad", "messages", "messages_argmin", "message_scale"]
LBP_BWD_PIXEL = ["cost", "edge", "in_grad", "messages", "messages_argmin", "message_scale"]


def _params(fn):
    return list(inspect.signature(fn).parameters)


def _load_lbp(monkeypatch, variant):
    if variant is None:
        monkeypatch.delenv("BPL_LBP_VARIANT", raising=False)
    else:
        monkeypatch.setenv("BPL_LBP_VARIANT", variant)
    sys.modules.pop("pytorch_cuda_lbp_op", None)
    return importlib.import_module("pytorch_cuda_lbp_op")


@pytest.mark.parametrize("variant,bwd,module", [(None, LBP_BWD, "lbp_stereo"), ("stereo", LBP_BWD, "lbp_stereo"),
                                                ("semantic_pw", LBP_BWD, "lbp_semantic_pw"),
                                                ("semantic_pw_pixel", LBP_BWD_PIXEL, "lbp_semantic_pw_pixel")])
def test_lbp_op_variants(monkeypatch, variant, bwd, module):
    mod = _load_lbp(monkeypatch, variant)
    try:
        assert _params(mod.forward_minsum) == LBP_FWD
        assert _params(mod.backward_minsum) == bwd
        assert mod.forward_minsum.__module__ == "bpl_gb300.compat." + module
    finally:
        sys.modules.pop("pytorch_cuda_lbp_op", None)


def test_lbp_op_unknown_variant(monkeypatch):
    with pytest.raises(ImportError):
        _load_lbp(monkeypatch, "sum_product")
    sys.modules.pop("pytorch_cuda_lbp_op", None)


def test_sad_and_flow_ops():
    sad = importlib.import_module("pytorch_cuda_stereo_sad_op")
    flow = importlib.import_module("pytorch_cuda_flow_mp_sad_op")
    assert _params(sad.forward) == ["f0", "f1", "min_disp", "max_disp", "step"]
    assert _params(sad.backward) == ["f0", "f1", "min_disp", "max_disp", "in_grad"]
    assert _params(flow.forward) == ["f0", "f1", "sws", "offset_u", "offset_v", "blockIdx_u", "blockIdx_v"]
    assert _params(flow.backward) == ["f0", "f1", "sws", "in_grad_u", "in_grad_v", "u_star", "v_star"]
