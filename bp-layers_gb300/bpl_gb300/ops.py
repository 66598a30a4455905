"""torch-tensor front end of the C ABI.

Each function checks its inputs the way the reference's pybind glue does
(CUDA, contiguous: ops/lbp_stereo/src/lbp.cpp:8-10) plus dtype and shape,
allocates outputs with torch on the input's device, and enqueues the CUDA
kernels on torch's current stream.  Errors raise BplError (the reference
aborts the process on CUDA errors; ops/include/error_util.h:13-23).
"""
from __future__ import annotations

import torch

import os

from ._lib import BplError, check, check_device_error, lib, read_device_error, set_wait_limit  # noqa: F401

LBP_STEREO, LBP_SEM_GLOBAL, LBP_SEM_PIXEL = 0, 1, 2
# the pixel variant fed the layer's (2,H,W,L,L) LR / UD pairwise planes (the
# kernels apply the shift and transpose of message_passing_op_pw_pixel.py:
# 27-38; the jump gradient comes back in the same two-plane layout)
LBP_SEM_PIXEL_LAYER = 3


def _pixel(variant: int) -> bool:
    return variant in (LBP_SEM_PIXEL, LBP_SEM_PIXEL_LAYER)


def _pixel_planes(variant: int) -> int:
    return 2 if variant == LBP_SEM_PIXEL_LAYER else 4
ARGMIN_NONE, ARGMIN_F32, ARGMIN_U8, ARGMIN_U16 = 0, 1, 2, 3

_ARGMIN_KIND = {torch.float32: ARGMIN_F32, torch.uint8: ARGMIN_U8, torch.int16: ARGMIN_U16,
                torch.uint16 if hasattr(torch, "uint16") else torch.int16: ARGMIN_U16}


def _stream(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def _check_input(name: str, t: torch.Tensor, dtype=torch.float32, dim=None):
    if not isinstance(t, torch.Tensor):
        raise BplError(f"{name} must be a tensor")
    if not t.is_cuda:
        raise BplError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise BplError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise BplError(f"{name} must be {dtype}, got {t.dtype}")
    if dim is not None and t.dim() != dim:
        raise BplError(f"{name} must have {dim} dimensions, got {t.dim()}")


def _ptr(t):
    return t.data_ptr() if t is not None else None


def lbp_forward(variant: int, cost: torch.Tensor, jump: torch.Tensor, edge: torch.Tensor,
                messages: torch.Tensor, delta: int, argmin_dtype=torch.float32, argmin=None,
                scale=None):
    """One LBP pass (RIGHT, LEFT, DOWN, UP sweeps), messages updated in place.

    Returns (messages, argmin, scale).  argmin has the messages' shape and
    `argmin_dtype` (float32 like the reference, or uint8/int16 for the
    compact storage); None skips storing it.  Preallocated argmin/scale
    buffers may be passed to avoid allocation.
    """
    _check_input("cost", cost, dim=4)
    _check_input("edge", edge, dim=4)
    _check_input("messages", messages, dim=5)
    _check_input("jump", jump)
    B, H, W, L = cost.shape
    if tuple(messages.shape) != (B, 4, H, W, L):
        raise BplError(f"messages must be {(B, 4, H, W, L)}, got {tuple(messages.shape)}")
    if edge.shape[1:] != (4, H, W) or edge.shape[0] not in (1, B):
        raise BplError(f"edge must be (B|1,4,H,W), got {tuple(edge.shape)}")
    Lv, jb = 0, 1
    if variant == LBP_STEREO:
        if jump.dim() != 5 or jump.shape[1] != 4 or jump.shape[3:] != (H, W) or jump.shape[0] not in (1, B):
            raise BplError(f"stereo jump must be (B|1,4,Lv,H,W), got {tuple(jump.shape)}")
        Lv, jb = jump.shape[2], jump.shape[0]
    elif variant == LBP_SEM_GLOBAL:
        if tuple(jump.shape[1:]) != (4, L, L):
            raise BplError(f"semantic jump must be (1,4,L,L), got {tuple(jump.shape)}")
    else:
        if tuple(jump.shape) != (_pixel_planes(variant), H, W, L, L):
            raise BplError(f"pixel jump must be ({_pixel_planes(variant)},H,W,L,L), got {tuple(jump.shape)}")
    if argmin_dtype is None:
        kind = ARGMIN_NONE
        argmin = None
    else:
        kind = _ARGMIN_KIND[argmin_dtype]
        if argmin is None:
            argmin = torch.zeros((B, 4, H, W, L), dtype=argmin_dtype, device=cost.device)
    if scale is None:
        scale = torch.zeros((B, 4, H, W), dtype=torch.float32, device=cost.device)
    st = _timed("lbp_forward", lambda: lib().bpl_lbp_forward(
        variant, _ptr(cost), _ptr(jump), _ptr(edge), _ptr(messages), _ptr(argmin), kind, _ptr(scale),
        B, H, W, L, Lv, jb, edge.shape[0], int(delta), _stream(cost)))
    check(st, "bpl_lbp_forward")
    return messages, argmin, scale


def lbp_backward_workspace_bytes(B: int, H: int, W: int, L: int) -> int:
    return int(lib().bpl_lbp_backward_workspace_size(B, H, W, L))


def lbp_backward(variant: int, jump, edge: torch.Tensor, in_grad: torch.Tensor, messages: torch.Tensor,
                 argmin: torch.Tensor, scale: torch.Tensor, workspace: torch.Tensor | None = None,
                 copy_grad_messages: bool = True, mode: str = "reference"):
    """Adjoint of one LBP pass.

    Returns (grad_cost, grad_jump, grad_edge, grad_messages).  mode
    "reference": the reference's adjoint, grad_messages is in_grad (copied
    unless copy_grad_messages=False); mode "exact": grad_messages is the
    gradient with respect to the pass's input messages (the other gradients
    are the same in both modes).  grad_edge is None for the pixel-pairwise
    variant.  `workspace` (uint8, at least lbp_backward_workspace_bytes) may
    be passed to avoid allocating it.
    """
    if mode not in ("reference", "exact"):
        raise BplError(f"unknown adjoint mode {mode!r}")
    _check_input("in_grad", in_grad, dim=5)
    _check_input("messages", messages, dim=5)
    _check_input("scale", scale, dim=4)
    _check_input("edge", edge, dim=4)
    _check_input("argmin", argmin, dtype=None, dim=5)
    B, _, H, W, L = messages.shape
    if tuple(in_grad.shape) != tuple(messages.shape) or tuple(argmin.shape) != tuple(messages.shape):
        raise BplError("in_grad/argmin must have the messages' shape")
    kind = _ARGMIN_KIND.get(argmin.dtype)
    if kind is None:
        raise BplError(f"argmin dtype {argmin.dtype} not supported")
    dev = messages.device
    Lv, jb = 0, 1
    if variant == LBP_STEREO:
        _check_input("jump", jump, dim=5)
        Lv, jb = jump.shape[2], jump.shape[0]
        grad_jump = torch.empty((jb, 4, Lv, H, W), dtype=torch.float32, device=dev)
    elif variant == LBP_SEM_GLOBAL:
        _check_input("jump", jump, dim=4)
        grad_jump = torch.empty((B, 4, L, L), dtype=torch.float32, device=dev)
    else:
        grad_jump = torch.empty((_pixel_planes(variant), H, W, L, L), dtype=torch.float32, device=dev)
    grad_cost = torch.empty((B, H, W, L), dtype=torch.float32, device=dev)
    grad_edge = None if _pixel(variant) else torch.empty(tuple(edge.shape), dtype=torch.float32, device=dev)
    need = lbp_backward_workspace_bytes(B, H, W, L)
    if workspace is None or workspace.numel() * workspace.element_size() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    if mode == "exact":
        grad_messages = torch.empty_like(messages)
        st = _timed("lbp_backward", lambda: lib().bpl_lbp_backward_exact(
            variant, _ptr(jump) if not _pixel(variant) else None, _ptr(edge), _ptr(in_grad),
            _ptr(messages), _ptr(argmin), kind, _ptr(scale), _ptr(grad_cost), _ptr(grad_jump),
            _ptr(grad_edge), _ptr(grad_messages), _ptr(workspace), workspace.numel() * workspace.element_size(),
            B, H, W, L, Lv, jb, edge.shape[0], _stream(messages)))
        check(st, "bpl_lbp_backward_exact")
        return grad_cost, grad_jump, grad_edge, grad_messages
    st = _timed("lbp_backward", lambda: lib().bpl_lbp_backward(
        variant, _ptr(jump) if not _pixel(variant) else None, _ptr(edge), _ptr(in_grad),
        _ptr(messages), _ptr(argmin), kind, _ptr(scale), _ptr(grad_cost), _ptr(grad_jump),
        _ptr(grad_edge), _ptr(workspace), workspace.numel() * workspace.element_size(),
        B, H, W, L, Lv, jb, edge.shape[0], _stream(messages)))
    check(st, "bpl_lbp_backward")
    grad_messages = in_grad.clone() if copy_grad_messages else in_grad
    return grad_cost, grad_jump, grad_edge, grad_messages


# ---------------------------------------------------------------------------
# Per-op CUDA-event timing (tracing).  When enabled, every C-ABI call made
# through this module records a start/end event pair on the stream it
# launches on; `timing_report()` returns {op: [ms, ...]}.
_timing = None


class timing:
    """Context manager: with ops.timing() as t: ...; then t.report()."""

    def __enter__(self):
        global _timing
        self.events = {}
        _timing = self.events
        return self

    def __exit__(self, *exc):
        global _timing
        _timing = None
        return False

    def report(self):
        torch.cuda.synchronize()
        return {k: [a.elapsed_time(b) for a, b in v] for k, v in self.events.items()}


# BPL_CHECK_DEVICE_ERRORS=1: every call made through this module synchronises
# and checks the device error word afterwards (a debugging mode; by default
# callers check with check_device_error() at their own synchronisation
# points).
_check_each_call = os.environ.get("BPL_CHECK_DEVICE_ERRORS", "0") not in ("", "0")


def _timed(name, fn):
    if _check_each_call:
        r = _timed_call(name, fn)
        if r == 0:
            check_device_error()
        return r
    return _timed_call(name, fn)


def _timed_call(name, fn):
    if _timing is None:
        return fn()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    r = fn()
    b.record()
    _timing.setdefault(name, []).append((a, b))
    return r


# ---------------------------------------------------------------------------
# SAD cost volumes

def sad_forward(f0: torch.Tensor, f1: torch.Tensor, min_disp: int, max_disp: int, step: float = 1.0,
                out: torch.Tensor | None = None) -> torch.Tensor:
    """Stereo SAD volume (B,H,W,D), bit-identical to the reference's
    stereo_sad_forward (every batch item processed)."""
    _check_input("f0", f0, dim=4)
    _check_input("f1", f1, dim=4)
    if f0.shape != f1.shape:
        raise BplError("f0 and f1 must have the same shape")
    B, C, H, W = f0.shape
    D = int(lib().bpl_sad_volume_depth(int(min_disp), int(max_disp), float(step)))
    if D < 1:
        raise BplError("empty disparity range")
    if out is None:
        out = torch.empty((B, H, W, D), dtype=torch.float32, device=f0.device)
    st = _timed("sad_forward", lambda: lib().bpl_sad_forward(
        _ptr(f0), _ptr(f1), _ptr(out), B, C, H, W, int(min_disp), int(max_disp), float(step), _stream(f0)))
    check(st, "bpl_sad_forward")
    return out


def sad_backward(f0: torch.Tensor, f1: torch.Tensor, min_disp: int, max_disp: int, in_grad: torch.Tensor,
                 reference_channel_limit: bool = False):
    """Gradients (df0, df1) of the SAD volume (step 1)."""
    _check_input("f0", f0, dim=4)
    _check_input("f1", f1, dim=4)
    _check_input("in_grad", in_grad, dim=4)
    B, C, H, W = f0.shape
    D = int(max_disp) - int(min_disp) + 1
    if tuple(in_grad.shape) != (B, H, W, D):
        raise BplError(f"in_grad must be {(B, H, W, D)}, got {tuple(in_grad.shape)}")
    df0 = torch.empty_like(f0)
    df1 = torch.empty_like(f1)
    st = _timed("sad_backward", lambda: lib().bpl_sad_backward(
        _ptr(f0), _ptr(f1), _ptr(in_grad), _ptr(df0), _ptr(df1), B, C, H, W, int(min_disp), int(max_disp),
        int(bool(reference_channel_limit)), _stream(f0)))
    check(st, "bpl_sad_backward")
    return df0, df1


def flow_forward(f0: torch.Tensor, f1: torch.Tensor, sws: int, offset_u: int = 0, offset_v: int = 0,
                 block_u: int = 0, block_v: int = 0):
    """Flow max-projected SAD: (cv_u, cv_v, u_star, v_star), each (B,H,W,sws+1)."""
    _check_input("f0", f0, dim=4)
    _check_input("f1", f1, dim=4)
    if f0.shape != f1.shape:
        raise BplError("f0 and f1 must have the same shape")
    B, C, H, W = f0.shape
    K = int(sws) + 1
    outs = [torch.empty((B, H, W, K), dtype=torch.float32, device=f0.device) for _ in range(4)]
    st = _timed("flow_forward", lambda: lib().bpl_flow_forward(
        _ptr(f0), _ptr(f1), *[_ptr(o) for o in outs], B, C, H, W, int(sws), int(offset_u), int(offset_v),
        int(block_u), int(block_v), _stream(f0)))
    check(st, "bpl_flow_forward")
    return tuple(outs)


def flow_backward(f0, f1, sws: int, in_grad_u, in_grad_v, u_star, v_star):
    """Gradients (df0, df1) of the flow SAD."""
    for nm, t in (("f0", f0), ("f1", f1)):
        _check_input(nm, t, dim=4)
    for nm, t in (("in_grad_u", in_grad_u), ("in_grad_v", in_grad_v), ("u_star", u_star), ("v_star", v_star)):
        _check_input(nm, t, dim=4)
    B, C, H, W = f0.shape
    df0 = torch.empty_like(f0)
    df1 = torch.empty_like(f1)
    nws = int(lib().bpl_flow_backward_workspace_size(B, C, H, W))
    ws = torch.empty((nws + 3) // 4, dtype=torch.float32, device=f0.device)
    st = _timed("flow_backward", lambda: lib().bpl_flow_backward_ws(
        _ptr(f0), _ptr(f1), _ptr(in_grad_u), _ptr(in_grad_v), _ptr(u_star), _ptr(v_star), _ptr(df0), _ptr(df1),
        _ptr(ws), nws, B, C, H, W, int(sws), _stream(f0)))
    check(st, "bpl_flow_backward_ws")
    return df0, df1


# ---------------------------------------------------------------------------
# FP16 storage (label axis padded to a multiple of 8)

def padded_labels(L: int) -> int:
    return (int(L) + 7) & ~7


def to_half_padded(t: torch.Tensor, L: int) -> torch.Tensor:
    """Copy a (..., L) tensor into a zero-padded (..., Lp) half tensor (one
    conversion pass when L is already a multiple of 8)."""
    Lp = padded_labels(L)
    if Lp == L and t.shape[-1] == L:
        return t.to(torch.float16).contiguous()
    out = torch.zeros(tuple(t.shape[:-1]) + (Lp,), dtype=torch.float16, device=t.device)
    out[..., :L] = t
    return out


def normalised_f16_messages(messages_h: torch.Tensor, L: int, scale: torch.Tensor | None = None) -> torch.Tensor:
    """(B,4,H,W,L) float log-normalised messages (the reference's form) from
    the min-referenced half rows of lbp_forward_f16: row - log(sum(exp(row)))
    over the L labels (or row - log(scale) with the scale lbp_forward_f16
    returned).  Rows no sweep writes (slot LEFT at x=0, RIGHT at x=W-1, UP at
    y=0, DOWN at y=H-1) are returned as stored."""
    m = messages_h[..., :L].float()
    if scale is not None:
        shift = torch.where(scale > 0, torch.log(scale), torch.zeros_like(scale)).unsqueeze(-1)
        return m - shift
    out = m - torch.logsumexp(m, dim=-1, keepdim=True)
    out[:, 0, :, 0] = m[:, 0, :, 0]
    out[:, 1, :, -1] = m[:, 1, :, -1]
    out[:, 2, 0] = m[:, 2, 0]
    out[:, 3, -1] = m[:, 3, -1]
    return out


def lbp_forward_f16(variant: int, cost_h: torch.Tensor, jump: torch.Tensor, edge: torch.Tensor,
                    messages_h: torch.Tensor, delta: int, L: int, argmin_dtype=torch.uint8, argmin=None, scale=None,
                    want_scale: bool = False):
    """One LBP pass with FP16 storage.  cost_h (B,H,W,Lp) and messages_h
    (B,4,H,W,Lp) half with Lp = padded_labels(L); messages updated in place.
    The pixel variant takes jump (4,H,W,L,Lp) half, the stereo variant float
    taps.  Returns (messages_h, argmin (B,4,H,W,Lp), scale).  Message rows
    are stored relative to the minimum of h (normalised_f16_messages gives
    the reference's log-normalised form).  The per-message scale, the sum
    of exp of the row, is computed only when asked for (a `scale` buffer or
    want_scale=True; None is returned otherwise): the FP16 adjoint
    recomputes the normalisation from the rows, and the stereo kernel's step
    is shorter without it."""
    _check_input("cost_h", cost_h, dtype=torch.float16, dim=4)
    _check_input("messages_h", messages_h, dtype=torch.float16, dim=5)
    _check_input("edge", edge, dim=4)
    Lp = padded_labels(L)
    B, H, W, Lc = cost_h.shape
    if Lc != Lp or tuple(messages_h.shape) != (B, 4, H, W, Lp):
        raise BplError(f"FP16 tensors need the label axis padded to {Lp}")
    Lv, jb = 0, 1
    if variant == LBP_STEREO:
        _check_input("jump", jump, dim=5)
        Lv, jb = jump.shape[2], jump.shape[0]
    elif _pixel(variant):
        _check_input("jump", jump, dtype=torch.float16, dim=5)
        if tuple(jump.shape) != (_pixel_planes(variant), H, W, L, Lp):
            raise BplError(f"pixel jump must be ({_pixel_planes(variant)},H,W,L,Lp) half, got {tuple(jump.shape)}")
    else:
        _check_input("jump", jump, dim=4)
        if tuple(jump.shape[1:]) != (4, L, L):
            raise BplError(f"semantic jump must be (1,4,L,L) float, got {tuple(jump.shape)}")
    # argmin_dtype=None: no argmin is written (inference)
    kind = ARGMIN_NONE if argmin_dtype is None else _ARGMIN_KIND[argmin_dtype]
    if argmin is None and kind != ARGMIN_NONE:
        argmin = torch.zeros((B, 4, H, W, Lp), dtype=argmin_dtype, device=cost_h.device)
    if scale is None and want_scale:
        scale = torch.zeros((B, 4, H, W), dtype=torch.float32, device=cost_h.device)
    if scale is not None:
        _check_input("scale", scale, dim=4)
    st = _timed("lbp_forward_f16", lambda: lib().bpl_lbp_forward_f16(
        variant, _ptr(cost_h), _ptr(jump), _ptr(edge), _ptr(messages_h), _ptr(argmin), kind, _ptr(scale),
        B, H, W, L, Lv, jb, edge.shape[0], int(delta), _stream(cost_h)))
    check(st, "bpl_lbp_forward_f16")
    return messages_h, argmin, scale


def lbp_backward_f16(variant: int, jump, edge: torch.Tensor, in_grad_h: torch.Tensor, messages_h: torch.Tensor,
                     argmin: torch.Tensor, scale: torch.Tensor | None, L: int, workspace: torch.Tensor | None = None):
    """Reference adjoint for FP16-stored messages (padded label axis).  The
    normalisation's Jacobian is formed from the rows themselves (softmax of
    the row), so `scale` is not needed (ignored; None allowed).
    Returns (grad_cost (B,H,W,Lp) float, grad_jump, grad_edge)."""
    _check_input("in_grad_h", in_grad_h, dtype=torch.float16, dim=5)
    _check_input("messages_h", messages_h, dtype=torch.float16, dim=5)
    _check_input("argmin", argmin, dtype=None, dim=5)
    _check_input("edge", edge, dim=4)
    B, _, H, W, Lp = messages_h.shape
    if Lp != padded_labels(L):
        raise BplError("messages_h must have the padded label axis")
    kind = _ARGMIN_KIND.get(argmin.dtype)
    dev = messages_h.device
    Lv, jb = 0, 1
    if variant == LBP_STEREO:
        _check_input("jump", jump, dim=5)
        Lv, jb = jump.shape[2], jump.shape[0]
        grad_jump = torch.empty((jb, 4, Lv, H, W), dtype=torch.float32, device=dev)
        grad_edge = torch.empty(tuple(edge.shape), dtype=torch.float32, device=dev)
    elif _pixel(variant):
        grad_jump = torch.empty((_pixel_planes(variant), H, W, L, L), dtype=torch.float32, device=dev)
        grad_edge = None
    else:
        _check_input("jump", jump, dim=4)
        grad_jump = torch.empty((B, 4, L, L), dtype=torch.float32, device=dev)
        grad_edge = torch.empty(tuple(edge.shape), dtype=torch.float32, device=dev)
    grad_cost = torch.empty((B, H, W, Lp), dtype=torch.float32, device=dev)
    need = lbp_backward_workspace_bytes(B, H, W, Lp)
    if workspace is None or workspace.numel() * workspace.element_size() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    st = _timed("lbp_backward_f16", lambda: lib().bpl_lbp_backward_f16(
        variant, _ptr(jump) if not _pixel(variant) else None, _ptr(edge), _ptr(in_grad_h), _ptr(messages_h),
        _ptr(argmin), kind, _ptr(scale), _ptr(grad_cost), _ptr(grad_jump), _ptr(grad_edge), _ptr(workspace),
        workspace.numel() * workspace.element_size(), B, H, W, L, Lv, jb, edge.shape[0], _stream(messages_h)))
    check(st, "bpl_lbp_backward_f16")
    return grad_cost, grad_jump, grad_edge


def lbp_backward_passes(variant: int, jump, edge: torch.Tensor, in_grad: torch.Tensor, messages: torch.Tensor,
                        argmins: torch.Tensor, scales: torch.Tensor, L: int | None = None,
                        workspace: torch.Tensor | None = None, grad_cost_into: torch.Tensor | None = None,
                        cost_sign: float = 1.0, layer_taps: bool = False):
    """Reference adjoint of P passes run in place on one messages tensor,
    in one launch: argmins (P,B,4,H,W,Ls) and scales (P,B,4,H,W) stacked in
    pass order; in_grad and messages shared (the reference's backward of each
    pass reads the final messages and passes in_grad through).  FP32
    (messages float32) or FP16 storage (messages half, padded label axis,
    L given; scales may be None, the FP16 adjoint normalising from the
    rows).  Returns (grad_cost, grad_jump, grad_edge) summed over the
    passes; the message gradient is in_grad.

    grad_cost_into: a float (B,H,W,L) or (B,H,W,Ls) tensor the cost
    gradient is added onto, times cost_sign (+1 or -1), instead of a new
    zeroed one (bpl_lbp_backward_passes_into); it is returned as grad_cost.
    layer_taps (with grad_cost_into; stereo, 6 taps): jump is the layer's
    packed taps [offset, L2, L1, 0, L1, L2] and grad_jump holds what the
    layer's fold needs (the L2 taps' gradient summed in tap 1, taps 3 and 5
    none)."""
    half = messages.dtype == torch.float16
    if not isinstance(in_grad, torch.Tensor) or in_grad.dtype != messages.dtype or in_grad.dim() != 5 \
            or not in_grad.is_cuda:
        raise BplError("in_grad must be a CUDA tensor of the messages' dtype and rank")
    # a (B,4,H,W,Ls) gradient, contiguous or the beliefs' (B,1,H,W,Ls)
    # gradient expanded over the four slots (slot stride 0): no copy
    if in_grad.shape[1] != 4 or in_grad.stride(4) != 1 or in_grad.stride(3) != in_grad.shape[4] \
            or in_grad.stride(2) != in_grad.shape[3] * in_grad.shape[4]:
        in_grad = in_grad.contiguous()
    g_bstride, g_sstride = in_grad.stride(0), in_grad.stride(1)
    _check_input("messages", messages, dtype=None, dim=5)
    _check_input("argmins", argmins, dtype=None, dim=6)
    _check_input("edge", edge, dim=4)
    B, _, H, W, Ls = messages.shape
    P = argmins.shape[0]
    if L is None:
        L = Ls
    if tuple(argmins.shape) != (P, B, 4, H, W, Ls):
        raise BplError("argmins must be stacked (P,B,4,H,W,Ls)")
    if scales is None:
        if not half:
            raise BplError("scales are required with FP32 storage (the reference's backward_minsum argument)")
    else:
        _check_input("scales", scales, dim=5)
        if tuple(scales.shape) != (P, B, 4, H, W):
            raise BplError("scales must be stacked (P,B,4,H,W)")
    if half and Ls != padded_labels(L):
        raise BplError("FP16 messages must have the padded label axis")
    kind = _ARGMIN_KIND.get(argmins.dtype)
    if kind is None:
        raise BplError(f"argmin dtype {argmins.dtype} not supported")
    dev = messages.device
    Lv, jb = 0, 1
    if variant == LBP_STEREO:
        _check_input("jump", jump, dim=5)
        Lv, jb = jump.shape[2], jump.shape[0]
        grad_jump = torch.empty((jb, 4, Lv, H, W), dtype=torch.float32, device=dev)
    elif variant == LBP_SEM_GLOBAL:
        _check_input("jump", jump, dim=4)
        grad_jump = torch.empty((B, 4, L, L), dtype=torch.float32, device=dev)
    else:
        grad_jump = torch.empty((_pixel_planes(variant), H, W, L, L), dtype=torch.float32, device=dev)
    grad_edge = None if _pixel(variant) else torch.empty(tuple(edge.shape), dtype=torch.float32, device=dev)
    need = P * lbp_backward_workspace_bytes(B, H, W, Ls)
    if workspace is None or workspace.numel() * workspace.element_size() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    name = "lbp_backward_f16" if half else "lbp_backward"
    ws_bytes = workspace.numel() * workspace.element_size()
    jp = _ptr(jump) if not _pixel(variant) else None
    if layer_taps and (grad_cost_into is None or variant != LBP_STEREO or Lv != 6):
        raise BplError("layer_taps: stereo with 6 taps, through grad_cost_into")
    if grad_cost_into is None:
        grad_cost = torch.empty((B, H, W, Ls), dtype=torch.float32, device=dev)
        fn = lib().bpl_lbp_backward_passes_f16 if half else lib().bpl_lbp_backward_passes
        st = _timed(name, lambda: fn(
            variant, jp, _ptr(edge), _ptr(in_grad), g_bstride, g_sstride, _ptr(messages), _ptr(argmins), kind,
            _ptr(scales), _ptr(grad_cost), _ptr(grad_jump), _ptr(grad_edge), _ptr(workspace), ws_bytes, B, H, W, L,
            Lv, jb, edge.shape[0], P, _stream(messages)))
    else:
        grad_cost = grad_cost_into
        _check_input("grad_cost_into", grad_cost, dim=4)
        if tuple(grad_cost.shape[:3]) != (B, H, W) or grad_cost.shape[3] not in (L, Ls):
            raise BplError("grad_cost_into must be (B,H,W,L) or (B,H,W,Ls)")
        if cost_sign not in (1.0, -1.0):
            raise BplError("cost_sign must be +1 or -1")
        st = _timed(name, lambda: lib().bpl_lbp_backward_passes_into(
            int(half), variant, jp, _ptr(edge), _ptr(in_grad), g_bstride, g_sstride, _ptr(messages), _ptr(argmins),
            kind, _ptr(scales), _ptr(grad_cost), grad_cost.shape[3], float(cost_sign), _ptr(grad_jump),
            _ptr(grad_edge), _ptr(workspace), ws_bytes, B, H, W, L, Lv, jb, edge.shape[0], P, int(bool(layer_taps)),
            _stream(messages)))
    check(st, "bpl_lbp_backward_passes")
    return grad_cost, grad_jump, grad_edge


def beliefs_forward(messages: torch.Tensor, cost: torch.Tensor, temperature: torch.Tensor, L: int | None = None,
                    out: torch.Tensor | None = None) -> torch.Tensor:
    """softmin(((((M0+M1)+M2)+M3)+cost)/T) over labels, fused (one pass).
    messages (B,4,H,W,Ls) float or half (padded), cost (B,H,W,L) float,
    temperature a one-element float CUDA tensor."""
    _check_input("messages", messages, dtype=None, dim=5)
    _check_input("cost", cost, dim=4)
    B, _, H, W, Ls = messages.shape
    L = cost.shape[-1] if L is None else L
    if out is None:
        out = torch.empty((B, H, W, L), dtype=torch.float32, device=cost.device)
    st = _timed("beliefs_forward", lambda: lib().bpl_beliefs_forward(
        _ptr(messages), int(messages.dtype == torch.float16), _ptr(cost), _ptr(temperature), _ptr(out),
        B, H, W, L, Ls, _stream(cost)))
    check(st, "bpl_beliefs_forward")
    return out


def broadcast_slots(src: torch.Tensor) -> torch.Tensor:
    """(B, ...) contiguous float or half -> (B, 4, ...) with src in every
    message slot (a materialised copy of src.unsqueeze(1).expand(...))."""
    if not src.is_cuda or not src.is_contiguous() or src.dtype not in (torch.float32, torch.float16):
        raise BplError("broadcast_slots: src must be a contiguous CUDA float or half tensor")
    B = src.shape[0]
    dst = torch.empty((B, 4) + tuple(src.shape[1:]), dtype=src.dtype, device=src.device)
    n = src.numel() // B
    st = _timed("broadcast_slots", lambda: lib().bpl_broadcast_slots(
        _ptr(src), _ptr(dst), B, n, src.element_size(), _stream(src)))
    check(st, "bpl_broadcast_slots")
    return dst


def upsample_add_beliefs(beliefs: torch.Tensor, pv: torch.Tensor, weight: float = 0.5) -> torch.Tensor:
    """pv (N,2h,2w,2d) += weight * trilinear x2 upsampling of beliefs
    (N,h,w,d), in place (stereo.py:104-113 with weight 0.5); returns pv."""
    _check_input("beliefs", beliefs, dim=4)
    _check_input("pv", pv, dim=4)
    N, h, w, d = beliefs.shape
    if tuple(pv.shape) != (N, 2 * h, 2 * w, 2 * d):
        raise BplError(f"pv must be {(N, 2 * h, 2 * w, 2 * d)}, got {tuple(pv.shape)}")
    st = _timed("upsample_add_beliefs", lambda: lib().bpl_upsample_add_beliefs(
        _ptr(beliefs), _ptr(pv), N, h, w, d, float(weight), _stream(pv)))
    check(st, "bpl_upsample_add_beliefs")
    return pv


def leaf_message_grad(in_grad: torch.Tensor) -> torch.Tensor:
    """The message gradient handed to a leaf message tensor: a slot-broadcast
    in_grad (stride 0 over the slots, as the fused beliefs return it) is
    written out by one kernel, which autograd then keeps as .grad without a
    copy of its own; anything else is returned as it is."""
    if in_grad.dim() == 5 and in_grad.stride(1) == 0 and in_grad.shape[1] == 4:
        src = in_grad[:, 0]
        if src.is_contiguous():
            return broadcast_slots(src)
    return in_grad


def half_padded(src: torch.Tensor, sign: float = 1.0) -> torch.Tensor:
    """(..., L) float -> (..., Lp) half of sign * src, labels L..Lp-1 zeroed,
    one kernel pass (bpl_half_padded); the FP16-storage cost volume from the
    probability volume with sign -1."""
    _check_input("src", src, dim=None)
    L = src.shape[-1]
    Lp = padded_labels(L)
    out = torch.empty(tuple(src.shape[:-1]) + (Lp,), dtype=torch.float16, device=src.device)
    rows = src.numel() // L
    st = _timed("half_padded", lambda: lib().bpl_half_padded(_ptr(src), float(sign), _ptr(out), rows, L, Lp,
                                                             _stream(src)))
    check(st, "bpl_half_padded")
    return out


def beliefs_forward_any_cost(messages: torch.Tensor, cost: torch.Tensor, temperature: torch.Tensor, L: int,
                             out: torch.Tensor | None = None, cost_sign: float = 1.0,
                             log_norm: torch.Tensor | None = None) -> torch.Tensor:
    """beliefs_forward with z = sum + cost_sign * cost, the cost float
    (B,H,W,L) or the FP16-storage half volume (B,H,W,Lp)
    (bpl_beliefs_forward_ex); cost_sign -1 takes the probability volume.
    log_norm: a (B,H,W) float tensor receiving min(z/T) - log(sum) per
    pixel, for beliefs_backward_fused."""
    _check_input("messages", messages, dtype=None, dim=5)
    _check_input("cost", cost, dtype=None, dim=4)
    B, _, H, W, Ls = messages.shape
    if out is None:
        out = torch.empty((B, H, W, L), dtype=torch.float32, device=cost.device)
    st = _timed("beliefs_forward", lambda: lib().bpl_beliefs_forward_ex(
        _ptr(messages), int(messages.dtype == torch.float16), _ptr(cost), int(cost.dtype == torch.float16),
        float(cost_sign), _ptr(temperature), _ptr(out), _ptr(log_norm), B, H, W, L, Ls, _stream(cost)))
    check(st, "bpl_beliefs_forward_ex")
    return out


BELIEF_COPY_NONE, BELIEF_COPY_HALF, BELIEF_COPY_SLOTS, BELIEF_COPY_FLOAT = 0, 1, 2, 3


def beliefs_backward_fused(messages: torch.Tensor, cost: torch.Tensor, temperature: torch.Tensor,
                           beliefs: torch.Tensor, grad_beliefs: torch.Tensor, grad_z_sign: float, copy_kind: int,
                           want_temperature: bool = True, cost_sign: float = 1.0,
                           log_norm: torch.Tensor | None = None):
    """Gradient of the fused epilogue for the layer's fused backward
    (bpl_beliefs_backward_ex): returns (grad_z_sign * grad_z (B,H,W,L),
    the copy of +grad_z selected by copy_kind or None, grad_T or None).
    copy_kind: BELIEF_COPY_HALF (B,1,H,W,Lp) half, BELIEF_COPY_SLOTS
    (B,4,H,W,L) float, BELIEF_COPY_FLOAT (B,1,H,W,L) float; cost and
    cost_sign as beliefs_forward_any_cost.  With the forward's log_norm the
    temperature's gradient takes z/T from the beliefs (messages and cost are
    not read)."""
    _check_input("beliefs", beliefs, dim=4)
    grad_beliefs = grad_beliefs.contiguous()
    _check_input("grad_beliefs", grad_beliefs, dim=4)
    B, _, H, W, Ls = messages.shape
    L = beliefs.shape[-1]
    dev = beliefs.device
    gz = torch.empty_like(beliefs)
    if copy_kind == BELIEF_COPY_HALF:
        copy = torch.empty((B, 1, H, W, padded_labels(L)), dtype=torch.float16, device=dev)
    elif copy_kind == BELIEF_COPY_SLOTS:
        copy = torch.empty((B, 4, H, W, L), dtype=torch.float32, device=dev)
    elif copy_kind == BELIEF_COPY_FLOAT:
        copy = torch.empty((B, 1, H, W, L), dtype=torch.float32, device=dev)
    else:
        copy = None
    gT = torch.empty(1, dtype=torch.float32, device=dev) if want_temperature else None
    st = _timed("beliefs_backward", lambda: lib().bpl_beliefs_backward_ex(
        _ptr(messages), int(messages.dtype == torch.float16), _ptr(cost), int(cost.dtype == torch.float16),
        float(cost_sign), _ptr(temperature), _ptr(beliefs), _ptr(grad_beliefs), _ptr(gz), float(grad_z_sign),
        _ptr(copy), copy_kind, _ptr(gT), _ptr(log_norm), B, H, W, L, Ls, _stream(beliefs)))
    check(st, "bpl_beliefs_backward_ex")
    return gz, copy, gT


def beliefs_backward(messages: torch.Tensor, cost: torch.Tensor, temperature: torch.Tensor, beliefs: torch.Tensor,
                     grad_beliefs: torch.Tensor, want_temperature: bool = True):
    """Gradient of the fused epilogue: (grad_z (B,H,W,L), grad_T (1,) or None)."""
    _check_input("beliefs", beliefs, dim=4)
    grad_beliefs = grad_beliefs.contiguous()
    _check_input("grad_beliefs", grad_beliefs, dim=4)
    B, _, H, W, Ls = messages.shape
    L = beliefs.shape[-1]
    gz = torch.empty_like(beliefs)
    gT = torch.empty(1, dtype=torch.float32, device=beliefs.device) if want_temperature else None
    st = _timed("beliefs_backward", lambda: lib().bpl_beliefs_backward(
        _ptr(messages), int(messages.dtype == torch.float16), _ptr(cost), _ptr(temperature), _ptr(beliefs),
        _ptr(grad_beliefs), _ptr(gz), _ptr(gT), B, H, W, L, Ls, _stream(beliefs)))
    check(st, "bpl_beliefs_backward")
    return gz, gT


# ---------------------------------------------------------------------------
# Epilogue kernels (cost from SAD, disparity from messages, inference)

def cost_from_sad(sad: torch.Tensor, temperature: float = 1.0, half: bool = False,
                  out: torch.Tensor | None = None) -> torch.Tensor:
    """cost = -softmax(-sad / T) over the disparities of a (B,H,W,D) SAD
    volume, one pass; half=True writes the FP16-storage layout (B,H,W,Lp)
    with the label axis padded to a multiple of 8 (padding zeroed)."""
    _check_input("sad", sad, dim=4)
    B, H, W, D = sad.shape
    if not temperature > 0:
        raise BplError("temperature must be positive")
    Ls = padded_labels(D) if half else D
    dtype = torch.float16 if half else torch.float32
    if out is None:
        out = torch.empty((B, H, W, Ls), dtype=dtype, device=sad.device)
    elif out.dtype != dtype or tuple(out.shape) != (B, H, W, Ls) or not out.is_contiguous():
        raise BplError(f"out must be a contiguous {(B, H, W, Ls)} {dtype} tensor")
    st = _timed("cost_from_sad", lambda: lib().bpl_cost_from_sad(
        _ptr(sad), _ptr(out), int(half), B, H, W, D, Ls, float(temperature), _stream(sad)))
    check(st, "bpl_cost_from_sad")
    return out


def messages_argmin(messages: torch.Tensor, cost: torch.Tensor, L: int | None = None,
                    out: torch.Tensor | None = None, out_dtype=torch.int64) -> torch.Tensor:
    """(B,H,W) disparity = argmin over labels of ((((M0+M1)+M2)+M3)+cost),
    first index: the beliefs' argmax without the belief volume.  messages
    (B,4,H,W,Ls) and cost (B,H,W,Lc), each float or half (padded rows)."""
    _check_input("messages", messages, dtype=None, dim=5)
    _check_input("cost", cost, dtype=None, dim=4)
    B, _, H, W, Ls = messages.shape
    Lc = cost.shape[-1]
    if messages.shape[1] != 4 or tuple(cost.shape[:3]) != (B, H, W):
        raise BplError(f"messages (B,4,H,W,Ls) and cost (B,H,W,Lc) disagree: {tuple(messages.shape)} / "
                       f"{tuple(cost.shape)}")
    L = min(Ls, Lc) if L is None else int(L)
    if L < 1 or L > min(Ls, Lc):
        raise BplError(f"L={L} outside the rows (messages {Ls}, cost {Lc})")
    for nm, t in (("messages", messages), ("cost", cost)):
        if t.dtype not in (torch.float32, torch.float16):
            raise BplError(f"{nm} must be float32 or float16")
    if out is None:
        out = torch.empty((B, H, W), dtype=out_dtype, device=messages.device)
    if out.dtype not in (torch.int64, torch.int32) or tuple(out.shape) != (B, H, W) or not out.is_contiguous():
        raise BplError("out must be a contiguous (B,H,W) int64 or int32 tensor")
    st = _timed("messages_argmin", lambda: lib().bpl_messages_argmin(
        _ptr(messages), int(messages.dtype == torch.float16), _ptr(cost), int(cost.dtype == torch.float16),
        _ptr(out), int(out.dtype == torch.int64), B, H, W, L, Ls, Lc, _stream(messages)))
    check(st, "bpl_messages_argmin")
    return out


def beliefs_infer(beliefs: torch.Tensor, mode: str = "wta", support: int = 3) -> torch.Tensor:
    """Inference on (B,H,W,L) beliefs: "wta" -> (B,H,W,1) int64 argmax,
    "sub-exp" -> (B,H,W,1) float expectation over the argmax's window."""
    _check_input("beliefs", beliefs, dim=4)
    B, H, W, L = beliefs.shape
    if mode not in ("wta", "sub-exp"):
        raise BplError(f"beliefs_infer mode must be wta or sub-exp, got {mode!r}")
    out = torch.empty((B, H, W, 1), dtype=torch.int64 if mode == "wta" else torch.float32, device=beliefs.device)
    st = _timed("beliefs_infer", lambda: lib().bpl_beliefs_infer(
        _ptr(beliefs), 0 if mode == "wta" else 1, int(support), _ptr(out), B, H, W, L, _stream(beliefs)))
    check(st, "bpl_beliefs_infer")
    return out


def pack_taps(affinities: torch.Tensor, offset: torch.Tensor) -> torch.Tensor:
    """(N,4,K,H,W) affinities + (N,4,H,W) offset -> (N,4,K+3,H,W) stereo
    jump taps, one kernel pass (message_passing_op_cuda.py:35-60)."""
    affinities = affinities.detach().float().contiguous()
    N, D, K, H, W = affinities.shape
    if D != 4:
        raise BplError(f"affinities must be (N,4,K,H,W), got {tuple(affinities.shape)}")
    offset = offset.detach().float().to(affinities.device).expand(N, 4, H, W).contiguous()
    _check_input("affinities", affinities, dim=5)
    taps = torch.empty((N, 4, K + 3, H, W), dtype=torch.float32, device=affinities.device)
    st = _timed("pack_taps", lambda: lib().bpl_pack_taps(
        _ptr(affinities), _ptr(offset), _ptr(taps), N, K, H, W, _stream(affinities)))
    check(st, "bpl_pack_taps")
    return taps


def unpack_tap_grad(grad_taps: torch.Tensor):
    """Gradient fold of pack_taps: (grad_affinities (N,4,K,H,W), grad_offset
    (N,4,H,W)), one kernel pass (message_passing_op_cuda.py:75-93)."""
    grad_taps = grad_taps.contiguous()
    _check_input("grad_taps", grad_taps, dim=5)
    N, D, Kp, H, W = grad_taps.shape
    gaff = torch.empty((N, 4, Kp - 3, H, W), dtype=torch.float32, device=grad_taps.device)
    goff = torch.empty((N, 4, H, W), dtype=torch.float32, device=grad_taps.device)
    st = _timed("unpack_tap_grad", lambda: lib().bpl_unpack_tap_grad(
        _ptr(grad_taps), _ptr(gaff), _ptr(goff), N, Kp - 3, H, W, _stream(grad_taps)))
    check(st, "bpl_unpack_tap_grad")
    return gaff, goff
