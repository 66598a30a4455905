"""Host-side mirror of the reference's stereo BP layer
(ops/lbp_stereo/message_passing_op_cuda.py, ops/lbp_stereo/inference_op.py,
ops/lbp_stereo/bp_op_cuda.py:130-210) on the GB300 kernels.

Same classes, argument meaning and results.  Differences, all without effect
on the values computed:
  * argmin indices are kept as uint8 (L <= 256) or int16 inside the autograd
    function instead of a float32 volume;
  * no torch.cuda.empty_cache() per iteration, and the default offset tensor
    is created on the device (the reference builds it on the host and copies
    it every iteration, message_passing_op_cuda.py:157-158).
"""
from __future__ import annotations

import torch
import torch.nn as nn
import torch.nn.functional as F

from .. import ops

# message slots (ops/lbp_stereo/src/util.cuh:7): slot k holds the message
# received from the neighbour on side k
LEFT, RIGHT, UP, DOWN = 0, 1, 2, 3


class TemperatureSoftmin(nn.Module):
    """softmin(x / T) along `dim` with a learnable temperature (corenet.py:106-113)."""

    def __init__(self, dim, init_temp=1.0, device=None):
        super().__init__()
        self.T = nn.Parameter(torch.ones(1, device=device).float() * init_temp, requires_grad=True)
        self.dim = dim

    def forward(self, x):
        return F.softmin(x / self.T, dim=self.dim)


class BeliefsSoftmin(torch.autograd.Function):
    """softmin((sum_k messages[:, k] + cost) / T) over the label axis, fused
    (message_passing_op_cuda.py:170-173 with TemperatureSoftmin,
    corenet.py:106-113): one kernel each way instead of the separate torch
    passes.  forward(messages (B,4,H,W,Ls) float or half, cost (B,H,W,L),
    T (1,)).  The gradient of z = sum + cost goes to the cost and, as a
    stride-0 view, to every message slot (no copy)."""

    @staticmethod
    def forward(ctx, messages, cost, T):
        cost = cost.contiguous()
        beliefs = ops.beliefs_forward(messages, cost, T)
        ctx.save_for_backward(messages, cost, T, beliefs)
        return beliefs

    @staticmethod
    def backward(ctx, grad_beliefs):
        messages, cost, T, beliefs = ctx.saved_tensors
        gz, gT = ops.beliefs_backward(messages, cost, T, beliefs, grad_beliefs, want_temperature=ctx.needs_input_grad[2])
        B, _, H, W, Ls = messages.shape
        L = cost.shape[-1]
        if messages.dtype == torch.float16:
            g1 = ops.to_half_padded(gz, L).unsqueeze(1)
        else:
            g1 = gz.unsqueeze(1)
        gm = g1.expand(B, 4, H, W, Ls)
        return gm, gz, (gT.view_as(T) if gT is not None else None)


def pack_affinities(affinities, offset):
    """(N,4,K,H,W) affinities [L2-, L2+, L1-, L1+, L3] (or [L1, L1, L2]) plus
    offset (N,4,H,W) -> (N,4,K+3,H,W) jump taps [offset, L3, L2-, L1-, 0, L1+,
    L2+, L3] with the reverse directions' +/- swapped
    (message_passing_op_cuda.py:35-60), in one kernel pass (ops.pack_taps)."""
    return ops.pack_taps(affinities, offset)


def unpack_affinity_grad(grad_taps):
    """Inverse of pack_affinities for the gradient (message_passing_op_cuda.py:75-93),
    in one kernel pass (ops.unpack_tap_grad).  Returns (grad_affinities
    (N,4,K,H,W), grad_offset (N,4,H,W))."""
    return ops.unpack_tap_grad(grad_taps)


class LBPMinSumFunction(torch.autograd.Function):
    """One LBP pass (message_passing_op_cuda.py:22-93).  forward(cost, edge,
    messages, delta, affinities, offset[, adjoint]) -> messages (updated in
    place, like the reference).

    adjoint "reference": the reference's backward, which uses the messages
    as they are when backward runs (the last pass's, for every pass) and
    returns in_grad as the message gradient.  adjoint "exact": the
    derivative of the forward; each pass keeps a copy of its own output
    messages and returns the gradient with respect to its input messages,
    so chained passes differentiate exactly.  (Argmin recomputation is an
    option of LBPMinSumLoop, which sees all passes of a call.)"""

    @staticmethod
    def forward(ctx, cost, edge, messages, delta, affinities, offset, adjoint="reference"):
        taps = pack_affinities(affinities, offset)
        L = cost.shape[-1]
        am_dtype = torch.uint8 if L <= 256 else torch.int16
        ctx.adjoint = adjoint
        ctx.leaf_messages = messages.is_leaf
        messages, argmin, scale = ops.lbp_forward(ops.LBP_STEREO, cost, taps, edge, messages, int(delta),
                                                  argmin_dtype=am_dtype)
        own = messages.clone() if adjoint == "exact" else messages
        ctx.save_for_backward(cost, taps, edge, own, argmin, scale)
        return messages

    @staticmethod
    def backward(ctx, in_grad):
        cost, taps, edge, messages, argmin, scale = ctx.saved_tensors
        gc, gtaps, ge, gm = ops.lbp_backward(ops.LBP_STEREO, taps, edge, in_grad.contiguous(), messages, argmin,
                                             scale, copy_grad_messages=False, mode=ctx.adjoint)
        g_aff, g_off = unpack_affinity_grad(gtaps)
        if ctx.leaf_messages and ctx.needs_input_grad[2]:
            gm = ops.leaf_message_grad(gm)
        return gc, ge, gm, None, g_aff, g_off, None


class LBPMinSumFunctionF16(torch.autograd.Function):
    """One LBP pass with FP16 storage of cost and messages (FP32 arithmetic).
    forward(cost, cost_h, edge, messages_h, delta, affinities, offset) with
    cost (N,H,W,L) float (the tensor the gradient is returned for), cost_h its
    half copy with the label axis padded to a multiple of 8, messages_h
    (N,4,H,W,Lp) half, updated in place like the float path."""

    @staticmethod
    def forward(ctx, cost, cost_h, edge, messages_h, delta, affinities, offset):
        taps = pack_affinities(affinities, offset)
        L = cost.shape[-1]
        am_dtype = torch.uint8 if L <= 256 else torch.int16
        messages_h, argmin, _ = ops.lbp_forward_f16(ops.LBP_STEREO, cost_h, taps, edge, messages_h, int(delta), L,
                                                    argmin_dtype=am_dtype)
        ctx.save_for_backward(taps, edge, messages_h, argmin)
        ctx.L = L
        ctx.leaf_messages = messages_h.is_leaf
        return messages_h

    @staticmethod
    def backward(ctx, in_grad):
        taps, edge, messages_h, argmin = ctx.saved_tensors
        gc, gtaps, ge = ops.lbp_backward_f16(ops.LBP_STEREO, taps, edge, in_grad.contiguous(), messages_h, argmin,
                                             None, ctx.L)
        g_aff, g_off = unpack_affinity_grad(gtaps)
        gm = ops.leaf_message_grad(in_grad) if ctx.leaf_messages and ctx.needs_input_grad[3] else in_grad
        return gc[..., :ctx.L], None, ge, gm, None, g_aff, g_off


class LBPMinSumLoop(torch.autograd.Function):
    """`iters` LBP passes run in place, as one autograd node.

    Reference adjoint: the reference's per-pass nodes
    (message_passing_op_cuda.py:161-168) each read the final, overwritten
    messages in backward and pass in_grad through as the message gradient,
    so their adjoints are independent of each other: here they run as one
    launch (bpl_lbp_backward_passes), which triples the scanlines of the
    latency-bound horizontal sweeps at 3 iterations.  Gradients equal the
    chained per-pass nodes'.  FP32 or FP16 storage (cost_h and messages
    half with the padded label axis).

    recompute=True stores no argmin indices.  The forward keeps only a copy
    of the initial messages' vertical slots (UP, DOWN): a pass reads its
    horizontal slots only where it has written them itself, except at the
    image borders no pass writes (LEFT at x=0, RIGHT at x=W-1), which the
    final messages still hold, so those two slots plus the final messages
    determine every pass exactly.  The backward re-runs the passes from that
    state, each warp regenerating its scanline's indices (bit-identical: the
    same kernel on the same inputs), and runs each pass's adjoint as soon as
    its indices exist.  Persistent memory: 2 slots of the initial messages
    in their storage type for the whole call (FP32: 8 B per pixel and
    label) instead of 4 argmin bytes per pixel and label per pass; the
    backward does `iters` forward passes more.  adjoint="exact" (FP32) runs
    the passes' exact adjoints in reverse from the re-run's outputs."""

    @staticmethod
    def forward(ctx, cost, cost_h, edge, messages, delta, affinities, offset, iters, adjoint="reference",
                recompute=False):
        taps = pack_affinities(affinities, offset)
        half = messages.dtype == torch.float16
        L = cost.shape[-1]
        B, _, H, W, Ls = messages.shape
        am_dtype = torch.uint8 if L <= 256 else torch.int16
        ctx.L, ctx.half, ctx.iters, ctx.delta = L, half, iters, int(delta)
        ctx.adjoint, ctx.recompute, ctx.am_dtype = adjoint, recompute, am_dtype
        ctx.leaf_messages = messages.is_leaf
        if recompute:
            vert0 = messages[:, UP:DOWN + 1].detach().clone()
            for _ in range(iters):
                if half:
                    ops.lbp_forward_f16(ops.LBP_STEREO, cost_h, taps, edge, messages, int(delta), L, argmin_dtype=None)
                else:
                    ops.lbp_forward(ops.LBP_STEREO, cost, taps, edge, messages, int(delta), argmin_dtype=None)
            ctx.save_for_backward(cost, cost_h, taps, edge, messages, vert0)
            return messages
        argmins = torch.empty((iters, B, 4, H, W, Ls), dtype=am_dtype, device=cost.device)
        # FP16: no scales (the adjoint normalises from the final rows)
        scales = None if half else torch.empty((iters, B, 4, H, W), dtype=torch.float32, device=cost.device)
        for k in range(iters):
            if half:
                ops.lbp_forward_f16(ops.LBP_STEREO, cost_h, taps, edge, messages, int(delta), L,
                                    argmin_dtype=am_dtype, argmin=argmins[k])
            else:
                ops.lbp_forward(ops.LBP_STEREO, cost, taps, edge, messages, int(delta), argmin_dtype=am_dtype,
                                argmin=argmins[k], scale=scales[k])
        ctx.save_for_backward(taps, edge, messages, argmins, scales)
        return messages

    @staticmethod
    def backward(ctx, in_grad):
        if ctx.recompute:
            gc, gtaps, ge, gm = LBPMinSumLoop._recompute_backward(ctx, in_grad)
        else:
            taps, edge, messages, argmins, scales = ctx.saved_tensors
            # in_grad as autograd hands it over: the beliefs' gradient expanded
            # over the four slots is read in place (slot stride 0), not materialised
            gc, gtaps, ge = ops.lbp_backward_passes(ops.LBP_STEREO, taps, edge, in_grad, messages, argmins, scales,
                                                    L=ctx.L)
            gm = in_grad
        g_aff, g_off = unpack_affinity_grad(gtaps)
        if ctx.half:
            gc = gc[..., :ctx.L]
        if ctx.leaf_messages and ctx.needs_input_grad[3]:
            gm = ops.leaf_message_grad(gm)
        return gc, None, ge, gm, None, g_aff, g_off, None, None, None

    @staticmethod
    def _recompute_backward(ctx, in_grad):
        cost, cost_h, taps, edge, messages, vert0 = ctx.saved_tensors
        half, L, delta = ctx.half, ctx.L, ctx.delta
        # the state before the first pass: the final messages with the
        # initial vertical slots back (see the class docstring)
        m = messages.detach().clone()
        m[:, UP:DOWN + 1] = vert0
        B, _, H, W, Ls = m.shape
        am = torch.empty((B, 4, H, W, Ls), dtype=ctx.am_dtype, device=m.device)
        sc = None if half else torch.empty((B, 4, H, W), device=m.device)
        ws = torch.empty(ops.lbp_backward_workspace_bytes(B, H, W, Ls), dtype=torch.uint8, device=m.device)
        gc = gtaps = ge = None

        def acc(a, b):
            return b if a is None else a.add_(b)
        if ctx.adjoint == "exact":
            # exact adjoints run in reverse and need every pass's own output:
            # keep them for the backward's duration (transient)
            outs = []
            for _ in range(ctx.iters):
                m, a_k, s_k = ops.lbp_forward(ops.LBP_STEREO, cost, taps, edge, m, delta, argmin_dtype=ctx.am_dtype)
                outs.append((m.clone(), a_k, s_k))
            g = in_grad.contiguous()
            for own, a_k, s_k in reversed(outs):
                c_k, t_k, e_k, g = ops.lbp_backward(ops.LBP_STEREO, taps, edge, g, own, a_k, s_k, workspace=ws,
                                                    copy_grad_messages=False, mode="exact")
                gc, gtaps, ge = acc(gc, c_k), acc(gtaps, t_k), acc(ge, e_k)
            return gc, gtaps, ge, g
        g_in = in_grad
        for _ in range(ctx.iters):
            if half:
                ops.lbp_forward_f16(ops.LBP_STEREO, cost_h, taps, edge, m, delta, L, argmin=am)
                c_k, t_k, e_k = ops.lbp_backward_passes(ops.LBP_STEREO, taps, edge, g_in, messages, am.unsqueeze(0),
                                                        None, L=L, workspace=ws)
            else:
                ops.lbp_forward(ops.LBP_STEREO, cost, taps, edge, m, delta, argmin_dtype=ctx.am_dtype, argmin=am,
                                scale=sc)
                c_k, t_k, e_k = ops.lbp_backward_passes(ops.LBP_STEREO, taps, edge, g_in, messages, am.unsqueeze(0),
                                                        sc.unsqueeze(0), L=L, workspace=ws)
            gc, gtaps, ge = acc(gc, c_k), acc(gtaps, t_k), acc(ge, e_k)
        return gc, gtaps, ge, in_grad


class BPLayerFn(torch.autograd.Function):
    """MessagePassing's passes and belief epilogue as one autograd node
    (reference adjoint, argmin indices stored), FP32 or FP16 storage.

    forward(prob_vol, edge, messages, affinities, offset, T, iters, delta)
    -> (beliefs, messages): cost = -prob_vol (message_passing_op_cuda.py:
    162), `iters` passes in place on messages (FP16: (N,4,H,W,Lp) half, the
    cost volume the half copy of -prob_vol), beliefs = softmin((sum + cost)
    / T) (:170-173, read from prob_vol with the sign folded in).  Values and
    gradients are those of the composition LBPMinSumLoop + BeliefsSoftmin
    (which the other modes run; the cost gradient up to the order of its
    float additions).  What the single node saves: the beliefs' backward
    writes its cost gradient negated into the buffer that becomes the
    probability volume's gradient, and the adjoint adds its own there with
    sign -1, so autograd's sum of the cost's two gradients and the
    negation's backward take no pass and the adjoint no zero-fill; the
    beliefs' backward also writes the adjoint's in_grad (for a leaf message
    tensor the materialised message gradient) in the same pass, and takes
    z/T for the temperature's gradient from the beliefs and one float per
    pixel the forward keeps, instead of re-reading messages and cost."""

    @staticmethod
    def forward(ctx, prob_vol, edge, messages, affinities, offset, T, iters, delta):
        ctx.set_materialize_grads(False)
        taps = pack_affinities(affinities, offset)
        half = messages.dtype == torch.float16
        prob = prob_vol.contiguous()
        B, H, W, L = prob.shape
        Ls = messages.shape[-1]
        am_dtype = torch.uint8 if L <= 256 else torch.int16
        cost = ops.half_padded(prob, -1.0) if half else -prob
        argmins = torch.empty((iters, B, 4, H, W, Ls), dtype=am_dtype, device=prob.device)
        # FP16: no scales (the adjoint normalises from the final rows)
        scales = None if half else torch.empty((iters, B, 4, H, W), dtype=torch.float32, device=prob.device)
        for k in range(iters):
            if half:
                ops.lbp_forward_f16(ops.LBP_STEREO, cost, taps, edge, messages, int(delta), L,
                                    argmin_dtype=am_dtype, argmin=argmins[k])
            else:
                ops.lbp_forward(ops.LBP_STEREO, cost, taps, edge, messages, int(delta), argmin_dtype=am_dtype,
                                argmin=argmins[k], scale=scales[k])
        lnorm = torch.empty((B, H, W), dtype=torch.float32, device=prob.device)
        beliefs = ops.beliefs_forward_any_cost(messages, prob, T, L, cost_sign=-1.0, log_norm=lnorm)
        ctx.save_for_backward(prob, taps, edge, messages, argmins, scales, T, beliefs, lnorm)
        ctx.half, ctx.L = half, L
        ctx.leaf_messages = messages.is_leaf
        return beliefs, messages

    @staticmethod
    def backward(ctx, grad_beliefs, grad_messages):
        prob, taps, edge, messages, argmins, scales, T, beliefs, lnorm = ctx.saved_tensors
        B, _, H, W, Ls = messages.shape
        need_m = ctx.needs_input_grad[2]
        if grad_beliefs is None:
            grad_beliefs = torch.zeros_like(beliefs)
        if ctx.half:
            kind = ops.BELIEF_COPY_HALF
        elif need_m and grad_messages is None:
            kind = ops.BELIEF_COPY_SLOTS
        else:
            kind = ops.BELIEF_COPY_FLOAT
        gprob, gcopy, gT = ops.beliefs_backward_fused(messages, prob, T, beliefs, grad_beliefs, -1.0, kind,
                                                      want_temperature=ctx.needs_input_grad[5], cost_sign=-1.0,
                                                      log_norm=lnorm)
        if grad_messages is not None:
            # the returned messages are used downstream too: their gradient
            # joins the beliefs' in every slot
            gin = (gcopy.float() + grad_messages.float()).to(messages.dtype).contiguous()
        elif kind == ops.BELIEF_COPY_SLOTS:
            gin = gcopy
        else:
            gin = gcopy.expand(B, 4, H, W, gcopy.shape[-1])
        # the packed taps of 3 affinities ([offset, L2, L1, 0, L1, L2]): the
        # adjoint bins for the fold below (taps 1 and 5 summed, tap 3 dropped)
        _, gtaps, ge = ops.lbp_backward_passes(ops.LBP_STEREO, taps, edge, gin, messages, argmins, scales, L=ctx.L,
                                               grad_cost_into=gprob, cost_sign=-1.0,
                                               layer_taps=taps.shape[2] == 6)
        g_aff, g_off = unpack_affinity_grad(gtaps)
        gm = None
        if need_m:
            gm = ops.leaf_message_grad(gin) if ctx.leaf_messages else gin
        return gprob, ge, gm, g_aff, g_off, (gT.view_as(T) if gT is not None else None), None, None


class MessagePassing(nn.Module):
    """message_passing_op_cuda.py:95-177.  storage="fp16" keeps the cost
    volume and the messages in half precision (label axis padded to a
    multiple of 8) with FP32 arithmetic; the returned messages are then the
    padded half tensor, each row stored relative to the minimum of h (a
    constant per pixel and direction away from the reference's normalised
    messages, which changes neither the beliefs' softmin nor a warm start)."""

    @property
    def L1(self):
        return self._L1

    @property
    def L2(self):
        return self._L2

    def setL1L2(self, value_L1, value_L2):
        if value_L1 > 0 and value_L2 > 0 and value_L1 <= value_L2:
            self._L1 = value_L1
            self._L2 = value_L2
        elif value_L1 < 0 or value_L2 < 0:
            raise ValueError("L1 or L2 is < 0!")
        elif value_L1 > value_L2:
            raise ValueError("L1 must be smaller than or equal L2!")

    def __init__(self, device, max_iter, num_labels, delta, mode="min-sum", storage="fp32", adjoint="reference",
                 recompute_argmin=False, fused=True):
        super().__init__()
        # fused: the reference adjoint with stored indices runs as one autograd
        # node (BPLayerFn); False keeps the composition of LBPMinSumLoop and
        # BeliefsSoftmin (the same values)
        self.fused = fused
        self.device = device
        self.max_iter = max_iter
        if mode != "min-sum":
            raise ValueError("Unknown message parsing mode " + mode)
        if storage not in ("fp32", "fp16"):
            raise ValueError("storage must be fp32 or fp16")
        if adjoint not in ("reference", "exact"):
            raise ValueError("adjoint must be reference or exact")
        if adjoint == "exact" and storage != "fp32":
            raise ValueError("the exact adjoint runs with fp32 storage")
        self.adjoint = adjoint
        self.recompute_argmin = recompute_argmin
        self.mode = mode
        self.storage = storage
        self._L1 = nn.Parameter(torch.tensor(0.1, device=device), requires_grad=True)
        self._L2 = nn.Parameter(torch.tensor(2.5, device=device), requires_grad=True)
        self.softmin = TemperatureSoftmin(dim=3, init_temp=1.0, device=device)
        self.delta = delta
        self.rescaleT = None

    def projectL1L2(self):
        self.L2.data = torch.max(self.L1.data, self.L2.data)

    def forward(self, prob_vol, edge_weights, affinities, offset, messages):
        N, H, W, C = prob_vol.shape
        dev = prob_vol.device
        if edge_weights is None:
            edge_weights = torch.ones((N, 4, H, W), device=dev)
        if affinities is None:
            if (self._L1 is not None) and (self._L2 is not None):
                affinities = torch.zeros((N, 4, 3, H, W), dtype=torch.float, device=dev)
                affinities[:, :, :2, :, :] = self._L1
                affinities[:, :, 2, :, :] = self._L2
        else:
            if (self._L1 is not None and self._L2 is None) or (self._L1 is None and self._L2 is not None):
                raise ValueError("L1 or L2 is None and affinities are not set!")
        if offset is None:
            offset = torch.zeros((N, 4, H, W), device=dev)
        fused = self.fused and self.adjoint == "reference" and not self.recompute_argmin and self.max_iter >= 1
        if fused and self.storage == "fp32":
            return BPLayerFn.apply(prob_vol, edge_weights, messages, affinities, offset, self.softmin.T,
                                   self.max_iter, self.delta)
        if self.storage == "fp16":
            if messages is None or messages.dtype != torch.float16:
                # a half copy of the caller's start (or zeros): no gradient
                # reaches the caller's float tensor through it, so none is kept
                m = torch.zeros((N, 4, H, W, ops.padded_labels(C)), dtype=torch.float16, device=dev)
                if messages is not None:
                    m[..., :C] = messages.detach()
                messages = m
            if fused:
                return BPLayerFn.apply(prob_vol, edge_weights, messages, affinities, offset, self.softmin.T,
                                       self.max_iter, self.delta)
            cost = -prob_vol
            cost_h = ops.to_half_padded(cost.detach(), C)
            messages = LBPMinSumLoop.apply(cost, cost_h, edge_weights, messages, self.delta, affinities, offset,
                                           self.max_iter, "reference", self.recompute_argmin)
            return BeliefsSoftmin.apply(messages, cost, self.softmin.T), messages
        cost = -prob_vol
        if self.adjoint == "reference" or self.recompute_argmin:
            messages = LBPMinSumLoop.apply(cost, None, edge_weights, messages, self.delta, affinities, offset,
                                           self.max_iter, self.adjoint, self.recompute_argmin)
        else:
            for _ in range(self.max_iter):
                messages = LBPMinSumFunction.apply(cost, edge_weights, messages, self.delta, affinities, offset,
                                                   self.adjoint)
        return BeliefsSoftmin.apply(messages, cost, self.softmin.T), messages


class Inference(nn.Module):
    """ops/lbp_stereo/inference_op.py:5-97: wta / expectation / norm / raw / sub-exp."""

    def __init__(self, device, mode="wta", mode_passing="min-sum"):
        super().__init__()
        if mode not in ("wta", "expectation", "norm", "raw", "sub-exp"):
            raise ValueError("Unknown inference mode " + mode)
        self.device = device
        self.mode = mode
        self.mode_passing = mode_passing

    def forward(self, beliefs):
        if self.mode == "wta":
            # one kernel pass (ops.beliefs_infer), the first index on ties like torch.argmax
            return ops.beliefs_infer(beliefs.detach().contiguous(), "wta")
        if self.mode == "expectation":
            bn = beliefs / beliefs.sum(dim=3, keepdim=True)
            labels = torch.arange(beliefs.shape[3], device=beliefs.device, dtype=torch.float32).view(1, 1, 1, -1)
            return (bn * labels).sum(dim=3, keepdim=True)
        if self.mode == "norm":
            return beliefs / beliefs.sum(dim=3, keepdim=True)
        if self.mode == "raw":
            return beliefs
        return self.compute_sub_expectation(beliefs)

    @staticmethod
    def compute_sub_expectation(beliefs, support=3):
        """+-support window around the argmax, renormalised expectation
        (inference_op.py:53-97).  Without a gradient to carry, one kernel pass
        (ops.beliefs_infer); with one, the torch form below (its gradient
        flows to the window's beliefs as in the reference)."""
        if not (beliefs.requires_grad and torch.is_grad_enabled()) and support <= 15:
            return ops.beliefs_infer(beliefs.contiguous(), "sub-exp", support)
        N, H, W, K = beliefs.shape
        disp = beliefs.argmax(dim=-1).unsqueeze(-1)
        win = torch.arange(-support, support + 1, device=beliefs.device) + disp
        win = win.clamp(0, K - 1)
        bw = torch.gather(beliefs, 3, win)
        bw = bw / bw.sum(dim=-1, keepdim=True)
        return torch.sum(bw * win, dim=-1, keepdim=True)


class BP(nn.Module):
    """ops/lbp_stereo/bp_op_cuda.py:80-127: MessagePassing plus Inference
    for a disparity volume (N,H,W,K) or a flow volume (N,2,H,W,K).

    The flow path is the reference's: u, then v, each from zero messages
    created with requires_grad, except that the v pass is handed the u
    pass's messages (bp_op_cuda.py:110 passes messages_u), which the u pass
    has updated in place, so v starts from u's final messages and both
    entries of the returned messages are that tensor after v.  With
    joint_flow=True the u and v volumes instead run as one batch of 2N items
    from zero messages each: one launch per kernel for both, twice the
    scanlines for the latency-bound sweeps; the results are those of two
    independent calls.  Checkpoint loading (SubNetwork) is not part of this
    module."""

    def __init__(self, device, args=None, max_iter=1, num_labels=None, delta=1, mode_inference="expectation",
                 mode_message_passing="min-sum", layer_idx=0, level=0, joint_flow=False, **mp_options):
        super().__init__()
        if mode_inference not in ("wta", "expectation", "norm", "raw", "sub-exp") or mode_message_passing != "min-sum":
            raise ValueError("Unknown inference/message passing mode " + mode_inference + " " + mode_message_passing)
        self.device = device
        self.max_iter = max_iter
        self.layer_idx = layer_idx
        self.level = level
        self.delta = delta
        self.joint_flow = joint_flow
        self.message_passing = MessagePassing(device, max_iter, num_labels, delta, mode_message_passing,
                                              **mp_options)
        self.inference = Inference(device, mode_inference, mode_passing=mode_message_passing)

    def _zeros(self, N, H, W, K):
        return torch.zeros((N, 4, H, W, K), requires_grad=True, device=self.device, dtype=torch.float)

    def forward(self, prob_vol, edge_weights, affinities=None, offsets=None):
        if prob_vol.dim() == 5:
            N, _, H, W, K = prob_vol.shape
            if self.joint_flow:
                pv = torch.cat((prob_vol[:, 0], prob_vol[:, 1]), dim=0).contiguous()
                twice = (lambda t: None if t is None else torch.cat((t, t), dim=0).contiguous())
                beliefs, messages = self.message_passing.forward(pv, twice(edge_weights), twice(affinities),
                                                                 twice(offsets), self._zeros(2 * N, H, W, K))
                result = self.inference.forward(beliefs)
                flow = torch.cat((result[:N], result[N:]), dim=-1).permute(0, 3, 1, 2)
                beliefs = torch.stack((beliefs[:N], beliefs[N:]), dim=1)
                messages = torch.stack((messages[:N], messages[N:]), dim=1)
                return flow, beliefs, messages
            messages_u = self._zeros(N, H, W, K)
            beliefs_u, messages_u = self.message_passing.forward(prob_vol[:, 0].contiguous(), edge_weights,
                                                                 affinities, offsets, messages_u)
            result_u = self.inference.forward(beliefs_u)
            beliefs_v, messages_v = self.message_passing.forward(prob_vol[:, 1].contiguous(), edge_weights,
                                                                 affinities, offsets, messages_u)
            result_v = self.inference.forward(beliefs_v)
            flow = torch.cat((result_u, result_v), dim=-1).permute(0, 3, 1, 2)
            beliefs = torch.cat((beliefs_u.unsqueeze(1), beliefs_v.unsqueeze(1)), dim=1)
            messages = torch.cat((messages_u.unsqueeze(1), messages_v.unsqueeze(1)), dim=1)
            return flow, beliefs, messages
        N, H, W, K = prob_vol.shape
        messages = self._zeros(N, H, W, K)
        beliefs, messages = self.message_passing.forward(prob_vol.contiguous(), edge_weights, affinities, offsets,
                                                         messages)
        result = self.inference.forward(beliefs)
        return result.permute(0, 3, 1, 2), beliefs, messages

    adjust_input_weights = staticmethod(lambda weights, idx: adjust_input_weights(weights, idx))
    adjust_input_affinities = staticmethod(lambda affinities: adjust_input_affinities(affinities))
    adjust_input_offsets = staticmethod(lambda offsets: adjust_input_offsets(offsets))

    def project_jumpcosts(self):
        self.message_passing.projectL1L2()


def coarse_to_fine(beliefs_in, pv_lvl):
    """The step between two BP levels of the stereo network (stereo.py:
    104-113): with the coarse beliefs requiring a gradient the reference only
    normalises the finer probability volume over its labels (the upsampled
    beliefs are dropped); otherwise it adds the beliefs, upsampled by 2
    trilinearly along rows, columns and labels and halved, in place, which
    is one kernel here.  Returns the volume for the finer level."""
    if beliefs_in is None:
        return pv_lvl
    if beliefs_in.requires_grad:
        return pv_lvl / pv_lvl.sum(dim=-1, keepdim=True)
    return ops.upsample_add_beliefs(beliefs_in.contiguous(), pv_lvl, 0.5)


def adjust_input_weights(weights, idx):
    """bp_op_cuda.py:130-154: (N,2,H,W) x/y weights -> (N,4,H,W) per direction."""
    if weights is None:
        return None
    out = torch.zeros((weights.shape[0], 4, weights.shape[2], weights.shape[3]), device=weights.device)
    out[:, 0] = weights[:, 0]
    out[:, 1, :, 1:] = weights[:, 0, :, :-1]
    out[:, 2] = weights[:, 1]
    out[:, 3, 1:, :] = weights[:, 1, :-1, :]
    return out.contiguous()


def adjust_input_affinities(affinities):
    """bp_op_cuda.py:156-188: order constraint then shift to 4 directions."""
    if affinities is None:
        return None
    a = affinities.clone()
    a[:, :, 0] = torch.max(affinities[:, :, 0], affinities[:, :, 2])
    a[:, :, 1] = torch.max(affinities[:, :, 1], affinities[:, :, 3])
    a[:, :, 4] = torch.max(affinities[:, :, 4], torch.max(a[:, :, 0].clone(), a[:, :, 1].clone()))
    s = torch.zeros((a.shape[0], a.shape[1] + 2, a.shape[2], a.shape[3], a.shape[4]), device=a.device)
    s[:, 0] = a[:, 0]
    s[:, 1, :, :, 1:] = a[:, 0, :, :, :-1]
    s[:, 2] = a[:, 1]
    s[:, 3, :, 1:, :] = a[:, 1, :, :-1, :]
    return s.contiguous()


def adjust_input_offsets(offsets):
    """bp_op_cuda.py:190-209."""
    if offsets is None:
        return None
    s = torch.zeros((offsets.shape[0], offsets.shape[1] + 2, offsets.shape[2], offsets.shape[3]), device=offsets.device)
    s[:, 0] = offsets[:, 0]
    s[:, 1, :, 1:] = -offsets[:, 0, :, :-1]
    s[:, 2] = offsets[:, 1]
    s[:, 3, 1:, :] = -offsets[:, 1, :-1, :]
    return s.contiguous()
