"""ctypes front end of the CPU oracle (oracle/bpl_oracle.cpp).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always as the test reference or the timed CPU
baseline, never as a code path of the product.

Each function mirrors one reference op (file:line citations are in
bpl_oracle.cpp) on numpy arrays and returns numpy arrays.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bpl_oracle.cpp")
LIB = os.path.join(HERE, "_build", "libbpl_oracle.so")

VAR_STEREO, VAR_SEM_GLOBAL, VAR_SEM_PIXEL = 0, 1, 2

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-ffp-contract=off keeps float arithmetic
    exactly as written; the sources call fmaf where the reference contracts)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
                               "-ffp-contract=off", "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def lbp_forward(variant, cost, jump, edge, messages, delta, *, all_batches=True, fp64=False,
                threads=0, iters=1, want_argmin=True):
    """Runs `iters` calls of forward_minsum, messages updated in place between
    calls as the reference does.  Returns (messages, argmin, scale) of the
    last call (argmin as float32, like the reference)."""
    B, H, W, L = cost.shape
    if variant == VAR_STEREO:
        Lv, jb = jump.shape[2], jump.shape[0]
    else:
        Lv, jb = 0, 1
    eb = edge.shape[0]
    conv = _f64 if fp64 else _f32
    c, j, e = conv(cost), conv(jump), conv(edge)
    m = conv(messages).copy()
    am = np.zeros((B, 4, H, W, L), np.float32) if want_argmin else None
    for _ in range(iters):
        sc = np.zeros((B, 4, H, W), np.float64 if fp64 else np.float32)
        if want_argmin:
            am[...] = 0
        fn = lib().oracle_lbp_forward_f64 if fp64 else lib().oracle_lbp_forward_f32
        fn(ctypes.c_int(variant), _p(c), _p(j), _p(e), _p(m), _p(am), _p(sc),
           *[ctypes.c_int(v) for v in (B, H, W, L, Lv, jb, eb, int(delta), int(all_batches), threads)])
    return m, am, sc


def lbp_backward_ref(variant, jump, edge, in_grad, messages, argmin, scale, *, threads=0,
                     batch=None):
    """Reference adjoint with double accumulation.  Returns
    (grad_cost, grad_jump, grad_edge, grad_messages) as float64."""
    B, _, H, W, L = messages.shape
    if variant == VAR_STEREO:
        Lv, jb = jump.shape[2], jump.shape[0]
        gj = np.zeros((B, 4, Lv, H, W))
    elif variant == VAR_SEM_GLOBAL:
        Lv, jb = 0, 1
        gj = np.zeros((B, 4, L, L))
    else:
        Lv, jb = 0, 1
        gj = np.zeros((4, H, W, L, L))
    eb = edge.shape[0]
    gc = np.zeros((B, H, W, L))
    ge = np.zeros((B, 4, H, W))
    gm = np.zeros((B, 4, H, W, L))
    lib().oracle_lbp_backward_ref(
        ctypes.c_int(variant), _p(_f32(jump)), _p(_f32(edge)), _p(_f32(in_grad)), _p(_f32(messages)),
        _p(_f32(argmin)), _p(_f32(scale)), _p(gc), _p(gj), _p(ge), _p(gm),
        *[ctypes.c_int(v) for v in (B, H, W, L, Lv, jb, eb, threads)])
    return gc, gj, ge, gm


def lbp_backward_exact(variant, jump, edge, in_grad, messages, argmin, scale, *, fp64=False, threads=0):
    """Exact adjoint of one pass (the reverse-mode derivative of the forward
    as written), from that pass's outputs (messages, argmin, scale) in float
    (fp64=False) or double (fp64=True).  Returns (grad_cost, grad_jump,
    grad_edge, grad_messages) as float64, grad_messages with respect to the
    pass's input messages."""
    B, _, H, W, L = messages.shape
    if variant == VAR_STEREO:
        Lv, jb = jump.shape[2], jump.shape[0]
        gj = np.zeros((B, 4, Lv, H, W))
    elif variant == VAR_SEM_GLOBAL:
        Lv, jb = 0, 1
        gj = np.zeros((B, 4, L, L))
    else:
        Lv, jb = 0, 1
        gj = np.zeros((4, H, W, L, L))
    eb = edge.shape[0]
    gc = np.zeros((B, H, W, L))
    ge = np.zeros((B, 4, H, W))
    gm = np.zeros((B, 4, H, W, L))
    conv = _f64 if fp64 else _f32
    fn = lib().oracle_lbp_backward_exact_f64 if fp64 else lib().oracle_lbp_backward_exact_f32
    fn(ctypes.c_int(variant), _p(conv(jump)), _p(conv(edge)), _p(conv(in_grad)), _p(conv(messages)),
       _p(_f32(argmin)), _p(conv(scale)), _p(gc), _p(gj), _p(ge), _p(gm),
       *[ctypes.c_int(v) for v in (B, H, W, L, Lv, jb, eb, threads)])
    return gc, gj, ge, gm


def sad_forward(f0, f1, min_disp, max_disp, step=1.0, *, all_batches=True, threads=0):
    B, C, H, W = f0.shape
    D = int((max_disp - min_disp + 1) / step)
    out = np.empty((B, H, W, D), np.float32)
    lib().oracle_sad_forward(_p(_f32(f0)), _p(_f32(f1)), _p(out), *[ctypes.c_int(v) for v in (B, C, H, W, min_disp, max_disp)],
                             ctypes.c_float(step), ctypes.c_int(int(all_batches)), ctypes.c_int(threads))
    return out


def sad_backward(f0, f1, in_grad, min_disp, max_disp, *, all_batches=True, channel_limit=None,
                 threads=0):
    B, C, H, W = f0.shape
    df0 = np.empty_like(_f32(f0))
    df1 = np.empty_like(_f32(f1))
    cl = C if channel_limit is None else channel_limit
    lib().oracle_sad_backward(_p(_f32(f0)), _p(_f32(f1)), _p(_f32(in_grad)), _p(df0), _p(df1),
                              *[ctypes.c_int(v) for v in (B, C, H, W, min_disp, max_disp, int(all_batches), cl, threads)])
    return df0, df1


def flow_forward(f0, f1, sws, offset_u=0, offset_v=0, block_u=0, block_v=0, *, all_batches=True,
                 threads=0):
    B, C, H, W = f0.shape
    K = sws + 1
    outs = [np.empty((B, H, W, K), np.float32) for _ in range(4)]
    lib().oracle_flow_forward(_p(_f32(f0)), _p(_f32(f1)), *[_p(o) for o in outs],
                              *[ctypes.c_int(v) for v in (B, C, H, W, sws, offset_u, offset_v, block_u, block_v, int(all_batches), threads)])
    return tuple(outs)


def flow_backward(f0, f1, sws, in_grad_u, in_grad_v, u_star, v_star, *, all_batches=True):
    B, C, H, W = f0.shape
    df0 = np.empty((B, C, H, W), np.float32)
    df1 = np.empty((B, C, H, W), np.float64)
    lib().oracle_flow_backward(_p(_f32(f0)), _p(_f32(f1)), _p(_f32(in_grad_u)), _p(_f32(in_grad_v)),
                               _p(_f32(u_star)), _p(_f32(v_star)), _p(df0), _p(df1),
                               *[ctypes.c_int(v) for v in (B, C, H, W, sws, int(all_batches))])
    return df0, df1
