"""Seeded input generators shared by the golden-fixture script, the tests,
the smoke check and the benchmark.

All generators use numpy's platform-independent PCG64 stream so that the same
seed gives the same bytes on x86 and on aarch64.  Where a value goes through a
transcendental function (softmax of a SAD volume) the result is stored in the
fixture rather than regenerated, because vectorised exp/log differ across
platforms in the last bit.

Shapes follow the reference ops:
  cost (B,H,W,L); messages (B,4,H,W,L); edge (B,4,H,W);
  stereo jump taps (B,4,Lv,H,W) with tap order [offset, L3, L2-, L1-, 0, L1+, L2+, L3]
  (Lv=8) or [offset, L2, L1, 0, L1, L2] (Lv=6)  (ops/lbp_stereo/message_passing_op_cuda.py:35-59,
  :149-151); semantic global jump (1,4,L,L); semantic pixel jump (4,H,W,L,L).
"""
from __future__ import annotations

import numpy as np

LEFT, RIGHT, UP, DOWN = 0, 1, 2, 3


def rng(seed: int) -> np.random.Generator:
    return np.random.default_rng(seed)


def softmax_np(x: np.ndarray, axis: int = -1) -> np.ndarray:
    x = x.astype(np.float64)
    x = x - x.max(axis=axis, keepdims=True)
    e = np.exp(x)
    return (e / e.sum(axis=axis, keepdims=True)).astype(np.float32)


def stereo_taps(B, H, W, L1=0.1, L2=0.5, Lv=6, offset=None):
    """Scalar truncated-linear pairwise packed as the reference packs it:
    Lv=6 -> [off, L2, L1, 0, L1, L2]."""
    if Lv != 6:
        raise ValueError("scalar taps use Lv=6")
    j = np.zeros((B, 4, 6, H, W), np.float32)
    j[:, :, 1] = L2
    j[:, :, 2] = L1
    j[:, :, 3] = 0.0
    j[:, :, 4] = L1
    j[:, :, 5] = L2
    if offset is not None:
        j[:, :, 0] = offset
    return j


def random_taps8(g, B, H, W, offset_scale=0.0):
    """Per-pixel affinity taps as AffinityNet produces them: 5 positive
    values (L2-, L2+, L1-, L1+, L3) made monotone the way
    BP.adjust_input_affinities does (ops/lbp_stereo/bp_op_cuda.py:156-170),
    then packed to 8 taps per direction."""
    a = g.uniform(0.05, 1.5, size=(B, 4, 5, H, W)).astype(np.float32)
    a[:, :, 0] = np.maximum(a[:, :, 0], a[:, :, 2])
    a[:, :, 1] = np.maximum(a[:, :, 1], a[:, :, 3])
    a[:, :, 4] = np.maximum(a[:, :, 4], np.maximum(a[:, :, 0], a[:, :, 1]))
    j = np.zeros((B, 4, 8, H, W), np.float32)
    if offset_scale:
        j[:, :, 0] = g.uniform(-offset_scale, offset_scale, size=(B, 4, H, W)).astype(np.float32)
    j[:, :, 1] = a[:, :, 4]
    j[:, :, 7] = a[:, :, 4]
    j[:, :, 4] = 0.0
    # i = 2,3 : (in_count, in_count+1) = (0,1), (2,3)
    for i, ic in ((2, 0), (3, 2)):
        j[:, 0::2, i] = a[:, 0::2, ic]
        j[:, 0::2, 8 - i] = a[:, 0::2, ic + 1]
        j[:, 1::2, i] = a[:, 1::2, ic + 1]
        j[:, 1::2, 8 - i] = a[:, 1::2, ic]
    return j


def random_cost(g, B, H, W, L, quantise=None):
    """cost = -softmax(scores) as in MessagePassing.forward (cost = -prob_vol).
    With `quantise`, values are rounded to multiples of 1/quantise, which
    makes exact ties in h and in the window candidates frequent."""
    s = g.normal(0.0, 2.0, size=(B, H, W, L)).astype(np.float32)
    c = -softmax_np(s, axis=-1)
    if quantise:
        c = (np.round(c * quantise) / quantise).astype(np.float32)
    return c


def random_messages(g, B, H, W, L, scale=1.0, quantise=None):
    m = (-np.abs(g.normal(0.0, scale, size=(B, 4, H, W, L)))).astype(np.float32)
    if quantise:
        m = (np.round(m * quantise) / quantise).astype(np.float32)
    return m


def edge_weights(g, B, H, W, kind="lognormal", quantise=None):
    if kind == "ones":
        e = np.ones((B, 4, H, W), np.float32)
    elif kind == "uniform":
        e = g.uniform(0.5, 2.0, size=(B, 4, H, W)).astype(np.float32)
    else:
        e = np.exp(g.normal(0.0, 0.3, size=(B, 4, H, W))).astype(np.float32)
    if quantise:
        e = (np.round(e * quantise) / quantise).astype(np.float32)
    return e


def semantic_global_jump(g, L, quantise=None):
    """(1,2,L,L) pairwise -> (1,4,L,L) per direction the way the semantic
    wrapper builds it: [P_x, P_x^T, P_y, P_y^T]
    (ops/lbp_semantic_pw/message_passing_op_cuda.py:28-33)."""
    p = g.uniform(0.2, 1.5, size=(1, 2, L, L)).astype(np.float32)
    p = 0.5 * (p + p.transpose(0, 1, 3, 2))
    for k in range(2):
        np.fill_diagonal(p[0, k], 0.0)
    if quantise:
        p = (np.round(p * quantise) / quantise).astype(np.float32)
    j = np.zeros((1, 4, L, L), np.float32)
    j[0, 0] = p[0, 0]
    j[0, 2] = p[0, 1]
    j[0, 1] = p[0, 0].T
    j[0, 3] = p[0, 1].T
    return np.ascontiguousarray(j), p


def semantic_pixel_jump(g, H, W, L):
    """(2,H,W,L,L) -> shifted/transposed (4,H,W,L,L) as the pixel wrapper does
    (ops/lbp_semantic_pw_pixel/message_passing_op_pw_pixel.py:147-156)."""
    base = g.uniform(0.2, 1.5, size=(L, L)).astype(np.float32)
    base = 0.5 * (base + base.T)
    np.fill_diagonal(base, 0.0)
    sc = np.exp(g.normal(0.0, 0.3, size=(2, H, W, 1, 1))).astype(np.float32)
    jp = (base[None, None, None] * sc).astype(np.float32)
    j = np.zeros((4, H, W, L, L), np.float32)
    j[0] = jp[0]
    j[1, :, 1:] = jp[0, :, :-1].transpose(0, 1, 3, 2)
    j[2] = jp[1]
    j[3, 1:] = jp[1, :-1].transpose(0, 1, 3, 2)
    return np.ascontiguousarray(j), jp


# ---------------------------------------------------------------------------
# Stereo scene synthesis (piecewise-planar disparity, warped features)

def planar_disparity(g, H, W, D, planes=6):
    ys, xs = np.mgrid[0:H, 0:W].astype(np.float64)
    cy = g.uniform(0, H, size=planes)
    cx = g.uniform(0, W, size=planes)
    base = g.uniform(0.1 * D, 0.9 * D, size=planes)
    ax = g.uniform(-0.15, 0.15, size=planes) * D / max(W, 1)
    ay = g.uniform(-0.15, 0.15, size=planes) * D / max(H, 1)
    dist = (ys[None] - cy[:, None, None]) ** 2 + (xs[None] - cx[:, None, None]) ** 2
    lab = np.argmin(dist, axis=0)
    disp = base[lab] + ax[lab] * (xs - cx[lab]) + ay[lab] * (ys - cy[lab])
    return np.clip(disp, 0, D - 1).astype(np.float32)


def stereo_features(g, B, C, H, W, D):
    """Left features ~N(0,1); right features = left warped by a
    piecewise-planar disparity + N(0,0.1).  Returns f0, f1 (B,C,H,W), disp."""
    f0 = g.normal(0.0, 1.0, size=(B, C, H, W)).astype(np.float32)
    f1 = np.empty_like(f0)
    disps = np.empty((B, H, W), np.float32)
    xs = np.arange(W)
    for b in range(B):
        disp = planar_disparity(g, H, W, D)
        disps[b] = disp
        src = np.clip(xs[None, :] + np.round(disp).astype(np.int64), 0, W - 1)
        f1[b] = np.take_along_axis(f0[b], np.broadcast_to(src[None], (C, H, W)), axis=2)
    f1 += g.normal(0.0, 0.1, size=f1.shape).astype(np.float32)
    return f0, f1.astype(np.float32), disps


def sad_volume_np(f0, f1, min_disp, max_disp):
    """float32 SAD in channel order, 40 outside (for input synthesis)."""
    B, C, H, W = f0.shape
    D = max_disp - min_disp + 1
    out = np.full((B, H, W, D), 40.0, np.float32)
    for di in range(D):
        d = di + min_disp
        lo, hi = max(d, 0), min(W, W + d)
        if hi <= lo:
            continue
        acc = np.zeros((B, H, hi - lo), np.float32)
        for c in range(C):
            acc += np.abs(f0[:, c, :, lo:hi] - f1[:, c, :, lo - d:hi - d])
        out[:, :, lo:hi, di] = acc
    return out


def stereo_cost_from_scene(g, B, H, W, C, D, T=1.0):
    """SAD -> softmax(-SAD/T) -> cost = -prob (matching.py:22-25 ->
    message_passing_op_cuda.py:162)."""
    f0, f1, disp = stereo_features(g, B, C, H, W, D)
    sad = sad_volume_np(f0, f1, 0, D - 1)
    prob = softmax_np(-sad / T, axis=-1)
    return (-prob).astype(np.float32), f0, f1, disp
