"""The oracle's stereo SAD beyond the golden fixtures (which stop at 12
disparities), against direct numpy statements of the reference kernels
(ops/sad/src/stereo_sad_kernel.cu:16-108): float32 channel-ordered sums,
d = (int)(di * step + min_disp) in float, 40 where x - d is outside the
row; the backward's sign gather summed over d in order, |diff| <= 1e-15
skipped.  The GPU tests compare the kernels with the oracle at these
sizes."""
import numpy as np
import pytest

import cases
import oracle


def sad_forward_numpy(f0, f1, lo, hi, step):
    B, C, H, W = f0.shape
    D = int(np.float32(hi - lo + 1) / np.float32(step))
    out = np.full((B, H, W, D), 40.0, np.float32)
    xs = np.arange(W)
    for di in range(D):
        d = int(np.trunc(np.float32(np.float32(di) * np.float32(step)) + np.float32(lo)))
        ok = (xs - d >= 0) & (xs - d < W)
        if not ok.any():
            continue
        s = np.zeros((B, H, int(ok.sum())), np.float32)
        for c in range(C):
            s = (s + np.abs((f0[:, c][:, :, ok] - f1[:, c][:, :, xs[ok] - d]).astype(np.float32))).astype(np.float32)
        out[:, :, ok, di] = s
    return out


def sad_backward_numpy(f0, f1, g, lo, hi):
    B, C, H, W = f0.shape
    df0 = np.zeros_like(f0)
    df1 = np.zeros_like(f1)
    xs = np.arange(W)
    for d in range(lo, hi + 1):
        i = d - lo
        a = (xs - d >= 0) & (xs - d < W)  # df0 term at x
        if a.any():
            diff = (f0[:, :, :, a] - f1[:, :, :, xs[a] - d]).astype(np.float32)
            t = np.where(diff > 0, 1.0, -1.0).astype(np.float32) * g[:, None, :, a, i]
            df0[:, :, :, a] = np.where(np.abs(diff) > 1e-15, (df0[:, :, :, a] + t).astype(np.float32), df0[:, :, :, a])
        b = (xs + d >= 0) & (xs + d < W)  # df1 term at x
        if b.any():
            diff = (f0[:, :, :, xs[b] + d] - f1[:, :, :, b]).astype(np.float32)
            t = np.where(diff > 0, 1.0, -1.0).astype(np.float32) * g[:, None, :, xs[b] + d, i]
            df1[:, :, :, b] = np.where(np.abs(diff) > 1e-15, (df1[:, :, :, b] - t).astype(np.float32), df1[:, :, :, b])
    return df0, df1


@pytest.mark.parametrize("lo,hi,step,q", [(0, 191, 1.0, None), (-40, 215, 1.0, 2), (0, 255, 1.0, None),
                                          (3, 120, 0.5, None), (-7, 60, 0.75, 4)])
def test_oracle_sad_forward_wide(lo, hi, step, q):
    g = cases.rng(80 + hi)
    B, C, H, W = 1, 5, 3, 300
    f0 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    f1 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    if q:
        f0 = (np.round(f0 * q) / q).astype(np.float32)
        f1 = (np.round(f1 * q) / q).astype(np.float32)
    np.testing.assert_array_equal(oracle.sad_forward(f0, f1, lo, hi, step), sad_forward_numpy(f0, f1, lo, hi, step))


@pytest.mark.parametrize("lo,hi,q", [(0, 191, None), (-40, 215, 2), (5, 255, None)])
def test_oracle_sad_backward_wide(lo, hi, q):
    g = cases.rng(90 + hi)
    B, C, H, W = 1, 4, 2, 280
    f0 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    f1 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    if q:
        f0 = (np.round(f0 * q) / q).astype(np.float32)
        f1 = (np.round(f1 * q) / q).astype(np.float32)
    gin = g.normal(0, 1, size=(B, H, W, hi - lo + 1)).astype(np.float32)
    got0, got1 = oracle.sad_backward(f0, f1, gin, lo, hi)
    ref0, ref1 = sad_backward_numpy(f0, f1, gin, lo, hi)
    np.testing.assert_array_equal(got0, ref0)
    np.testing.assert_array_equal(got1, ref1)
