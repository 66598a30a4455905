"""The oracle's flow max-projected SAD at window sizes beyond the golden
fixtures (which stop at 9 labels), checked against a direct numpy statement
of the reference kernel (ops/flow_mp_sad/src/flow_mp_sad_kernel.cu:10-124):
float32 channel-ordered sums, 40 outside the image, rows v only up to
sws/2, first index on ties for both minima.  The GPU tests compare the
kernels with the oracle at these sizes."""
import numpy as np
import pytest

import cases
import oracle


def flow_numpy(f0, f1, sws, ou=0, ov=0, bu=0, bv=0):
    B, C, H, W = f0.shape
    K, hs = sws + 1, sws // 2
    out = [np.empty((B, H, W, K), np.float32) for _ in range(4)]
    for n in range(B):
        for y in range(H):
            for x in range(W):
                win = np.full((K, K), 40.0, np.float32)  # [v_idx][u_idx]
                xm = x + ou + np.arange(K) - hs
                okx = (xm >= 0) & (xm < W)
                for vi in range(2 * hs + 1):
                    ym = y + ov + vi - hs
                    if ym < 0 or ym >= H or not okx.any():
                        continue
                    s = np.zeros(int(okx.sum()), np.float32)
                    for c in range(C):
                        d = (f0[n, c, y, x] - f1[n, c, ym, xm[okx]]).astype(np.float32)
                        s = (s + np.abs(d)).astype(np.float32)
                    win[vi, okx] = s
                au = np.argmin(win, axis=0)  # over v for each u: first index
                av = np.argmin(win, axis=1)  # over u for each v
                out[0][n, y, x] = win[au, np.arange(K)]
                out[1][n, y, x] = win[np.arange(K), av]
                out[2][n, y, x] = au + bv * sws
                out[3][n, y, x] = av + bu * sws
    return out


@pytest.mark.parametrize("sws,ou,ov,bu,bv,q", [(64, 0, 0, 0, 0, None), (65, 3, -2, 1, 0, 2), (216, 0, 0, 0, 0, None),
                                              (216, -54, 54, 0, 1, 2), (255, 0, 0, 0, 0, None)])
def test_oracle_flow_forward_large_windows(sws, ou, ov, bu, bv, q):
    g = cases.rng(70 + sws)
    B, C, H, W = 1, 2, 3, 26
    f0 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    f1 = g.normal(0, 1, size=(B, C, H, W)).astype(np.float32)
    if q:
        f0 = (np.round(f0 * q) / q).astype(np.float32)
        f1 = (np.round(f1 * q) / q).astype(np.float32)
    got = oracle.flow_forward(f0, f1, sws, ou, ov, bu, bv)
    ref = flow_numpy(f0, f1, sws, ou, ov, bu, bv)
    for nm, a, b in zip(("cv_u", "cv_v", "u_star", "v_star"), got, ref):
        np.testing.assert_array_equal(a, b, err_msg=nm)
