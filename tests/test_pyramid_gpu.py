"""Coarse-to-fine glue (stereo.py:104-113) on the GPU against torch's own
F.interpolate(..., scale_factor=2.0, mode='trilinear') + add: the weights
are exact multiples of 1/4, so values agree to the rounding of the few
products and sums (torch's kernel may contract them into FMAs); tolerance
2 ulp-scale, 1e-6 relative to the volume's magnitude."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("shape", [(1, 5, 7, 6), (2, 3, 4, 24), (1, 1, 1, 1), (1, 12, 20, 48)])
def test_upsample_add_matches_torch(shape):
    import torch.nn.functional as F
    from bpl_gb300.layers.stereo import coarse_to_fine
    dev = torch.device("cuda:0")
    g = cases.rng(41)
    N, h, w, d = shape
    b = torch.from_numpy(cases.softmax_np(g.normal(0, 2, size=shape).astype(np.float32))).to(dev)
    pv = torch.from_numpy(cases.softmax_np(g.normal(0, 2, size=(N, 2 * h, 2 * w, 2 * d)).astype(np.float32))).to(dev)
    ref = pv + F.interpolate(b.unsqueeze(1), scale_factor=2.0, mode="trilinear")[:, 0] / 2.0
    out = coarse_to_fine(b, pv.clone())
    tol = 1e-6 * float(ref.abs().max())
    assert float((out - ref).abs().max()) <= tol


def test_coarse_to_fine_with_gradient_normalises():
    from bpl_gb300.layers.stereo import coarse_to_fine
    dev = torch.device("cuda:0")
    b = torch.rand((1, 3, 4, 5), device=dev, requires_grad=True)
    pv = torch.rand((1, 6, 8, 10), device=dev)
    out = coarse_to_fine(b, pv)
    assert torch.allclose(out.sum(-1), torch.ones_like(out.sum(-1)))
