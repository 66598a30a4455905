"""The serving loop on the GPU: every request's disparity map is the same
when it is served in a mixed, continuously batched stream (graphs, several
shapes overlapping) as when it runs alone with plain launches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _requests(dev, n, shapes, C, seed=1, rate=400.0):
    from bpl_gb300 import serving
    g = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for i in range(n):
        t += g.exponential(1.0 / rate)
        H, W, D = shapes[g.integers(len(shapes))]
        f0, f1 = serving.synth_request_features(H, W, D, C, seed=100 + i, device=dev)
        reqs.append(serving.StereoRequest(i, f0, f1, D, arrival=t))
    return reqs


def test_served_mix_matches_each_request_alone():
    from bpl_gb300 import serving
    dev = torch.device("cuda:0")
    shapes = [(48, 64, 32), (40, 80, 48), (56, 72, 64)]
    C = 16
    reqs = _requests(dev, 14, shapes, C)
    alone = serving.run_plain([serving.StereoRequest(r.rid, r.f0, r.f1, r.D, 0.0) for r in reqs], realtime=False)
    ref = {r.rid: r.disparity.cpu() for r in alone}
    eng = serving.ServingEngine(shapes, C=C, max_batch=3, budget_bytes=2 << 30, max_sets_per_shape=2, device=dev)
    eng.warm_up()
    done = eng.serve(reqs)
    assert sorted(r.rid for r in done) == list(range(len(reqs)))
    for r in done:
        assert torch.equal(r.disparity.cpu(), ref[r.rid]), f"request {r.rid} differs in the mix"
    # and without graphs (eager batches) the same
    reqs2 = [serving.StereoRequest(r.rid, r.f0, r.f1, r.D, r.arrival) for r in reqs]
    for r in eng.serve(reqs2, use_graphs=False, realtime=False):
        assert torch.equal(r.disparity.cpu(), ref[r.rid])
    st = serving.latency_stats(done)
    assert st["p50_ms"] is not None and st["p99_ms"] >= st["p50_ms"]


def test_disparity_recovers_the_planar_scene():
    """Sanity of the served pipeline itself: on the synthetic scene most
    pixels away from the left border get the generating disparity."""
    from bpl_gb300 import serving
    dev = torch.device("cuda:0")
    H, W, D, C = 64, 160, 32, 32
    f0, f1 = serving.synth_request_features(H, W, D, C, seed=5, device=dev)
    r = serving.run_plain([serving.StereoRequest(0, f0, f1, D)], realtime=False)[0]
    # the SAD at disparity d compares left x with right x - d; the right
    # image is the left one warped by the scene, so a correct d matches the
    # features up to the N(0, 0.1) noise
    f0c, f1c = f0.cpu().numpy(), f1.cpu().numpy()
    disp = r.disparity.cpu().numpy()
    xs = np.arange(D, W)
    ok = []
    for y in range(H):
        d = disp[y, D:]
        ok.append(np.abs(f0c[:, y, xs] - f1c[:, y, xs - d]).mean(0) < 0.2)
    assert np.mean(ok) > 0.8
