"""Host logic of the serving loop (no GPU): slot-set planning under an HBM
budget and the latency statistics."""
import pytest

torch = pytest.importorskip("torch")

from bpl_gb300 import serving  # noqa: E402


def test_plan_fits_budget_and_serves_every_shape():
    shapes = [(376, 1240, 128), (540, 960, 192), (720, 1280, 256)]
    per = {s: serving.slot_bytes(*s, 64) for s in shapes}
    for budget_gb in (25, 60, 140):
        budget = budget_gb << 30
        plan = serving.plan_slot_sets(shapes, [0.5, 0.3, 0.2], 64, 4, budget)
        assert set(plan) == set(shapes)
        used = sum(per[s] * n * c for s, (n, c) in plan.items())
        assert used <= budget
        for s, (n, c) in plan.items():
            assert n >= 1 and 1 <= c <= 4
    # a larger budget never shrinks a shape's capacity
    small = serving.plan_slot_sets(shapes, [0.5, 0.3, 0.2], 64, 4, 25 << 30)
    big = serving.plan_slot_sets(shapes, [0.5, 0.3, 0.2], 64, 4, 140 << 30)
    for s in shapes:
        assert big[s][0] * big[s][1] >= small[s][0] * small[s][1]


def test_plan_rejects_budget_below_one_request_per_shape():
    shapes = [(720, 1280, 256), (540, 960, 192)]
    need = sum(serving.slot_bytes(*s, 64) for s in shapes)
    with pytest.raises(MemoryError):
        serving.plan_slot_sets(shapes, [1, 1], 64, 4, need - 1)


def test_latency_stats_percentiles():
    reqs = []
    for i in range(100):
        r = serving.StereoRequest(i, torch.zeros(1, 1, 1), torch.zeros(1, 1, 1), 1, arrival=i * 0.01)
        r.t_done = r.arrival + (i + 1) * 1e-3  # latencies 1..100 ms
        reqs.append(r)
    st = serving.latency_stats(reqs)
    assert abs(st["p50_ms"] - 50.0) < 1e-6
    assert abs(st["p99_ms"] - 99.0) < 1e-6
    assert st["requests_per_s"] == pytest.approx(100 / (reqs[-1].t_done - 0.0))
