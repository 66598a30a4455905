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


# ---------------------------------------------------------------------------
# The scheduler's failure handling, on fake slot sets (no GPU): a fake set
# finishes a batch `service` seconds after it was launched, on a simulated
# clock.

class _Clock:
    def __init__(self):
        self.t = 0.0


class FakeSet:
    def __init__(self, clock, cap=2, service=1.0):
        self.clock, self.cap, self.service = clock, cap, service
        self.reqs, self.t_end, self.batches = [], None, []

    @property
    def busy(self):
        return bool(self.reqs)

    def launch(self, batch, use_graphs=True):
        self.reqs = list(batch)
        self.t_end = self.clock.t + self.service
        self.batches.append([r.rid for r in batch])

    def poll(self, now):
        if not self.reqs or now < self.t_end:
            return []
        done, self.reqs = self.reqs, []
        for r in done:
            if r.status != serving.CANCELLED:
                r.disparity = "result"
        return done


def _req(rid, shape=(4, 6, 8), arrival=0.0, deadline=None):
    H, W, D = shape
    return serving.StereoRequest(rid, torch.zeros(1, H, W), torch.zeros(1, H, W), D, arrival=arrival,
                                 deadline=deadline)


def _run(sched, clock, reqs, until=20.0, dt=0.25, on_tick=None):
    pending = sorted(reqs, key=lambda r: r.arrival)
    while clock.t <= until and (pending or sched.active):
        while pending and pending[0].arrival <= clock.t:
            sched.submit(pending.pop(0), clock.t)
        if on_tick:
            on_tick(clock.t)
        sched.step(clock.t)
        clock.t += dt
    return {r.rid: r for r in sched.finished}


def test_scheduler_batches_arrivals_continuously():
    clock = _Clock()
    ss = FakeSet(clock, cap=2, service=1.0)
    sched = serving.Scheduler({(4, 6, 8): [ss]})
    out = _run(sched, clock, [_req(i, arrival=0.1 * i) for i in range(5)])
    assert all(r.status == serving.DONE and r.disparity == "result" for r in out.values())
    # the first arrival runs alone; later arrivals join batches of up to 2
    assert ss.batches[0] == [0] and all(len(b) <= 2 for b in ss.batches)
    assert sorted(sum(ss.batches, [])) == list(range(5))


def test_scheduler_cancels_waiting_and_running_requests():
    clock = _Clock()
    ss = FakeSet(clock, cap=1, service=2.0)
    sched = serving.Scheduler({(4, 6, 8): [ss]})

    def tick(t):
        if abs(t - 0.5) < 1e-9:
            assert sched.cancel(0, t)      # running: result dropped when the batch ends
            assert sched.cancel(2, t)      # waiting: never launched
            assert not sched.cancel(99, t)  # unknown
    out = _run(sched, clock, [_req(0), _req(1, arrival=0.25), _req(2, arrival=0.25)], on_tick=tick)
    assert out[0].status == serving.CANCELLED and out[0].disparity is None
    assert out[2].status == serving.CANCELLED and [2] not in ss.batches
    assert out[1].status == serving.DONE and out[1].disparity == "result"
    assert not sched.cancel(1, clock.t)  # already done


def test_scheduler_expires_requests_not_started_by_their_deadline():
    clock = _Clock()
    ss = FakeSet(clock, cap=1, service=3.0)
    sched = serving.Scheduler({(4, 6, 8): [ss]})
    out = _run(sched, clock, [_req(0), _req(1, arrival=0.1, deadline=1.0), _req(2, arrival=0.1, deadline=10.0)])
    assert out[0].status == serving.DONE
    assert out[1].status == serving.EXPIRED and "deadline" in out[1].error and out[1].t_done < 3.0
    assert out[2].status == serving.DONE


def test_scheduler_rejects_on_out_of_memory_and_keeps_serving():
    clock = _Clock()
    ss = FakeSet(clock, cap=2, service=0.5)
    made = []

    def make_set(shape):
        if shape == (900, 900, 256):
            raise MemoryError("budget exhausted")
        made.append(shape)
        return FakeSet(clock, cap=1, service=0.5)
    sched = serving.Scheduler({(4, 6, 8): [ss]}, make_set)
    reqs = [_req(0), _req(1, shape=(900, 900, 256), arrival=0.1), _req(2, shape=(5, 7, 8), arrival=0.2),
            _req(3, arrival=0.3)]
    out = _run(sched, clock, reqs)
    assert out[1].status == serving.REJECTED and "out of device memory" in out[1].error
    assert out[0].status == out[2].status == out[3].status == serving.DONE
    assert made == [(5, 7, 8)]
    # torch's own out-of-memory error is handled the same way
    sched2 = serving.Scheduler({}, lambda s: (_ for _ in ()).throw(torch.cuda.OutOfMemoryError("oom")))
    assert not sched2.submit(_req(7), 0.0) and sched2.finished[0].status == serving.REJECTED


def test_latency_stats_count_completed_requests_only():
    reqs = [_req(i, arrival=0.0) for i in range(4)]
    for i, r in enumerate(reqs):
        r.t_done = 0.01 * (i + 1)
        r.status = serving.DONE if i < 3 else serving.EXPIRED
    st = serving.latency_stats(reqs)
    assert st["p99_ms"] == pytest.approx(30.0)
