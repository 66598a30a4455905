"""Serving loop for stereo BP requests on one GPU.

A request carries left/right feature maps (C,H,W) already on the device (the
output of an upstream feature network) and asks for a disparity map: SAD
cost volume over D disparities, cost = -softmax(-SAD), a 3-iteration
FP16-storage min-sum BP forward (truncated-linear pairwise L1/L2, unit edge
weights), and the per-pixel argmin of the beliefs (the reference's stereo
path: ops/sad/stereo_sad.py, ops/lbp_stereo/message_passing_op_cuda.py:138-177,
inference_op.py:23-27).  The pipeline is this library's kernels and one
memset: SAD, the cost in FP16 storage (bpl_cost_from_sad), the BP passes,
the disparity straight from the messages (bpl_messages_argmin).

Design:
  * Admission by free-HBM budget: each (H,W,D) shape gets slot sets sized to
    a share of the free device memory at start-up; a waiting request is
    admitted when a slot of its shape frees up.  A request of a shape without
    slot sets gets one made for it while the budget and the device's free
    memory allow, and is rejected (status "rejected") when they do not,
    without stopping the stream.
  * Device-resident volumes: a slot set owns its feature, cost, message and
    output buffers for its lifetime; nothing is allocated per request.
  * Continuous batching: whenever a slot set is free, the requests of its
    shape that have arrived (up to its batch size) are launched as one
    batch, while other batches run; arrivals during a batch join the next.
  * Captured graphs: each slot set replays one CUDA graph per batch size on
    its own stream, so batches of different shapes overlap on the device.
  * A batch of b requests runs the kernels with B = b: every request is
    computed exactly as it would be alone (the kernels treat batch items
    independently), so results do not depend on the mix.
  * Failure handling on the host: cancel(rid) drops a waiting request or
    discards a running one's result (status "cancelled"); a request with a
    deadline that has not started when it passes is dropped (status
    "expired"); a request that cannot get device memory is rejected
    (status "rejected").  The kernels' device error word is read when a
    batch completes; a batch whose kernels reported an error fails its
    requests (status "failed").

The scheduling (queues, admission, deadlines, cancellation, batching) is the
host-only `Scheduler`, which drives any slot-set object with `cap`, `busy`,
`launch(batch, use_graphs)` and `poll(now)`; `ServingEngine` runs it over GPU
slot sets.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time
from typing import Callable, Iterable

import torch

from . import ops
from .layers.stereo import pack_affinities

# request states
PENDING, WAITING, RUNNING, DONE = "pending", "waiting", "running", "done"
CANCELLED, EXPIRED, REJECTED, FAILED = "cancelled", "expired", "rejected", "failed"


@dataclasses.dataclass
class StereoRequest:
    rid: int
    f0: torch.Tensor  # (C,H,W) float32, device
    f1: torch.Tensor
    D: int
    arrival: float = 0.0  # seconds after the start of the stream
    deadline: float | None = None  # seconds after arrival by which it must have started (None: no limit)
    disparity: torch.Tensor | None = None  # (H,W) int64, device (filled in)
    t_done: float | None = None
    status: str = PENDING
    error: str | None = None

    @property
    def shape(self):
        return (int(self.f0.shape[1]), int(self.f0.shape[2]), int(self.D))


def slot_bytes(H: int, W: int, D: int, C: int) -> int:
    """Device bytes one request of a slot set holds: features, SAD volume
    (float), cost and messages (half, padded labels), disparity."""
    Lp = ops.padded_labels(D)
    px = H * W
    return px * (2 * C * 4 + 4 * D + 2 * Lp + 4 * Lp * 2 + 8)


class SlotSet:
    """Buffers, stream and captured graphs for batches of up to `cap`
    requests of one shape."""

    def __init__(self, H, W, D, C, cap, iters, L1, L2, delta, device):
        self.H, self.W, self.D, self.C, self.cap = H, W, D, C, cap
        self.iters, self.delta = iters, delta
        self.device = device
        Lp = ops.padded_labels(D)
        self.f0 = torch.zeros((cap, C, H, W), device=device)
        self.f1 = torch.zeros((cap, C, H, W), device=device)
        self.sad = torch.zeros((cap, H, W, D), device=device)
        self.cost_h = torch.zeros((cap, H, W, Lp), dtype=torch.float16, device=device)
        self.msgs = torch.zeros((cap, 4, H, W, Lp), dtype=torch.float16, device=device)
        self.disp = torch.zeros((cap, H, W), dtype=torch.int64, device=device)
        aff = torch.zeros((1, 4, 3, H, W), device=device)
        aff[:, :, :2] = L1
        aff[:, :, 2] = L2
        self.taps = pack_affinities(aff, torch.zeros((1, 4, H, W), device=device))
        self.edge = torch.ones((1, 4, H, W), device=device)
        self.stream = torch.cuda.Stream(device)
        self.graphs: dict[int, torch.cuda.CUDAGraph] = {}
        self.pool = None  # one memory pool for all of the set's graphs (they never run at once)
        self.event = torch.cuda.Event()
        self.reqs: list[StereoRequest] = []

    def pipeline(self, b: int):
        """The batch computation on items [0, b) (eager; also what the graphs capture)."""
        D = self.D
        sad = self.sad[:b]
        ops.sad_forward(self.f0[:b], self.f1[:b], 0, D - 1, out=sad)
        ops.cost_from_sad(sad, 1.0, half=True, out=self.cost_h[:b])
        self.msgs[:b].zero_()
        for _ in range(self.iters):
            ops.lbp_forward_f16(ops.LBP_STEREO, self.cost_h[:b], self.taps, self.edge, self.msgs[:b], self.delta, D,
                                argmin_dtype=None)
        ops.messages_argmin(self.msgs[:b], self.cost_h[:b], D, out=self.disp[:b])

    def graph(self, b: int) -> torch.cuda.CUDAGraph:
        g = self.graphs.get(b)
        if g is None:
            with torch.cuda.stream(self.stream):
                self.pipeline(b)  # warm-up (lazy kernel attributes, allocator pool)
            self.stream.synchronize()
            g = torch.cuda.CUDAGraph()
            if self.pool is None:
                self.pool = torch.cuda.graph_pool_handle()
            with torch.cuda.graph(g, pool=self.pool, stream=self.stream):
                self.pipeline(b)
            self.graphs[b] = g
        return g

    @property
    def busy(self) -> bool:
        return bool(self.reqs)

    def launch(self, reqs: list[StereoRequest], use_graphs: bool = True):
        b = len(reqs)
        g = self.graph(b) if use_graphs else None
        # the request's features must be complete before this stream reads them
        self.stream.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(self.stream):
            for i, r in enumerate(reqs):
                self.f0[i].copy_(r.f0, non_blocking=True)
                self.f1[i].copy_(r.f1, non_blocking=True)
            if g is not None:
                g.replay()
            else:
                self.pipeline(b)
            self.event.record(self.stream)
        self.reqs = list(reqs)

    def poll(self, now: float) -> list[StereoRequest]:
        if not self.reqs or not self.event.query():
            return []
        done = self.reqs
        # the kernels' bounded waits report through the device error word
        # (the batch's event has completed, so reading it stalls nothing of
        # this set; it synchronises the device)
        code = ops.read_device_error()
        for i, r in enumerate(done):
            if code:
                r.status, r.error = FAILED, f"device error {code}"
            elif r.status != CANCELLED:
                with torch.cuda.stream(self.stream):
                    r.disparity = self.disp[i].clone()
            r.t_done = now
        self.reqs = []
        return done


class Scheduler:
    """Host-side scheduling over slot sets (no device work of its own).

    sets: {shape: [slot set, ...]}; make_set(shape) -> a new slot set for an
    unplanned shape, raising MemoryError (or torch.cuda.OutOfMemoryError)
    when the device cannot hold one; use_graphs is passed to launch()."""

    def __init__(self, sets: dict, make_set: Callable | None = None, use_graphs: bool = True):
        self.sets = {tuple(s): list(v) for s, v in sets.items()}
        self.make_set = make_set
        self.use_graphs = use_graphs
        self.waiting: dict[tuple, collections.deque] = {s: collections.deque() for s in self.sets}
        self.by_id: dict[int, StereoRequest] = {}
        self.finished: list[StereoRequest] = []

    # -- requests -------------------------------------------------------------
    def submit(self, r: StereoRequest, now: float) -> bool:
        """Queues an arrived request; False if it was rejected."""
        self.by_id[r.rid] = r
        s = r.shape
        if s not in self.sets:
            err = None
            try:
                if self.make_set is None:
                    raise MemoryError("no slot set for this shape")
                self.sets[s] = [self.make_set(s)]
                self.waiting[s] = collections.deque()
            except (MemoryError, torch.cuda.OutOfMemoryError) as exc:
                err = f"out of device memory for shape {s}: {exc}"
            if err is not None:
                self._finish(r, REJECTED, now, err)
                return False
        r.status = WAITING
        self.waiting[s].append(r)
        return True

    def cancel(self, rid: int, now: float = 0.0) -> bool:
        """Cancels a waiting request (dropped) or a running one (its result
        is discarded when its batch completes).  False if it already ended."""
        r = self.by_id.get(rid)
        if r is None or r.status not in (WAITING, RUNNING):
            return False
        if r.status == WAITING:
            self.waiting[r.shape].remove(r)
            self._finish(r, CANCELLED, now)
        else:
            r.status = CANCELLED  # its batch completes; the result is dropped then
        return True

    def _finish(self, r, status, now, err=None):
        r.status, r.error, r.t_done = status, err, now
        if status != DONE:
            r.disparity = None
        self.finished.append(r)

    # -- progress -------------------------------------------------------------
    @property
    def active(self) -> bool:
        return any(self.waiting.values()) or any(ss.busy for v in self.sets.values() for ss in v)

    def step(self, now: float) -> bool:
        """Collects completed batches, drops expired waiting requests and
        launches batches on free slot sets.  Returns whether anything moved."""
        moved = False
        for sets in self.sets.values():
            for ss in sets:
                for r in ss.poll(now):
                    moved = True
                    if r.status in (CANCELLED, FAILED):
                        self._finish(r, r.status, now, r.error)
                    else:
                        self._finish(r, DONE, now)
        for s, q in self.waiting.items():
            expired = [r for r in q if r.deadline is not None and now > r.arrival + r.deadline]
            for r in expired:
                q.remove(r)
                self._finish(r, EXPIRED, now, "deadline passed before the request started")
                moved = True
            for ss in self.sets[s]:
                if q and not ss.busy:
                    batch = [q.popleft() for _ in range(min(ss.cap, len(q)))]
                    for r in batch:
                        r.status = RUNNING
                    ss.launch(batch, use_graphs=self.use_graphs)
                    moved = True
        return moved


class ServingEngine:
    """Continuous-batching engine over the shapes of a request mix."""

    def __init__(self, shapes, C: int = 64, max_batch: int = 4, hbm_fraction: float = 0.5, weights=None,
                 iters: int = 3, L1: float = 0.1, L2: float = 0.5, delta: int = 3, device=None,
                 budget_bytes: int | None = None, max_sets_per_shape: int = 2, new_shapes: bool = True):
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        shapes = [tuple(s) for s in shapes]
        weights = list(weights) if weights is not None else [1.0] * len(shapes)
        if budget_bytes is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            budget_bytes = int(free * hbm_fraction)
        self.budget = budget_bytes
        self.C, self.iters, self.L1, self.L2, self.delta = C, iters, L1, L2, delta
        self.sets: dict[tuple, list[SlotSet]] = {s: [] for s in shapes}
        plan = plan_slot_sets(shapes, weights, C, max_batch, budget_bytes, max_sets_per_shape)
        self.used = 0
        for s, (n_sets, cap) in plan.items():
            H, W, D = s
            for _ in range(n_sets):
                self.sets[s].append(SlotSet(H, W, D, C, cap, iters, L1, L2, delta, self.device))
                self.used += slot_bytes(H, W, D, C) * cap
        self.plan = plan
        self.new_shapes = new_shapes
        self.scheduler: Scheduler | None = None
        self._now = lambda: 0.0

    def _make_set(self, shape) -> SlotSet:
        """One single-request slot set for a shape outside the plan, if it
        fits the budget and the device's free memory."""
        if not self.new_shapes:
            raise MemoryError("the engine serves only its planned shapes")
        H, W, D = shape
        need = slot_bytes(H, W, D, self.C)
        free, _ = torch.cuda.mem_get_info(self.device)
        if self.used + need > self.budget or need > free:
            raise MemoryError(f"needs {need} bytes, {max(0, self.budget - self.used)} left in the budget, "
                              f"{free} free on the device")
        ss = SlotSet(H, W, D, self.C, 1, self.iters, self.L1, self.L2, self.delta, self.device)
        self.used += need
        return ss

    def warm_up(self, use_graphs=True):
        """Captures every (slot set, batch size) graph before serving."""
        for sets in self.sets.values():
            for ss in sets:
                if use_graphs:
                    for b in range(1, ss.cap + 1):
                        ss.graph(b)
        torch.cuda.synchronize(self.device)

    def cancel(self, rid: int) -> bool:
        """Cancels a request of the stream being served (e.g. from on_tick)."""
        return self.scheduler.cancel(rid, self._now()) if self.scheduler else False

    def serve(self, requests: Iterable[StereoRequest], use_graphs: bool = True, realtime: bool = True,
              clock: Callable[[], float] = time.perf_counter,
              on_tick: Callable[["ServingEngine", float], None] | None = None) -> list[StereoRequest]:
        """Serves the requests (by arrival time) and returns all of them
        ended, each with its status.  on_tick(engine, now) is called on every
        turn of the loop (e.g. to cancel requests)."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        sched = Scheduler(self.sets, self._make_set, use_graphs)
        self.scheduler = sched
        t0 = clock()
        self._now = lambda: clock() - t0
        while pending or sched.active:
            now = clock() - t0
            while pending and (not realtime or pending[0].arrival <= now):
                sched.submit(pending.popleft(), now)
            if on_tick is not None:
                on_tick(self, now)
            if not sched.step(clock() - t0):
                if realtime and pending and not any(sched.waiting.values()):
                    time.sleep(max(0.0, min(2e-4, pending[0].arrival - (clock() - t0))))
                else:
                    time.sleep(2e-5)
        torch.cuda.synchronize(self.device)
        self.sets = sched.sets
        self.scheduler = None
        return sched.finished


def plan_slot_sets(shapes, weights, C, max_batch, budget_bytes, max_sets_per_shape=2):
    """Slot sets per shape within the HBM budget: every shape gets one set
    of at least one request; the rest of the budget goes, in proportion to
    the mix weights, to larger batches and a second set per shape.
    Returns {shape: (n_sets, batch capacity)}."""
    shapes = [tuple(s) for s in shapes]
    per = {s: slot_bytes(s[0], s[1], s[2], C) for s in shapes}
    if sum(per.values()) > budget_bytes:
        raise MemoryError("HBM budget below one request of every shape")
    tot_w = float(sum(weights)) or 1.0
    plan = {}
    for s, w in zip(shapes, weights):
        share = budget_bytes * (w / tot_w)
        cap = int(max(1, min(max_batch, share // per[s])))
        n_sets = int(max(1, min(max_sets_per_shape, share // (per[s] * cap))))
        plan[s] = (n_sets, cap)

    # shrink until the plan fits (shares are floors; the minimum of one set
    # of one request per shape can exceed a small shape's share)
    def used(p):
        return sum(per[s] * n * c for s, (n, c) in p.items())
    while used(plan) > budget_bytes:
        s = max(plan, key=lambda k: per[k] * plan[k][0] * plan[k][1])
        n, c = plan[s]
        plan[s] = (n - 1, c) if n > 1 else (1, max(1, c - 1))
        if n == 1 and c == 1:
            break
    return plan


def run_plain(requests: list[StereoRequest], iters=3, L1=0.1, L2=0.5, delta=3, realtime=True,
              clock: Callable[[], float] = time.perf_counter):
    """The baseline: one request at a time, eager launches with fresh
    tensors per request (the reference's per-call allocation pattern), in
    arrival order."""
    out = []
    t0 = clock()
    for r in sorted(requests, key=lambda r: r.arrival):
        if realtime:
            while clock() - t0 < r.arrival:
                time.sleep(5e-5)
        H, W, D = r.shape
        ss = SlotSet(H, W, D, r.f0.shape[0], 1, iters, L1, L2, delta, r.f0.device)
        with torch.cuda.stream(ss.stream):
            ss.f0[0].copy_(r.f0)
            ss.f1[0].copy_(r.f1)
            ss.pipeline(1)
        ss.stream.synchronize()
        r.disparity = ss.disp[0].clone()
        r.t_done = clock() - t0
        r.status = DONE
        out.append(r)
    return out


def latency_stats(reqs: list[StereoRequest]):
    """p50 / p99 latency (arrival to completion) and throughput of the
    completed requests (status done, or never scheduled)."""
    ok = [r for r in reqs if r.status in (DONE, PENDING) and r.t_done is not None]
    lat = sorted((r.t_done - r.arrival) * 1e3 for r in ok)
    if not lat:
        return {"p50_ms": None, "p99_ms": None, "requests_per_s": None}

    def pct(p):
        k = min(len(lat) - 1, max(0, int(math.ceil(p / 100.0 * len(lat))) - 1))
        return lat[k]
    span = max(r.t_done for r in ok) - min(r.arrival for r in ok)
    return {"p50_ms": pct(50), "p99_ms": pct(99), "requests_per_s": len(ok) / span if span > 0 else None}


def synth_request_features(H, W, D, C, seed, device):
    """Left/right features of a piecewise-planar stereo scene (disparity in
    [0, D-1]): left ~ N(0,1), right = left warped by the disparity + N(0,0.1)."""
    import numpy as np
    g = np.random.default_rng(seed)
    f0 = torch.from_numpy(g.normal(0.0, 1.0, size=(C, H, W)).astype(np.float32)).to(device)
    yy, xx = np.mgrid[0:H, 0:W]
    disp = np.zeros((H, W), np.float32)
    best = np.full((H, W), np.inf)
    for _ in range(6):
        cy, cx = g.uniform(0, H), g.uniform(0, W)
        a, b, c = g.uniform(-0.05, 0.05), g.uniform(-0.05, 0.05), g.uniform(0, D - 1)
        d = (yy - cy) ** 2 + (xx - cx) ** 2
        m = d < best
        best[m] = d[m]
        disp[m] = (c + a * (yy - cy) + b * (xx - cx))[m]
    disp = np.clip(disp, 0, D - 1).round().astype(np.int64)
    src = np.clip(xx + disp, 0, W - 1)
    f1 = torch.gather(f0, 2, torch.from_numpy(src).to(device).view(1, H, W).expand(C, H, W))
    gen = torch.Generator(device=device).manual_seed(seed)
    f1 = (f1 + 0.1 * torch.randn(f1.shape, device=device, generator=gen)).contiguous()
    return f0.contiguous(), f1
