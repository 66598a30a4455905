"""Serving loop for stereo BP requests on one GPU.

A request carries left/right feature maps (C,H,W) already on the device (the
output of an upstream feature network) and asks for a disparity map: SAD
cost volume over D disparities, cost = -softmax(-SAD), a 3-iteration
FP16-storage min-sum BP forward (truncated-linear pairwise L1/L2, unit edge
weights), and the per-pixel argmin of the beliefs (the reference's stereo
path: ops/sad/stereo_sad.py, ops/lbp_stereo/message_passing_op_cuda.py:138-177,
inference_op.py:23-27).

Design:
  * Admission by free-HBM budget: each (H,W,D) shape gets slot sets sized to
    a share of the free device memory at start-up; a waiting request is
    admitted when a slot of its shape frees up.
  * Device-resident volumes: a slot set owns its feature, cost, message and
    output buffers for its lifetime; nothing is allocated per request.
  * Continuous batching: whenever a slot set is free, the requests of its
    shape that have arrived (up to its batch size) are launched as one
    batch, while other batches run; arrivals during a batch join the next.
  * Captured graphs: each slot set replays one CUDA graph per batch size
    (SAD, softmax, FP16 conversion, the BP passes, beliefs and argmin), on
    its own stream, so batches of different shapes overlap on the device.
  * A batch of b requests runs the kernels with B = b: every request is
    computed exactly as it would be alone (the kernels treat batch items
    independently), so results do not depend on the mix.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time
from typing import Callable

import torch

from . import ops
from .layers.stereo import pack_affinities


@dataclasses.dataclass
class StereoRequest:
    rid: int
    f0: torch.Tensor  # (C,H,W) float32, device
    f1: torch.Tensor
    D: int
    arrival: float = 0.0  # seconds after the start of the stream
    disparity: torch.Tensor | None = None  # (H,W) int64, device (filled in)
    t_done: float | None = None

    @property
    def shape(self):
        return (int(self.f0.shape[1]), int(self.f0.shape[2]), int(self.D))


def slot_bytes(H: int, W: int, D: int, C: int) -> int:
    """Device bytes one request of a slot set holds (buffers and the graph's
    temporaries: SAD volume, softmax and belief volumes)."""
    Lp = ops.padded_labels(D)
    px = H * W
    # features; SAD, cost, softmax and belief volumes (float); cost and
    # messages (half); scales; disparity
    return px * (2 * C * 4 + 4 * D * 4 + Lp * 2 + 4 * Lp * 2 + 4 * 4 + 8)


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
        self.cost = torch.zeros((cap, H, W, D), device=device)
        self.cost_h = torch.zeros((cap, H, W, Lp), dtype=torch.float16, device=device)
        self.msgs = torch.zeros((cap, 4, H, W, Lp), dtype=torch.float16, device=device)
        self.scale = torch.zeros((cap, 4, H, W), device=device)
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
        sad.neg_()
        torch.neg(torch.softmax(sad, dim=-1), out=self.cost[:b])
        self.cost_h[:b, ..., :D].copy_(self.cost[:b])
        self.msgs[:b].zero_()
        for _ in range(self.iters):
            ops.lbp_forward_f16(ops.LBP_STEREO, self.cost_h[:b], self.taps, self.edge, self.msgs[:b], self.delta, D,
                                argmin_dtype=None, scale=self.scale[:b])
        beliefs = self.cost[:b].clone()
        for k in range(4):
            beliefs.add_(self.msgs[:b, k, ..., :D])
        torch.argmin(beliefs, dim=-1, out=self.disp[:b])

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
        for i, r in enumerate(done):
            with torch.cuda.stream(self.stream):
                r.disparity = self.disp[i].clone()
            r.t_done = now
        self.reqs = []
        return done


class ServingEngine:
    """Continuous-batching engine over the shapes of a request mix."""

    def __init__(self, shapes, C: int = 64, max_batch: int = 4, hbm_fraction: float = 0.5, weights=None,
                 iters: int = 3, L1: float = 0.1, L2: float = 0.5, delta: int = 3, device=None,
                 budget_bytes: int | None = None, max_sets_per_shape: int = 2):
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        shapes = [tuple(s) for s in shapes]
        weights = list(weights) if weights is not None else [1.0] * len(shapes)
        if budget_bytes is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            budget_bytes = int(free * hbm_fraction)
        self.budget = budget_bytes
        self.sets: dict[tuple, list[SlotSet]] = {s: [] for s in shapes}
        plan = plan_slot_sets(shapes, weights, C, max_batch, budget_bytes, max_sets_per_shape)
        for s, (n_sets, cap) in plan.items():
            H, W, D = s
            for _ in range(n_sets):
                self.sets[s].append(SlotSet(H, W, D, C, cap, iters, L1, L2, delta, self.device))
        self.plan = plan

    def warm_up(self, use_graphs=True):
        """Captures every (slot set, batch size) graph before serving."""
        for sets in self.sets.values():
            for ss in sets:
                if use_graphs:
                    for b in range(1, ss.cap + 1):
                        ss.graph(b)
        torch.cuda.synchronize(self.device)

    def serve(self, requests: list[StereoRequest], use_graphs: bool = True, realtime: bool = True,
              clock: Callable[[], float] = time.perf_counter) -> list[StereoRequest]:
        """Serves the requests (sorted by arrival) and returns them completed."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting: dict[tuple, collections.deque] = {s: collections.deque() for s in self.sets}
        for r in pending:
            if r.shape not in self.sets:
                raise ValueError(f"no slot set for shape {r.shape}")
        done: list[StereoRequest] = []
        t0 = clock()
        while pending or any(waiting.values()) or any(ss.busy for v in self.sets.values() for ss in v):
            now = clock() - t0
            while pending and (not realtime or pending[0].arrival <= now):
                r = pending.popleft()
                waiting[r.shape].append(r)
            progressed = False
            for sets in self.sets.values():
                for ss in sets:
                    fin = ss.poll(clock() - t0)
                    if fin:
                        done.extend(fin)
                        progressed = True
            for s, q in waiting.items():
                for ss in self.sets[s]:
                    if q and not ss.busy:
                        batch = [q.popleft() for _ in range(min(ss.cap, len(q)))]
                        ss.launch(batch, use_graphs=use_graphs)
                        progressed = True
            if not progressed:
                if realtime and pending and not any(waiting.values()):
                    time.sleep(max(0.0, min(2e-4, pending[0].arrival - (clock() - t0))))
                else:
                    time.sleep(5e-5)
        torch.cuda.synchronize(self.device)
        return done


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
        out.append(r)
    return out


def latency_stats(reqs: list[StereoRequest]):
    lat = sorted((r.t_done - r.arrival) * 1e3 for r in reqs)
    if not lat:
        return {"p50_ms": None, "p99_ms": None}

    def pct(p):
        k = min(len(lat) - 1, max(0, int(math.ceil(p / 100.0 * len(lat))) - 1))
        return lat[k]
    span = max(r.t_done for r in reqs) - min(r.arrival for r in reqs)
    return {"p50_ms": pct(50), "p99_ms": pct(99), "requests_per_s": len(reqs) / span if span > 0 else None}


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
