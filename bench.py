"""Benchmark of the BP-Layers hot path on GB300.

Workload (the full-size stereo configuration): one training step of the
stereo BP layer, FP32, B=1, H=376, W=1240, D=L=192 labels, 3 message-passing
iterations, truncated-linear pairwise with learnable L1=0.1 / L2=0.5
(delta=3), per-pixel/direction edge weights exp(N(0,0.3)), forward
(MessagePassing: 3 LBP passes, beliefs, softmin) and backward with an
upstream gradient N(0,1) on the beliefs.  The cost volume comes from a
synthetic piecewise-planar stereo scene (C=64 features, SAD over 192
disparities, softmax) built once on the device before timing.

One step = U = 2 * iters * L * (2H(W-1) + 2W(H-1)) message-label updates
(forward + backward).  `value` = U * steps / device time with all inputs
resident in HBM; `e2e` = the same step through the public API with the cost
volume, edge weights and upstream gradient copied from pinned host memory and
the cost gradient plus the disparity map copied back, every step.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
With --gpus N > 1 (launched by torchrun) every rank runs an independent
replica on its own GPU (the path does not shard; no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "bp-layers_gb300"), os.path.join(ROOT, "tests", "golden")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "min-sum msg-label updates/s & HBM GB/s vs peak; served p50/p99 vs plain"
UNIT = "msg-label updates/s"
H, W, L, C_FEAT, ITERS, DELTA = 376, 1240, 192, 64, 3, 3
FWD_BYTES_PER_UPDATE = 21  # cost + 3 incoming + 1 outgoing message (FP32) + 1 B argmin
BWD_BYTES_PER_UPDATE = 17  # argmin + upstream grad + saved message + RMW grad-cost
CPU_CROP_W = 310           # CPU baseline sample: one pass on a 376 x 310 x 192 crop


def edges(h, w):
    return 2 * h * (w - 1) + 2 * w * (h - 1)


def updates_per_step(h=H, w=W, l=L, iters=ITERS):
    return 2 * iters * l * edges(h, w)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region.

    Samples every 20 ms, each with nvidia-smi's own timestamp; sampling is
    running before the region starts (the first sample has arrived), and the
    summary keeps the samples taken between start() and stop().  A region
    shorter than the sampling interval keeps the first sample after start()."""
    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    INTERVAL_MS = 20

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.t_start = self.t_stop = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line))

    def __enter__(self):
        import threading
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return self
        self.reader = threading.Thread(target=self._read, daemon=True)
        self.reader.start()
        deadline = time.time() + 15.0
        while not self.lines and time.time() < deadline and self.proc.poll() is None:
            time.sleep(0.01)
        return self

    def start(self):
        self.t_start = time.time()

    def stop(self):
        self.t_stop = time.time()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.reader.join(timeout=5)
        return False

    @staticmethod
    def _stamp(text, arrival):
        import datetime
        try:
            return datetime.datetime.strptime(text, "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return arrival

    def summary(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = []
        for arrival, line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((self._stamp(f[0], arrival), float(f[1]), float(f[2]), f[5:9]))
            except ValueError:
                continue
        t0 = self.t_start if self.t_start is not None else float("-inf")
        t1 = self.t_stop if self.t_stop is not None else float("inf")
        inside = [r for r in rows if t0 <= r[0] <= t1]
        if not inside:
            inside = [r for r in rows if r[0] >= t0][:1]
        sms = [r[1] for r in inside]
        reasons = {n for r in inside for n, v in zip(names, r[3]) if v.lower().startswith("active")}
        return {"sm_mhz": statistics.median(sms) if sms else None,
                "sm_max_mhz": inside[-1][2] if inside else None,
                "samples": len(sms), "interval_ms": self.INTERVAL_MS,
                "region_s": (t1 - t0) if self.t_start is not None and self.t_stop is not None else None,
                "reasons": sorted(reasons)}


def synth_inputs(torch, dev, seed, H=H, W=W):
    """Piecewise-planar stereo scene -> SAD (C=64, D=192) -> softmax -> prob volume."""
    import numpy as np
    import cases
    g = cases.rng(seed)
    f0 = torch.from_numpy(g.normal(0.0, 1.0, size=(1, C_FEAT, H, W)).astype(np.float32)).to(dev)
    disp = torch.from_numpy(cases.planar_disparity(g, H, W, L)).to(dev)
    xs = torch.arange(W, device=dev).view(1, W).expand(H, W)
    src = (xs + disp.round().long()).clamp(0, W - 1)
    f1 = torch.gather(f0, 3, src.view(1, 1, H, W).expand(1, C_FEAT, H, W))
    f1 = f1 + 0.1 * torch.randn(f1.shape, device=dev, generator=torch.Generator(device=dev).manual_seed(seed))
    sad = torch.full((1, H, W, L), 40.0, device=dev)
    for d in range(L):
        if d < W:
            sad[0, :, d:, d] = (f0[0, :, :, d:] - f1[0, :, :, :W - d]).abs().sum(0)
    prob = torch.softmax(-sad, dim=-1).contiguous()
    gen = torch.Generator(device=dev).manual_seed(seed + 1)
    edge = torch.exp(0.3 * torch.randn((1, 4, H, W), device=dev, generator=gen)).contiguous()
    upstream = torch.randn((1, H, W, L), device=dev, generator=gen).contiguous()
    return prob, edge, upstream


def run_ours(args):
    import torch
    import torch.distributed as dist
    from bpl_gb300 import ops
    from bpl_gb300.layers.stereo import MessagePassing

    from bpl_gb300 import replicas
    rank, world, local = replicas.env_ranks()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl")

    prob, edge, upstream = synth_inputs(torch, dev, seed=replicas.replica_seed(1, rank))
    mp = MessagePassing(dev, ITERS, L, DELTA)
    with torch.no_grad():
        mp._L1.fill_(0.1)
        mp._L2.fill_(0.5)
    prob.requires_grad_(True)

    def step(p, e, g, before_backward=None):
        messages = torch.zeros((1, 4, H, W, L), device=dev, requires_grad=True)
        beliefs, _ = mp(p, e, None, None, messages)
        if before_backward is not None:
            before_backward()
        beliefs.backward(g)
        return beliefs

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        prob.grad = None
        step(prob, edge, upstream)
    barrier()

    stream = torch.cuda.current_stream()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk, ops.timing() as tm:
        barrier()
        torch.cuda.profiler.start()  # profiler range = the timed region (ncu --profile-from-start off)
        clk.start()
        t0.record(stream)
        for _ in range(args.steps):
            prob.grad = None
            step(prob, edge, upstream)
        t1.record(stream)
        barrier()
        clk.stop()
        torch.cuda.profiler.stop()
    ms = t0.elapsed_time(t1)
    per_op = tm.report()
    ms_max = replicas.max_over_ranks(ms, dev)

    # ---- e2e through the public API with host buffers --------------------
    # Every step copies its inputs from pinned host memory and its results
    # (cost gradient, disparity map) back; the copies run on their own
    # streams, double-buffered, so step i+1's inputs arrive and step i-1's
    # results leave while step i computes.  The forward waits for the
    # probability volume and edge weights only; the upstream gradient has
    # its own event, which the backward waits for (it lands while the
    # forward runs).  The timed region spans the first input copy to the
    # last result copy.
    prob_h = prob.detach().cpu().pin_memory()
    edge_h = edge.cpu().pin_memory()
    up_h = upstream.cpu().pin_memory()
    grad_h = [torch.empty(prob_h.shape, dtype=torch.float32).pin_memory() for _ in range(2)]
    disp_h = [torch.empty((1, H, W, 1), dtype=torch.int64).pin_memory() for _ in range(2)]
    h2d = (prob_h.numel() + edge_h.numel() + up_h.numel()) * 4
    d2h = grad_h[0].numel() * 4 + disp_h[0].numel() * 8
    cin, cout = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    bufs = [(torch.empty(prob_h.shape, device=dev), torch.empty(edge_h.shape, device=dev),
             torch.empty(up_h.shape, device=dev)) for _ in range(2)]
    in_ready = [torch.cuda.Event() for _ in range(2)]
    up_ready = [torch.cuda.Event() for _ in range(2)]
    in_free = [torch.cuda.Event() for _ in range(2)]
    out_done = [torch.cuda.Event() for _ in range(2)]
    for ev in in_free:
        ev.record(stream)

    def issue_inputs(i):
        k = i % 2
        with torch.cuda.stream(cin):
            cin.wait_event(in_free[k])  # step i-2 has finished reading buffer k
            bufs[k][0].copy_(prob_h, non_blocking=True)
            bufs[k][1].copy_(edge_h, non_blocking=True)
            in_ready[k].record(cin)
            bufs[k][2].copy_(up_h, non_blocking=True)
            up_ready[k].record(cin)

    def e2e_run(n):
        issue_inputs(0)
        for i in range(n):
            k = i % 2
            if i + 1 < n:
                issue_inputs(i + 1)
            stream.wait_event(in_ready[k])
            p = bufs[k][0].detach().requires_grad_(True)
            beliefs = step(p, bufs[k][1], bufs[k][2], before_backward=lambda: stream.wait_event(up_ready[k]))
            disp = torch.argmax(beliefs.detach(), dim=3, keepdim=True)
            in_free[k].record(stream)
            gr = p.grad
            with torch.cuda.stream(cout):
                cout.wait_stream(stream)
                cout.wait_event(out_done[k])  # the host buffer's previous copy has landed
                grad_h[k].copy_(gr, non_blocking=True)
                disp_h[k].copy_(disp, non_blocking=True)
                out_done[k].record(cout)
            gr.record_stream(cout)
            disp.record_stream(cout)
        stream.wait_stream(cout)

    e2e_run(max(2, args.warmup // 2))
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    cin.wait_event(e0)
    e2e_run(args.steps)
    e1.record(stream)
    barrier()
    e2e_ms = replicas.max_over_ranks(e0.elapsed_time(e1), dev)

    # ---- the same step with FP16 storage of cost and messages -----------------
    fp16 = None
    if not args.no_fp16:
        mp16 = MessagePassing(dev, ITERS, L, DELTA, storage="fp16")
        with torch.no_grad():
            mp16._L1.fill_(0.1)
            mp16._L2.fill_(0.5)

        def step16(p, e, g):
            beliefs, _ = mp16(p, e, None, None, None)
            beliefs.backward(g)
            return beliefs

        for _ in range(args.warmup):
            prob.grad = None
            step16(prob, edge, upstream)
        barrier()
        h0 = torch.cuda.Event(enable_timing=True)
        h1 = torch.cuda.Event(enable_timing=True)
        with ops.timing() as tm16:
            h0.record(stream)
            for _ in range(args.steps):
                prob.grad = None
                b16 = step16(prob, edge, upstream)
            h1.record(stream)
            barrier()
        ms16 = h0.elapsed_time(h1)
        per16 = tm16.report()
        prob.grad = None
        b32 = step(prob, edge, upstream)
        agree = float((b16.detach().argmax(-1) == b32.detach().argmax(-1)).float().mean().item())
        f16 = per16.get("lbp_forward_f16", [])
        bw16 = per16.get("lbp_backward_f16", [])
        n16 = args.steps * ITERS
        fp16 = {"value": replicas.whole_job_rate(updates_per_step(), args.steps, world, ms16), "unit": UNIT,
                "ms_per_step": ms16 / args.steps, "speedup_vs_fp32": ms_max / ms16,
                "label_agreement_vs_fp32": agree,
                "lbp_forward_pass_ms": sum(f16) / n16, "lbp_backward_pass_ms": sum(bw16) / n16,
                "bytes_per_update": {"forward": 11, "backward": 12}}

    # ---- the same step with argmin recomputation (no stored indices) -------
    recompute = None
    if not args.no_recompute:
        mpr = MessagePassing(dev, ITERS, L, DELTA, recompute_argmin=True)
        with torch.no_grad():
            mpr._L1.fill_(0.1)
            mpr._L2.fill_(0.5)

        def held_by_forward(model):
            prob.grad = None
            m0 = torch.zeros((1, 4, H, W, L), device=dev, requires_grad=True)
            torch.cuda.synchronize()
            before = torch.cuda.memory_allocated(dev)
            b, _ = model(prob, edge, None, None, m0)
            torch.cuda.synchronize()
            held = torch.cuda.memory_allocated(dev) - before - b.numel() * 4
            b.backward(upstream)
            return held

        held_rec, held_std = held_by_forward(mpr), held_by_forward(mp)
        n_rec = max(2, args.steps // 3)
        for _ in range(2):
            prob.grad = None
            b = mpr(prob, edge, None, None, torch.zeros((1, 4, H, W, L), device=dev, requires_grad=True))[0]
            b.backward(upstream)
        barrier()
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r0.record(stream)
        for _ in range(n_rec):
            prob.grad = None
            b = mpr(prob, edge, None, None, torch.zeros((1, 4, H, W, L), device=dev, requires_grad=True))[0]
            b.backward(upstream)
        r1.record(stream)
        barrier()
        ms_rec = r0.elapsed_time(r1) / n_rec
        recompute = {"ms_per_step": ms_rec, "value": updates_per_step() / (ms_rec / 1e3), "unit": UNIT,
                     "vs_stored_step": ms_rec / (ms_max / args.steps),
                     "bytes_held_by_forward": {"recompute": held_rec, "stored_indices": held_std,
                                               "indices_alone": ITERS * 4 * H * W * L},
                     "steps": n_rec}

    U = updates_per_step()
    value = replicas.whole_job_rate(U, args.steps, world, ms_max)
    e2e_value = replicas.whole_job_rate(U, args.steps, world, e2e_ms)
    peak, peak_kind = load_peaks()
    fwd = per_op.get("lbp_forward", [])
    bwd = per_op.get("lbp_backward", [])
    U_pass = L * edges(H, W)
    # per pass: the layer runs ITERS forward calls per step and one backward
    # call covering all ITERS passes (bpl_lbp_backward_passes)
    n_pass = args.steps * ITERS
    fwd_ms = sum(fwd) / n_pass
    bwd_ms = sum(bwd) / n_pass
    if sum(fwd) >= sum(bwd):
        kname, kms, kbytes = "lbp_forward_kernel", fwd_ms, U_pass * FWD_BYTES_PER_UPDATE
    else:
        kname, kms, kbytes = "lbp_backward_kernel", bwd_ms, U_pass * BWD_BYTES_PER_UPDATE
    achieved = kbytes / (kms / 1e3) / 1e9
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "stereo BP-Layer forward+backward, 376x1240x192, 3 iterations, FP32",
                   "B": 1, "H": H, "W": W, "L": L, "iters": ITERS, "delta": DELTA,
                   "updates_per_step": U, "l2": "inputs larger than L2 (cost 358 MB, messages 1.43 GB)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms / args.steps,
                "copies": "pinned host buffers, copy streams double-buffered: step i+1's inputs and step i-1's "
                          "results move while step i computes"},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
                     "launch_ms": kms, "algorithmic_bytes_per_launch": kbytes,
                     "launch": "per pass: the forward is 2 grid launches (horizontal, vertical sweeps) per pass, "
                               "the backward 2 launches covering the 3 passes; times are per pass"},
        "kernel_ms": {"lbp_forward_pass": fwd_ms, "lbp_backward_pass": bwd_ms,
                      "forward_GBps_21B": U_pass * FWD_BYTES_PER_UPDATE / (fwd_ms / 1e3) / 1e9 if fwd else None,
                      "backward_GBps_17B": U_pass * BWD_BYTES_PER_UPDATE / (bwd_ms / 1e3) / 1e9 if bwd else None},
        # forward passes (2 phases each), batched adjoint (2 phases), belief
        # epilogue (forward; backward, which also writes the initial
        # messages' gradient), tap packing and its gradient's fold
        "gpu_launches": args.steps * (ITERS * 2 + 2 + 2 + 2),
        "fp16": fp16,
        "recompute_argmin": recompute,
        "clocks": clk.summary(),
    }
    if world == 1 and not args.no_serving:
        result["serving"] = run_serving(args)
    if rank == 0 and world == 1 and not args.no_accuracy:
        result["accuracy_vs_fp64_oracle"] = run_accuracy()
    if rank == 0 and world == 1 and not args.no_other:
        result["other_configs"] = run_other_configs()
    if rank == 0 and world == 1 and not args.no_reference_gpu:
        try:
            result.setdefault("other_configs", {})[f"reference_gpu_ops_{H}x{W}x{L}"] = run_reference_gpu_ops(
                fwd_ms, bwd_ms, ms_max / args.steps)
        except Exception as exc:  # the reference arm never takes the bench down
            result.setdefault("other_configs", {})[f"reference_gpu_ops_{H}x{W}x{L}"] = {
                "unavailable": f"{type(exc).__name__}: {str(exc)[:200]}"}
    traffic = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(traffic):
        with open(traffic) as fh:
            tr = json.load(fh).get(kname)
        if tr:
            result["roofline"]["traffic"] = tr
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline_sample()
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(result))


SERVE_MIX = [((376, 1240, 128), 0.5), ((540, 960, 192), 0.3), ((720, 1280, 256), 0.2)]
SERVE_C = 64


def run_serving(args):
    """Served mixed stream of stereo requests (SAD + 3-iteration FP16-storage
    BP forward + disparity): Poisson arrivals (seed 1) over the shape mix,
    served by the continuous-batching engine (free-HBM admission, resident
    volumes, captured graphs), against plain per-request launches of the
    same requests.  Plain capacity is measured first (requests back to
    back); the stream is then offered at each of `serve_loads` times that
    capacity, to both, in real time.  Also the device time of each shape's
    captured graph per batch size (the batched cost per request)."""
    import numpy as np
    import torch
    from bpl_gb300 import serving
    dev = torch.device("cuda", 0)
    n = args.serve_requests
    g = np.random.default_rng(1)
    shapes = [s for s, _ in SERVE_MIX]
    probs = np.array([w for _, w in SERVE_MIX])
    kinds = g.choice(len(shapes), size=n, p=probs / probs.sum())
    feats = {}
    for k in range(len(shapes)):  # two distinct scenes per shape, reused
        H_, W_, D_ = shapes[k]
        feats[k] = [serving.synth_request_features(H_, W_, D_, SERVE_C, seed=10 * k + j, device=dev) for j in range(2)]

    def make(arrivals):
        return [serving.StereoRequest(i, *feats[int(kinds[i])][i % 2], shapes[int(kinds[i])][2], arrival=float(a))
                for i, a in enumerate(arrivals)]

    # plain capacity: back to back (after one warm-up request per shape)
    serving.run_plain([serving.StereoRequest(-1 - k, *feats[k][0], shapes[k][2]) for k in range(len(shapes))],
                      realtime=False)
    torch.cuda.synchronize()
    t = time.perf_counter()
    serving.run_plain(make(np.zeros(n)), realtime=False)
    plain_rps = n / (time.perf_counter() - t)
    eng = serving.ServingEngine(shapes, C=SERVE_C, max_batch=4, hbm_fraction=0.5, weights=probs, device=dev)
    eng.warm_up()
    # device time of each shape's graph per batch size
    graphs = {}
    for s, sets in eng.sets.items():
        ss = sets[0]
        row = {}
        for b in range(1, ss.cap + 1):
            gr = ss.graph(b)
            a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(ss.stream):
                gr.replay()
                a.record(ss.stream)
                for _ in range(3):
                    gr.replay()
                e.record(ss.stream)
            ss.stream.synchronize()
            ms = a.elapsed_time(e) / 3
            row[f"b{b}"] = {"ms": ms, "ms_per_request": ms / b}
        graphs[f"{s[0]}x{s[1]}x{s[2]}"] = row
    sweep = {}
    for load in args.serve_loads:
        rate = load * plain_rps
        arrivals = np.cumsum(g.exponential(1.0 / rate, size=n))
        plain = serving.latency_stats(serving.run_plain(make(arrivals)))
        served_reqs = eng.serve(make(arrivals))
        served = serving.latency_stats(served_reqs)
        ok = sum(r.status == serving.DONE for r in served_reqs)
        sweep[f"{load:g}x"] = {
            "offered_rate_rps": rate, "completed": ok,
            "served": {"requests_per_s": served["requests_per_s"], "p50_ms": served["p50_ms"],
                       "p99_ms": served["p99_ms"]},
            "plain": {"requests_per_s": plain["requests_per_s"], "p50_ms": plain["p50_ms"], "p99_ms": plain["p99_ms"]},
            "throughput_vs_plain": (served["requests_per_s"] / plain["requests_per_s"]
                                    if served["requests_per_s"] and plain["requests_per_s"] else None)}
    torch.cuda.synchronize()
    plan = eng.plan
    eng = None
    torch.cuda.empty_cache()
    top = sweep[f"{max(args.serve_loads):g}x"]
    return {
        "requests": n, "mix": [{"H": s[0], "W": s[1], "D": s[2], "p": w} for s, w in SERVE_MIX],
        "pipeline": "SAD (C=64) + cost -softmax(-SAD) in FP16 storage + 3-iteration FP16-storage BP forward + "
                    "disparity from the messages (argmin), each a library kernel",
        "plain_capacity_rps": plain_rps,
        "offered_load_vs_plain_capacity": max(args.serve_loads),
        "served": top["served"], "plain": top["plain"], "throughput_vs_plain": top["throughput_vs_plain"],
        "sweep": sweep, "graph_ms": graphs,
        "slot_plan": {f"{s[0]}x{s[1]}x{s[2]}": {"sets": v[0], "batch": v[1]} for s, v in plan.items()},
    }


def _softmin64(z):
    import numpy as np
    z = z.astype(np.float64)
    e = np.exp(-(z - z.min(-1, keepdims=True)))
    return e / e.sum(-1, keepdims=True)


def run_accuracy():
    """Argmin disagreement and belief max-abs error against the FP64 oracle,
    per configuration, for FP32 and FP16 storage (beliefs = softmin of the
    message sum plus cost; argmin = the per-pixel label).  Bounded CPU time:
    the full-size stereo case is a 376x310 crop, the semantic case a 256x512
    crop of each of its 2 images."""
    import numpy as np
    import torch
    from bpl_gb300 import ops
    import cases
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    out = {}

    def report(name, cost, jump_fp32, jump_f16, edge, delta, iters, variant, L):
        B, H, W, _ = cost.shape
        m64, _, _ = oracle.lbp_forward(variant, cost.astype(np.float64), jump_fp32, edge,
                                       np.zeros((B, 4, H, W, L)), delta, fp64=True, iters=iters, threads=0)
        b64 = _softmin64(m64.sum(1) + cost)
        lab64 = b64.argmax(-1)
        res = {}
        # FP32 storage
        m = torch.zeros((B, 4, H, W, L), device=dev)
        for _ in range(iters):
            ops.lbp_forward(variant, t(cost), t(jump_fp32), t(edge), m, delta, argmin_dtype=None)
        b = _softmin64(m.cpu().numpy().sum(1) + cost)
        res["fp32"] = {"argmin_disagreement": float((b.argmax(-1) != lab64).mean()),
                       "belief_max_abs_error": float(np.abs(b - b64).max())}
        # FP16 storage (same half-rounded cost for the oracle would isolate the
        # storage of messages; here the cost is rounded too, as the FP16 layer does)
        Lp = ops.padded_labels(L)
        ch = ops.to_half_padded(t(cost), L)
        mh = torch.zeros((B, 4, H, W, Lp), dtype=torch.float16, device=dev)
        jh = t(jump_fp32) if variant == 0 else ops.to_half_padded(t(jump_f16), L)
        for _ in range(iters):
            ops.lbp_forward_f16(variant, ch, jh, t(edge), mh, delta, L, argmin_dtype=None)
        b = _softmin64(mh[..., :L].float().cpu().numpy().sum(1) + cost)
        res["fp16"] = {"argmin_disagreement": float((b.argmax(-1) != lab64).mean()),
                       "belief_max_abs_error": float(np.abs(b - b64).max())}
        out[name] = res

    # c0: 96x128x32 SAD scene, 1 iteration, unit edges
    g = cases.rng(0)
    cost, *_ = cases.stereo_cost_from_scene(g, 1, 96, 128, 32, 32)
    report("stereo_96x128x32_1it", cost, cases.stereo_taps(1, 96, 128, 0.1, 0.5), None,
           np.ones((1, 4, 96, 128), np.float32), 3, 1, 0, 32)
    # c1 (crop): 376x310x192, 3 iterations, edges exp(N(0,0.3))
    g = cases.rng(1)
    cost, *_ = cases.stereo_cost_from_scene(g, 1, 376, 310, 64, 192)
    edge = np.exp(g.normal(0, 0.3, size=(1, 4, 376, 310))).astype(np.float32)
    report("stereo_376x310x192_3it_crop", cost, cases.stereo_taps(1, 376, 310, 0.1, 0.5), None, edge, 3, 3, 0, 192)
    # c3 (crop): semantic pixel-pairwise, B=2, 256x512, L=19, 2 iterations;
    # unaries FP16 log-softmax of N(0,2) logits + 32x32 block class bias
    g = cases.rng(3)
    B, H, W, L = 2, 256, 512, 19
    logits = g.normal(0, 2, size=(B, H, W, L)).astype(np.float32)
    bias = g.normal(0, 2, size=(B, H // 32, W // 32, L)).astype(np.float32)
    logits += np.repeat(np.repeat(bias, 32, axis=1), 32, axis=2)
    lsm = logits - logits.max(-1, keepdims=True)
    lsm = lsm - np.log(np.exp(lsm).sum(-1, keepdims=True))
    cost = (-lsm.astype(np.float16)).astype(np.float32)
    j4, _ = cases.semantic_pixel_jump(g, H, W, L)
    j4 = j4.astype(np.float16).astype(np.float32)  # the FP16 pairwise storage, for every path alike
    edge = np.ones((B, 4, H, W), np.float32)
    report("semantic_pixel_2x256x512x19_2it_crop", cost, j4, j4, edge, L, 2, 2, L)
    return out


def run_other_configs():
    """Device time of the other configurations' ops (inputs resident): the
    semantic pixel-pairwise pass at 2x512x1024, L=19 (FP32 and FP16 storage,
    per pass, with the reference adjoint), the flow SAD sub-case 384x512,
    C=32, window +-32 (and +-108 in one call), the flow BP in the reference's
    order and as one batch, the coarse-to-fine glue, and the stereo SAD at
    the full size."""
    import numpy as np
    import torch
    from bpl_gb300 import ops
    import cases
    dev = torch.device("cuda", 0)

    def timed(fn, n=3):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(n):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    out = {}
    g = cases.rng(3)
    B, Hs, Ws, Ls = 2, 512, 1024, 19
    cost = torch.from_numpy(cases.random_cost(g, B, Hs, Ws, Ls)).to(dev)
    j4, _ = cases.semantic_pixel_jump(g, Hs, Ws, Ls)
    j4 = torch.from_numpy(j4).to(dev)
    edge = torch.ones((B, 4, Hs, Ws), device=dev)
    m = torch.zeros((B, 4, Hs, Ws, Ls), device=dev)
    am = torch.empty((B, 4, Hs, Ws, Ls), dtype=torch.uint8, device=dev)
    sc = torch.empty((B, 4, Hs, Ws), device=dev)
    gin = torch.randn((B, 4, Hs, Ws, Ls), device=dev)
    U = B * Ls * edges(Hs, Ws)
    fwd = timed(lambda: ops.lbp_forward(ops.LBP_SEM_PIXEL, cost, j4, edge, m, Ls, argmin_dtype=torch.uint8,
                                        argmin=am, scale=sc))
    bwd = timed(lambda: ops.lbp_backward(ops.LBP_SEM_PIXEL, None, edge, gin, m, am, sc, copy_grad_messages=False))
    ch = ops.to_half_padded(cost, Ls)
    jh = ops.to_half_padded(j4, Ls)
    Lp = ops.padded_labels(Ls)
    mh = torch.zeros((B, 4, Hs, Ws, Lp), dtype=torch.float16, device=dev)
    amh = torch.empty((B, 4, Hs, Ws, Lp), dtype=torch.uint8, device=dev)
    sch = torch.empty((B, 4, Hs, Ws), device=dev)
    fwd16 = timed(lambda: ops.lbp_forward_f16(ops.LBP_SEM_PIXEL, ch, jh, edge, mh, Ls, Ls, argmin=amh, scale=sch))
    out["semantic_pixel_2x512x1024x19"] = {
        "fp32_forward_pass_ms": fwd, "fp32_backward_pass_ms": bwd, "fp16_forward_pass_ms": fwd16,
        "updates_per_pass": U, "fp32_forward_updates_per_s": U / (fwd / 1e3),
        "fp32_forward_GBps": U * (21 + 4 * Ls) / (fwd / 1e3) / 1e9}
    # one pass of the layer (message_passing_op_pw_pixel.py:27-51): the
    # reference's per-pass packing into (4,H,W,L,L) and the fold of the jump
    # gradient, against the two planes read and accumulated by the kernels
    jp = torch.from_numpy(g.uniform(0.0, 1.5, size=(2, Hs, Ws, Ls, Ls)).astype(np.float32)).to(dev)

    def packed_pass():
        js = torch.zeros((4, Hs, Ws, Ls, Ls), device=dev)
        js[0] = jp[0]
        js[1, :, 1:] = jp[0, :, :-1].permute(0, 1, 3, 2)
        js[2] = jp[1]
        js[3, 1:] = jp[1, :-1].permute(0, 1, 3, 2)
        ops.lbp_forward(ops.LBP_SEM_PIXEL, cost, js.contiguous(), edge, m, Ls, argmin_dtype=torch.uint8, argmin=am,
                        scale=sc)
        _, gj, _, _ = ops.lbp_backward(ops.LBP_SEM_PIXEL, None, edge, gin, m, am, sc, copy_grad_messages=False)
        gj[0, :, :-1] += gj[1, :, 1:].permute(0, 1, 3, 2)
        gj[1] = gj[2]
        gj[1, :-1] += gj[3, 1:].permute(0, 1, 3, 2)

    def planes_pass():
        ops.lbp_forward(ops.LBP_SEM_PIXEL_LAYER, cost, jp, edge, m, Ls, argmin_dtype=torch.uint8, argmin=am, scale=sc)
        ops.lbp_backward(ops.LBP_SEM_PIXEL_LAYER, None, edge, gin, m, am, sc, copy_grad_messages=False)

    out["semantic_pixel_2x512x1024x19"]["layer_pass_fwd_bwd_ms"] = {"materialised_packing": timed(packed_pass),
                                                                      "two_planes_in_kernels": timed(planes_pass)}
    del j4, ch, jh, mh, amh, sch, jp
    # the semantic configuration's global form (lbp_semantic_pw): one 19x19
    # matrix per axis (symmetric, zero diagonal, off-diagonal U[0.2,1.5]),
    # per-pixel edge weights exp(N(0,0.3)), per pass
    P = g.uniform(0.2, 1.5, size=(2, Ls, Ls)).astype(np.float32)
    P = 0.5 * (P + P.transpose(0, 2, 1))
    for k in range(2):
        np.fill_diagonal(P[k], 0.0)
    jg = torch.from_numpy(np.stack([P[0], P[0].T, P[1], P[1].T])[None].copy()).to(dev)
    eg = torch.exp(0.3 * torch.randn((B, 4, Hs, Ws), device=dev))
    fwd_g = timed(lambda: ops.lbp_forward(ops.LBP_SEM_GLOBAL, cost, jg, eg, m, Ls, argmin_dtype=torch.uint8,
                                          argmin=am, scale=sc))
    bwd_g = timed(lambda: ops.lbp_backward(ops.LBP_SEM_GLOBAL, jg, eg, gin, m, am, sc, copy_grad_messages=False))
    ch = ops.to_half_padded(cost, Ls)
    mh = torch.zeros((B, 4, Hs, Ws, ops.padded_labels(Ls)), dtype=torch.float16, device=dev)
    fwd_g16 = timed(lambda: ops.lbp_forward_f16(ops.LBP_SEM_GLOBAL, ch, jg, eg, mh, Ls, Ls, argmin_dtype=torch.uint8))
    out["semantic_global_2x512x1024x19"] = {
        "fp32_forward_pass_ms": fwd_g, "fp32_backward_pass_ms": bwd_g, "fp16_forward_pass_ms": fwd_g16,
        "updates_per_pass": U, "fp32_forward_updates_per_s": U / (fwd_g / 1e3),
        "fp32_forward_GBps_21B": U * 21 / (fwd_g / 1e3) / 1e9,
        "fp32_forward_frac_of_hbm": U * 21 / (fwd_g / 1e3) / 1e9 / load_peaks()[0],
        "fp32_backward_GBps_17B": U * 17 / (bwd_g / 1e3) / 1e9}
    del cost, m, am, sc, gin, ch, mh, jg, eg
    f0 = torch.randn((1, 32, 384, 512), device=dev)
    f1 = torch.randn((1, 32, 384, 512), device=dev)
    flow = timed(lambda: ops.flow_forward(f0, f1, 64))
    cu, cv, us, vs = ops.flow_forward(f0, f1, 64)
    flow_b = timed(lambda: ops.flow_backward(f0, f1, 64, cu, cv, us, vs))
    flow_rate = 384 * 512 * 65 * 65 * 32 / (flow / 1e3)
    out["flow_sad_384x512_C32_w65"] = {"forward_ms": flow, "backward_ms": flow_b,
                                       "forward_G_absdiff_per_s": flow_rate / 1e9,
                                       "forward_fp32_issue_frac": fp32_issue_frac(flow_rate)}
    del cu, cv, us, vs
    flow2 = timed(lambda: ops.flow_forward(f0, f1, 216), n=1)
    cu, cv, us, vs = ops.flow_forward(f0, f1, 216)
    flow2_b = timed(lambda: ops.flow_backward(f0, f1, 216, cu, cv, us, vs), n=1)
    out["flow_sad_384x512_C32_w217_one_call"] = {"forward_ms": flow2, "backward_ms": flow2_b}
    del cu, cv, us, vs, f0, f1
    # flow BP (bp_op_cuda.py:100-117) on a 384x512 two-component volume,
    # 65 labels, 3 iterations, inference: the reference's u-then-v order
    # against u and v as one batch
    from bpl_gb300.layers.stereo import BP, coarse_to_fine
    pvf = torch.softmax(torch.randn((1, 2, 384, 512, 65), device=dev), dim=-1)
    ew = torch.ones((1, 4, 384, 512), device=dev)
    with torch.no_grad():
        seq = BP(dev, None, 3, 65, 3, mode_inference="wta")
        joint = BP(dev, None, 3, 65, 3, mode_inference="wta", joint_flow=True)
        t_seq = timed(lambda: seq(pvf, ew))
        t_joint = timed(lambda: joint(pvf, ew))
    out["flow_bp_384x512x65_3it"] = {"reference_order_ms": t_seq, "joint_ms": t_joint}
    del pvf, ew
    # coarse-to-fine glue (stereo.py:104-113) into the full-size volume
    bc = torch.softmax(torch.randn((1, H // 2, W // 2, L // 2), device=dev), dim=-1)
    pvl = torch.softmax(torch.randn((1, H, W, L), device=dev), dim=-1)
    glue = timed(lambda: coarse_to_fine(bc, pvl))
    out[f"coarse_to_fine_{H // 2}x{W // 2}x{L // 2}_to_{H}x{W}x{L}"] = {
        "ms": glue, "GBps": (8 * H * W * L + bc.numel() * 4) / (glue / 1e3) / 1e9}
    del bc, pvl
    f0 = torch.randn((1, 64, H, W), device=dev)
    f1 = torch.randn((1, 64, H, W), device=dev)
    sad = timed(lambda: ops.sad_forward(f0, f1, 0, L - 1))
    vol = ops.sad_forward(f0, f1, 0, L - 1)
    sad_b = timed(lambda: ops.sad_backward(f0, f1, 0, L - 1, vol))
    sad_rate = H * W * L * 64 / (sad / 1e3)
    # backward: two sign-gather terms (df0 and df1) per volume entry and channel
    sad_b_rate = 2 * H * W * L * 64 / (sad_b / 1e3)
    out[f"stereo_sad_{H}x{W}_C64_D{L}"] = {"forward_ms": sad, "backward_ms": sad_b,
                                            "forward_G_absdiff_per_s": sad_rate / 1e9,
                                            "forward_fp32_issue_frac": fp32_issue_frac(sad_rate),
                                            "forward_GBps": (4 * 2 * 64 * H * W + 4 * H * W * L) / (sad / 1e3) / 1e9,
                                            "backward_G_terms_per_s": sad_b_rate / 1e9}
    return out


def run_reference_gpu_ops(ours_fwd_ms, ours_bwd_ms, ours_step_ms):
    """The reference's own CUDA op (ops/lbp_stereo, rebuilt on this machine
    from the copy tests/golden/prepare_reference.sh makes under
    baseline/_ref) timed on the full-size workload at B=1: ITERS in-place
    forward_minsum passes and ITERS backward_minsum calls, as its layer runs
    them (message_passing_op_cuda.py:161-168), beside this library's
    per-pass times.  Reported as unavailable when the copy is absent or does
    not build within the time limit."""
    import torch
    ref_ops = os.path.join(ROOT, "baseline", "_ref", "ops")
    if not os.path.isdir(ref_ops):
        return {"unavailable": "reference copy absent (baseline/_ref/ops; tests/golden/prepare_reference.sh)"}
    t = time.perf_counter()
    r = subprocess.run([sys.executable, "-c", "import make_golden; make_golden.build_reference(names=['ref_lbp_stereo'])"],
                       cwd=os.path.join(ROOT, "tests", "golden"), capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        return {"unavailable": "reference build failed: " + r.stderr.strip().splitlines()[-1][:200]}
    build_s = time.perf_counter() - t
    import make_golden
    st = make_golden.load("ref_lbp_stereo")
    dev = torch.device("cuda", 0)
    prob, edge, _ = synth_inputs(torch, dev, 0)
    cost = (-prob).contiguous()
    jump = torch.zeros((1, 4, 6, H, W), device=dev)
    jump[:, :, 1] = 0.5
    jump[:, :, 2] = 0.1
    jump[:, :, 4] = 0.1
    jump[:, :, 5] = 0.5
    gin = torch.randn((1, 4, H, W, L), device=dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def run():
        m = torch.zeros((1, 4, H, W, L), device=dev)
        a, b, c = ev(), ev(), ev()
        a.record()
        saved = []
        for _ in range(ITERS):
            m, am, sc = st.forward_minsum(cost, jump, edge, m, DELTA)
            saved.append((am, sc))
        b.record()
        for am, sc in saved:
            st.backward_minsum(cost, jump, edge, gin, m, am, sc)
        c.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b), b.elapsed_time(c)

    run()  # warm-up
    f, bw = run()
    step = f + bw
    return {"op": "ops/lbp_stereo forward_minsum / backward_minsum (the reference's CUDA kernels, built here with "
                  "nvcc 13 for sm_103)", "B": 1, "H": H, "W": W, "L": L, "iters": ITERS,
            "reference_forward_pass_ms": f / ITERS, "reference_backward_pass_ms": bw / ITERS,
            "reference_step_ms": step,
            "ours_forward_pass_ms": ours_fwd_ms, "ours_backward_pass_ms": ours_bwd_ms,
            "ours_layer_step_ms": ours_step_ms,
            "speedup_ops": step / (ITERS * (ours_fwd_ms + ours_bwd_ms)),
            "speedup_layer_step": step / ours_step_ms, "reference_build_s": build_s}


def fp32_issue_frac(absdiff_per_s):
    """Fraction of the FP32 issue bound of a SAD kernel: each abs-diff term is
    two FP32 instructions (a subtract and an add of its absolute value), at
    128 FP32 lanes per SM per clock, at the device's maximum SM clock."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    bound = sms * 128 * 2.07e9 / 2
    return absdiff_per_s / bound


def cpu_sample_inputs(wc=CPU_CROP_W):
    import numpy as np
    import cases
    g = cases.rng(5)
    cost = cases.random_cost(g, 1, H, wc, L)
    jump = cases.stereo_taps(1, H, wc, 0.1, 0.5)
    edge = cases.edge_weights(g, 1, H, wc)
    msgs = np.zeros((1, 4, H, wc, L), np.float32)
    gin = g.normal(0, 1, size=(1, 4, H, wc, L)).astype(np.float32)
    return cost, jump, edge, msgs, gin


def cpu_pass(inputs, threads):
    """One forward pass + reference adjoint with the oracle (the reference
    has no CPU implementation of this path)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    cost, jump, edge, msgs, gin = inputs
    m, am, sc = oracle.lbp_forward(0, cost, jump, edge, msgs, DELTA, threads=threads)
    oracle.lbp_backward_ref(0, jump, edge, gin, m, am, sc, threads=threads)


def cpu_baseline_sample():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    inp = cpu_sample_inputs()
    t = time.perf_counter()
    cpu_pass(inp, threads)
    dt = time.perf_counter() - t
    U = 2 * L * edges(H, CPU_CROP_W)
    return {"value": U / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"oracle (C++/OpenMP, FP32 emulation forward + double reference adjoint), one pass "
                      f"forward+backward on a {H}x{CPU_CROP_W}x{L} crop of the workload, {dt:.2f} s",
            "max_threads": oracle.max_threads()}


def run_reference(args):
    """The reference has no CPU implementation of the path; its arithmetic is
    timed through the oracle port on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    inp = cpu_sample_inputs()
    for _ in range(args.warmup):
        cpu_pass(inp, threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        cpu_pass(inp, threads)
    dt = time.perf_counter() - t
    U = 2 * L * edges(H, CPU_CROP_W)
    value = U * args.steps / dt
    sample = (f"oracle port of the reference recurrence (C++/OpenMP), per step one pass forward+backward on a "
              f"{H}x{CPU_CROP_W}x{L} crop of the workload")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "stereo BP-Layer forward+backward, 376x1240x192, 3 iterations, FP32",
                   "B": 1, "H": H, "W": W, "L": L, "iters": ITERS, "delta": DELTA, "cpu_crop_w": CPU_CROP_W},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_ncu_case(args):
    """Small cases for detailed ncu captures, inside a profiler range (the
    second run of each): the layer's batched adjoint of ITERS passes (packed
    taps) at 256x512x192, LBP forward and reference adjoint at 256x512x192
    (cost 100 MB, messages 400 MB: larger than L2, well under the capture
    size limit), the exact adjoint's message-gradient assembly, the belief
    epilogue, SAD at 384x512 C=64 D=192, the flow SAD at 384x512 C=32,
    window +-32, the coarse-to-fine glue into 256x512x192, the slot
    broadcast of a 256x512x192 volume, the semantic pixel-pairwise
    forward at 512x1024, L=19 (the layer's two pairwise planes), the FP16
    stereo forward at 256x512x192, the semantic global forward at
    512x1024, L=19, and the epilogue kernels (cost from the 384x512x192
    SAD volume, disparity from the FP16 messages)."""
    import torch
    from bpl_gb300 import ops
    import cases
    dev = torch.device("cuda", 0)
    h, w = 256, 512
    prob, edge, _ = synth_inputs(torch, dev, 3, H=h, W=w)
    cost = (-prob).contiguous()
    jump = torch.from_numpy(cases.stereo_taps(1, h, w, 0.1, 0.5)).to(dev)
    gin = torch.randn((1, 4, h, w, L), device=dev)
    m = torch.zeros((1, 4, h, w, L), device=dev)
    T = torch.ones(1, device=dev)
    f0 = torch.randn((1, 64, 384, 512), device=dev)
    f1 = torch.randn((1, 64, 384, 512), device=dev)
    g0 = torch.randn((1, 32, 384, 512), device=dev)
    g1 = torch.randn((1, 32, 384, 512), device=dev)
    bc = torch.rand((1, h // 2, w // 2, L // 2), device=dev)
    pvl = torch.rand((1, h, w, L), device=dev)
    pcost = -torch.softmax(torch.randn((1, 2 * h, 2 * w, 19), device=dev), dim=-1)
    pjp = torch.rand((2, 2 * h, 2 * w, 19, 19), device=dev)
    pedge = torch.ones((1, 4, 2 * h, 2 * w), device=dev)
    pm = torch.zeros((1, 4, 2 * h, 2 * w, 19), device=dev)
    # FP16 storage (the lean stereo kernel) and the semantic global form
    ch = ops.to_half_padded(cost, L)
    mh = torch.zeros((1, 4, h, w, ops.padded_labels(L)), dtype=torch.float16, device=dev)
    gP = torch.rand((1, 4, 19, 19), device=dev)
    gm = torch.zeros((1, 4, 2 * h, 2 * w, 19), device=dev)
    gh = ops.to_half_padded(gin, L)
    # the adjoint as the layer's step runs it: the layer's packed taps
    # ([offset, L2, L1, 0, L1, L2] from the L1/L2 affinities) and the ITERS
    # passes' indices in one launch, the cost gradient added into a buffer
    aff = torch.zeros((1, 4, 3, h, w), device=dev)
    aff[:, :, :2] = 0.1
    aff[:, :, 2] = 0.5
    lt = ops.pack_taps(aff, torch.zeros((1, 4, h, w), device=dev))
    m3 = torch.zeros((1, 4, h, w, L), device=dev)
    am3 = torch.empty((ITERS, 1, 4, h, w, L), dtype=torch.uint8, device=dev)
    sc3 = torch.empty((ITERS, 1, 4, h, w), device=dev)
    for k in range(ITERS):
        ops.lbp_forward(ops.LBP_STEREO, cost, lt, edge, m3, DELTA, argmin_dtype=torch.uint8, argmin=am3[k],
                        scale=sc3[k])
    gc3 = torch.zeros((1, h, w, L), device=dev)
    for it in range(2):
        if it == 1:
            torch.cuda.synchronize()
            torch.cuda.profiler.start()
        ops.lbp_backward_passes(ops.LBP_STEREO, lt, edge, gin, m3, am3, sc3, L=L, grad_cost_into=gc3,
                                cost_sign=-1.0, layer_taps=True)
        m, am, sc = ops.lbp_forward(ops.LBP_STEREO, cost, jump, edge, m, DELTA, argmin_dtype=torch.uint8)
        ops.lbp_backward(ops.LBP_STEREO, jump, edge, gin, m, am, sc, copy_grad_messages=False)
        ops.lbp_backward(ops.LBP_STEREO, jump, edge, gin, m, am, sc, mode="exact")
        b = ops.beliefs_forward(m, cost, T)
        ops.beliefs_backward(m, cost, T, b, prob)
        vol = ops.sad_forward(f0, f1, 0, L - 1)
        ops.sad_backward(f0, f1, 0, L - 1, vol)
        cu, cv, us, vs = ops.flow_forward(g0, g1, 64)
        ops.flow_backward(g0, g1, 64, cu, cv, us, vs)
        ops.upsample_add_beliefs(bc, pvl, 0.5)
        ops.broadcast_slots(cost)
        ops.lbp_forward(ops.LBP_SEM_PIXEL_LAYER, pcost, pjp, pedge, pm, 19, argmin_dtype=torch.uint8)
        _, amh, _ = ops.lbp_forward_f16(ops.LBP_STEREO, ch, jump, edge, mh, DELTA, L, argmin_dtype=torch.uint8)
        ops.lbp_backward_passes(ops.LBP_STEREO, jump, edge, gh, mh, amh.unsqueeze(0), None, L=L)
        ops.lbp_forward(ops.LBP_SEM_GLOBAL, pcost, gP, pedge, gm, 19, argmin_dtype=torch.uint8)
        ops.cost_from_sad(vol, 1.0, half=True)
        ops.messages_argmin(mh, ch, L)
        torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"ncu_case": f"{h}x{w}x{L}", "updates_per_pass": L * edges(h, w)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp16", action="store_true", help="skip the FP16-storage leg")
    ap.add_argument("--no-recompute", action="store_true", help="skip the argmin-recompute leg")
    ap.add_argument("--ncu-case", action="store_true", help="small case for ncu captures")
    ap.add_argument("--no-serving", action="store_true", help="skip the served-stream leg")
    ap.add_argument("--serving-only", action="store_true", help="run only the served-stream leg")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the per-config error against the FP64 oracle")
    ap.add_argument("--accuracy-only", action="store_true")
    ap.add_argument("--no-other", action="store_true", help="skip the other configurations' op timings")
    ap.add_argument("--other-only", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip timing the reference's own CUDA op (built from baseline/_ref)")
    ap.add_argument("--serve-requests", type=int, default=40)
    ap.add_argument("--serve-loads", type=float, nargs="+", default=[0.5, 1.0, 2.0, 4.0],
                    help="offered arrival rates as multiples of the plain per-request capacity")
    args = ap.parse_args()
    if args.ncu_case:
        run_ncu_case(args)
    elif args.serving_only:
        print(json.dumps(run_serving(args)))
    elif args.accuracy_only:
        print(json.dumps(run_accuracy()))
    elif args.other_only:
        print(json.dumps(run_other_configs()))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
