"""Continuous-batching request loop over the batched ragged engine.

Requests are independent 2-D runs of the ensemble type (bonded-ice
indentations and granular column collapses) that arrive over time, each with
its own particle count and step count. The loop keeps every admitted solve's
state on the device and advances all of them together in fixed-length step
blocks (one conditional CUDA graph launch each):

* admission: arrived requests are admitted first-come first-served while the
  HBM footprint of the live solves plus the newcomer stays within the budget
  (the engine itself is sized to the budget once);
* joining: an admitted request joins at the next step block (the block's first
  rebuild sorts it in);
* finishing: a request that has taken its steps is frozen on the device by its
  step limit; after the block its ledger (and optionally its state) is read in
  one read-back for all finishers, and it retires; its memory is reclaimed by
  the next block's compaction.

Reported: p50 / p95 / p99 time-to-completion (arrival to result), aggregate
particle-steps/s, queueing and occupancy figures.
"""

from __future__ import annotations

import json
import math
import time
from collections import deque
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np
import torch

from .batch import Batch, BatchConfig, ensemble_case


@dataclass
class Request:
    index: int
    arrival: float          # seconds after the trace start
    spec: object            # EnsembleSpec
    n: int = 0
    steps: int = 0
    admitted: float = math.nan
    done: float = math.nan
    iid: int = -1
    eval0: int = 0
    footprint: int = 0
    ledger: dict = field(default_factory=dict)
    state: dict | None = None


def mean_log_uniform(lo: float, hi: float) -> float:
    return (hi - lo) / math.log(hi / lo)


def make_trace(*, duration: float, rate: float | None = None, capacity: float | None = None,
               load: float = 0.8, n_min: int = 500, n_max: int = 200_000, s_min: int = 1000,
               s_max: int = 50_000, seed: int = 0, max_requests: int | None = None) -> list[Request]:
    """Poisson arrivals over ``duration`` seconds. The rate is ``rate`` or
    ``load`` x ``capacity`` (particle-steps/s) / E[N S] of the request mix."""
    if rate is None:
        if capacity is None:
            raise ValueError("give rate or capacity")
        rate = load * capacity / (mean_log_uniform(n_min, n_max) * mean_log_uniform(s_min, s_max))
    rng = np.random.default_rng(seed)
    times = []
    t = rng.exponential(1.0 / rate)
    while t < duration and (max_requests is None or len(times) < max_requests):
        times.append(t)
        t += rng.exponential(1.0 / rate)
    specs = ensemble_case(len(times), seed=seed + 7, n_min=n_min, n_max=n_max, steps=s_min, steps_max=s_max)
    return [Request(k, float(times[k]), specs[k], n=specs[k].n, steps=specs[k].steps) for k in range(len(times))]


def engine_for_budget(budget_bytes: int, *, keys_per_particle: float = 3.0, max_instances: int = 8192,
                      precision: int = 32, rebuild_every: int = 0) -> tuple[BatchConfig, float, float]:
    """Largest engine within the HBM budget, and its bytes per particle / per key."""
    def cfg(n):
        return BatchConfig(particle_capacity=int(n), key_capacity=int(max(64, keys_per_particle * n)),
                           max_instances=max_instances, precision=precision, rebuild_every=rebuild_every)
    a, b = cfg(1_000_000).bytes(), cfg(2_000_000).bytes()
    per = (b - a) / 1_000_000  # bytes per particle incl. its share of keys
    k1 = BatchConfig(particle_capacity=1_000_000, key_capacity=3_000_000, max_instances=max_instances,
                     precision=precision).bytes()
    k2 = BatchConfig(particle_capacity=1_000_000, key_capacity=4_000_000, max_instances=max_instances,
                     precision=precision).bytes()
    per_key = (k2 - k1) / 1_000_000
    per_particle = per - keys_per_particle * per_key
    fixed = a - 1_000_000 * per
    n = int((budget_bytes - fixed) / per)
    while n >= 1024 and cfg(n).bytes() > budget_bytes:  # alignment padding
        n -= 1024
    if n < 1024:
        raise ValueError("HBM budget too small")
    return cfg(n), per_particle, per_key


def serve(trace: list[Request], *, budget_bytes: int, block: int = 100, rebuild_every: int = 0,
          precision: int = 32, keep_state: bool = False, lookahead: float = 2.0, workers: int = 4,
          time_limit: float | None = None, log=None) -> dict:
    """Run the trace in real time; returns the report (requests carry their results)."""
    cfg, per_particle, per_key = engine_for_budget(budget_bytes, precision=precision,
                                                   rebuild_every=rebuild_every)
    b = Batch(cfg)
    pool = ThreadPoolExecutor(max_workers=workers)
    pending = deque(sorted(trace, key=lambda r: r.arrival))
    builds: dict[int, object] = {}
    waiting: deque[Request] = deque()
    live: dict[int, Request] = {}
    done: list[Request] = []
    used = 0
    evals = 0
    peak_live_particles = peak_used = 0
    steps_run = 0
    blocks = 0
    busy = 0.0
    input_waits = 0
    processed = 0  # particle-steps advanced (finished or not)
    t0 = time.perf_counter()

    def clock():
        return time.perf_counter() - t0

    while pending or waiting or live or builds:
        now = clock()
        if time_limit is not None and now > time_limit:
            break
        # build inputs ahead of their arrival (host-side synthetic inputs)
        while pending and pending[0].arrival <= now + lookahead:
            r = pending.popleft()
            builds[r.index] = (r, pool.submit(r.spec.build))
        # arrived requests whose inputs are ready join the FIFO queue
        for idx in sorted(builds, key=lambda i: builds[i][0].arrival):
            r, fut = builds[idx]
            if r.arrival > now:
                break
            if not fut.done():
                input_waits += 1
                break
            r.inst = fut.result()
            r.n = r.inst.n
            r.footprint = int(r.inst.n * per_particle + r.inst.keys * per_key)
            waiting.append(r)
            del builds[idx]
        # first-come first-served admission under the HBM budget
        while waiting and used + waiting[0].footprint <= budget_bytes:
            r = waiting.popleft()
            try:
                r.iid = b.admit(r.inst)
            except RuntimeError:  # capacity held by retired solves: compact, then retry once
                b.step(0)
                try:
                    r.iid = b.admit(r.inst)
                except RuntimeError:
                    waiting.appendleft(r)
                    break
            b.set_steps(r.iid, r.steps)
            r.eval0 = evals
            r.admitted = clock()
            del r.inst
            live[r.iid] = r
            used += r.footprint
        if not live:
            nxt = min([r.arrival for r, _ in builds.values()] + ([pending[0].arrival] if pending else []),
                      default=None)
            if nxt is not None:
                time.sleep(max(0.0, min(nxt - clock(), 0.05)))
            continue
        processed += sum(r.n * max(0, min(block, r.steps - (evals - r.eval0))) for r in live.values())
        peak_live_particles = max(peak_live_particles, sum(r.n for r in live.values()))
        peak_used = max(peak_used, used)
        ts = clock()
        b.step(block)
        torch.cuda.synchronize()
        busy += clock() - ts
        evals += block
        steps_run += block
        blocks += 1
        finished = [r for r in live.values() if evals - r.eval0 >= r.steps]
        if finished:
            ledgers = b.ledgers([r.iid for r in finished])
            for r, led in zip(finished, ledgers):
                if keep_state:
                    r.state = b.read(r.iid)
                r.ledger = led
                b.retire(r.iid)
                r.done = clock()
                used -= r.footprint
                del live[r.iid]
                done.append(r)
        if log and blocks % 50 == 0:
            log(f"t={clock():7.2f}s live={len(live)} waiting={len(waiting)} done={len(done)}")
    wall = clock()
    pool.shutdown(wait=False, cancel_futures=True)
    lat = np.array([r.done - r.arrival for r in done]) if done else np.zeros(1)
    wait = np.array([r.admitted - r.arrival for r in done]) if done else np.zeros(1)
    work = float(sum(r.n * r.steps for r in done))
    info = b.info()
    return {
        "requests": len(trace), "completed": len(done),
        "wall_s": wall, "busy_s": busy,
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                      "p99": float(np.percentile(lat, 99)), "mean": float(lat.mean()), "max": float(lat.max())},
        "queue_wait_s": {"p50": float(np.percentile(wait, 50)), "p99": float(np.percentile(wait, 99))},
        "particle_steps_per_s": work / wall if wall > 0 else 0.0,
        "particle_steps_per_s_busy": work / busy if busy > 0 else 0.0,
        "completed_particle_steps": work,
        "processed_particle_steps_per_s_busy": processed / busy if busy > 0 else 0.0,
        "blocks": blocks, "block_steps": block, "batch_steps": steps_run,
        "peak_live_particles": peak_live_particles, "peak_footprint_gb": peak_used / 1e9,
        "budget_gb": budget_bytes / 1e9, "engine_bytes": info["bytes"], "rebuilds": info["rebuilds"],
        "bytes_per_particle": per_particle, "bytes_per_key": per_key,
        "input_build_waits": input_waits,
        "status_errors": sum(1 for r in done if r.ledger.get("status", 0) != 0),
        "status_examples": [{"index": r.index, "kind": r.spec.kind, "n": r.n, "steps": r.steps,
                             "young": r.spec.young, "status": int(r.ledger.get("status", 0))}
                            for r in done if r.ledger.get("status", 0) != 0][:12],
        "done": done,
    }


def calibrate(*, seconds: float, budget_bytes: int, block: int, seed: int, n_min: int, n_max: int, s_min: int,
              s_max: int, guess: float = 1e10) -> float:
    """Capacity of the engine on this request mix: particle-steps/s advanced
    while requests are offered faster than it can serve them."""
    trace = make_trace(duration=seconds, capacity=guess, load=2.0, seed=seed + 1000, n_min=n_min, n_max=n_max,
                       s_min=s_min, s_max=s_max)
    rep = serve(trace, budget_bytes=budget_bytes, block=block, time_limit=seconds)
    return rep["processed_particle_steps_per_s_busy"]


def main(args) -> dict:
    capacity = args.capacity
    budget = int(args.budget_gb * 1e9)
    calibrated = capacity is None
    if calibrated:
        capacity = calibrate(seconds=args.calibrate_seconds, budget_bytes=budget, block=args.block, seed=args.seed,
                             n_min=args.n_min, n_max=args.n_max, s_min=args.s_min, s_max=args.s_max)
    trace = make_trace(duration=args.duration, capacity=capacity, load=args.load, seed=args.seed,
                       n_min=args.n_min, n_max=args.n_max, s_min=args.s_min, s_max=args.s_max)
    rep = serve(trace, budget_bytes=budget, block=args.block, rebuild_every=args.rebuild_every,
                time_limit=args.duration * 3 + 60)
    rep.pop("done")
    out = {"metric": "served time-to-completion and particle-steps/s", "load": args.load,
           "capacity_particle_steps_per_s": capacity, "capacity_measured": calibrated,
           "arrival_rate_per_s": len(trace) / args.duration, "duration_s": args.duration, **rep}
    print(json.dumps(out))
    return out
