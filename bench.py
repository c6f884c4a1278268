"""Benchmark of the 2-D Hertz-Mindlin DEM step on GB300 (one JSON line on rank 0).

Workload: the seeded 1,048,576-disc polydisperse settling case (radii
U[0.8, 1.2] mm, rho 2500, E 70 GPa, nu 0.25, mu 0.5, e 0.8, jittered grid at
area fraction 0.55, four walls, gravity, dt = 0.2 Rayleigh time), FP32
contacts with compensated sums and an FP64 ledger. A bench step is one
velocity-Verlet DEM step of all discs; the run's state is device-resident and
L2 is flushed (a buffer larger than L2 written, then read) before every timed
step, outside its CUDA-event bracket.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU: the path does not shard ("replicas only"): under
torchrun every rank runs its own replica (seeded by rank) and the line reports
the aggregate particle-steps/s over the slowest rank's time (weak scaling).
``--impl reference`` times the CPU oracle (the FP64 restatement of the
reference's algorithm, oracle/hm2d.py) on a bounded sample of the same
workload on every host core (one slab of discs per core).
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "particle-steps/s @1M discs"
UNIT = "particle-steps/s"
N_SIDE = 1024
L2_FLUSH_BYTES = 256 << 20
FALLBACK_HBM_GBS = 6800.0


def _args():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10000, help="timed DEM steps (the full 10,000-step run)")
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--cpu-sample-steps", type=int, default=100)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-ensemble and served-trace leg")
    return ap.parse_args()


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, device) -> float:
    """The largest value over all ranks (the slowest rank's time); the value
    itself when no process group is running."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world: int, units_per_rank: int, steps: int, seconds: float) -> float:
    """Whole-job throughput: every rank's units over the slowest rank's time."""
    return world * units_per_rank * steps / seconds


def workload_config(seed: int = 0) -> dict:
    return {"workload": "2-D polydisperse Hertz-Mindlin disc settling, 1,048,576 discs "
                        "(1024x1024 jittered grid, area fraction 0.55, 4 walls, gravity), "
                        "radii U[0.8,1.2] mm, E 70 GPa, nu 0.25, mu 0.5, e 0.8, dt 0.2 Rayleigh",
            "discs": N_SIDE * N_SIDE, "seed": seed, "precision": "fp32 contacts on fp32 cell offsets with fp32 rounding remainders, compensated sums, fp64 ledger",
            "l2": "flushed before every timed step (256 MiB written, another 256 MiB read)",
            "parallelism": "replicas"}


# ----------------------------------------------------------------- CPU side
def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _slab_rate(job) -> tuple[int, float]:
    """One worker: the oracle on one slab of discs, `steps` timed steps after a
    priming half kick and two warm-up steps. Returns (discs, seconds)."""
    arrays, params, steps = job
    from oracle.hm2d import HM2DOracle, HMParams
    o = HM2DOracle(*arrays, HMParams(**params))
    o.prime()
    o.step(2)
    t0 = time.perf_counter()
    o.step(steps)
    return len(arrays[0]), time.perf_counter() - t0


def cpu_oracle_rate(steps: int, *, n_side: int = N_SIDE, workers: int | None = None) -> dict:
    """Time the numpy FP64 oracle on the same workload (bounded sample) with
    every host core: the discs are cut into as many vertical slabs of equal
    disc count as there are cores, and each slab is stepped by the unchanged
    oracle in its own process (spawned, never forked). Slabs exchange nothing,
    so contacts across slab faces are not evaluated (a negligible share of the
    work in this dilute gas). Rate = all discs x steps / the slowest slab's time."""
    import multiprocessing

    import numpy as np

    from tensordem_gb300.hm2d import granular_gas_case
    cfg, st = granular_gas_case(n_side, seed=0)
    params = dict(young=cfg.young, poisson=cfg.poisson, restitution=cfg.restitution, mu=cfg.mu,
                  mu_wall=cfg.mu_wall, dt=cfg.dt, gravity=tuple(cfg.gravity), box=tuple(cfg.box), skin=cfg.skin)
    p = max(1, min(workers or host_cores(), cfg.n))
    slabs = np.array_split(np.argsort(st["pos"][:, 0], kind="stable"), p)
    keys = ("pos", "vel", "omega", "radius", "mass", "inertia")
    jobs = [(tuple(np.ascontiguousarray(st[k][s]) for k in keys), params, steps) for s in slabs]
    t0 = time.perf_counter()
    with multiprocessing.get_context("spawn").Pool(p) as pool:
        done = pool.map(_slab_rate, jobs)
    wall = time.perf_counter() - t0
    discs = sum(n for n, _ in done)
    slowest = max(s for _, s in done)
    return {"value": discs * steps / slowest, "unit": UNIT, "cores": p, "kind": "port",
            "sample": f"{steps} velocity-Verlet steps of the {discs:,}-disc case after a 3-step warm-up, "
                      f"numpy FP64 oracle (oracle/hm2d.py) on {p} host cores: {p} vertical slabs of equal "
                      f"disc count, one spawned process each, no exchange across slab faces; slowest slab "
                      f"{slowest:.2f} s, {wall:.1f} s with process start-up"}


def run_reference(a) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    steps = max(1, min(a.steps, a.cpu_sample_steps))
    cb = cpu_oracle_rate(steps)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * (N_SIDE * N_SIDE) / cb["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(),
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU side
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profiled_traffic() -> float | None:
    """DRAM bytes per step-kernel launch from the committed ncu summary (1M discs)."""
    try:
        with open(os.path.join(ROOT, "profiles", "hm_step_1M_traffic.json")) as f:
            return float(json.load(f)["dram_bytes_per_launch"])
    except Exception:
        return None


def algorithmic_bytes(n: int, head_bytes: int, contact_sides: int, remainder: bool = False) -> int:
    """Bytes one step must move in this layout: state read + write (pos, vel:
    2 x 2 x 16 B per disc), the list head (16 B per disc), the position
    remainder when the engine keeps one (8 B read + 8 B write per disc) and
    the tangential history of every touching contact side (8 B read + 8 B
    write)."""
    return n * (64 + head_bytes + (16 if remainder else 0)) + 16 * contact_sides


def cell_list_bytes(n: int, k: int, c: int, b: int, r: float) -> float:
    """The hot-path byte model N*64 + K*4 + C*16 + B*20 + 96*N/R: particle
    state read and written, one 4-byte candidate index per candidate pair, 16 B
    of history per active contact, 20 B per bond, and the rebuild's sort
    traffic (96 B per particle) spread over the rebuild interval R."""
    return n * 64 + k * 4 + c * 16 + b * 20 + (96.0 * n / r if r > 0 else 0.0)


def timed_steps(eng, steps, warmup, flush_l2, stream, dev):
    """Warm-up steps, then `steps` timed steps: L2 flushed (untimed), the step
    kernel in its own event bracket, and a list rebuild, when the device says
    one is due, in a bracket of its own. Returns (step ms, rebuild ms, wall s)."""
    import torch
    # the warm-up runs right before the timed steps in the same loop shape: a
    # first launch after an idle spell takes ~5x longer
    for _ in range(max(3, warmup)):
        flush_l2()
        eng.step_kernel()
        if eng.rebuild_pending():
            eng.rebuild()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    rebuild_evs = []
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for e0, e1 in evs:
        flush_l2()
        e0.record(stream)
        eng.step_kernel()
        e1.record(stream)
        if eng.rebuild_pending():
            r0 = torch.cuda.Event(enable_timing=True)
            r1 = torch.cuda.Event(enable_timing=True)
            r0.record(stream)
            eng.rebuild()
            r1.record(stream)
            rebuild_evs.append((r0, r1))
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    eng.check()
    return ([e0.elapsed_time(e1) for e0, e1 in evs], [r0.elapsed_time(r1) for r0, r1 in rebuild_evs], wall)


def flushed_trial(eng, flush_l2, stream, dev, steps: int = 20) -> dict:
    """Choose the step-kernel variant under the timed loop's own conditions.

    The engine's autotuner times back-to-back steps, which at 1M discs run
    with the state resident in L2 (about 100 MB of a 129 MB L2); the timed
    loop flushes L2 before every step. Each variant (all bit-identical) runs
    `steps` flushed steps here and the fastest mean is kept. Returns the mean
    step-kernel microseconds per variant."""
    from tensordem_gb300 import _lib
    means = {}
    for v in range(int(_lib.lib().tdem_hm_num_variants())):
        eng.variant = v
        step_ms, _, _ = timed_steps(eng, steps, 3, flush_l2, stream, dev)
        means[v] = 1e3 * sum(step_ms) / len(step_ms)
    eng.variant = min(means, key=means.get)
    return means


def form_rate(seed, steps, warmup, flush_l2, stream, dev, *, precision=64, sum_precision=32,
              position_remainder=1) -> dict:
    """Another numeric form of the same kernels on the same workload and loop:
    the plain FP64 build, the FP32 build with FP64 per-particle sums, or the
    FP32 build without position remainders."""
    from dataclasses import replace

    from tensordem_gb300.hm2d import HM2D, granular_gas_case
    cfg, st = granular_gas_case(N_SIDE, seed=seed, precision=precision)
    cfg = replace(cfg, sum_precision=sum_precision, position_remainder=position_remainder)
    eng = HM2D(cfg, device=dev)
    eng.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
    eng.step(2)
    flushed_trial(eng, flush_l2, stream, dev, steps=8)
    step_ms, rebuild_ms, _ = timed_steps(eng, steps, warmup, flush_l2, stream, dev)
    total = sum(step_ms) + sum(rebuild_ms)
    return {"value": cfg.n * steps / (total / 1e3), "unit": UNIT, "steps": steps, "variant": eng.variant,
            "step_kernel_us_mean": 1e3 * sum(step_ms) / len(step_ms), "rebuilds": len(rebuild_ms),
            "note": ("precision=64 build of the same kernels (FP64 contacts, sums and ledger)" if precision == 64
                     else "FP32 contacts with FP64 per-particle force/torque sums" if sum_precision == 64
                     else "FP32 contacts, plain FP32 position offsets (no remainder pair)") +
                    ", same seeded 1,048,576-disc state and the same flushed per-step loop"}


ICE_STEPS = 2000


def ice_leg(seed: int, dev, peak: float) -> dict:
    """The bonded 1M-disc ice sheet (2048 x 512 hex lattice, 3.1M bonds,
    indenter): every disc carries its six bond forces every step, so this
    is the contact-dense counterpart of the settling gas. 2,000 steps in the
    conditional step graph (strain kernel, step kernel, rebuild IF), the
    variant autotuned and the graph built before the clock starts; the
    state and bond arrays (~350 MB) exceed L2, so no flush is needed."""
    import torch

    from tensordem_gb300.hm2d import HM2D, ice_sheet_case
    cfg, st, bonds, strength = ice_sheet_case(2048, 512, seed=seed, steps=ICE_STEPS)
    eng = HM2D(cfg, device=dev)
    eng.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
    eng.set_bonds(bonds, strength)
    eng.autotune(steps=10)
    eng.step(0)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    eng.step(ICE_STEPS, check=False)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    eng.check()
    ms = e0.elapsed_time(e1)
    led = eng.ledger()
    n, nb = cfg.n, len(bonds)
    # bytes a step must move: the gas step's 96 B per disc, two slot copies
    # per bond (partner word 4 B, reference vector 8 B, strength 4 B, history
    # 8 B read and 8 B written) and the strain (4 B written, 4 B read)
    alg = n * (96 + 8) + 2 * nb * 32
    us = 1e3 * ms / ICE_STEPS
    return {"workload": "bonded ice sheet, 2048 x 512 hex lattice (1,048,576 discs, 3,140,609 bonds), indenter "
                        "R = 2 m at 0.5 m/s, FP32 contacts and bonds, FP64 ledger; 2,000 graph-launched steps",
            "value": n * ICE_STEPS / (ms / 1e3), "unit": UNIT, "us_per_step": us, "variant": eng.variant,
            "bytes_per_step_model": alg, "achieved_gbs": alg / (us / 1e6) / 1e9,
            "frac": alg / (us / 1e6) / 1e9 / peak, "bonds": nb, "broken": led["broken"],
            "tool_work_J": led["tool_work"], "ledger_total_rel_work": led["total"] / max(led["tool_work"], 1e-300)}


BATCH_INSTANCES = 512
BATCH_STEPS = 1000
BATCH_SAMPLE = 64


def batched_leg(seed: int = 0, *, serve_seconds: float = 20.0, calibrate_seconds: float = 4.0) -> dict:
    """The metric's second half on this GPU, in this run.

    A seeded ensemble of the 4096-run mix's shape (half bonded-ice
    indentations, half granular column collapses, N log-uniform 100-20,000,
    mu U[0.3, 0.7], E log-uniform 1-70 GPa) cut to 512 runs x 1,000 steps: all
    of them solved in one batched engine (FP32 contacts, FP64 ledger), and a
    seeded sample of 64 of them solved one by one through the plain FP64
    single-solve engine (create, upload, steps, read-back each), extrapolated
    to the 512. Then a short served Poisson trace: requests of the same mix with
    N log-uniform 500-200,000 and S log-uniform 100-5,000 steps arrive for 20 s
    at 0.8 of the capacity measured by a 4 s saturated run, under a 150 GB HBM
    budget; p50 / p95 / p99 time-to-completion."""
    import numpy as np

    from tensordem_gb300 import ensemble, serve
    from tensordem_gb300.batch import ensemble_case
    specs = ensemble_case(BATCH_INSTANCES, seed=seed, steps=BATCH_STEPS)
    rng = np.random.default_rng(seed + 1)
    sample = sorted(rng.choice(len(specs), size=BATCH_SAMPLE, replace=False).tolist())
    rep, ledgers = ensemble.run_batched(specs, precision=32, autotune_steps=2)
    seq = ensemble.run_sequential_fp64(specs, sample)
    mean_s = float(np.mean([x["seconds"] for x in seq.values()]))
    one_by_one = len(specs) / (mean_s * len(specs))
    agree = ensemble.compare(ledgers, seq)
    budget = int(150e9)
    n_min, n_max, s_min, s_max, block = 500, 200_000, 100, 5000, 100
    capacity = serve.calibrate(seconds=calibrate_seconds, budget_bytes=budget, block=block, seed=seed,
                               n_min=n_min, n_max=n_max, s_min=s_min, s_max=s_max)
    trace = serve.make_trace(duration=serve_seconds, capacity=capacity, load=0.8, seed=seed, n_min=n_min,
                             n_max=n_max, s_min=s_min, s_max=s_max)
    srv = serve.serve(trace, budget_bytes=budget, block=block, time_limit=serve_seconds * 4 + 30)
    srv.pop("done")
    return {
        "workload": f"{BATCH_INSTANCES} runs x {BATCH_STEPS} steps of the mixed ensemble (half bonded-ice "
                    "indentations, half granular column collapses; N log-uniform 100-20,000; seed "
                    f"{seed}); served trace: Poisson arrivals for {serve_seconds:g} s at 0.8 of the measured "
                    f"capacity, N log-uniform {n_min}-{n_max}, S log-uniform {s_min}-{s_max}, 150 GB budget",
        "solves_per_s": rep["solves_per_s"],
        "one_by_one_fp64_solves_per_s": one_by_one,
        "one_by_one_sample": f"{BATCH_SAMPLE} of the {BATCH_INSTANCES} runs (seeded), mean {mean_s:.4f} s per "
                             "solve incl. create, upload, steps, read-back; extrapolated",
        "speedup": rep["solves_per_s"] / one_by_one,
        "particle_steps_per_s": rep["particle_steps_per_s"],
        "particles": rep["particles"], "instances_with_status": rep["instances_with_status"],
        "peak_load_rel_err_max": agree["peak_load_rel_err_max"],
        "ledger_total_rel_diff_max": agree["ledger_total_rel_diff_max"],
        "ledger_rel_diff_max_by_kind": agree["ledger_rel_diff_max_by_kind"],
        "ledger_normalisation": agree["ledger_normalisation"],
        "served": {"capacity_particle_steps_per_s": capacity, "requests": srv["requests"],
                   "completed": srv["completed"], "latency_s": srv["latency_s"],
                   "queue_wait_s": srv["queue_wait_s"], "particle_steps_per_s": srv["particle_steps_per_s"],
                   "status_errors": srv["status_errors"]},
    }


def run_ours(a) -> None:
    import numpy as np
    import torch

    from tensordem_gb300.hm2d import HM2D, granular_gas_case

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    cfg, st = granular_gas_case(N_SIDE, seed=rank)
    eng = HM2D(cfg, device=dev)
    eng.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
    tuning = eng.autotune(steps=10)
    eng.step(max(3, a.warmup))
    # L2 flush: write one buffer larger than L2, then read another, so the
    # cache is left holding clean, unrelated lines (no write-backs in the step)
    flush_w = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    flush_r = torch.ones(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def flush_l2():
        flush_w.fill_(1.0)
        flush_r.sum()

    stream = torch.cuda.current_stream(dev)
    trial = flushed_trial(eng, flush_l2, stream, dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clocks:
        step_ms, rebuild_ms, wall = timed_steps(eng, a.steps, a.warmup, flush_l2, stream, dev)
    kernel_ms = sum(step_ms) / len(step_ms)
    total_ms = sum(step_ms) + sum(rebuild_ms)
    if world > 1:
        total_ms = max_over_ranks(total_ms, dev)
        torch.distributed.barrier()
    led1 = eng.ledger()
    clk = clocks.summary()
    n = cfg.n
    value = aggregate_rate(world, n, a.steps, total_ms / 1e3)

    # candidate pairs K, touching contacts C (with stored history), bonds B
    # and the rebuild interval R of the run so far, for the byte models
    hist = eng.history()
    k_pairs = len(eng.pairs())
    c_contacts = len(hist)
    r_interval = led1["evals"] / max(1, led1["rebuilds"])
    alg = algorithmic_bytes(n, 16, 2 * c_contacts, remainder=cfg.precision == 32 and cfg.position_remainder == 1)
    peak, peak_kind = measured_peak()
    achieved = alg / (kernel_ms / 1e3) / 1e9
    traffic = profiled_traffic()
    sb = cell_list_bytes(n, k_pairs, c_contacts, 0, r_interval)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_step": alg,
                "cell_list_model": {"bytes_per_step": sb, "achieved": sb / (kernel_ms / 1e3) / 1e9,
                                 "frac": sb / (kernel_ms / 1e3) / 1e9 / peak,
                                 "N": n, "K": k_pairs, "C": c_contacts, "B": 0, "R": r_interval},
                "dram": None if traffic is None else {
                    "bytes_per_launch": traffic, "achieved": traffic / (kernel_ms / 1e3) / 1e9,
                    "frac": traffic / (kernel_ms / 1e3) / 1e9 / peak,
                    "note": "DRAM bytes of one ncu-captured launch: the new state stays in L2 during the "
                            "launch and is written back after it"}}

    # end to end through the C ABI with host buffers (rank-local)
    e2e_eng = HM2D(cfg, device=dev)
    e2e_eng.variant = eng.variant
    host = {k: np.ascontiguousarray(v) for k, v in st.items()}
    out_pos = np.empty((n, 2))
    out_vel = np.empty((n, 2))
    out_om = np.empty(n)
    flush_l2()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    e2e_eng.set_state(host["pos"], host["vel"], host["omega"], host["radius"], host["mass"], host["inertia"])
    e2e_eng.step(a.steps, check=False)
    e2e_eng.read_state_host(out_pos, out_vel, out_om)
    e2e_s = time.perf_counter() - t0
    e2e_eng.check()
    del e2e_eng
    if world > 1:
        e2e_s = max_over_ranks(e2e_s, dev)
    h2d = 8 * n * (2 + 2 + 1 + 1 + 1 + 1)
    d2h = 8 * n * (2 + 2 + 1)
    e2e = {"value": aggregate_rate(world, n, a.steps, e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": h2d / a.steps, "d2h_bytes_per_step": d2h / a.steps,
           "note": "one solve through tdem_hm_set_state/step/read_state with host arrays: upload, "
                   f"{a.steps} steps, download; L2 flushed before it"}

    fp64 = form_rate(rank, min(a.steps, 200), a.warmup, flush_l2, stream, dev, precision=64)
    sums64 = form_rate(rank, min(a.steps, 200), a.warmup, flush_l2, stream, dev, precision=32, sum_precision=64)
    plain32 = form_rate(rank, min(a.steps, 200), a.warmup, flush_l2, stream, dev, precision=32,
                        position_remainder=0)
    ice = ice_leg(rank, dev, peak) if (rank == 0 and world == 1 and not a.no_batched) else None
    batched = None
    if rank == 0 and world == 1 and not a.no_batched:
        del eng
        batched = batched_leg(0)
    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        cpu = cpu_oracle_rate(max(1, a.cpu_sample_steps))
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": total_ms / a.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": workload_config(), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": a.steps + 12 * len(rebuild_ms),
                "clocks": clk, "batched": batched,
                "extra": {"variant": led1["variant"], "graph": led1["graph"], "autotune_ms_per_10_steps": tuning,
                          "flushed_trial_us_per_step": trial,
                          "rebuilds_in_timed_region": len(rebuild_ms), "rebuild_ms_total": sum(rebuild_ms),
                          "step_kernel_us_mean": 1e3 * kernel_ms,
                          "step_kernel_us_median": 1e3 * statistics.median(step_ms),
                          "wall_s_timed_loop": wall,
                          "max_neighbors_seen": led1["max_neighbors"],
                          "touching_contacts_end": c_contacts, "fp64": fp64, "fp32_fp64_sums": sums64,
                          "fp32_no_position_remainder": plain32, "bonded_sheet_1M": ice}}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
