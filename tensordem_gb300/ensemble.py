"""Ensemble measurement: a mixed list of independent 2-D runs solved in one
batched engine, against the same runs one-by-one through the plain FP64
single-solve engine.

``python -m tensordem_gb300 ensemble`` (defaults: 4096 instances, 5000 steps
each, seed 0) admits every instance into one :class:`~tensordem_gb300.batch.Batch`
(FP32 contacts, FP64 ledger), advances them together in one conditional CUDA
graph launch, reads every ledger and retires them. The baseline runs a seeded
random sample of the same list, one at a time, through
:class:`~tensordem_gb300.hm2d.HM2D` at ``precision=64`` (create, upload,
steps, read back), and extrapolates its mean time to the whole list. The
sampled instances also give the FP32-vs-FP64 agreement of the batched results
(indenter peak load, energy ledger).
"""

from __future__ import annotations

import json
import math
import time

import numpy as np
import torch

from .batch import Batch, BatchConfig, ensemble_case


def _sync():
    torch.cuda.synchronize()


def run_batched(specs, *, precision=32, autotune_steps=2, variant=None, rebuild_every=0, keep=None):
    """Solve every spec in one batch. Returns (report, per-instance ledgers)."""
    t_build = time.perf_counter()
    insts = [s.build() for s in specs]
    t_build = time.perf_counter() - t_build
    steps = insts[0].steps
    if any(i.steps != steps for i in insts):
        raise ValueError("run_batched advances every instance by the same step count")
    n_tot = sum(i.n for i in insts)
    k_tot = sum(i.keys for i in insts)
    cfg = BatchConfig(particle_capacity=n_tot + 64, key_capacity=k_tot + 64,
                      max_instances=max(64, len(insts)), precision=precision, rebuild_every=rebuild_every)
    b = Batch(cfg)
    _sync()
    t0 = time.perf_counter()
    ids = [b.admit(i) for i in insts]
    _sync()
    t_admit = time.perf_counter() - t0
    tuning = None
    done = 0
    if variant is not None:
        b.variant = variant
    elif autotune_steps > 0:
        tuning = b.autotune(autotune_steps)
        done = autotune_steps * len(tuning)
    b.step(0)  # builds the step graph for the chosen variant (inside the wall time, outside the stepping time)
    t1 = time.perf_counter()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    b.step(steps - done)
    ev1.record()
    _sync()
    t_steps = time.perf_counter() - t1
    gpu_ms = ev0.elapsed_time(ev1)
    info = b.info()
    t2 = time.perf_counter()
    ledgers = {k: {"ledger": led} for k, led in enumerate(b.ledgers(ids))}
    for k in keep or ():
        ledgers[k].update(b.read(ids[k]))
    for iid in ids:
        b.retire(iid)
    _sync()
    t_read = time.perf_counter() - t2
    wall = time.perf_counter() - t0
    bad = [k for k, r in ledgers.items() if r["ledger"]["status"] != 0]
    rep = {
        "instances": len(insts), "steps": steps, "particles": n_tot, "keys": k_tot,
        "solve_wall_s": wall, "admit_s": t_admit, "step_wall_s": t_steps, "step_gpu_s": gpu_ms / 1e3,
        "read_retire_s": t_read, "build_host_s": t_build,
        "solves_per_s": len(insts) / wall, "particle_steps_per_s": n_tot * steps / wall,
        "particle_steps_per_s_stepping": n_tot * (steps - done) / (gpu_ms / 1e3),
        "rebuilds": info["rebuilds"], "variant": info["variant"], "graph": info["graph"],
        "device_bytes": info["bytes"], "instances_with_status": len(bad),
        "status_examples": [{"index": specs[k].index, "kind": specs[k].kind, "n": insts[k].n,
                             "young": specs[k].young, "status": int(ledgers[k]["ledger"]["status"]),
                             "evals": ledgers[k]["ledger"]["evals"]} for k in bad[:12]],
        "max_neighbors_seen": info["max_neighbors"],
        "autotune_ms": tuning,
    }
    return rep, ledgers


def run_sequential_fp64(specs, sample):
    """The sampled specs one at a time through the plain FP64 engine."""
    from .hm2d import HM2D
    out = {}
    for k in sample:
        inst = specs[k].build()
        cfg = inst.config
        if inst.bonds is not None:
            from dataclasses import replace
            cfg = replace(cfg, load_capacity=inst.steps + 8)
        cfg = _fp64(cfg)
        pe0 = _potential(inst.state, cfg.gravity)
        _sync()
        t0 = time.perf_counter()
        e = HM2D(cfg)
        st = inst.state
        e.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
        if inst.bonds is not None:
            e.set_bonds(inst.bonds, inst.strength)
        e.step(inst.steps)
        led = e.ledger()
        peak = None
        if inst.bonds is not None:
            load = e.load_curve()
            peak = float(np.hypot(load[:, 0], load[:, 1]).max()) if len(load) else 0.0
        _sync()
        out[k] = {"seconds": time.perf_counter() - t0, "ledger": led, "peak_load": peak, "n": inst.n,
                  "kind": inst.kind, "potential0": pe0}
        del e
    return out


def _fp64(cfg):
    from dataclasses import replace
    return replace(cfg, precision=64, max_neighbors=12)


def _potential(state, gravity) -> float:
    """Gravitational potential energy of the free discs (the ledger's convention)."""
    m = np.asarray(state["mass"], dtype=np.float64)
    free = np.isfinite(m)
    x = np.asarray(state["pos"], dtype=np.float64)[free]
    return float(-np.sum(m[free] * (x @ np.asarray(gravity, dtype=np.float64))))


def compare(batched: dict, seq: dict) -> dict:
    """FP32 batched vs FP64 one-by-one on the sampled instances.

    The ledger residual (energies + dissipated + fracture - tool work; the
    engines' `total`) of the FP32 run minus the FP64 run's, relative to the
    energy put in: the indenter's work for an indentation, the potential
    energy released so far for a collapse under gravity."""
    peak_err, resid = [], {"ice": [], "column": []}
    for k, s in seq.items():
        g = batched[k]["ledger"]
        led = s["ledger"]
        if s["peak_load"]:
            peak_err.append(abs(g["peak_load"] - s["peak_load"]) / s["peak_load"])
        if s["kind"] == "ice":
            scale = abs(led["tool_work"])
        else:
            scale = s["potential0"] - led["potential"]
        scale = max(scale, abs(led["kinetic"]) + abs(led["dissipated"]), 1e-300)
        resid.setdefault(s["kind"], []).append(abs(g["total"] - led["total"]) / scale)
    every = [r for v in resid.values() for r in v]
    return {"peak_load_rel_err_max": max(peak_err) if peak_err else None,
            "peak_load_rel_err_median": float(np.median(peak_err)) if peak_err else None,
            "ledger_total_rel_diff_max": max(every) if every else None,
            "ledger_total_rel_diff_median": float(np.median(every)) if every else None,
            "ledger_rel_diff_max_by_kind": {k: (max(v) if v else None) for k, v in resid.items()},
            "ledger_normalisation": "tool work (indentations); potential energy released (collapses)"}


def main(args) -> dict:
    specs = ensemble_case(args.instances, seed=args.seed, n_min=args.n_min, n_max=args.n_max, steps=args.steps)
    if args.kind != "all":
        specs = [s for s in specs if s.kind == args.kind]
    rng = np.random.default_rng(args.seed + 1)
    sample = sorted(rng.choice(len(specs), size=min(args.baseline_sample, len(specs)), replace=False).tolist())
    rep, ledgers = run_batched(specs, precision=args.precision, autotune_steps=args.autotune_steps,
                               variant=args.variant, rebuild_every=args.rebuild_every)
    out = {"metric": "ensemble solves/s", "batched": rep}
    if args.baseline_sample > 0:
        seq = run_sequential_fp64(specs, sample)
        mean_s = float(np.mean([s["seconds"] for s in seq.values()]))
        total = mean_s * len(specs)
        out["sequential_fp64"] = {
            "sample": len(sample), "mean_solve_s": mean_s, "extrapolated_total_s": total,
            "solves_per_s": len(specs) / total,
            "sample_particle_steps_per_s": sum(s["n"] for s in seq.values()) * args.steps
            / sum(s["seconds"] for s in seq.values()),
        }
        out["speedup_solves_per_s"] = rep["solves_per_s"] / out["sequential_fp64"]["solves_per_s"]
        out["fp32_batched_vs_fp64"] = compare(ledgers, seq)
    print(json.dumps(out))
    return out
