"""Command line: ``python -m tensordem_gb300 <command>``.

* ``dem-2d`` - the reference's 2-D ice-breaking demo
  (src/tensordem/cli.py:42-110, 254-285), same flags and the same outputs
  (history.csv, trajectory.pt, accounting.json), stepped by the FP64 CUDA
  reference-mode kernel.
* ``dem-3d`` - the reference's 3-D bonded-sphere indentation
  (src/tensordem/dem3d_cli.py:12-150), same flags and outputs (history.csv,
  checkpoint_3d.pt, trajectory_3d.pt, restart from a checkpoint), stepped by
  the FP64 CUDA 3-D reference-mode kernel.
* ``bench-3d`` - step rate of the 3-D reference mode on indentation specimens.
* ``hm2d`` - the Hertz-Mindlin disc settling case on the GB300 engine: run,
  time and report (used for profiling runs as well).
* ``ensemble`` - a seeded mixed ensemble of independent runs in the batched
  engine, against the same runs one-by-one through the FP64 engine.
* ``serve`` - a Poisson trace of such runs served by continuous batching
  under an HBM budget (time-to-completion percentiles, throughput).
"""

from __future__ import annotations

import argparse
import csv
import json
import math
import sys
import time
from dataclasses import asdict
from pathlib import Path

import numpy as np
import torch


def read_hull_profile(path: Path) -> torch.Tensor:
    """Hull vertices from a CSV file in metres: a header row with columns named
    x and y, then one vertex per row (the file the reference's dem-2d command
    reads, src/tensordem/cli.py:15-39). Raises ValueError on an unreadable
    file, missing headers, a bad or non-finite number, fewer than two
    vertices or a zero-length segment."""
    try:
        text = path.read_text(encoding="utf-8-sig")
    except OSError as exc:
        raise ValueError(f"cannot read hull profile CSV: {exc}") from exc
    table = [(number, row) for number, row in enumerate(csv.reader(text.splitlines()), start=1) if row]
    if not table or not {"x", "y"} <= set(table[0][1]):
        raise ValueError("hull profile CSV must contain x,y column headers")
    ix, iy = table[0][1].index("x"), table[0][1].index("y")
    vertices = []
    for number, row in table[1:]:
        try:
            vertices.append((float(row[ix]), float(row[iy])))
        except (IndexError, ValueError) as exc:
            raise ValueError(f"invalid x,y value in hull profile CSV line {number}") from exc
    if len(vertices) < 2:
        raise ValueError("hull profile CSV must contain at least two vertices")
    v = np.asarray(vertices, dtype=np.float64)
    if not np.isfinite(v).all():
        raise ValueError("hull profile coordinates must be finite")
    if (np.hypot(*np.diff(v, axis=0).T) <= 1e-12).any():
        raise ValueError("hull profile must not contain zero-length segments")
    return torch.from_numpy(v)


# history.csv columns (the diagnostics record) and where each comes from in a
# device-side sample row: the clock, the tool, the reactions, the broken-bond
# count, the kinetic energy, then ledger slots (impulses x/y, energies).
_HISTORY = ("time", "tool_x", "tool_y", "reaction_x", "reaction_y", "boundary_reaction_x", "boundary_reaction_y",
            "broken_bonds", "kinetic_energy", "tool_impulse_on_ice_x_Ns", "tool_impulse_on_ice_y_Ns",
            "support_impulse_x_Ns", "support_impulse_y_Ns", "drag_impulse_x_Ns", "drag_impulse_y_Ns",
            "external_impulse_x_Ns", "external_impulse_y_Ns", "fracture_release_J", "pair_contact_acquired_J",
            "tool_work_J", "damping_dissipation_J", "external_work_J")
_LEDGER_COLUMNS = (11, 12, 7, 8, 9, 10, 5, 6, 1, 2, 3, 4, 0)  # ledger slots of the last 13 columns


class _Samples:
    """The samples of a dem-2d run recorded on the device: one history row
    (forces evaluated on the device, ledger copied device to device), the
    positions, velocities, intact-bond flags and tool position. Nothing is
    copied to the host until the run ends."""

    def __init__(self, sim, count: int):
        dev, n = sim.device, len(sim.positions)
        self.sim = sim
        self.rows = torch.zeros((count, len(_HISTORY)), dtype=torch.float64, device=dev)
        self.positions = torch.empty((count, n, 2), dtype=torch.float64, device=dev)
        self.velocities = torch.empty_like(self.positions)
        self.bonds = torch.empty((count, int(sim.bonded.sum())), dtype=torch.bool, device=dev)
        self.tool = torch.empty((count, 2), dtype=torch.float64, device=dev)
        self.ledger = torch.empty(32, dtype=torch.float64, device=dev)
        self.columns = torch.tensor(_LEDGER_COLUMNS, dtype=torch.int64, device=dev)
        self.times: list[float] = []

    def take(self) -> None:
        from . import _lib
        sim, k = self.sim, len(self.times)
        force, reaction = sim.forces()
        row = self.rows[k]
        tool = sim.tool_position
        row[0] = sim.time
        row[1:3] = tool
        row[3:5] = reaction
        row[5:7] = -force[sim.fixed].sum(dim=0)
        row[7] = (sim.bonded & ~sim.alive).sum()
        row[8] = 0.5 * sim.config.mass * sim.velocities.square().sum()
        stream = torch.cuda.current_stream(sim.device).cuda_stream
        rc = _lib.lib().tdem_icedem_ledger_to_device(sim._handle.ptr, self.ledger.data_ptr(), stream)
        _lib.check(rc, sim._handle.ptr, "tdem_icedem_ledger_to_device")
        row[9:] = self.ledger[self.columns]
        self.positions[k] = sim.positions
        self.velocities[k] = sim.velocities
        self.bonds[k] = sim.alive[sim.bonded]
        self.tool[k] = tool
        self.times.append(sim.time)

    def write_history(self, path: Path) -> None:
        count = len(self.times)
        with path.open("w", newline="", encoding="utf-8") as stream:
            writer = csv.writer(stream)
            writer.writerow(_HISTORY)
            for values in self.rows[:count].cpu().tolist():
                values[7] = int(values[7])
                writer.writerow(values)


def _cmd_dem_2d(args: argparse.Namespace) -> None:
    from .dem import DEMConfig, IceDEM

    if args.steps < 1 or args.save_every < 1:
        sys.exit("--steps and --save-every must be positive")
    try:
        hull = read_hull_profile(args.hull_profile) if args.hull_profile else None
        # the time-step bound must cover the faster of the tool and the hull
        speed = max(args.speed, math.hypot(args.hull_velocity_x, args.hull_velocity_y), 1e-12)
        config = DEMConfig(nx=args.nx, ny=args.ny, dt=args.dt, tool_speed=speed,
                           breaking_strain=args.breaking_strain, shear_breaking_strain=args.shear_breaking_strain,
                           device=args.device)
        placement = {} if hull is None else dict(hull_profile=hull, hull_start=(args.hull_start_x, args.hull_start_y),
                                                 hull_velocity=(args.hull_velocity_x, args.hull_velocity_y))
        sim = IceDEM(config, **placement)
    except (ValueError, RuntimeError, TypeError) as exc:
        sys.exit(str(exc))
    # sample at every multiple of save_every and at the last step; the steps in
    # between run as one kernel launch each
    stops = sorted(set(range(0, args.steps + 1, args.save_every)) | {args.steps})
    samples = _Samples(sim, len(stops))
    done = 0
    for stop in stops:
        if stop > done:
            sim.run(stop - done)
            done = stop
        samples.take()
    args.output.mkdir(parents=True, exist_ok=True)
    samples.write_history(args.output / "history.csv")
    torch.save({"config": asdict(sim.config), "dt": sim.dt,
                "times": torch.tensor(samples.times, dtype=torch.float64),
                "positions": samples.positions.cpu(), "velocities": samples.velocities.cpu(),
                "bond_pairs": sim.pairs[sim.bonded].cpu(), "bond_alive": samples.bonds.cpu(),
                "fixed": sim.fixed.cpu(), "tool_positions": samples.tool.cpu(),
                "hull_profile": None if sim.hull_profile is None else sim.hull_profile.cpu(),
                "hull_velocity": sim.hull_velocity.cpu()}, args.output / "trajectory.pt")
    total = int(sim.bonded.sum())
    record = dict(sim.accounting, total_bonds=total, broken_bonds=sim.broken_bonds,
                  failure_energy_sum_J=float(sim.failure_energy_J.sum()),
                  total_mass_kg=float(sim.config.mass * len(sim.positions)), dt=sim.dt, steps=sim.step_count)
    (args.output / "accounting.json").write_text(json.dumps(record, indent=2, sort_keys=True, allow_nan=False),
                                                 encoding="utf-8")
    print(f"done: t={sim.time:.6f} s, dt={sim.dt:.6g} s, broken bonds={sim.broken_bonds}/{total}; "
          f"output: {args.output}")


def _cmd_hm2d(args: argparse.Namespace) -> None:
    from .hm2d import HM2D, granular_gas_case, ice_sheet_case

    bonds = None
    if args.case == "ice":
        nx = args.n_side * 2
        cfg, st, bonds, strength = ice_sheet_case(nx, max(2, args.n_side // 2), precision=args.precision,
                                                  seed=args.seed, steps=max(args.steps, 1))
    else:
        cfg, st = granular_gas_case(args.n_side, seed=args.seed, precision=args.precision,
                                    max_neighbors=args.max_neighbors)
    eng = HM2D(cfg)
    if args.no_graph:
        eng.use_graph(False)
    eng.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
    if bonds is not None:
        eng.set_bonds(bonds, strength)
    if args.variant is not None:
        eng.variant = args.variant
    elif args.autotune:
        eng.autotune(steps=10)
    eng.step(0)  # builds the step graph outside the timing
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.step(args.steps)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    led = eng.ledger()
    print(json.dumps({"discs": cfg.n, "steps": args.steps, "seconds": dt,
                      "particle_steps_per_s": cfg.n * args.steps / dt, "ledger": led}))


def _cmd_scale(args: argparse.Namespace) -> None:
    """Step-kernel time against disc count: plain launches between CUDA events
    on the engine's stream, L2 flushed before each (one buffer larger than L2
    written, another read), list rebuilds outside the brackets."""
    from .hm2d import HM2D, granular_gas_case

    dev = torch.device("cuda", 0)
    flush_w = torch.empty(64 << 20, dtype=torch.float32, device=dev)
    flush_r = torch.ones(64 << 20, dtype=torch.float32, device=dev)
    rows = []
    for side in args.sides:
        cfg, st = granular_gas_case(side, seed=args.seed)
        eng = HM2D(cfg, device=dev)
        eng.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
        for v in args.variants:
            eng.variant = v
            eng.step(5)
            times = []
            stream = torch.cuda.current_stream(dev)
            for _ in range(args.repeats):
                flush_w.fill_(1.0)
                flush_r.sum()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                eng.step_kernel()
                e1.record(stream)
                if eng.rebuild_pending():
                    eng.rebuild()
                torch.cuda.synchronize(dev)
                times.append(e0.elapsed_time(e1) * 1e3)
            times.sort()
            med = times[len(times) // 2]
            rows.append({"discs": cfg.n, "variant": v, "us_median": med, "us_mean": sum(times) / len(times),
                         "us_min": times[0], "alg_GBs": cfg.n * 80 / (med * 1e-6) / 1e9})
            print(json.dumps(rows[-1]), flush=True)
        del eng


def _cmd_ensemble(args: argparse.Namespace) -> None:
    import os

    from . import ensemble

    if args.no_graph:
        os.environ["TDEM_GRAPH"] = "0"
    out = ensemble.main(args)
    if args.output:
        Path(args.output).write_text(json.dumps(out, indent=1))


def _cmd_serve(args: argparse.Namespace) -> None:
    from . import serve

    out = serve.main(args)
    if args.output:
        Path(args.output).write_text(json.dumps(out, indent=1))


def _cmd_dem_3d(args: argparse.Namespace) -> None:
    from .dem3d import DEM3DConfig, IceDEM3D

    if args.steps < 1 or args.save_every < 1:
        sys.exit("--steps and --save-every must be positive")
    if args.stability_report:
        sys.exit("--stability-report (src/tensordem/stability.py) is not built in tensordem_gb300")
    try:
        if args.restart is not None:
            if not args.restart.is_file():
                sys.exit(f"restart checkpoint not found: {args.restart}")
            checkpoint = torch.load(args.restart, map_location="cpu", weights_only=False)
            if not isinstance(checkpoint, dict) or "state" not in checkpoint:
                sys.exit("restart file must be a TensorDEM 3-D checkpoint with a 'state' entry")
            saved = checkpoint["state"].get("config")
            if not isinstance(saved, dict):
                sys.exit("restart checkpoint has no valid saved configuration")
            saved = {k: tuple(v) if isinstance(v, list) else v for k, v in saved.items()}
            sim = IceDEM3D(DEM3DConfig(**{**saved, "device": args.device}))
            sim.load_state_dict(checkpoint["state"])
        else:
            sim = IceDEM3D(DEM3DConfig(
                nx=args.nx, ny=args.ny, nz=args.nz, dt=args.dt, tool_speed=args.speed, radius=args.radius,
                tool_radius=args.tool_radius, breaking_strain=args.breaking_strain,
                shear_breaking_strain=args.shear_breaking_strain, device=args.device, geometry=args.geometry,
                fix_bottom=args.fix_bottom, top_platen_enabled=args.top_platen,
                bottom_platen_enabled=args.bottom_platen, platen_stiffness=args.platen_stiffness,
                platen_damping=args.platen_damping, top_platen_gap=args.top_platen_gap,
                bottom_platen_gap=args.bottom_platen_gap, top_platen_velocity=args.top_platen_velocity,
                bottom_platen_velocity=args.bottom_platen_velocity))
    except (ValueError, RuntimeError, TypeError, OSError, KeyError, NotImplementedError) as exc:
        sys.exit(str(exc))
    args.output.mkdir(parents=True, exist_ok=True)
    frames, velocities, alive_frames, times, tool_positions = [], [], [], [], []
    history = args.output / "history.csv"
    append = args.restart is not None and history.exists()
    with history.open("a" if append else "w", newline="", encoding="utf-8") as stream:
        writer = None
        step = 0
        while step <= args.steps:
            if (step % args.save_every == 0 or step == args.steps) and not (append and step == 0):
                row = sim.diagnostics()
                row.setdefault("time_s", row["time"])
                if writer is None:
                    writer = csv.DictWriter(stream, fieldnames=list(row))
                    if not append:
                        writer.writeheader()
                writer.writerow(row)
                frames.append(sim.positions.cpu().clone())
                velocities.append(sim.velocities.cpu().clone())
                alive_frames.append(sim.alive[sim.bonded].cpu().clone())
                times.append(sim.time)
                tool_positions.append(sim.tool_position.cpu().clone())
                torch.save({"format": "tensordem-dem3d-checkpoint-v1",
                            "state": {k: (v.cpu() if isinstance(v, torch.Tensor) else v)
                                      for k, v in sim.state_dict().items()}},
                           args.output / "checkpoint_3d.pt")
            if step == args.steps:
                break
            nxt = min(args.steps, (step // args.save_every + 1) * args.save_every)
            sim.run(nxt - step)  # one kernel launch to the next sample point
            step = nxt
    torch.save({
        "dimension": 3, "config": asdict(sim.config), "dt": sim.dt,
        "times": torch.tensor(times, dtype=torch.float64),
        "positions": torch.stack(frames), "velocities": torch.stack(velocities),
        "bond_pairs": sim.pairs[sim.bonded].cpu(), "bond_alive": torch.stack(alive_frames),
        "fixed": sim.fixed.cpu(), "tool_positions": torch.stack(tool_positions),
        "failure_mode": sim.failure_mode.cpu(), "failure_time_s": sim.failure_time_s.cpu(),
        "failure_extension_m": sim.failure_extension_m.cpu(), "failure_energy_J": sim.failure_energy_J.cpu(),
    }, args.output / "trajectory_3d.pt")
    print(f"3-D done: t={sim.time:.6g} s, dt={sim.dt:.4g} s, particles={len(sim.positions)}, "
          f"broken={sim.broken_bonds}, output={args.output}")


def _cmd_bench_3d(args: argparse.Namespace) -> None:
    """Steps per second of the 3-D reference mode on indentation specimens."""
    from .dem3d import DEM3DConfig, IceDEM3D

    rows = []
    for size in args.sizes:
        nx, ny, nz = (int(v) for v in size.split("x"))
        sim = IceDEM3D(DEM3DConfig(nx=nx, ny=ny, nz=nz, breaking_strain=0.004, shear_breaking_strain=0.008,
                                   friction_coefficient=args.friction, restitution_coefficient=0.7))
        sim.run(args.warmup)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.run(args.steps)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        n = len(sim.positions)
        rows.append({"specimen": size, "particles": n, "bonds": len(sim.pairs), "steps": args.steps,
                     "us_per_step": 1e6 * dt / args.steps, "particle_steps_per_s": n * args.steps / dt,
                     "broken": sim.broken_bonds,
                     "contacts": int(sim.read_ledger()[12])})
        print(json.dumps(rows[-1]), flush=True)


def main(argv: list[str] | None = None) -> None:
    parser = argparse.ArgumentParser(description="tensordem_gb300: GB300 2-D DEM step")
    sub = parser.add_subparsers(dest="command")
    d = sub.add_parser("dem-2d", help="2-D ice-breaking DEM simulation (reference mode, FP64)")
    d.add_argument("--nx", type=int, default=21)
    d.add_argument("--ny", type=int, default=5)
    d.add_argument("--steps", type=int, default=2000)
    d.add_argument("--dt", type=float, default=None)
    d.add_argument("--speed", type=float, default=1.0)
    d.add_argument("--hull-profile", type=Path, default=None)
    d.add_argument("--hull-start-x", type=float, default=0.0)
    d.add_argument("--hull-start-y", type=float, default=0.0)
    d.add_argument("--hull-velocity-x", type=float, default=0.0)
    d.add_argument("--hull-velocity-y", type=float, default=0.0)
    d.add_argument("--breaking-strain", type=float, default=0.015)
    d.add_argument("--shear-breaking-strain", type=float, default=0.03)
    d.add_argument("--device", default="cuda")
    d.add_argument("--output", type=Path, default=Path("results"))
    d.add_argument("--save-every", type=int, default=20)
    d.set_defaults(func=_cmd_dem_2d)
    d3 = sub.add_parser("dem-3d", help="3-D bonded-sphere indentation (reference mode, FP64)")
    d3.add_argument("--nx", type=int, default=9)
    d3.add_argument("--ny", type=int, default=5)
    d3.add_argument("--nz", type=int, default=3)
    d3.add_argument("--steps", type=int, default=1000)
    d3.add_argument("--dt", type=float, default=None)
    d3.add_argument("--speed", type=float, default=0.5)
    d3.add_argument("--radius", type=float, default=0.025)
    d3.add_argument("--tool-radius", type=float, default=0.1)
    d3.add_argument("--breaking-strain", type=float, default=0.015)
    d3.add_argument("--shear-breaking-strain", type=float, default=0.03)
    d3.add_argument("--device", default="cuda")
    d3.add_argument("--geometry", choices=("box", "cylinder_xz"), default="box")
    d3.add_argument("--save-every", type=int, default=20)
    d3.add_argument("--output", type=Path, default=Path("results-3d"))
    d3.add_argument("--restart", type=Path, default=None)
    d3.add_argument("--fix-bottom", action="store_true")
    d3.add_argument("--top-platen", action="store_true")
    d3.add_argument("--bottom-platen", action="store_true")
    d3.add_argument("--platen-stiffness", type=float, default=5000.0)
    d3.add_argument("--platen-damping", type=float, default=0.0)
    d3.add_argument("--top-platen-gap", type=float, default=0.0)
    d3.add_argument("--bottom-platen-gap", type=float, default=0.0)
    d3.add_argument("--top-platen-velocity", type=float, default=0.0)
    d3.add_argument("--bottom-platen-velocity", type=float, default=0.0)
    d3.add_argument("--stability-report", action="store_true")
    d3.set_defaults(func=_cmd_dem_3d)
    b3 = sub.add_parser("bench-3d", help="3-D reference-mode step rate on indentation specimens")
    b3.add_argument("--sizes", nargs="+", default=["9x5x3", "20x10x6", "40x20x10", "60x30x15"])
    b3.add_argument("--steps", type=int, default=2000)
    b3.add_argument("--warmup", type=int, default=200)
    b3.add_argument("--friction", type=float, default=0.3)
    b3.set_defaults(func=_cmd_bench_3d)
    h = sub.add_parser("hm2d", help="Hertz-Mindlin disc settling case on the GPU engine")
    h.add_argument("--case", choices=("gas", "ice"), default="gas",
                   help="gas: n-side^2 disc settling case; ice: (2 n-side) x (n-side / 2) bonded hex sheet")
    h.add_argument("--n-side", type=int, default=1024)
    h.add_argument("--steps", type=int, default=100)
    h.add_argument("--seed", type=int, default=0)
    h.add_argument("--precision", type=int, choices=(32, 64), default=32)
    h.add_argument("--max-neighbors", type=int, default=16)
    h.add_argument("--variant", type=int, default=None)
    h.add_argument("--autotune", action="store_true")
    h.add_argument("--no-graph", action="store_true", help="plain launches (visible to profilers)")
    h.set_defaults(func=_cmd_hm2d)
    sc = sub.add_parser("scale", help="step-kernel time against disc count (L2 flushed per launch)")
    sc.add_argument("--sides", type=int, nargs="+", default=[362, 512, 724, 1024, 1448, 2048])
    sc.add_argument("--variants", type=int, nargs="+", default=[1])
    sc.add_argument("--repeats", type=int, default=100)
    sc.add_argument("--seed", type=int, default=0)
    sc.set_defaults(func=_cmd_scale)
    en = sub.add_parser("ensemble", help="mixed ensemble of 2-D runs: batched engine vs one-by-one FP64")
    en.add_argument("--instances", type=int, default=4096)
    en.add_argument("--steps", type=int, default=5000)
    en.add_argument("--seed", type=int, default=0)
    en.add_argument("--n-min", type=int, default=100)
    en.add_argument("--n-max", type=int, default=20000)
    en.add_argument("--precision", type=int, choices=(32, 64), default=32)
    en.add_argument("--baseline-sample", type=int, default=64)
    en.add_argument("--autotune-steps", type=int, default=2)
    en.add_argument("--variant", type=int, default=None)
    en.add_argument("--rebuild-every", type=int, default=0)
    en.add_argument("--kind", choices=("all", "ice", "column"), default="all")
    en.add_argument("--no-graph", action="store_true", help="plain launches (visible to profilers)")
    en.add_argument("--output", type=Path, default=None)
    en.set_defaults(func=_cmd_ensemble)
    sv = sub.add_parser("serve", help="Poisson request trace served by continuous batching")
    sv.add_argument("--duration", type=float, default=600.0, help="arrival window (s)")
    sv.add_argument("--load", type=float, default=0.8, help="fraction of the capacity offered")
    sv.add_argument("--capacity", type=float, default=None,
                    help="engine capacity in particle-steps/s (default: measured by a saturated calibration run)")
    sv.add_argument("--calibrate-seconds", type=float, default=20.0)
    sv.add_argument("--budget-gb", type=float, default=150.0)
    sv.add_argument("--block", type=int, default=100, help="steps per step block")
    sv.add_argument("--rebuild-every", type=int, default=0)
    sv.add_argument("--seed", type=int, default=0)
    sv.add_argument("--n-min", type=int, default=500)
    sv.add_argument("--n-max", type=int, default=200_000)
    sv.add_argument("--s-min", type=int, default=1000)
    sv.add_argument("--s-max", type=int, default=50_000)
    sv.add_argument("--output", type=Path, default=None)
    sv.set_defaults(func=_cmd_serve)
    args = parser.parse_args(argv)
    if not hasattr(args, "func"):
        parser.print_help()
        sys.exit(1)
    args.func(args)


if __name__ == "__main__":
    main()
