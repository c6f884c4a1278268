"""Time the reference's own 2-D disc engine on this host's CPU (a CPU data
point beside the 1M-disc settling case; the reference tree must be importable)::

    PYTHONPATH=<reference>/src python oracle/time_reference2d.py [--discs-side 1024] [--steps 20]

The reference has no 2-D Hertz-Mindlin engine; its closest 2-D cell-list
engine is ``tensordem.granular2d.DiskSystem`` (linear spring-dashpot,
Coulomb friction with history, rolling resistance; src/tensordem/granular2d/engine.py:144-630).
It is built on the same 1024 x 1024 polydisperse disc set as the settling case
(positions and radii of ``tensordem_gb300.hm2d.granular_gas_case``, seed 0),
inside four walls with gravity, at its own stable step, and timed over a few
steps after one warm-up step. Measurement only: nothing in the package or the
tests runs this file.
"""

import argparse
import time

import numpy as np

from tensordem.granular2d.engine import DiskConfig, DiskSystem, box_walls  # reference package


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--discs-side", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=20)
    a = ap.parse_args()
    from tensordem_gb300.hm2d import granular_gas_case
    cfg, st = granular_gas_case(a.discs_side, seed=0)
    pos = np.asarray(st["pos"], dtype=np.float64)
    rad = np.asarray(st["radius"], dtype=np.float64)
    box = cfg.box
    sim = DiskSystem(pos, rad, DiskConfig(gravity=(0.0, -9.81), density=2500.0, thickness=2e-3),
                     walls=box_walls(box[0], box[1]))
    sim.vel[:] = np.asarray(st["vel"], dtype=np.float64)
    sim.step(1)
    t0 = time.perf_counter()
    sim.step(a.steps)
    dt = (time.perf_counter() - t0) / a.steps
    n = len(rad)
    print(f"DiskSystem, {n} discs: {dt * 1e3:.1f} ms/step, {n / dt:.3e} particle-steps/s "
          f"(its dt {sim.dt:.3e} s)", flush=True)


if __name__ == "__main__":
    main()
