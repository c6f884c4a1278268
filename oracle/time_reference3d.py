"""Time the reference's own 3-D step on this host's CPU (the CPU baseline of
the 3-D reference mode; the reference tree must be importable)::

    PYTHONPATH=<reference>/src python oracle/time_reference3d.py

It builds the reference's ``tensordem.dem3d.IceDEM3D`` on the indentation
specimens of ``python -m tensordem_gb300 bench-3d`` (breaking strains
0.004 / 0.008, friction 0.3, restitution 0.7), with one torch thread as the
reference's CLI sets (src/tensordem/dem3d_cli.py:101-102), and times its first
steps, before contacts form, so the figures are lower bounds on its cost.
Measurement only: nothing in the package or the tests runs this file.
"""

import time

import torch

from tensordem.dem3d import DEM3DConfig, IceDEM3D  # reference package


def main() -> None:
    torch.set_num_threads(1)
    for size, steps in (("9x5x3", 200), ("20x10x6", 50), ("40x20x10", 10)):
        nx, ny, nz = map(int, size.split("x"))
        sim = IceDEM3D(DEM3DConfig(nx=nx, ny=ny, nz=nz, breaking_strain=0.004, shear_breaking_strain=0.008,
                                   friction_coefficient=0.3, restitution_coefficient=0.7))
        sim.step()
        t0 = time.perf_counter()
        for _ in range(steps):
            sim.step()
        dt = (time.perf_counter() - t0) / steps
        print(f"{size}: {len(sim.positions)} particles, {dt * 1e3:.2f} ms/step, "
              f"{len(sim.positions) / dt:.3e} particle-steps/s", flush=True)


if __name__ == "__main__":
    main()
