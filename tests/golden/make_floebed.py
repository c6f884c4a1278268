"""Golden trajectories of the reference's own FP64 Hertz-Mindlin engine.

Run where the reference source tree is available::

    PYTHONPATH=<reference>/src python tests/golden/make_floebed.py

It imports ``tensordem.scale_ceiling.kernel.FloeBed``
(src/tensordem/scale_ceiling/kernel.py:155-455: Hertz normal force with the
Tsuji dashpot, Cundall-Strack history, planar floor / side walls, gravity,
velocity-Verlet in float64) and runs it on a planar, frictionless bed: every
sphere centre in the plane y = d/2 with in-plane velocities, so the run is a
2-D disc problem (gravity along -z, walls at x = 0, x = Lx and z = 0). With
mu = 0 there is no tangential force, so neither the history conventions nor
rotation enter, and the 2-D Hertz-Mindlin step must reproduce the trajectory.
Output: tests/golden/floebed_planar.npz (initial state, parameters, checkpoints).
"""

from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np
import torch

OUT = Path(__file__).resolve().parent / "floebed_planar.npz"
CHECKPOINTS = (1, 10, 50, 200)


def main() -> None:
    from tensordem.scale_ceiling.kernel import FloeBed, FloeBedConfig

    torch.set_num_threads(1)
    cfg = FloeBedConfig(n=96, diameter=0.02, polydispersity=0.2, density=2500.0, young=1.0e8, poisson=0.25,
                        mu_grain=0.0, mu_wall=0.0, restitution=0.6, skin=0.004, layers_y=1, height_layers=8,
                        gravity=9.81, dt_safety=0.03, seed=4, floor=True, left_wall=True, right_wall=True)
    bed = FloeBed(cfg)
    rng = np.random.default_rng(11)
    with torch.no_grad():
        bed.pos[:, 1] = 0.5 * cfg.diameter
        v = torch.from_numpy(rng.normal(0.0, 0.4, (cfg.n, 2)))
        bed.vel[:, 0] = v[:, 0]
        bed.vel[:, 2] = v[:, 1]
    bed._force = None
    bed.build_neighbours(keep_state=False)
    init = dict(pos=bed.pos[:, [0, 2]].numpy().copy(), vel=bed.vel[:, [0, 2]].numpy().copy(),
                radius=bed.radii.numpy().copy(), mass=bed.mass.numpy().copy())
    traj = {}
    done = 0
    for stop in CHECKPOINTS:
        bed.step(stop - done)
        done = stop
        assert float(bed.pos[:, 1].sub(0.5 * cfg.diameter).abs().max()) == 0.0
        traj[f"pos_{stop}"] = bed.pos[:, [0, 2]].numpy().copy()
        traj[f"vel_{stop}"] = bed.vel[:, [0, 2]].numpy().copy()
    np.savez(OUT, **{f"init_{k}": v for k, v in init.items()}, **traj,
             checkpoints=np.array(CHECKPOINTS), dt=bed.dt, young=cfg.young, poisson=cfg.poisson,
             restitution=cfg.restitution, gravity=cfg.gravity, box=np.array([bed.box[0], bed.box[2]]),
             skin=cfg.skin)
    print(f"wrote {OUT} (n={cfg.n}, dt={bed.dt:.3e}, box={bed.box})")


if __name__ == "__main__":
    sys.exit(main())
