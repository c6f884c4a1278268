"""The 2-D Hertz-Mindlin step against the reference's own FP64 engine.

tests/golden/floebed_planar.npz holds a trajectory of the reference's FloeBed
(src/tensordem/scale_ceiling/kernel.py:155-455), made by
tests/golden/make_floebed.py: 96 polydisperse spheres with centres in one
plane, in-plane velocities, gravity, floor and side walls, restitution 0.6,
no friction. Without friction there is no tangential force and no rotation,
so the 2-D step (Hertz normal force, Tsuji dashpot on the half-step velocity,
walls, gravity, velocity-Verlet) must give the same trajectory to rounding.
"""

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle.hm2d import HM2DOracle, HMParams

GOLDEN = Path(__file__).resolve().parent / "golden" / "floebed_planar.npz"
# FP64 bounds per checkpoint (positions, velocities), relative to the largest entry
BOUNDS = {1: (1e-14, 1e-13), 10: (1e-14, 1e-13), 50: (1e-13, 1e-12), 200: (1e-12, 1e-11)}


def _golden():
    return np.load(GOLDEN)


def _oracle(g):
    n = len(g["init_radius"])
    p = HMParams(young=float(g["young"]), poisson=float(g["poisson"]), restitution=float(g["restitution"]),
                 mu=0.0, mu_wall=0.0, dt=float(g["dt"]), gravity=(0.0, -float(g["gravity"])),
                 box=tuple(g["box"]), walls=(True, True, True, False), skin=float(g["skin"]))
    r, m = g["init_radius"], g["init_mass"]
    return HM2DOracle(g["init_pos"], g["init_vel"], np.zeros(n), r, m, 0.4 * m * r * r, p)


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_oracle_reproduces_the_reference_engine():
    g = _golden()
    o = _oracle(g)
    done = 0
    for c in g["checkpoints"]:
        o.step(int(c) - done)
        done = int(c)
        bp, bv = BOUNDS[int(c)]
        assert _rel(o.pos, g[f"pos_{c}"]) <= bp, c
        assert _rel(o.vel, g[f"vel_{c}"]) <= bv, c
    # the run is not trivial: collisions dissipated over half of the energy
    led = o.energies()
    assert led["dissipated"] > 0.5 * led["total"]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_gpu_step_reproduces_the_reference_engine(precision):
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300.hm2d import WALL_BOTTOM, WALL_LEFT, WALL_RIGHT, HM2D, HM2DConfig
    g = _golden()
    n = len(g["init_radius"])
    r, m = g["init_radius"], g["init_mass"]
    lx = float(g["box"][0])
    skin = float(g["skin"])
    ncx = int(lx // (2 * r.max() + skin))
    cell = lx / ncx
    cfg = HM2DConfig(n=n, ncx=ncx, ncy=int(2 * float(g["box"][1]) / cell) + 2, cell=cell, skin=skin,
                     dt=float(g["dt"]), young=float(g["young"]), poisson=float(g["poisson"]),
                     restitution=float(g["restitution"]), mu=0.0, mu_wall=0.0, gravity=(0.0, -float(g["gravity"])),
                     walls=WALL_LEFT | WALL_RIGHT | WALL_BOTTOM, precision=precision, max_neighbors=12,
                     inertia_factor=0.4)
    e = HM2D(cfg)
    e.set_state(g["init_pos"], g["init_vel"], np.zeros(n), r, m, 0.4 * m * r * r)
    done = 0
    for c in g["checkpoints"]:
        e.step(int(c) - done)
        done = int(c)
        s = e.state()
        pos, vel = s["pos"].cpu().numpy(), s["vel"].cpu().numpy()
        ep, ev = _rel(pos, g[f"pos_{c}"]), _rel(vel, g[f"vel_{c}"])
        print(f"fp{precision} vs FloeBed after {c} steps: pos {ep:.2e} vel {ev:.2e}")
        if precision == 64:
            bp, bv = BOUNDS[int(c)]
            assert ep <= 10 * bp and ev <= 10 * bv, c
        else:
            # FP32 contacts: a stiff Hertz contact resolves the overlap to ~1e-7 relative
            assert ep <= 1e-5 and ev <= 5e-2, c
    assert e.ledger()["status"] == 0
