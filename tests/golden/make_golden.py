"""Generate golden vectors for the 2-D bonded-disc step from the reference itself.

Run in a container where the reference source tree is mounted::

    PYTHONPATH=<reference>/src python tests/golden/make_golden.py

It imports the reference ``tensordem.dem.IceDEM`` (``src/tensordem/dem.py``),
runs it on CPU in float64 with one torch thread (as its CLI does,
``src/tensordem/cli.py:65-66``) and writes ``tests/golden/*.npz``. The fixtures
are committed; nothing at test time reads the reference tree.

Cases:
* ``demo_b0.01_s0.02`` and ``demo_b0.015_s0.03``: the 21x5 icebreaking demo
  (``python -m tensordem dem-2d --steps 2000``) at the two strain pairs.
* ``repro_7x3``: the indentation of ``tests/test_reproducibility.py``.
* ``hull_9x3``: a polyline hull ploughing through a 9x3 strip
  (``src/tensordem/hull_contact.py``).
* ``loads_5x3``: seeded external nodal loads, stepped with ``load_time``.
* ``unit_*``: single ``forces()`` evaluations on hand-edited states taken from
  ``tests/test_dem.py`` (shear, tension, compression, coincident discs).
* ``calibrated_21x5``: the demo at 0.01/0.02 with per-bond stiffness
  (``src/tensordem/calibrated_dem.py``), seeded U[0.5, 1] x the config's.
"""

from __future__ import annotations

import hashlib
import json
import math
import sys
from pathlib import Path

import numpy as np
import torch

from tensordem.dem import DEMConfig, IceDEM  # reference package

OUT = Path(__file__).resolve().parent
FRAMES = sorted(set([0, 1, 2, 5, 10, 20, 50] + list(range(200, 2001, 200))))


def _acc_vector(acc: dict) -> np.ndarray:
    keys = ("external_work_J", "fracture_release_J", "pair_contact_acquired_J",
            "tool_work_J", "damping_dissipation_J")
    vec = [acc[k] for k in keys]
    for k in ("external_impulse_Ns", "support_impulse_Ns", "drag_impulse_Ns",
              "tool_impulse_on_ice_Ns"):
        vec.extend(acc[k])
    return np.asarray(vec, dtype=np.float64)


def _record_run(sim: IceDEM, steps: int, frames, loads_fn=None) -> dict:
    rec = {k: [] for k in ("frame_step", "frame_pos", "frame_vel", "frame_alive",
                           "frame_force", "frame_reaction", "frame_acc", "frame_time")}
    bonded = sim.bonded
    for s in range(steps + 1):
        if s in frames:
            # forces() at an unchanged state is idempotent: breaks already
            # committed stay committed and nothing new crosses a threshold.
            loads = None if loads_fn is None else loads_fn(s)
            f, r = sim.forces(loads)
            rec["frame_step"].append(s)
            rec["frame_pos"].append(sim.positions.numpy().copy())
            rec["frame_vel"].append(sim.velocities.numpy().copy())
            rec["frame_alive"].append(sim.alive[bonded].numpy().copy())
            rec["frame_force"].append(f.numpy().copy())
            rec["frame_reaction"].append(r.numpy().copy())
            rec["frame_acc"].append(_acc_vector(sim.accounting))
            rec["frame_time"].append(sim.time)
        if s < steps:
            if loads_fn is None:
                sim.step()
            else:
                sim.step(loads_fn(s), load_time=sim.time)
    out = {k: np.asarray(v) for k, v in rec.items()}
    out["bond_pairs"] = sim.pairs[bonded].numpy()
    out["bond_pair_index"] = torch.nonzero(bonded).flatten().numpy()
    out["failure_mode"] = sim.failure_mode[bonded].numpy()
    out["failure_time_s"] = sim.failure_time_s[bonded].numpy()
    out["failure_extension_m"] = sim.failure_extension_m[bonded].numpy()
    out["failure_energy_J"] = sim.failure_energy_J[bonded].numpy()
    out["final_pos"] = sim.positions.numpy()
    out["final_vel"] = sim.velocities.numpy()
    out["final_acc"] = _acc_vector(sim.accounting)
    out["fixed"] = sim.fixed.numpy()
    out["dt"] = np.float64(sim.dt)
    out["final_time"] = np.float64(sim.time)
    me = sim.mechanical_energy()
    out["final_mech"] = np.asarray([me[k] for k in ("kinetic_J", "bond_J", "pair_contact_J",
                                                    "tool_contact_J", "mechanical_J")])
    last = sim.last_step
    out["last_step"] = np.asarray([last.get("external_work_J", 0.0), *last.get("support_force_N", [0, 0]),
                                   *last.get("tool_reaction_N", [0, 0]), *last.get("external_force_N", [0, 0]),
                                   last.get("external_moment_Nm", 0.0)])
    digest = hashlib.sha256(sim.failure_mode.numpy().tobytes()
                            + sim.failure_time_s.numpy().tobytes()).hexdigest()[:16]
    out["break_digest"] = np.asarray(digest)
    return out


def _config_array(cfg: DEMConfig) -> np.ndarray:
    d = {k: v for k, v in cfg.__dict__.items() if k != "device"}
    return np.asarray(json.dumps(d, sort_keys=True))


def demo(bs: float, ss: float) -> None:
    cfg = DEMConfig(breaking_strain=bs, shear_breaking_strain=ss)
    sim = IceDEM(cfg)
    out = _record_run(sim, 2000, FRAMES)
    out["config"] = _config_array(cfg)
    np.savez_compressed(OUT / f"demo_b{bs}_s{ss}.npz", **out)
    print(f"demo {bs}/{ss}: broken {sim.broken_bonds}/{int(sim.bonded.sum())} digest {out['break_digest']}")


def repro() -> None:
    cfg = DEMConfig(nx=7, ny=3, tool_speed=0.2, breaking_strain=0.008, shear_breaking_strain=0.02)
    sim = IceDEM(cfg)
    out = _record_run(sim, 160, set(range(0, 161, 10)))
    out["config"] = _config_array(cfg)
    np.savez_compressed(OUT / "repro_7x3.npz", **out)
    print("repro broken", sim.broken_bonds)


HULL = [[-0.35, 0.10], [-0.12, -0.02], [0.0, -0.05], [0.12, -0.02], [0.35, 0.10]]


def hull() -> None:
    cfg = DEMConfig(nx=9, ny=3, breaking_strain=0.01, shear_breaking_strain=0.02,
                    tool_speed=0.6)
    sim = IceDEM(cfg, hull_profile=torch.tensor(HULL, dtype=torch.float64),
                 hull_start=(0.0, 0.16), hull_velocity=(0.1, -0.5))
    out = _record_run(sim, 600, set(range(0, 601, 50)))
    out["config"] = _config_array(cfg)
    out["hull_profile"] = np.asarray(HULL)
    out["hull_start"] = np.asarray([0.0, 0.16])
    out["hull_velocity"] = np.asarray([0.1, -0.5])
    np.savez_compressed(OUT / "hull_9x3.npz", **out)
    print("hull broken", sim.broken_bonds)


def loads() -> None:
    cfg = DEMConfig(nx=5, ny=3, drag=0.5)
    sim = IceDEM(cfg)
    rng = np.random.default_rng(7)
    table = rng.normal(0.0, 0.05, size=(121, 15, 2))

    def fn(s):
        return torch.tensor(table[s], dtype=torch.float64)

    out = _record_run(sim, 120, set(range(0, 121, 20)), loads_fn=fn)
    out["config"] = _config_array(cfg)
    out["loads"] = table
    np.savez_compressed(OUT / "loads_5x3.npz", **out)
    print("loads broken", sim.broken_bonds)


def calibrated() -> None:
    """Per-bond stiffness (src/tensordem/calibrated_dem.py): the 21x5 demo at
    0.01/0.02 with seeded bond stiffness U[0.5, 1] x the config's."""
    from tensordem.calibrated_dem import CalibratedIceDEM
    cfg = DEMConfig(breaking_strain=0.01, shear_breaking_strain=0.02)
    probe = IceDEM(cfg)
    rng = np.random.default_rng(21)
    k = cfg.bond_stiffness * rng.uniform(0.5, 1.0, len(probe.bond_indices))
    sim = CalibratedIceDEM(cfg, bond_stiffness=torch.tensor(k))
    out = _record_run(sim, 2000, FRAMES)
    out["config"] = _config_array(cfg)
    out["bond_stiffness"] = k
    np.savez_compressed(OUT / "calibrated_21x5.npz", **out)
    print(f"calibrated: broken {sim.broken_bonds}/{int(sim.bonded.sum())} digest {out['break_digest']}")


def unit_cases() -> None:
    """Single forces() calls on edited states (tests/test_dem.py:21-139)."""
    out = {}

    def model(**kw):
        return IceDEM(DEMConfig(nx=3, ny=2, drag=0, fix_edges=False, **kw))

    def save(name, sim, f, r):
        out[f"{name}_pos"] = sim.positions.numpy().copy()
        out[f"{name}_vel"] = sim.velocities.numpy().copy()
        out[f"{name}_force"] = f.numpy().copy()
        out[f"{name}_reaction"] = r.numpy().copy()
        out[f"{name}_alive"] = sim.alive[sim.bonded].numpy().copy()

    # shear (test_dem.py:57-76)
    sim = model(shear_breaking_strain=0.02, breaking_strain=0.5)
    sim.positions = sim.initial_positions.clone()
    sim.positions[:, 0] += 0.08 * sim.positions[:, 1]
    out["shear_alive_in"] = sim.alive[sim.bonded].numpy().copy()
    f, r = sim.forces()
    save("shear", sim, f, r)
    # rigid rotation (test_dem.py:30-40)
    sim = model()
    a = 0.6
    rot = torch.tensor([[math.cos(a), -math.sin(a)], [math.sin(a), math.cos(a)]], dtype=torch.float64)
    sim.positions = sim.positions @ rot.T + torch.tensor([4.0, -4.0], dtype=torch.float64)
    out["rotation_alive_in"] = sim.alive[sim.bonded].numpy().copy()
    f, r = sim.forces()
    save("rotation", sim, f, r)
    # tension then compression (test_dem.py:42-55)
    sim = model()
    sim.positions = sim.initial_positions * 1.02
    out["tension_alive_in"] = sim.alive[sim.bonded].numpy().copy()
    f, r = sim.forces()
    save("tension", sim, f, r)
    sim.positions = sim.initial_positions * 0.9
    out["compress_alive_in"] = sim.alive[sim.bonded].numpy().copy()
    f, r = sim.forces()
    save("compress", sim, f, r)
    # contact with moving discs (test_dem.py:78-87)
    sim = model()
    sim.alive[:] = False
    sim.positions[1, 0] -= 0.005
    sim.velocities[:, 1] = torch.linspace(-0.3, 0.3, 6, dtype=torch.float64)
    out["contact_alive_in"] = sim.alive[sim.bonded].numpy().copy()
    f, r = sim.forces()
    save("contact", sim, f, r)
    # coincident particles (test_dem.py:133-139)
    sim = model()
    sim.alive[:] = False
    sim.positions[1] = sim.positions[0]
    out["coincident_alive_in"] = sim.alive[sim.bonded].numpy().copy()
    f, r = sim.forces()
    save("coincident", sim, f, r)
    # tool in contact, with drag (test_dem.py:89-100)
    sim = IceDEM(DEMConfig(nx=5, ny=3))
    sim.time = 0.02
    sim.velocities[:, 0] = 0.01
    out["tool_alive_in"] = sim.alive[sim.bonded].numpy().copy()
    f, r = sim.forces()
    save("tool", sim, f, r)
    np.savez_compressed(OUT / "unit_cases.npz", **out)
    print("unit cases", len(out))


if __name__ == "__main__":
    torch.set_num_threads(1)
    which = sys.argv[1:] or ["demo", "repro", "hull", "loads", "unit", "calibrated"]
    if "demo" in which:
        demo(0.01, 0.02)
        demo(0.015, 0.03)
    if "repro" in which:
        repro()
    if "hull" in which:
        hull()
    if "loads" in which:
        loads()
    if "unit" in which:
        unit_cases()
    if "calibrated" in which:
        calibrated()
