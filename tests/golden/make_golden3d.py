"""Generate golden vectors for the 3-D bonded-sphere step from the reference itself.

Run in a container where the reference source tree is mounted::

    PYTHONPATH=<reference>/src python tests/golden/make_golden3d.py

It imports the reference ``tensordem.dem3d.IceDEM3D`` (``src/tensordem/dem3d.py``),
runs it on CPU in float64 with one torch thread (as its CLI does,
``src/tensordem/dem3d_cli.py:101-102``) and writes ``tests/golden/dem3d_*.npz``.
The fixtures are committed; nothing at test time reads the reference tree.

Cases (each records, at the frame steps, positions, velocities, bond states,
the side-effect-free ``forces(update_fracture=False, update_history=False)``
probe and ``diagnostics()``; at the end the failure ledger, ``energy()`` and
the bond-law state). For a one-step replay from the reference's own state,
each frame (but the last) also stores the pair friction history, the platen
spring offsets, the Maxwell branch state, the lateral platen positions, and
the positions, velocities and bond states one step later:

* ``dem3d_box``: the 9x5x3 default specimen under the spherical indenter at
  breaking strains 0.004 / 0.008 with restitution 0.7 (fixed x edges, so
  pinned pairs take the full particle mass).
* ``dem3d_hertz_friction``: Hertz contacts, Cundall-Strack friction with the
  tanh static/dynamic cone, rolling resistance, gravity, a bottom platen with
  friction, free edges.
* ``dem3d_mindlin``: Hertz contacts with the Mindlin-Deresiewicz partial-slip
  law for pairs and for a frictional bottom platen, gravity, free edges.
* ``dem3d_calibrated``: Hertz contacts with the calibrated restitution
  dashpot (``contact_damping_model="restitution_calibrated"``, e = 0.5), the
  reference's damping ratio recorded as ``zeta``; fixed bottom layer, friction.
* ``dem3d_cylinder``: the ``cylinder_xz`` geometry with Maxwell-Wiechert bonds,
  the creep clock, Weibull strengths, dual-cone friction, an absolute dashpot,
  buoyancy and wet drag, a descending top platen and four lateral platens
  driven inward.
* ``dem3d_loads``: a 5x3x2 specimen with seeded external nodal loads that
  change every step.
* ``dem3d_unit``: single probes of hand-edited states (coincident particles,
  a particle at the indenter centre, a stretched and a compressed pair).
"""

from __future__ import annotations

import json
import math
from dataclasses import asdict
from pathlib import Path

import numpy as np
import torch

from tensordem.contact_calibration import hertz_damping_ratio_for_restitution  # reference package
from tensordem.dem3d import DEM3DConfig, IceDEM3D  # reference package

OUT = Path(__file__).resolve().parent
DIAG_KEYS = ("reaction_x", "reaction_y", "reaction_z", "top_platen_reaction_z_N",
             "bottom_platen_reaction_z_N", "boundary_reaction_x", "boundary_reaction_y",
             "boundary_reaction_z", "broken_bonds", "kinetic_energy_J", "bond_elastic_energy_J",
             "particle_contact_energy_J", "tool_contact_energy_J", "platen_contact_energy_J",
             "released_bond_energy_J", "lateral_platen_energy_J", "mechanical_energy_J",
             "gravity_force_z_N", "buoyancy_force_z_N", "wet_drag_force_z_N", "net_body_force_z_N",
             "submerged_volume_m3")
ENERGY_KEYS = ("kinetic_energy_J", "bond_elastic_energy_J", "particle_contact_energy_J",
               "tool_contact_energy_J", "platen_contact_energy_J", "released_bond_energy_J",
               "mechanical_energy_J")


def _np(t):
    return t.detach().cpu().numpy().copy()


def _frame(sim: IceDEM3D, rec: dict, step: int) -> None:
    force, reaction = sim.forces(update_fracture=False, update_history=False)
    diag = sim.diagnostics()
    rec["frame_step"].append(step)
    rec["frame_time"].append(sim.time)
    rec["frame_pos"].append(_np(sim.positions))
    rec["frame_vel"].append(_np(sim.velocities))
    rec["frame_alive"].append(_np(sim.alive))
    rec["frame_force"].append(_np(force))
    rec["frame_reaction"].append(_np(reaction))
    rec["frame_diag"].append([float(diag[k]) for k in DIAG_KEYS])
    rec["frame_lateral"].append(list(diag["lateral_platen_reaction"]))


def run_case(name: str, cfg: DEM3DConfig, steps: int, frames, *, setup=None, loads_fn=None,
             extra=None) -> None:
    torch.manual_seed(0)
    sim = IceDEM3D(cfg)
    if setup is not None:
        setup(sim)
    rec = {k: [] for k in ("frame_step", "frame_time", "frame_pos", "frame_vel", "frame_alive",
                           "frame_force", "frame_reaction", "frame_diag", "frame_lateral")}
    teach = {k: [] for k in ("hist_count", "hist_pairs", "hist_disp", "top_tang", "bottom_tang",
                             "offsets", "elong_prev", "damage", "lateral_pos", "dissipation",
                             "next_pos", "next_vel", "next_alive")}
    loads_log = []
    for s in range(steps + 1):
        frame = s in frames
        if frame:
            _frame(sim, rec, s)
        if s == steps:
            break
        if frame:
            # everything a one-step replay needs beyond the frame itself
            keys = sorted(sim._tangential_state)
            teach["hist_count"].append(len(keys))
            teach["hist_pairs"].extend([(k // 1_000_003, k % 1_000_003) for k in keys])
            teach["hist_disp"].extend([_np(sim._tangential_state[k][0]) for k in keys])
            teach["top_tang"].append(_np(sim._top_platen_tang_disp))
            teach["bottom_tang"].append(_np(sim._bottom_platen_tang_disp))
            teach["offsets"].append(_np(sim.branch_offsets))
            teach["elong_prev"].append(_np(sim._bond_elongation_prev))
            teach["damage"].append(_np(sim.bond_damage))
            teach["lateral_pos"].append(_np(sim.lateral_platen_pos))
            teach["dissipation"].append(sim.cumulative_bond_dissipation_J)
        loads = None if loads_fn is None else loads_fn(sim, s)
        if loads is not None:
            loads_log.append(_np(loads))
        sim.step(loads)
        if frame:
            teach["next_pos"].append(_np(sim.positions))
            teach["next_vel"].append(_np(sim.velocities))
            teach["next_alive"].append(_np(sim.alive))
    energy = sim.energy()
    out = {k: np.asarray(v) for k, v in rec.items()}
    teach["hist_pairs"] = np.asarray(teach["hist_pairs"], dtype=np.int64).reshape(-1, 2)
    teach["hist_disp"] = np.asarray(teach["hist_disp"], dtype=np.float64).reshape(-1, 3)
    out.update({f"teach_{k}": np.asarray(v) for k, v in teach.items()})
    out.update(
        config=json.dumps(asdict(cfg)), dt=sim.dt, steps=steps,
        lateral_velocity=_np(sim.lateral_platen_velocity),
        failure_mode=_np(sim.failure_mode), failure_time_s=_np(sim.failure_time_s),
        failure_extension_m=_np(sim.failure_extension_m), failure_energy_J=_np(sim.failure_energy_J),
        energy=np.asarray([energy[k] for k in ENERGY_KEYS]),
        branch_offsets=_np(sim.branch_offsets), bond_damage=_np(sim.bond_damage),
        bond_dissipation=sim.cumulative_bond_dissipation_J,
        friction_power=sim._last_friction_power, rolling_power=sim._last_rolling_power,
        lateral_pos=_np(sim.lateral_platen_pos), pairs=_np(sim.pairs),
        fixed=_np(sim.fixed), initial_positions=_np(sim.initial_positions),
    )
    if sim.bond_breaking_strain is not None:
        out["bond_breaking_strain"] = _np(sim.bond_breaking_strain)
    if loads_log:
        out["loads"] = np.stack(loads_log)
    out.update(extra or {})
    np.savez_compressed(OUT / f"{name}.npz", **out)
    broken = int((out["failure_mode"] > 0).sum())
    print(f"{name}: n={len(sim.positions)} bonds={len(sim.pairs)} dt={sim.dt:.6g} broken={broken} "
          f"modes={np.bincount(out['failure_mode'], minlength=5).tolist()}")


def unit_case() -> None:
    """Probes of hand-edited states (tests/test_dem3d.py:22-115 style)."""
    out = {}
    gen = torch.Generator().manual_seed(7)
    cfg = DEM3DConfig(nx=3, ny=3, nz=2, drag=0.0, fix_x_edges=False, friction_coefficient=0.3,
                      rolling_resistance_coefficient=0.1, restitution_coefficient=0.5)
    cases = {}
    sim = IceDEM3D(cfg)
    x0 = sim.initial_positions.clone()
    r = cfg.radius
    jitter = (torch.rand(x0.shape, generator=gen, dtype=torch.float64) - 0.5) * 0.3 * r
    cases["jitter"] = (x0 + jitter, (torch.rand(x0.shape, generator=gen, dtype=torch.float64) - 0.5) * 0.2)
    coincide = x0.clone()
    coincide[1] = coincide[0]
    cases["coincident"] = (coincide, torch.zeros_like(x0))
    stretch = x0.clone()
    stretch[:, 0] *= 1.01
    cases["stretch"] = (stretch, torch.zeros_like(x0))
    squeeze = x0.clone()
    squeeze[:, 2] *= 0.5
    cases["squeeze"] = (squeeze, (torch.rand(x0.shape, generator=gen, dtype=torch.float64) - 0.5) * 0.1)
    tool = x0.clone()
    tool[4] = torch.tensor([0.0, 0.0, float(sim.tool_start[2])], dtype=torch.float64)
    cases["tool_centre"] = (tool, torch.zeros_like(x0))
    for name, (p, v) in cases.items():
        s = IceDEM3D(cfg)
        s.positions = p.clone()
        s.velocities = v.clone()
        f, rr = s.forces(update_fracture=False, update_history=False)
        f2, rr2 = s.forces()  # commits breaks and advances the friction history
        out[f"{name}_pos"] = _np(p)
        out[f"{name}_vel"] = _np(v)
        out[f"{name}_force_probe"] = _np(f)
        out[f"{name}_reaction_probe"] = _np(rr)
        out[f"{name}_force"] = _np(f2)
        out[f"{name}_reaction"] = _np(rr2)
        out[f"{name}_alive"] = _np(s.alive)
        out[f"{name}_friction_power"] = np.float64(s._last_friction_power)
        out[f"{name}_rolling_power"] = np.float64(s._last_rolling_power)
    out["config"] = json.dumps(asdict(cfg))
    np.savez_compressed(OUT / "dem3d_unit.npz", **out)
    print("dem3d_unit:", sorted(cases))


def main() -> None:
    torch.set_num_threads(1)
    frames = sorted(set([0, 1, 2, 5, 10, 50] + list(range(100, 1401, 100))))
    run_case("dem3d_box", DEM3DConfig(breaking_strain=0.004, shear_breaking_strain=0.008,
                                      restitution_coefficient=0.7), 1400, frames)
    hertz = DEM3DConfig(nx=7, ny=4, nz=3, contact_model="hertz", young_modulus=2.0e6, poisson_ratio=0.3,
                        friction_coefficient=0.4, rolling_resistance_coefficient=0.05,
                        restitution_coefficient=0.6, breaking_strain=0.004, shear_breaking_strain=0.008,
                        tool_gap=0.002, fix_x_edges=False, bottom_platen_enabled=True,
                        platen_friction_coefficient=0.3, friction_regularization="tanh",
                        static_friction_coefficient=0.5, dynamic_friction_coefficient=0.3,
                        gravity=9.81)
    run_case("dem3d_hertz_friction", hertz, 1200, sorted(set([0, 1, 5, 50] + list(range(100, 1201, 100)))))
    mindlin = DEM3DConfig(nx=6, ny=4, nz=3, contact_model="hertz", young_modulus=2.0e6, poisson_ratio=0.3,
                          tangential_model="mindlin_partial_slip", friction_coefficient=0.4,
                          breaking_strain=0.004, shear_breaking_strain=0.008, tool_gap=0.002, fix_x_edges=False,
                          bottom_platen_enabled=True, platen_friction_coefficient=0.3, gravity=9.81)
    run_case("dem3d_mindlin", mindlin, 1000, sorted(set([0, 1, 5, 50] + list(range(100, 1001, 100)))))
    calibrated = DEM3DConfig(nx=6, ny=4, nz=3, contact_model="hertz", young_modulus=2.0e6, poisson_ratio=0.3,
                             contact_damping_model="restitution_calibrated", restitution_coefficient=0.5,
                             friction_coefficient=0.3, breaking_strain=0.004, shear_breaking_strain=0.008,
                             tool_gap=0.002, fix_bottom=True)
    run_case("dem3d_calibrated", calibrated, 1000, sorted(set([0, 1, 5, 50] + list(range(100, 1001, 100)))),
             extra={"zeta": hertz_damping_ratio_for_restitution(0.5)})
    cyl = DEM3DConfig(nx=7, ny=3, nz=7, geometry="cylinder_xz", bond_model="maxwell_wiechert",
                      bond_creep_exponent=2, bond_creep_time_s=0.05, bond_strength_weibull_modulus=5.0,
                      bond_strength_seed=3, lateral_platens=True, water_level=0.0, gravity=9.81,
                      wet_drag_coefficient=0.5, friction_coefficient=0.3, friction_regularization="dual",
                      static_friction_coefficient=0.4, dynamic_friction_coefficient=0.25,
                      breaking_strain=0.006, shear_breaking_strain=0.012, top_platen_enabled=True,
                      top_platen_velocity=-0.3, platen_damping=0.5, contact_damping_model="absolute",
                      contact_damping=2.0, tool_speed=0.3)

    def squeeze(sim):
        sim.lateral_platen_velocity = torch.tensor([0.05, -0.05, 0.05, -0.05], dtype=torch.float64)

    run_case("dem3d_cylinder", cyl, 1200, sorted(set([0, 1, 5, 50] + list(range(100, 1201, 100)))),
             setup=squeeze)
    gen = torch.Generator().manual_seed(11)

    def loads(sim, s):
        return (torch.rand(sim.positions.shape, generator=gen, dtype=torch.float64) - 0.5) * 4.0

    run_case("dem3d_loads", DEM3DConfig(nx=5, ny=3, nz=2, breaking_strain=0.004, shear_breaking_strain=0.008),
             60, set(range(0, 61, 5)), loads_fn=loads)
    unit_case()


if __name__ == "__main__":
    main()
