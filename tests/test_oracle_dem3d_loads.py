"""The reference's 3-D external-load and platen-damper checks (its
tests/test_dem3d_external_load_balance.py:23-129) on the numpy oracle of the 3-D
step (oracle/icedem3d.py), which the CUDA path is checked against: nodal loads
add exactly to the internal forces, the vertical resultant equals the applied
load, fixed supports stay pinned under load, and both platen dampers oppose
the approach with exactly c v per disc."""

import numpy as np

from oracle.icedem3d import IceDEM3DOracle, Oracle3DConfig

_BASE = dict(nx=5, ny=2, nz=2, radius=0.01, density=917.0, bond_stiffness=2_000.0, contact_stiffness=5_000.0,
             contact_damping=0.05, drag=0.2, fix_x_edges=False, tool_gap=1.0, tool_radius=0.01, tool_speed=0.01)


def _small(**overrides):
    from tensordem_gb300.dem3d import DEM3DConfig
    params = {**_BASE, **overrides}
    dt = DEM3DConfig(**params).recommended_dt
    o = IceDEM3DOracle(Oracle3DConfig(**params), dt=dt)
    # park the indenter far away: only bonds, loads and platens act
    o.tool_start[:] = 1e6
    o.tool_velocity[:] = 0.0
    return o


def test_external_loads_add_to_the_internal_forces():
    o = _small()
    loads = np.zeros_like(o.positions)
    loads[3, 2] = -0.75
    loads[7, 0] = 1.25
    base, _ = o.forces(update_fracture=False)
    loaded, _ = o.forces(loads, update_fracture=False)
    assert np.array_equal(loaded - base, loads)


def test_vertical_resultant_equals_the_applied_load():
    o = _small(drag=0.0)
    loads = np.zeros_like(o.positions)
    loads[:, 2] = -0.01
    force, _ = o.forces(loads, update_fracture=False)
    assert abs(float(force[:, 2].sum()) - float(loads[:, 2].sum())) < 5e-16


def test_fixed_supports_stay_pinned_under_load():
    o = _small()
    o.fixed[:] = False
    o.fixed[[0, len(o.positions) - 1]] = True
    loads = np.zeros_like(o.positions)
    loads[:, 2] = -0.02
    for _ in range(20):
        o.step(loads)
    assert np.array_equal(o.positions[o.fixed], o.initial_positions[o.fixed])
    assert not o.velocities[o.fixed].any()


def _platen_force_z(o, layer, vz):
    o.velocities[:] = 0.0
    o.velocities[layer, 2] = vz
    force, _ = o.forces(update_fracture=False)
    return float(force[:, 2].sum())


def test_bottom_platen_damper_opposes_approach():
    o = _small(bottom_platen_enabled=True, platen_stiffness=4_000.0, platen_damping=50.0, drag=0.0)
    bottom = o.positions[:, 2] == o.positions[:, 2].min()
    o.positions[bottom, 2] -= 0.002  # pressed into the platen
    count = int(bottom.sum())
    assert count > 0
    static = _platen_force_z(o, bottom, 0.0)
    damping = 50.0 * 0.03 * count
    assert abs(_platen_force_z(o, bottom, -0.03) - static - damping) <= 1e-12
    assert abs(_platen_force_z(o, bottom, +0.03) - static + damping) <= 1e-12


def test_top_platen_damper_opposes_approach():
    o = _small(top_platen_enabled=True, platen_stiffness=4_000.0, platen_damping=50.0, drag=0.0)
    top = o.positions[:, 2] == o.positions[:, 2].max()
    o.positions[top, 2] += 0.002
    count = int(top.sum())
    static = _platen_force_z(o, top, 0.0)
    damping = 50.0 * 0.03 * count
    assert abs(_platen_force_z(o, top, +0.03) - static + damping) <= 1e-12
    assert abs(_platen_force_z(o, top, -0.03) - static - damping) <= 1e-12
