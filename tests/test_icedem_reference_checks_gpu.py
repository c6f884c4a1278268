"""More of the reference's own 2-D checks on the CUDA path of ``IceDEM``, with
the reference's inputs and bounds:

* tests/test_mechanics_invariants.py:15-131 - internal forces conserve the
  resultant and the moment of the external loads; the support reaction is the
  negative fixed-node force residual; a zero load equals an omitted one; halving
  dt reduces the trajectory error;
* tests/test_load_interface.py:12-48 - loads are additive and used by step();
  shape / finiteness / type guards; fixed supports stay put under loads;
* tests/test_fracture_events.py:24-83 - tensile and shear failures recorded with
  mode, time, midpoint and energy; restart keeps the fracture ledger and rejects
  an inconsistent one; a repeated force evaluation adds nothing;
* tests/test_hull_contact_integration.py:12-50 - a prescribed polyline hull
  gives a balanced horizontal reaction, moves at its velocity, and a
  zero-length segment is rejected.
"""

import copy

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def td():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    import tensordem_gb300
    return tensordem_gb300


def _cpu(x):
    return x.detach().cpu()


# -- mechanics invariants -----------------------------------------------------

def test_internal_forces_conserve_resultant_and_moment(td):
    sim = td.IceDEM(td.DEMConfig(nx=4, ny=3, drag=0.0, fix_edges=False, breaking_strain=10.0,
                                 shear_breaking_strain=10.0, tool_gap=10.0, tool_speed=0.01))
    sim.positions[5, 0] += 1.0e-3
    loads = torch.arange(2 * len(sim.positions), dtype=torch.float64).reshape(-1, 2) * 0.25 - 1.0
    force, reaction = sim.forces(external_forces=loads)
    force, pos = _cpu(force), _cpu(sim.positions)
    torch.testing.assert_close(force.sum(0), loads.sum(0), atol=1e-10, rtol=1e-10)
    assert bool(torch.isfinite(_cpu(reaction)).all())
    moment = (pos[:, 0] * force[:, 1] - pos[:, 1] * force[:, 0]).sum()
    load_moment = (pos[:, 0] * loads[:, 1] - pos[:, 1] * loads[:, 0]).sum()
    torch.testing.assert_close(moment, load_moment, atol=1e-10, rtol=1e-10)


def test_support_reaction_is_negative_fixed_node_residual(td):
    sim = td.IceDEM(td.DEMConfig(nx=5, ny=3, drag=0.0, breaking_strain=10.0, shear_breaking_strain=10.0,
                                 tool_gap=10.0, tool_speed=0.01))
    sim.positions[7, 0] += 5.0e-4
    loads = torch.zeros_like(sim.positions)
    loads[sim.fixed, 0] = 2.0
    loads[2, 1] = 1.5
    force, _ = sim.forces(external_forces=loads)
    expected = _cpu(-force[sim.fixed].sum(0))
    diag = sim.diagnostics(external_forces=loads)
    got = torch.tensor([diag["boundary_reaction_x"], diag["boundary_reaction_y"]], dtype=torch.float64)
    torch.testing.assert_close(got, expected, atol=1e-10, rtol=1e-10)


def test_zero_load_is_identical_to_omitted_load(td):
    sim = td.IceDEM(td.DEMConfig(nx=4, ny=3, drag=0.0, fix_edges=False, tool_gap=10.0, tool_speed=0.01))
    sim.positions[4, 0] += 2.0e-4
    f_none, r_none = sim.forces()
    f_zero, r_zero = sim.forces(external_forces=torch.zeros_like(sim.positions))
    torch.testing.assert_close(f_zero, f_none, atol=0.0, rtol=0.0)
    torch.testing.assert_close(r_zero, r_none, atol=0.0, rtol=0.0)


def test_halving_the_timestep_reduces_the_trajectory_error(td):
    base = dict(nx=4, ny=3, drag=0.0, breaking_strain=10.0, shear_breaking_strain=10.0, tool_gap=10.0,
                tool_speed=0.01)
    coarse_dt = 0.5 * td.DEMConfig(**base).recommended_dt
    horizon = 8 * coarse_dt
    loads = torch.zeros((12, 2), dtype=torch.float64)
    loads[5, 0] = 0.02

    def final(dt):
        sim = td.IceDEM(td.DEMConfig(**base, dt=dt))
        for _ in range(round(horizon / dt)):
            sim.step(external_forces=loads)
        assert abs(sim.time - horizon) < 5e-13
        return _cpu(sim.positions)

    coarse, medium, fine = final(coarse_dt), final(coarse_dt / 2), final(coarse_dt / 4)
    assert bool(torch.isfinite(fine).all())
    e_coarse = float(torch.linalg.vector_norm(coarse - fine))
    e_medium = float(torch.linalg.vector_norm(medium - fine))
    assert e_coarse > 0.0 and e_medium < e_coarse


# -- load interface -----------------------------------------------------------

def test_external_load_is_additive_and_step_uses_it(td):
    sim = td.IceDEM(td.DEMConfig(nx=3, ny=2, drag=0, fix_edges=False))
    baseline, _ = sim.forces()
    loads = torch.zeros_like(sim.positions)
    loads[2, 1] = 12.5
    loaded, _ = sim.forces(external_forces=loads)
    torch.testing.assert_close(loaded - baseline, loads)
    sim.step(external_forces=loads)
    assert float(sim.velocities[2, 1]) > 0.0
    assert bool(torch.isfinite(sim.positions).all())


def test_external_load_guards(td):
    sim = td.IceDEM(td.DEMConfig(nx=3, ny=2, fix_edges=False))
    with pytest.raises(ValueError):
        sim.forces(torch.zeros((len(sim.positions), 3), dtype=torch.float64))
    invalid = torch.zeros_like(sim.positions)
    invalid[0, 0] = float("nan")
    with pytest.raises(ValueError):
        sim.step(invalid)
    with pytest.raises(TypeError):
        sim.forces([[0.0, 0.0]] * len(sim.positions))


def test_fixed_supports_hold_under_loads(td):
    sim = td.IceDEM(td.DEMConfig(nx=5, ny=3, drag=0))
    loads = torch.zeros_like(sim.positions)
    loads[sim.fixed, 0] = 3.0
    force, _ = sim.forces(external_forces=loads)
    assert bool(torch.isfinite(-force[sim.fixed].sum(0)).all())
    sim.step(external_forces=loads)
    assert torch.equal(sim.positions[sim.fixed], sim.initial_positions[sim.fixed])
    diag = sim.diagnostics(external_forces=loads)
    assert "boundary_reaction_x" in diag and "boundary_reaction_y" in diag
    assert torch.isfinite(torch.tensor(diag["boundary_reaction_x"]))


# -- fracture events ----------------------------------------------------------

def _fracture_sim(td, tensile=1.0e-4, shear=10.0):
    return td.IceDEM(td.DEMConfig(nx=4, ny=3, fix_edges=False, drag=0.0, breaking_strain=tensile,
                                  shear_breaking_strain=shear, tool_gap=10.0, tool_speed=0.01))


def _stretched(td):
    sim = _fracture_sim(td)
    sim.positions[5, 0] += 1.0e-3
    sim.forces()
    return sim


def test_tensile_failure_records_mode_time_location_and_energy(td):
    sim = _stretched(td)
    events = sim.fracture_events()
    assert events
    assert all(e["mode"] == "tensile" for e in events)
    assert all(e["time_s"] == 0.0 for e in events)
    assert all(e["released_spring_energy_J"] >= 0.0 for e in events)
    assert all(len(e["midpoint_m"]) == 2 for e in events)
    total = sum(e["released_spring_energy_J"] for e in events)
    assert abs(total - sim.accounting["fracture_release_J"]) < 5e-15


def test_shear_failure_is_reported_separately(td):
    sim = _fracture_sim(td, tensile=10.0, shear=1.0e-3)
    sim.positions[:, 0] += 0.02 * sim.positions[:, 1]  # affine simple shear
    sim.forces()
    events = sim.fracture_events()
    assert events and all(e["mode"] == "shear" for e in events)


def test_restart_preserves_the_fracture_ledger(td):
    sim = _stretched(td)
    restored = td.IceDEM.from_snapshot(sim.snapshot())
    assert restored.fracture_events() == sim.fracture_events()
    assert restored.broken_bonds == sim.broken_bonds
    assert restored.accounting["fracture_release_J"] == sim.accounting["fracture_release_J"]


def test_restart_rejects_an_inconsistent_failure_ledger(td):
    sim = _stretched(td)
    state = copy.deepcopy(sim.snapshot())
    broken = next(i for i, mode in enumerate(state["failure_mode"]) if mode > 0)
    state["failure_mode"][broken] = 0
    with pytest.raises(ValueError):
        td.IceDEM.from_snapshot(state)


def test_repeated_force_evaluation_adds_no_failure_energy(td):
    sim = _stretched(td)
    energy, events = sim.accounting["fracture_release_J"], sim.fracture_events()
    sim.forces()
    assert sim.accounting["fracture_release_J"] == energy
    assert sim.fracture_events() == events


# -- prescribed hull ----------------------------------------------------------

_PROFILE = torch.tensor([[0.0, -0.1], [0.0, 0.2]], dtype=torch.float64)


def test_polyline_hull_gives_a_balanced_horizontal_reaction(td):
    sim = td.IceDEM(td.DEMConfig(nx=5, ny=3, tool_speed=0.2, fix_edges=False), hull_profile=_PROFILE,
                    hull_start=(0.01, 0.0), hull_velocity=(0.2, 0.0))
    force, reaction = sim.forces()
    assert float(reaction[0]) > 0.0
    torch.testing.assert_close(_cpu(force.sum(0) + reaction), torch.zeros(2, dtype=torch.float64), rtol=0,
                               atol=1e-12)
    assert abs(float(sim.tool_position[0]) - 0.01) < 5e-13


def test_hull_moves_at_its_prescribed_velocity(td):
    sim = td.IceDEM(td.DEMConfig(nx=5, ny=3, tool_speed=0.2, fix_edges=False), hull_profile=_PROFILE,
                    hull_start=(-0.3, 0.0), hull_velocity=(0.2, 0.0))
    x0 = float(sim.tool_position[0])
    sim.step()
    assert abs(float(sim.tool_position[0]) - (x0 + 0.2 * sim.dt)) < 5e-13


def test_zero_length_hull_segment_is_rejected(td):
    with pytest.raises(ValueError, match="zero-length"):
        td.IceDEM(td.DEMConfig(nx=5, ny=3), hull_profile=torch.tensor([[0.0, 0.0], [0.0, 0.0]]))
