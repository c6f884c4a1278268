"""The reference's 2-D mechanics-invariant and load-interface checks (its
tests/test_mechanics_invariants.py:15-131 and tests/test_load_interface.py:12-48)
on the numpy oracle of the reference mode (oracle/icedem.py), with the same
inputs and bounds: the oracle itself obeys them before it checks the CUDA
path (tests/test_icedem_reference_checks_gpu.py runs them there)."""

import numpy as np

from oracle.icedem import IceDEMOracle, OracleConfig


def _sim(**kw):
    return IceDEMOracle(OracleConfig(**kw))


def test_internal_forces_conserve_resultant_and_moment():
    sim = _sim(nx=4, ny=3, drag=0.0, fix_edges=False, breaking_strain=10.0, shear_breaking_strain=10.0,
               tool_gap=10.0, tool_speed=0.01)
    sim.positions[5, 0] += 1.0e-3
    loads = np.arange(2 * len(sim.positions), dtype=np.float64).reshape(-1, 2) * 0.25 - 1.0
    force, reaction = sim.forces(loads)
    np.testing.assert_allclose(force.sum(0), loads.sum(0), atol=1e-10, rtol=1e-10)
    assert np.isfinite(reaction).all()
    pos = sim.positions
    moment = (pos[:, 0] * force[:, 1] - pos[:, 1] * force[:, 0]).sum()
    load_moment = (pos[:, 0] * loads[:, 1] - pos[:, 1] * loads[:, 0]).sum()
    assert abs(moment - load_moment) <= 1e-10 + 1e-10 * abs(load_moment)


def test_zero_load_is_identical_to_omitted_load():
    sim = _sim(nx=4, ny=3, drag=0.0, fix_edges=False, tool_gap=10.0, tool_speed=0.01)
    sim.positions[4, 0] += 2.0e-4
    f_none, r_none = sim.forces()
    f_zero, r_zero = sim.forces(np.zeros_like(sim.positions))
    assert np.array_equal(f_zero, f_none) and np.array_equal(r_zero, r_none)


def test_halving_the_timestep_reduces_the_trajectory_error():
    base = dict(nx=4, ny=3, drag=0.0, breaking_strain=10.0, shear_breaking_strain=10.0, tool_gap=10.0,
                tool_speed=0.01)
    coarse_dt = 0.5 * OracleConfig(**base).recommended_dt
    horizon = 8 * coarse_dt
    loads = np.zeros((12, 2))
    loads[5, 0] = 0.02

    def final(dt):
        sim = _sim(**base, dt=dt)
        for _ in range(round(horizon / dt)):
            sim.step(loads)
        assert abs(sim.time - horizon) < 5e-13
        return sim.positions.copy()

    coarse, medium, fine = final(coarse_dt), final(coarse_dt / 2), final(coarse_dt / 4)
    assert np.isfinite(fine).all()
    e_coarse, e_medium = np.linalg.norm(coarse - fine), np.linalg.norm(medium - fine)
    assert e_coarse > 0.0 and e_medium < e_coarse


def test_external_load_is_additive_and_step_uses_it():
    sim = _sim(nx=3, ny=2, drag=0, fix_edges=False)
    baseline, _ = sim.forces()
    loads = np.zeros_like(sim.positions)
    loads[2, 1] = 12.5
    loaded, _ = sim.forces(loads)
    np.testing.assert_allclose(loaded - baseline, loads, rtol=1.3e-6, atol=1e-5)
    sim.step(loads)
    assert sim.velocities[2, 1] > 0.0 and np.isfinite(sim.positions).all()


def test_fixed_supports_hold_under_loads():
    sim = _sim(nx=5, ny=3, drag=0)
    loads = np.zeros_like(sim.positions)
    loads[sim.fixed, 0] = 3.0
    force, _ = sim.forces(loads)
    assert np.isfinite(-force[sim.fixed].sum(0)).all()
    sim.step(loads)
    assert np.array_equal(sim.positions[sim.fixed], sim.initial_positions[sim.fixed])

