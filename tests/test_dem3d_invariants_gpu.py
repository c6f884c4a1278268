"""The reference's own 3-D known-answer checks (its tests/test_dem3d.py:22-347),
restated against the CUDA path of ``tensordem_gb300.dem3d``.

Each test names the reference test it follows. They exercise the drop-in's
surface (forces, step, diagnostics, state_dict / load_state_dict, platens,
the cylinder geometry, the CLI) with the reference's own inputs and bounds.
"""

import csv
import math

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def m3():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300 import dem3d
    return dem3d


def _small(m3, **kw):
    return m3.IceDEM3D(m3.DEM3DConfig(nx=3, ny=3, nz=2, drag=0.0, fix_x_edges=False, **kw))


def test_initial_equilibrium_and_force_balance(m3):
    sim = _small(m3)
    force, reaction = sim.forces()
    assert bool(torch.isfinite(force).all())
    torch.testing.assert_close(force.sum(0), -reaction, atol=1e-10, rtol=0)
    assert float(force.abs().max()) < 1e-8


def test_rigid_rotation_does_not_break_bonds(m3):
    sim = _small(m3)
    a, b = 0.41, -0.27
    rx = torch.tensor([[1.0, 0.0, 0.0], [0.0, math.cos(a), -math.sin(a)], [0.0, math.sin(a), math.cos(a)]],
                      dtype=torch.float64, device="cuda")
    ry = torch.tensor([[math.cos(b), 0.0, math.sin(b)], [0.0, 1.0, 0.0], [-math.sin(b), 0.0, math.cos(b)]],
                      dtype=torch.float64, device="cuda")
    sim.positions = sim.initial_positions @ (rx @ ry).T + torch.tensor([2.0, -3.0, 4.0], dtype=torch.float64,
                                                                       device="cuda")
    force, _ = sim.forces()
    assert sim.broken_bonds == 0
    assert float(force.abs().max()) < 1e-7


def test_tension_failure_is_irreversible(m3):
    sim = _small(m3, breaking_strain=0.01, shear_breaking_strain=0.5)
    sim.positions = sim.initial_positions * 1.03
    sim.forces()
    broken = sim.broken_bonds
    assert broken > 0
    sim.positions = sim.initial_positions.clone()
    sim.forces()
    assert sim.broken_bonds == broken


def test_external_load_shape_and_finiteness(m3):
    sim = _small(m3)
    with pytest.raises(ValueError):
        sim.forces(torch.zeros((len(sim.positions), 2), dtype=torch.float64, device="cuda"))
    loads = torch.zeros_like(sim.positions)
    loads[0, 0] = 1.0
    force, _ = sim.forces(loads)
    assert bool(torch.isfinite(force).all())
    loads[0, 0] = float("nan")
    with pytest.raises(ValueError):
        sim.forces(loads)


def test_step_fixed_boundary_and_finite_state(m3):
    sim = m3.IceDEM3D(m3.DEM3DConfig(nx=4, ny=3, nz=2))
    fixed0 = sim.positions[sim.fixed].clone()
    for _ in range(20):
        sim.step()
    assert torch.equal(sim.positions[sim.fixed], fixed0)
    assert bool(torch.isfinite(sim.positions).all())
    assert sim.step_count == 20


def test_cell_list_covers_all_overlapping_pairs_without_duplicates(m3):
    sim = _small(m3)
    gen = torch.Generator().manual_seed(73)
    sim.positions = (torch.randn(sim.positions.shape, generator=gen, dtype=torch.float64) * 0.035).to("cuda")
    sim.forces(update_fracture=False, update_history=False)
    pairs = sim.contact_pairs().tolist()
    assert len(pairs) == len(set(map(tuple, pairs)))
    d = torch.cdist(sim.positions, sim.positions)
    truth = {tuple(p) for p in torch.triu(d < 2 * sim.config.radius, 1).nonzero().tolist()}
    assert truth == set(map(tuple, pairs))


def test_broken_bond_is_still_eligible_for_contact(m3):
    sim = _small(m3)
    i, j = (int(v) for v in sim.pairs[0])
    sim.positions[j] = sim.positions[i] + torch.tensor([sim.config.radius, 0.0, 0.0], dtype=torch.float64,
                                                       device="cuda")
    sim.alive[0] = False
    force, _ = sim.forces(update_fracture=False, update_history=False)
    assert (i, j) in {tuple(p) for p in sim.contact_pairs().tolist()}
    assert float(force[j, 0]) > 0.0  # a live contact pushes j away from i along +x


def test_checkpoint_rejects_incompatible_or_corrupt_state(m3):
    sim = _small(m3)
    snap = sim.state_dict()
    broken = dict(snap)
    broken["positions"] = torch.zeros((1, 3), dtype=torch.float64)
    with pytest.raises(ValueError):
        sim.load_state_dict(broken)
    other = m3.IceDEM3D(m3.DEM3DConfig(nx=4, ny=3, nz=2, drag=0.0, fix_x_edges=False))
    with pytest.raises(ValueError):
        other.load_state_dict(snap)


def _assert_state_equal(a: dict, b: dict) -> None:
    for key, value in a.items():
        if isinstance(value, torch.Tensor):
            assert torch.equal(value, b[key]), key
        elif isinstance(value, dict):
            for sub, sv in value.items():
                if isinstance(sv, torch.Tensor):
                    assert torch.equal(sv, b[key][sub]), f"{key}.{sub}"
                else:
                    assert sv == b[key][sub], f"{key}.{sub}"
        else:
            assert value == b[key], key


def test_diagnostics_is_pure_even_when_pending_fracture_exceeds_threshold(m3):
    sim = _small(m3)
    sim.positions = sim.initial_positions * 1.03
    sim.last_reaction = torch.tensor([1.0, 2.0, 3.0], dtype=torch.float64)
    before = sim.state_dict()
    reaction_before = sim.last_reaction.clone()
    for _ in range(3):
        row = sim.diagnostics()
        assert row["broken_bonds"] == 0
        assert row["bond_elastic_energy_J"] > 0
    _assert_state_equal(before, sim.state_dict())
    assert torch.equal(sim.last_reaction.cpu(), reaction_before)
    sim.forces()  # the default call still commits the pending fracture
    assert sim.broken_bonds > 0


def test_observation_frequency_preserves_fracture_history_and_force_evolution(m3):
    unobserved, observed = _small(m3), _small(m3)
    for scale in (1.005, 1.01, 1.03, 1.0, 1.04):
        for sim in (unobserved, observed):
            sim.positions = sim.initial_positions * scale
        for _ in range(5):
            observed.diagnostics()
        unobserved.step()
        observed.step()
        for key in ("positions", "velocities", "alive", "failure_mode", "failure_time_s", "failure_extension_m",
                    "failure_energy_J"):
            assert torch.equal(getattr(unobserved, key), getattr(observed, key)), key
        for a, b in zip(unobserved.forces(update_fracture=False), observed.forces(update_fracture=False)):
            assert torch.equal(a, b)
    assert unobserved.broken_bonds > 0


def test_checkpoint_dtype_corruption_rejected_atomically_before_conversion(m3):
    sim = _small(m3)
    original = sim.state_dict()
    corruptions = {
        "alive": torch.full(sim.alive.shape, float("nan"), dtype=torch.float64),
        "pairs": sim.pairs.to(torch.float64) + 0.2,
        "failure_mode": sim.failure_mode.to(torch.int64) + 256,
        "positions": sim.positions.to(torch.float32),
    }
    for key, tensor in corruptions.items():
        corrupt = dict(original)
        corrupt[key] = tensor
        with pytest.raises(ValueError, match="dtype"):
            sim.load_state_dict(corrupt)
        _assert_state_equal(original, sim.state_dict())


def test_moving_plane_platens_report_action_reaction_and_energy(m3):
    sim = _small(m3, top_platen_enabled=True, bottom_platen_enabled=True, platen_stiffness=4000.0,
                 platen_damping=0.0, top_platen_velocity=-0.1, bottom_platen_velocity=0.1)
    sim.time = 0.01
    force, _ = sim.forces(update_fracture=False)
    assert bool(torch.isfinite(force).all())
    assert float(sim.last_top_platen_reaction_z) > 0.0
    assert float(sim.last_bottom_platen_reaction_z) < 0.0
    row = sim.diagnostics()
    assert row["top_platen_reaction_z_N"] > 0.0 and row["bottom_platen_reaction_z_N"] < 0.0
    assert row["platen_contact_energy_J"] > 0.0
    assert math.isfinite(row["mechanical_energy_J"])


def test_plane_platen_configuration_validation(m3):
    for bad in (dict(platen_stiffness=0.0), dict(top_platen_gap=-1e-3), dict(bottom_platen_velocity=float("nan"))):
        with pytest.raises(ValueError):
            _small(m3, **bad)


def test_checkpoint_without_new_platen_keys_remains_loadable(m3):
    original = _small(m3)
    snap = original.state_dict()
    for key in ("top_platen_enabled", "bottom_platen_enabled", "platen_stiffness", "platen_damping",
                "top_platen_gap", "bottom_platen_gap", "top_platen_velocity", "bottom_platen_velocity"):
        snap["config"].pop(key, None)
    resumed = _small(m3)
    resumed.load_state_dict(snap)
    assert torch.equal(resumed.positions, original.positions)


def test_cli_can_run_with_moving_plane_platens(m3, tmp_path):
    from tensordem_gb300.cli import main
    out = tmp_path / "platen-cli"
    main(["dem-3d", "--nx", "3", "--ny", "3", "--nz", "2", "--steps", "2", "--save-every", "1", "--top-platen",
          "--bottom-platen", "--top-platen-velocity", "-0.05", "--bottom-platen-velocity", "0.05",
          "--output", str(out)])
    with (out / "history.csv").open(newline="", encoding="utf-8") as stream:
        rows = list(csv.DictReader(stream))
    assert rows
    for key in ("top_platen_reaction_z_N", "bottom_platen_reaction_z_N", "platen_contact_energy_J"):
        assert key in rows[0]


def test_cylinder_xz_geometry_is_compact_and_bonded(m3):
    sim = m3.IceDEM3D(m3.DEM3DConfig(nx=9, ny=3, nz=9, geometry="cylinder_xz", fix_x_edges=False, drag=0.0))
    n = len(sim.positions)
    assert n < 9 * 3 * 9 and tuple(sim.positions.shape) == (len(sim.velocities), 3)
    assert bool((sim.pairs >= 0).all()) and bool((sim.pairs < n).all())
    assert len(torch.unique(sim.pairs[:, 0] * n + sim.pairs[:, 1])) == len(sim.pairs)
    radial = torch.sqrt(sim.initial_positions[:, 0] ** 2 + sim.initial_positions[:, 2] ** 2)
    assert float(radial.max()) <= 4 * 2 * sim.config.radius + 1e-12
    force, reaction = sim.forces(update_fracture=False)
    assert bool(torch.isfinite(force).all())
    torch.testing.assert_close(force.sum(0), -reaction, atol=1e-9, rtol=0)
    assert float(force.abs().max()) < 1e-7


def test_cylinder_geometry_validation_and_checkpoint_round_trip(m3):
    with pytest.raises(ValueError):
        m3.DEM3DConfig(nx=2, nz=5, geometry="cylinder_xz")
    with pytest.raises(ValueError):
        m3.DEM3DConfig(geometry="sphere")
    cfg = m3.DEM3DConfig(nx=7, ny=2, nz=7, geometry="cylinder_xz", fix_x_edges=False)
    sim = m3.IceDEM3D(cfg)
    snap = sim.state_dict()
    resumed = m3.IceDEM3D(cfg)
    resumed.load_state_dict(snap)
    assert torch.equal(resumed.positions, sim.positions) and torch.equal(resumed.pairs, sim.pairs)
