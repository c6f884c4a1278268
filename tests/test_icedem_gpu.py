"""GPU parity of the reference-mode CUDA step against the reference's own outputs.

Golden vectors: tests/golden/*.npz (made by the reference IceDEM,
src/tensordem/dem.py, via tests/golden/make_golden.py). Tolerances: break
ledger bit-exact; frames, forces and accounting within 1e-12 normwise
(tests/_icedem_parity.py).
"""

import math

import numpy as np
import pytest
import torch

from tests import _icedem_parity as P

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


@pytest.fixture(scope="module")
def tdem():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    import tensordem_gb300 as m
    return m


def _sim(tdem, g, **extra):
    return tdem.IceDEM(tdem.DEMConfig(**P.config_dict(g)), **extra)


@pytest.mark.parametrize("name", ["demo_b0.01_s0.02", "demo_b0.015_s0.03"])
def test_demo_parity(tdem, name):
    g = P.load(name)
    sim = _sim(tdem, g)
    worst = P.replay(g, sim, to_np=_np)
    assert sim.broken_bonds == int((g["failure_mode"] > 0).sum())
    print(name, "worst normwise errors", worst, "min break margin", sim.min_break_margin)


def test_demo_run_block_matches_single_steps(tdem):
    g = P.load("demo_b0.01_s0.02")
    a = _sim(tdem, g)
    b = _sim(tdem, g)
    for _ in range(300):
        a.step()
    b.run(300)
    assert torch.equal(a.positions, b.positions)
    assert torch.equal(a.velocities, b.velocities)
    assert torch.equal(a.alive, b.alive)
    assert a.accounting_vector() == b.accounting_vector()
    assert a.time == b.time and a.step_count == b.step_count


def test_reproducibility_bitwise(tdem):
    g = P.load("repro_7x3")
    runs = []
    for _ in range(2):
        sim = _sim(tdem, g)
        sim.run(160)
        runs.append((sim.positions.clone(), sim.velocities.clone(), sim.alive.clone()))
    for x, y in zip(*runs):
        assert torch.equal(x, y)
    P.replay(g, _sim(tdem, g), to_np=_np)


def test_hull_parity(tdem):
    g = P.load("hull_9x3")
    sim = _sim(tdem, g, hull_profile=torch.tensor(g["hull_profile"]),
               hull_start=tuple(g["hull_start"]), hull_velocity=tuple(g["hull_velocity"]))
    P.replay(g, sim, to_np=_np)


def test_external_loads_parity(tdem):
    g = P.load("loads_5x3")
    sim = _sim(tdem, g)
    P.replay(g, sim, to_np=_np,
             loads_fn=lambda s: torch.tensor(g["loads"][s], dtype=torch.float64, device="cuda"))
    last = sim.last_step
    want = g["last_step"]
    assert abs(last["external_work_J"] - want[0]) <= 1e-12 * max(1e-30, abs(want).max())
    assert abs(last["external_moment_Nm"] - want[7]) <= 1e-12 * max(1e-30, abs(want).max())


@pytest.mark.parametrize("case", ["shear", "rotation", "tension", "compress", "contact",
                                  "coincident", "tool"])
def test_unit_force_cases(tdem, case):
    g = P.load("unit_cases")
    if case == "tool":
        sim = tdem.IceDEM(tdem.DEMConfig(nx=5, ny=3))
        sim.time = 0.02
    elif case == "shear":
        sim = tdem.IceDEM(tdem.DEMConfig(nx=3, ny=2, drag=0, fix_edges=False,
                                         shear_breaking_strain=0.02, breaking_strain=0.5))
    else:
        sim = tdem.IceDEM(tdem.DEMConfig(nx=3, ny=2, drag=0, fix_edges=False))
    dev = sim.device
    sim.positions = torch.tensor(g[f"{case}_pos"], device=dev)
    sim.velocities = torch.tensor(g[f"{case}_vel"], device=dev)
    alive = sim.alive.clone()
    alive[sim.bonded] = torch.tensor(g[f"{case}_alive_in"], device=dev)
    if case == "compress":
        alive[sim.bonded] = False
    sim.alive = alive
    f, r = sim.forces()
    want = g[f"{case}_force"]
    assert np.abs(_np(f) - want).max() <= 1e-12 * max(1.0, np.abs(want).max())
    assert np.abs(_np(r) - g[f"{case}_reaction"]).max() <= 1e-12 * max(1.0, np.abs(want).max())
    assert np.array_equal(_np(sim.alive[sim.bonded]), g[f"{case}_alive"])


def test_invariants_from_reference_tests(tdem):
    """tests/test_dem.py:21-119 restated on the GPU path."""
    cfg = dict(nx=3, ny=2, drag=0, fix_edges=False)
    sim = tdem.IceDEM(tdem.DEMConfig(**cfg))
    force, reaction = sim.forces()
    assert float(force.abs().max()) <= 1e-10 and float(reaction.abs().max()) == 0.0
    sim.positions[1, 0] += 0.0001
    force, _ = sim.forces()
    assert float(force.sum(0).abs().max()) <= 1e-15
    # momentum conservation without drag/tool/supports
    sim = tdem.IceDEM(tdem.DEMConfig(**cfg))
    sim.positions += torch.tensor([0.0, -10.0], device=sim.device, dtype=torch.float64)
    sim.velocities[:] = torch.tensor([0.1, 0.05], device=sim.device, dtype=torch.float64)
    p0 = sim.velocities.sum(0).clone()
    for _ in range(50):
        sim.step()
    torch.testing.assert_close(sim.velocities.sum(0), p0)
    # fixed edges stay exactly put under the tool
    sim = tdem.IceDEM(tdem.DEMConfig(nx=5, ny=3, drag=0))
    sim.time = 0.02
    force, reaction = sim.forces()
    assert float(reaction[1]) > 0
    torch.testing.assert_close(force.sum(0), -reaction)
    sim.run(100)
    assert torch.equal(sim.positions[sim.fixed], sim.initial_positions[sim.fixed])
    assert not bool(sim.velocities[sim.fixed].any())


def test_validation_and_errors(tdem):
    with pytest.raises(ValueError):
        tdem.IceDEM(tdem.DEMConfig(dt=1.0))
    with pytest.raises(ValueError):
        tdem.IceDEM(tdem.DEMConfig(device="cpu"))
    sim = tdem.IceDEM(tdem.DEMConfig(nx=3, ny=2))
    with pytest.raises(TypeError):
        sim.step([[0.0, 0.0]] * 6)
    with pytest.raises(ValueError):
        sim.step(torch.zeros(5, 2, dtype=torch.float64, device="cuda"))
    bad = torch.zeros(6, 2, dtype=torch.float64, device="cuda")
    bad[0, 0] = math.nan
    with pytest.raises(ValueError):
        sim.step(bad)
    with pytest.raises(ValueError):
        sim.step(load_time=1.0)


def test_nonfinite_state_raises_floating_point_error(tdem):
    sim = tdem.IceDEM(tdem.DEMConfig(nx=3, ny=2, fix_edges=False))
    sim.velocities[0, 0] = math.inf
    with pytest.raises(FloatingPointError):
        sim.step()
    assert sim.step_count == 1


def test_snapshot_round_trip(tdem):
    sim = tdem.IceDEM(tdem.DEMConfig(nx=7, ny=3, breaking_strain=0.008, shear_breaking_strain=0.02,
                                     tool_speed=0.2))
    sim.run(120)
    state = sim.snapshot()
    other = tdem.IceDEM.from_snapshot(state)
    for _ in range(40):
        sim.step()
        other.step()
    assert torch.equal(sim.positions, other.positions)
    assert torch.equal(sim.alive, other.alive)
    assert sim.accounting_vector() == other.accounting_vector()
    assert other.exchange_state()["schema"] == "tensordem.exchange/1"


def test_fragments_partition_the_surviving_bond_graph():
    """fragments() (dem.py:462-484 output): components of the surviving bonds,
    isolated discs included, ordered by their smallest particle id."""
    import tensordem_gb300 as tdem
    sim = tdem.IceDEM(tdem.DEMConfig(nx=21, ny=5, breaking_strain=0.01, shear_breaking_strain=0.02))
    sim.run(2000)
    frags = sim.fragments()
    n = len(sim.positions)
    seen = sorted(i for f in frags for i in f["particle_ids"])
    assert seen == list(range(n))
    assert [f["particle_ids"][0] for f in frags] == sorted(f["particle_ids"][0] for f in frags)
    label = np.empty(n, dtype=int)
    for k, f in enumerate(frags):
        label[f["particle_ids"]] = k
        assert abs(f["mass_kg"] - len(f["particle_ids"]) * sim.config.mass) < 1e-12
    pairs = sim.pairs[sim.alive].cpu().numpy()
    assert (label[pairs[:, 0]] == label[pairs[:, 1]]).all()  # no surviving bond crosses fragments
    assert len(frags) > 1


def test_per_bond_stiffness_parity(tdem):
    """CalibratedIceDEM on the GPU against the reference's calibrated run."""
    from tensordem_gb300.calibrated import CalibratedIceDEM
    g = P.load("calibrated_21x5")
    sim = CalibratedIceDEM(tdem.DEMConfig(**P.config_dict(g)), bond_stiffness=g["bond_stiffness"])
    worst = P.replay(g, sim, to_np=_np)
    me = sim.mechanical_energy()
    got = [me[k] for k in ("kinetic_J", "bond_J", "pair_contact_J", "tool_contact_J", "mechanical_J")]
    assert P.normwise(got, g["final_mech"]) <= P.RTOL
    print("calibrated worst normwise errors", worst)


def test_per_bond_stiffness_validation_and_restart(tdem):
    from tensordem_gb300.calibrated import CalibratedIceDEM
    cfg = tdem.DEMConfig(nx=7, ny=3, tool_speed=0.2, breaking_strain=0.008, shear_breaking_strain=0.02)
    nb = int(tdem.IceDEM(cfg).bonded.sum())
    k = np.linspace(0.6, 1.0, nb) * cfg.bond_stiffness
    with pytest.raises(ValueError):
        CalibratedIceDEM(cfg)
    with pytest.raises(ValueError):
        CalibratedIceDEM(cfg, bond_stiffness=k[:-1])
    with pytest.raises(ValueError):
        CalibratedIceDEM(cfg, bond_stiffness=k * 1.5)
    sim = CalibratedIceDEM(cfg, bond_stiffness=k)
    sim.run(40)
    snap = sim.snapshot()
    again = CalibratedIceDEM.from_snapshot(snap)
    sim.run(40)
    again.run(40)
    assert torch.equal(sim.positions, again.positions)
    assert torch.equal(sim.alive, again.alive)
    sim.coefficients[0] *= 0.5  # a mutated host copy no longer matches the kernel's
    with pytest.raises(ValueError):
        sim.step()
