"""GPU parity of the 3-D reference-mode CUDA step against the reference's outputs.

Golden vectors: tests/golden/dem3d_*.npz (made by the reference IceDEM3D,
src/tensordem/dem3d.py, via tests/golden/make_golden3d.py). Tolerances (in
tests/_icedem3d_parity.py): bond states and break ledger bit-exact; frames,
forces, reactions, diagnostics and energies within 1e-12 normwise.
"""

import math

import numpy as np
import pytest
import torch

from tests import _icedem3d_parity as P

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


@pytest.fixture(scope="module")
def m3():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300 import dem3d
    return dem3d


def _sim(m3, g):
    sim = m3.IceDEM3D(m3.DEM3DConfig(**{**P.config_dict(g), "device": "cuda"}))
    sim.lateral_platen_velocity = torch.tensor(g["lateral_velocity"], dtype=torch.float64, device="cuda")
    return sim


class _Loaded:
    """Golden loads arrive as numpy arrays: hand them over as CUDA tensors."""

    def __init__(self, sim):
        object.__setattr__(self, "sim", sim)

    def __getattr__(self, name):
        return getattr(self.sim, name)

    def __setattr__(self, name, value):
        setattr(self.sim, name, value)

    def step(self, loads=None):
        self.sim.step(None if loads is None else torch.as_tensor(loads, device="cuda"))


def _cuda(a):
    return torch.as_tensor(np.asarray(a), device="cuda").clone()


@pytest.mark.parametrize("mapping", ["lanes", "particle"])
@pytest.mark.parametrize("name", P.FREE_RUN)
def test_golden_trajectory(m3, name, mapping):
    g = P.load(name)
    sim = _sim(m3, g)
    sim.set_thread_mapping(mapping)
    assert sim.dt == float(g["dt"])
    assert np.array_equal(_np(sim.pairs), g["pairs"])
    assert np.array_equal(_np(sim.initial_positions), g["initial_positions"])
    worst = P.replay(g, _Loaded(sim), to_np=_np)
    print(name, "worst normwise errors", worst, "broken", sim.broken_bonds)


@pytest.mark.parametrize("mapping", ["lanes", "particle"])
@pytest.mark.parametrize("name", P.CASES)
def test_golden_one_step(m3, name, mapping):
    g = P.load(name)
    sim = _sim(m3, g)
    sim.set_thread_mapping(mapping)
    worst = P.replay_one_step(g, _Loaded(sim), to_np=_np, to_device=_cuda)
    print(name, "one-step worst normwise errors", worst)


@pytest.mark.parametrize("name", [c for c in P.CASES if c not in P.FREE_RUN])
def test_free_run_statistics(m3, name):
    """The free-running Hertz cases end in the reference's regime."""
    g = P.load(name)
    sim = _sim(m3, g)
    sim.run(int(g["steps"]))
    want = int((g["failure_mode"] > 0).sum())
    assert abs(sim.broken_bonds - want) <= 0.05 * want
    agree = np.mean(_np(sim.alive) == g["frame_alive"][-1])
    assert agree >= 0.9


@pytest.mark.parametrize("case", ["jitter", "coincident", "stretch", "squeeze", "tool_centre"])
def test_unit_probes(m3, case):
    g = P.load("dem3d_unit")
    sim = m3.IceDEM3D(m3.DEM3DConfig(**{**P.config_dict(g), "device": "cuda"}))
    sim.positions = torch.tensor(g[f"{case}_pos"], device="cuda")
    sim.velocities = torch.tensor(g[f"{case}_vel"], device="cuda")
    f, r = sim.forces(update_fracture=False, update_history=False)
    scale = max(1.0, np.abs(g[f"{case}_force_probe"]).max())
    assert np.abs(_np(f) - g[f"{case}_force_probe"]).max() <= 1e-12 * scale
    assert np.abs(_np(r) - g[f"{case}_reaction_probe"]).max() <= 1e-12 * scale
    f2, r2 = sim.forces()
    scale = max(1.0, np.abs(g[f"{case}_force"]).max())
    assert np.abs(_np(f2) - g[f"{case}_force"]).max() <= 1e-12 * scale
    assert np.abs(_np(r2) - g[f"{case}_reaction"]).max() <= 1e-12 * scale
    assert np.array_equal(_np(sim.alive), g[f"{case}_alive"])
    for key in ("friction_power", "rolling_power"):
        want = float(g[f"{case}_{key}"])
        got = getattr(sim, f"_last_{key}")
        assert abs(got - want) <= 1e-12 * max(1.0, abs(want))


def test_contact_pairs_match_brute_force(m3):
    """tests/test_dem3d.py:83-98: the cell list finds every overlapping pair once."""
    g = P.load("dem3d_hertz_friction")
    sim = _sim(m3, g)
    sim.run(700)
    sim.forces(update_fracture=False, update_history=False)
    got = {tuple(p) for p in sim.contact_pairs().tolist()}
    x = _np(sim.positions)
    d = np.linalg.norm(x[None, :, :] - x[:, None, :], axis=2)
    i, j = np.nonzero(np.triu(d < 2 * sim.config.radius, 1))
    assert got == set(zip(i.tolist(), j.tolist()))
    assert len(got) > 10


def test_run_block_matches_single_steps(m3):
    g = P.load("dem3d_cylinder")
    a, b = _sim(m3, g), _sim(m3, g)
    for _ in range(300):
        a.step()
    b.run(300)
    for name in ("positions", "velocities", "alive", "branch_offsets", "bond_damage", "lateral_platen_pos"):
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    assert a.time == b.time and a.step_count == b.step_count


def test_reproducible_and_restart(m3):
    """tests/test_dem3d.py:143-159: a checkpoint resumes identically."""
    g = P.load("dem3d_box")
    first = _sim(m3, g)
    first.run(900)
    snap = first.state_dict()
    first.run(200)
    resumed = _sim(m3, g)
    resumed.load_state_dict(snap)
    resumed.run(200)
    assert torch.equal(resumed.positions, first.positions)
    assert torch.equal(resumed.alive, first.alive)
    assert resumed.time == first.time and resumed.step_count == first.step_count
    bad = dict(snap)
    bad["alive"] = snap["alive"].to(torch.uint8)
    with pytest.raises(ValueError):
        resumed.load_state_dict(bad)


def test_validation_and_errors(m3):
    with pytest.raises(ValueError):
        m3.IceDEM3D(m3.DEM3DConfig(dt=1.0))
    with pytest.raises(ValueError):
        m3.DEM3DConfig(device="cpu")
    with pytest.raises(ValueError):
        m3.DEM3DConfig(contact_damping_model="restitution_calibrated", restitution_coefficient=0.5)  # linear
    sim = m3.IceDEM3D(m3.DEM3DConfig(nx=3, ny=3, nz=2, fix_x_edges=False))
    with pytest.raises(ValueError):
        sim.step(torch.zeros(5, 3, dtype=torch.float64, device="cuda"))
    bad = torch.zeros(18, 3, dtype=torch.float64, device="cuda")
    bad[0, 0] = math.nan
    with pytest.raises(ValueError):
        sim.step(bad)
    sim.velocities[0, 0] = math.inf
    with pytest.raises(FloatingPointError):
        sim.step()
    assert sim.step_count == 1
    # a multi-step launch stops after the offending step, as step() does
    other = m3.IceDEM3D(m3.DEM3DConfig(nx=3, ny=3, nz=2, fix_x_edges=False))
    other.run(3)
    other.velocities[0, 0] = math.inf
    with pytest.raises(FloatingPointError):
        other.run(10)
    assert other.step_count == 4


def test_cli_restart_workflow(m3, tmp_path):
    """tests/test_dem3d.py:116-141: history, checkpoint and restart through the CLI."""
    from tensordem_gb300.cli import main
    out = tmp_path / "run"
    main(["dem-3d", "--nx", "3", "--ny", "3", "--nz", "2", "--steps", "2", "--save-every", "1",
          "--output", str(out)])
    ck = out / "checkpoint_3d.pt"
    first = torch.load(ck, map_location="cpu", weights_only=False)
    assert first["format"] == "tensordem-dem3d-checkpoint-v1" and first["state"]["step_count"] == 2
    main(["dem-3d", "--steps", "2", "--save-every", "1", "--output", str(out), "--restart", str(ck)])
    second = torch.load(ck, map_location="cpu", weights_only=False)
    assert second["state"]["step_count"] == 4
    assert abs(second["state"]["time"] - 4 * second["state"]["dt"]) <= 1e-15
    rows = (out / "history.csv").read_text().strip().splitlines()
    assert len(rows) == 1 + 5  # header, steps 0..2, then 3..4 appended
    traj = torch.load(out / "trajectory_3d.pt", map_location="cpu", weights_only=False)
    assert traj["dimension"] == 3 and traj["positions"].shape[1:] == (18, 3)


def test_contact_capacity_overflow_raises(m3):
    """40 particles squeezed into one spot: more than 32 overlapping partners
    per particle is reported as an error, not written past the lists."""
    sim = m3.IceDEM3D(m3.DEM3DConfig(nx=5, ny=4, nz=2, fix_x_edges=False))
    gen = torch.Generator(device="cpu").manual_seed(3)
    sim.positions = ((torch.rand(40, 3, generator=gen, dtype=torch.float64) - 0.5) * 0.002).to("cuda")
    with pytest.raises(RuntimeError):
        sim.forces(update_fracture=False, update_history=False)


def test_bench_sizes_agree_across_mappings(m3):
    """A specimen above the size where the mapping switches: the per-particle
    and the lane mappings step to identical states."""
    cfg = m3.DEM3DConfig(nx=40, ny=20, nz=10, breaking_strain=0.004, shear_breaking_strain=0.008,
                         friction_coefficient=0.3, restitution_coefficient=0.7)
    a, b = m3.IceDEM3D(cfg), m3.IceDEM3D(cfg)
    a.set_thread_mapping("particle")
    b.set_thread_mapping("lanes")
    a.run(1300)
    b.run(1300)
    assert a.broken_bonds > 0
    for name in ("positions", "velocities", "alive", "failure_energy_J"):
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    assert a.friction_history() == b.friction_history()
