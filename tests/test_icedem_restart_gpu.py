"""The reference's restart and load-coupling checks (its tests/test_coupling_restart.py:9-224)
on the CUDA path of ``IceDEM``: bitwise restart through a JSON checkpoint that
fails closed on corrupt fields, the external work / moment / impulse of one
loaded step, support impulse and fracture release without double counting,
first-order convergence of a uniform translation, and the restart boundary
matrix: every leaf of the checkpoint compared exactly at the interruption
point and after further steps (with supports, at the first failure, with the
hull in contact)."""

import copy
import json
import math

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def td():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    import tensordem_gb300
    return tensordem_gb300


def _diffs(ref, act, path="state"):
    """Every leaf that differs between two restart records (types included)."""
    out = []
    if type(ref) is not type(act):
        out.append(f"{path}: type {type(ref).__name__} != {type(act).__name__}")
    elif isinstance(ref, dict):
        if set(ref) != set(act):
            out.append(f"{path}: field set differs by {sorted(set(ref) ^ set(act))}")
        for key in sorted(set(ref) & set(act)):
            out.extend(_diffs(ref[key], act[key], f"{path}.{key}"))
    elif isinstance(ref, list):
        if len(ref) != len(act):
            out.append(f"{path}: length {len(ref)} != {len(act)}")
        for k, (a, b) in enumerate(zip(ref, act)):
            out.extend(_diffs(a, b, f"{path}[{k}]"))
    elif ref != act:
        out.append(f"{path}: {ref!r} != {act!r}")
    return out


def _same(ref, act, context):
    d = _diffs(ref, act)
    assert not d, f"{context}: {len(d)} field(s) disagree; " + "; ".join(d[:4])


def _json(snapshot):
    return json.loads(json.dumps(snapshot, allow_nan=False))


def _loads(sim, step):
    """Step-dependent nodal loads, so no branch is free of load history."""
    pattern = torch.linspace(-1.0, 1.0, sim.positions.numel(), dtype=torch.float64)
    return (0.5 + 0.1 * step) * pattern.reshape(sim.positions.shape)


def test_restart_is_bitwise_and_fails_closed(td):
    sim = td.IceDEM(td.DEMConfig(nx=3, ny=2, drag=0, fix_edges=False, tool_gap=1))
    load = torch.ones_like(sim.positions)
    for _ in range(12):
        sim.step(load, load_time=sim.time)
    saved = _json(sim.snapshot())
    restarted = td.IceDEM.from_snapshot(saved)
    for _ in range(8):
        sim.step(load)
        restarted.step(load)
    assert sim.snapshot() == restarted.snapshot()
    for key, value in (("schema", "unknown"), ("positions_m", [[0.0, 0.0]]), ("time_s", float("nan"))):
        broken = copy.deepcopy(saved)
        broken[key] = value
        with pytest.raises(ValueError):
            td.IceDEM.from_snapshot(broken)
    with pytest.raises(ValueError):
        sim.step(load, load_time=0)


def test_load_work_moment_and_momentum_impulse(td):
    sim = td.IceDEM(td.DEMConfig(nx=3, ny=2, drag=0, fix_edges=False, tool_gap=1))
    old = sim.positions.detach().cpu().clone()
    loads = torch.arange(12, dtype=torch.float64).reshape(6, 2)
    sim.step(loads)
    new = sim.positions.detach().cpu()
    assert sim.last_step["external_work_J"] == pytest.approx(float((loads * (new - old)).sum()))
    assert sim.last_step["external_moment_Nm"] == pytest.approx(
        float((old[:, 0] * loads[:, 1] - old[:, 1] * loads[:, 0]).sum()))
    torch.testing.assert_close(sim.config.mass * sim.velocities.detach().cpu().sum(0), sim.dt * loads.sum(0))
    assert sum(f["mass_kg"] for f in sim.fragments()) == pytest.approx(6 * sim.config.mass)


def test_support_impulse_and_release_are_not_double_counted(td):
    sim = td.IceDEM(td.DEMConfig(nx=3, ny=2, drag=0))
    loads = torch.ones_like(sim.positions)
    sim.step(loads)
    torch.testing.assert_close(torch.tensor(sim.last_step["support_force_N"], dtype=torch.float64),
                               (-loads[sim.fixed].sum(0)).cpu())
    sim.positions[:, 0] *= 1.2
    sim.forces()
    release = sim.accounting["fracture_release_J"]
    assert release > 0
    sim.forces()
    sim.diagnostics()
    assert sim.accounting["fracture_release_J"] == release


def test_timestep_refinement_of_a_uniform_translation(td):
    cfg = td.DEMConfig(nx=3, ny=2, drag=0, fix_edges=False, tool_gap=1)
    duration = 20 * cfg.recommended_dt
    errors = []
    for divisor in (1, 2, 4):
        sim = td.IceDEM(td.DEMConfig(nx=3, ny=2, drag=0, fix_edges=False, tool_gap=1,
                                     dt=cfg.recommended_dt / divisor))
        loads = torch.zeros_like(sim.positions)
        loads[:, 0] = sim.config.mass  # 1 m/s^2 on every disc
        initial = sim.positions.clone()
        for _ in range(20 * divisor):
            sim.step(loads)
        exact = initial[:, 0] + 0.5 * duration ** 2
        errors.append(float((sim.positions[:, 0] - exact).abs().max()))
        torch.testing.assert_close(sim.velocities[:, 0], torch.full_like(sim.velocities[:, 0], duration),
                                   atol=1e-13, rtol=1e-12)
    assert errors[1] < 0.51 * errors[0]
    assert errors[2] < 0.51 * errors[1]


@pytest.mark.parametrize("interrupt_step", (0, 1, 2, 5, 11, 13))
@pytest.mark.parametrize("fix_edges", (False, True))
def test_restart_boundary_fieldwise_before_and_after_a_step(td, interrupt_step, fix_edges):
    sim = td.IceDEM(td.DEMConfig(nx=3, ny=2, drag=0, fix_edges=fix_edges, tool_gap=1, tool_speed=0.3))
    for step in range(interrupt_step):
        sim.step(_loads(sim, step), load_time=sim.time)
    committed = sim.snapshot()
    _same(committed, _json(committed), f"json round trip at step {interrupt_step}")
    restarted = td.IceDEM.from_snapshot(_json(committed))
    _same(committed, restarted.snapshot(), f"interruption state at step {interrupt_step}")
    assert restarted.time == sim.time and restarted.step_count == interrupt_step
    for offset in (-1, 1):
        with pytest.raises(ValueError):
            restarted.step(_loads(restarted, interrupt_step), load_time=restarted.time + offset * restarted.dt)
    sim.step(_loads(sim, interrupt_step), load_time=sim.time)
    restarted.step(_loads(restarted, interrupt_step), load_time=restarted.time)
    _same(sim.snapshot(), restarted.snapshot(), f"first step after interruption {interrupt_step}")
    for step in range(interrupt_step, interrupt_step + 3):
        sim.step(_loads(sim, step))
        restarted.step(_loads(restarted, step))
        _same(sim.snapshot(), restarted.snapshot(), f"trajectory after interruption {step}")


def test_restart_at_the_first_failure_keeps_the_ledger(td):
    sim = td.IceDEM(td.DEMConfig(nx=3, ny=2, drag=0, tool_gap=1))
    loads = torch.zeros_like(sim.positions)
    loads[:, 0] = 20.0
    for _ in range(100):
        sim.step(loads)
        if bool((sim.failure_mode > 0).any()):
            break
    assert bool((sim.failure_mode > 0).any()) and bool((sim.failure_mode == 0).any())
    assert sim.accounting["fracture_release_J"] > 0
    saved = _json(sim.snapshot())
    restarted = td.IceDEM.from_snapshot(saved)
    _same(saved, restarted.snapshot(), "failure-boundary interruption state")
    for key in ("failure_mode", "failure_time_s", "failure_extension_m", "failure_energy_J", "alive"):
        assert restarted.snapshot()[key] == saved[key], key
    sim.step(loads)
    restarted.step(loads)
    _same(sim.snapshot(), restarted.snapshot(), "first step after the failure boundary")
    assert restarted.accounting["fracture_release_J"] == sim.accounting["fracture_release_J"]
    shifted = copy.deepcopy(saved)
    shifted["step_count"] += 1
    with pytest.raises(ValueError):
        td.IceDEM.from_snapshot(shifted)


def test_restart_with_the_hull_in_contact(td):
    profile = torch.tensor([[0.0, -0.1], [0.0, 0.2]], dtype=torch.float64)
    sim = td.IceDEM(td.DEMConfig(nx=5, ny=3, tool_speed=0.2, fix_edges=False, drag=0.0), hull_profile=profile,
                    hull_start=(0.01, 0.0), hull_velocity=(0.2, 0.0))
    loads = torch.zeros_like(sim.positions)
    loads[:, 0] = 1.0
    for _ in range(6):
        sim.step(loads)
    assert float(sim.last_step["tool_reaction_N"][0]) > 0.0
    saved = _json(sim.snapshot())
    restarted = td.IceDEM.from_snapshot(saved)
    _same(saved, restarted.snapshot(), "hull-contact interruption state")
    assert restarted.snapshot()["hull_profile_m"] == profile.tolist()
    sim.step(loads)
    restarted.step(loads)
    _same(sim.snapshot(), restarted.snapshot(), "first step after the hull-contact interruption")


def test_the_comparator_flags_a_single_leaf_drift(td):
    sim = td.IceDEM(td.DEMConfig(nx=3, ny=2, drag=0, fix_edges=False, tool_gap=1))
    sim.step(_loads(sim, 0))
    good = _json(sim.snapshot())
    assert not _diffs(good, copy.deepcopy(good))

    def bump(v):
        return math.nextafter(v, math.inf)

    mutations = {
        "state.positions_m[0][0]": lambda s: s["positions_m"][0].__setitem__(0, bump(s["positions_m"][0][0])),
        "state.velocities_m_s[1][1]": lambda s: s["velocities_m_s"][1].__setitem__(1, bump(s["velocities_m_s"][1][1])),
        "state.accounting.external_impulse_Ns[0]": lambda s: s["accounting"]["external_impulse_Ns"].__setitem__(
            0, bump(s["accounting"]["external_impulse_Ns"][0])),
        "state.last_step.external_work_J": lambda s: s["last_step"].__setitem__(
            "external_work_J", bump(s["last_step"]["external_work_J"])),
        "state.failure_mode[7]": lambda s: s["failure_mode"].__setitem__(7, 1),
        "state.step_count": lambda s: s.__setitem__("step_count", s["step_count"] + 1),
    }
    for path, mutate in mutations.items():
        broken = copy.deepcopy(good)
        mutate(broken)
        d = _diffs(good, broken)
        assert d and any(x.startswith(path) for x in d), (path, d)
        with pytest.raises(AssertionError, match=r"field\(s\) disagree"):
            _same(good, broken, path)
