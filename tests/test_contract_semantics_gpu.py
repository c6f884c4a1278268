"""The reference binding contract's behavioural probes
(src/tensordem/binding_contract.py:605-755, ``probe_semantics``) on the CUDA
path of ``IceDEM`` and ``IceDEM3D``, with the same models, loads and bounds:
load guards (shape, type, finiteness, stale stamps), the exact impulse-
momentum identity n dt F of a held load and its non-accumulation, the
external-impulse ledger, the clock, the bitwise restart round trip, forces()
against step() for one load, and the 3-D counterparts."""

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def td():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    import tensordem_gb300
    return tensordem_gb300


def _fresh_2d(td):
    # a free 6x3 strip: no supports, no dashpot, no drag, tool far away
    return td.IceDEM(td.DEMConfig(nx=6, ny=3, fix_edges=False, tool_gap=10.0, contact_damping=0.0, drag=0.0))


def test_load_guards(td):
    m = _fresh_2d(td)
    with pytest.raises(ValueError):
        m.step(external_forces=torch.zeros((m.positions.shape[0] + 1, 2), dtype=torch.float64))
    with pytest.raises(TypeError):
        m.step(external_forces=[[0.0, 0.0]] * len(m.positions))
    nan = torch.zeros_like(m.positions)
    nan[0, 0] = float("nan")
    with pytest.raises(ValueError):
        m.step(external_forces=nan)
    m = _fresh_2d(td)
    with pytest.raises(ValueError):
        m.step(external_forces=torch.zeros_like(m.positions), load_time=m.time + 1e-6)


@pytest.mark.parametrize("n_steps", [1, 4, 16, 64])
def test_impulse_momentum_identity_and_no_accumulation(td, n_steps):
    m = _fresh_2d(td)
    load = torch.zeros_like(m.positions)
    load[:, 0] = 0.25
    load[:, 1] = -0.1
    v0 = m.velocities.clone()
    for _ in range(n_steps):
        m.step(external_forces=load, load_time=m.time)
    dp = m.config.mass * (m.velocities - v0).sum(dim=0)
    ref = n_steps * m.dt * load.sum(dim=0)
    err = float((dp - ref).abs().max() / ref.abs().max())
    assert err < 1e-12, err
    assert abs(float((dp / ref).mean()) - 1.0) < 1e-12


def test_external_impulse_ledger_cross_path(td):
    m = _fresh_2d(td)
    load = torch.zeros_like(m.positions)
    load[:, 1] = 0.3
    for _ in range(8):
        m.step(external_forces=load, load_time=m.time)
    ledger = m.accounting["external_impulse_Ns"]
    ref = (8 * m.dt * load.sum(dim=0)).tolist()
    assert max(abs(a - b) / max(abs(b), 1e-300) for a, b in zip(ledger, ref)) < 1e-12


def test_clock_advances_by_native_dt(td):
    m = _fresh_2d(td)
    zero = torch.zeros_like(m.positions)
    for _ in range(5):
        m.step(external_forces=zero, load_time=m.time)
    assert abs(m.time - 5 * m.dt) / (5 * m.dt) < 1e-12
    assert m.step_count == 5


def test_restart_round_trip_is_bitwise(td):
    m = _fresh_2d(td)
    load = torch.zeros_like(m.positions)
    load[:, 1] = 0.3
    for _ in range(3):
        m.step(external_forces=load, load_time=m.time)
    snap = m.snapshot()
    clone = td.IceDEM.from_snapshot(snap)
    assert snap["schema"] == "tensordem.restart/1"
    assert torch.equal(clone.positions, m.positions) and torch.equal(clone.velocities, m.velocities)
    assert clone.time == m.time and clone.step_count == m.step_count


def test_forces_matches_step_load(td):
    a, b = _fresh_2d(td), _fresh_2d(td)
    load = torch.zeros_like(a.positions)
    load[:, 1] = 0.3
    fa, _ = a.forces(external_forces=load)
    b.step(external_forces=load, load_time=b.time)
    assert tuple(fa.shape) == tuple(b.positions.shape)
    # one semi-implicit step from rest: v = dt F / m for every free disc
    torch.testing.assert_close(b.velocities, b.dt * fa / b.config.mass, rtol=1e-12, atol=0.0)


def test_3d_impulse_momentum_identity_and_load_guard(td):
    m = td.IceDEM3D(td.DEM3DConfig(nx=4, ny=4, nz=4, fix_bottom=False, fix_x_edges=False, contact_damping=0.0,
                                   drag=0.0, tool_gap=10.0))
    load = torch.zeros_like(m.positions)
    load[:, 2] = -0.2
    v0 = m.velocities.clone()
    for _ in range(8):
        m.step(external_forces=load)
    dp = m.config.mass * (m.velocities - v0).sum(dim=0)
    ref = 8 * m.dt * load.sum(dim=0)
    assert float((dp - ref).abs().max() / ref.abs().max()) < 1e-12
    assert abs(float((dp @ ref) / (ref @ ref)) - 1.0) < 1e-12
    with pytest.raises(ValueError):
        m.step(external_forces=torch.zeros((len(m.positions), 2), dtype=torch.float64, device=m.positions.device))
