"""The reference's 2-D ledger known-answer checks on the CUDA path of
``tensordem_gb300.IceDEM``: its tests/test_accounting_ledger_validation.py
(momentum balance of the impulse channels, retained pair-contact energy,
energy closure, old checkpoints) and tests/test_dem2d_fracture_ledger.py
(controlled break, k xi^2 scaling, per-event closed forms, sub-threshold
control), with the reference's inputs and bounds (cases in
tests/_ledger_cases.py, run on the oracle by tests/test_oracle_ledger.py)."""

import math

import numpy as np
import pytest
import torch

from tests import _ledger_cases as lc

pytestmark = pytest.mark.gpu


def _arr(x):
    return x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)


@pytest.fixture(scope="module")
def b():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300 import DEMConfig, IceDEM
    return lc.Backend("cuda", make=lambda **kw: IceDEM(DEMConfig(**kw)), arr=_arr,
                      put=lambda sim, x: torch.as_tensor(np.array(x), device=sim.device))


@pytest.fixture(scope="module")
def indentation(b):
    return lc.indentation(b)


def test_integral_momentum_balance_closes_to_roundoff(b):
    lc.check_uniform_load_momentum(b)


def test_momentum_balance_covers_drag_tool_and_support_channels(b):
    lc.check_drag_tool_support_momentum(b)


def test_broken_overlapping_bond_retains_pair_contact_energy(b, indentation):
    lc.check_retained_contact_energy(b, indentation)


def test_energy_ledger_closes_with_retained_contact_term(indentation):
    lc.check_energy_closure(indentation)


@pytest.fixture(scope="module")
def indentation_half(b):
    return lc.indentation(b, dt_scale=0.5)


def test_energy_residual_is_bookkeeping_not_timestep_error(indentation, indentation_half):
    lc.check_residual_is_bookkeeping(indentation, indentation_half)


def test_drag_decay_matches_closed_form(b):
    lc.check_drag_decay(lc.drag_decay(b), lc.drag_decay(b, dt_scale=0.5))


def test_bonded_oscillator_ledger_and_integrator(b):
    lc.check_oscillator(lc.bonded_oscillator(b), lc.bonded_oscillator(b, dt_scale=0.5))


def test_tool_work_residual_shrinks_with_dt(indentation, indentation_half):
    lc.check_tool_channel(indentation, indentation_half)


def test_balance_gate_rejects_single_channel_faults(indentation):
    lc.check_balance_gate_and_negative_controls(indentation)


def test_restart_accepts_checkpoint_without_new_ledger_channel():
    from tensordem_gb300 import DEMConfig, IceDEM
    sim = IceDEM(DEMConfig(nx=5, ny=3, tool_speed=0.2))
    for _ in range(5):
        sim.step()
    state = sim.snapshot()
    del state["accounting"]["pair_contact_acquired_J"]
    restored = IceDEM.from_snapshot(state)
    assert restored.accounting["pair_contact_acquired_J"] == 0.0
    assert math.isfinite(restored.accounting["fracture_release_J"])


def test_controlled_break_matches_closed_form(b):
    lc.check_controlled_break(b)


def test_channel_scales_as_k_xi_squared(b):
    lc.check_scaling(b)


def test_indentation_events_match_closed_forms(b):
    lc.check_indentation_events(b)


def test_subthreshold_negative_control(b):
    lc.check_subthreshold(b)


def test_ledger_channels_equal_the_oracle(b, indentation):
    """The whole indentation's ledger, break table and state against the
    oracle run on the same inputs (both follow the reference's arithmetic)."""
    from oracle.icedem import IceDEMOracle, OracleConfig
    ob = lc.Backend("oracle", make=lambda **kw: IceDEMOracle(OracleConfig(**kw)), arr=np.asarray,
                    put=lambda sim, x: np.array(x, copy=True))
    ref = lc.indentation(ob)
    g, o = indentation["sim"], ref["sim"]
    assert indentation["steps"] == ref["steps"]
    for key in ("external_work_J", "fracture_release_J", "pair_contact_acquired_J", "tool_work_J",
                "damping_dissipation_J"):
        assert abs(indentation["accounting"][key] - ref["accounting"][key]) <= 1e-12 * max(
            1.0, abs(ref["accounting"][key])), key
    for key in lc.IMPULSE_KEYS:
        np.testing.assert_allclose(indentation["accounting"][key], ref["accounting"][key], rtol=1e-12, atol=1e-15)
    assert np.array_equal(_arr(g.failure_mode), o.failure_mode)
    np.testing.assert_allclose(_arr(g.positions), o.positions, rtol=0, atol=1e-12)
