"""The reference's 2-D ledger known-answer cases (tests/_ledger_cases.py) on
the numpy oracle: the oracle itself is pinned to the reference's own
closed-form ledger checks before it checks the CUDA path."""

import numpy as np
import pytest

from oracle.icedem import IceDEMOracle, OracleConfig
from tests import _ledger_cases as lc

B = lc.Backend("oracle", make=lambda **kw: IceDEMOracle(OracleConfig(**kw)), arr=np.asarray,
               put=lambda sim, x: np.array(x, copy=True))


@pytest.fixture(scope="module")
def indentation():
    return lc.indentation(B)


def test_integral_momentum_balance_closes_to_roundoff():
    lc.check_uniform_load_momentum(B)


def test_momentum_balance_covers_drag_tool_and_support_channels():
    lc.check_drag_tool_support_momentum(B)


def test_broken_overlapping_bond_retains_pair_contact_energy(indentation):
    lc.check_retained_contact_energy(B, indentation)


def test_energy_ledger_closes_with_retained_contact_term(indentation):
    lc.check_energy_closure(indentation)


@pytest.fixture(scope="module")
def indentation_half():
    return lc.indentation(B, dt_scale=0.5)


def test_energy_residual_is_bookkeeping_not_timestep_error(indentation, indentation_half):
    lc.check_residual_is_bookkeeping(indentation, indentation_half)


def test_drag_decay_matches_closed_form():
    lc.check_drag_decay(lc.drag_decay(B), lc.drag_decay(B, dt_scale=0.5))


def test_bonded_oscillator_ledger_and_integrator():
    lc.check_oscillator(lc.bonded_oscillator(B), lc.bonded_oscillator(B, dt_scale=0.5))


def test_tool_work_residual_shrinks_with_dt(indentation, indentation_half):
    lc.check_tool_channel(indentation, indentation_half)


def test_balance_gate_rejects_single_channel_faults(indentation):
    lc.check_balance_gate_and_negative_controls(indentation)


def test_controlled_break_matches_closed_form():
    lc.check_controlled_break(B)


def test_channel_scales_as_k_xi_squared():
    lc.check_scaling(B)


def test_indentation_events_match_closed_forms():
    lc.check_indentation_events(B)


def test_subthreshold_negative_control():
    lc.check_subthreshold(B)
