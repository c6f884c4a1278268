"""The reference's accounting-output checks (its tests/test_accounting_output.py:14-140)
on the CUDA path: the flattened accounting fields of ``IceDEM.diagnostics()``
and the ``accounting.json`` the ``dem-2d`` CLI writes (with and without a hull
profile): required channels, extra fields, types, finiteness, and the fracture
release equal to the sum of the per-bond failure energies."""

import json
import math

import pytest
import torch

pytestmark = pytest.mark.gpu

ACCOUNTING = ("external_work_J", "fracture_release_J", "tool_work_J", "damping_dissipation_J",
              "external_impulse_Ns", "support_impulse_Ns", "drag_impulse_Ns", "tool_impulse_on_ice_Ns")
EXTRA = ("total_bonds", "broken_bonds", "failure_energy_sum_J", "total_mass_kg", "dt", "steps")


@pytest.fixture(scope="module")
def td():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    import tensordem_gb300
    return tensordem_gb300


def test_diagnostics_accounting_fields(td):
    sim = td.IceDEM(td.DEMConfig(nx=5, ny=3, tool_speed=0.2))
    for _ in range(10):
        sim.step()
    diag = sim.diagnostics()
    for field in ("tool_impulse_on_ice_x_Ns", "tool_impulse_on_ice_y_Ns", "support_impulse_x_Ns",
                  "support_impulse_y_Ns", "drag_impulse_x_Ns", "drag_impulse_y_Ns", "external_impulse_x_Ns",
                  "external_impulse_y_Ns", "fracture_release_J", "tool_work_J", "damping_dissipation_J",
                  "external_work_J"):
        assert field in diag and math.isfinite(diag[field]), field
    for field in ("time", "tool_x", "tool_y", "reaction_x", "reaction_y", "boundary_reaction_x",
                  "boundary_reaction_y", "broken_bonds", "kinetic_energy"):
        assert field in diag, field


def _check_accounting(acc: dict) -> None:
    for field in ACCOUNTING + EXTRA:
        assert field in acc, field
    for key, value in acc.items():
        values = value if isinstance(value, list) else [value]
        for v in values:
            if isinstance(v, (int, float)):
                assert math.isfinite(v), key
    assert isinstance(acc["total_bonds"], int) and isinstance(acc["broken_bonds"], int)
    assert isinstance(acc["steps"], int)
    for key in ("failure_energy_sum_J", "total_mass_kg", "dt"):
        assert isinstance(acc[key], float), key
    assert acc["fracture_release_J"] >= 0.0
    assert abs(acc["failure_energy_sum_J"] - acc["fracture_release_J"]) <= 1e-10


def test_accounting_json_output(td, tmp_path):
    from tensordem_gb300.cli import main
    out = tmp_path / "run"
    main(["dem-2d", "--nx", "5", "--ny", "3", "--steps", "10", "--output", str(out)])
    acc = json.loads((out / "accounting.json").read_text())
    _check_accounting(acc)
    assert acc["steps"] == 10 and acc["total_bonds"] > 0


def test_accounting_json_with_hull_profile(td, tmp_path):
    from tensordem_gb300.cli import main
    hull = tmp_path / "hull.csv"
    hull.write_text("x,y\n0.0,0.0\n0.1,0.0\n0.1,0.1\n")
    out = tmp_path / "hull-run"
    main(["dem-2d", "--nx", "5", "--ny", "3", "--steps", "10", "--hull-profile", str(hull),
          "--hull-velocity-x", "0.2", "--output", str(out)])
    _check_accounting(json.loads((out / "accounting.json").read_text()))
