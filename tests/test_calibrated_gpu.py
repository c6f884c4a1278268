"""The reference's per-bond-stiffness checks (its tests/test_calibrated_dem.py:11-71)
on the CUDA path of ``CalibratedIceDEM``: the little-endian coefficient digest
in snapshots (restored and stepped without torch's numpy bridge), release of
exactly the stored bond energy when every strained bond breaks, the bond force
as the gradient of the bond energy, bit-identical dynamic restart, the dt bound
and the rejection of corrupted snapshots or mutated coefficients.

The reference builds its per-bond stiffnesses with a material-calibration
helper that is not part of this step; a seeded ramp of stiffnesses below the
config's bound exercises the same properties here."""

import copy
import hashlib
import struct
from unittest.mock import patch

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def td():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    import tensordem_gb300
    return tensordem_gb300


def _make(td, dt=None, threshold=1.0):
    cfg = td.DEMConfig(nx=5, ny=3, radius=0.1, thickness=0.2, bond_stiffness=150000.0, contact_damping=0.0,
                       drag=0.0, fix_edges=False, tool_gap=10.0, breaking_strain=threshold,
                       shear_breaking_strain=1.0, dt=dt)
    nb = int(td.IceDEM(cfg).bonded.sum())
    k = np.linspace(0.55, 0.95, nb) * cfg.bond_stiffness
    return td.CalibratedIceDEM(cfg, bond_stiffness=k)


def test_legacy_digest_restart_without_numpy_bridge(td):
    sim = _make(td)
    values = sim.coefficients.detach().to(device="cpu", dtype=torch.float64).tolist()
    digest = hashlib.sha256(struct.pack(f"<{len(values)}d", *values)).hexdigest()
    state = sim.snapshot()
    assert state["coefficient_sha256"] == digest
    with patch.object(torch.Tensor, "numpy", side_effect=RuntimeError("numpy bridge unavailable")):
        restored = td.CalibratedIceDEM.from_snapshot(state)
        assert restored.coefficient_hash == digest
        restored.step(torch.zeros_like(restored.positions))
        assert restored._hash() == digest


def test_force_balance_and_release_of_the_stored_energy(td):
    sim = _make(td, threshold=0.001)
    sim.positions[:, 0] *= 1.01
    stored = sim.mechanical_energy()["bond_J"]
    forces, _ = sim.forces()
    assert float(forces.sum(0).abs().max()) < 1e-10
    assert abs(sim.accounting["fracture_release_J"] - stored) < 5e-11
    sim.forces()
    assert abs(sim.accounting["fracture_release_J"] - stored) < 5e-11


def test_bond_force_is_the_energy_gradient(td):
    sim = _make(td)
    sim.positions[6, 0] += 1e-4
    force, _ = sim.forces()
    eps = 1e-8
    sim.positions[6, 0] += eps
    plus = sim.mechanical_energy()["bond_J"]
    sim.positions[6, 0] -= 2 * eps
    minus = sim.mechanical_energy()["bond_J"]
    assert abs(float(force[6, 0]) + (plus - minus) / (2 * eps)) < 5e-6


def test_dynamic_restart_bound_and_corruption(td):
    sim = _make(td)
    load = torch.zeros_like(sim.positions)
    load[:, 0] = 0.01
    for _ in range(5):
        sim.step(load, load_time=sim.time)
    restored = td.CalibratedIceDEM.from_snapshot(sim.snapshot())
    for _ in range(5):
        sim.step(load)
        restored.step(load)
    assert sim.snapshot() == restored.snapshot()
    assert sim.dt <= sim.config.recommended_dt
    bad = copy.deepcopy(sim.snapshot())
    bad["bond_stiffness_N_per_m"][0] = float("nan")
    with pytest.raises(ValueError):
        td.CalibratedIceDEM.from_snapshot(bad)
    bad = copy.deepcopy(sim.snapshot())
    bad["bond_stiffness_N_per_m"][0] *= 0.5
    with pytest.raises(ValueError):
        td.CalibratedIceDEM.from_snapshot(bad)
    sim.coefficients[0] *= 0.5
    with pytest.raises(ValueError):
        sim.step(load)
