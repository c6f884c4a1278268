"""Known answers of the bonded oracle (oracle/hm2d.py, BondedHM2DOracle).

Restated on the hexagonal sheet from the reference's own bond tests
(tests/test_dem.py:21-76): equilibrium, action-reaction, objectivity of the
shear measure under rigid rotation, irreversible tensile and shear breakage;
and on a single bonded pair the oscillator and dashpot ledger checks of
tests/test_dem2d_energy_ledger.py.
"""

import math

import numpy as np
import pytest

from tests._hm_cases import bonded_oracle_for, small_sheet


def _free_sheet(**kw):
    cfg, st, bonds, strength = small_sheet(8, 4, **kw)
    st = dict(st)
    st["mass"] = np.where(np.isfinite(st["mass"]), st["mass"], st["mass"][np.isfinite(st["mass"])][0])
    st["inertia"] = 0.5 * st["mass"] * st["radius"] ** 2
    cfg = type(cfg)(**{**cfg.__dict__, "indenter_radius": 0.0})
    return cfg, st, bonds, strength


def test_equilibrium_and_action_reaction():
    cfg, st, bonds, strength = _free_sheet()
    o = bonded_oracle_for(cfg, st, bonds, strength)
    f, tq, _ = o.evaluate(o.pos, o.vel, o.omega, advance=False)
    assert np.abs(f).max() <= 1e-6 and np.abs(tq).max() <= 1e-9
    pos = o.pos.copy()
    pos[5, 0] += 1e-4
    f, _, _ = o.evaluate(pos, o.vel, o.omega, advance=False)
    assert np.abs(f.sum(0)).max() <= 1e-9 * np.abs(f).max()
    assert np.abs(f).max() > 1.0


def test_rigid_rotation_has_no_strain_and_breaks_nothing():
    cfg, st, bonds, strength = _free_sheet()
    o = bonded_oracle_for(cfg, st, bonds, strength)
    a = 0.6
    rot = np.array([[math.cos(a), -math.sin(a)], [math.sin(a), math.cos(a)]])
    c = o.pos.mean(0)
    pos = (o.pos - c) @ rot.T + c + np.array([0.3, -0.2])
    assert np.abs(o.strains(pos)).max() <= 1e-9
    o.evaluate(pos, o.vel, o.omega, advance=True)
    assert o.alive.all()


def test_tension_breaks_irreversibly_compression_does_not():
    cfg, st, bonds, strength = _free_sheet()
    o = bonded_oracle_for(cfg, st, bonds, strength)
    c = o.pos.mean(0)
    o.evaluate(c + (o.pos - c) * 0.995, o.vel, o.omega, advance=True)
    assert o.alive.all()
    o.evaluate(c + (o.pos - c) * 1.05, o.vel, o.omega, advance=True)
    assert not o.alive.any()
    assert np.all(o.fail_mode & 1)
    o.evaluate(o.pos, o.vel, o.omega, advance=True)
    assert not o.alive.any()  # irreversible


def test_objective_shear_breaks_bonds():
    cfg, st, bonds, strength = _free_sheet(breaking_strain=0.5)
    o = bonded_oracle_for(cfg, st, bonds, strength)
    pos = o.pos.copy()
    pos[:, 0] += 0.08 * (pos[:, 1] - pos[:, 1].mean())
    o.evaluate(pos, o.vel, o.omega, advance=True)
    assert (~o.alive).any()
    assert np.all(o.fail_mode[~o.alive] == 2)


def test_indented_sheet_energy_budget_closes_to_integration_error():
    """Kinetic + elastic + dissipated + fracture (net of acquired contact
    energy) - indenter work stays constant up to the velocity-Verlet error of
    this coarse step (a 20 m/s indenter): bound 3% of the work input."""
    cfg, st, bonds, strength = small_sheet(24, 8, steps=600, speed=20.0)
    o = bonded_oracle_for(cfg, st, bonds, strength)
    e0 = o.energies()["total"]
    o.step(300)
    led = o.energies()
    assert o.tool_work > 0.0 and (~o.alive).sum() > 50
    assert abs(led["total"] - e0) <= 0.03 * o.tool_work


def _bonded_pair(zeta, stretch=0.002):
    """Two free discs (r 0.05 m, 7 kg) joined by one bond at rest length 2 r,
    then stretched by ``stretch`` of it; no gravity, no contact."""
    from oracle.hm2d import BondedHM2DOracle, HMParams
    r, m, kn, ks = 0.05, 7.0, 5e8, 2e8
    period = 2.0 * math.pi * math.sqrt(0.5 * m / kn)
    p = HMParams(young=5e9, poisson=0.3, restitution=0.5, mu=0.3, mu_wall=0.0, dt=period / 200.0,
                 gravity=(0.0, 0.0), box=None, skin=0.01)
    o = BondedHM2DOracle(np.array([[0.0, 0.0], [2.0 * r, 0.0]]), np.zeros((2, 2)), np.zeros(2), np.full(2, r),
                         np.full(2, m), np.full(2, 0.5 * m * r * r), p, bonds=[(0, 1)], strength=[1.0],
                         k_n=kn, k_s=ks, zeta=zeta, eps_t=0.01, eps_s=0.02)
    o.pos[1, 0] += stretch * 2.0 * r
    return o, period


def test_undamped_bond_oscillates_at_its_natural_period_and_keeps_its_energy():
    """The reference's bonded-oscillator ledger check (tests/test_dem2d_energy_ledger.py):
    an undamped bond pair oscillates at 2 pi sqrt(m*/k) and velocity-Verlet
    keeps kinetic + bond energy within its O((omega dt)^2) band, back to
    rounding after whole periods; momentum stays zero."""
    o, period = _bonded_pair(zeta=0.0)
    e0 = o.energies()["total"]
    gap, energy = [], []
    for _ in range(1000):  # five periods
        o.step(1)
        gap.append(o.pos[1, 0] - o.pos[0, 0] - 0.1)
        energy.append(o.energies()["total"])
    gap = np.asarray(gap)
    down = np.flatnonzero((gap[:-1] > 0) & (gap[1:] <= 0))
    assert np.diff(down).mean() * o.p.dt == pytest.approx(period, rel=1e-3)
    omega_dt = 2.0 * math.pi / 200.0
    assert np.abs(np.asarray(energy) - e0).max() <= 0.25 * omega_dt**2 * e0
    assert abs(energy[-1] - e0) <= 1e-8 * e0
    assert np.abs(o.vel.sum(axis=0)).max() <= 1e-12 and o.alive.all()


def test_damped_bond_ledger_closes_on_its_dissipation():
    """With the bond dashpot on, the stored energy decays and the dissipated
    energy books the difference: after five periods 96% of the energy is
    dissipated and the ledger total is at its start within 1e-6 (measured
    3.9e-8)."""
    o, _ = _bonded_pair(zeta=0.05)
    e0 = o.energies()
    o.step(1000)
    e1 = o.energies()
    assert e1["bond_elastic"] + e1["kinetic"] < 0.3 * e0["bond_elastic"]
    assert e1["dissipated"] > 0.6 * e0["bond_elastic"]
    assert abs(e1["total"] - e0["total"]) <= 1e-6 * e0["total"]
