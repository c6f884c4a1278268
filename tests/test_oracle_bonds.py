"""Known answers of the bonded oracle (oracle/hm2d.py, BondedHM2DOracle).

Restated on the hexagonal sheet from the reference's own bond tests
(tests/test_dem.py:21-76): equilibrium, action-reaction, objectivity of the
shear measure under rigid rotation, irreversible tensile and shear breakage.
"""

import math

import numpy as np

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
