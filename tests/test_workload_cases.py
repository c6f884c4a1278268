"""CPU checks that the seeded synthetic workloads are the measured configurations.

The 1,048,576-disc settling case (``granular_gas_case(1024)``): radii
U[0.8, 1.2] mm, density 2500 kg/m^3, E 70 GPa, nu 0.25, mu 0.5, restitution
0.8, jittered square grid at area fraction 0.55 inside four walls, no overlap
at t = 0, velocities Gaussian with sigma 0.1 m/s, gravity -9.81 m/s^2, dt 0.2
Rayleigh time. The 2048 x 512 bonded ice sheet (``ice_sheet_case``): hex
lattice of r = 0.05 m discs, rho 900 kg/m^3, E 5 GPa, six-neighbour bonds
(3,140,609), per-bond strength factor lognormal(0, 0.1), break strains
0.01 / 0.02, both short ends clamped, an indenter of radius 2 m moving down at
0.5 m/s. Both are seeded: the same seed gives the same bytes.
"""

import math

import numpy as np
import pytest

from tensordem_gb300.hm2d import ALL_WALLS, granular_gas_case, ice_sheet_case, rayleigh_dt


@pytest.fixture(scope="module")
def gas():
    return granular_gas_case(1024, seed=0)


@pytest.fixture(scope="module")
def sheet():
    return ice_sheet_case(2048, 512, seed=0)


def test_settling_case_parameters(gas):
    cfg, st = gas
    r = st["radius"]
    assert cfg.n == len(r) == 1024 * 1024
    assert r.min() >= 0.8e-3 and r.max() <= 1.2e-3
    assert r.mean() == pytest.approx(1.0e-3, rel=1e-3)
    mass = 2500.0 * math.pi * r * r * (2.0 * r)
    assert np.allclose(st["mass"], mass, rtol=1e-14)
    assert np.allclose(st["inertia"], 0.5 * mass * r * r, rtol=1e-14)
    assert (cfg.young, cfg.poisson, cfg.mu, cfg.mu_wall, cfg.restitution) == (70e9, 0.25, 0.5, 0.5, 0.8)
    assert cfg.gravity == (0.0, -9.81) and cfg.walls == ALL_WALLS
    assert cfg.dt == pytest.approx(0.2 * rayleigh_dt(float(r.min()), 2500.0, 70e9, 0.25), rel=1e-14)


def test_settling_case_packing(gas):
    cfg, st = gas
    pos, r = st["pos"], st["radius"]
    box = cfg.box
    assert np.all(pos - r[:, None] > 0.0) and np.all(pos[:, 0] + r < box[0]) and np.all(pos[:, 1] + r < box[1])
    assert float(np.sum(math.pi * r * r)) / (box[0] * box[1]) == pytest.approx(0.55, rel=0.01)
    v = st["vel"]
    assert v.mean() == pytest.approx(0.0, abs=1e-3) and v.std() == pytest.approx(0.1, rel=0.01)
    assert np.all(st["omega"] == 0.0)


def test_settling_case_starts_without_overlap(gas):
    spatial = pytest.importorskip("scipy.spatial")
    _, st = gas
    pos, r = st["pos"], st["radius"]
    pairs = spatial.cKDTree(pos).query_pairs(2.0 * float(r.max()), output_type="ndarray")
    d = np.sqrt(((pos[pairs[:, 0]] - pos[pairs[:, 1]]) ** 2).sum(axis=1))
    assert np.all(d > r[pairs[:, 0]] + r[pairs[:, 1]])


def test_ice_sheet_parameters(sheet):
    cfg, st, bonds, strength = sheet
    assert cfg.n == 2048 * 512
    assert len(bonds) == len(strength) == 3_140_609
    assert np.all(st["radius"] == 0.05)
    free = np.isfinite(st["mass"])
    r = 0.05
    assert np.allclose(st["mass"][free], 900.0 * math.pi * r * r * (2.0 * r), rtol=1e-14)
    assert (~free).sum() == 2 * 512  # both short ends clamped
    assert cfg.young == 5e9 and cfg.max_bonds == 6
    assert (cfg.breaking_strain, cfg.shear_breaking_strain) == (0.01, 0.02)
    assert cfg.indenter_radius == 2.0 and cfg.indenter_velocity == (0.0, -0.5)
    logs = np.log(strength)
    assert logs.mean() == pytest.approx(0.0, abs=1e-3) and logs.std() == pytest.approx(0.1, rel=0.01)


def test_ice_sheet_is_a_six_neighbour_hex_lattice(sheet):
    cfg, st, bonds, _ = sheet
    b = np.asarray(bonds)
    deg = np.bincount(b.ravel(), minlength=cfg.n)
    assert deg.max() == 6 and np.mean(deg == 6) > 0.99
    d = st["pos"][b[:, 0]] - st["pos"][b[:, 1]]
    length = np.sqrt((d * d).sum(axis=1))
    assert np.allclose(length, 2.0 * 0.05, rtol=1e-9)  # touching neighbours at rest
    lo, hi = np.minimum(b[:, 0], b[:, 1]), np.maximum(b[:, 0], b[:, 1])
    assert len(np.unique(lo.astype(np.int64) * cfg.n + hi)) == len(b)  # no pair bonded twice


def test_cases_are_seeded():
    a = granular_gas_case(64, seed=3)[1]
    b = granular_gas_case(64, seed=3)[1]
    c = granular_gas_case(64, seed=4)[1]
    assert all(np.array_equal(a[k], b[k]) for k in a)
    assert not np.array_equal(a["pos"], c["pos"])
    s1, s2 = ice_sheet_case(64, 16, seed=3)[3], ice_sheet_case(64, 16, seed=3)[3]
    assert np.array_equal(s1, s2)
