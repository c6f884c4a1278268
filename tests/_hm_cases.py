"""Small seeded Hertz-Mindlin cases shared by the oracle and GPU tests."""

from __future__ import annotations

import math

import numpy as np

from oracle.hm2d import HM2DOracle, HMParams
from tensordem_gb300.hm2d import HM2DConfig, granular_gas_case


def dense_gas(n_side=24, *, seed=3, precision=64, skin=0.02e-3, sigma_v=2.0, walls=15,
              gravity=(0.0, -9.81), mu=0.5, restitution=0.8, max_neighbors=16):
    """A colliding disc gas: area fraction 0.7, radii U[0.9, 1.0] mm, fast particles."""
    cfg, st = granular_gas_case(n_side, seed=seed, r_min=0.9e-3, r_max=1.0e-3, area_fraction=0.7,
                                sigma_v=sigma_v, skin=skin, precision=precision,
                                max_neighbors=max_neighbors, mu=mu, restitution=restitution)
    st["omega"] = np.random.default_rng(seed + 100).normal(0.0, 50.0, cfg.n)
    cfg = HM2DConfig(**{**cfg.__dict__, "walls": walls, "gravity": gravity})
    return cfg, st


def oracle_for(cfg: HM2DConfig, st: dict, *, skin=None) -> HM2DOracle:
    box = cfg.box if cfg.walls else None
    walls = tuple(bool(cfg.walls & b) for b in (1, 2, 4, 8))
    p = HMParams(young=cfg.young, poisson=cfg.poisson, restitution=cfg.restitution, mu=cfg.mu,
                 mu_wall=cfg.mu_wall, dt=cfg.dt, gravity=cfg.gravity, box=box, walls=walls,
                 skin=cfg.skin if skin is None else skin)
    return HM2DOracle(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"], p)


def two_disc_state(delta=1e-6, r=1e-3, rho=2500.0, v_t=0.0, omega=(0.0, 0.0)):
    """Two equal discs overlapping by delta along x, centred in a 10 mm box."""
    pos = np.array([[5e-3, 5e-3], [5e-3 + 2 * r - delta, 5e-3]])
    vel = np.array([[0.0, v_t], [0.0, 0.0]])
    radius = np.array([r, r])
    mass = rho * math.pi * radius**2 * (2 * radius)
    inertia = 0.5 * mass * radius**2
    return dict(pos=pos, vel=vel, omega=np.array(omega, dtype=float), radius=radius, mass=mass,
                inertia=inertia)


def bonded_oracle_for(cfg, st, bonds, strength):
    from oracle.hm2d import BondedHM2DOracle
    p = HMParams(young=cfg.young, poisson=cfg.poisson, restitution=cfg.restitution, mu=cfg.mu,
                 mu_wall=cfg.mu_wall, dt=cfg.dt, gravity=cfg.gravity,
                 box=cfg.box if cfg.walls else None,
                 walls=tuple(bool(cfg.walls & b) for b in (1, 2, 4, 8)), skin=cfg.skin)
    ind = None
    if cfg.indenter_radius > 0:
        ind = dict(center=cfg.indenter_center, velocity=cfg.indenter_velocity, radius=cfg.indenter_radius)
    return BondedHM2DOracle(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"], p,
                            bonds=bonds, strength=strength, k_n=cfg.bond_kn, k_s=cfg.bond_ks,
                            zeta=cfg.bond_damping, eps_t=cfg.breaking_strain,
                            eps_s=cfg.shear_breaking_strain, indenter=ind)


def small_sheet(nx=24, ny=8, *, precision=64, steps=400, speed=2.0, **kw):
    """A small clamped hexagonal sheet with a fast indenter (cracks within a few hundred steps)."""
    from tensordem_gb300.hm2d import ice_sheet_case
    return ice_sheet_case(nx, ny, radius=0.05, indenter_radius=0.3, indenter_speed=speed,
                          precision=precision, steps=steps, **kw)
