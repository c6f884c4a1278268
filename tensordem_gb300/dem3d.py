"""Drop-in ``DEM3DConfig`` / ``IceDEM3D`` on the GB300 CUDA path (3-D reference mode).

Same public surface as the reference's ``tensordem.dem3d`` (src/tensordem/dem3d.py
and its frozen binder contract, src/tensordem/binding_contract.py:204-310):
state tensors ``positions``, ``velocities``, ``initial_positions``, ``fixed``,
``pairs`` / ``bonded`` / ``alive`` and the per-bond failure ledger, ``step``,
``forces(update_fracture=, update_history=)``, ``diagnostics``, ``energy``,
``state_dict`` / ``load_state_dict``, and the diagnostics helpers
(``body_forces``, ``submerged_fraction``, ``body_force_ledger``,
``bond_stored_energy``, ``bond_law_report``, ``lateral_platen_energy``). The
step runs in the FP64 CUDA kernel of ``csrc/icedem3d.cu``.

The constant topology (lattice, bonds, rest lengths, Weibull strengths, the
pseudo-inverse of every particle's bond covariance, Maxwell branch factors) is
built on the host in float64 with the same torch operations the reference
uses, so the kernel starts from the reference's bits.

Differences from the reference, by design:
* CUDA only: ``device`` defaults to ``"cuda"``; any other device raises
  ``ValueError`` (there is no CPU fallback).
* ``run(steps)`` advances many steps in one kernel launch.
* The pair friction history lives on the device (per particle, at most 64
  partners; more raises ``RuntimeError``), so it is not a Python dict. As in
  the reference, an entry is never dropped and is not part of ``state_dict``.
* Not kept: the diagnostic accumulators ``_rolling_torque`` and
  ``last_*_platen_friction``.
"""

from __future__ import annotations

import ctypes as C
import functools
import math
from dataclasses import asdict, dataclass
from typing import Any

import numpy as np
import torch

from . import _lib


# ---------------------------------------------------------------------------
# Hertz helpers (dem3d.py:57-113)
# ---------------------------------------------------------------------------
def _hertz_argument(value) -> torch.Tensor:
    if isinstance(value, torch.Tensor):
        if not value.is_floating_point():
            raise TypeError("overlap must be a floating-point tensor")
        return value.to(torch.float64) if value.dtype != torch.float64 else value
    return torch.tensor(float(value), dtype=torch.float64)


def hertz_reduced_modulus(young_modulus: float, poisson_ratio: float, *, rigid_counterpart: bool = False) -> float:
    """``E*``: E / (2 (1 - nu^2)) for equal spheres, E / (1 - nu^2) against a rigid body."""
    if not math.isfinite(young_modulus) or young_modulus <= 0.0:
        raise ValueError("young_modulus must be finite and positive")
    if not (math.isfinite(poisson_ratio) and 0.0 <= poisson_ratio < 0.5):
        raise ValueError("poisson_ratio must be in [0, 0.5)")
    compliance = 1.0 - poisson_ratio ** 2
    return float(young_modulus / (compliance if rigid_counterpart else 2.0 * compliance))


def hertz_effective_radius(radius: float, *, rigid_counterpart: bool = False) -> float:
    """``R*``: R / 2 for equal spheres, R against a plane."""
    if not math.isfinite(radius) or radius <= 0.0:
        raise ValueError("radius must be finite and positive")
    return float(radius) if rigid_counterpart else 0.5 * float(radius)


def hertz_normal_force(overlap, e_star: float, r_eff: float) -> torch.Tensor:
    """``F = (4/3) E* sqrt(R*) delta^(3/2)``."""
    delta = _hertz_argument(overlap).clamp_min(0.0)
    return (4.0 / 3.0) * float(e_star) * math.sqrt(float(r_eff)) * delta.pow(1.5)


def hertz_contact_potential(overlap, e_star: float, r_eff: float) -> torch.Tensor:
    """``U = (8/15) E* sqrt(R*) delta^(5/2)``."""
    delta = _hertz_argument(overlap).clamp_min(0.0)
    return (8.0 / 15.0) * float(e_star) * math.sqrt(float(r_eff)) * delta.pow(2.5)


def hertz_secant_stiffness(overlap, e_star: float, r_eff: float) -> torch.Tensor:
    """``k_s = F / delta = (4/3) E* sqrt(R*) sqrt(delta)``."""
    delta = _hertz_argument(overlap).clamp_min(0.0)
    return (4.0 / 3.0) * float(e_star) * math.sqrt(float(r_eff)) * delta.sqrt()


def hertz_equivalent_linear_stiffness(young_modulus: float, poisson_ratio: float, radius: float, overlap: float,
                                      *, rigid_counterpart: bool = False) -> float:
    e_star = hertz_reduced_modulus(young_modulus, poisson_ratio, rigid_counterpart=rigid_counterpart)
    r_eff = hertz_effective_radius(radius, rigid_counterpart=rigid_counterpart)
    return float(hertz_secant_stiffness(overlap, e_star, r_eff))


def hertz_reduced_shear_modulus(young_modulus: float, poisson_ratio: float, *,
                                rigid_counterpart: bool = False) -> float:
    """``G*`` of the Mindlin tangential stiffness (hertz_mindlin.py:51-91)."""
    if not math.isfinite(young_modulus) or young_modulus <= 0.0:
        raise ValueError("young_modulus must be finite and positive")
    if not (math.isfinite(poisson_ratio) and 0.0 <= poisson_ratio < 0.5):
        raise ValueError("poisson_ratio must be in [0, 0.5)")
    denom = (2.0 - poisson_ratio) * (1.0 + poisson_ratio)
    return float(young_modulus / ((2.0 if rigid_counterpart else 4.0) * denom))


# ---------------------------------------------------------------------------
# Configuration (dem3d.py:116-561)
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class DEM3DConfig:
    """Numerical and physical parameters of the 3-D bonded-sphere model."""

    nx: int = 9
    ny: int = 5
    nz: int = 3
    radius: float = 0.025
    density: float = 917.0
    bond_stiffness: float = 2_000.0
    contact_stiffness: float = 5_000.0
    tangential_stiffness: float | None = None
    breaking_strain: float = 0.015
    shear_breaking_strain: float = 0.03
    contact_damping: float = 5.0
    drag: float = 2.0
    tool_radius: float = 0.1
    tool_speed: float = 0.5
    tool_gap: float = 0.01
    dt: float | None = None
    device: str = "cuda"
    geometry: str = "box"
    fix_x_edges: bool = True
    fix_bottom: bool = False
    top_platen_enabled: bool = False
    bottom_platen_enabled: bool = False
    platen_stiffness: float = 5_000.0
    platen_damping: float = 0.0
    platen_friction_coefficient: float = 0.0
    platen_friction_stiffness: float | None = None
    top_platen_gap: float = 0.0
    bottom_platen_gap: float = 0.0
    top_platen_velocity: float = 0.0
    bottom_platen_velocity: float = 0.0
    lateral_platens: bool = False
    lateral_platen_stiffness: float | None = None
    lateral_platen_damping: float | None = None
    lateral_platen_gap: float = 0.0
    friction_coefficient: float = 0.0
    rolling_resistance_coefficient: float = 0.0
    restitution_coefficient: float = 1.0
    friction_regularization: str = "none"
    static_friction_coefficient: float | None = None
    dynamic_friction_coefficient: float | None = None
    friction_transition_speed: float = 1.0e-3
    contact_model: str = "linear"
    young_modulus: float = 1.0e9
    poisson_ratio: float = 0.3
    hertz_stability_overlap_fraction: float = 0.1
    contact_damping_model: str = "restitution"
    tangential_model: str = "cundall_strack"
    gravity: float = 0.0
    water_level: float | None = None
    water_density: float = 1025.0
    wet_drag_coefficient: float = 0.0
    bond_model: str = "linear"
    bond_equilibrium_fraction: float = 0.35
    bond_delayed_elastic_fraction: tuple[float, ...] = (0.45, 0.20)
    bond_relaxation_time_s: tuple[float, ...] = (0.5, 30.0)
    bond_creep_exponent: int = 0
    bond_creep_time_s: float = 1.0
    bond_creep_force_fraction: float = 1.0
    bond_strength_weibull_modulus: float = 0.0
    bond_strength_seed: int = 0

    def __post_init__(self) -> None:  # the reference's checks (dem3d.py:268-432)
        def finite_pos(name, v, what="finite and positive"):
            if not math.isfinite(v) or v <= 0:
                raise ValueError(f"{name} must be {what}")

        def finite_nonneg(name, v):
            if not math.isfinite(v) or v < 0:
                raise ValueError(f"{name} must be finite and nonnegative")

        for name in ("nx", "ny", "nz"):
            v = getattr(self, name)
            if isinstance(v, bool) or not isinstance(v, int) or v < 2:
                raise ValueError(f"{name} must be an integer >= 2")
        for name in ("radius", "density", "bond_stiffness", "contact_stiffness", "breaking_strain",
                     "shear_breaking_strain", "tool_radius", "tool_speed"):
            finite_pos(name, getattr(self, name))
        for name in ("contact_damping", "drag", "tool_gap", "platen_damping", "top_platen_gap",
                     "bottom_platen_gap"):
            finite_nonneg(name, getattr(self, name))
        finite_pos("platen_stiffness", self.platen_stiffness)
        finite_nonneg("platen_friction_coefficient", self.platen_friction_coefficient)
        if self.platen_friction_stiffness is not None:
            finite_pos("platen_friction_stiffness", self.platen_friction_stiffness, "finite and positive when given")
        for name in ("top_platen_velocity", "bottom_platen_velocity"):
            if not math.isfinite(getattr(self, name)):
                raise ValueError(f"{name} must be finite")
        for name in ("top_platen_enabled", "bottom_platen_enabled", "lateral_platens"):
            if not isinstance(getattr(self, name), bool):
                raise ValueError(f"{name} must be a boolean")
        if self.dt is not None:
            finite_pos("dt", self.dt)
        if self.lateral_platen_stiffness is not None:
            finite_pos("lateral_platen_stiffness", self.lateral_platen_stiffness, "positive when given")
        if self.lateral_platen_damping is not None and (
                not math.isfinite(self.lateral_platen_damping) or self.lateral_platen_damping < 0):
            raise ValueError("lateral_platen_damping must be nonnegative when given")
        if not math.isfinite(self.lateral_platen_gap) or self.lateral_platen_gap < 0:
            raise ValueError("lateral_platen_gap must be nonnegative")
        if not isinstance(self.device, str) or not self.device.startswith("cuda"):
            raise ValueError("tensordem_gb300.IceDEM3D runs on CUDA devices only (device='cuda')")
        if self.geometry not in ("box", "cylinder_xz"):
            raise ValueError("geometry must be 'box' or 'cylinder_xz'")
        if self.geometry == "cylinder_xz" and (self.nx < 3 or self.nz < 3):
            raise ValueError("cylinder_xz geometry requires nx and nz >= 3")
        finite_nonneg("friction_coefficient", self.friction_coefficient)
        finite_nonneg("rolling_resistance_coefficient", self.rolling_resistance_coefficient)
        if self.friction_regularization not in ("none", "tanh", "dual"):
            raise ValueError("friction_regularization must be 'none', 'tanh' or 'dual'")
        mu_s, mu_d = self.static_friction_coefficient, self.dynamic_friction_coefficient
        for name, value in (("static_friction_coefficient", mu_s), ("dynamic_friction_coefficient", mu_d)):
            if value is not None and (not math.isfinite(value) or value < 0.0):
                raise ValueError(f"{name} must be finite and nonnegative, or None")
        if mu_s is not None and mu_d is not None and mu_d > mu_s:
            raise ValueError("dynamic_friction_coefficient must not exceed static_friction_coefficient")
        finite_pos("friction_transition_speed", self.friction_transition_speed)
        if not (0.0 < self.restitution_coefficient <= 1.0):
            raise ValueError("restitution_coefficient must be in (0, 1]")
        if self.tangential_stiffness is not None:
            finite_pos("tangential_stiffness", self.tangential_stiffness, "finite and positive, or None")
        if self.contact_damping_model not in ("restitution", "absolute", "restitution_calibrated"):
            raise ValueError("contact_damping_model must be 'restitution', 'absolute' or 'restitution_calibrated'")
        if self.contact_damping_model == "restitution_calibrated" and self.contact_model != "hertz":
            raise ValueError("contact_damping_model='restitution_calibrated' requires contact_model='hertz'")
        if self.tangential_model not in ("cundall_strack", "mindlin_partial_slip"):
            raise ValueError("tangential_model must be 'cundall_strack' or 'mindlin_partial_slip'")
        if self.tangential_model == "mindlin_partial_slip":
            if self.contact_model != "hertz":
                raise ValueError("tangential_model='mindlin_partial_slip' requires contact_model='hertz'")
            if self.friction_regularization != "none":
                raise ValueError("tangential_model='mindlin_partial_slip' requires friction_regularization='none'")
        if self.contact_damping_model == "absolute" and self.restitution_coefficient < 1.0:
            raise ValueError("contact_damping_model='absolute' and restitution_coefficient < 1 "
                             "specify the same dashpot twice; pick one convention")
        if self.contact_model not in ("linear", "hertz"):
            raise ValueError("contact_model must be 'linear' or 'hertz'")
        finite_pos("young_modulus", self.young_modulus)
        if not (math.isfinite(self.poisson_ratio) and 0.0 <= self.poisson_ratio < 0.5):
            raise ValueError("poisson_ratio must be in [0, 0.5)")
        if not (math.isfinite(self.hertz_stability_overlap_fraction)
                and 0.0 < self.hertz_stability_overlap_fraction < 1.0):
            raise ValueError("hertz_stability_overlap_fraction must be in (0, 1)")
        if not math.isfinite(self.gravity) or self.gravity < 0.0:
            raise ValueError("gravity must be finite and nonnegative")
        if self.water_level is not None and not math.isfinite(self.water_level):
            raise ValueError("water_level must be finite or None")
        finite_pos("water_density", self.water_density)
        finite_nonneg("wet_drag_coefficient", self.wet_drag_coefficient)
        if self.bond_model not in ("linear", "maxwell_wiechert"):
            raise ValueError("bond_model must be 'linear' or 'maxwell_wiechert'")
        if not (math.isfinite(self.bond_equilibrium_fraction) and 0.0 < self.bond_equilibrium_fraction < 1.0):
            raise ValueError("bond_equilibrium_fraction must be in (0, 1)")
        if len(self.bond_delayed_elastic_fraction) != len(self.bond_relaxation_time_s):
            raise ValueError("bond_delayed_elastic_fraction and bond_relaxation_time_s must have equal length")
        if self.bond_model == "maxwell_wiechert" and not self.bond_relaxation_time_s:
            raise ValueError("bond_model='maxwell_wiechert' needs at least one relaxation time")
        for value in self.bond_relaxation_time_s:
            if not (math.isfinite(value) and value > 0.0):
                raise ValueError("bond_relaxation_time_s entries must be finite and positive")
        for value in self.bond_delayed_elastic_fraction:
            if not (math.isfinite(value) and value > 0.0):
                raise ValueError("bond_delayed_elastic_fraction entries must be finite and positive")
        if (isinstance(self.bond_creep_exponent, bool) or not isinstance(self.bond_creep_exponent, int)
                or self.bond_creep_exponent < 0):
            raise ValueError("bond_creep_exponent must be a nonnegative integer")
        if self.bond_creep_exponent > 0:
            finite_pos("bond_creep_time_s", self.bond_creep_time_s)
            finite_pos("bond_creep_force_fraction", self.bond_creep_force_fraction)
        if isinstance(self.bond_strength_weibull_modulus, bool) or not isinstance(
                self.bond_strength_weibull_modulus, (int, float)):
            raise TypeError("bond_strength_weibull_modulus must be a real number")
        finite_nonneg("bond_strength_weibull_modulus", self.bond_strength_weibull_modulus)
        if isinstance(self.bond_strength_seed, bool) or not isinstance(self.bond_strength_seed, int):
            raise TypeError("bond_strength_seed must be an integer")

    @property
    def mass(self) -> float:
        return self.density * (4.0 / 3.0) * math.pi * self.radius**3

    @property
    def friction_coefficient_pair(self) -> tuple[float, float]:
        mu = float(self.friction_coefficient)
        mu_s = mu if self.static_friction_coefficient is None else float(self.static_friction_coefficient)
        mu_d = mu if self.dynamic_friction_coefficient is None else float(self.dynamic_friction_coefficient)
        return mu_s, mu_d

    def cone_law(self, coefficient: float | None = None) -> tuple[int, tuple[float, float, float]]:
        """The friction-cone law as (TDEM_CONE_* mode, constants) for the kernel."""
        fallback = float(self.friction_coefficient if coefficient is None else coefficient)
        if self.friction_regularization == "none":
            return _lib.CONE_SINGLE, (fallback, 0.0, 0.0)
        mu_s = fallback if self.static_friction_coefficient is None else float(self.static_friction_coefficient)
        mu_d = fallback if self.dynamic_friction_coefficient is None else float(self.dynamic_friction_coefficient)
        if mu_s == mu_d:
            return _lib.CONE_SINGLE, (mu_s, 0.0, 0.0)
        if self.friction_regularization == "tanh":
            return _lib.CONE_TANH, (mu_d, mu_s - mu_d, float(self.friction_transition_speed))
        return _lib.CONE_DUAL, (mu_s, mu_d, 0.0)

    def friction_cone_limit(self, tangential_force_mag: torch.Tensor, normal_force: torch.Tensor,
                            slip_speed: torch.Tensor, *, coefficient: float | None = None):
        """Coulomb cone limit |F_t| <= mu N of the active regularization (dem3d.py:453-498)."""
        mode, c = self.cone_law(coefficient)
        if mode == _lib.CONE_SINGLE:
            return c[0] * normal_force
        if mode == _lib.CONE_TANH:
            blend = 0.5 * (1.0 - torch.tanh(slip_speed / c[2]))
            return (c[0] + c[1] * blend) * normal_force
        static_limit = c[0] * normal_force
        return torch.where(tangential_force_mag > static_limit,
                           torch.as_tensor(c[1], dtype=normal_force.dtype, device=normal_force.device)
                           * normal_force, static_limit)

    @property
    def effective_tangential_stiffness(self) -> float:
        return float(self.contact_stiffness if self.tangential_stiffness is None else self.tangential_stiffness)

    def _bound_stiffness(self, linear_stiffness: float, *, rigid_counterpart: bool) -> float:
        if self.contact_model == "linear":
            return float(linear_stiffness)
        delta_ref = self.hertz_stability_overlap_fraction * self.radius
        return float(hertz_secant_stiffness(
            delta_ref, hertz_reduced_modulus(self.young_modulus, self.poisson_ratio,
                                             rigid_counterpart=rigid_counterpart),
            hertz_effective_radius(self.radius, rigid_counterpart=rigid_counterpart)))

    @property
    def recommended_dt(self) -> float:
        """Conservative explicit stability / travel bound (dem3d.py:531-561)."""
        n = self.nx * self.ny * self.nz
        degree_bound = min(n - 1, 26)
        platen_k = (self.platen_stiffness if self.platen_friction_stiffness is None
                    else max(self.platen_stiffness, self.platen_friction_stiffness))
        lat_k = self.lateral_platen_stiffness if self.lateral_platen_stiffness is not None else self.platen_stiffness
        lat_c = self.lateral_platen_damping if self.lateral_platen_damping is not None else self.platen_damping
        n_platens = int(self.top_platen_enabled) + int(self.bottom_platen_enabled) + (4 if self.lateral_platens else 0)
        contact_stiffness = max(
            self.bond_stiffness,
            self._bound_stiffness(self.contact_stiffness, rigid_counterpart=False),
            self._bound_stiffness(self.effective_tangential_stiffness, rigid_counterpart=False),
            self._bound_stiffness(max(platen_k, lat_k if self.lateral_platens else 0.0), rigid_counterpart=True)
            if n_platens else 0.0,
        )
        k = (2 * degree_bound + 1) * contact_stiffness
        c = ((2 * degree_bound + 1) * self.contact_damping + self.drag
             + n_platens * max(self.platen_damping, lat_c if self.lateral_platens else 0.0))
        elastic = 0.15 * math.sqrt(self.mass / k)
        damping = 0.15 * self.mass / c if c > 0 else math.inf
        travel = 0.1 * self.radius / self.tool_speed
        return min(elastic, damping, travel)


# ---------------------------------------------------------------------------
# Bond-law constants (ice_bond_viscoelastic.py:98-183)
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class MaxwellWiechertBond:
    """Equilibrium spring k0 plus Maxwell branches (k_a, tau_a)."""

    equilibrium_stiffness: float
    branch_stiffness: tuple[float, ...]
    relaxation_time: tuple[float, ...]

    @classmethod
    def from_unrelaxed_stiffness(cls, unrelaxed_stiffness: float, *, equilibrium_fraction: float,
                                 delayed_elastic_fraction: tuple[float, ...],
                                 relaxation_time: tuple[float, ...]) -> "MaxwellWiechertBond":
        shares = tuple(float(f) for f in delayed_elastic_fraction)
        share_sum = sum(shares)
        k_total = float(unrelaxed_stiffness)
        k0 = equilibrium_fraction * k_total
        branches = tuple((1.0 - equilibrium_fraction) * k_total * (f / share_sum) for f in shares)
        return cls(k0, branches, tuple(float(t) for t in relaxation_time))

    @property
    def n_branches(self) -> int:
        return len(self.branch_stiffness)

    @property
    def unrelaxed_stiffness(self) -> float:
        return float(self.equilibrium_stiffness + sum(self.branch_stiffness))


@functools.lru_cache(maxsize=256)
def hertz_damping_ratio_for_restitution(e_requested: float) -> float:
    """Damping ratio whose Hertz + Tsuji dashpot delivers the restitution
    ``e_requested`` (contact_calibration.py:219-248), from the library's host
    routine ``tdem_hertz_damping_ratio`` (RK4 on the universal impact ODE,
    secant inversion)."""
    out = C.c_double()
    rc = _lib.lib().tdem_hertz_damping_ratio(float(e_requested), C.byref(out))
    if rc != _lib.TDEM_OK:
        raise ValueError("restitution must be in (0, 1]")
    return float(out.value)


def weibull_strength_factors(n: int, modulus: float, seed: int) -> torch.Tensor:
    """Per-bond strength factors with median 1 (ice_bond_viscoelastic.py:300-323):
    ``scale * (-log(1 - U))**(1/m)``, ``scale = 1 / ln(2)**(1/m)``, U from a
    private CPU ``torch.Generator`` seeded with ``seed``."""
    generator = torch.Generator(device="cpu").manual_seed(int(seed))
    scale = 1.0 / math.log(2.0) ** (1.0 / float(modulus))
    u = torch.rand(n, generator=generator, dtype=torch.float64)
    u = u.clamp_min(torch.finfo(torch.float64).tiny)
    return scale * (-torch.log1p(-u)).pow(1.0 / float(modulus))


def submerged_fraction_sphere_tensor(z: torch.Tensor, radius: float, water_level: float = 0.0) -> torch.Tensor:
    """Spherical-cap submerged volume fraction (buoyancy_wet3d.py:134-155)."""
    if radius <= 0.0:
        raise ValueError("radius must be positive")
    h = z - water_level
    hc = torch.clamp(h, -radius, radius)
    f = (radius - hc) ** 2 * (2.0 * radius + hc) / (4.0 * radius ** 3)
    f = torch.clamp(f, 0.0, 1.0)
    f = torch.where(h >= radius, torch.zeros_like(f), f)
    return torch.where(h <= -radius, torch.ones_like(f), f)


class _Handle3D:
    """Owns one native 3-D reference-mode instance."""

    def __init__(self, cfg_c: _lib.IceDEM3DConfigC, topo: _lib.IceDEM3DTopologyC):
        ptr = C.c_void_p()
        rc = _lib.lib().tdem_icedem3d_create(C.byref(cfg_c), C.byref(topo), C.byref(ptr))
        _lib.check(rc, None, "tdem_icedem3d_create")
        self.ptr = ptr

    def __del__(self):
        if getattr(self, "ptr", None) is not None and _lib._lib is not None:
            _lib._lib.tdem_icedem3d_destroy(self.ptr)
            self.ptr = None


def _host_ptr(t: torch.Tensor | None):
    return None if t is None else t.data_ptr()


# Checkpoint layout of IceDEM3D.state_dict: required keys, the per-particle
# and per-pair tensors restored, and the ones that must equal the solver's own.
_CHECKPOINT_KEYS = frozenset({
    "dimension", "config", "dt", "time", "step_count", "positions", "velocities", "initial_positions", "fixed",
    "pairs", "bonded", "alive", "failure_mode", "failure_time_s", "failure_extension_m", "failure_energy_J"})
_CHECKPOINT_TENSORS = ("positions", "velocities", "initial_positions", "fixed", "pairs", "bonded", "alive",
                       "failure_mode", "failure_time_s", "failure_extension_m", "failure_energy_J")
_CHECKPOINT_FROZEN = (("initial_positions", "checkpoint reference geometry does not match this solver"),
                      ("pairs", "checkpoint pair topology does not match this solver"),
                      ("bonded", "checkpoint bond topology does not match this solver"),
                      ("fixed", "checkpoint fixed-boundary mask does not match this solver"))


class IceDEM3D:
    """3-D bonded-sphere DEM with a spherical indenter, stepped on the GPU.

    State arrays have shape (N, 3); external forces are instantaneous nodal
    loads in newtons. Bond failure is irreversible; contacts come from a cell
    list rebuilt at every force evaluation (dem3d.py:564-577).
    """

    def __init__(self, config: DEM3DConfig = DEM3DConfig()) -> None:
        self.config = config
        self.device = torch.device(config.device)
        if not torch.cuda.is_available():
            raise ValueError("CUDA requested but unavailable")
        self.dtype = torch.float64
        self.dt = config.dt if config.dt is not None else config.recommended_dt
        if self.dt > config.recommended_dt:
            raise ValueError(f"dt exceeds conservative limit {config.recommended_dt:.6g} s")
        host = self._build_topology()
        dev = self.device
        self.initial_positions = host["initial_positions"].to(dev)
        self.fixed = host["fixed"].to(dev)
        self.pairs = host["pairs"].to(dev)
        self.rest_lengths = host["rest_lengths"].to(dev)
        self.bonded = host["bonded"].to(dev)
        self.reference_bond_vectors = host["reference_bond_vectors"].to(dev)
        self.initial_normals = host["initial_normals"].to(dev)
        self.positions = self.initial_positions.clone()
        self.velocities = torch.zeros_like(self.positions)
        self.alive = self.bonded.clone()
        self.bond_indices = self.pairs
        b = len(self.pairs)
        self.failure_mode = torch.zeros(b, dtype=torch.uint8, device=dev)
        self.failure_time_s = torch.full((b,), -1.0, dtype=self.dtype, device=dev)
        self.failure_extension_m = torch.zeros(b, dtype=self.dtype, device=dev)
        self.failure_energy_J = torch.zeros(b, dtype=self.dtype, device=dev)
        self.bond_law = host["bond_law"]
        m = self.bond_law.n_branches if self.bond_law is not None else 0
        self.branch_offsets = torch.zeros((b, m), dtype=self.dtype, device=dev)
        self._bond_elongation_prev = torch.zeros(b, dtype=self.dtype, device=dev)
        self.bond_damage = torch.zeros(b, dtype=self.dtype, device=dev)
        self.bond_strength_factors = host["strength_factors"]
        self.bond_breaking_strain = host["breaking_strain"]
        if self.bond_strength_factors is not None:
            self.bond_strength_factors = self.bond_strength_factors.to(dev)
            self.bond_breaking_strain = self.bond_breaking_strain.to(dev)
        self._dissipation = torch.zeros(1, dtype=self.dtype, device=dev)
        self.time = 0.0
        self.step_count = 0
        self.energy_audit = None
        self.tool_start = torch.tensor(
            [0.0, 0.0, (config.nz - 1) * 2 * config.radius + config.radius + config.tool_radius + config.tool_gap],
            dtype=self.dtype, device=dev)
        self.tool_velocity = torch.tensor([0.0, 0.0, -config.tool_speed], dtype=self.dtype, device=dev)
        self.last_reaction = torch.zeros(3, dtype=self.dtype, device=dev)
        x0 = host["initial_positions"]
        self.top_platen_start_z = float(x0[:, 2].max()) + config.radius + config.top_platen_gap
        self.bottom_platen_start_z = float(x0[:, 2].min()) - config.radius - config.bottom_platen_gap
        self.last_top_platen_reaction_z = torch.zeros((), dtype=self.dtype, device=dev)
        self.last_bottom_platen_reaction_z = torch.zeros((), dtype=self.dtype, device=dev)
        self.lateral_platen_pos = torch.zeros(4, dtype=self.dtype, device=dev)
        self.lateral_platen_velocity = torch.zeros(4, dtype=self.dtype, device=dev)
        if config.lateral_platens:
            g = config.lateral_platen_gap
            self.lateral_platen_pos[0] = float(x0[:, 0].min()) - config.radius - g
            self.lateral_platen_pos[1] = float(x0[:, 0].max()) + config.radius + g
            self.lateral_platen_pos[2] = float(x0[:, 1].min()) - config.radius - g
            self.lateral_platen_pos[3] = float(x0[:, 1].max()) + config.radius + g
        self.last_lateral_platen_reaction = torch.zeros(4, dtype=self.dtype, device=dev)
        n = len(self.positions)
        self._top_platen_tang_disp = torch.zeros((n, 3), dtype=self.dtype, device=dev)
        self._bottom_platen_tang_disp = torch.zeros((n, 3), dtype=self.dtype, device=dev)
        self._last_friction_power = 0.0
        self._last_rolling_power = 0.0
        self.rolling_resistance_torque_physical = config.rolling_resistance_coefficient > 0.0
        self._build_native(host)

    # ----------------------------------------------------------- topology
    def _build_topology(self) -> dict:
        """Lattice, bonds and per-particle constants on the CPU in float64,
        with the reference's torch operations (dem3d.py:579-757, 875-901)."""
        cfg = self.config
        f64 = torch.float64
        axes = [torch.arange(v, dtype=f64) for v in (cfg.nx, cfg.ny, cfg.nz)]
        zz, yy, xx = torch.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
        full_grid = torch.stack((xx, yy, zz), dim=-1).reshape(-1, 3)
        if cfg.geometry == "cylinder_xz":
            xc, zc = (cfg.nx - 1) / 2.0, (cfg.nz - 1) / 2.0
            disk_radius = min(cfg.nx - 1, cfg.nz - 1) / 2.0
            keep = ((xx - xc).square() + (zz - zc).square()) <= disk_radius**2 + 1e-12
        else:
            keep = torch.ones_like(xx, dtype=torch.bool)
        keep = keep.reshape(-1)
        compact_to_full = torch.nonzero(keep, as_tuple=False).flatten()
        full_to_compact = np.full(len(full_grid), -1, dtype=np.int64)
        full_to_compact[compact_to_full.numpy()] = np.arange(len(compact_to_full))
        grid = full_grid[compact_to_full]
        z_origin = (cfg.nz - 1) / 2.0 if cfg.geometry == "cylinder_xz" else 0.0
        positions = (grid - torch.tensor([(cfg.nx - 1) / 2, (cfg.ny - 1) / 2, z_origin], dtype=f64)) \
            * (2 * cfg.radius)
        fixed = torch.zeros(len(grid), dtype=torch.bool)
        gx, gy, gz = grid.unbind(dim=1)
        if cfg.fix_x_edges and cfg.geometry == "box":
            fixed |= (gx == 0) | (gx == cfg.nx - 1)
        if cfg.fix_bottom:
            fixed |= gz == 0
        # lattice neighbours within one cell in each axis, half-space offsets
        n = len(grid)
        x, y, z = np.meshgrid(np.arange(cfg.nx), np.arange(cfg.ny), np.arange(cfg.nz), indexing="ij")
        pairs = []
        for dz in (0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    if (dx, dy, dz) == (0, 0, 0) or not (dz > 0 or (dz == 0 and dy > 0) or
                                                         (dz == 0 and dy == 0 and dx > 0)):
                        continue
                    x2, y2, z2 = x + dx, y + dy, z + dz
                    ok = (x2 >= 0) & (x2 < cfg.nx) & (y2 >= 0) & (y2 < cfg.ny) & (z2 >= 0) & (z2 < cfg.nz)
                    a = full_to_compact[((z * cfg.ny + y) * cfg.nx + x)[ok]]
                    bb = full_to_compact[((z2 * cfg.ny + y2) * cfg.nx + x2)[ok]]
                    sel = (a >= 0) & (bb >= 0)
                    pairs.append(np.stack((np.minimum(a, bb)[sel], np.maximum(a, bb)[sel]), axis=1))
        pairs = np.concatenate(pairs) if pairs else np.zeros((0, 2), dtype=np.int64)
        pairs = pairs[np.argsort(pairs[:, 0] * n + pairs[:, 1], kind="stable")]
        pairs_t = torch.from_numpy(pairs.astype(np.int64))
        i, j = pairs_t.T
        ref = positions[j] - positions[i]
        rest = torch.linalg.vector_norm(ref, dim=1)
        normals = ref / rest.clamp_min(torch.finfo(f64).eps)[:, None]
        # per-particle bond covariance, its pseudo-inverse and rank (dem3d.py:875-901)
        rr = ref[:, :, None] * ref[:, None, :]
        cov = torch.zeros((n, 3, 3), dtype=f64)
        cov.index_add_(0, i, rr)
        cov.index_add_(0, j, rr)
        full_rank = torch.linalg.matrix_rank(cov) >= 3
        pinv = torch.linalg.pinv(cov)
        bond_law = None
        if cfg.bond_model == "maxwell_wiechert":
            bond_law = MaxwellWiechertBond.from_unrelaxed_stiffness(
                cfg.bond_stiffness, equilibrium_fraction=cfg.bond_equilibrium_fraction,
                delayed_elastic_fraction=cfg.bond_delayed_elastic_fraction,
                relaxation_time=cfg.bond_relaxation_time_s)
            if bond_law.n_branches > 4:
                raise NotImplementedError("at most 4 Maxwell branches are built on the CUDA path")
        factors = threshold = None
        if cfg.bond_strength_weibull_modulus > 0.0 and len(pairs):
            factors = weibull_strength_factors(len(pairs), float(cfg.bond_strength_weibull_modulus),
                                               cfg.bond_strength_seed)
            threshold = cfg.breaking_strain * factors
        creep_ref = None
        if cfg.bond_creep_exponent > 0:
            k_unrel = bond_law.unrelaxed_stiffness if bond_law is not None else float(cfg.bond_stiffness)
            thr = cfg.breaking_strain if threshold is None else threshold
            creep_ref = cfg.bond_creep_force_fraction * k_unrel * thr * rest
        return dict(positions=positions, initial_positions=positions.clone(), fixed=fixed, pairs=pairs_t,
                    rest_lengths=rest, bonded=torch.ones(len(pairs), dtype=torch.bool),
                    reference_bond_vectors=ref, initial_normals=normals, pinv=pinv.contiguous(),
                    full_rank=full_rank.to(torch.uint8).contiguous(), bond_law=bond_law,
                    strength_factors=factors, breaking_strain=threshold, creep_reference=creep_ref)

    def _build_native(self, host: dict) -> None:
        cfg = self.config
        c = _lib.IceDEM3DConfigC()
        n, b = len(host["positions"]), len(host["pairs"])
        c.n, c.nbond = n, b
        hertz = cfg.contact_model == "hertz"
        c.hertz = int(hertz)
        e_pair, r_pair = self._hertz_pair_params
        e_rig, r_rig = self._hertz_rigid_params
        c.hertz_kn = (4.0 / 3.0) * float(e_pair) * math.sqrt(float(r_pair))
        c.hertz_kn_rigid = (4.0 / 3.0) * float(e_rig) * math.sqrt(float(r_rig))
        c.hertz_pot = (8.0 / 15.0) * float(e_pair) * math.sqrt(float(r_pair))
        c.hertz_kt = 8.0 * float(self._hertz_g_star) * math.sqrt(float(r_pair))
        c.hertz_tangential = int(hertz and cfg.tangential_stiffness is None)
        c.tangential_k = cfg.effective_tangential_stiffness
        c.radius, c.mass, c.dt, c.drag = cfg.radius, cfg.mass, self.dt, cfg.drag
        c.contact_k = cfg.contact_stiffness
        c.mass_mobile, c.mass_pinned = cfg.mass / 2.0, cfg.mass
        if cfg.contact_damping_model == "absolute":
            c.damping, c.damping_c = 2, cfg.contact_damping
        elif cfg.restitution_coefficient < 1.0:
            if cfg.contact_damping_model == "restitution_calibrated":
                zeta = hertz_damping_ratio_for_restitution(cfg.restitution_coefficient)
            else:
                ln_e = math.log(cfg.restitution_coefficient)
                abs_ln_e = -ln_e
                zeta = abs_ln_e / math.sqrt(math.pi ** 2 + abs_ln_e ** 2)
            c.damping, c.damping_c = 1, 2.0 * zeta
            c.gamma_mobile = 2.0 * zeta * math.sqrt(cfg.contact_stiffness * (cfg.mass / 2.0))
            c.gamma_pinned = 2.0 * zeta * math.sqrt(cfg.contact_stiffness * cfg.mass)
        c.any_fixed = int(bool(host["fixed"].any()))
        if cfg.friction_coefficient > 0.0:
            mode, cc = cfg.cone_law()
            c.cone = mode
            c.cone_c[:] = cc
        if cfg.platen_friction_coefficient > 0.0:
            mode, cc = cfg.cone_law(cfg.platen_friction_coefficient)
            c.platen_cone = mode
            c.platen_cone_c[:] = cc
        if cfg.tangential_model == "mindlin_partial_slip":
            # Mindlin-Deresiewicz partial slip (mindlin_partial_slip.py:119-232): the
            # platen's no-slip stiffness is 8 G* a of the rigid counterpart
            c.mindlin = 1
            c.mindlin_platen_8g = 8.0 * hertz_reduced_shear_modulus(cfg.young_modulus, cfg.poisson_ratio,
                                                                    rigid_counterpart=True)
            c.rigid_radius = r_rig
            c.rigid_4e = 4.0 * e_rig
        c.rolling = int(cfg.rolling_resistance_coefficient > 0.0)
        c.roll_mu = cfg.rolling_resistance_coefficient
        c.tool_radius, c.tool_damping = cfg.tool_radius, cfg.contact_damping
        c.tool_start[:] = self.tool_start.tolist()
        c.tool_velocity[:] = self.tool_velocity.tolist()
        c.platens = (int(cfg.top_platen_enabled) | (int(cfg.bottom_platen_enabled) << 1)
                     | (int(cfg.lateral_platens) << 2))
        c.platen_k, c.platen_c, c.platen_kt = cfg.platen_stiffness, cfg.platen_damping, self.platen_friction_k
        c.top_start_z, c.top_velocity = self.top_platen_start_z, cfg.top_platen_velocity
        c.bottom_start_z, c.bottom_velocity = self.bottom_platen_start_z, cfg.bottom_platen_velocity
        c.lateral_k = cfg.lateral_platen_stiffness if cfg.lateral_platen_stiffness is not None else cfg.platen_stiffness
        c.lateral_c = cfg.lateral_platen_damping if cfg.lateral_platen_damping is not None else cfg.platen_damping
        body = cfg.gravity > 0.0 or cfg.water_level is not None
        c.body = (int(body) | (int(cfg.water_level is not None) << 1)
                  | (int(cfg.water_level is not None and cfg.wet_drag_coefficient > 0.0) << 2))
        c.gravity_force = cfg.mass * cfg.gravity
        volume = (4.0 / 3.0) * math.pi * cfg.radius ** 3
        c.buoyancy_force = cfg.water_density * cfg.gravity * volume
        c.wet_drag = cfg.wet_drag_coefficient
        c.water_level = 0.0 if cfg.water_level is None else cfg.water_level
        c.cap_denominator = 4.0 * cfg.radius ** 3
        c.breaking_strain, c.shear_breaking_strain = cfg.breaking_strain, cfg.shear_breaking_strain
        law = self.bond_law
        if law is None:
            c.bond_k = cfg.bond_stiffness
        else:
            c.bond_k = float(law.equilibrium_stiffness)
            c.n_branches = law.n_branches
            for a, (k, tau) in enumerate(zip(law.branch_stiffness, law.relaxation_time)):
                c.branch_k[a], c.branch_tau[a] = float(k), float(tau)
                arg = torch.tensor(-self.dt / float(tau), dtype=torch.float64)
                c.branch_decay[a] = float(torch.exp(arg))
                c.branch_one_minus[a] = float(-torch.expm1(arg))
        if cfg.bond_creep_exponent > 0:
            c.creep = 1
            c.creep_exponent = float(cfg.bond_creep_exponent)
            c.creep_dt_over_time = self.dt / float(cfg.bond_creep_time_s)
        keep = {}

        def arr(t, dtype):
            if t is None:
                return None
            a = t.detach().to("cpu", dtype).contiguous()
            keep[id(a)] = a
            return a.data_ptr()

        topo = _lib.IceDEM3DTopologyC()
        topo.bond_i = arr(host["pairs"][:, 0], torch.int32)
        topo.bond_j = arr(host["pairs"][:, 1], torch.int32)
        topo.rest_length = arr(host["rest_lengths"], torch.float64)
        topo.reference = arr(host["reference_bond_vectors"], torch.float64)
        topo.initial_normal = arr(host["initial_normals"], torch.float64)
        topo.threshold = arr(host["breaking_strain"], torch.float64)
        topo.creep_reference = arr(host["creep_reference"], torch.float64)
        topo.pinv = arr(host["pinv"], torch.float64)
        topo.full_rank = arr(host["full_rank"], torch.uint8)
        self._cfg_c = c
        self._handle = _Handle3D(c, topo)
        self._fixed_u8 = self.fixed.to(torch.uint8)

    # ----------------------------------------------------------- properties
    @property
    def platen_friction_k(self) -> float:
        k_t = self.config.platen_friction_stiffness
        return float(self.config.platen_stiffness if k_t is None else k_t)

    @property
    def _hertz_pair_params(self) -> tuple[float, float]:
        return (hertz_reduced_modulus(self.config.young_modulus, self.config.poisson_ratio),
                hertz_effective_radius(self.config.radius))

    @property
    def _hertz_rigid_params(self) -> tuple[float, float]:
        return (hertz_reduced_modulus(self.config.young_modulus, self.config.poisson_ratio, rigid_counterpart=True),
                hertz_effective_radius(self.config.radius, rigid_counterpart=True))

    @property
    def _hertz_g_star(self) -> float:
        return hertz_reduced_shear_modulus(self.config.young_modulus, self.config.poisson_ratio)

    @property
    def tool_position(self) -> torch.Tensor:
        return self.tool_start + self.time * self.tool_velocity

    @property
    def broken_bonds(self) -> int:
        return int((self.bonded & ~self.alive).sum().item())

    @property
    def unrelaxed_bond_stiffness(self) -> float:
        return float(self.config.bond_stiffness if self.bond_law is None else self.bond_law.unrelaxed_stiffness)

    @property
    def cumulative_bond_dissipation_J(self) -> float:
        return float(self._dissipation[0])

    @cumulative_bond_dissipation_J.setter
    def cumulative_bond_dissipation_J(self, value: float) -> None:
        self._dissipation.fill_(float(value))

    @property
    def buoyancy_active(self) -> bool:
        return self.config.water_level is not None

    def friction_coefficient_pair(self) -> tuple[float, float]:
        return self.config.friction_coefficient_pair

    def friction_cone_limit(self, tangential_force_mag, normal_force, slip_speed, *, coefficient=None):
        return self.config.friction_cone_limit(tangential_force_mag, normal_force, slip_speed,
                                               coefficient=coefficient)

    # ----------------------------------------------------------- native calls
    def _state(self) -> _lib.IceDEM3DStateC:
        for name in ("positions", "velocities", "alive", "failure_mode", "failure_time_s",
                     "failure_extension_m", "failure_energy_J", "branch_offsets", "_bond_elongation_prev",
                     "bond_damage", "_top_platen_tang_disp", "_bottom_platen_tang_disp",
                     "lateral_platen_pos", "lateral_platen_velocity"):
            t = getattr(self, name)
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.is_contiguous()):
                t = torch.as_tensor(t).to(device=self.device).contiguous()
                setattr(self, name, t)
        if self.positions.dtype != torch.float64 or self.velocities.dtype != torch.float64:
            raise ValueError("positions and velocities must be float64")
        if self.alive.dtype != torch.bool:
            raise ValueError("alive must be a bool tensor")
        st = _lib.IceDEM3DStateC()
        st.positions, st.velocities = self.positions.data_ptr(), self.velocities.data_ptr()
        st.initial_positions = self.initial_positions.data_ptr()
        st.fixed = self._fixed_u8.data_ptr()
        st.alive = self.alive.data_ptr()
        st.failure_mode = self.failure_mode.data_ptr()
        st.failure_time_s = self.failure_time_s.data_ptr()
        st.failure_extension_m = self.failure_extension_m.data_ptr()
        st.failure_energy_J = self.failure_energy_J.data_ptr()
        if self._cfg_c.n_branches:
            st.branch_offsets = self.branch_offsets.data_ptr()
            st.elongation_prev = self._bond_elongation_prev.data_ptr()
        st.damage = self.bond_damage.data_ptr()
        st.bond_dissipation = self._dissipation.data_ptr()
        st.top_tangential = self._top_platen_tang_disp.data_ptr()
        st.bottom_tangential = self._bottom_platen_tang_disp.data_ptr()
        st.lateral_position = self.lateral_platen_pos.data_ptr()
        st.lateral_velocity = self.lateral_platen_velocity.data_ptr()
        return st

    def _stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def _loads(self, external_forces):
        if external_forces is None:
            return None
        if not isinstance(external_forces, torch.Tensor) or tuple(external_forces.shape) != tuple(
                self.positions.shape):
            raise ValueError(f"external_forces must be a tensor of shape {tuple(self.positions.shape)}")
        loads = external_forces.to(device=self.device, dtype=self.dtype).contiguous()
        if not bool(torch.isfinite(loads).all()):
            raise ValueError("external_forces must contain only finite values")
        return loads

    def read_ledger(self) -> np.ndarray:
        out = (C.c_double * _lib.L3_COUNT)()
        rc = _lib.lib().tdem_icedem3d_read_ledger(self._handle.ptr, out, _lib.L3_COUNT, self._stream())
        _lib.check(rc, self._handle.ptr, "tdem_icedem3d_read_ledger")
        return np.frombuffer(out, dtype=np.float64).copy()

    def _publish(self, led: np.ndarray, *, update_fracture: bool, update_history: bool,
                 reaction: torch.Tensor) -> None:
        if update_fracture:
            self.last_reaction.copy_(reaction)
        self.last_top_platen_reaction_z.fill_(float(led[_lib.L3_TOP]))
        self.last_bottom_platen_reaction_z.fill_(float(led[_lib.L3_BOTTOM]))
        self.last_lateral_platen_reaction.copy_(torch.as_tensor(led[_lib.L3_LATERAL:_lib.L3_LATERAL + 4]))
        if update_history:
            self._last_friction_power = float(led[_lib.L3_FRICTION_POWER])
            self._last_rolling_power = float(led[_lib.L3_ROLLING_POWER])

    def _evaluate(self, loads, update_fracture: bool, update_history: bool):
        st = self._state()
        force = torch.empty_like(self.positions)
        rc = _lib.lib().tdem_icedem3d_forces(self._handle.ptr, C.byref(st), _host_ptr(loads), float(self.time),
                                              int(update_fracture), int(update_history), force.data_ptr(),
                                              self._stream())
        _lib.check(rc, self._handle.ptr, "tdem_icedem3d_forces")
        led = self.read_ledger()
        reaction = torch.tensor(led[_lib.L3_REACTION:_lib.L3_REACTION + 3], dtype=self.dtype, device=self.device)
        return force, reaction, led

    # ----------------------------------------------------------- public API
    @torch.no_grad()
    def forces(self, external_forces: torch.Tensor | None = None, *, update_fracture: bool = True,
               update_history: bool = True) -> tuple[torch.Tensor, torch.Tensor]:
        """Total force (N,3) and ice-on-tool reaction (3,) (dem3d.py:1301-1642)."""
        loads = self._loads(external_forces)
        force, reaction, led = self._evaluate(loads, update_fracture, update_history)
        self._publish(led, update_fracture=update_fracture, update_history=update_history, reaction=reaction)
        return force, reaction

    @torch.no_grad()
    def step(self, external_forces: torch.Tensor | None = None) -> None:
        """Single explicit Euler step (dem3d.py:1644-1663)."""
        self._advance(1, self._loads(external_forces))

    @torch.no_grad()
    def run(self, steps: int, external_forces: torch.Tensor | None = None) -> None:
        """``steps`` steps in one kernel launch (loads, if given, held over all)."""
        if isinstance(steps, bool) or not isinstance(steps, int) or steps < 0:
            raise ValueError("steps must be a nonnegative integer")
        loads = self._loads(external_forces)
        if self.energy_audit is not None:
            for _ in range(steps):
                self._advance(1, loads)
            return
        if steps:
            self._advance(steps, loads)

    def _advance(self, steps: int, loads) -> None:
        st = self._state()
        rc = _lib.lib().tdem_icedem3d_step(self._handle.ptr, C.byref(st), _host_ptr(loads), int(steps),
                                            float(self.time), self._stream())
        led = self.read_ledger()
        done = int(led[_lib.L3_STEPS_DONE])
        for _ in range(done):
            self.time += self.dt
        self.step_count += done
        reaction = torch.tensor(led[_lib.L3_REACTION:_lib.L3_REACTION + 3], dtype=self.dtype, device=self.device)
        self._publish(led, update_fracture=True, update_history=True, reaction=reaction)
        if rc == _lib.TDEM_ERR_NONFINITE:
            raise FloatingPointError("non-finite DEM3D state; reduce dt or contact stiffness")
        _lib.check(rc, self._handle.ptr, "tdem_icedem3d_step")
        if self.energy_audit is not None:
            self.energy_audit.observe(self)

    def set_thread_mapping(self, mapping: str) -> None:
        """``"auto"`` (default), ``"lanes"`` or ``"particle"``: how the kernel maps
        threads onto particles. Results are bitwise the same; speed differs."""
        modes = {"auto": 0, "lanes": 1, "particle": 2}
        if mapping not in modes:
            raise ValueError("mapping must be 'auto', 'lanes' or 'particle'")
        rc = _lib.lib().tdem_icedem3d_set_mapping(self._handle.ptr, modes[mapping])
        _lib.check(rc, self._handle.ptr, "tdem_icedem3d_set_mapping")

    def contact_pairs(self) -> torch.Tensor:
        """Overlapping pairs (i < j) found by the last force evaluation (int64, (K,2))."""
        cap = max(16, 32 * len(self.positions))
        buf = np.empty((cap, 2), dtype=np.int32)
        count = C.c_int64()
        rc = _lib.lib().tdem_icedem3d_read_contacts(self._handle.ptr, buf.ctypes.data, cap, C.byref(count),
                                                     self._stream())
        _lib.check(rc, self._handle.ptr, "tdem_icedem3d_read_contacts")
        return torch.from_numpy(buf[:count.value].astype(np.int64))

    def friction_history(self) -> dict[tuple[int, int], tuple[float, float, float]]:
        """The pair friction history: {(i, j): stored tangential displacement}, i < j."""
        cap = 64 * len(self.positions)
        pairs = np.empty((cap, 2), dtype=np.int32)
        disp = np.empty((cap, 3), dtype=np.float64)
        count = C.c_int64()
        rc = _lib.lib().tdem_icedem3d_read_history(self._handle.ptr, pairs.ctypes.data, disp.ctypes.data, cap,
                                                    C.byref(count), self._stream())
        _lib.check(rc, self._handle.ptr, "tdem_icedem3d_read_history")
        return {(int(a), int(b)): tuple(float(x) for x in d) for (a, b), d in zip(pairs[:count.value],
                                                                                  disp[:count.value])}

    def set_friction_history(self, history: dict[tuple[int, int], Any]) -> None:
        """Replace the pair friction history ({(i, j): (dx, dy, dz)}, i < j)."""
        items = sorted(history.items())
        pairs = np.ascontiguousarray([p for p, _ in items], dtype=np.int32).reshape(-1, 2)
        disp = np.ascontiguousarray([tuple(float(x) for x in d) for _, d in items], dtype=np.float64).reshape(-1, 3)
        rc = _lib.lib().tdem_icedem3d_set_history(self._handle.ptr, pairs.ctypes.data if len(items) else None,
                                                   disp.ctypes.data if len(items) else None, len(items),
                                                   self._stream())
        _lib.check(rc, self._handle.ptr, "tdem_icedem3d_set_history")

    # ----------------------------------------------------------- energy / diagnostics
    @torch.no_grad()
    def submerged_fraction(self) -> torch.Tensor:
        cfg = self.config
        if cfg.water_level is None:
            return torch.zeros(len(self.positions), dtype=self.dtype, device=self.device)
        return submerged_fraction_sphere_tensor(self.positions[:, 2], cfg.radius, cfg.water_level)

    def _body_terms(self):
        """Per-particle vertical weight and buoyancy (N) and the wet-drag
        coefficient times the submerged fraction (N s/m), from which both
        ``body_forces`` and ``body_force_ledger`` are formed. Buoyancy lifts
        the submerged volume fraction of each sphere with the water's weight;
        the drag opposes the velocity in proportion to that fraction."""
        cfg = self.config
        n = len(self.positions)
        frac = self.submerged_fraction()
        weight = torch.full((n,), -cfg.mass * cfg.gravity if cfg.gravity > 0.0 else 0.0, dtype=self.dtype,
                            device=self.device)
        if cfg.water_level is None:
            return weight, torch.zeros_like(weight), torch.zeros_like(weight), frac
        sphere = (4.0 / 3.0) * math.pi * cfg.radius ** 3
        lift = cfg.water_density * cfg.gravity * sphere * frac
        drag = cfg.wet_drag_coefficient * frac if cfg.wet_drag_coefficient > 0.0 else torch.zeros_like(frac)
        return weight, lift, drag, frac

    @torch.no_grad()
    def body_forces(self) -> torch.Tensor:
        """Gravity, buoyancy and wet drag on every particle, (N, 3) in N."""
        weight, lift, drag, _ = self._body_terms()
        body = -drag[:, None] * self.velocities
        body[:, 2] += weight + lift
        return body

    @torch.no_grad()
    def body_force_ledger(self) -> dict[str, float]:
        """Vertical totals of the body forces and the submerged volume."""
        cfg = self.config
        weight, lift, drag, frac = self._body_terms()
        g = -cfg.mass * cfg.gravity * len(self.positions)
        b = float(lift.sum())
        w = float(-(drag * self.velocities[:, 2]).sum())
        sphere = (4.0 / 3.0) * math.pi * cfg.radius ** 3
        return {"gravity_force_z_N": float(g), "buoyancy_force_z_N": b, "wet_drag_force_z_N": w,
                "net_body_force_z_N": float(g + b + w), "submerged_volume_m3": float((sphere * frac).sum())}

    @torch.no_grad()
    def bond_stored_energy(self, extension: torch.Tensor | None = None) -> torch.Tensor:
        """Elastic energy of every pair's bond springs at its current extension:
        one spring (linear law) or the equilibrium spring plus each Maxwell
        branch stretched by its extension minus the branch's offset."""
        if extension is None:
            i, j = self.pairs.T
            extension = torch.linalg.vector_norm(self.positions[j] - self.positions[i], dim=1) - self.rest_lengths
        if self.bond_law is None:
            springs = [(float(self.config.bond_stiffness), None)]
        else:
            springs = [(float(self.bond_law.equilibrium_stiffness), None)]
            springs += [(float(k), self.branch_offsets[:, a]) for a, k in enumerate(self.bond_law.branch_stiffness)]
        energy = torch.zeros_like(extension)
        for k, offset in springs:
            stretch = extension if offset is None else extension - offset
            energy = energy + 0.5 * k * stretch.square()
        return energy

    @torch.no_grad()
    def bond_creep_reference_force(self) -> torch.Tensor:
        cfg = self.config
        thr = cfg.breaking_strain if self.bond_breaking_strain is None else self.bond_breaking_strain
        return cfg.bond_creep_force_fraction * self.unrelaxed_bond_stiffness * thr * self.rest_lengths

    def bond_law_report(self) -> dict[str, Any]:
        """The bond law's parameters and state: stiffnesses, creep, strength
        scatter and damage (the report of the reference's bonded-sphere model)."""
        cfg = self.config
        law = self.bond_law
        report: dict[str, Any] = dict(
            bond_model=cfg.bond_model,
            unrelaxed_stiffness_N_m=self.unrelaxed_bond_stiffness,
            relaxed_stiffness_N_m=float(cfg.bond_stiffness if law is None else law.equilibrium_stiffness),
            creep_exponent=float(cfg.bond_creep_exponent), creep_time_s=float(cfg.bond_creep_time_s),
            cumulative_bond_dissipation_J=self.cumulative_bond_dissipation_J,
            creep_failed_bonds=int((self.failure_mode == 4).sum()),
            strength_weibull_modulus=float(cfg.bond_strength_weibull_modulus),
            strength_weibull_seed=int(cfg.bond_strength_seed),
            max_bond_damage=float(self.bond_damage.max()) if len(self.bond_damage) else 0.0)
        strain = self.bond_breaking_strain
        if strain is not None:
            for name, value in (("median", strain.median()), ("min", strain.min()), ("max", strain.max())):
                report[f"bond_breaking_strain_{name}"] = float(value)
        if law is not None:
            report["branch_stiffness_N_m"] = list(map(float, law.branch_stiffness))
            report["relaxation_time_s"] = list(map(float, law.relaxation_time))
        return report

    @torch.no_grad()
    def lateral_platen_energy(self) -> float:
        cfg = self.config
        if not cfg.lateral_platens:
            return 0.0
        k = cfg.lateral_platen_stiffness if cfg.lateral_platen_stiffness is not None else cfg.platen_stiffness
        px, py = self.positions[:, 0], self.positions[:, 1]
        lp = self.lateral_platen_pos
        total = ((lp[0] - px + cfg.radius).clamp_min(0.0).square().sum()
                 + (px + cfg.radius - lp[1]).clamp_min(0.0).square().sum()
                 + (lp[2] - py + cfg.radius).clamp_min(0.0).square().sum()
                 + (py + cfg.radius - lp[3]).clamp_min(0.0).square().sum())
        return float(0.5 * k * total)

    def _tool_energy(self) -> float:
        cfg = self.config
        ov = (cfg.radius + cfg.tool_radius
              - torch.linalg.vector_norm(self.positions - self.tool_position, dim=1)).clamp_min(0)
        if cfg.contact_model == "hertz":
            return float(hertz_contact_potential(ov, *self._hertz_rigid_params).sum())
        return float((0.5 * cfg.contact_stiffness * ov.square()).sum())

    def _platen_energy(self) -> float:
        cfg = self.config
        total = 0.0
        z = self.positions[:, 2]
        for on, ov in ((cfg.top_platen_enabled,
                        lambda: (z + cfg.radius - (self.top_platen_start_z + self.time * cfg.top_platen_velocity))),
                       (cfg.bottom_platen_enabled,
                        lambda: (self.bottom_platen_start_z + self.time * cfg.bottom_platen_velocity
                                 + cfg.radius - z))):
            if not on:
                continue
            o = ov().clamp_min(0.0)
            total += (float(hertz_contact_potential(o, *self._hertz_rigid_params).sum())
                      if cfg.contact_model == "hertz" else float((0.5 * cfg.platen_stiffness * o.square()).sum()))
        return total

    def _contact_energy(self) -> float:
        """Contact potential of the current configuration (a side-effect-free kernel probe)."""
        _, _, led = self._evaluate(None, False, False)
        return float(led[_lib.L3_CONTACT_ENERGY])

    @torch.no_grad()
    def diagnostics(self, external_forces: torch.Tensor | None = None) -> dict[str, Any]:
        """Full diagnostic record (the keys of the reference's dem3d.py:1665-1738):
        clock and tool, reactions from a side-effect-free force probe, the
        stored energies (the probe's contact energy from the device ledger),
        the platen state and the body-force totals."""
        force, reaction = self.forces(external_forces, update_fracture=False, update_history=False)
        support = -force[self.fixed].sum(dim=0)
        parts = dict(kinetic_energy_J=float(0.5 * self.config.mass * self.velocities.square().sum()),
                     bond_elastic_energy_J=float((self.bond_stored_energy() * self.alive).sum()),
                     particle_contact_energy_J=float(self.read_ledger()[_lib.L3_CONTACT_ENERGY]),
                     tool_contact_energy_J=self._tool_energy(), platen_contact_energy_J=self._platen_energy())
        lateral = self.lateral_platen_energy()
        record: dict[str, Any] = {"time": self.time}
        record.update(zip(("tool_x", "tool_y", "tool_z"), map(float, self.tool_position)))
        record.update(zip(("reaction_x", "reaction_y", "reaction_z"), map(float, reaction)))
        record["top_platen_reaction_z_N"] = float(self.last_top_platen_reaction_z)
        record["bottom_platen_reaction_z_N"] = float(self.last_bottom_platen_reaction_z)
        record.update(zip(("boundary_reaction_x", "boundary_reaction_y", "boundary_reaction_z"), map(float, support)))
        record["broken_bonds"] = self.broken_bonds
        record["particle_count"] = len(self.positions)
        record.update(parts)
        record["released_bond_energy_J"] = float(self.failure_energy_J.sum())
        record["lateral_platen_reaction"] = [float(v) for v in self.last_lateral_platen_reaction]
        record["lateral_platen_energy_J"] = lateral
        record["mechanical_energy_J"] = sum(parts.values()) + lateral
        record.update(self.body_force_ledger())
        return record

    @torch.no_grad()
    def energy(self) -> dict[str, float]:
        """Mechanical energy components in J (dem3d.py:1740-1805)."""
        cfg = self.config
        kinetic = 0.5 * cfg.mass * float((self.velocities ** 2).sum())
        i, j = self.pairs.T
        extension = torch.linalg.vector_norm(self.positions[j] - self.positions[i], dim=1) - self.rest_lengths
        bond_energy = float(self.bond_stored_energy(extension)[self.alive].sum())
        contact_energy = self._contact_energy()
        tool_energy = self._tool_energy()
        platen_energy = self._platen_energy() + self.lateral_platen_energy()
        released = 0.5 * cfg.bond_stiffness * float((extension[~self.alive] ** 2).sum())
        return {
            "time_s": self.time, "step": self.step_count, "broken_bonds": self.broken_bonds,
            "particle_count": len(self.positions), "kinetic_energy_J": float(kinetic),
            "bond_elastic_energy_J": bond_energy, "particle_contact_energy_J": contact_energy,
            "tool_contact_energy_J": tool_energy, "platen_contact_energy_J": platen_energy,
            "released_bond_energy_J": released,
            "mechanical_energy_J": float(kinetic + bond_energy + contact_energy + tool_energy + platen_energy),
        }

    # ----------------------------------------------------------- restart
    def state_dict(self) -> dict[str, Any]:
        """Restart payload (dem3d.py:1828-1853)."""
        return {
            "dimension": 3, "config": asdict(self.config), "dt": self.dt,
            "time": self.time, "step_count": self.step_count,
            "positions": self.positions.clone(), "velocities": self.velocities.clone(),
            "initial_positions": self.initial_positions.clone(), "fixed": self.fixed.clone(),
            "pairs": self.pairs.clone(), "bonded": self.bonded.clone(), "alive": self.alive.clone(),
            "failure_mode": self.failure_mode.clone(), "failure_time_s": self.failure_time_s.clone(),
            "failure_extension_m": self.failure_extension_m.clone(), "failure_energy_J": self.failure_energy_J.clone(),
            "bond_law": {
                "branch_offsets": self.branch_offsets.clone(),
                "elongation_prev": self._bond_elongation_prev.clone(),
                "damage": self.bond_damage.clone(),
                "cumulative_bond_dissipation_J": self.cumulative_bond_dissipation_J,
            },
        }

    def _check_checkpoint_config(self, saved) -> None:
        """The checkpoint's configuration, completed with the defaults of
        fields added since, must equal this solver's (the device aside)."""
        if not isinstance(saved, dict):
            raise ValueError("checkpoint config must be a dictionary")
        mine = asdict(self.config)
        theirs = {**asdict(DEM3DConfig()), **saved}
        mine["device"] = theirs["device"] = "cuda"  # an execution choice, not physical state
        if {k: (tuple(v) if isinstance(v, list) else v) for k, v in theirs.items()} != mine:
            raise ValueError("checkpoint config does not match this solver configuration")

    def _checkpoint_tensor(self, name: str, value, target: torch.Tensor) -> torch.Tensor:
        if not isinstance(value, torch.Tensor) or tuple(value.shape) != tuple(target.shape):
            raise ValueError(f"checkpoint {name} must be a tensor with shape {tuple(target.shape)}")
        if value.dtype != target.dtype:
            raise ValueError(f"checkpoint {name} dtype must be {target.dtype}, got {value.dtype}")
        value = value.to(device=self.device)
        if value.is_floating_point() and not bool(torch.isfinite(value).all()):
            raise ValueError(f"checkpoint {name} contains non-finite values")
        return value

    @torch.no_grad()
    def load_state_dict(self, state: dict[str, Any]) -> None:
        """Restore a ``state_dict`` snapshot; every check runs before anything is
        written, so a rejected checkpoint leaves the solver unchanged (the
        restart rules of the reference's dem3d.py:1855-1967: same keys, same
        configuration and dt, tensors of the solver's shapes and dtypes, finite,
        the same lattice, pairs, bonds and supports, a bond-law state when the
        law is rate dependent)."""
        if not isinstance(state, dict):
            raise TypeError("state must be a dictionary returned by state_dict()")
        missing = _CHECKPOINT_KEYS.difference(state)
        if missing:
            raise ValueError(f"checkpoint is missing keys: {sorted(missing)}")
        if state["dimension"] != 3:
            raise ValueError("checkpoint dimension must be 3")
        self._check_checkpoint_config(state["config"])
        if not math.isfinite(float(state["dt"])) or float(state["dt"]) != self.dt:
            raise ValueError("checkpoint dt does not match this solver")
        time_value = float(state["time"])
        step_value = state["step_count"]
        if not math.isfinite(time_value) or time_value < 0:
            raise ValueError("checkpoint time must be finite and nonnegative")
        if isinstance(step_value, bool) or not isinstance(step_value, int) or step_value < 0:
            raise ValueError("checkpoint step_count must be a nonnegative integer")
        staged = {name: self._checkpoint_tensor(name, state[name], getattr(self, name))
                  for name in _CHECKPOINT_TENSORS}
        for name, message in _CHECKPOINT_FROZEN:
            if not torch.equal(staged[name], getattr(self, name)):
                raise ValueError(message)
        if bool((staged["alive"] & ~staged["bonded"]).any()):
            raise ValueError("checkpoint marks a non-bond pair as alive")
        bond_state = state.get("bond_law")
        if self.bond_law is not None:
            if not isinstance(bond_state, dict):
                raise ValueError("checkpoint has no bond-law state but the solver uses a rate-dependent bond")
            for key, shape in (("branch_offsets", tuple(self.branch_offsets.shape)), ("damage", (len(self.pairs),)),
                               ("elongation_prev", (len(self.pairs),))):
                v = bond_state.get(key)
                if not isinstance(v, torch.Tensor) or tuple(v.shape) != shape or v.dtype != self.dtype:
                    raise ValueError(f"checkpoint {key} must be a {self.dtype} tensor with shape {shape}")
                if not bool(torch.isfinite(v).all()):
                    raise ValueError("checkpoint bond-law state is non-finite")
        for name, value in staged.items():
            getattr(self, name).copy_(value)
        self._fixed_u8 = self.fixed.to(torch.uint8)
        if self.bond_law is not None:
            for attr, key in (("branch_offsets", "branch_offsets"), ("bond_damage", "damage"),
                              ("_bond_elongation_prev", "elongation_prev")):
                getattr(self, attr).copy_(bond_state[key].to(self.device))
            self.cumulative_bond_dissipation_J = float(bond_state.get("cumulative_bond_dissipation_J", 0.0))
        self.time = time_value
        self.step_count = step_value
        self.last_reaction.zero_()
