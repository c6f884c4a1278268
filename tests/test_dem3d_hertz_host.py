"""The reference's 3-D Hertz-law and Hertz-configuration checks (its
tests/test_dem3d_hertz_contact.py:47-146) on the host side of
``tensordem_gb300.dem3d``: the public Hertz helpers against the classical
two-body relations written independently here,

    1/E* = sum (1 - nu_i^2) / E_i,   1/R* = sum 1 / R_i,
    F = (4/3) E* sqrt(R*) delta^(3/2),   U = (8/15) E* sqrt(R*) delta^(5/2),

and the contact-model validation and time-step bounds of ``DEM3DConfig``."""

import math
from dataclasses import replace

import pytest
import torch

from tensordem_gb300.dem3d import (DEM3DConfig, hertz_contact_potential, hertz_effective_radius,
                                   hertz_equivalent_linear_stiffness, hertz_normal_force, hertz_reduced_modulus,
                                   hertz_secant_stiffness)

E_YOUNG = 1.0e9
NU = 0.3
RADIUS = 0.025


def _sphere_sphere(overlap):
    e_eff = 1.0 / (2.0 * (1.0 - NU ** 2) / E_YOUNG)
    r_eff = 1.0 / (1.0 / RADIUS + 1.0 / RADIUS)
    return (4.0 / 3.0) * e_eff * math.sqrt(r_eff) * overlap ** 1.5


def _rigid_plane(overlap):
    e_eff = 1.0 / ((1.0 - NU ** 2) / E_YOUNG)
    return (4.0 / 3.0) * e_eff * math.sqrt(RADIUS) * overlap ** 1.5


def test_force_matches_the_closed_form():
    for overlap in (1e-6, 1e-4, 1e-3, 1e-2):
        f = float(hertz_normal_force(torch.tensor(overlap, dtype=torch.float64), hertz_reduced_modulus(E_YOUNG, NU),
                                     hertz_effective_radius(RADIUS)))
        assert abs(f / _sphere_sphere(overlap) - 1.0) < 1e-12
        rigid = float(hertz_normal_force(torch.tensor(overlap, dtype=torch.float64),
                                         hertz_reduced_modulus(E_YOUNG, NU, rigid_counterpart=True),
                                         hertz_effective_radius(RADIUS, rigid_counterpart=True)))
        assert abs(rigid / _rigid_plane(overlap) - 1.0) < 1e-12


def test_reduced_modulus_and_effective_radius():
    assert hertz_reduced_modulus(E_YOUNG, NU) == pytest.approx(E_YOUNG / (2.0 * (1.0 - NU ** 2)), abs=5e-7)
    assert hertz_reduced_modulus(E_YOUNG, NU, rigid_counterpart=True) == pytest.approx(E_YOUNG / (1.0 - NU ** 2),
                                                                                       abs=5e-7)
    assert hertz_effective_radius(RADIUS) == pytest.approx(0.5 * RADIUS, abs=5e-8)
    assert hertz_effective_radius(RADIUS, rigid_counterpart=True) == pytest.approx(RADIUS, abs=5e-8)


def test_force_exponent_is_three_halves():
    deltas = torch.logspace(-6, -2, 33, dtype=torch.float64)
    forces = hertz_normal_force(deltas, hertz_reduced_modulus(E_YOUNG, NU), hertz_effective_radius(RADIUS))
    slope = float((torch.log(forces).diff() / torch.log(deltas).diff()).mean())
    assert abs(slope - 1.5) < 5e-11


def test_potential_is_the_force_integral():
    e_star, r_eff = hertz_reduced_modulus(E_YOUNG, NU), hertz_effective_radius(RADIUS)
    delta, intervals = 2e-3, 20000
    h = delta / intervals
    total = 0.0
    for i in range(intervals):
        total += 0.5 * (float(hertz_normal_force(i * h, e_star, r_eff))
                        + float(hertz_normal_force((i + 1) * h, e_star, r_eff))) * h
    assert abs(float(hertz_contact_potential(delta, e_star, r_eff)) / total - 1.0) < 1e-9


def test_secant_and_equivalent_linear_stiffness():
    e_star, r_eff, delta = hertz_reduced_modulus(E_YOUNG, NU), hertz_effective_radius(RADIUS), 1e-3
    assert float(hertz_secant_stiffness(delta, e_star, r_eff)) == pytest.approx(
        float(hertz_normal_force(delta, e_star, r_eff)) / delta, abs=5e-7)
    k = hertz_equivalent_linear_stiffness(E_YOUNG, NU, RADIUS, 5e-4, rigid_counterpart=True)
    assert k * 5e-4 == pytest.approx(_rigid_plane(5e-4), abs=5e-7)


def test_negative_overlap_gives_no_force_or_energy():
    e_star, r_eff = hertz_reduced_modulus(E_YOUNG, NU), hertz_effective_radius(RADIUS)
    assert float(hertz_normal_force(-1e-4, e_star, r_eff)) == 0.0
    assert float(hertz_contact_potential(-1e-4, e_star, r_eff)) == 0.0


def test_default_model_and_validation():
    assert DEM3DConfig().contact_model == "linear"
    assert DEM3DConfig().recommended_dt > 0.0
    with pytest.raises(ValueError):
        DEM3DConfig(contact_model="mindlin")
    for kwargs in ({"poisson_ratio": 0.5}, {"poisson_ratio": -0.1}, {"young_modulus": 0.0},
                   {"young_modulus": float("nan")}, {"hertz_stability_overlap_fraction": 0.0},
                   {"hertz_stability_overlap_fraction": 1.5}):
        with pytest.raises(ValueError):
            DEM3DConfig(contact_model="hertz", **kwargs)


def test_hertz_bound_is_stiffer_than_the_linear_bound():
    linear = DEM3DConfig()
    hertz = DEM3DConfig(contact_model="hertz", young_modulus=E_YOUNG, poisson_ratio=NU)
    assert hertz.recommended_dt < linear.recommended_dt
    assert hertz._bound_stiffness(5_000.0, rigid_counterpart=False) > 5_000.0


@pytest.mark.gpu
def test_step_guard_rejects_a_step_above_the_bound():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300.dem3d import IceDEM3D
    base = DEM3DConfig(nx=3, ny=3, nz=3, contact_model="hertz", young_modulus=E_YOUNG, poisson_ratio=NU)
    with pytest.raises(ValueError, match="dt exceeds"):
        IceDEM3D(replace(base, dt=2.0 * base.recommended_dt))


def test_pair_damping_mode_contract():
    """The reference's tests/test_dem3d_pair_contact_damping.py:82-101: the
    restitution mapping stays the default dashpot convention, unknown modes
    and two conventions at once are refused, and the absolute mode takes any
    non-negative damping."""
    assert DEM3DConfig().contact_damping_model == "restitution"
    with pytest.raises(ValueError):
        DEM3DConfig(contact_damping_model="viscous")
    with pytest.raises(ValueError):
        DEM3DConfig(contact_damping_model="absolute", restitution_coefficient=0.5)
    for damping in (0.0, 5.0, 40.0):
        assert DEM3DConfig(contact_damping_model="absolute", contact_damping=damping).contact_damping_model == \
            "absolute"
