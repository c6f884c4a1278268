"""Unit checks of the FP64 oracle's per-contact Hertz-Mindlin law
(oracle/hm2d.py, ``contact_law``), restated from the reference's own unit
tests of its contact pieces:

* Mindlin stick and Coulomb slip, and the history projected back onto the
  friction cone after slip (tests/test_hertz_mindlin.py:106-180);
* zero friction, saturation and the sub-limit spring
  (tests/test_contact_tangential.py:89-125);
* the tangential history integration: no growth under a purely normal
  relative velocity, full growth under a tangential one, increments on a
  stored history (tests/test_contact_tangential.py:129-158);
* the stiffness ratio at any overlap and zero stiffness at zero overlap
  (tests/test_hertz_mindlin.py:64-80, 234-250);
* the restitution-to-damping map: zero at e = 1, monotonic, invertible,
  invalid e rejected (tests/test_contact_tangential.py:19-70).

The reference's functions work on 3-D or separate normal / tangential
pieces; here they are checked through the one 2-D law the engines and the
oracle share, with the Tsuji dashpot off (e = 1) wherever the normal force
has to be known exactly.
"""

import math

import numpy as np
import pytest

from oracle.hm2d import HMParams, contact_law, effective_modulus, effective_shear, tsuji_beta

E, NU = 1e9, 0.3
R = 0.01


def _params(mu=0.5, restitution=1.0, dt=1e-3):
    return HMParams(young=E, poisson=NU, restitution=restitution, mu=mu, mu_wall=0.0, dt=dt,
                    gravity=(0.0, 0.0), box=None)


def _one(p, delta, xi=(0.0, 0.0), vel_a=(0.0, 0.0), vel_b=(0.0, 0.0), om=(0.0, 0.0), n=(1.0, 0.0)):
    """One contact between two discs of radius R and unit mass, normal n from a to b."""
    a = lambda v: np.array([v], dtype=np.float64)
    return contact_law(p, a(delta)[0:1], a(n), a(R)[0:1], a(R)[0:1], a(1.0)[0:1], a(1.0)[0:1], a(vel_a),
                       a(vel_b), a(om[0])[0:1], a(om[1])[0:1], a(xi))


def _stiffness(delta):
    reff = 0.5 * R
    s_n = 2.0 * effective_modulus(E, NU) * math.sqrt(reff * delta)
    s_t = 8.0 * effective_shear(E, NU) * math.sqrt(reff * delta)
    return s_n, s_t


def test_stick_below_coulomb_limit_is_the_mindlin_spring():
    delta = 1e-4
    p = _params(mu=0.5)
    out = _one(p, delta, xi=(0.0, 1e-6))
    _, s_t = _stiffness(delta)
    assert not out["sliding"][0]
    assert out["s_t"][0] == pytest.approx(s_t, rel=1e-14)
    # force on a: -F_n n - s_t xi; its tangential part is the spring
    assert out["f_a"][0, 1] == pytest.approx(-s_t * 1e-6, rel=1e-12)
    assert abs(out["f_a"][0, 1]) < p.mu * out["f_n"][0]
    assert out["xi"][0, 1] == pytest.approx(1e-6, rel=1e-14)


def test_slip_saturates_at_the_coulomb_limit():
    delta = 1e-4
    p = _params(mu=0.3)
    out = _one(p, delta, xi=(0.0, 0.1))
    assert out["sliding"][0]
    assert abs(out["f_a"][0, 1]) == pytest.approx(p.mu * out["f_n"][0], rel=1e-12)


def test_history_is_projected_onto_the_friction_cone_after_slip():
    delta = 1e-4
    p = _params(mu=0.3)
    out = _one(p, delta, xi=(0.0, 0.1))
    _, s_t = _stiffness(delta)
    xi = out["xi"][0]
    # the stored history is the saturated force over the stiffness, same direction
    assert s_t * np.hypot(*xi) == pytest.approx(p.mu * out["f_n"][0], rel=1e-12)
    assert xi[0] == 0.0 and xi[1] > 0.0
    assert out["f_a"][0, 1] == pytest.approx(-s_t * xi[1], rel=1e-12)
    assert out["slip_loss"] > 0.0


def test_zero_friction_gives_no_tangential_force():
    p = _params(mu=0.0)
    out = _one(p, 1e-4, xi=(0.0, 1.0))
    assert out["f_a"][0, 1] == 0.0
    assert np.all(out["xi"][0] == 0.0)
    assert out["f_a"][0, 0] < 0.0  # the normal force remains


def test_sub_limit_tangential_force_is_linear_in_the_history():
    delta = 1e-4
    p = _params(mu=0.5)
    _, s_t = _stiffness(delta)
    f1 = _one(p, delta, xi=(0.0, 1e-7))["f_a"][0, 1]
    f2 = _one(p, delta, xi=(0.0, 2e-7))["f_a"][0, 1]
    assert f2 == pytest.approx(2.0 * f1, rel=1e-12)
    assert f1 == pytest.approx(-s_t * 1e-7, rel=1e-12)


def test_purely_normal_relative_velocity_leaves_no_tangential_history():
    p = _params(mu=0.5, dt=0.01)
    out = _one(p, 1e-4, vel_a=(1.0, 0.0))
    assert np.all(out["xi"][0] == 0.0)


def test_purely_tangential_relative_velocity_accumulates_in_full():
    dt = 0.01
    p = _params(mu=1e9, dt=dt)  # no slip
    out = _one(p, 1e-4, vel_a=(0.0, 1.0))
    assert out["xi"][0, 0] == 0.0
    assert out["xi"][0, 1] == pytest.approx(1.0 * dt, rel=1e-15)


def test_spin_counts_as_tangential_velocity_of_the_contact_points():
    dt = 0.01
    p = _params(mu=1e9, dt=dt)
    # omega_a r_a + omega_b r_b along t = (-n_y, n_x) = (0, 1)
    out = _one(p, 1e-4, om=(30.0, 20.0))
    assert out["xi"][0, 1] == pytest.approx((30.0 + 20.0) * R * dt, rel=1e-14)


def test_stored_history_is_incremented():
    dt = 0.01
    p = _params(mu=1e9, dt=dt)
    out = _one(p, 1e-4, xi=(0.0, 0.05), vel_a=(0.0, 2.0))
    assert out["xi"][0, 1] == pytest.approx(0.05 + 2.0 * dt, rel=1e-15)


@pytest.mark.parametrize("delta", [1e-8, 1e-6, 1e-4, 1e-3])
def test_stiffness_ratio_does_not_depend_on_the_overlap(delta):
    out = _one(_params(), delta)
    s_n = 1.5 * out["f_el"][0] / delta  # f_el = (2/3) s_n delta
    assert out["s_t"][0] / s_n == pytest.approx(2.0 * (1.0 - NU) / (2.0 - NU), rel=1e-12)


def test_zero_overlap_gives_zero_stiffness_and_force():
    out = _one(_params(restitution=0.5), 0.0, vel_a=(-1.0, 0.3))
    assert out["s_t"][0] == 0.0
    assert out["f_n"][0] == 0.0
    assert np.all(out["f_a"][0] == 0.0)


def test_restitution_map_is_zero_at_one_monotonic_and_invertible():
    assert tsuji_beta(1.0) == 0.0
    es = np.linspace(0.05, 0.999, 60)
    betas = np.array([tsuji_beta(float(e)) for e in es])
    assert np.all(np.diff(betas) < 0.0)
    assert np.all((betas > 0.0) & (betas < 1.0))
    back = np.exp(-math.pi * betas / np.sqrt(1.0 - betas**2))
    assert np.allclose(back, es, rtol=1e-12, atol=0.0)


@pytest.mark.parametrize("e", [0.0, -0.5])
def test_invalid_restitution_is_rejected(e):
    with pytest.raises(ValueError):
        tsuji_beta(e)


def test_normal_dashpot_adds_the_viscous_term_while_approaching_and_clamps_at_zero():
    """The reference's dashpot convention (tests/test_contact_mindlin_history.py:148-156):
    F_n = max(F_el + gamma sqrt(S_n m*) v_n, 0) with v_n > 0 while approaching."""
    delta = 1e-4
    p = _params(restitution=0.5)
    s_n, _ = _stiffness(delta)
    meff = 0.5
    approach = _one(p, delta, vel_a=(0.2, 0.0))
    expect = approach["f_el"][0] + p.damp * math.sqrt(s_n * meff) * 0.2
    assert approach["f_n"][0] == pytest.approx(expect, rel=1e-12)
    assert approach["dashpot_loss"] > 0.0
    fast_out = _one(p, delta, vel_a=(-1e3, 0.0))  # separating fast: the dashpot would pull
    assert fast_out["f_n"][0] == 0.0


def test_separated_pairs_forget_their_history():
    """A contact that opens drops its tangential history; when the two discs
    touch again the history starts from zero (the reference's
    tests/test_contact_mindlin_history.py:133-146, inactive contacts forget)."""
    from oracle.hm2d import HM2DOracle
    r = np.full(2, R)
    m = np.ones(2)
    inertia = 0.5 * m * r * r
    p = _params(mu=10.0, dt=1e-3)  # sticks: 320 N of spring against a 518 N cap
    o = HM2DOracle(np.array([[0.0, 0.0], [2 * R - 1e-4, 0.0]]), np.zeros((2, 2)), np.zeros(2), r, m, inertia, p)
    touching = o.pos.copy()
    moving = np.array([[0.0, 0.5], [0.0, 0.0]])  # tangential sliding of disc 0
    o.evaluate(touching, moving, np.zeros(2), advance=True)
    assert len(o.state.keys) == 1 and abs(o.state.xi[0, 1]) > 0.0
    apart = np.array([[0.0, 0.0], [2 * R + 1e-4, 0.0]])
    o.evaluate(apart, np.zeros((2, 2)), np.zeros(2), advance=True)
    assert len(o.state.keys) == 0
    force, torque, _ = o.evaluate(touching, np.zeros((2, 2)), np.zeros(2), advance=False)
    assert force[0, 1] == 0.0 and force[1, 1] == 0.0 and np.all(torque == 0.0)


def test_disc_launched_on_a_frictional_floor_leaves_rolling_at_two_thirds():
    """The reference's analytic sliding-disc anchor
    (tests/test_granular2d_column_collapse.py:55-79): a uniform disc launched
    at v0 on a floor with friction spins up and leaves rolling without slip
    at 2 v0 / 3; the friction work is m v0^2 / 6, and the ledger closes on
    it. Here with the oracle's Hertz floor and Mindlin spring (no dashpot),
    the disc starting at its static overlap."""
    from oracle.hm2d import HM2DOracle, rayleigh_dt
    r, rho, young, nu, g, mu, v0 = 0.01, 1000.0, 1e7, 0.3, 9.81, 0.3, 0.5
    m = rho * math.pi * r * r
    inertia = 0.5 * m * r * r
    overlap = (3.0 * m * g / (4.0 * effective_modulus(young, nu) * math.sqrt(r))) ** (2.0 / 3.0)
    dt = 0.05 * rayleigh_dt(r, rho, young, nu)
    p = HMParams(young=young, poisson=nu, restitution=1.0, mu=0.0, mu_wall=mu, dt=dt, gravity=(0.0, -g),
                 box=(1.0, 0.2), walls=(True, False, True, False), skin=0.1 * r)
    o = HM2DOracle(np.array([[0.1, r - overlap]]), np.array([[v0, 0.0]]), np.zeros(1), np.array([r]),
                   np.array([m]), np.array([inertia]), p)
    e0 = o.energies()
    o.step(int(1.3 * v0 / (3.0 * mu * g) / dt))  # 30% past the analytic end of slip
    e1 = o.energies()
    analytic = m * v0 * v0 / 6.0
    assert o.vel[0, 0] == pytest.approx(2.0 * v0 / 3.0, rel=0.01)
    assert abs(o.vel[0, 0] + o.omega[0] * r) < 0.01 * v0  # rolling, up to the spring's micro-slip
    assert o.dissipated == pytest.approx(analytic, rel=0.01)
    stored = lambda e: e["kinetic"] + e["potential"] + e["elastic_normal"] + e["elastic_tangential"]
    assert abs(stored(e0) - stored(e1) - o.dissipated) < 1e-3 * analytic
