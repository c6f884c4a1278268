"""Known-answer tests pinning the FP64 Hertz-Mindlin oracle (oracle/hm2d.py).

Anchors restated from the reference's own tests: Hertz normal law
(tests/test_scale_ceiling_dem.py:114-127), Mindlin stiffness ratio
(tests/test_hertz_mindlin.py:40-70), restitution-to-damping anchors
(tests/test_contact_tangential.py:73-83), single-collision restitution
(tests/test_scale_ceiling_dem.py:130-144), elastic energy conservation and
free flight (:147-172), Coulomb cycle area
(src/tensordem/contact_tangential.py:215-256), brute-force pair sets (:41-50),
the Hertz contact duration of tests/test_dem3d_hertz_impact_time.py and the
second-order convergence of tests/test_dem3d_integration_order.py.
"""

import math

import numpy as np
import pytest

from oracle.hm2d import (HM2DOracle, HMParams, brute_force_pairs, effective_modulus,
                         effective_shear, tsuji_beta)
from tests._hm_cases import dense_gas, oracle_for, two_disc_state

E, NU = 70e9, 0.25


def _params(**kw):
    base = dict(young=E, poisson=NU, restitution=1.0, mu=0.0, mu_wall=0.0, dt=1e-8,
                gravity=(0.0, 0.0), box=None, skin=1e-4)
    base.update(kw)
    return HMParams(**base)


def test_hertz_normal_force_matches_analytic_law():
    st = two_disc_state(delta=2e-6)
    o = HM2DOracle(**st, params=_params())
    f, _, _ = o.evaluate(o.pos, o.vel, o.omega, advance=False)
    r_eff = 0.5e-3
    expected = (4.0 / 3.0) * effective_modulus(E, NU) * math.sqrt(r_eff) * (2e-6) ** 1.5
    assert abs(f[0, 0]) == pytest.approx(expected, rel=1e-12)
    assert f[0, 0] == -f[1, 0] and f[0, 1] == 0.0


@pytest.mark.parametrize("nu,ratio", [(0.3, 3 * 0.7 / 1.7), (0.25, 3 * 0.75 / 1.75), (0.0, 1.5)])
def test_mindlin_stiffness_ratio(nu, ratio):
    # k_t / k_n with k_n the secant (4/3) E* sqrt(R d) and k_t = 8 G* sqrt(R d)
    kt_over_kn = 8.0 * effective_shear(1e9, nu) / ((4.0 / 3.0) * effective_modulus(1e9, nu))
    assert kt_over_kn == pytest.approx(ratio, rel=1e-12)


@pytest.mark.parametrize("e,gamma", [(0.5, 13.626), (0.8, 4.481), (1.0, 0.0)])
def test_restitution_damping_anchor(e, gamma):
    assert 2.0 * tsuji_beta(e) * math.sqrt(1000.0 * 1.0) == pytest.approx(gamma, abs=0.01)


def test_restitution_of_a_single_collision():
    r = 1e-3
    st = two_disc_state(delta=-0.05e-3, r=r)
    st["vel"] = np.array([[2.0, 0.0], [-2.0, 0.0]])
    o = HM2DOracle(**st, params=_params(restitution=0.5, dt=1e-8))
    e0 = 0.5 * float(np.sum(o.mass * (o.vel**2).sum(1)))
    for _ in range(100):
        o.step(50)
        if o.vel[0, 0] < 0 and o.pos[1, 0] - o.pos[0, 0] > 2 * r:
            break
    e_eff = abs(o.vel[0, 0]) / 2.0
    assert 0.35 < e_eff < 0.75
    assert 0.5 * float(np.sum(o.mass * (o.vel**2).sum(1))) < e0


def test_elastic_gas_conserves_energy():
    cfg, st = dense_gas(16, seed=5, restitution=1.0, mu=0.0, gravity=(0.0, 0.0), walls=0)
    o = oracle_for(cfg, st)
    e0 = o.energies()["total"]
    o.step(300)
    led = o.energies()
    assert o.state.keys.size > 0 or led["elastic_normal"] >= 0.0
    assert abs(led["total"] - e0) / e0 < 2e-2


def test_free_flight_conserves_momentum_and_energy():
    rng = np.random.default_rng(6)
    n = 50
    pos = rng.uniform(0, 1.0, (n, 2)) * np.array([1.0, 0.02])
    pos[:, 0] = np.arange(n) * 0.01
    radius = np.full(n, 1e-3)
    mass = 2500 * math.pi * radius**2 * 2 * radius
    o = HM2DOracle(pos, rng.normal(0, 0.3, (n, 2)), np.zeros(n), radius, mass, 0.5 * mass * radius**2,
                   _params(dt=1e-6))
    p0 = (o.mass[:, None] * o.vel).sum(0)
    k0 = 0.5 * np.sum(o.mass * (o.vel**2).sum(1))
    o.step(100)
    assert np.allclose((o.mass[:, None] * o.vel).sum(0), p0, atol=1e-15, rtol=0)
    assert abs(0.5 * np.sum(o.mass * (o.vel**2).sum(1)) - k0) / k0 < 1e-14


def test_coulomb_cycle_dissipation_matches_closed_form():
    """Harmonic tangential drive at fixed overlap: W = 4 mu F_n (a - mu F_n / k_t)."""
    mu, delta, r = 0.3, 2e-6, 1e-3
    st = two_disc_state(delta=delta, r=r)
    p = _params(mu=mu, dt=1e-7)
    o = HM2DOracle(**st, params=p)
    r_eff = 0.5 * r
    sq = math.sqrt(r_eff * delta)
    f_n = (2.0 / 3.0) * 2.0 * p.estar * sq * delta
    k_t = 8.0 * p.gstar * sq
    amp = 5.0 * mu * f_n / k_t
    period = 4000 * p.dt
    w = 2 * math.pi / period
    dissipated = []
    for cycle in range(3):
        d0 = o.dissipated
        for k in range(4000):
            t = (cycle * 4000 + k) * p.dt
            vel = np.array([[0.0, amp * w * math.cos(w * t)], [0.0, 0.0]])
            _, _, d = o.evaluate(o.pos, vel, o.omega, advance=True)
            o.dissipated += d
        dissipated.append(o.dissipated - d0)
    expected = 4.0 * mu * f_n * (amp - mu * f_n / k_t)
    assert dissipated[-1] == pytest.approx(expected, rel=2e-3)


def test_kdtree_candidates_equal_brute_force():
    rng = np.random.default_rng(0)
    n = 5000
    pos = rng.uniform(0, 0.2, (n, 2))
    radius = rng.uniform(0.8e-3, 1.2e-3, n)
    mass = 2500 * math.pi * radius**3 * 2
    o = HM2DOracle(pos, np.zeros((n, 2)), np.zeros(n), radius, mass, 0.5 * mass * radius**2,
                   _params(skin=1e-3))
    i, j = o.candidate_pairs()
    bi, bj = brute_force_pairs(pos, 0.0, radius, skin=1e-3)
    assert set(zip(i.tolist(), j.tolist())) == set(zip(bi.tolist(), bj.tolist()))
    assert len(bi) > 100


def test_frictionless_walls_give_no_tangential_force():
    cfg, st = dense_gas(12, seed=2, mu=0.0)
    cfg = type(cfg)(**{**cfg.__dict__, "mu_wall": 0.0})
    o = oracle_for(cfg, st)
    o.step(200)
    assert np.all(o.wall_xi == 0.0)


def _head_on_collision(v0, r=1e-3, steps_per_contact=2000):
    """Two equal discs meeting head-on at relative speed v0 (no damping, no
    friction): the contact duration from the overlap's zero crossings, the
    Johnson closed form t_c = C (5 m* / (4 k_h))^(2/5) v0^(-1/5) with
    k_h = (4/3) E* sqrt(R*) and C = (4/5) B(2/5, 1/2) (the reference's
    tests/test_dem3d_hertz_impact_time.py), and the rebound ratio."""
    st = two_disc_state(delta=-1e-9, r=r)
    mstar, rstar = 0.5 * st["mass"][0], 0.5 * r
    k_h = (4.0 / 3.0) * effective_modulus(E, NU) * math.sqrt(rstar)
    c = 0.8 * math.gamma(0.4) * math.gamma(0.5) / math.gamma(0.9)
    t_c = c * (5.0 * mstar / (4.0 * k_h)) ** 0.4 * v0 ** -0.2
    st["vel"] = np.array([[0.5 * v0, 0.0], [-0.5 * v0, 0.0]])
    o = HM2DOracle(**st, params=_params(dt=t_c / steps_per_contact))
    overlap = [2.0 * r - (o.pos[1, 0] - o.pos[0, 0])]
    while not (overlap[-1] < 0.0 < max(overlap)) and len(overlap) < 3 * steps_per_contact:
        o.step(1)
        overlap.append(2.0 * r - (o.pos[1, 0] - o.pos[0, 0]))
    d = np.asarray(overlap)
    inside = np.flatnonzero(d > 0.0)
    a, b = inside[0], inside[-1]
    t_in = (a - 1) + d[a - 1] / (d[a - 1] - d[a])
    t_out = b + d[b] / (d[b] - d[b + 1])
    return (t_out - t_in) * o.p.dt, t_c, -o.vel[0, 0] / (0.5 * v0)


def test_hertz_contact_duration_matches_the_johnson_closed_form():
    """The trajectory-level Hertz check: duration within 1e-5 of the closed
    form (measured 1.3e-7 at 2,000 steps per contact), the v0^(-1/5) law
    to 1e-6 in the exponent over 0.1-3 m/s, and an elastic rebound."""
    speeds = (0.1, 0.3, 1.0, 3.0)
    runs = [_head_on_collision(v) for v in speeds]
    for t, t_c, rebound in runs:
        assert t == pytest.approx(t_c, rel=1e-5)
        assert rebound == pytest.approx(1.0, abs=1e-7)
    slope = np.polyfit(np.log(speeds), np.log([t for t, _, _ in runs]), 1)[0]
    assert slope == pytest.approx(-0.2, abs=1e-6)


def test_velocity_verlet_is_second_order_through_a_hertz_contact():
    """The integration-order check of the reference's 3-D suite
    (tests/test_dem3d_integration_order.py) on the oracle's 2-D step: halving
    dt quarters the position and velocity errors at a fixed time inside a
    head-on Hertz contact (reference: 64,000 steps per contact time)."""
    r, v0 = 1e-3, 1.0
    st0 = two_disc_state(delta=2e-6, r=r)
    mstar, rstar = 0.5 * st0["mass"][0], 0.5 * r
    k_h = (4.0 / 3.0) * effective_modulus(E, NU) * math.sqrt(rstar)
    t_c = 2.9432751843247047 * (5.0 * mstar / (4.0 * k_h)) ** 0.4 * v0 ** -0.2

    def state_at(per_contact):
        st = dict(st0, vel=np.array([[0.5 * v0, 0.0], [-0.5 * v0, 0.0]]))
        o = HM2DOracle(**st, params=_params(dt=t_c / per_contact))
        o.step(int(round(0.3 * per_contact)))  # the same end time 0.3 t_c for every dt
        return o.pos[1, 0] - o.pos[0, 0], o.vel[0, 0]

    ref = state_at(64000)
    runs = [state_at(n) for n in (500, 1000, 2000, 4000)]
    for k in (0, 1):
        err = [abs(s[k] - ref[k]) for s in runs]
        ratios = [err[i] / err[i + 1] for i in range(3)]
        assert all(3.9 < q < 4.1 for q in ratios), (k, ratios)
