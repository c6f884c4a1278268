"""Ledger known-answer cases of the reference's 2-D bonded-disc engine,
written once for any backend with the ``IceDEM`` surface: the CUDA drop-in
(``tensordem_gb300.IceDEM``) or the numpy oracle (``oracle.icedem``).

Restated from the reference's
* tests/test_accounting_ledger_validation.py:31-157 - momentum balance of the
  impulse channels, the pair-contact energy a broken overlapping bond keeps,
  and closure of the energy ledger (bookkeeping, not time-step error);
* scripts/verify_dem2d_fracture_ledger.py:48-200, as exercised by
  tests/test_dem2d_fracture_ledger.py:57-94 - a controlled single-bond break
  against 0.5 k xi^2, the k xi^2 scaling of the channel, every break event of
  an indentation re-scored from the pre-step geometry, and a sub-threshold
  negative control;
* scripts/verify_dem2d_energy_ledger.py:82-262, as exercised by
  tests/test_dem2d_energy_ledger.py:71-146 - a free particle's viscous decay
  v0 exp(-t/tau) and its dissipation 0.5 m v0^2 (1 - exp(-2t/tau)) with the
  predicted first-order bookkeeping residual, a bonded harmonic oscillator
  A cos(omega t) with omega = sqrt(2k/m), and the tool-work residual under
  time-step refinement;
* tests/test_dem2d_energy_fracture_ledger_negative.py:56-533 - the energy
  balance gate closes on a clean indentation and rejects a run in which one
  ledger channel is zeroed, tripled or (for the dormant external-work channel)
  offset by the tool work, while a sign flip of a dormant channel is vacuous.

The inputs and bounds are the reference's own.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any, Callable

import numpy as np

INDENT_LATTICE = (7, 3)
INDENT_SECONDS = 0.12
R = 0.025
L0 = 2.0 * R
EPS_B = 0.015
IMPULSE_KEYS = ("external_impulse_Ns", "support_impulse_Ns", "drag_impulse_Ns", "tool_impulse_on_ice_Ns")


@dataclass
class Backend:
    """make(**config) builds a simulation; arr() reads one of its arrays as
    numpy; put(sim, x) turns a numpy array into the backend's array type."""

    name: str
    make: Callable[..., Any]
    arr: Callable[[Any], np.ndarray]
    put: Callable[[Any, np.ndarray], Any]


def indentation(b: Backend, dt_scale: float = 1.0, seconds: float = INDENT_SECONDS) -> dict:
    """A 7x3 strip indented at 0.2 m/s; the terms of the energy identity."""
    nx, ny = INDENT_LATTICE
    dt0 = b.make(nx=nx, ny=ny, tool_speed=0.2).dt
    sim = b.make(nx=nx, ny=ny, tool_speed=0.2, dt=dt0 * dt_scale)
    e0 = sim.mechanical_energy()["mechanical_J"]
    steps = int(round(seconds / sim.dt))
    for _ in range(steps):
        sim.step()
    e1 = sim.mechanical_energy()["mechanical_J"]
    acc = dict(sim.accounting)
    # dE_mech = W_ext + W_tool - Q_damping - E_fracture (+ E_acquired)
    raw = (e1 - e0) - acc["tool_work_J"] - acc["external_work_J"] + acc["damping_dissipation_J"] \
        + acc["fracture_release_J"]
    scale = abs(acc["tool_work_J"]) + abs(acc["damping_dissipation_J"]) + abs(e1 - e0)
    return dict(sim=sim, steps=steps, accounting=acc, raw=raw, closed=raw - acc["pair_contact_acquired_J"],
                scale=scale, e0=e0, e_end=e1)


def momentum_gap(b: Backend, sim) -> tuple[float, float]:
    """(max |m sum v - sum of impulse channels|, max of the two magnitudes)."""
    momentum = sim.config.mass * b.arr(sim.velocities).sum(axis=0)
    ledger = sum(np.asarray(sim.accounting[k], dtype=np.float64) for k in IMPULSE_KEYS)
    return float(np.abs(momentum - ledger).max()), max(float(np.abs(momentum).max()), float(np.abs(ledger).max()))


def uniform_load_momentum(b: Backend) -> tuple[float, float]:
    """A 3x3 lattice under a uniform 1 mN nodal load, no damping, tool far away."""
    sim = b.make(nx=3, ny=3, tool_gap=10.0, tool_speed=1e-9, drag=0.0, contact_damping=0.0)
    load = np.zeros(b.arr(sim.positions).shape)
    load[:, 1] = 1e-3
    load = b.put(sim, load)
    for _ in range(40):
        sim.step(external_forces=load)
    momentum = sim.config.mass * b.arr(sim.velocities).sum(axis=0)
    return momentum_gap(b, sim)[0], float(np.abs(momentum).max())


def drag_tool_support_momentum(b: Backend) -> dict:
    nx, ny = INDENT_LATTICE
    sim = b.make(nx=nx, ny=ny, tool_speed=0.2, drag=0.5, contact_damping=5.0)
    for _ in range(int(round(INDENT_SECONDS / sim.dt))):
        sim.step()
    gap, ref = momentum_gap(b, sim)
    return dict(gap=gap, ref=ref, drag_y=sim.accounting["drag_impulse_Ns"][1],
                tool_y=sim.accounting["tool_impulse_on_ice_Ns"][1])


def retained_contact_energy(b: Backend, run: dict) -> tuple[float, float]:
    """(analytic 0.5 k_c overlap^2 over broken pairs, the credited channel).

    A broken pair with recorded failure extension e and rest length L starts
    as a contact with overlap (2r - (L + e))+."""
    sim = run["sim"]
    r = sim.config.radius
    overlap = np.maximum(2.0 * r - (b.arr(sim.rest_lengths) + b.arr(sim.failure_extension_m)), 0.0)
    broken = b.arr(sim.failure_energy_J) > 0.0
    analytic = float((0.5 * sim.config.contact_stiffness * overlap[broken] ** 2).sum())
    return analytic, run["accounting"]["pair_contact_acquired_J"]


def _pair_index(b: Backend, sim, i: int, j: int) -> int:
    pairs = b.arr(sim.pairs)
    return int(np.flatnonzero((pairs[:, 0] == i) & (pairs[:, 1] == j))[0])


def single_bond(b: Backend, k: float, xi0: float):
    """2x2 lattice with only the axial bond 0-1 alive, pre-stretched by xi0;
    no damping, tool parked 1 m above at 1e-6 m/s (no contact)."""
    sim = b.make(nx=2, ny=2, radius=R, bond_stiffness=k, contact_stiffness=2000.0, breaking_strain=EPS_B,
                 shear_breaking_strain=0.03, contact_damping=0.0, drag=0.0, tool_speed=1e-6, tool_gap=1.0,
                 fix_edges=False)
    alive = np.zeros(len(b.arr(sim.pairs)), dtype=bool)
    alive[_pair_index(b, sim, 0, 1)] = True
    sim.alive = b.put(sim, alive)
    pos = b.arr(sim.initial_positions).copy()
    pos[1, 0] += xi0
    sim.positions = b.put(sim, pos)
    sim.velocities = b.put(sim, np.zeros_like(pos))
    return sim


def controlled_break(b: Backend, k: float = 2000.0, xi0: float | None = None) -> dict:
    if xi0 is None:
        xi0 = L0 * (EPS_B + 1e-4)
    sim = single_bond(b, k, xi0)
    m = sim.config.mass
    u0 = sim.mechanical_energy()["mechanical_J"]
    ke0 = 0.5 * m * float((b.arr(sim.velocities) ** 2).sum())
    sim.step()
    u1 = sim.mechanical_energy()["mechanical_J"]
    ke1 = 0.5 * m * float((b.arr(sim.velocities) ** 2).sum())
    released = sim.accounting["fracture_release_J"]
    acquired = sim.accounting["pair_contact_acquired_J"]
    closed = 0.5 * k * xi0 ** 2
    p01 = _pair_index(b, sim, 0, 1)
    return dict(xi0=xi0, broken=bool(b.arr(sim.failure_mode)[p01] != 0), released=released, closed=closed,
                rel_err=abs(released - closed) / closed, acquired=acquired,
                extension=float(b.arr(sim.failure_extension_m)[p01]),
                # the reference's single-step identity, term for term
                residual=(u1 + ke1 - u0 - ke0) + released - acquired)


def scaling_rows(b: Backend) -> list[dict]:
    rows = []
    for k in (2000.0, 4000.0):
        for xi0 in (0.0008, 0.0016):
            row = controlled_break(b, k, xi0)
            row["ratio"] = (k / 2000.0) * (xi0 / 0.0008) ** 2
            rows.append(row)
    return rows


def indentation_events(b: Backend) -> dict:
    """Every break of the 7x3 indentation re-scored from the positions before
    its step (the break test sees the pre-step geometry)."""
    nx, ny = INDENT_LATTICE
    sim = b.make(nx=nx, ny=ny, tool_speed=0.2)
    r, k, kc = sim.config.radius, sim.config.bond_stiffness, sim.config.contact_stiffness
    pairs = b.arr(sim.pairs)
    bonded = b.arr(sim.bonded)
    rest = b.arr(sim.rest_lengths)
    seen: set[int] = set()
    events = []
    for _ in range(int(round(INDENT_SECONDS / sim.dt))):
        pre = b.arr(sim.positions).copy()
        sim.step()
        gone = np.flatnonzero(bonded & ~b.arr(sim.alive))
        fresh = [int(p) for p in gone if int(p) not in seen]
        if not fresh:
            continue
        energy = b.arr(sim.failure_energy_J)
        for p in fresh:
            seen.add(p)
            d = float(np.hypot(*(pre[pairs[p, 1]] - pre[pairs[p, 0]])))
            events.append(dict(overlap=max(0.0, 2.0 * r - d), released=0.5 * k * (d - rest[p]) ** 2,
                               acquired=0.5 * kc * max(0.0, 2.0 * r - d) ** 2, recorded=float(energy[p])))
    acc = sim.accounting
    tot_rel = sum(e["released"] for e in events)
    tot_acq = sum(e["acquired"] for e in events)
    return dict(events=events, n_overlap=sum(e["overlap"] > 0.0 for e in events),
                rel_err_released=abs(acc["fracture_release_J"] - tot_rel) / tot_rel if tot_rel else 0.0,
                rel_err_acquired=abs(acc["pair_contact_acquired_J"] - tot_acq) / tot_acq if tot_acq else 0.0)


def subthreshold(b: Backend) -> dict:
    sim = single_bond(b, 2000.0, 0.99 * L0 * EPS_B)
    for _ in range(50):
        sim.step()
    return dict(alive=bool(b.arr(sim.alive)[_pair_index(b, sim, 0, 1)]),
                released=sim.accounting["fracture_release_J"], acquired=sim.accounting["pair_contact_acquired_J"])


def ledger_residual(sim, e0: float) -> float:
    """E_now - E0 + damping + fracture - tool work - external work - acquired
    (positive: the ledger missed an energy input)."""
    acc = sim.accounting
    return (sim.mechanical_energy()["mechanical_J"] - e0 + acc["damping_dissipation_J"]
            + acc["fracture_release_J"] - acc["tool_work_J"] - acc["external_work_J"]
            - acc["pair_contact_acquired_J"])


def park(b: Backend, sim) -> None:
    """Every disc 1 m from the next on the x axis, at rest, free, unbonded."""
    n = len(b.arr(sim.positions))
    sim.positions = b.put(sim, np.stack((np.arange(n, dtype=np.float64), np.zeros(n)), axis=1))
    sim.velocities = b.put(sim, np.zeros((n, 2)))
    sim.fixed = b.put(sim, np.zeros(n, dtype=bool))
    sim.alive = b.put(sim, np.zeros(len(b.arr(sim.alive)), dtype=bool))


def drag_decay(b: Backend, dt_scale: float = 1.0, v0: float = 0.5, c: float = 2.0, tau_fraction: float = 1.5) -> dict:
    """Case A: one free disc under linear drag c, nothing else acting."""
    kw = dict(nx=2, ny=2, drag=c, contact_damping=0.0, tool_speed=1e-9, fix_edges=False)
    dt0 = b.make(**kw).dt
    sim = b.make(**kw, dt=dt0 * dt_scale)
    park(b, sim)
    vel = b.arr(sim.velocities).copy()
    vel[0, 0] = v0
    sim.velocities = b.put(sim, vel)
    m = sim.config.mass
    tau = m / c
    e0 = sim.mechanical_energy()["mechanical_J"]
    for _ in range(int(round(tau_fraction * tau / sim.dt))):
        sim.step()
    t = sim.time
    v_sim = float(b.arr(sim.velocities)[0, 0])
    v_ref = v0 * math.exp(-t / tau)
    d_sim = sim.accounting["damping_dissipation_J"]
    d_ref = 0.5 * m * v0 ** 2 * (1.0 - math.exp(-2.0 * t / tau))
    ke_sim = sim.mechanical_energy()["mechanical_J"]
    ke_ref = 0.5 * m * v_ref ** 2
    r = ledger_residual(sim, e0)
    # the ledger samples the dissipated power at the pre-update velocity
    r_pred = 0.5 * (c / m) * sim.dt * d_ref
    return dict(v_sim=v_sim, v_ref=v_ref, v_relerr=abs(v_sim - v_ref) / v_ref,
                ke_relerr=abs(ke_sim - ke_ref) / ke_ref, d_sim=d_sim, d_relerr=abs(d_sim - d_ref) / d_ref,
                residual=r, r_pred=r_pred, r_pred_relerr=abs(r - r_pred) / abs(r_pred),
                r_over_d=abs(r) / d_ref)


def bonded_oscillator(b: Backend, dt_scale: float = 1.0, k: float = 2000.0, amplitude_ratio: float = 0.005,
                      periods: float = 3.0) -> dict:
    """Case B: discs 0 and 1 joined by their bond alone, released from rest at
    an extension of 0.5% of the rest length; no drag, no damping."""
    kw = dict(nx=2, ny=2, bond_stiffness=k, contact_stiffness=k, drag=0.0, contact_damping=0.0, tool_speed=1e-9,
              fix_edges=False, breaking_strain=10.0, shear_breaking_strain=10.0)
    dt0 = b.make(**kw).dt
    sim = b.make(**kw, dt=dt0 * dt_scale)
    m = sim.config.mass
    rest = 2.0 * sim.config.radius
    amp = amplitude_ratio * rest
    alive = np.zeros(len(b.arr(sim.alive)), dtype=bool)
    alive[_pair_index(b, sim, 0, 1)] = True
    sim.alive = b.put(sim, alive)
    sim.fixed = b.put(sim, np.zeros(len(b.arr(sim.fixed)), dtype=bool))
    pos = b.arr(sim.positions).copy()
    pos[0] = (-rest / 2 - amp / 2, 0.0)
    pos[1] = (rest / 2 + amp / 2, 0.0)
    sim.positions = b.put(sim, pos)
    sim.velocities = b.put(sim, np.zeros_like(pos))
    omega = math.sqrt(2.0 * k / m)
    e0 = sim.mechanical_energy()["mechanical_J"]
    worst = 0.0
    for _ in range(int(round(periods * 2.0 * math.pi / omega / sim.dt))):
        sim.step()
        p = b.arr(sim.positions)
        ext = float(np.hypot(*(p[1] - p[0]))) - rest
        worst = max(worst, abs(ext - amp * math.cos(omega * sim.time)) / amp)
    acc = sim.accounting
    return dict(e0=e0, k=k, amp=amp, xi_relerr_max=worst, r_over_e0=abs(ledger_residual(sim, e0)) / e0,
                damping=acc["damping_dissipation_J"], tool=acc["tool_work_J"], fracture=acc["fracture_release_J"])


# -- the assertions, shared by the CPU and GPU test modules ------------------

def check_uniform_load_momentum(b: Backend) -> None:
    gap, ref = uniform_load_momentum(b)
    assert ref > 0.0
    assert gap <= 1e-6 * ref, (gap, ref)


def check_drag_tool_support_momentum(b: Backend) -> None:
    m = drag_tool_support_momentum(b)
    assert m["ref"] > 1e-9
    assert abs(m["drag_y"]) > 0.0 and abs(m["tool_y"]) > 0.0
    assert m["gap"] <= 1e-6 * m["ref"], m


def check_retained_contact_energy(b: Backend, run: dict) -> None:
    assert run["sim"].broken_bonds > 0
    analytic, credited = retained_contact_energy(b, run)
    assert analytic > 0.0
    assert abs(credited - analytic) <= 1e-12 * max(analytic, 1.0), (credited, analytic)
    assert 0.2 < credited / run["accounting"]["fracture_release_J"] < 0.8


def check_energy_closure(run: dict) -> None:
    raw = abs(run["raw"]) / run["scale"]
    closed = abs(run["closed"]) / run["scale"]
    assert raw > 0.01, raw
    assert closed < 0.005, closed
    assert closed < raw / 5.0


def check_residual_is_bookkeeping(coarse: dict, fine: dict) -> None:
    assert 0.7 < abs(coarse["raw"]) / abs(fine["raw"]) < 1.4
    assert abs(coarse["closed"]) / abs(fine["closed"]) > 1.2


def check_controlled_break(b: Backend) -> None:
    row = controlled_break(b)
    assert row["broken"]
    assert row["rel_err"] < 1e-12, row
    assert row["acquired"] == 0.0
    assert abs(row["extension"] - row["xi0"]) <= 1e-12
    assert abs(row["residual"]) < 0.05 * row["closed"], row


def check_scaling(b: Backend) -> None:
    rows = scaling_rows(b)
    base = rows[0]["released"]
    for row in rows:
        expected = base * row["ratio"]
        assert abs(row["released"] - expected) <= 1e-12 * max(1.0, expected), row


def check_indentation_events(b: Backend) -> None:
    c = indentation_events(b)
    assert len(c["events"]) >= 1 and c["n_overlap"] >= 1
    assert c["rel_err_released"] < 1e-12 and c["rel_err_acquired"] < 1e-12, c
    for e in c["events"]:
        assert abs(e["recorded"] - e["released"]) <= 1e-15, e


def check_subthreshold(b: Backend) -> None:
    d = subthreshold(b)
    assert d["alive"]
    assert d["released"] == 0.0 and d["acquired"] == 0.0


LEDGER_TOL = 0.03  # the reference's acceptance for the closed-form ledger cases


def check_drag_decay(a: dict, a_half: dict) -> None:
    assert a["v_sim"] < a["v_ref"] * 1.02
    assert a["v_relerr"] < LEDGER_TOL and a["ke_relerr"] < LEDGER_TOL and a["d_relerr"] < LEDGER_TOL, a
    assert a["r_over_d"] < LEDGER_TOL
    assert a["r_pred"] > 0.0 and a["r_pred_relerr"] < 0.10, a
    assert 0.4 < a_half["r_over_d"] / a["r_over_d"] < 0.6
    assert a_half["d_relerr"] < a["d_relerr"]
    # negative control: without the dissipation channel the identity is open
    assert a["d_sim"] > 0.0 and a["d_sim"] / max(abs(a["residual"]), 1e-18) > 50.0


def check_oscillator(coarse: dict, fine: dict) -> None:
    assert coarse["r_over_e0"] < LEDGER_TOL
    for key in ("damping", "tool", "fracture"):
        assert abs(coarse[key]) <= 1e-12, key
    assert abs(coarse["e0"] - 0.5 * coarse["k"] * coarse["amp"] ** 2) <= 1e-10 * coarse["e0"]
    # semi-implicit Euler's phase error at omega dt = 0.11: a trajectory miss,
    # not a ledger one, and first order in dt
    assert LEDGER_TOL < coarse["xi_relerr_max"] < 0.10
    assert 0.35 < fine["xi_relerr_max"] / coarse["xi_relerr_max"] < 0.65
    assert fine["r_over_e0"] <= coarse["r_over_e0"]


def check_tool_channel(run: dict, run_half: dict) -> None:
    def over_scale(r):
        return abs(r["closed"]) / max(r["e_end"], r["accounting"]["damping_dissipation_J"], 1e-12)
    assert run["accounting"]["tool_work_J"] > 0.0
    assert over_scale(run) < LEDGER_TOL
    assert 0.2 < over_scale(run_half) / over_scale(run) < 0.7


# signed coefficients of dE - W_tool - W_ext + Q_damping + E_fracture - E_acquired
BALANCE_SIGNS = {"tool_work_J": -1.0, "external_work_J": -1.0, "damping_dissipation_J": 1.0,
                 "fracture_release_J": 1.0, "pair_contact_acquired_J": -1.0}
BALANCE_TOL = 0.005


def balance_error(run: dict, acc: dict | None = None) -> float:
    """The balance gate's relative residual, over |W_tool| + |Q_damping| + |E_fracture|
    of the same ledger."""
    acc = run["accounting"] if acc is None else acc
    r = run["e_end"] - run["e0"] + sum(s * float(acc[k]) for k, s in BALANCE_SIGNS.items())
    scale = abs(acc["tool_work_J"]) + abs(acc["damping_dissipation_J"]) + abs(acc["fracture_release_J"])
    return abs(r) / max(scale, 1e-18)


def check_balance_gate_and_negative_controls(run: dict) -> None:
    clean = balance_error(run)
    assert run["sim"].broken_bonds > 0
    assert clean < BALANCE_TOL, clean  # positive control
    faults = [("fracture_release_J", 0.0, 0.0), ("fracture_release_J", 3.0, 0.0),
              ("pair_contact_acquired_J", 0.0, 0.0), ("pair_contact_acquired_J", 3.0, 0.0),
              ("tool_work_J", 0.0, 0.0), ("damping_dissipation_J", 0.0, 0.0)]
    # external work is dormant in this run: fault it additively by the tool work
    assert run["accounting"]["external_work_J"] == 0.0
    faults.append(("external_work_J", 1.0, run["accounting"]["tool_work_J"]))
    for channel, factor, offset in faults:
        acc = dict(run["accounting"])
        acc[channel] = acc[channel] * factor + offset
        assert acc[channel] != run["accounting"][channel], channel  # the fault is not vacuous
        err = balance_error(run, acc)
        assert err > BALANCE_TOL and err > clean, (channel, factor, offset, err)
    # a sign flip of the dormant channel changes nothing: a vacuous control
    acc = dict(run["accounting"])
    acc["external_work_J"] *= -1.0
    assert acc["external_work_J"] == run["accounting"]["external_work_J"]
    assert balance_error(run, acc) == clean
