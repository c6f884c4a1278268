"""Per-contact friction fixtures from the reference's own contact-law functions.

Run where the reference source tree is available::

    PYTHONPATH=<reference>/src python tests/golden/make_friction.py

For 240 seeded contact sequences of 16 steps each (six materials; four kinds:
stick, slip, reversal, separation) it calls, step by step:

* ``hertz_mindlin.hertz_mindlin_tangential_stiffness``
  (src/tensordem/hertz_mindlin.py:94-115): k_t = 8 G* sqrt(R* delta);
* ``contact_tangential.advance_tangential_contact``
  (src/tensordem/contact_tangential.py:377-417): the history increment by the
  tangential relative velocity, the Coulomb-cone projection and the reset of a
  contact without normal force;
* ``hertz_mindlin.hertz_mindlin_tangential_force``
  (src/tensordem/hertz_mindlin.py:118-176): the Mindlin spring with Coulomb
  saturation on the incremented displacement;
* ``contact_tangential.reset_tangential_displacement``
  (src/tensordem/contact_tangential.py:356-374) for a step without overlap.

A second set pins the 2-D rotation conventions of the reference's disc engine
(src/tensordem/granular2d/engine.py:466-475, 502-503): for 200 seeded contact
states (normal, radii, spins, velocities, a force on disc i) the contact-point
velocity difference v_i - v_j and both torques are formed with the engine's
own ``DiskSystem._perp`` / ``DiskSystem._cross`` and its lever arms
(lever_i = -r_i n_all, lever_j = r_j n_all with n_all = -n_ij, n_ij from i to j).

G* comes from ``hertz_mindlin.hertz_reduced_shear_modulus``
(src/tensordem/hertz_mindlin.py:51-91). The normal force handed to the
reference is the Hertz elastic force (4/3) E* sqrt(R*) delta^(3/2) with
E* = E / (2 (1 - nu^2)) (src/tensordem/scale_ceiling/kernel.py:103-105,
300-310), no dashpot. The relative velocity (partner j minus disc i) carries a
normal component that the increment must discard.
Output: tests/golden/friction_cases.npz.
"""

from __future__ import annotations

import math
from pathlib import Path

import numpy as np
import torch

OUT = Path(__file__).resolve().parent / "friction_cases.npz"
SEQUENCES = 240
STEPS = 16
MATERIALS = ((70e9, 0.25, 0.5), (5e9, 0.3, 0.3), (1e9, 0.2, 0.7), (30e9, 0.35, 0.4), (12e9, 0.15, 0.6),
             (50e9, 0.28, 0.2))
KINDS = ("stick", "slip", "reversal", "separation")


def rayleigh_dt(radius, density, young, poisson):
    g = young / (2.0 * (1.0 + poisson))
    return math.pi * radius * math.sqrt(density / g) / (0.1631 * poisson + 0.8766)


def main() -> None:
    from tensordem import contact_tangential as ct
    from tensordem import hertz_mindlin as hm

    torch.set_num_threads(1)
    rng = np.random.default_rng(2024)
    S, T = SEQUENCES, STEPS
    mat = np.arange(S) % len(MATERIALS)
    kind = (np.arange(S) // len(MATERIALS)) % len(KINDS)
    r1 = rng.uniform(0.8e-3, 1.2e-3, S)
    r2 = rng.uniform(0.8e-3, 1.2e-3, S)
    theta = rng.uniform(0.0, 2.0 * math.pi, S)
    normal = np.stack((np.cos(theta), np.sin(theta)), axis=1)
    delta0 = np.exp(rng.uniform(math.log(1e-7), math.log(1e-5), S))
    phase = rng.uniform(0.0, 2.0 * math.pi, S)
    sign = np.where(rng.uniform(size=S) < 0.5, -1.0, 1.0)
    normal_share = rng.uniform(-0.5, 0.5, S)

    overlap = np.zeros((S, T))
    v_rel = np.zeros((S, T, 2))
    f_n = np.zeros((S, T))
    k_t = np.zeros((S, T))
    disp_in = np.zeros((S, T, 2))
    disp_out = np.zeros((S, T, 2))
    f_t = np.zeros((S, T, 2))
    sliding = np.zeros((S, T), dtype=bool)
    disp_sat = np.zeros((S, T, 2))
    f_t_sat = np.zeros((S, T, 2))
    dt = np.zeros(S)
    e_star = np.zeros(S)
    g_star = np.zeros(S)
    mu = np.zeros(S)
    for s in range(S):
        young, poisson, mu_s = MATERIALS[mat[s]]
        es = young / (2.0 * (1.0 - poisson**2))
        gs = hm.hertz_reduced_shear_modulus(young, poisson)
        reff = r1[s] * r2[s] / (r1[s] + r2[s])
        dt_s = 0.2 * rayleigh_dt(0.8e-3, 2500.0, young, poisson)
        dt[s], e_star[s], g_star[s], mu[s] = dt_s, es, gs, mu_s
        k = np.arange(T)
        d = delta0[s] * (1.0 + 0.25 * np.sin(0.7 * k + phase[s]))
        if KINDS[kind[s]] == "separation":
            d[6:9] = -0.2 * delta0[s]
        overlap[s] = d
        # cone radius mu F_n / k_t at the base overlap
        limit0 = mu_s * es * delta0[s] / (6.0 * gs)
        name = KINDS[kind[s]]
        if name == "stick":
            u = np.full(T, sign[s] * 0.3 * 0.75 * limit0 / (T * dt_s))
        elif name == "slip":
            u = np.full(T, sign[s] * 3.0 * limit0 / dt_s)
        elif name == "reversal":
            u = np.where(k < 8, 0.6, -0.6) * sign[s] * limit0 / dt_s
        else:
            u = np.full(T, sign[s] * 0.6 * limit0 / dt_s)
        t_dir = np.array([-normal[s, 1], normal[s, 0]])
        v_rel[s] = u[:, None] * t_dir[None, :] + (normal_share[s] * u)[:, None] * normal[s][None, :]
        disp = torch.zeros((1, 2), dtype=torch.float64)
        nrm = torch.tensor(normal[s][None, :], dtype=torch.float64)
        for j in range(T):
            disp_in[s, j] = disp.numpy()[0]
            vr = torch.tensor(v_rel[s, j][None, :], dtype=torch.float64)
            if d[j] > 0.0:
                fn = (4.0 / 3.0) * es * math.sqrt(reff) * d[j] ** 1.5
                kt = hm.hertz_mindlin_tangential_stiffness(torch.tensor([d[j]], dtype=torch.float64), es, gs, reff)
                ft, new, sl = ct.advance_tangential_contact(disp, vr, nrm, torch.tensor([fn], dtype=torch.float64),
                                                            float(kt[0]), mu_s, dt_s)
                raw = ct.integrate_tangential_displacement(disp, vr, nrm, dt_s)
                ft2, new2 = hm.hertz_mindlin_tangential_force(torch.tensor([d[j]], dtype=torch.float64), raw, es, gs,
                                                              reff, mu_s, torch.tensor([fn], dtype=torch.float64))
                f_n[s, j], k_t[s, j] = fn, float(kt[0])
                f_t[s, j], sliding[s, j] = ft.numpy()[0], bool(sl[0])
                f_t_sat[s, j], disp_sat[s, j] = ft2.numpy()[0], new2.numpy()[0]
            else:
                new = ct.reset_tangential_displacement(disp, torch.tensor([False]))
            disp_out[s, j] = new.numpy()[0]
            disp = new
    # rotation conventions of the 2-D disc engine
    from tensordem.granular2d.engine import DiskSystem
    R = 200
    th = rng.uniform(0.0, 2.0 * math.pi, R)
    n_ij = np.stack((np.cos(th), np.sin(th)), axis=1)
    rot_r = rng.uniform(0.8e-3, 1.2e-3, (R, 2))
    rot_w = rng.normal(0.0, 100.0, (R, 2))
    rot_v = rng.normal(0.0, 0.1, (R, 2, 2))
    rot_f = rng.normal(0.0, 1.0, (R, 2))
    n_all = -n_ij
    lever_i = -rot_r[:, 0:1] * n_all
    lever_j = rot_r[:, 1:2] * n_all
    v_i = rot_v[:, 0] + DiskSystem._perp(rot_w[:, 0:1] * lever_i)
    v_j = rot_v[:, 1] + DiskSystem._perp(rot_w[:, 1:2] * lever_j)
    rot_vrel = v_i - v_j
    rot_torque = np.stack((DiskSystem._cross(lever_i, rot_f), DiskSystem._cross(lever_j, -rot_f)), axis=1)
    np.savez_compressed(OUT, rot_normal=n_ij, rot_radius=rot_r, rot_omega=rot_w, rot_vel=rot_v, rot_force=rot_f,
                        rot_vrel=rot_vrel, rot_torque=rot_torque, material=mat, kind=kind, r1=r1, r2=r2,
                        normal=normal, overlap=overlap, v_rel=v_rel,
                        f_n=f_n, k_t=k_t, disp_in=disp_in, disp_out=disp_out, f_t=f_t, sliding=sliding,
                        disp_sat=disp_sat, f_t_sat=f_t_sat, dt=dt, e_star=e_star, g_star=g_star, mu=mu,
                        young=np.array([m[0] for m in MATERIALS]), poisson=np.array([m[1] for m in MATERIALS]),
                        mu_material=np.array([m[2] for m in MATERIALS]))
    print(f"wrote {OUT}: {S} sequences x {T} steps, {int(sliding.sum())} sliding steps, "
          f"{int((overlap <= 0).sum())} open steps")


if __name__ == "__main__":
    main()
