"""CPU FP64 restatement of the 2-D Hertz-Mindlin disc step (Hertz-Mindlin mode).

TEST INFRASTRUCTURE ONLY: the parity oracle and the timed CPU baseline for the
CUDA engine in ``tensordem_gb300/csrc/hm2d.cu``. Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` may use it; the product path never does.

The reference has no single 2-D Hertz-Mindlin engine; this module assembles
the step from the reference's own formulas (file:line of the reference tree):

* Hertz normal force ``(2/3) S_n delta`` with ``S_n = 2 E* sqrt(R* delta)`` and
  the Tsuji dashpot ``2 sqrt(5/6) beta sqrt(S_n m*) v_n``, clamped at zero:
  src/tensordem/scale_ceiling/kernel.py:300-310, damping ``beta`` :216-227;
  ``E* = E / (2 (1 - nu^2))``: kernel.py:103-105.
* Mindlin tangential stiffness ``S_t = 8 G* sqrt(R* delta)`` with
  ``G* = E / (4 (2 - nu)(1 + nu))``: src/tensordem/hertz_mindlin.py:51-115;
  incremental history ``xi += v_t dt``, rotation of the stored displacement
  into the current tangent plane and the Coulomb cap ``|S_t xi| <= mu F_n``
  with state projection: scale_ceiling/kernel.py:311-326,
  src/tensordem/granular2d/engine.py:483-497, hertz_mindlin.py:118-176.
* History lives only while the contact is active (reset on separation):
  src/tensordem/contact_tangential.py:356-417; it is keyed by the
  original-id pair ``i * N + j`` and looked up by binary search:
  granular2d/engine.py:388-396, 452-456, scale_ceiling/kernel.py:250-263.
* 2-D lever arms and torques ``r x F`` with the contact point at ``r_i n``:
  granular2d/engine.py:458-503.
* Planar walls with their own per-particle tangential history:
  scale_ceiling/kernel.py:338-401 (the wall cap here compares the spring force
  ``S_t |xi|`` with ``mu F_n``, as the particle-particle contact does).
* Velocity-Verlet with one force evaluation per step (the initial one primes
  the first half kick): scale_ceiling/kernel.py:410-419.
* Candidate pairs from a Verlet list rebuilt when a particle has moved more
  than ``skin / 2``: granular2d/engine.py:298-307 (cKDTree with a skin).

Dissipation ledger: normal dashpot work ``(F_n - F_el) v_n dt`` and Coulomb
slip loss ``mu F_n (|xi_trial| - |xi|)`` per contact and step
(granular2d/engine.py:489-496, 576-588); elastic energies ``0.4 F_el delta``
(Hertz) and ``0.5 S_t |xi|^2`` (scale_ceiling/kernel.py:461-487).

Parity is pinned two ways.
* Known-answer tests on the reference's own anchors (tests/test_oracle_hm2d.py):
  k_t/k_n ratios (tests/test_hertz_mindlin.py), the restitution-to-damping map
  (tests/test_contact_tangential.py:73-83), the Coulomb stick/slip cycle area
  and brute-force pair sets (tests/test_scale_ceiling_dem.py:41-80).
* A trajectory of the reference's own FP64 engine, FloeBed
  (scale_ceiling/kernel.py:155-455), on a planar frictionless bed
  (tests/golden/floebed_planar.npz, tests/test_floebed_golden.py). This oracle
  reproduces it to 1e-14 (positions) after 200 steps: the Hertz normal law,
  the dashpot on the half-step velocity, walls, gravity and velocity-Verlet
  of the assembled step are pinned against a reference executable.
The tangential history has no reference engine with this module's
conventions: FloeBed keeps an unprojected history for separated pairs still in
its list, and it has no rotation. Friction and rotation are pinned only by
the anchors above.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

try:  # scipy's KD-tree is only a faster candidate search; brute force is exact too
    from scipy.spatial import cKDTree
except Exception:  # pragma: no cover
    cKDTree = None

WALL_NORMALS = np.array([[1.0, 0.0], [-1.0, 0.0], [0.0, 1.0], [0.0, -1.0]])


def effective_modulus(young: float, poisson: float) -> float:
    """E* for two like discs, scale_ceiling/kernel.py:103-105."""
    return young / (2.0 * (1.0 - poisson**2))


def effective_shear(young: float, poisson: float) -> float:
    """G* = E / (4 (2 - nu)(1 + nu)), hertz_mindlin.py:86-91."""
    return young / (4.0 * (2.0 - poisson) * (1.0 + poisson))


def tsuji_beta(restitution: float) -> float:
    """beta = -ln e / sqrt(ln^2 e + pi^2), scale_ceiling/kernel.py:216-222."""
    if restitution >= 1.0:
        return 0.0
    ln_e = math.log(restitution)
    return -ln_e / math.sqrt(ln_e * ln_e + math.pi**2)


def rayleigh_dt(radius: float, density: float, young: float, poisson: float) -> float:
    """Rayleigh time pi r sqrt(rho/G) / (0.1631 nu + 0.8766), xval/oss_rolling.py:183-200."""
    g = young / (2.0 * (1.0 + poisson))
    return math.pi * radius * math.sqrt(density / g) / (0.1631 * poisson + 0.8766)


@dataclass
class HMParams:
    young: float
    poisson: float
    restitution: float
    mu: float
    mu_wall: float
    dt: float
    gravity: tuple[float, float] = (0.0, -9.81)
    box: tuple[float, float] | None = None   # walls at 0 and box[a]; None = no walls
    walls: tuple[bool, bool, bool, bool] = (True, True, True, True)  # left, right, bottom, top
    skin: float = 0.0

    @property
    def estar(self) -> float:
        return effective_modulus(self.young, self.poisson)

    @property
    def gstar(self) -> float:
        return effective_shear(self.young, self.poisson)

    @property
    def damp(self) -> float:
        return 2.0 * math.sqrt(5.0 / 6.0) * tsuji_beta(self.restitution)


def contact_law(p: HMParams, delta, nrm, ra, rb, inv_ma, inv_mb, vel_a, vel_b, om_a, om_b, xi) -> dict:
    """The per-contact Hertz-Mindlin law for K active contacts (delta > 0).

    ``nrm`` is the unit normal from a to b (K, 2), ``xi`` the stored
    tangential history in a's orientation. The relative velocity of the
    contact points is v_a - v_b + (omega_a r_a + omega_b r_b) t with
    t = (-n_y, n_x) (granular2d/engine.py:458-482). Returns the force on a,
    ``cr`` = n x F_a (torque on a = r_a cr, on b = r_b cr), the updated
    history, the normal force, the elastic part and the two dissipation terms
    of the step (kernel.py:300-326, hertz_mindlin.py:118-176,
    contact_tangential.py:377-417, granular2d/engine.py:483-497).
    """
    dt = p.dt
    tng = np.stack((-nrm[:, 1], nrm[:, 0]), axis=1)
    reff = ra * rb / (ra + rb)
    meff = 1.0 / (inv_ma + inv_mb)
    sq = np.sqrt(reff * delta)
    s_n = 2.0 * p.estar * sq
    f_el = (2.0 / 3.0) * s_n * delta
    v_rel = vel_a - vel_b + (om_a * ra + om_b * rb)[:, None] * tng
    v_n = (v_rel * nrm).sum(axis=1)
    f_n = np.maximum(f_el + p.damp * np.sqrt(s_n * meff) * v_n, 0.0)
    v_t = v_rel - v_n[:, None] * nrm
    xi = xi + v_t * dt
    xi = xi - (xi * nrm).sum(axis=1)[:, None] * nrm
    s_t = 8.0 * p.gstar * sq
    fmag = s_t * np.sqrt((xi * xi).sum(axis=1))
    cap = p.mu * f_n
    slip = fmag > cap
    scale = np.where(slip, cap / np.maximum(fmag, 1e-300), 1.0)
    slip_loss = float(np.sum(np.where(slip, cap * (fmag - cap) / np.maximum(s_t, 1e-300), 0.0)))
    xi = xi * scale[:, None]
    f_a = -f_n[:, None] * nrm - s_t[:, None] * xi
    cr = nrm[:, 0] * f_a[:, 1] - nrm[:, 1] * f_a[:, 0]
    return dict(f_a=f_a, cr=cr, xi=xi, f_n=f_n, f_el=f_el, s_t=s_t, sliding=slip, slip_loss=slip_loss,
                dashpot_loss=float(np.sum((f_n - f_el) * v_n)) * dt)


@dataclass
class ContactState:
    keys: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    xi: np.ndarray = field(default_factory=lambda: np.zeros((0, 2)))


def brute_force_pairs(pos: np.ndarray, reach_extra: np.ndarray | float, radius: np.ndarray,
                      *, skin: float = 0.0) -> tuple[np.ndarray, np.ndarray]:
    """All (i, j), i < j, with |x_j - x_i| <= r_i + r_j + skin (exact, O(N^2))."""
    n = len(pos)
    ii, jj = [], []
    for s in range(0, n, 2048):
        e = min(n, s + 2048)
        d = pos[None, :, :] - pos[s:e, None, :]
        dist = np.sqrt((d * d).sum(axis=2))
        reach = radius[s:e, None] + radius[None, :] + skin
        ok = (dist <= reach) & (np.arange(n)[None, :] > np.arange(s, e)[:, None])
        a, b = np.nonzero(ok)
        ii.append(a + s)
        jj.append(b)
    return np.concatenate(ii).astype(np.int64), np.concatenate(jj).astype(np.int64)


class HM2DOracle:
    """FP64 2-D Hertz-Mindlin discs with walls, gravity and velocity-Verlet."""

    def __init__(self, pos, vel, omega, radius, mass, inertia, params: HMParams):
        self.pos = np.array(pos, dtype=np.float64)
        self.vel = np.array(vel, dtype=np.float64)
        self.omega = np.array(omega, dtype=np.float64)
        self.radius = np.array(radius, dtype=np.float64)
        self.mass = np.array(mass, dtype=np.float64)
        self.inertia = np.array(inertia, dtype=np.float64)
        # clamped discs carry infinite mass and inertia: zero inverse mass
        with np.errstate(divide="ignore"):
            self.inv_mass = np.where(np.isfinite(self.mass), 1.0 / self.mass, 0.0)
            self.inv_inertia = np.where(np.isfinite(self.inertia), 1.0 / self.inertia, 0.0)
        self.p = params
        self.n = len(self.pos)
        self.state = ContactState()
        self.wall_xi = np.zeros((4, self.n, 2))
        self.dissipated = 0.0       # cumulative dashpot + slip loss (J)
        self.time = 0.0
        self.steps = 0
        self.force = None
        self.torque = None
        self._cand = None
        self._cand_pos = None
        self.rebuilds = 0

    # ------------------------------------------------------------ candidates
    def candidate_pairs(self):
        """Verlet list with skin, rebuilt after a move of more than skin / 2."""
        skin = self.p.skin
        if (self._cand is None or self._cand_pos is None or
                np.sqrt(((self.pos - self._cand_pos) ** 2).sum(axis=1)).max(initial=0.0) > 0.5 * skin):
            reach = 2.0 * float(self.radius.max()) + skin
            if cKDTree is not None and self.n > 4096:
                pairs = cKDTree(self.pos).query_pairs(reach, output_type="ndarray").astype(np.int64)
                pairs = pairs.reshape(-1, 2)
                i = np.minimum(pairs[:, 0], pairs[:, 1])
                j = np.maximum(pairs[:, 0], pairs[:, 1])
                d = self.pos[j] - self.pos[i]
                keep = np.sqrt((d * d).sum(axis=1)) <= self.radius[i] + self.radius[j] + skin
                i, j = i[keep], j[keep]
                order = np.argsort(i * self.n + j, kind="stable")
                i, j = i[order], j[order]
            else:
                i, j = brute_force_pairs(self.pos, 0.0, self.radius, skin=skin)
            self._cand = (i, j)
            self._cand_pos = self.pos.copy()
            self.rebuilds += 1
        return self._cand

    # ---------------------------------------------------------------- forces
    def evaluate(self, pos, vel, omega, *, advance: bool):
        """Forces, torques and dissipation of one evaluation at (pos, vel, omega)."""
        p = self.p
        n = self.n
        dt = p.dt
        force = np.zeros((n, 2))
        torque = np.zeros(n)
        diss = 0.0
        self.before_contacts(pos, advance=advance)
        i, j = self.candidate_pairs()
        d = pos[j] - pos[i]
        dist = np.sqrt((d * d).sum(axis=1))
        delta = self.radius[i] + self.radius[j] - dist
        act = delta > 0.0
        excl = self.contact_exclusions()
        if excl is not None and len(excl):
            act &= ~np.isin(i * n + j, excl)
        act &= (self.inv_mass[i] + self.inv_mass[j]) > 0  # two clamped discs exchange no force
        i, j, d, dist, delta = i[act], j[act], d[act], dist[act], delta[act]
        keys = i * n + j
        xi = np.zeros((len(i), 2))
        st = self.state
        if len(st.keys) and len(keys):
            at = np.clip(np.searchsorted(st.keys, keys), 0, len(st.keys) - 1)
            hit = st.keys[at] == keys
            xi[hit] = st.xi[at[hit]]
        if len(i):
            nrm = d / dist[:, None]
            ra, rb = self.radius[i], self.radius[j]
            c = contact_law(p, delta, nrm, ra, rb, self.inv_mass[i], self.inv_mass[j], vel[i], vel[j],
                            omega[i], omega[j], xi)
            xi, f_a, cr = c["xi"], c["f_a"], c["cr"]
            diss += c["slip_loss"]
            np.add.at(force, i, f_a)
            np.add.at(force, j, -f_a)
            np.add.at(torque, i, ra * cr)
            np.add.at(torque, j, rb * cr)
            diss += c["dashpot_loss"]
        if advance:
            self.state = ContactState(keys, xi)
        # walls
        if p.box is not None:
            for w in range(4):
                if not p.walls[w]:
                    continue
                nw = WALL_NORMALS[w]
                if w == 0:
                    gap = pos[:, 0]
                elif w == 1:
                    gap = p.box[0] - pos[:, 0]
                elif w == 2:
                    gap = pos[:, 1]
                else:
                    gap = p.box[1] - pos[:, 1]
                delta_w = self.radius - gap
                idx = np.flatnonzero(delta_w > 0.0)
                new_xi = np.zeros((n, 2))
                if len(idx):
                    r = self.radius[idx]
                    dw = delta_w[idx]
                    sq = np.sqrt(r * dw)
                    s_n = 2.0 * p.estar * sq
                    f_el = (2.0 / 3.0) * s_n * dw
                    perp = np.array([-nw[1], nw[0]])
                    v_c = vel[idx] - (omega[idx] * r)[:, None] * perp[None, :]
                    v_n = -(v_c @ nw)
                    f_n = np.maximum(f_el + p.damp * np.sqrt(s_n / self.inv_mass[idx]) * v_n, 0.0)
                    v_t = v_c - (v_c @ nw)[:, None] * nw[None, :]
                    xw = self.wall_xi[w, idx] + v_t * dt
                    xw = xw - (xw @ nw)[:, None] * nw[None, :]
                    s_t = 8.0 * p.gstar * sq
                    fmag = s_t * np.sqrt((xw * xw).sum(axis=1))
                    cap = p.mu_wall * f_n
                    slip = fmag > cap
                    scale = np.where(slip, cap / np.maximum(fmag, 1e-300), 1.0)
                    diss += float(np.sum(np.where(slip, cap * (fmag - cap) / np.maximum(s_t, 1e-300), 0.0)))
                    xw = xw * scale[:, None]
                    f = f_n[:, None] * nw[None, :] - s_t[:, None] * xw
                    force[idx] += f
                    torque[idx] += -r * (nw[0] * f[:, 1] - nw[1] * f[:, 0])
                    diss += float(np.sum((f_n - f_el) * v_n)) * dt
                    new_xi[idx] = xw
                if advance:
                    self.wall_xi[w] = new_xi
        force, torque, diss = self.extra_forces(pos, vel, omega, force, torque, diss, advance=advance)
        free = self.inv_mass > 0
        force[free] += self.mass[free, None] * np.asarray(p.gravity)[None, :]
        return force, torque, diss

    # hooks for the bonded engine
    def before_contacts(self, pos, *, advance):
        pass

    def contact_exclusions(self):
        return None

    def energy_exclusions(self):
        """Pair keys without contact energy in the committed state."""
        return None

    def extra_forces(self, pos, vel, omega, force, torque, diss, *, advance):
        return force, torque, diss

    # ----------------------------------------------------------- integration
    def prime(self) -> None:
        self.force, self.torque, d = self.evaluate(self.pos, self.vel, self.omega, advance=True)
        self.dissipated += d

    def step(self, n: int = 1) -> None:
        """Velocity-Verlet (scale_ceiling/kernel.py:410-419)."""
        if self.force is None:
            self.prime()
        h = 0.5 * self.p.dt
        for _ in range(n):
            self.vel = self.vel + h * self.force * self.inv_mass[:, None]
            self.omega = self.omega + h * self.torque * self.inv_inertia
            self.pos = self.pos + self.p.dt * self.vel
            self.steps += 1
            self.force, self.torque, d = self.evaluate(self.pos, self.vel, self.omega, advance=True)
            self.dissipated += d
            self.vel = self.vel + h * self.force * self.inv_mass[:, None]
            self.omega = self.omega + h * self.torque * self.inv_inertia
            self.time += self.p.dt

    # ---------------------------------------------------------------- ledger
    def energies(self) -> dict:
        """Kinetic, gravitational, Hertz elastic and tangential spring energy (J)."""
        p = self.p
        free = self.inv_mass > 0
        ke = 0.5 * float(np.sum(self.mass[free] * (self.vel[free]**2).sum(axis=1))
                         + np.sum(self.inertia[free] * self.omega[free]**2))
        pe = -float(np.sum(self.mass[free] * (self.pos[free] @ np.asarray(p.gravity))))
        un = ut = 0.0
        i, j = self.candidate_pairs()
        d = self.pos[j] - self.pos[i]
        dist = np.sqrt((d * d).sum(axis=1))
        delta = self.radius[i] + self.radius[j] - dist
        act = delta > 0
        # the pairs evaluate() gives no contact force hold no contact energy
        excl = self.energy_exclusions()
        if excl is not None and len(excl):
            act &= ~np.isin(i * self.n + j, excl)
        act &= (self.inv_mass[i] + self.inv_mass[j]) > 0
        if act.any():
            ia, ja, da = i[act], j[act], delta[act]
            reff = self.radius[ia] * self.radius[ja] / (self.radius[ia] + self.radius[ja])
            sq = np.sqrt(reff * da)
            un += float(np.sum(0.4 * (2.0 / 3.0) * 2.0 * p.estar * sq * da * da))
            keys = ia * self.n + ja
            st = self.state
            if len(st.keys):
                at = np.clip(np.searchsorted(st.keys, keys), 0, len(st.keys) - 1)
                hit = st.keys[at] == keys
                xi2 = np.zeros(len(keys))
                xi2[hit] = (st.xi[at[hit]] ** 2).sum(axis=1)
                ut += float(np.sum(0.5 * 8.0 * p.gstar * sq * xi2))
        if p.box is not None:
            gaps = (self.pos[:, 0], p.box[0] - self.pos[:, 0], self.pos[:, 1], p.box[1] - self.pos[:, 1])
            for w in range(4):
                if not p.walls[w]:
                    continue
                dw = self.radius - gaps[w]
                idx = np.flatnonzero(dw > 0)
                if len(idx):
                    sq = np.sqrt(self.radius[idx] * dw[idx])
                    un += float(np.sum(0.4 * (2.0 / 3.0) * 2.0 * p.estar * sq * dw[idx] ** 2))
                    ut += float(np.sum(0.5 * 8.0 * p.gstar * sq * (self.wall_xi[w, idx] ** 2).sum(axis=1)))
        extra = self.extra_energies()
        total = ke + pe + un + ut + self.dissipated + sum(extra.values())
        return dict(kinetic=ke, potential=pe, elastic_normal=un, elastic_tangential=ut,
                    dissipated=self.dissipated, **extra, total=total)

    def extra_energies(self) -> dict:
        return {}

    def active_pairs(self) -> set[tuple[int, int]]:
        return set(zip(*(x.tolist() for x in divmod(self.state.keys, self.n))))


def pinv_sym2(a: float, b: float, c: float) -> np.ndarray:
    """Pseudo-inverse of [[a, b], [b, c]] (cutoff 2 eps sigma_max as torch.linalg.pinv)."""
    return np.linalg.pinv(np.array([[a, b], [b, c]], dtype=np.float64))


class BondedHM2DOracle(HM2DOracle):
    """FP64 bonded discs: the reference's bond model on top of Hertz-Mindlin contacts.

    * Bonds carry a normal spring ``k_n (d - L0)`` (the central bond of
      src/tensordem/dem.py:286-288) plus a shear spring ``k_s u_s`` on the
      incremental tangential displacement and dashpots ``2 zeta sqrt(k m*)``.
    * Irreversible breakage on tensile strain ``(d - L0)/L0 > eps_t f`` or on
      the bond's objective shear ``(s_i + s_j)/2 > eps_s f`` (dem.py:243-268),
      with ``f`` the bond's strength factor and ``s`` the per-disc
      Green-Lagrange shear invariant of the least-squares deformation gradient
      over the disc's initial bonds (dem.py:182-208), written as
      ``E = (G + G^T + G^T G)/2`` with ``G = F - I``.
    * A broken (or never bonded) pair interacts through the Hertz contact.
    * A rigid circular indenter (Hertz normal + dashpot, frictionless) moves at
      constant velocity (dem.py:294-312); its work on the discs is booked.
    """

    def __init__(self, pos, vel, omega, radius, mass, inertia, params: HMParams, *, bonds, strength,
                 k_n, k_s, zeta, eps_t, eps_s, indenter=None):
        super().__init__(pos, vel, omega, radius, mass, inertia, params)
        b = np.asarray(bonds, dtype=np.int64).reshape(-1, 2)
        self.bi = np.minimum(b[:, 0], b[:, 1])
        self.bj = np.maximum(b[:, 0], b[:, 1])
        self.ref = self.pos[self.bj] - self.pos[self.bi]
        self.l0 = np.sqrt((self.ref * self.ref).sum(axis=1))
        self.strength = np.asarray(strength, dtype=np.float64)
        self.alive = np.ones(len(self.bi), dtype=bool)
        self.us = np.zeros((len(self.bi), 2))
        self.fail_eval = np.full(len(self.bi), -1, dtype=np.int64)
        self.fail_mode = np.zeros(len(self.bi), dtype=np.uint8)
        self.k_n, self.k_s, self.zeta = float(k_n), float(k_s), float(zeta)
        self.eps_t, self.eps_s = float(eps_t), float(eps_s)
        self.fracture_released = 0.0
        self.tool_work = 0.0
        self.indenter = indenter  # dict(center=(x, y), velocity=(vx, vy), radius=R)
        self.evals = 0
        self.reaction = np.zeros(2)
        # constant pseudo-inverse of each disc's bond covariance
        n = self.n
        cov = np.zeros((n, 2, 2))
        outer = self.ref[:, :, None] * self.ref[:, None, :]
        np.add.at(cov, self.bi, outer)
        np.add.at(cov, self.bj, outer)
        self.pinv = np.linalg.pinv(cov)
        self.bond_keys = np.sort(self.bi * n + self.bj)

    def contact_exclusions(self):
        # bonds intact after this evaluation's break test (dem.py:251 precedes
        # the pair forces: a bond broken now already acts as a contact)
        return (self.bi * self.n + self.bj)[self._alive_now]

    def energy_exclusions(self):
        # bonds intact in the committed state (no peeked break test)
        return (self.bi * self.n + self.bj)[self.alive]

    def before_contacts(self, pos, *, advance):
        """Break test at this evaluation's positions (dem.py:243-277)."""
        p = self.p
        s = self.strains(pos)
        i, j = self.bi, self.bj
        cur = pos[j] - pos[i]
        d = np.sqrt((cur * cur).sum(axis=1))
        u = cur - self.ref
        ext = (2.0 * (self.ref * u).sum(axis=1) + (u * u).sum(axis=1)) / (d + self.l0)
        tensile = ext / self.l0
        shear = 0.5 * (s[i] + s[j])
        tf = tensile > self.eps_t * self.strength
        sf = shear > self.eps_s * self.strength
        new = self.alive & (tf | sf)
        self._ext = ext
        self._alive_now = self.alive & ~new
        if advance and new.any():
            self.fail_eval[new] = self.evals
            self.fail_mode[new] = tf[new].astype(np.uint8) + 2 * sf[new].astype(np.uint8)
            # spring energy released, minus the Hertz energy a still-overlapping
            # pair acquires as a contact at once (dem.py:270-277 books both)
            ov = np.maximum(self.radius[i[new]] + self.radius[j[new]] - d[new], 0.0)
            reff = self.radius[i[new]] * self.radius[j[new]] / (self.radius[i[new]] + self.radius[j[new]])
            acquired = 0.4 * (2.0 / 3.0) * 2.0 * p.estar * np.sqrt(reff * ov) * ov * ov
            self.fracture_released += float(np.sum(0.5 * self.k_n * ext[new] ** 2
                                                    + 0.5 * self.k_s * (self.us[new] ** 2).sum(axis=1)
                                                    - acquired))

    def strains(self, pos) -> np.ndarray:
        """Objective shear invariant per disc (dem.py:182-208, displacement form)."""
        cur = pos[self.bj] - pos[self.bi]
        u = cur - self.ref
        g = np.zeros((self.n, 2, 2))
        m = u[:, :, None] * self.ref[:, None, :]
        np.add.at(g, self.bi, m)
        np.add.at(g, self.bj, m)
        g = g @ self.pinv
        e = 0.5 * (g + np.transpose(g, (0, 2, 1)) + np.transpose(g, (0, 2, 1)) @ g)
        return np.sqrt((e[:, 0, 0] - e[:, 1, 1]) ** 2 + 4.0 * e[:, 0, 1] ** 2)

    def extra_forces(self, pos, vel, omega, force, torque, diss, *, advance):
        p = self.p
        dt = p.dt
        i, j = self.bi, self.bj
        cur = pos[j] - pos[i]
        d = np.sqrt((cur * cur).sum(axis=1))
        ext = self._ext
        alive = self._alive_now
        a = np.flatnonzero(alive & ((self.inv_mass[i] + self.inv_mass[j]) > 0))
        if len(a):
            ia, ja = i[a], j[a]
            nrm = cur[a] / d[a, None]
            tng = np.stack((-nrm[:, 1], nrm[:, 0]), axis=1)
            ra, rb = self.radius[ia], self.radius[ja]
            meff = 1.0 / (self.inv_mass[ia] + self.inv_mass[ja])
            v_rel = vel[ia] - vel[ja] + (omega[ia] * ra + omega[ja] * rb)[:, None] * tng
            v_n = (v_rel * nrm).sum(axis=1)
            v_t = v_rel - v_n[:, None] * nrm
            us = self.us[a] + v_t * dt
            us = us - (us * nrm).sum(axis=1)[:, None] * nrm
            c_n = 2.0 * self.zeta * np.sqrt(self.k_n * meff)
            c_s = 2.0 * self.zeta * np.sqrt(self.k_s * meff)
            f_a = (self.k_n * ext[a] - c_n * v_n)[:, None] * nrm - self.k_s * us - c_s[:, None] * v_t
            cr = nrm[:, 0] * f_a[:, 1] - nrm[:, 1] * f_a[:, 0]
            np.add.at(force, ia, f_a)
            np.add.at(force, ja, -f_a)
            np.add.at(torque, ia, ra * cr)
            np.add.at(torque, ja, rb * cr)
            diss += float(np.sum(c_n * v_n**2 + c_s * (v_t * v_t).sum(axis=1))) * dt
            if advance:
                self.us[a] = us
        if advance:
            self.alive = alive
        # indenter
        self.reaction = np.zeros(2)
        if self.indenter is not None:
            t = self.evals * dt
            c = np.asarray(self.indenter["center"]) + t * np.asarray(self.indenter["velocity"])
            R = float(self.indenter["radius"])
            dv = pos - c[None, :]
            dd = np.sqrt((dv * dv).sum(axis=1))
            delta = R + self.radius - dd
            k = np.flatnonzero(delta > 0)
            if len(k):
                nw = dv[k] / dd[k, None]
                r = self.radius[k]
                reff = R * r / (R + r)
                sq = np.sqrt(reff * delta[k])
                s_n = 2.0 * p.estar * sq
                f_el = (2.0 / 3.0) * s_n * delta[k]
                v_app = -((vel[k] - np.asarray(self.indenter["velocity"])) * nw).sum(axis=1)
                meff = np.where(self.inv_mass[k] > 0, 1.0 / np.maximum(self.inv_mass[k], 1e-300), 0.0)
                f_n = np.maximum(f_el + p.damp * np.sqrt(s_n * meff) * v_app, 0.0)
                f = f_n[:, None] * nw
                np.add.at(force, k, f)
                self.reaction = -f.sum(axis=0)
                diss += float(np.sum((f_n - f_el) * v_app)) * dt
                if advance:
                    self.tool_work += dt * float(-(self.reaction @ np.asarray(self.indenter["velocity"])))
        if advance:
            self.evals += 1
        return force, torque, diss

    def extra_energies(self) -> dict:
        i, j = self.bi, self.bj
        cur = self.pos[j] - self.pos[i]
        d = np.sqrt((cur * cur).sum(axis=1))
        u = cur - self.ref
        ext = (2.0 * (self.ref * u).sum(axis=1) + (u * u).sum(axis=1)) / (d + self.l0)
        a = self.alive & ((self.inv_mass[i] + self.inv_mass[j]) > 0)
        bond = float(np.sum(0.5 * self.k_n * ext[a] ** 2 + 0.5 * self.k_s * (self.us[a] ** 2).sum(axis=1)))
        # Hertz energy stored at the indenter (state at t = (evals - 1) dt)
        tool_elastic = 0.0
        if self.indenter is not None and self.evals > 0:
            t = (self.evals - 1) * self.p.dt
            c = np.asarray(self.indenter["center"]) + t * np.asarray(self.indenter["velocity"])
            R = float(self.indenter["radius"])
            dd = np.sqrt(((self.pos - c[None, :]) ** 2).sum(axis=1))
            delta = R + self.radius - dd
            k = (delta > 0) & (self.inv_mass > 0)
            if k.any():
                reff = R * self.radius[k] / (R + self.radius[k])
                sq = np.sqrt(reff * delta[k])
                tool_elastic = float(np.sum(0.4 * (2.0 / 3.0) * 2.0 * self.p.estar * sq * delta[k] ** 2))
        # fracture release leaves the mechanical budget; the tool feeds it
        return dict(bond_elastic=bond, tool_elastic=tool_elastic, fracture_released=self.fracture_released,
                    tool_work=-self.tool_work)
