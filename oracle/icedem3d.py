"""CPU FP64 restatement of TensorDEM's 3-D bonded-sphere step (``IceDEM3D``).

TEST INFRASTRUCTURE ONLY. This module is the parity oracle for the CUDA 3-D
reference-mode path in ``tensordem_gb300``. Only ``tests/`` and
``__graft_entry__.smoke()`` may import it, and only to check results; the
product path never calls it.

It restates, in numpy float64, the algorithm of ``src/tensordem/dem3d.py`` of
the reference (cited per method below): the cubic lattice and its bonds, the
objective shear strain, tensile / shear / creep breakage, linear and
Maxwell-Wiechert bonds, the cell-list sphere contacts with the pair-keyed
Cundall-Strack history, the rolling-resistance couple, the spherical
indenter, the plane platens with Coulomb friction, body forces and
semi-implicit Euler. Forces are accumulated with ``np.add.at`` (sequential in
index order, as the reference's ``index_add_``), contacts in the reference's
pair-list order. The rounding of the reference's CPU reductions is restated:
``vector_norm`` of a 3-vector as sqrt(fma(z, z, fma(y, y, x*x))) and the
9-term square sum of the shear invariant in the lane order of torch's inner
sum; numpy has no fused multiply-add, so ``_fma`` restates it exactly with
Dekker's product and Knuth's sum.

Pinning: checked against golden vectors produced by the reference itself
(``tests/golden/make_golden3d.py``) in ``tests/test_oracle_icedem3d.py``.

The calibrated Hertz restitution map (``restitution_calibrated``) is not
restated here: its damping ratio is given (``zeta=``), pinned to the
reference's own value recorded with the golden vectors.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

EPS = float(np.finfo(np.float64).eps)


def _split(a):
    c = 134217729.0 * a
    hi = c - (c - a)
    return hi, a - hi


def _fma(a, b, c):
    """Correctly rounded a*b + c (Dekker two-product, Knuth two-sum)."""
    p = a * b
    ah, al = _split(a)
    bh, bl = _split(b)
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    s = p + c
    bb = s - p
    t = (p - (s - bb)) + (c - bb)
    return s + (t + e)


def partial_slip_magnitude(delta, fn, mu, kt):
    """Mindlin-Deresiewicz |F_t| (mindlin_partial_slip.py:155-198)."""
    tiny = float(np.finfo(np.float64).tiny)
    delta = np.maximum(delta, 0.0)
    fn = np.maximum(fn, 0.0)
    ds = ((3.0 * mu) * fn) / (2.0 * np.maximum(kt, tiny))
    cap = mu * fn
    ratio = np.where(ds > 0.0, delta / np.maximum(ds, tiny), 1.0)
    ratio = np.clip(ratio, 0.0, 1.0)
    return cap * (1.0 - np.maximum(1.0 - ratio, 0.0) ** 1.5)


def vnorm(v):
    """torch.linalg.vector_norm(v, dim=-1) of 3-vectors on the CPU."""
    x, y, z = v[..., 0], v[..., 1], v[..., 2]
    return np.sqrt(_fma(z, z, _fma(y, y, x * x)))


@dataclass(frozen=True)
class Oracle3DConfig:
    """Mirror of ``DEM3DConfig`` (dem3d.py:116-266) without the device field."""

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
    bond_delayed_elastic_fraction: tuple = (0.45, 0.20)
    bond_relaxation_time_s: tuple = (0.5, 30.0)
    bond_creep_exponent: int = 0
    bond_creep_time_s: float = 1.0
    bond_creep_force_fraction: float = 1.0
    bond_strength_weibull_modulus: float = 0.0
    bond_strength_seed: int = 0

    @property
    def mass(self) -> float:
        return self.density * (4.0 / 3.0) * math.pi * self.radius**3


@dataclass
class _Consts:
    """Scalar constants as the reference computes them (Python floats)."""

    e_pair: float = 0.0
    r_pair: float = 0.0
    e_rig: float = 0.0
    r_rig: float = 0.0
    g_star: float = 0.0
    zeta: float = 0.0
    k0: float = 0.0
    branch_k: list = field(default_factory=list)
    branch_tau: list = field(default_factory=list)


class IceDEM3DOracle:
    """numpy restatement of ``IceDEM3D`` (dem3d.py:564-1663)."""

    def __init__(self, config: Oracle3DConfig, *, dt: float, pinv=None, full_rank=None,
                 thresholds=None, zeta=None) -> None:
        """``dt`` is the resolved step; ``pinv`` / ``full_rank`` (per particle) and
        the per-bond tensile ``thresholds`` (Weibull scatter) may be given to pin
        the constants the reference draws from LAPACK and from torch's RNG; the
        pseudo-inverse defaults to numpy's."""
        cfg = config
        self.config = cfg
        self.dt = float(dt)
        self._lattice()
        n, b = len(self.positions), len(self.pairs)
        i, j = self.pairs.T
        ref = self.initial_positions[j] - self.initial_positions[i]
        self.rest_lengths = vnorm(ref)
        self.reference_bond_vectors = ref
        self.initial_normals = ref / np.maximum(self.rest_lengths, EPS)[:, None]
        if pinv is None:
            rr = ref[:, :, None] * ref[:, None, :]
            cov = np.zeros((n, 3, 3))
            np.add.at(cov, i, rr)
            np.add.at(cov, j, rr)
            pinv = np.linalg.pinv(cov)
            full_rank = np.linalg.matrix_rank(cov) >= 3
        self.pinv = np.asarray(pinv, dtype=np.float64)
        self.full_rank = np.asarray(full_rank, dtype=bool)
        self.alive = np.ones(b, dtype=bool)
        self.failure_mode = np.zeros(b, dtype=np.uint8)
        self.failure_time_s = np.full(b, -1.0)
        self.failure_extension_m = np.zeros(b)
        self.failure_energy_J = np.zeros(b)
        c = self.c = _Consts()
        nu = cfg.poisson_ratio
        comp = 1.0 - nu ** 2
        c.e_pair, c.r_pair = float(cfg.young_modulus / (2.0 * comp)), 0.5 * float(cfg.radius)
        c.e_rig, c.r_rig = float(cfg.young_modulus / comp), float(cfg.radius)
        c.g_star = float(cfg.young_modulus / (4.0 * ((2.0 - nu) * (1.0 + nu))))
        if cfg.restitution_coefficient < 1.0 and cfg.contact_damping_model == "restitution":
            a = -math.log(cfg.restitution_coefficient)
            c.zeta = a / math.sqrt(math.pi ** 2 + a ** 2)
        elif cfg.restitution_coefficient < 1.0 and cfg.contact_damping_model == "restitution_calibrated":
            c.zeta = float(zeta)
        self.maxwell = cfg.bond_model == "maxwell_wiechert"
        if self.maxwell:
            shares = [float(f) for f in cfg.bond_delayed_elastic_fraction]
            total = sum(shares)
            k = float(cfg.bond_stiffness)
            c.k0 = cfg.bond_equilibrium_fraction * k
            c.branch_k = [(1.0 - cfg.bond_equilibrium_fraction) * k * (f / total) for f in shares]
            c.branch_tau = [float(t) for t in cfg.bond_relaxation_time_s]
        m = len(c.branch_k)
        self.branch_offsets = np.zeros((b, m))
        self.elongation_prev = np.zeros(b)
        self.damage = np.zeros(b)
        self.bond_dissipation = 0.0
        self.threshold = None if thresholds is None else np.asarray(thresholds, dtype=np.float64)
        k_unrel = (c.k0 + sum(c.branch_k)) if self.maxwell else float(cfg.bond_stiffness)
        thr = cfg.breaking_strain if self.threshold is None else self.threshold
        self.creep_reference = cfg.bond_creep_force_fraction * k_unrel * thr * self.rest_lengths
        self.time = 0.0
        self.step_count = 0
        self.tool_start = np.array([0.0, 0.0, (cfg.nz - 1) * 2 * cfg.radius + cfg.radius + cfg.tool_radius
                                    + cfg.tool_gap])
        self.tool_velocity = np.array([0.0, 0.0, -cfg.tool_speed])
        x0 = self.initial_positions
        self.top_start_z = float(x0[:, 2].max()) + cfg.radius + cfg.top_platen_gap
        self.bottom_start_z = float(x0[:, 2].min()) - cfg.radius - cfg.bottom_platen_gap
        self.lateral_pos = np.zeros(4)
        self.lateral_velocity = np.zeros(4)
        if cfg.lateral_platens:
            g = cfg.lateral_platen_gap
            self.lateral_pos[:] = [float(x0[:, 0].min()) - cfg.radius - g, float(x0[:, 0].max()) + cfg.radius + g,
                                   float(x0[:, 1].min()) - cfg.radius - g, float(x0[:, 1].max()) + cfg.radius + g]
        self.history: dict[tuple[int, int], np.ndarray] = {}
        self.top_tang = np.zeros((n, 3))
        self.bottom_tang = np.zeros((n, 3))
        self.friction_power = 0.0
        self.rolling_power = 0.0
        self.reaction = np.zeros(3)
        self.platen_reaction = np.zeros(2)
        self.lateral_reaction = np.zeros(4)

    # -- lattice and bonds (dem3d.py:590-663)
    def _lattice(self) -> None:
        cfg = self.config
        zz, yy, xx = np.meshgrid(np.arange(cfg.nz, dtype=float), np.arange(cfg.ny, dtype=float),
                                 np.arange(cfg.nx, dtype=float), indexing="ij")
        if cfg.geometry == "cylinder_xz":
            xc, zc = (cfg.nx - 1) / 2.0, (cfg.nz - 1) / 2.0
            rad = min(cfg.nx - 1, cfg.nz - 1) / 2.0
            keep = ((xx - xc) ** 2 + (zz - zc) ** 2) <= rad ** 2 + 1e-12
        else:
            keep = np.ones_like(xx, dtype=bool)
        keep = keep.reshape(-1)
        full = np.stack((xx.reshape(-1), yy.reshape(-1), zz.reshape(-1)), axis=1)
        compact = np.full(len(full), -1)
        compact[keep] = np.arange(int(keep.sum()))
        grid = full[keep]
        z0 = (cfg.nz - 1) / 2.0 if cfg.geometry == "cylinder_xz" else 0.0
        self.positions = (grid - np.array([(cfg.nx - 1) / 2, (cfg.ny - 1) / 2, z0])) * (2 * cfg.radius)
        self.initial_positions = self.positions.copy()
        self.velocities = np.zeros_like(self.positions)
        fixed = np.zeros(len(grid), dtype=bool)
        if cfg.fix_x_edges and cfg.geometry == "box":
            fixed |= (grid[:, 0] == 0) | (grid[:, 0] == cfg.nx - 1)
        if cfg.fix_bottom:
            fixed |= grid[:, 2] == 0
        self.fixed = fixed
        pairs = []
        for dz in (0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    if not (dz > 0 or (dz == 0 and dy > 0) or (dz == 0 and dy == 0 and dx > 0)):
                        continue
                    for z in range(cfg.nz - dz):
                        for y in range(cfg.ny):
                            if not 0 <= y + dy < cfg.ny:
                                continue
                            for x in range(cfg.nx):
                                if not 0 <= x + dx < cfg.nx:
                                    continue
                                a = compact[(z * cfg.ny + y) * cfg.nx + x]
                                b = compact[((z + dz) * cfg.ny + y + dy) * cfg.nx + x + dx]
                                if a >= 0 and b >= 0:
                                    pairs.append((min(a, b), max(a, b)))
        n = len(grid)
        pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        self.pairs = pairs[np.argsort(pairs[:, 0] * n + pairs[:, 1], kind="stable")]

    # -- shear strain invariant (dem3d.py:875-901)
    def shear_strain(self) -> np.ndarray:
        n = len(self.positions)
        i, j = self.pairs.T
        q = self.positions[j] - self.positions[i]
        qr = q[:, :, None] * self.reference_bond_vectors[:, None, :]
        cross = np.zeros((n, 3, 3))
        np.add.at(cross, i, qr)
        np.add.at(cross, j, qr)
        P = self.pinv
        f = np.zeros_like(cross)
        for a in range(3):
            for b in range(3):
                f[:, a, b] = (cross[:, a, 0] * P[:, 0, b] + cross[:, a, 1] * P[:, 1, b]) + cross[:, a, 2] * P[:, 2, b]
        e = np.zeros_like(cross)
        for a in range(3):
            for b in range(3):
                g = (f[:, 0, a] * f[:, 0, b] + f[:, 1, a] * f[:, 1, b]) + f[:, 2, a] * f[:, 2, b]
                e[:, a, b] = 0.5 * (g - (1.0 if a == b else 0.0))
        mean = ((e[:, 0, 0] + e[:, 1, 1]) + e[:, 2, 2]) / 3.0
        for a in range(3):
            e[:, a, a] = e[:, a, a] - mean
        sq = (e * e).reshape(n, 9)
        s2 = sq[:, 8].copy()
        for k in range(4):
            s2 = s2 + (sq[:, k] + sq[:, k + 4])
        shear = np.sqrt((2.0 / 3.0) * np.maximum(s2, 0.0))
        return np.where(self.full_rank, shear, 0.0)

    # -- cell list (dem3d.py:825-856)
    def candidate_pairs(self) -> list[tuple[int, int]]:
        width = 2.0 * self.config.radius
        cells: dict[tuple[int, int, int], list[int]] = {}
        for idx, p in enumerate(self.positions):
            key = tuple(int(math.floor(float(v) / width)) for v in p)
            cells.setdefault(key, []).append(idx)
        out = []
        for (x, y, z), members in cells.items():
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        other = cells.get((x + dx, y + dy, z + dz))
                        if other is None:
                            continue
                        for a in members:
                            for b in other:
                                if b > a:
                                    out.append((a, b))
        return out

    def _cone(self, ft_mag, normal, slip, coefficient):
        cfg = self.config
        mode = cfg.friction_regularization
        if mode == "none":
            return coefficient * normal
        mu_s = coefficient if cfg.static_friction_coefficient is None else float(cfg.static_friction_coefficient)
        mu_d = coefficient if cfg.dynamic_friction_coefficient is None else float(cfg.dynamic_friction_coefficient)
        if mu_s == mu_d:
            return mu_s * normal
        if mode == "tanh":
            blend = 0.5 * (1.0 - np.tanh(slip / float(cfg.friction_transition_speed)))
            return (mu_d + (mu_s - mu_d) * blend) * normal
        static = mu_s * normal
        return np.where(ft_mag > static, mu_d * normal, static)

    def _bond_force(self, ext, update_history):
        """Linear or Maxwell-Wiechert bond force (dem3d.py:1018-1049,
        ice_bond_viscoelastic.py:186-253)."""
        cfg, c = self.config, self.c
        if not self.maxwell:
            return cfg.bond_stiffness * ext
        if update_history:
            d_old = self.elongation_prev
            d_dot = (ext - d_old) / self.dt
            diss = np.zeros_like(ext)
            new = np.empty_like(self.branch_offsets)
            for a, (k, tau) in enumerate(zip(c.branch_k, c.branch_tau)):
                decay = math.exp(-self.dt / tau)
                one_minus = -math.expm1(-self.dt / tau)
                s0 = d_old - self.branch_offsets[:, a]
                amp = d_dot * tau
                s_new = amp * one_minus + s0 * decay
                new[:, a] = ext - s_new
                sa = s0 - amp
                i2 = (amp * amp * self.dt + 2.0 * amp * sa * tau * one_minus
                      + 0.5 * (sa * sa) * tau * (one_minus * (1.0 + decay)))
                diss = diss + (k / tau) * i2
            self.branch_offsets = np.where(self.alive[:, None], new, ext[:, None])
            self.bond_dissipation += float(np.where(self.alive, diss, 0.0).sum())
            self.elongation_prev = ext.copy()
        force = c.k0 * ext
        for a, k in enumerate(c.branch_k):
            force = force + k * (ext - self.branch_offsets[:, a])
        return force

    def _stored_energy(self, ext):
        cfg, c = self.config, self.c
        if not self.maxwell:
            return 0.5 * cfg.bond_stiffness * (ext * ext)
        energy = (0.5 * c.k0) * (ext * ext)
        for a, k in enumerate(c.branch_k):
            s = ext - self.branch_offsets[:, a]
            energy = energy + (0.5 * k) * (s * s)
        return energy

    def forces(self, loads=None, *, update_fracture=True, update_history=True):
        """Total force (N,3) and tool reaction (3,) (dem3d.py:1301-1642)."""
        cfg, c = self.config, self.c
        pos, vel = self.positions, self.velocities
        i, j = self.pairs.T
        delta = pos[j] - pos[i]
        dist = vnorm(delta)
        normal = delta / np.maximum(dist, EPS)[:, None]
        normal = np.where((dist > EPS)[:, None], normal, self.initial_normals)
        ext = dist - self.rest_lengths
        mag = self._bond_force(ext, update_history)
        if update_fracture:
            shear = self.shear_strain()
            thr = cfg.breaking_strain if self.threshold is None else self.threshold
            tf = ext / self.rest_lengths > thr
            sf = 0.5 * (shear[i] + shear[j]) > cfg.shear_breaking_strain
            newly = self.alive & (tf | sf)
            self.alive &= ~(tf | sf)
            self.failure_mode[newly] = (tf[newly].astype(np.uint8) + 2 * sf[newly].astype(np.uint8))
            self.failure_time_s[newly] = self.time
            self.failure_extension_m[newly] = ext[newly]
            self.failure_energy_J[newly] = self._stored_energy(ext)[newly]
            if cfg.bond_creep_exponent > 0 and self.alive.any():
                ratio = np.abs(mag) / np.maximum(self.creep_reference, 1e-30)
                m = float(cfg.bond_creep_exponent)
                inc = ratio * ratio if m == 2.0 else (ratio if m == 1.0 else
                                                      (ratio * ratio * ratio if m == 3.0 else ratio ** m))
                inc = inc * (self.dt / float(cfg.bond_creep_time_s))
                self.damage = self.damage + np.where(self.alive, inc, 0.0)
                failed = self.alive & (self.damage >= 1.0)
                self.alive &= ~failed
                self.failure_mode[failed] = 4
                self.failure_time_s[failed] = self.time
                self.failure_extension_m[failed] = ext[failed]
                self.failure_energy_J[failed] = self._stored_energy(ext)[failed]
        force = (-cfg.drag) * vel
        if cfg.gravity > 0.0 or cfg.water_level is not None:
            force = force + self.body_forces()
        if loads is not None:
            force = force + loads
        abf = np.where(self.alive[:, None], mag[:, None] * normal, 0.0)
        np.add.at(force, i, abf)
        np.add.at(force, j, -abf)
        self.contact_energy = 0.0
        pairs = [p for p in self.candidate_pairs()]
        fpow = rpow = 0.0
        if pairs:
            ci, cj = np.asarray(pairs).T
            cd = pos[cj] - pos[ci]
            cdist = vnorm(cd)
            ov = np.maximum(2 * cfg.radius - cdist, 0.0)
            near = ov > 0
            ci, cj, cd, cdist, ov = ci[near], cj[near], cd[near], cdist[near], ov[near]
            if len(ci):
                n_ = cd / np.maximum(cdist, EPS)[:, None]
                bond_of = {(int(a), int(b)): k for k, (a, b) in enumerate(self.pairs)}
                balive = np.array([bool(self.alive[bond_of[(a, b)]]) if (a, b) in bond_of else False
                                   for a, b in zip(ci.tolist(), cj.tolist())], dtype=bool)
                rv = vel[cj] - vel[ci]
                vn = (rv[:, 0] * n_[:, 0] + rv[:, 1] * n_[:, 1]) + rv[:, 2] * n_[:, 2]
                pinned = self.fixed[ci] ^ self.fixed[cj]
                m_eff = np.where(pinned, cfg.mass, cfg.mass / 2.0)
                hertz = cfg.contact_model == "hertz"
                k_local = ((4.0 / 3.0) * c.e_pair * math.sqrt(c.r_pair)) * np.sqrt(ov) if hertz \
                    else np.full_like(ov, cfg.contact_stiffness)
                if cfg.contact_damping_model == "absolute":
                    gamma = np.full_like(ov, cfg.contact_damping)
                elif cfg.restitution_coefficient < 1.0 and hertz:
                    gamma = (2.0 * c.zeta) * np.sqrt(k_local * m_eff)
                elif cfg.restitution_coefficient < 1.0:
                    gamma = (2.0 * c.zeta) * np.sqrt(cfg.contact_stiffness * m_eff)
                else:
                    gamma = np.zeros_like(ov)
                cmag = np.maximum(k_local * ov - gamma * vn, 0.0)
                cmag = np.where(balive, 0.0, cmag)
                pot = (((8.0 / 15.0) * c.e_pair * math.sqrt(c.r_pair)) * ov ** 2.5 if hertz
                       else (0.5 * cfg.contact_stiffness) * (ov * ov))
                self.contact_energy = float(np.where(balive, 0.0, pot).sum())
                cforce = (-cmag)[:, None] * n_
                vt = rv - vn[:, None] * n_
                if cfg.friction_coefficient > 0.0:
                    td = np.array([self.history.get((int(a), int(b)), np.zeros(3))
                                   for a, b in zip(ci.tolist(), cj.tolist())])
                    if update_history:
                        td = td + vt * self.dt
                    kt = (((8.0 * c.g_star) * math.sqrt(c.r_pair)) * np.sqrt(ov)
                          if hertz and cfg.tangential_stiffness is None else
                          np.full_like(ov, float(cfg.contact_stiffness if cfg.tangential_stiffness is None
                                                 else cfg.tangential_stiffness)))
                    if cfg.tangential_model == "mindlin_partial_slip":
                        dm = vnorm(td)
                        tiny = float(np.finfo(np.float64).tiny)
                        fmag = partial_slip_magnitude(dm, cmag, float(cfg.friction_coefficient), kt)
                        unit = np.where((dm > 0.0)[:, None], td / np.maximum(dm, tiny)[:, None], 0.0)
                        ft = fmag[:, None] * unit
                    else:
                        raw = kt[:, None] * td
                        fm = vnorm(raw)
                        lim = self._cone(fm, cmag, vnorm(vt), float(cfg.friction_coefficient))
                        scale = np.where(fm > lim, lim / np.maximum(fm, 1e-15), 1.0)
                        ft = raw * scale[:, None]
                    fpow = float((ft * (vel[ci] - vel[cj])).sum())
                    np.add.at(force, ci, ft)
                    np.add.at(force, cj, -ft)
                    if update_history:
                        nxt = td if cfg.tangential_model == "mindlin_partial_slip" else ft / kt[:, None]
                        for a, b, d in zip(ci.tolist(), cj.tolist(), nxt):
                            self.history[(a, b)] = d.copy()
                if cfg.rolling_resistance_coefficient > 0.0:
                    vtm = vnorm(vt)
                    hat = np.where((vtm > 1e-15)[:, None], vt / np.maximum(vtm, EPS)[:, None], 0.0)
                    fj = (-(cfg.rolling_resistance_coefficient * cmag))[:, None] * hat
                    rpow = float(((-fj) * (vel[ci] - vel[cj])).sum())
                    np.add.at(force, ci, -fj)
                    np.add.at(force, cj, fj)
                np.add.at(force, ci, cforce)
                np.add.at(force, cj, -cforce)
        if update_history:
            self.friction_power, self.rolling_power = fpow, rpow
        tp = self.tool_start + self.time * self.tool_velocity
        td = pos - tp
        tdist = vnorm(td)
        tn = np.where((tdist > EPS)[:, None], td / np.maximum(tdist, EPS)[:, None], np.array([0.0, 0.0, -1.0]))
        tov = np.maximum(cfg.radius + cfg.tool_radius - tdist, 0.0)
        rvt = vel - self.tool_velocity
        tvn = (rvt[:, 0] * tn[:, 0] + rvt[:, 1] * tn[:, 1]) + rvt[:, 2] * tn[:, 2]
        hertz = cfg.contact_model == "hertz"
        krig = (4.0 / 3.0) * c.e_rig * math.sqrt(c.r_rig)
        tel = krig * tov ** 1.5 if hertz else cfg.contact_stiffness * tov
        tmag = np.where(tov > 0, np.maximum(tel - cfg.contact_damping * tvn, 0.0), 0.0)
        tforce = tmag[:, None] * tn
        self.reaction = -tforce.sum(axis=0)
        force = force + tforce
        self.platen_reaction[:] = 0.0
        for side, on in ((0, cfg.top_platen_enabled), (1, cfg.bottom_platen_enabled)):
            if not on:
                continue
            if side == 0:
                z = self.top_start_z + self.time * cfg.top_platen_velocity
                ov_ = np.maximum(pos[:, 2] + cfg.radius - z, 0.0)
                el = krig * ov_ ** 1.5 if hertz else cfg.platen_stiffness * ov_
                pm = np.where(ov_ > 0, np.maximum(el + cfg.platen_damping * (vel[:, 2] - cfg.top_platen_velocity),
                                                  0.0), 0.0)
                force[:, 2] += -pm
                self.platen_reaction[0] = pm.sum()
            else:
                z = self.bottom_start_z + self.time * cfg.bottom_platen_velocity
                ov_ = np.maximum(z + cfg.radius - pos[:, 2], 0.0)
                el = krig * ov_ ** 1.5 if hertz else cfg.platen_stiffness * ov_
                pm = np.where(ov_ > 0, np.maximum(el - cfg.platen_damping * (vel[:, 2] - cfg.bottom_platen_velocity),
                                                  0.0), 0.0)
                force[:, 2] += pm
                self.platen_reaction[1] = -pm.sum()
            if cfg.platen_friction_coefficient > 0.0:
                touch = ov_ > 0
                u = np.where(touch[:, None], vel, 0.0)
                u[:, 2] = 0.0
                tang = self.top_tang if side == 0 else self.bottom_tang
                if update_history:
                    tang = np.where(touch[:, None], tang + u * self.dt, 0.0)
                    if side == 0:
                        self.top_tang = tang
                    else:
                        self.bottom_tang = tang
                if cfg.tangential_model == "mindlin_partial_slip":
                    g_rig = float(cfg.young_modulus / (2.0 * ((2.0 - cfg.poisson_ratio) * (1.0 + cfg.poisson_ratio))))
                    a = np.maximum((3.0 * np.maximum(pm, 0.0)) * c.r_rig / (4.0 * c.e_rig), 0.0) ** (1.0 / 3.0)
                    dm = vnorm(tang)
                    fmag = partial_slip_magnitude(dm, pm, float(cfg.platen_friction_coefficient), (8.0 * g_rig) * a)
                    force = force + (-fmag)[:, None] * (tang / np.maximum(dm, EPS)[:, None])
                else:
                    k_t = float(cfg.platen_stiffness if cfg.platen_friction_stiffness is None
                                else cfg.platen_friction_stiffness)
                    spring = (-k_t) * tang
                    sm = vnorm(spring)
                    lim = self._cone(sm, pm, vnorm(u), float(cfg.platen_friction_coefficient))
                    scale = np.where(sm > lim, lim / np.maximum(sm, EPS), 1.0)
                    force = force + spring * scale[:, None]
        self.lateral_reaction[:] = 0.0
        if cfg.lateral_platens:
            k = cfg.lateral_platen_stiffness if cfg.lateral_platen_stiffness is not None else cfg.platen_stiffness
            cc = cfg.lateral_platen_damping if cfg.lateral_platen_damping is not None else cfg.platen_damping
            lp, lv = self.lateral_pos, self.lateral_velocity
            px, py, vx, vy = pos[:, 0], pos[:, 1], vel[:, 0], vel[:, 1]
            # inward normals: x_min +x, x_max -x, y_min +y, y_max -y; both planes
            # of an axis use the velocity of the first one (dem3d.py:1595)
            for q, col, ov_, vrel in ((0, 0, (lp[0] - px) + cfg.radius, vx - lv[0]),
                                      (1, 0, (px + cfg.radius) - lp[1], vx - lv[0]),
                                      (2, 1, (lp[2] - py) + cfg.radius, vy - lv[2]),
                                      (3, 1, (py + cfg.radius) - lp[3], vy - lv[2])):
                ov_ = np.maximum(ov_, 0.0)
                if q % 2 == 0:
                    mg = np.where(ov_ > 0, np.maximum(k * ov_ - cc * vrel, 0.0), 0.0)
                    force[:, col] += mg
                    self.lateral_reaction[q] = -mg.sum()
                else:
                    mg = np.where(ov_ > 0, np.maximum(k * ov_ + cc * vrel, 0.0), 0.0)
                    force[:, col] -= mg
                    self.lateral_reaction[q] = mg.sum()
        return force, self.reaction.copy()

    def submerged_fraction(self):
        cfg = self.config
        if cfg.water_level is None:
            return np.zeros(len(self.positions))
        r = cfg.radius
        h = self.positions[:, 2] - cfg.water_level
        hc = np.clip(h, -r, r)
        f = ((r - hc) * (r - hc)) * (2.0 * r + hc) / (4.0 * r ** 3)
        f = np.clip(f, 0.0, 1.0)
        f = np.where(h >= r, 0.0, f)
        return np.where(h <= -r, 1.0, f)

    def body_forces(self):
        """Gravity, buoyancy and wet drag (dem3d.py:937-963)."""
        cfg = self.config
        body = np.zeros_like(self.positions)
        if cfg.gravity > 0.0:
            body[:, 2] -= cfg.mass * cfg.gravity
        if cfg.water_level is None:
            return body
        f = self.submerged_fraction()
        volume = (4.0 / 3.0) * math.pi * cfg.radius ** 3
        body[:, 2] += (cfg.water_density * cfg.gravity * volume) * f
        if cfg.wet_drag_coefficient > 0.0:
            body = body - (cfg.wet_drag_coefficient * f)[:, None] * self.velocities
        return body

    def step(self, loads=None) -> None:
        """Semi-implicit Euler (dem3d.py:1644-1663)."""
        force, _ = self.forces(loads)
        acc = force / self.config.mass
        acc[self.fixed] = 0.0
        self.velocities = self.velocities + acc * self.dt
        self.velocities[self.fixed] = 0.0
        self.positions = self.positions + self.velocities * self.dt
        self.positions[self.fixed] = self.initial_positions[self.fixed]
        if self.config.lateral_platens:
            self.lateral_pos = self.lateral_pos + self.lateral_velocity * self.dt
        self.time += self.dt
        self.step_count += 1

    def run(self, steps: int) -> None:
        for _ in range(steps):
            self.step()
