"""CPU FP64 restatement of TensorDEM's 2-D bonded-disc step (``IceDEM``).

TEST INFRASTRUCTURE ONLY. This module is the parity oracle for the CUDA
reference-mode path in ``tensordem_gb300``. Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of ``bench.py`` may
import it, and only to check results or as the timed CPU baseline; the product path
never calls it.

It restates, in numpy float64, the algorithm of ``src/tensordem/dem.py`` of
the reference (cited per function below) with the reference's dense all-pairs
layout: pairs are ``triu_indices(N, N, 1)`` in row-major order and the
per-particle force is accumulated in pair order, first the ``i`` side then the
``j`` side, exactly as the reference's two ``index_add_`` calls do.

Pinning: the oracle is checked against golden vectors produced by the
reference itself (``tests/golden/make_golden.py``), see
``tests/test_oracle_icedem.py``.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class OracleConfig:
    """Mirror of ``DEMConfig`` (dem.py:17-35) without the device field."""

    nx: int = 21
    ny: int = 5
    radius: float = 0.025
    thickness: float = 0.2
    density: float = 917.0
    bond_stiffness: float = 2_000.0
    contact_stiffness: float = 2_000.0
    breaking_strain: float = 0.015
    shear_breaking_strain: float = 0.03
    contact_damping: float = 5.0
    drag: float = 2.0
    tool_radius: float = 0.1
    tool_speed: float = 1.0
    tool_gap: float = 0.01
    dt: float | None = None
    fix_edges: bool = True

    @property
    def mass(self) -> float:
        # dem.py:57-59
        return self.density * math.pi * self.radius**2 * self.thickness

    @property
    def recommended_dt(self) -> float:
        # dem.py:61-72: bound over all N-1 possible pair contacts plus the tool.
        neighbors = self.nx * self.ny - 1
        stiffness = (2 * neighbors + 1) * max(self.bond_stiffness, self.contact_stiffness)
        damping = (2 * neighbors + 1) * self.contact_damping + self.drag
        elastic_dt = 0.2 * math.sqrt(self.mass / stiffness)
        damping_dt = 0.2 * self.mass / damping if damping else math.inf
        travel_dt = 0.1 * self.radius / self.tool_speed
        return min(elastic_dt, damping_dt, travel_dt)


def _fma(a, b, c):
    """Correctly rounded a*b + c (Dekker two-product, Knuth two-sum): numpy has
    no fused multiply-add."""
    p = a * b
    s_ = 134217729.0
    ca, cb = s_ * a, s_ * b
    ah = ca - (ca - a)
    bh = cb - (cb - b)
    al, bl = a - ah, b - bh
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    s = p + c
    bb = s - p
    t = (p - (s - bb)) + (c - bb)
    return s + (t + e)


def vnorm2(delta: np.ndarray) -> np.ndarray:
    """torch.linalg.vector_norm of 2-vectors on the CPU: sqrt(fma(y, y, x*x))."""
    x, y = delta[..., 0], delta[..., 1]
    return np.sqrt(_fma(y, y, x * x))


def _pinv2x2_batch(m: np.ndarray) -> np.ndarray:
    """Moore-Penrose pseudo-inverse of a batch of 2x2 matrices (SVD based)."""
    return np.linalg.pinv(m)


def polyline_contact(p, v, vertices, hull_velocity, *, particle_radius, hull_radius,
                     stiffness, damping):
    """Disc / polyline penalty contact (hull_contact.py:7-75)."""
    eps = np.finfo(np.float64).eps
    starts = vertices[:-1]
    segments = vertices[1:] - vertices[:-1]
    length_sq = (segments * segments).sum(axis=1)
    rel = p[:, None, :] - starts[None, :, :]
    fraction = np.clip((rel * segments[None]).sum(axis=2) / length_sq[None, :], 0.0, 1.0)
    closest = starts[None] + fraction[:, :, None] * segments[None]
    delta = p[:, None, :] - closest
    distance_sq = (delta * delta).sum(axis=2)
    nearest = distance_sq.argmin(axis=1)
    rows = np.arange(p.shape[0])
    d = delta[rows, nearest]
    distance = np.sqrt(distance_sq[rows, nearest])
    tangent = segments[nearest] / np.sqrt(length_sq[nearest])[:, None]
    flip = (tangent[:, 0] < 0) | ((tangent[:, 0] == 0) & (tangent[:, 1] < 0))
    canonical = np.where(flip[:, None], -tangent, tangent)
    fallback = np.stack((-canonical[:, 1], canonical[:, 0]), axis=1)
    approach = ((v - hull_velocity) * fallback).sum(axis=1)
    fallback = np.where((approach > 0)[:, None], -fallback, fallback)
    normal = d / np.maximum(distance, eps)[:, None]
    normal = np.where((distance > eps)[:, None], normal, fallback)
    overlap = np.maximum(particle_radius + hull_radius - distance, 0.0)
    normal_speed = ((v - hull_velocity) * normal).sum(axis=1)
    magnitude = np.maximum(stiffness * overlap - damping * normal_speed, 0.0)
    magnitude = np.where(overlap > 0, magnitude, 0.0)
    forces = magnitude[:, None] * normal
    return forces, -forces.sum(axis=0)


class IceDEMOracle:
    """numpy restatement of ``IceDEM`` (dem.py:75-624), FP64, all pairs."""

    LEDGER_KEYS = ("external_work_J", "fracture_release_J", "pair_contact_acquired_J",
                   "tool_work_J", "damping_dissipation_J")
    IMPULSE_KEYS = ("external_impulse_Ns", "support_impulse_Ns", "drag_impulse_Ns",
                    "tool_impulse_on_ice_Ns")

    def __init__(self, config: OracleConfig = OracleConfig(), *, hull_profile=None,
                 hull_start=(0.0, 0.0), hull_velocity=(0.0, 0.0), bond_stiffness=None):
        cfg = config
        self.config = cfg
        # dem.py:100-104
        self.dt = cfg.dt if cfg.dt is not None else cfg.recommended_dt
        if self.dt > cfg.recommended_dt:
            raise ValueError(f"dt exceeds conservative limit {cfg.recommended_dt:.6g} s")
        # dem.py:105-111: square lattice, spacing 2r, centred in x
        yy, xx = np.meshgrid(np.arange(cfg.ny, dtype=np.float64),
                             np.arange(cfg.nx, dtype=np.float64), indexing="ij")
        self.positions = np.stack((xx.ravel() - (cfg.nx - 1) / 2, yy.ravel()), axis=1) \
            * (2 * cfg.radius)
        self.initial_positions = self.positions.copy()
        self.velocities = np.zeros_like(self.positions)
        n = len(self.positions)
        # dem.py:113-115
        self.fixed = np.zeros(n, dtype=bool)
        if cfg.fix_edges:
            self.fixed = (xx.ravel() == 0) | (xx.ravel() == cfg.nx - 1)
        # dem.py:116-129: all pairs, bonds at d <= 2r*sqrt(2)*(1+1e-10)
        iu, ju = np.triu_indices(n, k=1)
        self.pairs = np.stack((iu, ju), axis=1).astype(np.int64)
        delta = self.positions[ju] - self.positions[iu]
        distances = vnorm2(delta)
        self.initial_normals = delta / distances[:, None]
        self.bonded = distances <= 2 * cfg.radius * math.sqrt(2) * (1 + 1e-10)
        self.bond_indices = self.pairs[self.bonded]
        self.reference_bond_vectors = (self.initial_positions[self.bond_indices[:, 1]]
                                       - self.initial_positions[self.bond_indices[:, 0]])
        self.rest_lengths = distances.copy()
        self.alive = self.bonded.copy()
        # dem.py:131-136: per-pair fracture ledger
        p = len(self.pairs)
        self.failure_mode = np.zeros(p, dtype=np.uint8)
        self.failure_time_s = np.full(p, -1.0)
        self.failure_extension_m = np.zeros(p)
        self.failure_energy_J = np.zeros(p)
        self.time = 0.0
        self.step_count = 0
        self.accounting = {k: 0.0 for k in self.LEDGER_KEYS}
        for k in self.IMPULSE_KEYS:
            self.accounting[k] = [0.0, 0.0]
        self.last_step = {}
        # dem.py:146-153
        self.tool_start = np.array([0.0, (cfg.ny - 1) * 2 * cfg.radius + cfg.radius
                                    + cfg.tool_radius + cfg.tool_gap])
        self.tool_velocity = np.array([0.0, -cfg.tool_speed])
        self.hull_profile = None if hull_profile is None else np.asarray(hull_profile, np.float64)
        self.hull_start = np.asarray(hull_start, np.float64)
        self.hull_velocity = np.asarray(hull_velocity, np.float64)
        # per-bond stiffness (calibrated_dem.py:20-42): None = the config's for every bond
        self.pair_coefficients = None
        if bond_stiffness is not None:
            k = np.asarray(bond_stiffness, np.float64)
            if k.shape != (len(self.bond_indices),) or not np.isfinite(k).all() or (k <= 0).any() \
                    or (k > cfg.bond_stiffness).any():
                raise ValueError("per-bond stiffness shape/finite/positive/conservative upper bound mismatch")
            self.pair_coefficients = np.zeros(len(self.pairs))
            self.pair_coefficients[self.bonded] = k

    # dem.py:171-176
    @property
    def tool_position(self) -> np.ndarray:
        if self.hull_profile is not None:
            return self.hull_start + self.time * self.hull_velocity
        return self.tool_start + self.time * self.tool_velocity

    # dem.py:178-180
    @property
    def broken_bonds(self) -> int:
        return int((self.bonded & ~self.alive).sum())

    def local_objective_shear_strain(self) -> np.ndarray:
        """dem.py:182-208: LSQ deformation gradient over the initial bonds."""
        n = len(self.positions)
        i, j = self.bond_indices.T
        ref = self.reference_bond_vectors
        cur = self.positions[j] - self.positions[i]
        ref_outer = ref[:, :, None] * ref[:, None, :]
        cur_ref = cur[:, :, None] * ref[:, None, :]
        cov = np.zeros((n, 2, 2))
        cross = np.zeros((n, 2, 2))
        np.add.at(cov, i, ref_outer)
        np.add.at(cov, j, ref_outer)
        np.add.at(cross, i, cur_ref)
        np.add.at(cross, j, cur_ref)
        f = cross @ _pinv2x2_batch(cov)
        strain = 0.5 * (np.transpose(f, (0, 2, 1)) @ f - np.eye(2))
        return np.sqrt((strain[:, 0, 0] - strain[:, 1, 1]) ** 2 + 4.0 * strain[:, 0, 1] ** 2)

    def forces(self, external_forces=None):
        """dem.py:226-345: total particle force and ice-on-tool reaction."""
        cfg = self.config
        eps = np.finfo(np.float64).eps
        i, j = self.pairs.T
        delta = self.positions[j] - self.positions[i]
        distance = vnorm2(delta)
        normal = delta / np.maximum(distance, eps)[:, None]
        normal = np.where((distance > 0)[:, None], normal, self.initial_normals)
        extension = distance - self.rest_lengths
        tensile_strain = extension / self.rest_lengths
        local_shear = self.local_objective_shear_strain()
        ib, jb = self.bond_indices.T
        bond_shear = 0.5 * (local_shear[ib] + local_shear[jb])
        shear_failed = bond_shear > cfg.shear_breaking_strain
        tensile_failed = tensile_strain[self.bonded] > cfg.breaking_strain
        previous = self.alive.copy()
        alive_b = self.alive[self.bonded] & ~(tensile_failed | shear_failed)
        self.alive[self.bonded] = alive_b
        newly = previous & ~self.alive
        tens = np.zeros_like(self.bonded)
        shr = np.zeros_like(self.bonded)
        tens[self.bonded] = tensile_failed
        shr[self.bonded] = shear_failed
        self.failure_mode[newly] = tens[newly].astype(np.uint8) + 2 * shr[newly].astype(np.uint8)
        self.failure_time_s[newly] = self.time
        self.failure_extension_m[newly] = extension[newly]
        self.failure_energy_J[newly] = 0.5 * cfg.bond_stiffness * extension[newly] ** 2
        self.accounting["fracture_release_J"] += float(self.failure_energy_J[newly].sum())
        acquired = 0.5 * cfg.contact_stiffness * np.maximum(2 * cfg.radius - distance[newly], 0) ** 2
        self.accounting["pair_contact_acquired_J"] += float(acquired.sum())
        normal_speed = ((self.velocities[j] - self.velocities[i]) * normal).sum(axis=1)
        overlap = np.maximum(2 * cfg.radius - distance, 0.0)
        repulsion = np.maximum(cfg.contact_stiffness * overlap - cfg.contact_damping * normal_speed, 0.0)
        contact = (overlap > 0) & ~self.alive
        repulsion = np.where(contact, repulsion, 0.0)
        magnitude = np.where(self.alive, cfg.bond_stiffness * extension, -repulsion)
        pair_force = magnitude[:, None] * normal
        force = -cfg.drag * self.velocities
        np.add.at(force, i, pair_force)
        np.add.at(force, j, -pair_force)
        if self.hull_profile is None:
            tool_delta = self.positions - self.tool_position
            tool_distance = vnorm2(tool_delta)
            tool_normal = tool_delta / np.maximum(tool_distance, eps)[:, None]
            fallback = np.zeros_like(tool_normal)
            fallback[:, 1] = -1
            tool_normal = np.where((tool_distance > 0)[:, None], tool_normal, fallback)
            tool_overlap = np.maximum(cfg.radius + cfg.tool_radius - tool_distance, 0.0)
            tool_speed = ((self.velocities - self.tool_velocity) * tool_normal).sum(axis=1)
            tool_mag = np.maximum(cfg.contact_stiffness * tool_overlap - cfg.contact_damping * tool_speed, 0.0)
            tool_mag = np.where(tool_overlap > 0, tool_mag, 0.0)
            tool_force = tool_mag[:, None] * tool_normal
            tool_reaction = -tool_force.sum(axis=0)
            conservative_tool = cfg.contact_stiffness * tool_overlap[:, None] * tool_normal
            tool_v = self.tool_velocity
        else:
            vertices = self.hull_profile + self.tool_position
            tool_force, tool_reaction = polyline_contact(
                self.positions, self.velocities, vertices, self.hull_velocity,
                particle_radius=cfg.radius, hull_radius=cfg.tool_radius,
                stiffness=cfg.contact_stiffness, damping=cfg.contact_damping)
            conservative_tool, _ = polyline_contact(
                self.positions, self.velocities, vertices, self.hull_velocity,
                particle_radius=cfg.radius, hull_radius=cfg.tool_radius,
                stiffness=cfg.contact_stiffness, damping=0.0)
            tool_v = self.hull_velocity
        pair_diss = (repulsion - cfg.contact_stiffness * overlap) * (-normal_speed)
        pair_diss = np.where(contact, pair_diss, 0.0)
        tool_diss = -((tool_force - conservative_tool) * (self.velocities - tool_v)).sum()
        self._damping_power = float(pair_diss.sum() + tool_diss
                                    + cfg.drag * (self.velocities ** 2).sum())
        self._tool_power = float(-tool_reaction @ tool_v)
        force = force + tool_force
        if external_forces is not None:
            force = force + external_forces
        if self.pair_coefficients is not None:
            # calibrated_dem.py:62-84: (k_b - k) (d - L0) n on the surviving
            # bonds, added after the base force (i side, then j side), and the
            # actual spring energy of the bonds broken in this evaluation
            difference = self.pair_coefficients - cfg.bond_stiffness
            correction = (difference * extension * self.alive)[:, None] * normal
            np.add.at(force, i, correction)
            np.add.at(force, j, -correction)
            energy_correction = 0.5 * difference[newly] * extension[newly] ** 2
            self.accounting["fracture_release_J"] += float(energy_correction.sum())
            self.failure_energy_J[newly] += energy_correction
        return force, tool_reaction

    def step(self, external_forces=None, *, load_time=None):
        """dem.py:347-382: semi-implicit (symplectic) Euler with ledgers."""
        if load_time is not None and (not math.isfinite(load_time) or
                                      abs(load_time - self.time) > 1e-12 * max(1.0, abs(self.time))):
            raise ValueError("load_time must equal current DEM time in seconds")
        loads = None if external_forces is None else np.asarray(external_forces, np.float64)
        old = self.positions.copy()
        force, reaction = self.forces(loads)
        support = -force[self.fixed].sum(axis=0)
        external = np.zeros(2) if loads is None else loads.sum(axis=0)
        for name, vec in (("external_impulse_Ns", external), ("support_impulse_Ns", support),
                          ("drag_impulse_Ns", -self.config.drag * self.velocities.sum(axis=0)),
                          ("tool_impulse_on_ice_Ns", -reaction)):
            self.accounting[name] = [a + self.dt * float(b) for a, b in zip(self.accounting[name], vec)]
        self.velocities = self.velocities + self.dt * force / self.config.mass
        self.velocities[self.fixed] = 0
        self.positions = self.positions + self.dt * self.velocities
        self.positions[self.fixed] = self.initial_positions[self.fixed]
        disp = self.positions - old
        work = 0.0 if loads is None else float((loads * disp).sum())
        self.accounting["external_work_J"] += work
        self.accounting["tool_work_J"] += self.dt * self._tool_power
        self.accounting["damping_dissipation_J"] += self.dt * self._damping_power
        self.last_step = dict(
            time_start_s=self.time, time_end_s=self.time + self.dt, external_work_J=work,
            support_force_N=support.tolist(), tool_reaction_N=reaction.tolist(),
            external_force_N=external.tolist(),
            external_moment_Nm=0.0 if loads is None else float(
                (old[:, 0] * loads[:, 1] - old[:, 1] * loads[:, 0]).sum()))
        self.time += self.dt
        self.step_count += 1
        if not (np.isfinite(self.positions).all() and np.isfinite(self.velocities).all()):
            raise FloatingPointError("Non-finite simulation state; reduce dt")

    def mechanical_energy(self) -> dict:
        """dem.py:603-624."""
        cfg = self.config
        delta = self.positions[self.pairs[:, 1]] - self.positions[self.pairs[:, 0]]
        dist = vnorm2(delta)
        ext = dist - self.rest_lengths
        overlap = np.maximum(2 * cfg.radius - dist, 0.0)
        if self.pair_coefficients is None:
            bond = 0.5 * cfg.bond_stiffness * (ext[self.alive] ** 2).sum()
        else:  # calibrated_dem.py:86-93
            bond = 0.5 * (self.pair_coefficients[self.alive] * ext[self.alive] ** 2).sum()
        contact = 0.5 * cfg.contact_stiffness * (overlap[~self.alive] ** 2).sum()
        d = np.sqrt(((self.positions - self.tool_position) ** 2).sum(axis=1))
        tool_ov = np.maximum(cfg.radius + cfg.tool_radius - d, 0.0)
        tool = 0.5 * cfg.contact_stiffness * (tool_ov ** 2).sum()
        kinetic = 0.5 * cfg.mass * (self.velocities ** 2).sum()
        return dict(kinetic_J=float(kinetic), bond_J=float(bond), pair_contact_J=float(contact),
                    tool_contact_J=float(tool), mechanical_J=float(kinetic + bond + contact + tool))

    # -- flat views used by the parity replay ---------------------------------
    def accounting_vector(self) -> np.ndarray:
        acc = self.accounting
        vec = [acc[k] for k in self.LEDGER_KEYS]
        for k in self.IMPULSE_KEYS:
            vec.extend(acc[k])
        return np.asarray(vec, dtype=np.float64)

    def bond_alive(self) -> np.ndarray:
        return self.alive[self.bonded]

    def failure_ledger(self):
        b = self.bonded
        return (self.failure_mode[b], self.failure_time_s[b],
                self.failure_extension_m[b], self.failure_energy_J[b])
