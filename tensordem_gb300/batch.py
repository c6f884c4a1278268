"""Batched ragged engine: many independent 2-D DEM solves on one GPU.

:class:`Batch` owns one ``tdem_batch`` of ``libtdem_sm103.so``
(include/tdem.h). Each admitted instance is an :class:`~tensordem_gb300.hm2d.HM2DConfig`
plus its state and optional bonds, exactly what :class:`~tensordem_gb300.hm2d.HM2D`
takes for one solve. All live instances advance together, one persistent step
kernel per step and one conditional CUDA graph launch per step block. Instances
join and retire between step blocks.

:func:`ensemble_case` draws the mixed ensemble of 2-D runs the batched engine
is measured on (seeded): half bonded-ice indentations (the hexagonal ice sheet
of :func:`~tensordem_gb300.hm2d.ice_sheet_case`, scaled down), half granular
column collapses with aspect ratio U[0.5, 4]. Particle counts are
log-uniform, as are Young's moduli (1-70 GPa). Friction is U[0.3, 0.7] and
radii U[0.8, 1.2] x r0.
"""

from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field, replace

import numpy as np
import torch

from . import _lib
from .hm2d import ALL_WALLS, HM2DConfig, rayleigh_dt

LEDGER_NAMES = ("kinetic", "potential", "hertz", "tangential", "total", "dissipated", "evals", "rebuilds",
                "max_neighbors", "status", "graph", "variant", "bond_elastic", "fracture_released",
                "tool_work", "broken", "peak_load", "peak_eval", "reaction_x", "reaction_y")


@dataclass(frozen=True)
class BatchConfig:
    """Capacities of one batched engine (all device memory is allocated once)."""

    particle_capacity: int
    key_capacity: int
    max_instances: int = 8192
    max_neighbors: int = 12
    max_bonds: int = 6
    precision: int = 32
    rebuild_every: int = 0
    # FP32: 1 keeps each position's FP32 rounding remainder (see HM2DConfig)
    position_remainder: int = 1

    def to_c(self) -> _lib.BatchConfigC:
        c = _lib.BatchConfigC()
        c.precision, c.max_neighbors, c.max_bonds = self.precision, self.max_neighbors, self.max_bonds
        c.max_instances, c.particle_capacity, c.key_capacity = (self.max_instances, self.particle_capacity,
                                                                 self.key_capacity)
        c.rebuild_every = self.rebuild_every
        c.position_remainder = self.position_remainder
        return c

    def bytes(self) -> int:
        """Device bytes this configuration allocates."""
        out = C.c_int64()
        rc = _lib.lib().tdem_batch_bytes(C.byref(self.to_c()), C.byref(out))
        _lib.check(rc, None, "tdem_batch_bytes")
        return int(out.value)


@dataclass
class Instance:
    """One solve: configuration, state (host FP64, local order), bonds, steps."""

    config: HM2DConfig
    state: dict
    bonds: np.ndarray | None = None
    strength: np.ndarray | None = None
    steps: int = 0
    kind: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.config.n

    @property
    def keys(self) -> int:
        return self.config.ncx * self.config.ncy


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class Batch:
    """A batched ragged engine on the current CUDA device."""

    def __init__(self, config: BatchConfig, device: str | torch.device = "cuda"):
        self.config = config
        self.device = torch.device(device)
        if self.device.type != "cuda" or not torch.cuda.is_available():
            raise ValueError("Batch runs on CUDA devices only")
        self._lib = _lib.lib()
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_batch_create(C.byref(config.to_c()), C.byref(h))
        _lib.check(rc, None, "tdem_batch_create")
        self._h = h
        self.sizes: dict[int, int] = {}
        # TDEM_GRAPH=0: plain launches (visible to profilers), same results
        if os.environ.get("TDEM_GRAPH", "1") == "0":
            self.use_graph(False)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.tdem_batch_destroy(h)
            self._h = None

    def _stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def use_graph(self, on: bool) -> None:
        self._lib.tdem_batch_use_graph(self._h, 1 if on else 0)

    def admit(self, inst: Instance) -> int:
        """Add one instance; it joins at the next step. Returns its id."""
        cfg = inst.config
        n = cfg.n
        st = {k: _f64(inst.state[k]) for k in ("pos", "vel", "omega", "radius", "mass", "inertia")}
        for k, shape in (("pos", (n, 2)), ("vel", (n, 2)), ("omega", (n,)), ("radius", (n,)),
                         ("mass", (n,)), ("inertia", (n,))):
            if st[k].shape != shape:
                raise ValueError(f"{k} has shape {st[k].shape}, expected {shape}")
        if inst.bonds is not None and len(inst.bonds):
            bonds = np.ascontiguousarray(inst.bonds, dtype=np.int32)
            strength = _f64(inst.strength if inst.strength is not None else np.ones(len(bonds)))
            nb, bp, sp = len(bonds), bonds.ctypes.data, strength.ctypes.data
        else:
            bonds = strength = None
            nb, bp, sp = 0, None, None
        out = C.c_int32(-1)
        c = replace(cfg, precision=self.config.precision, max_bonds=self.config.max_bonds,
                    max_neighbors=self.config.max_neighbors).to_c()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_batch_admit(self._h, C.byref(c), st["pos"].ctypes.data, st["vel"].ctypes.data,
                                            st["omega"].ctypes.data, st["radius"].ctypes.data,
                                            st["mass"].ctypes.data, st["inertia"].ctypes.data, bp, sp, nb,
                                            C.byref(out), self._stream())
        _lib.check(rc, self._h, "tdem_batch_admit")
        self.sizes[int(out.value)] = n
        return int(out.value)

    def step(self, n: int) -> None:
        """Advance every live instance by n steps (asynchronous). ``step(0)``
        sorts in admissions, compacts retirements and builds the step graph."""
        from . import ops
        if not hasattr(self, "_anchor"):
            self._anchor = torch.zeros(1, device=self.device)  # the device of the torch op
        with torch.cuda.device(self.device):
            ops.batch_step(self._h.value, int(n), self._anchor)

    def read(self, iid: int, state: bool = True) -> dict:
        """Integer-time state (host FP64, local order) and ledger of one instance."""
        n = self.sizes[iid]
        led = np.zeros(_lib.BATCH_L_COUNT)
        if state:
            pos, vel = np.empty((n, 2)), np.empty((n, 2))
            omega, force, torque = np.empty(n), np.empty((n, 2)), np.empty(n)
            ptrs = [a.ctypes.data for a in (pos, vel, omega, force, torque)]
        else:
            ptrs = [None] * 5
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_batch_read(self._h, iid, *ptrs, led.ctypes.data, _lib.BATCH_L_COUNT,
                                           self._stream())
        _lib.check(rc, self._h, "tdem_batch_read")
        out = {"ledger": dict(zip(LEDGER_NAMES, led.tolist()))}
        if state:
            out.update(pos=pos, vel=vel, omega=omega, force=force, torque=torque)
        return out

    def ledgers(self, ids) -> list[dict]:
        """Ledgers of many instances from one read-back evaluation."""
        ids = np.ascontiguousarray(list(ids), dtype=np.int32)
        out = np.zeros((len(ids), _lib.BATCH_L_COUNT))
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_batch_read_ledgers(self._h, ids.ctypes.data, len(ids), out.ctypes.data,
                                                   self._stream())
        _lib.check(rc, self._h, "tdem_batch_read_ledgers")
        return [dict(zip(LEDGER_NAMES, row.tolist())) for row in out]

    def set_steps(self, iid: int, steps: int) -> None:
        """Freeze the instance once it has taken ``steps`` steps (0: no limit)."""
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_batch_set_steps(self._h, iid, int(steps), self._stream())
        _lib.check(rc, self._h, "tdem_batch_set_steps")

    def retire(self, iid: int) -> None:
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_batch_retire(self._h, iid, self._stream())
        _lib.check(rc, self._h, "tdem_batch_retire")
        self.sizes.pop(iid, None)

    def bonds(self, iid: int) -> dict[str, np.ndarray]:
        cap = 6 * self.sizes[iid] + 8
        pairs = np.zeros((cap, 2), dtype=np.int32)
        state = np.zeros((cap, 2), dtype=np.int32)
        count = C.c_int64()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_batch_read_bonds(self._h, iid, pairs.ctypes.data, state.ctypes.data, cap,
                                                 C.byref(count), self._stream())
        _lib.check(rc, self._h, "tdem_batch_read_bonds")
        k = min(int(count.value), cap)
        order = np.lexsort((pairs[:k, 1], pairs[:k, 0]))
        return {"pairs": pairs[:k][order], "mode": state[:k, 0][order], "fail_eval": state[:k, 1][order]}

    def info(self) -> dict[str, int]:
        out = (C.c_int64 * len(_lib.BATCH_INFO))()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_batch_info(self._h, out, len(_lib.BATCH_INFO), self._stream())
        _lib.check(rc, self._h, "tdem_batch_info")
        return dict(zip(_lib.BATCH_INFO, (int(x) for x in out)))

    @property
    def variant(self) -> int:
        return int(self._lib.tdem_batch_get_variant(self._h))

    @variant.setter
    def variant(self, v: int) -> None:
        _lib.check(self._lib.tdem_batch_set_variant(self._h, int(v)), self._h, "tdem_batch_set_variant")

    def autotune(self, steps: int = 5) -> dict[int, float]:
        """Time ``steps`` real steps of every step-kernel variant; keep the fastest."""
        nv = int(self._lib.tdem_batch_num_variants())
        ms = (C.c_float * nv)()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_batch_autotune(self._h, int(steps), ms, self._stream())
        _lib.check(rc, self._h, "tdem_batch_autotune")
        return {v: float(ms[v]) for v in range(nv)}


# ---------------------------------------------------------------------------
# Seeded ensemble of mixed 2-D runs
# ---------------------------------------------------------------------------

def _grid(width: float, height: float, reach: float) -> tuple[int, int, float]:
    """Cell grid covering width x height with square cells of at least ``reach``."""
    ncx = max(1, int(math.floor(width / reach)))
    ncy = max(1, int(math.floor(height / reach)))
    cell = max(width / ncx, height / ncy)
    return max(1, int(math.ceil(width / cell))), max(1, int(math.ceil(height / cell))), cell


def ice_instance(n_target: int, rng: np.random.Generator, *, young: float, mu: float, steps: int,
                 r0: float = 0.05, density: float = 900.0, poisson: float = 0.3, restitution: float = 0.5,
                 bond_damping: float = 0.05, breaking_strain: float = 0.01, shear_breaking_strain: float = 0.02,
                 strength_sigma: float = 0.1, speed: float = 0.5, dt_factor: float = 0.1,
                 skin_factor: float = 0.5) -> Instance:
    """Bonded hexagonal ice strip (about 4:1, both short ends clamped), indented
    from above at mid-span by a rigid disc; radii U[0.8, 1.2] r0. The lattice
    spacing is 2 r_max = 2.4 r0, so bonded neighbours never overlap at rest
    and a broken bond never starts as a compressed contact. Fragments released
    by brittle breaks fly off at metres per second, so the domain is a walled
    tank, and the skin is 0.5 r0: an intact lattice has no candidate inside it
    (bonded pairs are excluded, the next shell is at 4.2 r0), and the wide skin
    keeps list rebuilds rare."""
    nx = max(4, int(round(math.sqrt(4.0 * n_target))))
    ny = max(2, int(round(n_target / nx)))
    n = nx * ny
    r_max = 1.2 * r0
    half = r_max  # half the lattice spacing
    dt = dt_factor * rayleigh_dt(0.8 * r0, density, young, poisson)
    travel = speed * dt * steps
    below = travel + 4.0 * r_max  # room for the sheet to bend under the indenter
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    x = (2.0 * ii + (jj % 2)) * half + 2.0 * r_max
    y = jj * math.sqrt(3.0) * half + below
    pos = np.stack((x.ravel(), y.ravel()), axis=1)
    idx = jj * nx + ii
    pairs = [np.stack((idx[:, :-1].ravel(), idx[:, 1:].ravel()), axis=1)]
    for parity in (0, 1):
        rows = np.arange(parity, ny - 1, 2)
        if len(rows) == 0:
            continue
        if parity == 0:
            pairs += [np.stack((idx[rows][:, 1:].ravel(), idx[rows + 1][:, :-1].ravel()), axis=1),
                      np.stack((idx[rows].ravel(), idx[rows + 1].ravel()), axis=1)]
        else:
            pairs += [np.stack((idx[rows].ravel(), idx[rows + 1].ravel()), axis=1),
                      np.stack((idx[rows][:, :-1].ravel(), idx[rows + 1][:, 1:].ravel()), axis=1)]
    bonds = np.sort(np.concatenate(pairs).astype(np.int64), axis=1)
    bonds = bonds[np.lexsort((bonds[:, 1], bonds[:, 0]))]
    strength = np.exp(rng.normal(0.0, strength_sigma, len(bonds)))
    radius = rng.uniform(0.8 * r0, 1.2 * r0, n)
    thickness = 2.0 * r0
    mass = density * math.pi * radius**2 * thickness
    clamped = (ii.ravel() == 0) | (ii.ravel() == nx - 1)
    mass[clamped] = np.inf
    inertia = 0.5 * mass * radius**2
    kn = young * thickness
    ks = kn / (2.0 * (1.0 + poisson))
    skin = skin_factor * r0
    ind_r = max(2.0 * r0, 2.0 * nx / 2048.0)
    width = (2.0 * nx + 1) * half + 4.0 * r_max
    top = (ny - 1) * math.sqrt(3.0) * half + below
    height = top + r_max + 2.0 * ind_r + travel + 4.0 * r_max
    ncx, ncy, cell = _grid(width, height, 2.0 * r_max + skin)
    center = (0.5 * (x.min() + x.max()), top + r_max + ind_r + 0.02 * r0)
    cfg = HM2DConfig(n=n, ncx=ncx, ncy=ncy, cell=cell, skin=skin, dt=dt, young=young, poisson=poisson,
                     restitution=restitution, mu=mu, mu_wall=mu, gravity=(0.0, 0.0), walls=ALL_WALLS,
                     max_neighbors=8,
                     max_bonds=6, bond_kn=kn, bond_ks=ks, bond_damping=bond_damping,
                     breaking_strain=breaking_strain, shear_breaking_strain=shear_breaking_strain,
                     indenter_center=center, indenter_velocity=(0.0, -speed), indenter_radius=ind_r)
    state = dict(pos=pos, vel=np.zeros((n, 2)), omega=np.zeros(n), radius=radius, mass=mass, inertia=inertia)
    return Instance(cfg, state, bonds, strength, steps, "ice", {"nx": nx, "ny": ny})


def column_instance(n_target: int, rng: np.random.Generator, *, young: float, mu: float, aspect: float,
                    steps: int, r0: float = 1e-3, density: float = 2500.0, poisson: float = 0.25,
                    restitution: float = 0.8, area_fraction: float = 0.55, sigma_v: float = 0.1,
                    skin_factor: float = 0.1) -> Instance:
    """Granular column (height / width = ``aspect``) against the left wall of a
    closed box with room to run out and head room above; jittered grid at area
    fraction 0.55, Gaussian velocities, gravity; radii U[0.8, 1.2] r0."""
    nx = max(2, int(round(math.sqrt(n_target / aspect))))
    ny = max(2, int(round(n_target / nx)))
    n = nx * ny
    r_min, r_max = 0.8 * r0, 1.2 * r0
    radius = rng.uniform(r_min, r_max, n)
    mean_r2 = (r_max**3 - r_min**3) / (3.0 * (r_max - r_min))
    a = max(math.sqrt(math.pi * mean_r2 / area_fraction), 2.0 * r_max * 1.0001)
    skin = skin_factor * r0
    w, h = nx * a, ny * a
    ncx, ncy, cell = _grid(w + h, h + max(0.25 * h, 0.02) + 2.0 * a, 2.0 * r_max + skin)
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    centre = np.stack(((ii.ravel() + 0.5) * a, (jj.ravel() + 0.5) * a), axis=1)
    room = np.maximum(0.5 * a - radius, 0.0)[:, None]
    pos = centre + rng.uniform(-1.0, 1.0, (n, 2)) * room * 0.999
    vel = rng.normal(0.0, sigma_v, (n, 2))
    mass = density * math.pi * radius**2 * (2.0 * radius)
    inertia = 0.5 * mass * radius**2
    dt = 0.2 * rayleigh_dt(r_min, density, young, poisson)
    cfg = HM2DConfig(n=n, ncx=ncx, ncy=ncy, cell=cell, skin=skin, dt=dt, young=young, poisson=poisson,
                     restitution=restitution, mu=mu, mu_wall=mu, gravity=(0.0, -9.81),
                     walls=ALL_WALLS, max_neighbors=12)
    state = dict(pos=pos, vel=vel, omega=np.zeros(n), radius=radius, mass=mass, inertia=inertia)
    return Instance(cfg, state, None, None, steps, "column", {"nx": nx, "ny": ny, "aspect": aspect})


@dataclass(frozen=True)
class EnsembleSpec:
    """Draw of one instance of the ensemble (built on demand by :meth:`build`)."""

    index: int
    kind: str
    n: int
    young: float
    mu: float
    aspect: float
    steps: int
    seed: int

    def build(self) -> Instance:
        rng = np.random.default_rng(self.seed)
        if self.kind == "ice":
            return ice_instance(self.n, rng, young=self.young, mu=self.mu, steps=self.steps)
        return column_instance(self.n, rng, young=self.young, mu=self.mu, aspect=self.aspect, steps=self.steps)


def ensemble_case(count: int = 4096, *, seed: int = 0, n_min: int = 100, n_max: int = 20_000,
                  steps: int = 5000, steps_max: int | None = None) -> list[EnsembleSpec]:
    """The seeded mixed ensemble: even indices bonded-ice indentations, odd
    indices granular column collapses. N log-uniform [n_min, n_max], E
    log-uniform [1, 70] GPa, mu U[0.3, 0.7], aspect U[0.5, 4]; steps fixed, or
    log-uniform [steps, steps_max] when ``steps_max`` is given."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(math.log(n_min), math.log(n_max), count))
    young = np.exp(rng.uniform(math.log(1e9), math.log(70e9), count))
    mu = rng.uniform(0.3, 0.7, count)
    aspect = rng.uniform(0.5, 4.0, count)
    if steps_max is None:
        st = np.full(count, steps)
    else:
        st = np.exp(rng.uniform(math.log(steps), math.log(steps_max), count))
    seeds = rng.integers(0, 2**63 - 1, count)
    return [EnsembleSpec(k, "ice" if k % 2 == 0 else "column", int(round(n[k])), float(young[k]), float(mu[k]),
                         float(aspect[k]), int(round(st[k])), int(seeds[k])) for k in range(count)]
