"""Hertz-Mindlin 2-D disc engine (Hertz-Mindlin mode) on the GB300 CUDA path.

:class:`HM2D` owns one engine of ``libtdem_sm103.so`` (include/tdem.h,
``tdem_hm_*``): device-resident particle state sorted by cell, a Verlet
neighbour list rebuilt on the device when the accumulated displacement bound
reaches half the skin, and one fused force + velocity-Verlet kernel per step,
all driven by a conditional CUDA graph. ``precision=32`` is the production
form (FP32 contacts on FP32 offsets from an integer cell origin, compensated
per-particle sums, FP64 ledger); ``precision=64`` is the plain FP64 kernel.

:func:`granular_gas_case` builds the seeded 1,048,576-disc settling case:
radii U[0.8, 1.2] mm, density 2500 kg/m^3, E = 70 GPa, nu = 0.25, mu = 0.5,
restitution 0.8, a jittered square grid at area fraction 0.55 in a box with
four rigid walls, Gaussian velocities (sigma 0.1 m/s), gravity -9.81 m/s^2,
dt = 0.2 Rayleigh time of the smallest disc.
"""

from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

WALL_LEFT, WALL_RIGHT, WALL_BOTTOM, WALL_TOP = 1, 2, 4, 8
ALL_WALLS = 15


@dataclass(frozen=True)
class HM2DConfig:
    """Engine configuration. The box is [0, ncx*cell] x [0, ncy*cell]."""

    n: int
    ncx: int
    ncy: int
    cell: float
    skin: float
    dt: float
    young: float
    poisson: float
    restitution: float
    mu: float
    mu_wall: float
    gravity: tuple[float, float] = (0.0, -9.81)
    walls: int = ALL_WALLS
    precision: int = 32
    max_neighbors: int = 16
    inertia_factor: float = 0.5
    # bonded-particle model (max_bonds == 0: none)
    max_bonds: int = 0
    bond_kn: float = 0.0
    bond_ks: float = 0.0
    bond_damping: float = 0.0
    breaking_strain: float = 0.01
    shear_breaking_strain: float = 0.02
    # rigid circular indenter (radius 0: none)
    indenter_center: tuple[float, float] = (0.0, 0.0)
    indenter_velocity: tuple[float, float] = (0.0, 0.0)
    indenter_radius: float = 0.0
    load_capacity: int = 0
    # FP32 engines: 64 sums each particle's terms in FP64 (else float-float)
    sum_precision: int = 32
    # FP32 engines: 1 keeps each position's FP32 rounding remainder (positions
    # integrate to ~48 bits; the energy ledger closes as in FP64 before breaks)
    position_remainder: int = 1

    @property
    def box(self) -> tuple[float, float]:
        c = float(np.float32(self.cell)) if self.precision == 32 else float(self.cell)
        return (self.ncx * c, self.ncy * c)

    def to_c(self) -> _lib.HMConfigC:
        c = _lib.HMConfigC()
        c.n, c.precision, c.max_neighbors, c.walls = self.n, self.precision, self.max_neighbors, self.walls
        c.ncx, c.ncy = self.ncx, self.ncy
        c.cell, c.skin, c.dt = self.cell, self.skin, self.dt
        c.young, c.poisson, c.restitution = self.young, self.poisson, self.restitution
        c.mu, c.mu_wall = self.mu, self.mu_wall
        c.gravity[0], c.gravity[1] = self.gravity
        c.inertia_factor = self.inertia_factor
        c.max_bonds = self.max_bonds
        c.bond_kn, c.bond_ks, c.bond_damping = self.bond_kn, self.bond_ks, self.bond_damping
        c.breaking_strain, c.shear_breaking_strain = self.breaking_strain, self.shear_breaking_strain
        c.indenter_center[0], c.indenter_center[1] = self.indenter_center
        c.indenter_velocity[0], c.indenter_velocity[1] = self.indenter_velocity
        c.indenter_radius = self.indenter_radius
        c.load_capacity = self.load_capacity
        c.sum_precision = self.sum_precision
        c.position_remainder = self.position_remainder
        return c


def grid_for_box(box: float, r_max: float, skin: float) -> tuple[int, float]:
    """Largest cell count whose cells still hold the reach 2 r_max + skin."""
    ncell = max(1, int(math.floor(box / (2.0 * r_max + skin))))
    return ncell, box / ncell


def rayleigh_dt(radius: float, density: float, young: float, poisson: float) -> float:
    """pi r sqrt(rho/G) / (0.1631 nu + 0.8766) (xval/oss_rolling.py:183-200 of the reference)."""
    g = young / (2.0 * (1.0 + poisson))
    return math.pi * radius * math.sqrt(density / g) / (0.1631 * poisson + 0.8766)


def granular_gas_case(n_side: int = 1024, *, seed: int = 0, r_min: float = 0.8e-3,
                      r_max: float = 1.2e-3, density: float = 2500.0, young: float = 70e9,
                      poisson: float = 0.25, mu: float = 0.5, restitution: float = 0.8,
                      area_fraction: float = 0.55, sigma_v: float = 0.1, skin: float = 0.1e-3,
                      precision: int = 32, max_neighbors: int = 16) -> tuple[HM2DConfig, dict]:
    """Seeded polydisperse disc gas in a walled square box (numpy PCG64 ``seed``).

    Discs sit on an n_side x n_side grid of spacing ``a`` chosen so that the
    expected disc area fills ``area_fraction`` of the box; each centre is
    jittered inside its grid square without touching its borders, so no two
    discs overlap at t = 0. Disc thickness is 2 r (mass 2 pi rho r^3,
    I = m r^2 / 2).
    """
    rng = np.random.default_rng(seed)
    n = n_side * n_side
    radius = rng.uniform(r_min, r_max, n)
    mean_r2 = (r_max**3 - r_min**3) / (3.0 * (r_max - r_min))
    a = math.sqrt(math.pi * mean_r2 / area_fraction)
    if a < 2.0 * r_max:
        raise ValueError("area fraction too high for a non-overlapping jittered grid")
    box_req = n_side * a
    ncell, cell = grid_for_box(box_req, r_max, skin)
    c32 = float(np.float32(cell)) if precision == 32 else cell
    box = ncell * c32
    a = box / n_side  # spread the grid over the exact wall-to-wall box
    jj, ii = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="ij")
    centre = np.stack(((ii.ravel() + 0.5) * a, (jj.ravel() + 0.5) * a), axis=1)
    room = np.maximum(0.5 * a - radius, 0.0)[:, None]
    pos = centre + rng.uniform(-1.0, 1.0, (n, 2)) * room * 0.999
    vel = rng.normal(0.0, sigma_v, (n, 2))
    omega = np.zeros(n)
    thickness = 2.0 * radius
    mass = density * math.pi * radius**2 * thickness
    inertia = 0.5 * mass * radius**2
    dt = 0.2 * rayleigh_dt(float(radius.min()), density, young, poisson)
    cfg = HM2DConfig(n=n, ncx=ncell, ncy=ncell, cell=cell, skin=skin, dt=dt, young=young,
                     poisson=poisson, restitution=restitution, mu=mu, mu_wall=mu,
                     gravity=(0.0, -9.81), walls=ALL_WALLS, precision=precision,
                     max_neighbors=max_neighbors)
    state = dict(pos=pos, vel=vel, omega=omega, radius=radius, mass=mass, inertia=inertia)
    return cfg, state


def _as_f64(x, device) -> tuple[object, int, object]:
    """(pointer, host flag, keep-alive) for an FP64 array on the host or the GPU."""
    if isinstance(x, torch.Tensor):
        t = x.detach().to(dtype=torch.float64).contiguous()
        if t.is_cuda:
            return t.data_ptr(), 0, t
        return t.data_ptr(), 1, t
    a = np.ascontiguousarray(x, dtype=np.float64)
    return a.ctypes.data, 1, a


class HM2D:
    """One Hertz-Mindlin engine instance on the current CUDA device."""

    def __init__(self, config: HM2DConfig, device: str | torch.device = "cuda"):
        self.config = config
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("HM2D runs on CUDA devices only")
        if not torch.cuda.is_available():
            raise ValueError("CUDA requested but unavailable")
        self._lib = _lib.lib()
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_create(C.byref(config.to_c()), C.byref(h))
        _lib.check(rc, None, "tdem_hm_create")
        self._h = h
        self.steps = 0
        self._anchor = torch.zeros(1, device=self.device)  # the device of the torch ops
        # TDEM_GRAPH=0 runs steps as plain launches (profilers cannot see
        # kernels inside conditional CUDA graphs); results are identical.
        if os.environ.get("TDEM_GRAPH", "1") == "0":
            self.use_graph(False)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.tdem_hm_destroy(h)
            self._h = None

    def _stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    @property
    def handle(self) -> int:
        """The engine's C-ABI handle (tdem_hm*), as the torch ops take it."""
        return int(self._h.value)

    @property
    def anchor(self) -> torch.Tensor:
        """A one-element tensor on the engine's device: the torch ops' device argument."""
        return self._anchor

    def use_graph(self, on: bool) -> None:
        self._lib.tdem_hm_use_graph(self._h, 1 if on else 0)

    def set_state(self, pos, vel, omega, radius, mass, inertia) -> None:
        """Upload a state given in original particle order (host or device arrays)."""
        n = self.config.n
        args = [_as_f64(x, self.device) for x in (pos, vel, omega, radius, mass, inertia)]
        for (_, _, a), shape in zip(args, [(n, 2), (n, 2), (n,), (n,), (n,), (n,)]):
            if tuple(a.shape) != shape:
                raise ValueError(f"state array of shape {tuple(a.shape)}, expected {shape}")
        hosts = {h for _, h, _ in args}
        if len(hosts) != 1:
            raise ValueError("state arrays must all be on the host or all on the GPU")
        self._keep = args
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_set_state(self._h, *[p for p, _, _ in args], hosts.pop(), self._stream())
        _lib.check(rc, self._h, "tdem_hm_set_state")
        self.check()
        self.steps = 0

    def step(self, n_steps: int = 1, *, check: bool = True) -> None:
        """Advance n velocity-Verlet steps (one graph launch). ``step(0)``
        only builds the step graph for the current variant (about half a
        second), which the first stepping call would otherwise pay."""
        from . import ops
        with torch.cuda.device(self.device):
            ops.hm_step(self._h.value, int(n_steps), self._anchor)
            self.steps += int(n_steps)
            if check:
                self.check()

    def check(self) -> None:
        rc = self._lib.tdem_hm_status(self._h, self._stream())
        _lib.check(rc, self._h, "tdem_hm_status")

    def state(self) -> dict[str, torch.Tensor]:
        """Integer-time state in original order as FP64 CUDA tensors."""
        n = self.config.n
        out = dict(pos=torch.empty((n, 2), dtype=torch.float64, device=self.device),
                   vel=torch.empty((n, 2), dtype=torch.float64, device=self.device),
                   omega=torch.empty(n, dtype=torch.float64, device=self.device),
                   force=torch.empty((n, 2), dtype=torch.float64, device=self.device),
                   torque=torch.empty(n, dtype=torch.float64, device=self.device))
        from . import ops
        with torch.cuda.device(self.device):
            ops.hm_read_state(self._h.value, out["pos"], out["vel"], out["omega"], out["force"], out["torque"])
        return out

    def read_state_host(self, pos: np.ndarray, vel: np.ndarray, omega: np.ndarray) -> None:
        """Copy positions, velocities and omega into host arrays (synchronizes)."""
        for a in (pos, vel, omega):
            if a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("host outputs must be C-contiguous float64")
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_read_state(self._h, pos.ctypes.data, vel.ctypes.data,
                                              omega.ctypes.data, None, None, 1, self._stream())
        _lib.check(rc, self._h, "tdem_hm_read_state")

    def ledger(self) -> dict[str, float]:
        buf = (C.c_double * _lib.HM_COUNT)()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_read_ledger(self._h, buf, _lib.HM_COUNT, self._stream())
        _lib.check(rc, self._h, "tdem_hm_read_ledger")
        v = list(buf)
        return dict(kinetic=v[0], potential=v[1], elastic_normal=v[2], elastic_tangential=v[3],
                    total=v[4], dissipated=v[5], evals=int(v[6]), rebuilds=int(v[7]),
                    max_neighbors=int(v[8]), status=int(v[9]), graph=bool(v[10]), variant=int(v[11]),
                    bond_elastic=v[12], fracture_released=v[13], tool_work=v[14], broken=int(v[15]))

    def pairs(self) -> np.ndarray:
        """Current candidate pairs (original ids, i < j), sorted, as an (M, 2) array."""
        cap = self.config.n * self.config.max_neighbors
        out = np.empty((cap, 2), dtype=np.int32)
        count = C.c_int64()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_read_pairs(self._h, out.ctypes.data, cap, C.byref(count), self._stream())
        _lib.check(rc, self._h, "tdem_hm_read_pairs")
        m = min(int(count.value), cap)
        pairs = out[:m].astype(np.int64)
        order = np.lexsort((pairs[:, 1], pairs[:, 0]))
        return pairs[order]

    def rebuild(self) -> None:
        """Rebuild the neighbour list now (history carried over by pair key)."""
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_rebuild(self._h, self._stream())
        _lib.check(rc, self._h, "tdem_hm_rebuild")

    def history(self) -> dict[tuple[int, int], tuple[float, float]]:
        """Non-zero tangential history per original-id pair (lo, hi): xi of lo relative to hi."""
        cap = self.config.n * self.config.max_neighbors
        pairs = np.empty((cap, 2), dtype=np.int32)
        xi = np.empty((cap, 2), dtype=np.float64)
        count = C.c_int64()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_read_history(self._h, pairs.ctypes.data, xi.ctypes.data, cap,
                                                C.byref(count), self._stream())
        _lib.check(rc, self._h, "tdem_hm_read_history")
        m = min(int(count.value), cap)
        return {(int(a), int(b)): (float(x), float(y)) for (a, b), (x, y) in zip(pairs[:m], xi[:m])}

    @property
    def variant(self) -> int:
        return int(self._lib.tdem_hm_get_variant(self._h))

    @variant.setter
    def variant(self, v: int) -> None:
        _lib.check(self._lib.tdem_hm_set_variant(self._h, int(v)), self._h, "tdem_hm_set_variant")

    def autotune(self, steps: int = 20) -> dict[int, float]:
        """Time every step-kernel variant on the live state and keep the fastest.

        The simulation advances while tuning (variants compute bit-identical
        states). Returns milliseconds per variant for ``steps`` steps.
        """
        nv = int(self._lib.tdem_hm_num_variants())
        ms = (C.c_float * nv)()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_autotune(self._h, int(steps), ms, self._stream())
        _lib.check(rc, self._h, "tdem_hm_autotune")
        self.steps += nv * (int(steps) + 2)
        return {v: float(ms[v]) for v in range(nv)}

    def step_kernel(self) -> None:
        """One step as a single plain launch of the step kernel (no rebuild)."""
        rc = self._lib.tdem_hm_step_kernel(self._h, self._stream())
        _lib.check(rc, self._h, "tdem_hm_step_kernel")
        self.steps += 1

    def rebuild_pending(self) -> bool:
        """Synchronize and report whether the list must be rebuilt before the next step."""
        r = int(self._lib.tdem_hm_rebuild_pending(self._h, self._stream()))
        if r < 0:
            _lib.check(-r, self._h, "tdem_hm_rebuild_pending")
        return r == 1

    def set_bonds(self, pairs, strength) -> None:
        """Bonds (original ids, (B, 2)) with a strength factor each; after set_state."""
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        st = np.ascontiguousarray(np.asarray(strength, dtype=np.float64).reshape(-1))
        if len(st) != len(pr):
            raise ValueError("one strength factor per bond")
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_set_bonds(self._h, pr.ctypes.data, st.ctypes.data, len(pr), self._stream())
        _lib.check(rc, self._h, "tdem_hm_set_bonds")
        self.check()

    def bonds(self) -> dict[str, np.ndarray]:
        """Bond states sorted by (lo, hi) original ids: mode (0 intact) and failure evaluation."""
        cap = self.config.n * max(self.config.max_bonds, 1)
        pairs = np.empty((cap, 2), dtype=np.int32)
        state = np.empty((cap, 2), dtype=np.int32)
        count = C.c_int64()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_read_bonds(self._h, pairs.ctypes.data, state.ctypes.data, cap,
                                              C.byref(count), self._stream())
        _lib.check(rc, self._h, "tdem_hm_read_bonds")
        m = min(int(count.value), cap)
        order = np.lexsort((pairs[:m, 1], pairs[:m, 0]))
        return dict(pairs=pairs[:m][order].astype(np.int64), mode=state[:m, 0][order],
                    fail_eval=state[:m, 1][order])

    def fragments(self) -> dict:
        """Connected components of the intact bonds, computed on the device:
        per-disc labels (the smallest original id of its fragment, original
        order), the fragment count, and each fragment's size."""
        n = self.config.n
        labels = np.empty(n, dtype=np.int32)
        count = C.c_int64()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_fragments(self._h, labels.ctypes.data, C.byref(count), self._stream())
        _lib.check(rc, self._h, "tdem_hm_fragments")
        ids, sizes = np.unique(labels, return_counts=True)
        return {"labels": labels, "count": int(count.value), "fragment_ids": ids, "sizes": sizes}

    def load_curve(self) -> np.ndarray:
        """Indenter reaction (ice on indenter) per committed evaluation, (E, 2)."""
        cap = max(self.config.load_capacity, 1)
        out = np.empty((cap, 2))
        count = C.c_int64()
        with torch.cuda.device(self.device):
            rc = self._lib.tdem_hm_read_load(self._h, out.ctypes.data, cap, C.byref(count), self._stream())
        _lib.check(rc, self._h, "tdem_hm_read_load")
        return out[:min(int(count.value), cap)].copy()


def contact_law(config: HM2DConfig, rows) -> np.ndarray:
    """The engine's per-contact Hertz-Mindlin law on a batch of pair states.

    ``rows`` is (K, 16): overlap delta, unit normal (x, y) from a to b, r_a,
    r_b, v_a (x, y), omega_a, v_b (x, y), omega_b, 1/m_a, 1/m_b, the stored
    tangential history (x, y) in a's orientation and one unused column.
    Returns (K, 8): force on a (x, y), n x F_a, the updated history (x, y),
    the step's dissipated energy, the Hertz and the spring energy; zeros for a
    pair without overlap (its history resets). Runs the step kernel's own device function
    in ``config.precision`` with ``config``'s material and time step
    (include/tdem.h, ``tdem_hm_contact_law``).
    """
    a = np.ascontiguousarray(np.asarray(rows, dtype=np.float64).reshape(-1, 16))
    out = np.empty((len(a), 8))
    lib = _lib.lib()
    rc = lib.tdem_hm_contact_law(C.byref(config.to_c()), len(a), a.ctypes.data, out.ctypes.data,
                                 torch.cuda.current_stream().cuda_stream)
    _lib.check(rc, None, "tdem_hm_contact_law")
    return out


def ice_sheet_case(nx: int = 2048, ny: int = 512, *, radius: float = 0.05, density: float = 900.0,
                   young: float = 5e9, poisson: float = 0.3, mu: float = 0.3, restitution: float = 0.5,
                   bond_damping: float = 0.05, breaking_strain: float = 0.01,
                   shear_breaking_strain: float = 0.02, strength_sigma: float = 0.1, seed: int = 0,
                   indenter_radius: float = 2.0, indenter_speed: float = 0.5, dt_factor: float = 0.1,
                   skin_factor: float = 0.1, precision: int = 32, steps: int = 20000,
                   max_neighbors: int = 8) -> tuple[HM2DConfig, dict, np.ndarray, np.ndarray]:
    """Bonded ice sheet on a hexagonal lattice, clamped at both short ends.

    nx discs per row, ny rows (row spacing sqrt(3) r, odd rows shifted by r),
    thickness 2r, 6-neighbour bonds with normal stiffness E t and shear
    stiffness E t / (2 (1 + nu)), per-bond strength factor lognormal(0, sigma)
    (numpy PCG64 ``seed``) scaling the break strains 0.01 / 0.02. The left and
    right end columns are clamped (infinite mass). A rigid circular indenter of
    radius 2 m starts just above the sheet's mid-span and moves down at
    0.5 m/s. Returns (config, state, bond pairs, strength factors).
    """
    rng = np.random.default_rng(seed)
    r = radius
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    x = (2.0 * ii + (jj % 2)) * r + 2.0 * r
    y = jj * math.sqrt(3.0) * r + 2.0 * r
    pos = np.stack((x.ravel(), y.ravel()), axis=1)
    n = nx * ny
    idx = (jj * nx + ii)
    pairs = [np.stack((idx[:, :-1].ravel(), idx[:, 1:].ravel()), axis=1)]  # along rows
    for parity in (0, 1):
        rows = np.arange(parity, ny - 1, 2)
        if parity == 0:   # even row j: partners (i-1, j+1) and (i, j+1)
            a = idx[rows][:, 1:]
            pairs += [np.stack((a.ravel(), idx[rows + 1][:, :-1].ravel()), axis=1),
                      np.stack((idx[rows].ravel(), idx[rows + 1].ravel()), axis=1)]
        else:             # odd row j: partners (i, j+1) and (i+1, j+1)
            pairs += [np.stack((idx[rows].ravel(), idx[rows + 1].ravel()), axis=1),
                      np.stack((idx[rows][:, :-1].ravel(), idx[rows + 1][:, 1:].ravel()), axis=1)]
    bonds = np.concatenate(pairs).astype(np.int64)
    bonds = np.sort(bonds, axis=1)
    bonds = bonds[np.lexsort((bonds[:, 1], bonds[:, 0]))]
    strength = np.exp(rng.normal(0.0, strength_sigma, len(bonds)))
    thickness = 2.0 * r
    mass = np.full(n, density * math.pi * r * r * thickness)
    clamped = (ii.ravel() == 0) | (ii.ravel() == nx - 1)
    mass[clamped] = np.inf
    inertia = 0.5 * mass * r * r
    radius_arr = np.full(n, r)
    kn = young * thickness
    ks = kn / (2.0 * (1.0 + poisson))
    dt = dt_factor * rayleigh_dt(r, density, young, poisson)
    skin = skin_factor * r
    width = (2.0 * nx + 1) * r + 4.0 * r
    top = (ny - 1) * math.sqrt(3.0) * r + 2.0 * r
    travel = indenter_speed * dt * steps
    height = top + r + 2.0 * indenter_radius + travel + 4.0 * r
    reach = 2.0 * r + skin
    ncx = int(math.floor(width / reach))
    ncy = int(math.floor(height / reach))
    cell = max(width / ncx, height / ncy)
    ncx = int(math.ceil(width / cell))
    ncy = int(math.ceil(height / cell))
    center = (0.5 * (x.min() + x.max()), top + r + indenter_radius + 0.02 * r)
    cfg = HM2DConfig(n=n, ncx=ncx, ncy=ncy, cell=cell, skin=skin, dt=dt, young=young, poisson=poisson,
                     restitution=restitution, mu=mu, mu_wall=mu, gravity=(0.0, 0.0), walls=0,
                     precision=precision, max_neighbors=max_neighbors, max_bonds=6, bond_kn=kn,
                     bond_ks=ks, bond_damping=bond_damping, breaking_strain=breaking_strain,
                     shear_breaking_strain=shear_breaking_strain, indenter_center=center,
                     indenter_velocity=(0.0, -indenter_speed), indenter_radius=indenter_radius,
                     load_capacity=steps + 8)
    state = dict(pos=pos, vel=np.zeros((n, 2)), omega=np.zeros(n), radius=radius_arr, mass=mass,
                 inertia=inertia)
    return cfg, state, bonds, strength
