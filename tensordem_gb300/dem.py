"""Drop-in ``DEMConfig`` / ``IceDEM`` on the GB300 CUDA path (reference mode).

Same public surface as the reference's ``tensordem.dem`` (src/tensordem/dem.py
and its frozen binder contract, src/tensordem/binding_contract.py:86-202):
state tensors ``positions``, ``velocities``, ``initial_positions``, ``fixed``,
the all-pairs ``pairs`` / ``bonded`` / ``alive`` and fracture ledger, the
``accounting`` dict, ``step``, ``forces``, ``diagnostics``, ``exchange_state``,
``snapshot`` / ``from_snapshot``, ``mechanical_energy``, ``fracture_events``,
``fragments``. The step itself runs in the FP64 CUDA kernel of
``csrc/icedem.cu`` through the torch custom ops of :mod:`tensordem_gb300.ops`.

Differences from the reference, by design:
* CUDA only. ``device`` defaults to ``"cuda"``; any other device raises
  ``ValueError`` (there is no CPU fallback).
* ``accounting`` and ``last_step`` live on the device and are read on access
  (each read synchronizes the stream).
* ``run(steps)`` advances many steps in one kernel launch.
"""

from __future__ import annotations

import copy
import ctypes as C
import json
import math
from dataclasses import asdict, dataclass

import numpy as np
import torch

from . import _lib, ops

ADDITIVE_ACCOUNTING_KEYS = frozenset({"pair_contact_acquired_J"})
_ENERGY_KEYS = ("external_work_J", "fracture_release_J", "pair_contact_acquired_J",
                "tool_work_J", "damping_dissipation_J")
_IMPULSE_KEYS = ("external_impulse_Ns", "support_impulse_Ns", "drag_impulse_Ns",
                 "tool_impulse_on_ice_Ns")


# Configuration checks: (fields, predicate, message template). The messages
# are the reference's, which callers match on (src/tensordem/dem.py:37-55).
_CONFIG_RULES = (
    (("nx", "ny"), lambda v: not isinstance(v, bool) and isinstance(v, int) and v >= 2,
     "{} must be an integer >= 2"),
    (("radius", "thickness", "density", "bond_stiffness", "contact_stiffness", "breaking_strain",
      "shear_breaking_strain", "tool_radius", "tool_speed"), lambda v: math.isfinite(v) and v > 0,
     "{} must be finite and positive"),
    (("contact_damping", "drag", "tool_gap"), lambda v: math.isfinite(v) and v >= 0,
     "{} must be finite and nonnegative"),
    (("dt",), lambda v: v is None or (math.isfinite(v) and v > 0), "{} must be finite and positive"),
)


@dataclass(frozen=True)
class DEMConfig:
    """Configuration of the 2-D bonded-disc lattice (fields and defaults of dem.py:17-35)."""

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
    device: str = "cuda"
    fix_edges: bool = True

    def __post_init__(self) -> None:
        for fields, ok, message in _CONFIG_RULES:
            for name in fields:
                if not ok(getattr(self, name)):
                    raise ValueError(message.format(name))

    @property
    def mass(self) -> float:
        """Disc mass rho pi r^2 t (kg)."""
        return self.density * math.pi * self.radius**2 * self.thickness

    @property
    def recommended_dt(self) -> float:
        """The reference's conservative step (dem.py:61-72): the smallest of an
        elastic bound that assumes every other disc may touch (2 (N - 1) + 1
        springs at the stiffer constant), the matching damping bound, and a
        tenth of a radius of tool travel."""
        springs = 2 * (self.nx * self.ny - 1) + 1
        k_max = springs * max(self.bond_stiffness, self.contact_stiffness)
        c_sum = springs * self.contact_damping + self.drag
        bounds = [0.2 * math.sqrt(self.mass / k_max), 0.1 * self.radius / self.tool_speed]
        if c_sum:
            bounds.insert(1, 0.2 * self.mass / c_sum)
        return min(bounds)


def _square_lattice(config: DEMConfig, device) -> dict:
    """The reference's lattice (dem.py:105-131): nx x ny discs on a square grid
    of spacing 2r centred on x = 0, row by row from y = 0; every pair (i < j)
    in upper-triangle order with its initial distance and unit normal; the two
    end columns fixed when ``fix_edges``. Distances use torch's vector norm,
    as the reference does."""
    nx, ny, spacing = config.nx, config.ny, 2 * config.radius
    column = torch.arange(nx, dtype=torch.float64, device=device).repeat(ny)
    row = torch.arange(ny, dtype=torch.float64, device=device).repeat_interleave(nx)
    positions = torch.stack((column - (nx - 1) / 2, row), dim=1) * spacing
    count = nx * ny
    pairs = torch.triu_indices(count, count, offset=1, device=device).T
    chord = positions[pairs[:, 1]] - positions[pairs[:, 0]]
    length = torch.linalg.vector_norm(chord, dim=1)
    edge = (column == 0) | (column == nx - 1)
    return dict(positions=positions, pairs=pairs, length=length, normal=chord / length[:, None],
                fixed=edge if config.fix_edges else torch.zeros_like(edge))


def _check_hull(profile, start, velocity, device):
    """Validated hull placement and polyline (dem.py:146-170 semantics)."""
    start = torch.tensor(start, dtype=torch.float64, device=device)
    velocity = torch.tensor(velocity, dtype=torch.float64, device=device)
    if not bool(torch.isfinite(start).all() and torch.isfinite(velocity).all()):
        raise ValueError("hull_start and hull_velocity must be finite")
    if profile is None:
        return None, start, velocity
    if not isinstance(profile, torch.Tensor):
        raise TypeError("hull_profile must be a torch.Tensor with shape (M, 2)")
    if profile.ndim != 2 or profile.shape[1] != 2 or profile.shape[0] < 2:
        raise ValueError("hull_profile must have shape (M, 2), M >= 2")
    profile = profile.to(device=device, dtype=torch.float64).clone()
    if not bool(torch.isfinite(profile).all()):
        raise ValueError("hull_profile must contain only finite values")
    seg = torch.linalg.vector_norm(profile[1:] - profile[:-1], dim=1)
    if bool((seg <= torch.finfo(torch.float64).eps).any()):
        raise ValueError("hull_profile must not contain zero-length segments")
    return profile, start, velocity


_RESTART_KEYS = frozenset({
    "schema", "config", "dt_s", "time_s", "step_count", "positions_m", "velocities_m_s", "initial_positions_m",
    "fixed", "alive", "failure_mode", "failure_time_s", "failure_extension_m", "failure_energy_J",
    "tool_start_m", "tool_velocity_m_s", "hull_profile_m", "hull_start_m", "hull_velocity_m_s", "accounting",
    "last_step"})


def _restart_array(values, kind, device):
    """A restart list as a device tensor of its kind, or None if it is not one:
    "f64" finite float64, "bool" a list of Python bools, "mode" uint8."""
    if kind == "bool":
        if not isinstance(values, list) or any(type(v) is not bool for v in values):
            return None
        return torch.tensor(values, dtype=torch.bool, device=device)
    t = torch.as_tensor(values, dtype=torch.uint8 if kind == "mode" else torch.float64, device=device)
    if kind == "f64" and not bool(torch.isfinite(t).all()):
        return None
    return t


def _intact(sim):
    return sim.failure_mode == 0


# Restored arrays in restore order (later checks see earlier fields already
# restored): snapshot key, IceDEM attribute, kind, [(check(sim, value), message)].
_RESTART_ARRAYS = (
    ("positions_m", "positions", "f64", ()),
    ("velocities_m_s", "velocities", "f64", ()),
    ("initial_positions_m", "initial_positions", "f64",
     ((lambda sim, v: torch.equal(v, sim.initial_positions), "reference lattice mismatch"),)),
    ("tool_start_m", "tool_start", "f64", ()),
    ("tool_velocity_m_s", "tool_velocity", "f64", ()),
    ("fixed", "fixed", "bool", ((lambda sim, v: torch.equal(v, sim.fixed), "fixed boundary mismatch"),)),
    ("alive", "alive", "bool", ((lambda sim, v: not bool((v & ~sim.bonded).any()), "nonbonded pair cannot be alive"),)),
    ("failure_mode", "failure_mode", "mode",
     ((lambda sim, v: not bool((v > 3).any()) and not bool((v[~sim.bonded] != 0).any()),
       "invalid restart failure modes"),
      (lambda sim, v: torch.equal(v > 0, sim.bonded & ~sim.alive), "failure ledger inconsistent with bond state"))),
    ("failure_time_s", "failure_time_s", "f64",
     ((lambda sim, v: not bool((v[~_intact(sim)] < 0).any()), "failed bond has invalid failure time"),
      (lambda sim, v: not bool((v[_intact(sim)] != -1).any()), "intact bond has failure time"))),
    ("failure_extension_m", "failure_extension_m", "f64", ()),
    ("failure_energy_J", "failure_energy_J", "f64",
     ((lambda sim, v: not bool((v < 0).any()), "negative restart failure energy"),
      (lambda sim, v: not bool((v[_intact(sim)] != 0).any()), "intact bond has failure energy"))),
)


def _restart_accounting(accounting) -> dict:
    """The restart's accounting dict, checked against the ledger's channels;
    channels added after a checkpoint was written restore as zero."""
    expected = set(_ENERGY_KEYS) | set(_IMPULSE_KEYS)
    if not isinstance(accounting, dict) or set(accounting) - expected or \
            (expected - set(accounting)) - ADDITIVE_ACCOUNTING_KEYS:
        raise ValueError("restart accounting fields mismatch")
    out = {key: 0.0 for key in expected - set(accounting)}
    for key, value in accounting.items():
        t = torch.as_tensor(value, dtype=torch.float64)
        if tuple(t.shape) != ((2,) if "impulse" in key else ()) or not bool(torch.isfinite(t).all()):
            raise ValueError("invalid restart accounting")
        if key == "fracture_release_J" and value < 0:
            raise ValueError("negative fracture release")
        out[key] = copy.deepcopy(value)
    return out


class _Handle:
    """Owns one native reference-mode instance."""

    def __init__(self, cfg_c: _lib.IceDEMConfigC, x0_host: torch.Tensor):
        lib = _lib.lib()
        ptr = C.c_void_p()
        x0 = x0_host.contiguous()
        rc = lib.tdem_icedem_create(C.byref(cfg_c),
                                    C.cast(x0.data_ptr(), C.POINTER(C.c_double)), C.byref(ptr))
        _lib.check(rc, None, "tdem_icedem_create")
        self.ptr = ptr
        self.value = ptr.value

    def __del__(self):
        if getattr(self, "ptr", None) is not None and _lib._lib is not None:
            _lib._lib.tdem_icedem_destroy(self.ptr)
            self.ptr = None


class IceDEM:
    """A small ice lattice stepped on the GPU (dem.py:75-84).

    Positions, velocities and externally applied forces have shape (N, 2).
    External forces use SI newtons in the global x/y frame and are evaluated
    at the current step (not accumulated internally). Bond and contact forces
    are central and equal/opposite. Tensile failure uses axial bond strain;
    shear failure uses an objective local Green-Lagrange strain invariant.
    """

    def __init__(self, config: DEMConfig = DEMConfig(), *, hull_profile: torch.Tensor | None = None,
                 hull_start: tuple[float, float] = (0.0, 0.0),
                 hull_velocity: tuple[float, float] = (0.0, 0.0)) -> None:
        self.config = config
        self.device = torch.device(config.device)
        if self.device.type != "cuda":
            raise ValueError("tensordem_gb300.IceDEM runs on CUDA devices only")
        if not torch.cuda.is_available():
            raise ValueError("CUDA requested but unavailable")
        limit = config.recommended_dt
        self.dt = limit if config.dt is None else config.dt
        if self.dt > limit:
            raise ValueError(f"dt exceeds conservative limit {limit:.6g} s")
        dev = self.device
        self.hull_profile, self.hull_start, self.hull_velocity = _check_hull(hull_profile, hull_start,
                                                                             hull_velocity, dev)
        lattice = _square_lattice(config, dev)
        self.positions = lattice["positions"]
        self.initial_positions = self.positions.clone()
        self.velocities = torch.zeros_like(self.positions)
        self.fixed = lattice["fixed"]
        self.pairs = lattice["pairs"]
        self.rest_lengths = lattice["length"]
        self.initial_normals = lattice["normal"]
        top = (config.ny - 1) * 2 * config.radius + config.radius
        self.tool_start = torch.tensor([0.0, top + config.tool_radius + config.tool_gap], dtype=torch.float64,
                                       device=dev)
        self.tool_velocity = torch.tensor([0.0, -config.tool_speed], dtype=torch.float64, device=dev)
        # the native engine builds the bond topology (bonds: pairs at most
        # 2 r sqrt(2) apart); the Python side mirrors its pair list as a mask
        self._build_native()
        npair = len(self.pairs)
        self.bonded = torch.zeros(npair, dtype=torch.bool, device=dev)
        self.bonded[self._bond_pair_index.to(dev)] = True
        self.bond_indices = self.pairs[self.bonded]
        self.reference_bond_vectors = (self.initial_positions[self.bond_indices[:, 1]]
                                       - self.initial_positions[self.bond_indices[:, 0]])
        self.alive = self.bonded.clone()
        self.failure_mode = torch.zeros(npair, dtype=torch.uint8, device=dev)
        self.failure_time_s = torch.full((npair,), -1.0, dtype=torch.float64, device=dev)
        self.failure_extension_m = torch.zeros(npair, dtype=torch.float64, device=dev)
        self.failure_energy_J = torch.zeros(npair, dtype=torch.float64, device=dev)
        self.time = 0.0
        self.step_count = 0
        self._last_step: dict | None = {}

    # ------------------------------------------------------------------ native
    def _build_native(self) -> None:
        cfg = self.config
        c = _lib.IceDEMConfigC()
        c.n = len(self.positions)
        c.radius, c.mass = cfg.radius, cfg.mass
        c.bond_stiffness, c.contact_stiffness = cfg.bond_stiffness, cfg.contact_stiffness
        c.breaking_strain, c.shear_breaking_strain = cfg.breaking_strain, cfg.shear_breaking_strain
        c.contact_damping, c.drag, c.tool_radius, c.dt = cfg.contact_damping, cfg.drag, cfg.tool_radius, self.dt
        c.tool_start[0], c.tool_start[1] = self.tool_start.tolist()
        c.tool_velocity[0], c.tool_velocity[1] = self.tool_velocity.tolist()
        c.hull_start[0], c.hull_start[1] = self.hull_start.tolist()
        c.hull_velocity[0], c.hull_velocity[1] = self.hull_velocity.tolist()
        self._hull_host = None
        c.hull_vertices = 0
        if self.hull_profile is not None:
            self._hull_host = self.hull_profile.cpu().contiguous()
            c.hull_vertices = self._hull_host.shape[0]
            c.hull_profile_host = C.cast(self._hull_host.data_ptr(), C.POINTER(C.c_double))
        self._handle = _Handle(c, self.initial_positions.cpu())
        nb = _lib.lib().tdem_icedem_num_bonds(self._handle.ptr)
        index = torch.empty(nb, dtype=torch.int64)
        _lib.lib().tdem_icedem_bond_pairs(self._handle.ptr, C.cast(index.data_ptr(), C.POINTER(C.c_int64)))
        self._bond_pair_index = index

    def _tensor(self, name: str, dtype: torch.dtype, shape: tuple) -> torch.Tensor:
        t = getattr(self, name)
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{name} must be a torch.Tensor")
        if tuple(t.shape) != shape:
            raise ValueError(f"{name} must have shape {shape}")
        if t.device != self.device or t.dtype != dtype or not t.is_contiguous():
            t = t.to(device=self.device, dtype=dtype).contiguous()
            setattr(self, name, t)
        return t

    def _state_args(self):
        n = len(self.initial_positions)
        p = len(self.pairs)
        return (self._tensor("positions", torch.float64, (n, 2)),
                self._tensor("velocities", torch.float64, (n, 2)),
                self._tensor("initial_positions", torch.float64, (n, 2)),
                self._tensor("fixed", torch.bool, (n,)),
                self._tensor("alive", torch.bool, (p,)),
                self._tensor("failure_mode", torch.uint8, (p,)),
                self._tensor("failure_time_s", torch.float64, (p,)),
                self._tensor("failure_extension_m", torch.float64, (p,)),
                self._tensor("failure_energy_J", torch.float64, (p,)))

    def _ledger(self) -> list[float]:
        buf = (C.c_double * _lib.L_COUNT)()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        rc = _lib.lib().tdem_icedem_read_ledger(self._handle.ptr, buf, _lib.L_COUNT, stream)
        _lib.check(rc, self._handle.ptr, "tdem_icedem_read_ledger")
        return list(buf)

    def _write_ledger(self, values: list[float]) -> None:
        buf = (C.c_double * len(values))(*values)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        rc = _lib.lib().tdem_icedem_write_ledger(self._handle.ptr, buf, len(values), stream)
        _lib.check(rc, self._handle.ptr, "tdem_icedem_write_ledger")

    # ------------------------------------------------------------- properties
    @property
    def accounting(self) -> dict:
        led = self._ledger()
        acc = {k: led[i] for i, k in enumerate(_ENERGY_KEYS)}
        for q, k in enumerate(_IMPULSE_KEYS):
            acc[k] = [led[_lib.L_IMPULSES + 2 * q], led[_lib.L_IMPULSES + 2 * q + 1]]
        return acc

    @accounting.setter
    def accounting(self, value: dict) -> None:
        led = self._ledger()
        for i, k in enumerate(_ENERGY_KEYS):
            led[i] = float(value.get(k, 0.0))
        for q, k in enumerate(_IMPULSE_KEYS):
            pair = value.get(k, [0.0, 0.0])
            led[_lib.L_IMPULSES + 2 * q] = float(pair[0])
            led[_lib.L_IMPULSES + 2 * q + 1] = float(pair[1])
        self._write_ledger(led)

    def accounting_vector(self) -> list[float]:
        """The 13 accounting numbers in the reference's dict order."""
        return self._ledger()[:13]

    @property
    def last_step(self) -> dict:
        if self._last_step is not None:
            return self._last_step
        led = self._ledger()
        return dict(time_start_s=led[_lib.L_LAST_TIME_START], time_end_s=led[_lib.L_LAST_TIME_END],
                    external_work_J=led[_lib.L_LAST_EXTERNAL_WORK],
                    support_force_N=led[_lib.L_LAST_SUPPORT:_lib.L_LAST_SUPPORT + 2],
                    tool_reaction_N=led[_lib.L_LAST_REACTION:_lib.L_LAST_REACTION + 2],
                    external_force_N=led[_lib.L_LAST_EXTERNAL:_lib.L_LAST_EXTERNAL + 2],
                    external_moment_Nm=led[_lib.L_LAST_EXTERNAL_MOMENT])

    @last_step.setter
    def last_step(self, value: dict) -> None:
        self._last_step = copy.deepcopy(value)

    @property
    def min_break_margin(self) -> float:
        """Smallest relative distance of a surviving bond to a break threshold so far."""
        return self._ledger()[_lib.L_MIN_BREAK_MARGIN]

    @property
    def tool_position(self) -> torch.Tensor:
        if self.hull_profile is not None:
            return self.hull_start + self.time * self.hull_velocity
        return self.tool_start + self.time * self.tool_velocity

    @property
    def broken_bonds(self) -> int:
        return int((self.bonded & ~self.alive).sum().item())

    def bond_alive(self) -> torch.Tensor:
        return self.alive[self.bonded]

    def failure_ledger(self):
        b = self.bonded
        return (self.failure_mode[b], self.failure_time_s[b], self.failure_extension_m[b],
                self.failure_energy_J[b])

    # --------------------------------------------------------------- stepping
    def _validate_external_forces(self, external_forces):
        if external_forces is None:
            return None
        if not isinstance(external_forces, torch.Tensor):
            raise TypeError("external_forces must be a torch.Tensor with shape (N, 2)")
        if tuple(external_forces.shape) != tuple(self.positions.shape):
            raise ValueError(f"external_forces must have shape {tuple(self.positions.shape)}")
        loads = external_forces.to(device=self.device, dtype=torch.float64).contiguous()
        if not bool(torch.isfinite(loads).all()):
            raise ValueError("external_forces must contain only finite values")
        return loads

    @torch.no_grad()
    def forces(self, external_forces: torch.Tensor | None = None) -> tuple[torch.Tensor, torch.Tensor]:
        """Return total particle force and ice-on-tool reaction (dem.py:226-345)."""
        loads = self._validate_external_forces(external_forces)
        args = self._state_args()
        force = torch.empty_like(args[0])
        reaction = torch.empty(2, dtype=torch.float64, device=self.device)
        ops.icedem_forces(self._handle.value, *args, loads, float(self.time), force, reaction)
        return force, reaction

    def _advance_clock(self, steps: int) -> None:
        for _ in range(steps):
            self.time += self.dt
            self.step_count += 1

    @torch.no_grad()
    def step(self, external_forces: torch.Tensor | None = None, *, load_time: float | None = None) -> None:
        """Semi-implicit Euler; optional nodal loads are supplied in newtons."""
        if load_time is not None and (not math.isfinite(load_time) or
                                      abs(load_time - self.time) > 1e-12 * max(1.0, abs(self.time))):
            raise ValueError("load_time must equal current DEM time in seconds")
        loads = self._validate_external_forces(external_forces)
        self._run(1, loads)

    @torch.no_grad()
    def run(self, steps: int) -> None:
        """Advance ``steps`` unloaded steps in one kernel launch."""
        if isinstance(steps, bool) or not isinstance(steps, int) or steps < 1:
            raise ValueError("steps must be a positive integer")
        self._run(steps, None)

    def _run(self, steps: int, loads) -> None:
        args = self._state_args()
        rc = ops.icedem_step(self._handle.value, *args, loads, steps, float(self.time))
        self._last_step = None
        if rc == _lib.TDEM_ERR_NONFINITE:
            # the kernel stops after finishing the first non-finite step
            self._advance_clock(_lib.lib().tdem_icedem_steps_done(self._handle.ptr))
            raise FloatingPointError("Non-finite simulation state; reduce dt")
        self._advance_clock(steps)

    # ------------------------------------------------------------ diagnostics
    @torch.no_grad()
    def diagnostics(self, external_forces: torch.Tensor | None = None) -> dict[str, float | int]:
        force, reaction = self.forces(external_forces=external_forces)
        boundary_reaction = -force[self.fixed].sum(dim=0)
        acc = self.accounting
        tool = self.tool_position
        return {
            "time": self.time,
            "tool_x": float(tool[0].item()),
            "tool_y": float(tool[1].item()),
            "reaction_x": float(reaction[0].item()),
            "reaction_y": float(reaction[1].item()),
            "boundary_reaction_x": float(boundary_reaction[0].item()),
            "boundary_reaction_y": float(boundary_reaction[1].item()),
            "broken_bonds": self.broken_bonds,
            "kinetic_energy": float((0.5 * self.config.mass * self.velocities.square().sum()).item()),
            "tool_impulse_on_ice_x_Ns": float(acc["tool_impulse_on_ice_Ns"][0]),
            "tool_impulse_on_ice_y_Ns": float(acc["tool_impulse_on_ice_Ns"][1]),
            "support_impulse_x_Ns": float(acc["support_impulse_Ns"][0]),
            "support_impulse_y_Ns": float(acc["support_impulse_Ns"][1]),
            "drag_impulse_x_Ns": float(acc["drag_impulse_Ns"][0]),
            "drag_impulse_y_Ns": float(acc["drag_impulse_Ns"][1]),
            "external_impulse_x_Ns": float(acc["external_impulse_Ns"][0]),
            "external_impulse_y_Ns": float(acc["external_impulse_Ns"][1]),
            "fracture_release_J": float(acc["fracture_release_J"]),
            "pair_contact_acquired_J": float(acc["pair_contact_acquired_J"]),
            "tool_work_J": float(acc["tool_work_J"]),
            "damping_dissipation_J": float(acc["damping_dissipation_J"]),
            "external_work_J": float(acc["external_work_J"]),
        }

    def exchange_state(self) -> dict:
        """SI global x/y state at t_n; supplied forces are held over [t_n, t_n+dt]."""
        return dict(schema="tensordem.exchange/1", time_s=self.time, dt_s=self.dt,
                    positions_m=self.positions.tolist(), velocities_m_s=self.velocities.tolist(),
                    masses_kg=[self.config.mass] * len(self.positions),
                    fixed=self.fixed.tolist(), particle_radius_m=self.config.radius,
                    thickness_m=self.config.thickness)

    def fracture_events(self) -> list[dict]:
        """Per-bond failure records in SI units, in pair order (the records of
        dem.py:437-460). The broken bonds, their endpoints, midpoints and
        failure data are gathered on the device and copied once."""
        broken = torch.nonzero(self.failure_mode > 0).flatten()
        ends = self.pairs[broken]
        mid = 0.5 * (self.positions[ends[:, 0]] + self.positions[ends[:, 1]])
        ints = torch.cat((broken[:, None], ends, self.failure_mode[broken, None].long()), dim=1).cpu().tolist()
        reals = torch.stack((self.failure_time_s[broken], mid[:, 0], mid[:, 1], self.failure_extension_m[broken],
                             self.failure_energy_J[broken]), dim=1).cpu().tolist()
        names = {1: "tensile", 2: "shear", 3: "mixed"}
        return [{"pair_index": p, "particle_i": i, "particle_j": j, "time_s": t, "mode": names[m],
                 "midpoint_m": [mx, my], "extension_at_failure_m": e, "released_spring_energy_J": w}
                for (p, i, j, m), (t, mx, my, e, w) in zip(ints, reals)]

    def fragments(self) -> list[dict]:
        """Connected components of the surviving bonds, isolated discs included,
        ordered by their smallest disc id (the output of dem.py:462-484): disc
        ids, mass, centroid and mean velocity of each. The components come from
        a union-find kernel over the intact bonds (``tdem_icedem_fragments``);
        the per-fragment means are device reductions."""
        n = len(self.positions)
        labels = np.empty(n, dtype=np.int32)
        alive = self._tensor("alive", torch.bool, (len(self.pairs),))
        stream = torch.cuda.current_stream(self.device).cuda_stream
        rc = _lib.lib().tdem_icedem_fragments(self._handle.ptr, alive.data_ptr(), labels.ctypes.data, stream)
        _lib.check(rc, self._handle.ptr, "tdem_icedem_fragments")
        roots, inverse, counts = torch.unique(torch.from_numpy(labels).to(self.device, torch.int64),
                                              return_inverse=True, return_counts=True)
        sums = torch.zeros((len(roots), 4), dtype=torch.float64, device=self.device)
        sums.index_add_(0, inverse, torch.cat((self.positions, self.velocities), dim=1))
        means = (sums / counts[:, None]).cpu().tolist()
        members = np.split(np.argsort(labels, kind="stable"), np.cumsum(counts.cpu().numpy())[:-1])
        return [dict(particle_ids=ids.tolist(), mass_kg=len(ids) * self.config.mass, centroid_m=m[:2],
                     mean_velocity_m_s=m[2:]) for ids, m in zip(members, means)]

    def snapshot(self) -> dict:
        """Complete JSON restart (schema tensordem.restart/1, dem.py:486-502)."""
        return dict(schema="tensordem.restart/1", config=asdict(self.config),
                    dt_s=self.dt, time_s=self.time, step_count=self.step_count,
                    positions_m=self.positions.tolist(), velocities_m_s=self.velocities.tolist(),
                    initial_positions_m=self.initial_positions.tolist(), fixed=self.fixed.tolist(),
                    alive=self.alive.tolist(), failure_mode=self.failure_mode.tolist(),
                    failure_time_s=self.failure_time_s.tolist(),
                    failure_extension_m=self.failure_extension_m.tolist(),
                    failure_energy_J=self.failure_energy_J.tolist(),
                    tool_start_m=self.tool_start.tolist(), tool_velocity_m_s=self.tool_velocity.tolist(),
                    hull_profile_m=None if self.hull_profile is None else self.hull_profile.tolist(),
                    hull_start_m=self.hull_start.tolist(), hull_velocity_m_s=self.hull_velocity.tolist(),
                    accounting=copy.deepcopy(self.accounting), last_step=copy.deepcopy(self.last_step))

    @classmethod
    def from_snapshot(cls, state: dict, *, device: str | None = None) -> "IceDEM":
        """Restore a tensordem.restart/1 record; fail closed (ValueError) on a
        missing or unknown field, an incompatible lattice or a non-finite or
        inconsistent value (the checks of dem.py:504-601, driven by the field
        table ``_RESTART_ARRAYS``)."""
        if not isinstance(state, dict) or state.get("schema") != "tensordem.restart/1":
            raise ValueError("unsupported DEM restart schema")
        if set(state) != _RESTART_KEYS:
            raise ValueError("restart fields missing or unknown")
        cfg = dict(state["config"])
        if device is not None:
            cfg["device"] = device
        if str(cfg.get("device", "cuda")).startswith("cpu"):
            cfg["device"] = "cuda"
        hull = state["hull_profile_m"]
        sim = cls(DEMConfig(**cfg), hull_profile=None if hull is None else torch.tensor(hull, dtype=torch.float64),
                  hull_start=state["hull_start_m"], hull_velocity=state["hull_velocity_m_s"])
        t, count = state["time_s"], state["step_count"]
        if state["dt_s"] != sim.dt or not math.isfinite(t) or t < 0:
            raise ValueError("invalid restart time or timestep")
        if isinstance(count, bool) or not isinstance(count, int) or count < 0:
            raise ValueError("invalid restart step_count")
        if abs(t - count * sim.dt) > 1e-10 * max(1.0, t):
            raise ValueError("restart time inconsistent with step count")
        for key, attr, kind, checks in _RESTART_ARRAYS:
            value = _restart_array(state[key], kind, sim.device)
            if value is None or value.shape != getattr(sim, attr).shape:
                raise ValueError(f"invalid restart {key}")
            for check, message in checks:
                if not check(sim, value):
                    raise ValueError(message)
            setattr(sim, attr, value)
        pinned = sim.fixed
        if not torch.equal(sim.positions[pinned], sim.initial_positions[pinned]) or \
                bool((sim.velocities[pinned] != 0).any()):
            raise ValueError("fixed particle state mismatch")
        sim.accounting = _restart_accounting(state["accounting"])
        json.dumps(state["last_step"], allow_nan=False)
        sim.last_step = copy.deepcopy(state["last_step"])
        sim.time, sim.step_count = t, count
        return sim

    @torch.no_grad()
    def mechanical_energy(self) -> dict:
        """Stored energy of the current state without advancing failure
        (the record of dem.py:603-624), summed on the device by
        ``tdem_icedem_energy``: kinetic, intact-bond springs, penalty energy
        of overlapping pairs that are not intact bonds, tool penalty energy."""
        pos, vel = self._tensor("positions", torch.float64, tuple(self.initial_positions.shape)), \
            self._tensor("velocities", torch.float64, tuple(self.initial_positions.shape))
        alive = self._tensor("alive", torch.bool, (len(self.pairs),))
        out = (C.c_double * 5)()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        rc = _lib.lib().tdem_icedem_energy(self._handle.ptr, pos.data_ptr(), vel.data_ptr(), alive.data_ptr(),
                                           float(self.time), out, stream)
        _lib.check(rc, self._handle.ptr, "tdem_icedem_energy")
        return dict(kinetic_J=out[0], bond_J=out[1], pair_contact_J=out[2], tool_contact_J=out[3],
                    mechanical_J=out[4])
