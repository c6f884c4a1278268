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


@dataclass(frozen=True)
class DEMConfig:
    """Configuration of the 2-D bonded-disc lattice (dem.py:17-72)."""

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
        for name in ("nx", "ny"):
            value = getattr(self, name)
            if isinstance(value, bool) or not isinstance(value, int) or value < 2:
                raise ValueError(f"{name} must be an integer >= 2")
        for name in ("radius", "thickness", "density", "bond_stiffness", "contact_stiffness",
                     "breaking_strain", "shear_breaking_strain", "tool_radius", "tool_speed"):
            value = getattr(self, name)
            if not math.isfinite(value) or value <= 0:
                raise ValueError(f"{name} must be finite and positive")
        for name in ("contact_damping", "drag", "tool_gap"):
            value = getattr(self, name)
            if not math.isfinite(value) or value < 0:
                raise ValueError(f"{name} must be finite and nonnegative")
        if self.dt is not None and (not math.isfinite(self.dt) or self.dt <= 0):
            raise ValueError("dt must be finite and positive")

    @property
    def mass(self) -> float:
        return self.density * math.pi * self.radius**2 * self.thickness

    @property
    def recommended_dt(self) -> float:
        # dem.py:61-72: bounds all N-1 possible pair contacts plus the tool.
        neighbors = self.nx * self.ny - 1
        stiffness = (2 * neighbors + 1) * max(self.bond_stiffness, self.contact_stiffness)
        damping = (2 * neighbors + 1) * self.contact_damping + self.drag
        elastic_dt = 0.2 * math.sqrt(self.mass / stiffness)
        damping_dt = 0.2 * self.mass / damping if damping else math.inf
        travel_dt = 0.1 * self.radius / self.tool_speed
        return min(elastic_dt, damping_dt, travel_dt)


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
        self.dt = config.dt if config.dt is not None else config.recommended_dt
        if self.dt > config.recommended_dt:
            raise ValueError(f"dt exceeds conservative limit {config.recommended_dt:.6g} s")
        dev = self.device
        x = torch.arange(config.nx, dtype=torch.float64, device=dev)
        y = torch.arange(config.ny, dtype=torch.float64, device=dev)
        yy, xx = torch.meshgrid(y, x, indexing="ij")
        self.positions = torch.stack((xx.flatten() - (config.nx - 1) / 2, yy.flatten()), dim=1) \
            * (2 * config.radius)
        self.initial_positions = self.positions.clone()
        self.velocities = torch.zeros_like(self.positions)
        n = len(self.positions)
        self.fixed = torch.zeros(n, dtype=torch.bool, device=dev)
        if config.fix_edges:
            self.fixed = (xx.flatten() == 0) | (xx.flatten() == config.nx - 1)
        self.pairs = torch.triu_indices(n, n, offset=1, device=dev).T
        delta = self.positions[self.pairs[:, 1]] - self.positions[self.pairs[:, 0]]
        distances = torch.linalg.vector_norm(delta, dim=1)
        self.initial_normals = delta / distances[:, None]
        self.bonded = distances <= 2 * config.radius * math.sqrt(2) * (1 + 1e-10)
        self.bond_indices = self.pairs[self.bonded]
        self.reference_bond_vectors = (self.initial_positions[self.bond_indices[:, 1]]
                                       - self.initial_positions[self.bond_indices[:, 0]])
        self.rest_lengths = distances.clone()
        self.alive = self.bonded.clone()
        p = len(self.pairs)
        self.failure_mode = torch.zeros(p, dtype=torch.uint8, device=dev)
        self.failure_time_s = torch.full((p,), -1.0, dtype=torch.float64, device=dev)
        self.failure_extension_m = torch.zeros(p, dtype=torch.float64, device=dev)
        self.failure_energy_J = torch.zeros(p, dtype=torch.float64, device=dev)
        self.time = 0.0
        self.step_count = 0
        self._last_step: dict | None = {}
        self.tool_start = torch.tensor(
            [0.0, (config.ny - 1) * 2 * config.radius + config.radius + config.tool_radius
             + config.tool_gap], dtype=torch.float64, device=dev)
        self.tool_velocity = torch.tensor([0.0, -config.tool_speed], dtype=torch.float64, device=dev)
        self.hull_profile = None
        self.hull_start = torch.tensor(hull_start, dtype=torch.float64, device=dev)
        self.hull_velocity = torch.tensor(hull_velocity, dtype=torch.float64, device=dev)
        if not bool(torch.isfinite(self.hull_start).all() and torch.isfinite(self.hull_velocity).all()):
            raise ValueError("hull_start and hull_velocity must be finite")
        if hull_profile is not None:
            if not isinstance(hull_profile, torch.Tensor):
                raise TypeError("hull_profile must be a torch.Tensor with shape (M, 2)")
            if hull_profile.ndim != 2 or hull_profile.shape[1] != 2 or hull_profile.shape[0] < 2:
                raise ValueError("hull_profile must have shape (M, 2), M >= 2")
            self.hull_profile = hull_profile.to(device=dev, dtype=torch.float64).clone()
            if not bool(torch.isfinite(self.hull_profile).all()):
                raise ValueError("hull_profile must contain only finite values")
            if bool((torch.linalg.vector_norm(self.hull_profile[1:] - self.hull_profile[:-1], dim=1)
                     <= torch.finfo(self.hull_profile.dtype).eps).any()):
                raise ValueError("hull_profile must not contain zero-length segments")
        self._build_native()

    # ------------------------------------------------------------------ native
    def _build_native(self) -> None:
        cfg = self.config
        c = _lib.IceDEMConfigC()
        c.n = len(self.positions)
        c.radius, c.mass = cfg.radius, cfg.mass
        c.bond_stiffness, c.contact_stiffness = cfg.bond_stiffness, cfg.contact_stiffness
        c.breaking_strain, c.shear_breaking_strain = cfg.breaking_strain, cfg.shear_breaking_strain
        c.contact_damping, c.drag, c.tool_radius, c.dt = cfg.contact_damping, cfg.drag, cfg.tool_radius, self.dt
        ts, tv = self.tool_start.tolist(), self.tool_velocity.tolist()
        c.tool_start[0], c.tool_start[1] = ts
        c.tool_velocity[0], c.tool_velocity[1] = tv
        hs, hv = self.hull_start.tolist(), self.hull_velocity.tolist()
        c.hull_start[0], c.hull_start[1] = hs
        c.hull_velocity[0], c.hull_velocity[1] = hv
        self._hull_host = None
        if self.hull_profile is not None:
            self._hull_host = self.hull_profile.cpu().contiguous()
            c.hull_vertices = self._hull_host.shape[0]
            c.hull_profile_host = C.cast(self._hull_host.data_ptr(), C.POINTER(C.c_double))
        else:
            c.hull_vertices = 0
        self._handle = _Handle(c, self.initial_positions.cpu())
        nb = _lib.lib().tdem_icedem_num_bonds(self._handle.ptr)
        native = torch.empty(nb, dtype=torch.int64)
        _lib.lib().tdem_icedem_bond_pairs(self._handle.ptr,
                                          C.cast(native.data_ptr(), C.POINTER(C.c_int64)))
        expect = torch.nonzero(self.bonded).flatten().cpu()
        if not torch.equal(native, expect):
            raise RuntimeError("native bond topology disagrees with the lattice bond mask")

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
        """Deterministic per-bond failure records in SI units (dem.py:437-460)."""
        labels = {1: "tensile", 2: "shear", 3: "mixed"}
        mode = self.failure_mode.cpu()
        idx = torch.nonzero(mode > 0, as_tuple=False).flatten().tolist()
        pairs = self.pairs.cpu()
        pos = self.positions.cpu()
        t = self.failure_time_s.cpu()
        ext = self.failure_extension_m.cpu()
        en = self.failure_energy_J.cpu()
        events = []
        for p in idx:
            i, j = pairs[p].tolist()
            events.append({
                "pair_index": p, "particle_i": i, "particle_j": j,
                "time_s": float(t[p]), "mode": labels[int(mode[p])],
                "midpoint_m": ((pos[i] + pos[j]) * 0.5).tolist(),
                "extension_at_failure_m": float(ext[p]),
                "released_spring_energy_J": float(en[p]),
            })
        return events

    def fragments(self) -> list[dict]:
        """Connected components of the surviving bonds, isolated discs included,
        ordered by their smallest particle id (the output of dem.py:462-484):
        particle ids, mass, centroid and mean velocity per fragment."""
        from scipy.sparse import coo_matrix
        from scipy.sparse.csgraph import connected_components

        n = len(self.positions)
        ij = self.pairs[self.alive].cpu().numpy().reshape(-1, 2)
        graph = coo_matrix((np.ones(len(ij)), (ij[:, 0], ij[:, 1])), shape=(n, n))
        _, label = connected_components(graph, directed=False)
        pos = self.positions.cpu()
        vel = self.velocities.cpu()
        members: dict[int, list[int]] = {}
        for i, c in enumerate(label.tolist()):  # ascending i: member lists come out sorted
            members.setdefault(c, []).append(i)
        result = []
        for ids in sorted(members.values(), key=lambda m: m[0]):
            result.append(dict(particle_ids=ids, mass_kg=len(ids) * self.config.mass,
                               centroid_m=pos[ids].mean(0).tolist(),
                               mean_velocity_m_s=vel[ids].mean(0).tolist()))
        return result

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
        """Fail closed on missing fields, incompatible topology or nonfinite data (dem.py:504-601)."""
        if not isinstance(state, dict) or state.get("schema") != "tensordem.restart/1":
            raise ValueError("unsupported DEM restart schema")
        required = {"schema", "config", "dt_s", "time_s", "step_count", "positions_m",
                    "velocities_m_s", "initial_positions_m", "fixed", "alive", "failure_mode",
                    "failure_time_s", "failure_extension_m", "failure_energy_J", "tool_start_m",
                    "tool_velocity_m_s", "hull_profile_m", "hull_start_m", "hull_velocity_m_s",
                    "accounting", "last_step"}
        if set(state) != required:
            raise ValueError("restart fields missing or unknown")
        cfg = dict(state["config"])
        if device is not None:
            cfg["device"] = device
        if str(cfg.get("device", "cuda")).startswith("cpu"):
            cfg["device"] = "cuda"
        config = DEMConfig(**cfg)
        hull = state["hull_profile_m"]
        result = cls(config, hull_profile=None if hull is None else torch.tensor(hull, dtype=torch.float64),
                     hull_start=state["hull_start_m"], hull_velocity=state["hull_velocity_m_s"])
        if state["dt_s"] != result.dt or not math.isfinite(state["time_s"]) or state["time_s"] < 0:
            raise ValueError("invalid restart time or timestep")
        count = state["step_count"]
        if isinstance(count, bool) or not isinstance(count, int) or count < 0:
            raise ValueError("invalid restart step_count")
        if abs(state["time_s"] - count * result.dt) > 1e-10 * max(1.0, state["time_s"]):
            raise ValueError("restart time inconsistent with step count")
        for key, attribute in (("positions_m", "positions"), ("velocities_m_s", "velocities"),
                               ("initial_positions_m", "initial_positions"),
                               ("tool_start_m", "tool_start"), ("tool_velocity_m_s", "tool_velocity")):
            original = getattr(result, attribute)
            tensor = torch.tensor(state[key], dtype=torch.float64, device=result.device)
            if tensor.shape != original.shape or not bool(torch.isfinite(tensor).all()):
                raise ValueError(f"invalid restart {key}")
            if attribute == "initial_positions" and not torch.equal(tensor, original):
                raise ValueError("reference lattice mismatch")
            setattr(result, attribute, tensor)
        for key in ("fixed", "alive"):
            values = state[key]
            if not isinstance(values, list) or any(type(v) is not bool for v in values):
                raise ValueError(f"invalid boolean restart {key}")
            tensor = torch.tensor(values, dtype=torch.bool, device=result.device)
            if tensor.shape != getattr(result, key).shape:
                raise ValueError(f"invalid restart {key} shape")
            if key == "alive" and bool((tensor & ~result.bonded).any()):
                raise ValueError("nonbonded pair cannot be alive")
            if key == "fixed" and not torch.equal(tensor, result.fixed):
                raise ValueError("fixed boundary mismatch")
            setattr(result, key, tensor)
        for key in ("failure_mode", "failure_time_s", "failure_extension_m", "failure_energy_J"):
            dtype = torch.uint8 if key == "failure_mode" else torch.float64
            tensor = torch.as_tensor(state[key], dtype=dtype, device=result.device)
            if tensor.shape != getattr(result, key).shape:
                raise ValueError(f"invalid restart {key} shape")
            if key == "failure_mode":
                if bool((tensor > 3).any()) or bool((tensor[~result.bonded] != 0).any()):
                    raise ValueError("invalid restart failure modes")
                if not torch.equal(tensor > 0, result.bonded & ~result.alive):
                    raise ValueError("failure ledger inconsistent with bond state")
            else:
                if not bool(torch.isfinite(tensor).all()):
                    raise ValueError(f"nonfinite restart {key}")
                if key == "failure_time_s" and bool((tensor[result.failure_mode > 0] < 0).any()):
                    raise ValueError("failed bond has invalid failure time")
                if key == "failure_time_s" and bool((tensor[result.failure_mode == 0] != -1).any()):
                    raise ValueError("intact bond has failure time")
                if key == "failure_energy_J" and bool((tensor < 0).any()):
                    raise ValueError("negative restart failure energy")
                if key == "failure_energy_J" and bool((tensor[result.failure_mode == 0] != 0).any()):
                    raise ValueError("intact bond has failure energy")
            setattr(result, key, tensor)
        if not torch.equal(result.positions[result.fixed], result.initial_positions[result.fixed]) or \
                bool((result.velocities[result.fixed] != 0).any()):
            raise ValueError("fixed particle state mismatch")
        accounting = state["accounting"]
        expected = set(_ENERGY_KEYS) | set(_IMPULSE_KEYS)
        missing = expected - set(accounting)
        if missing - ADDITIVE_ACCOUNTING_KEYS:
            raise ValueError("restart accounting fields mismatch")
        if set(accounting) - expected:
            raise ValueError("restart accounting fields mismatch")
        for key, value in accounting.items():
            tensor = torch.as_tensor(value, dtype=torch.float64)
            expected_shape = (2,) if "impulse" in key else ()
            if tuple(tensor.shape) != expected_shape or not bool(torch.isfinite(tensor).all()):
                raise ValueError("invalid restart accounting")
            if key == "fracture_release_J" and value < 0:
                raise ValueError("negative fracture release")
        json.dumps(state["last_step"], allow_nan=False)
        acc = copy.deepcopy(accounting)
        for key in missing:
            acc[key] = 0.0
        result.accounting = acc
        result.last_step = copy.deepcopy(state["last_step"])
        result.time, result.step_count = state["time_s"], count
        return result

    @torch.no_grad()
    def mechanical_energy(self) -> dict:
        """Actual current spring/contact potential; does not advance failure (dem.py:603-624)."""
        delta = self.positions[self.pairs[:, 1]] - self.positions[self.pairs[:, 0]]
        distances = torch.linalg.vector_norm(delta, dim=1)
        extension = distances - self.rest_lengths
        overlap = (2 * self.config.radius - distances).clamp_min(0)
        bond = 0.5 * self.config.bond_stiffness * extension[self.alive].square().sum()
        contact = 0.5 * self.config.contact_stiffness * overlap[~self.alive].square().sum()
        if self.hull_profile is None:
            distance = torch.linalg.vector_norm(self.positions - self.tool_position, dim=1)
        else:
            vertices = self.hull_profile + self.tool_position
            segments = vertices[1:] - vertices[:-1]
            rel = self.positions[:, None] - vertices[None, :-1]
            fraction = ((rel * segments).sum(2) / segments.square().sum(1)).clamp(0, 1)
            nearest = vertices[None, :-1] + fraction[:, :, None] * segments
            distance = torch.linalg.vector_norm(self.positions[:, None] - nearest, dim=2).min(1).values
        tool_overlap = (self.config.radius + self.config.tool_radius - distance).clamp_min(0)
        tool = 0.5 * self.config.contact_stiffness * tool_overlap.square().sum()
        kinetic = 0.5 * self.config.mass * self.velocities.square().sum()
        return dict(kinetic_J=float(kinetic), bond_J=float(bond), pair_contact_J=float(contact),
                    tool_contact_J=float(tool), mechanical_J=float(kinetic + bond + contact + tool))
