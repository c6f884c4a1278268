"""Per-bond stiffness: the drop-in for the reference's ``CalibratedIceDEM``.

``CalibratedIceDEM`` keeps disc mass, contacts and failure criteria of
:class:`~tensordem_gb300.dem.IceDEM` and gives every bond its own central
spring stiffness (N/m), each at most the config's ``bond_stiffness`` so that
the inherited time-step bound stays conservative
(src/tensordem/calibrated_dem.py:11-93). The force correction
``(k_b - k) (d - L0) n`` and the corrected break energy are applied by the
reference-mode CUDA kernel (``tdem_icedem_set_bond_stiffness``) inside every
force evaluation, in the reference's summation order.
"""

from __future__ import annotations

import ctypes as C
import hashlib
import json
import struct

import torch

from . import _lib
from .dem import DEMConfig, IceDEM


class CalibratedIceDEM(IceDEM):
    """IceDEM with per-bond central-spring stiffness (bond order = pair order)."""

    def __init__(self, config: DEMConfig = DEMConfig(), *, bond_stiffness=None, **kwargs):
        super().__init__(config, **kwargs)
        if bond_stiffness is None:
            raise ValueError("explicit per-bond stiffness required")
        coefficients = torch.as_tensor(bond_stiffness, dtype=torch.float64).detach().to(self.device).clone()
        if (coefficients.shape != (len(self.bond_indices),) or not bool(torch.isfinite(coefficients).all())
                or bool((coefficients <= 0).any()) or bool((coefficients > config.bond_stiffness).any())):
            raise ValueError("per-bond stiffness shape/finite/positive/conservative upper bound mismatch")
        self.coefficients = coefficients
        self.coefficient_hash = self._hash()
        self.pair_coefficients = torch.zeros(len(self.pairs), dtype=torch.float64, device=self.device)
        self.pair_coefficients[self.bonded] = self.coefficients
        host = self.coefficients.cpu().contiguous()
        rc = _lib.lib().tdem_icedem_set_bond_stiffness(self._handle.ptr, C.cast(host.data_ptr(),
                                                       C.POINTER(C.c_double)), int(host.numel()))
        _lib.check(rc, self._handle.ptr, "tdem_icedem_set_bond_stiffness")

    def _hash(self) -> str:
        values = self.coefficients.detach().to(device="cpu", dtype=torch.float64).tolist()
        return hashlib.sha256(struct.pack(f"<{len(values)}d", *values)).hexdigest()

    def _check(self) -> None:
        """The coefficients live in the kernel: a mutated host copy is an error."""
        if (self._hash() != self.coefficient_hash
                or not torch.equal(self.pair_coefficients[self.bonded], self.coefficients)
                or bool((self.pair_coefficients[~self.bonded] != 0).any())):
            raise ValueError("per-bond stiffness mutated after construction")

    def forces(self, external_forces: torch.Tensor | None = None) -> tuple[torch.Tensor, torch.Tensor]:
        self._check()
        return super().forces(external_forces)

    def step(self, external_forces: torch.Tensor | None = None, *, load_time: float | None = None) -> None:
        self._check()
        super().step(external_forces, load_time=load_time)

    def run(self, steps: int) -> None:
        self._check()
        super().run(steps)

    def mechanical_energy(self) -> dict:
        """The energy record; the kernel sums the bond springs with the
        per-bond stiffness it holds (calibrated_dem.py:79-93)."""
        self._check()
        return super().mechanical_energy()

    def snapshot(self) -> dict:
        """Restart record, schema ``tensordem.calibrated-restart/1``."""
        self._check()
        return dict(schema="tensordem.calibrated-restart/1", base=IceDEM.snapshot(self),
                    bond_stiffness_N_per_m=self.coefficients.tolist(), coefficient_sha256=self.coefficient_hash)

    @classmethod
    def from_snapshot(cls, state: dict, *, device: str | None = None) -> "CalibratedIceDEM":
        if (not isinstance(state, dict)
                or set(state) != {"schema", "base", "bond_stiffness_N_per_m", "coefficient_sha256"}
                or state["schema"] != "tensordem.calibrated-restart/1"):
            raise ValueError("invalid calibrated restart schema/fields")
        json.dumps(state, allow_nan=False)
        base = IceDEM.from_snapshot(state["base"], device=device)
        result = cls(base.config, bond_stiffness=state["bond_stiffness_N_per_m"], hull_profile=base.hull_profile,
                     hull_start=tuple(base.hull_start.tolist()), hull_velocity=tuple(base.hull_velocity.tolist()))
        if result.coefficient_hash != state["coefficient_sha256"]:
            raise ValueError("calibrated restart coefficient hash mismatch")
        for name in ("positions", "velocities", "alive", "failure_mode", "failure_time_s", "failure_extension_m",
                     "failure_energy_J", "tool_start", "tool_velocity"):
            setattr(result, name, getattr(base, name).clone())
        result.time = base.time
        result.step_count = base.step_count
        result.accounting = base.accounting
        result.last_step = base.last_step
        return result
