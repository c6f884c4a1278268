"""torch custom ops over the C ABI (namespace ``tensordem_gb300``).

Each op is a thin shim: it hands the device pointers of the (contiguous CUDA)
tensors and the current CUDA stream to libtdem_sm103.so and maps its status
to the reference's exception types. The kernels mutate the state tensors in
place, which the ``mutates_args`` declarations tell torch.
"""

from __future__ import annotations

import ctypes as C
from typing import Optional

import torch

from . import _lib

_NS = "tensordem_gb300"


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _stream(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def _state(positions, velocities, initial_positions, fixed, alive, failure_mode,
           failure_time_s, failure_extension_m, failure_energy_J) -> _lib.IceDEMStateC:
    return _lib.IceDEMStateC(positions.data_ptr(), velocities.data_ptr(),
                             initial_positions.data_ptr(), fixed.data_ptr(), alive.data_ptr(),
                             failure_mode.data_ptr(), failure_time_s.data_ptr(),
                             failure_extension_m.data_ptr(), failure_energy_J.data_ptr())


_STATE_MUT = ("positions", "velocities", "alive", "failure_mode", "failure_time_s",
              "failure_extension_m", "failure_energy_J")


@torch.library.custom_op(f"{_NS}::icedem_step", mutates_args=_STATE_MUT)
def icedem_step(handle: int, positions: torch.Tensor, velocities: torch.Tensor,
                initial_positions: torch.Tensor, fixed: torch.Tensor, alive: torch.Tensor,
                failure_mode: torch.Tensor, failure_time_s: torch.Tensor,
                failure_extension_m: torch.Tensor, failure_energy_J: torch.Tensor,
                loads: Optional[torch.Tensor], n_steps: int, time: float) -> int:
    """``n_steps`` reference-mode steps from ``time`` (IceDEM.step, dem.py:347-382).

    Returns the TDEM status (0 or TDEM_ERR_NONFINITE); other errors raise.
    """
    st = _state(positions, velocities, initial_positions, fixed, alive, failure_mode,
                failure_time_s, failure_extension_m, failure_energy_J)
    rc = _lib.lib().tdem_icedem_step(C.c_void_p(handle), C.byref(st), _ptr(loads), int(n_steps),
                                     float(time), _stream(positions))
    if rc not in (_lib.TDEM_OK, _lib.TDEM_ERR_NONFINITE):
        _lib.check(rc, C.c_void_p(handle), "tdem_icedem_step")
    return int(rc)


@torch.library.custom_op(f"{_NS}::icedem_forces",
                         mutates_args=("alive", "failure_mode", "failure_time_s",
                                       "failure_extension_m", "failure_energy_J",
                                       "out_force", "out_reaction"))
def icedem_forces(handle: int, positions: torch.Tensor, velocities: torch.Tensor,
                  initial_positions: torch.Tensor, fixed: torch.Tensor, alive: torch.Tensor,
                  failure_mode: torch.Tensor, failure_time_s: torch.Tensor,
                  failure_extension_m: torch.Tensor, failure_energy_J: torch.Tensor,
                  loads: Optional[torch.Tensor], time: float, out_force: torch.Tensor,
                  out_reaction: torch.Tensor) -> None:
    """One force evaluation that commits breaks (IceDEM.forces, dem.py:226-345)."""
    st = _state(positions, velocities, initial_positions, fixed, alive, failure_mode,
                failure_time_s, failure_extension_m, failure_energy_J)
    rc = _lib.lib().tdem_icedem_forces(C.c_void_p(handle), C.byref(st), _ptr(loads), float(time),
                                       out_force.data_ptr(), out_reaction.data_ptr(),
                                       _stream(positions))
    _lib.check(rc, C.c_void_p(handle), "tdem_icedem_forces")


# ---------------------------------------------------------------------------
# Hertz-Mindlin engine (HM2D) and the batched engine (Batch). Their state lives
# in the native engine; ``anchor`` is a small CUDA tensor of the engine's
# device that gives the op its device (for dispatch and the current stream).


@torch.library.custom_op(f"{_NS}::hm_step", mutates_args=())
def hm_step(handle: int, n_steps: int, anchor: torch.Tensor) -> None:
    """``n_steps`` velocity-Verlet steps of a Hertz-Mindlin engine (one
    conditional CUDA graph launch; the step of IceDEM.step, dem.py:347-382,
    for the Hertz-Mindlin disc engine)."""
    rc = _lib.lib().tdem_hm_step(C.c_void_p(handle), int(n_steps), _stream(anchor))
    _lib.check(rc, C.c_void_p(handle), "tdem_hm_step")


@torch.library.custom_op(f"{_NS}::hm_read_state", mutates_args=("pos", "vel", "omega", "force", "torque"))
def hm_read_state(handle: int, pos: torch.Tensor, vel: torch.Tensor, omega: torch.Tensor, force: torch.Tensor,
                  torque: torch.Tensor) -> None:
    """Integer-time state of a Hertz-Mindlin engine in original disc order into
    FP64 CUDA tensors: positions, velocities, spins, forces and torques."""
    rc = _lib.lib().tdem_hm_read_state(C.c_void_p(handle), pos.data_ptr(), vel.data_ptr(), omega.data_ptr(),
                                       force.data_ptr(), torque.data_ptr(), 0, _stream(pos))
    _lib.check(rc, C.c_void_p(handle), "tdem_hm_read_state")


@torch.library.custom_op(f"{_NS}::batch_step", mutates_args=())
def batch_step(handle: int, n_steps: int, anchor: torch.Tensor) -> None:
    """``n_steps`` steps of every live instance of a batched engine (one
    conditional CUDA graph launch)."""
    rc = _lib.lib().tdem_batch_step(C.c_void_p(handle), int(n_steps), _stream(anchor))
    _lib.check(rc, C.c_void_p(handle), "tdem_batch_step")
