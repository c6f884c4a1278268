"""ctypes binding of libtdem_sm103.so (the C ABI declared in include/tdem.h).

There is no fallback: if the library is missing or fails to load, every call
raises. The library is built in-tree by ``tensordem_gb300.build``.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from .build import LIB

TDEM_OK = 0
TDEM_ERR_BADARG = 1
TDEM_ERR_CUDA = 2
TDEM_ERR_NONFINITE = 3
TDEM_ERR_CAPACITY = 4
TDEM_ERR_STATE = 5

# Ledger slots (include/tdem.h, TDEM_L_*)
L_EXTERNAL_WORK = 0
L_FRACTURE_RELEASE = 1
L_CONTACT_ACQUIRED = 2
L_TOOL_WORK = 3
L_DAMPING_DISSIPATION = 4
L_IMPULSES = 5  # 8 values: external, support, drag, tool (x, y each)
L_LAST_SUPPORT = 13
L_LAST_REACTION = 15
L_LAST_EXTERNAL = 17
L_LAST_EXTERNAL_WORK = 19
L_LAST_EXTERNAL_MOMENT = 20
L_LAST_TIME_START = 21
L_LAST_TIME_END = 22
L_DAMPING_POWER = 23
L_TOOL_POWER = 24
L_MIN_BREAK_MARGIN = 25
L_COUNT = 32


class IceDEMConfigC(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("radius", C.c_double), ("mass", C.c_double),
        ("bond_stiffness", C.c_double), ("contact_stiffness", C.c_double),
        ("breaking_strain", C.c_double), ("shear_breaking_strain", C.c_double),
        ("contact_damping", C.c_double), ("drag", C.c_double),
        ("tool_radius", C.c_double), ("dt", C.c_double),
        ("tool_start", C.c_double * 2), ("tool_velocity", C.c_double * 2),
        ("hull_vertices", C.c_int32),
        ("hull_profile_host", C.POINTER(C.c_double)),
        ("hull_start", C.c_double * 2), ("hull_velocity", C.c_double * 2),
    ]


class IceDEMStateC(C.Structure):
    _fields_ = [
        ("positions", C.c_void_p), ("velocities", C.c_void_p),
        ("initial_positions", C.c_void_p), ("fixed", C.c_void_p),
        ("alive", C.c_void_p), ("failure_mode", C.c_void_p),
        ("failure_time_s", C.c_void_p), ("failure_extension_m", C.c_void_p),
        ("failure_energy_J", C.c_void_p),
    ]


class HMConfigC(C.Structure):
    _fields_ = [
        ("n", C.c_int32), ("precision", C.c_int32), ("max_neighbors", C.c_int32),
        ("walls", C.c_int32), ("ncx", C.c_int32), ("ncy", C.c_int32),
        ("cell", C.c_double), ("skin", C.c_double), ("dt", C.c_double),
        ("young", C.c_double), ("poisson", C.c_double), ("restitution", C.c_double),
        ("mu", C.c_double), ("mu_wall", C.c_double), ("gravity", C.c_double * 2),
        ("inertia_factor", C.c_double),
        ("max_bonds", C.c_int32), ("bond_kn", C.c_double), ("bond_ks", C.c_double),
        ("bond_damping", C.c_double), ("breaking_strain", C.c_double),
        ("shear_breaking_strain", C.c_double), ("indenter_center", C.c_double * 2),
        ("indenter_velocity", C.c_double * 2), ("indenter_radius", C.c_double),
        ("load_capacity", C.c_int32), ("sum_precision", C.c_int32), ("position_remainder", C.c_int32),
    ]


class BatchConfigC(C.Structure):
    _fields_ = [
        ("precision", C.c_int32), ("max_neighbors", C.c_int32), ("max_bonds", C.c_int32),
        ("max_instances", C.c_int32), ("particle_capacity", C.c_int64), ("key_capacity", C.c_int64),
        ("rebuild_every", C.c_int32), ("position_remainder", C.c_int32),
    ]


class IceDEM3DConfigC(C.Structure):
    _fields_ = [
        ("n", C.c_int32), ("nbond", C.c_int32), ("hertz", C.c_int32), ("damping", C.c_int32),
        ("hertz_tangential", C.c_int32), ("rolling", C.c_int32), ("platens", C.c_int32),
        ("body", C.c_int32), ("n_branches", C.c_int32), ("creep", C.c_int32), ("any_fixed", C.c_int32),
        ("radius", C.c_double), ("mass", C.c_double), ("dt", C.c_double), ("drag", C.c_double),
        ("bond_k", C.c_double), ("branch_k", C.c_double * 4), ("branch_tau", C.c_double * 4),
        ("branch_decay", C.c_double * 4), ("branch_one_minus", C.c_double * 4),
        ("breaking_strain", C.c_double), ("shear_breaking_strain", C.c_double),
        ("creep_exponent", C.c_double), ("creep_dt_over_time", C.c_double),
        ("contact_k", C.c_double), ("hertz_kn", C.c_double), ("hertz_kn_rigid", C.c_double),
        ("hertz_pot", C.c_double), ("tangential_k", C.c_double), ("hertz_kt", C.c_double),
        ("damping_c", C.c_double), ("gamma_mobile", C.c_double), ("gamma_pinned", C.c_double),
        ("mass_mobile", C.c_double), ("mass_pinned", C.c_double),
        ("cone", C.c_int32), ("platen_cone", C.c_int32),
        ("cone_c", C.c_double * 3), ("platen_cone_c", C.c_double * 3),
        ("roll_mu", C.c_double), ("tool_radius", C.c_double), ("tool_damping", C.c_double),
        ("tool_start", C.c_double * 3), ("tool_velocity", C.c_double * 3),
        ("platen_k", C.c_double), ("platen_c", C.c_double), ("platen_kt", C.c_double),
        ("top_start_z", C.c_double), ("top_velocity", C.c_double),
        ("bottom_start_z", C.c_double), ("bottom_velocity", C.c_double),
        ("lateral_k", C.c_double), ("lateral_c", C.c_double),
        ("gravity_force", C.c_double), ("buoyancy_force", C.c_double), ("wet_drag", C.c_double),
        ("water_level", C.c_double), ("cap_denominator", C.c_double),
        ("mindlin", C.c_int32), ("pad3", C.c_int32), ("mindlin_platen_8g", C.c_double),
        ("rigid_radius", C.c_double), ("rigid_4e", C.c_double),
    ]


class IceDEM3DTopologyC(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in (
        "bond_i", "bond_j", "rest_length", "reference", "initial_normal", "threshold",
        "creep_reference", "pinv", "full_rank")]


class IceDEM3DStateC(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in (
        "positions", "velocities", "initial_positions", "fixed", "alive", "failure_mode",
        "failure_time_s", "failure_extension_m", "failure_energy_J", "branch_offsets",
        "elongation_prev", "damage", "bond_dissipation", "top_tangential", "bottom_tangential",
        "lateral_position", "lateral_velocity")]


# 3-D reference-mode ledger slots (TDEM_L3_*)
L3_REACTION, L3_TOP, L3_BOTTOM, L3_LATERAL = 0, 3, 4, 5
L3_FRICTION_POWER, L3_ROLLING_POWER, L3_CONTACT_ENERGY, L3_CONTACTS = 9, 10, 11, 12
L3_HISTORY_MAX, L3_STEPS_DONE, L3_STATUS, L3_MIN_BREAK_MARGIN = 13, 14, 15, 16
L3_COUNT = 20
CONE_OFF, CONE_SINGLE, CONE_TANH, CONE_DUAL = 0, 1, 2, 3


# Batched engine: extra ledger slots (TDEM_BATCH_L_*) and info slots (TDEM_BATCH_I_*)
BATCH_PEAK_LOAD, BATCH_PEAK_EVAL, BATCH_REACTION_X, BATCH_REACTION_Y = 16, 17, 18, 19
BATCH_L_COUNT = 20
BATCH_INFO = ("live_particles", "live_instances", "evals", "rebuilds", "tiles", "particle_capacity",
              "bytes", "key_hi", "status", "variant", "graph", "max_neighbors")

# Hertz-Mindlin ledger slots (TDEM_HM_L_*)
HM_KINETIC, HM_POTENTIAL, HM_HERTZ, HM_TANGENTIAL, HM_TOTAL, HM_DISSIPATED = range(6)
HM_EVALS, HM_REBUILDS, HM_MAX_NEIGHBORS, HM_STATUS = 6, 7, 8, 9
HM_COUNT = 16

_lock = threading.Lock()
_lib: C.CDLL | None = None


def _declare(lib: C.CDLL) -> None:
    vp, i32, dbl = C.c_void_p, C.c_int, C.c_double
    sig = {
        "tdem_version": (i32, []),
        "tdem_icedem_max_discs": (i32, []),
        "tdem_icedem_create": (i32, [C.POINTER(IceDEMConfigC), C.POINTER(C.c_double), C.POINTER(vp)]),
        "tdem_icedem_destroy": (None, [vp]),
        "tdem_icedem_num_bonds": (i32, [vp]),
        "tdem_icedem_bond_pairs": (i32, [vp, C.POINTER(C.c_int64)]),
        "tdem_icedem_set_bond_stiffness": (i32, [vp, C.POINTER(C.c_double), i32]),
        "tdem_icedem_forces": (i32, [vp, C.POINTER(IceDEMStateC), vp, dbl, vp, vp, vp]),
        "tdem_icedem_step": (i32, [vp, C.POINTER(IceDEMStateC), vp, i32, dbl, vp]),
        "tdem_icedem_steps_done": (i32, [vp]),
        "tdem_icedem_read_ledger": (i32, [vp, C.POINTER(C.c_double), i32, vp]),
        "tdem_icedem_write_ledger": (i32, [vp, C.POINTER(C.c_double), i32, vp]),
        "tdem_icedem_last_error": (i32, [vp, C.c_char_p, C.c_size_t]),
        "tdem_icedem_energy": (i32, [vp, vp, vp, vp, dbl, C.POINTER(C.c_double), vp]),
        "tdem_icedem_fragments": (i32, [vp, vp, vp, vp]),
        "tdem_icedem_ledger_to_device": (i32, [vp, vp, vp]),
        "tdem_icedem3d_max_particles": (i32, []),
        "tdem_icedem3d_create": (i32, [C.POINTER(IceDEM3DConfigC), C.POINTER(IceDEM3DTopologyC),
                                       C.POINTER(vp)]),
        "tdem_icedem3d_destroy": (None, [vp]),
        "tdem_icedem3d_forces": (i32, [vp, C.POINTER(IceDEM3DStateC), vp, dbl, i32, i32, vp, vp]),
        "tdem_icedem3d_step": (i32, [vp, C.POINTER(IceDEM3DStateC), vp, C.c_int64, dbl, vp]),
        "tdem_icedem3d_read_ledger": (i32, [vp, C.POINTER(C.c_double), i32, vp]),
        "tdem_icedem3d_read_contacts": (i32, [vp, vp, C.c_int64, C.POINTER(C.c_int64), vp]),
        "tdem_icedem3d_set_history": (i32, [vp, vp, vp, C.c_int64, vp]),
        "tdem_icedem3d_read_history": (i32, [vp, vp, vp, C.c_int64, C.POINTER(C.c_int64), vp]),
        "tdem_icedem3d_last_error": (i32, [vp, C.c_char_p, C.c_size_t]),
        "tdem_icedem3d_set_mapping": (i32, [vp, i32]),
        "tdem_hertz_damping_ratio": (i32, [dbl, C.POINTER(C.c_double)]),
        "tdem_hm_create": (i32, [C.POINTER(HMConfigC), C.POINTER(vp)]),
        "tdem_hm_destroy": (None, [vp]),
        "tdem_hm_set_state": (i32, [vp, vp, vp, vp, vp, vp, vp, i32, vp]),
        "tdem_hm_step": (i32, [vp, C.c_int64, vp]),
        "tdem_hm_read_state": (i32, [vp, vp, vp, vp, vp, vp, i32, vp]),
        "tdem_hm_read_ledger": (i32, [vp, C.POINTER(C.c_double), i32, vp]),
        "tdem_hm_status": (i32, [vp, vp]),
        "tdem_hm_read_pairs": (i32, [vp, vp, C.c_int64, C.POINTER(C.c_int64), vp]),
        "tdem_hm_use_graph": (i32, [vp, i32]),
        "tdem_hm_num_variants": (i32, []),
        "tdem_hm_step_kernel": (i32, [vp, vp]),
        "tdem_hm_set_bonds": (i32, [vp, vp, vp, C.c_int64, vp]),
        "tdem_hm_read_bonds": (i32, [vp, vp, vp, C.c_int64, C.POINTER(C.c_int64), vp]),
        "tdem_hm_read_load": (i32, [vp, vp, C.c_int64, C.POINTER(C.c_int64), vp]),
        "tdem_hm_fragments": (i32, [vp, vp, C.POINTER(C.c_int64), vp]),
        "tdem_hm_rebuild_pending": (i32, [vp, vp]),
        "tdem_hm_set_variant": (i32, [vp, i32]),
        "tdem_hm_get_variant": (i32, [vp]),
        "tdem_hm_autotune": (i32, [vp, i32, C.POINTER(C.c_float), vp]),
        "tdem_hm_rebuild": (i32, [vp, vp]),
        "tdem_hm_read_history": (i32, [vp, vp, vp, C.c_int64, C.POINTER(C.c_int64), vp]),
        "tdem_hm_last_error": (i32, [vp, C.c_char_p, C.c_size_t]),
        "tdem_hm_contact_law": (i32, [C.POINTER(HMConfigC), C.c_int64, vp, vp, vp]),
        "tdem_hm_set_wait_budget": (i32, [vp, C.c_int64]),
        "tdem_icedem3d_set_barrier_spins": (i32, [vp, C.c_uint64]),
        "tdem_batch_bytes": (i32, [C.POINTER(BatchConfigC), C.POINTER(C.c_int64)]),
        "tdem_batch_create": (i32, [C.POINTER(BatchConfigC), C.POINTER(vp)]),
        "tdem_batch_destroy": (None, [vp]),
        "tdem_batch_admit": (i32, [vp, C.POINTER(HMConfigC), vp, vp, vp, vp, vp, vp, vp, vp, C.c_int64,
                                   C.POINTER(C.c_int32), vp]),
        "tdem_batch_step": (i32, [vp, C.c_int64, vp]),
        "tdem_batch_read": (i32, [vp, C.c_int32, vp, vp, vp, vp, vp, vp, C.c_int32, vp]),
        "tdem_batch_retire": (i32, [vp, C.c_int32, vp]),
        "tdem_batch_set_steps": (i32, [vp, C.c_int32, C.c_int64, vp]),
        "tdem_batch_read_ledgers": (i32, [vp, vp, C.c_int32, vp, vp]),
        "tdem_batch_read_bonds": (i32, [vp, C.c_int32, vp, vp, C.c_int64, C.POINTER(C.c_int64), vp]),
        "tdem_batch_info": (i32, [vp, C.POINTER(C.c_int64), C.c_int32, vp]),
        "tdem_batch_num_variants": (i32, []),
        "tdem_batch_set_variant": (i32, [vp, i32]),
        "tdem_batch_get_variant": (i32, [vp]),
        "tdem_batch_autotune": (i32, [vp, i32, C.POINTER(C.c_float), vp]),
        "tdem_batch_use_graph": (i32, [vp, i32]),
        "tdem_batch_last_error": (i32, [vp, C.c_char_p, C.c_size_t]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def lib() -> C.CDLL:
    """Load (once) and return the native library; raise if it is absent."""
    global _lib
    with _lock:
        if _lib is None:
            path = Path(LIB)
            if not path.exists():
                raise RuntimeError(
                    f"{path} is missing: build it with `python -m tensordem_gb300.build` "
                    "(CUDA toolkit with sm_103a support required); there is no CPU fallback")
            handle = C.CDLL(str(path), mode=C.RTLD_GLOBAL)
            _declare(handle)
            _lib = handle
    return _lib


def last_error(fn_name: str, handle) -> str:
    buf = C.create_string_buffer(1024)
    if fn_name.startswith("tdem_hm"):
        lib().tdem_hm_last_error(handle, buf, len(buf))
    elif fn_name.startswith("tdem_batch"):
        lib().tdem_batch_last_error(handle, buf, len(buf))
    elif fn_name.startswith("tdem_icedem3d"):
        lib().tdem_icedem3d_last_error(handle, buf, len(buf))
    else:
        lib().tdem_icedem_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, handle, what: str) -> None:
    """Map a TDEM status to the reference's exception types."""
    if rc == TDEM_OK:
        return
    msg = last_error(what, handle) or what
    if rc == TDEM_ERR_BADARG:
        raise ValueError(msg)
    if rc == TDEM_ERR_NONFINITE:
        raise FloatingPointError(msg)
    raise RuntimeError(f"{what}: {msg} (status {rc})")
