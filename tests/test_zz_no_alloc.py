"""The allocation-free contact-force entry point, called through the C ABI.

Some callers cannot call cudaMalloc: plug-ins whose host application owns all
device memory, and real-time coupling loops in which an allocation's latency
or failure cannot be accepted. ``tdem_hm_contact_forces_noalloc`` serves them
from a fixed device array inside the library. These checks compare its output
with the engine's own entry points (``tdem_hm_set_state`` +
``tdem_hm_read_state``) and with the FP64 oracle on two calls in a row with
different inputs, so that a call that reused the previous call's scratch
contents would show up. They also check that bad configurations are rejected
before any launch and that a call which ended in a capacity error leaves the
shared array usable for the next call.

Tolerances: 1e-6 of the largest force against the engine (both paths run the
same FP32 kernels); 2e-3 normwise against the FP64 oracle evaluated at the
FP32-representable positions the path holds (the FP32 single-evaluation bound
of the engine's own tests).
"""

import ctypes as C
import math

import numpy as np
import pytest
import torch

from tests._hm_cases import dense_gas, oracle_for

pytestmark = pytest.mark.gpu

MAX_DISCS = 16384


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300 import _lib
    handle = _lib.lib()
    fn = handle.tdem_hm_contact_forces_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(_lib.HMConfigC)] + [C.c_void_p] * 8 + [C.c_char_p, C.c_size_t, C.c_void_p]
    return handle


def _noalloc(lib, cfg, st):
    dev = torch.device("cuda")
    t = {k: torch.as_tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev) for k, v in st.items()}
    force = torch.empty((cfg.n, 2), dtype=torch.float64, device=dev)
    torque = torch.empty(cfg.n, dtype=torch.float64, device=dev)
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.tdem_hm_contact_forces_noalloc(
        C.byref(cfg.to_c()), t["pos"].data_ptr(), t["vel"].data_ptr(), t["omega"].data_ptr(),
        t["radius"].data_ptr(), t["mass"].data_ptr(), t["inertia"].data_ptr(), force.data_ptr(),
        torque.data_ptr(), err, len(err), stream)
    return rc, err.value.decode(), force.cpu().numpy(), torque.cpu().numpy()


def _engine_forces(cfg, st):
    from tensordem_gb300.hm2d import HM2D
    e = HM2D(cfg)
    e.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
    s = e.state()
    return s["force"].cpu().numpy(), s["torque"].cpu().numpy()


def _fp32_positions(cfg, pos):
    """The positions the FP32 path holds: an integer cell origin plus an FP32
    offset, as the pack kernel forms them."""
    c = float(np.float32(cfg.cell))
    cx = np.clip(np.floor(pos[:, 0] / c), 0, cfg.ncx - 1)
    cy = np.clip(np.floor(pos[:, 1] / c), 0, cfg.ncy - 1)
    ox = (pos[:, 0] - cx * c).astype(np.float32).astype(np.float64)
    oy = (pos[:, 1] - cy * c).astype(np.float32).astype(np.float64)
    return np.stack((cx * c + ox, cy * c + oy), axis=1)


def _push_contacts(st):
    # a few overlapping pairs so that contacts, not only gravity, are compared
    for a in range(0, 40, 4):
        st["pos"][a + 1] = st["pos"][a] + np.array([st["radius"][a] + st["radius"][a + 1] - 2e-6, 0.0])
    return st


def _check_against_engine(lib, cfg, st):
    rc, msg, f, tq = _noalloc(lib, cfg, st)
    assert rc == 0, msg
    fe, te = _engine_forces(cfg, st)
    scale = np.abs(fe).max()
    assert np.abs(f - fe).max() <= 1e-6 * scale
    assert np.abs(tq - te).max() <= 1e-6 * max(np.abs(te).max(), 1e-30) or np.abs(tq - te).max() == 0.0
    assert np.abs(fe[:, 0]).max() > 0.0  # contact forces are present, not gravity alone
    return f, tq


def test_two_calls_in_a_row_match_the_engine_and_the_oracle(lib):
    cases = [dense_gas(24, seed=31, precision=32), dense_gas(40, seed=32, precision=32)]
    for cfg, st in cases:
        st = _push_contacts(st)
        f, tq = _check_against_engine(lib, cfg, st)
        o = oracle_for(cfg, dict(st, pos=_fp32_positions(cfg, st["pos"])))
        fo, to, _ = o.evaluate(o.pos, o.vel, o.omega, advance=False)
        err_f = np.abs(f - fo).max() / np.abs(fo).max()
        err_t = np.abs(tq - to).max() / max(np.abs(to).max(), 1e-300)
        print(f"allocation-free path vs FP64 oracle: force {err_f:.2e}, torque {err_t:.2e}")
        assert err_f <= 2e-3 and err_t <= 2e-3


def test_oversize_input_is_rejected_with_a_clear_error(lib):
    cfg, st = dense_gas(130, seed=33, precision=32)  # 16900 discs
    assert cfg.n > MAX_DISCS
    rc, msg, _, _ = _noalloc(lib, cfg, st)
    assert rc == 1 and str(MAX_DISCS) in msg


def test_bad_configurations_are_rejected_before_any_launch(lib):
    from tensordem_gb300.hm2d import HM2DConfig
    cfg, st = dense_gas(16, seed=34, precision=32)
    # a grid far wider than the cell-id packing allows (the key count would
    # wrap in 32-bit arithmetic), a negative skin and friction, bonds
    for bad, words in ((dict(ncx=134_217_729, ncy=32), "32768"), (dict(skin=-1e-6), "invalid"),
                       (dict(mu=-0.1), "invalid"), (dict(max_bonds=6, bond_kn=1e6, bond_ks=1e6), "max_bonds"),
                       (dict(ncx=300, ncy=300), "256 x 256")):
        rc, msg, _, _ = _noalloc(lib, HM2DConfig(**{**cfg.__dict__, **bad}), st)
        assert rc == 1 and words in msg, (bad, rc, msg)
    # the array is untouched by the rejected calls: a valid call still matches
    _check_against_engine(lib, cfg, _push_contacts(st))


def _crowded_state(cfg, st):
    """Twelve discs on a ring of radius 1.95 r around disc 0: disc 0 has
    twelve candidate partners, more than the path's eight slots."""
    st = {k: np.array(v, copy=True) for k, v in st.items()}
    r = float(st["radius"].max())
    c = np.array([0.5 * cfg.box[0], 0.5 * cfg.box[1]])
    st["radius"][:13] = r
    st["mass"][:13] = 2500.0 * math.pi * r**2 * (2 * r)
    st["inertia"][:13] = 0.5 * st["mass"][:13] * r**2
    ang = 2.0 * math.pi * np.arange(12) / 12.0
    st["pos"][0] = c
    st["pos"][1:13] = c + 1.95 * r * np.stack((np.cos(ang), np.sin(ang)), axis=1)
    # keep every other disc out of the crowd's reach
    far = np.linalg.norm(st["pos"][13:] - c, axis=1) < 6 * r
    st["pos"][13:][far] = st["pos"][13:][far] + np.array([8 * r, 0.0])
    return st


def test_capacity_errors_leave_the_array_usable(lib):
    cfg, st = dense_gas(24, seed=35, precision=32)
    rc, msg, _, _ = _noalloc(lib, cfg, _crowded_state(cfg, st))
    assert rc == 4 and "candidate partners" in msg, (rc, msg)
    # the next valid call on the same array is correct
    _check_against_engine(lib, cfg, _push_contacts(dict(st)))
    # a disc far outside the cell grid
    st2 = {k: np.array(v, copy=True) for k, v in st.items()}
    st2["pos"][5] = (cfg.box[0] + 5.0 * cfg.cell, 0.5 * cfg.box[1])
    rc, msg, _, _ = _noalloc(lib, cfg, st2)
    assert rc == 4 and "outside the cell grid" in msg, (rc, msg)
    _check_against_engine(lib, cfg, _push_contacts(dict(st)))
