"""The allocation-free contact-force entry point, called through the C ABI.

Some callers cannot call cudaMalloc: code that runs while another solver's
CUDA graph is being captured, real-time coupling loops, plug-ins whose host
application owns all device memory. ``tdem_hm_contact_forces_noalloc`` serves
them from a fixed device array inside the library. These checks compare its
output with the engine's own entry points (``tdem_hm_set_state`` +
``tdem_hm_read_state``) on two calls in a row with different inputs, so that a
call that reused the previous call's scratch contents would show up.
Tolerance: 1e-6 of the largest force (both paths run the same FP32 kernels).
"""

import ctypes as C

import numpy as np
import pytest
import torch

from tests._hm_cases import dense_gas

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


def _push_contacts(st):
    # a few overlapping pairs so that contacts, not only gravity, are compared
    for a in range(0, 40, 4):
        st["pos"][a + 1] = st["pos"][a] + np.array([st["radius"][a] + st["radius"][a + 1] - 2e-6, 0.0])
    return st


def test_two_calls_in_a_row_match_the_engine(lib):
    cases = [dense_gas(24, seed=31, precision=32), dense_gas(40, seed=32, precision=32)]
    for cfg, st in cases:
        st = _push_contacts(st)
        rc, msg, f, tq = _noalloc(lib, cfg, st)
        assert rc == 0, msg
        fe, te = _engine_forces(cfg, st)
        scale = np.abs(fe).max()
        assert np.abs(f - fe).max() <= 1e-6 * scale
        assert np.abs(tq - te).max() <= 1e-6 * max(np.abs(te).max(), 1e-30) or np.abs(tq - te).max() == 0.0
        assert np.abs(fe[:, 0]).max() > 0.0  # contact forces are present, not gravity alone


def test_oversize_input_is_rejected_with_a_clear_error(lib):
    cfg, st = dense_gas(130, seed=33, precision=32)  # 16900 discs
    assert cfg.n > MAX_DISCS
    rc, msg, _, _ = _noalloc(lib, cfg, st)
    assert rc == 1 and str(MAX_DISCS) in msg
