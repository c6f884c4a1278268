"""CPU checks of the spec engine's configuration validation.

``tdem_hm_create`` and ``tdem_batch_create`` reject a bad configuration with
TDEM_ERR_BADARG and a message before any CUDA call, so these run without a
GPU. The Python layer maps the status to ValueError, as the reference's
configuration classes raise it for bad parameters
(tests/test_scale_ceiling_dem.py:94-101: no discs, restitution above 1,
negative skin; src/tensordem/dem.py:37-55).
"""

import ctypes as C
from dataclasses import replace

import pytest

from tensordem_gb300 import _lib
from tensordem_gb300.hm2d import HM2DConfig

BASE = HM2DConfig(n=1000, ncx=40, ncy=40, cell=2.5e-3, skin=2e-4, dt=1e-7, young=70e9, poisson=0.25,
                  restitution=0.8, mu=0.5, mu_wall=0.5)

CASES = [
    (dict(n=0), "n out of range"),
    (dict(max_neighbors=0), "max_neighbors must be in 1..24"),
    (dict(max_neighbors=25), "max_neighbors must be in 1..24"),
    (dict(inertia_factor=0.0), "inertia_factor must be positive"),
    (dict(max_bonds=9), "max_bonds must be in 0..8"),
    (dict(max_bonds=-1), "max_bonds must be in 0..8"),
    (dict(max_bonds=6, bond_kn=0.0, bond_ks=1.0), "invalid bond stiffness"),
    (dict(max_bonds=6, bond_kn=1.0, bond_ks=1.0, breaking_strain=0.0), "invalid bond stiffness"),
    (dict(max_bonds=6, bond_kn=1.0, bond_ks=-1.0), "invalid bond stiffness"),
    (dict(indenter_radius=-1.0), "indenter_radius must be >= 0"),
    (dict(ncx=0), "cell grid must be 1..32768 per axis"),
    (dict(ncy=40000), "cell grid must be 1..32768 per axis"),
    (dict(cell=0.0), "invalid material, cell or time-step parameter"),
    (dict(skin=-0.1), "invalid material, cell or time-step parameter"),
    (dict(dt=0.0), "invalid material, cell or time-step parameter"),
    (dict(dt=float("nan")), "invalid material, cell or time-step parameter"),
    (dict(young=0.0), "invalid material, cell or time-step parameter"),
    (dict(poisson=0.5), "invalid material, cell or time-step parameter"),
    (dict(restitution=1.5), "invalid material, cell or time-step parameter"),
    (dict(restitution=0.0), "invalid material, cell or time-step parameter"),
    (dict(mu=-0.1), "invalid material, cell or time-step parameter"),
    (dict(mu_wall=-0.1), "invalid material, cell or time-step parameter"),
    (dict(precision=16), "precision must be 32 or 64"),
    (dict(sum_precision=48), "sum_precision must be 0, 32 or 64"),
    (dict(position_remainder=2), "position_remainder must be 0 or 1"),
]


@pytest.mark.parametrize("change,message", CASES, ids=[next(iter(c)) + "=" + str(next(iter(c.values())))
                                                      for c, _ in CASES])
def test_bad_configuration_is_rejected_before_any_launch(change, message):
    lib = _lib.lib()
    h = C.c_void_p()
    rc = lib.tdem_hm_create(C.byref(replace(BASE, **change).to_c()), C.byref(h))
    assert rc == _lib.TDEM_ERR_BADARG
    assert h.value is None
    assert message in _lib.last_error("tdem_hm_create", None)
    with pytest.raises(ValueError, match=message.split(" ")[0]):
        _lib.check(rc, None, "tdem_hm_create")


def test_null_arguments_are_rejected():
    lib = _lib.lib()
    h = C.c_void_p()
    assert lib.tdem_hm_create(None, C.byref(h)) == _lib.TDEM_ERR_BADARG
    assert lib.tdem_hm_create(C.byref(BASE.to_c()), None) == _lib.TDEM_ERR_BADARG


BATCH_CASES = [
    (dict(precision=16), "precision must be 32 or 64"),
    (dict(max_neighbors=0), "max_neighbors must be in 1..24"),
    (dict(max_bonds=9), "max_bonds must be in 0..8"),
    (dict(max_instances=0), "max_instances must be in 1..1048576"),
    (dict(particle_capacity=16), "particle_capacity must be in 32..2^29-64"),
    (dict(key_capacity=1), "key_capacity must be in 2..2^31-1"),
    (dict(rebuild_every=-1), "rebuild_every must be >= 0"),
    (dict(position_remainder=2), "position_remainder must be 0 or 1"),
]


@pytest.mark.parametrize("change,message", BATCH_CASES,
                         ids=[next(iter(c)) + "=" + str(next(iter(c.values()))) for c, _ in BATCH_CASES])
def test_bad_batch_configuration_is_rejected_before_any_allocation(change, message):
    from tensordem_gb300.batch import BatchConfig
    cfg = replace(BatchConfig(particle_capacity=100_000, key_capacity=1 << 20), **change)
    lib = _lib.lib()
    h = C.c_void_p()
    rc = lib.tdem_batch_create(C.byref(cfg.to_c()), C.byref(h))
    assert rc == _lib.TDEM_ERR_BADARG
    assert h.value is None
    assert message in _lib.last_error("tdem_batch_create", None)
