"""Bounded device waits that run out: the kernel returns, the status is set,
the host raises, and the engine recovers.

No fault is provoked: the waits are the real ones of the kernels, given a
test-only budget short enough that they give up before the data they wait
for arrives (copies in flight are drained before a block exits).

* Hertz-Mindlin engine, bulk-copy step variants (4, 5: own-state tiles;
  6: the neighbour window), ``tdem_hm_set_wait_budget``: an mbarrier wait of
  0 cycles runs out, the step loop stops, ``check()`` raises the timeout, and
  after a normal budget and a fresh ``set_state`` the engine steps to the same
  bits as a fresh engine.
* 3-D cooperative step, ``tdem_icedem3d_set_barrier_spins``: a grid barrier
  allowed no wait runs out in every block but the last to arrive, each block
  returns, the step raises "grid barrier timed out", and with the default
  limit restored the next step runs from a restored state to the same bits as
  an untouched copy.
"""

import numpy as np
import pytest
import torch

from tests._hm_cases import dense_gas

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def libs():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300 import _lib, hm2d
    return _lib, hm2d


def _fresh(hm2d, cfg, st, variant):
    e = hm2d.HM2D(cfg)
    e.variant = variant
    e.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
    return e


@pytest.mark.parametrize("variant", [4, 5, 6])
def test_bulk_copy_wait_runs_out_and_the_engine_recovers(libs, variant):
    _lib, hm2d = libs
    cfg, st = dense_gas(64, seed=41, precision=32)   # 4096 discs: several tiles and window blocks
    e = _fresh(hm2d, cfg, st, variant)
    e.step(3)
    assert _lib.lib().tdem_hm_set_wait_budget(e._h, 0) == 0
    with pytest.raises(RuntimeError, match="bounded wait"):
        e.step(5)
    assert e.ledger()["status"] & 16  # the timeout bit
    # normal budget, state uploaded again: the engine steps as a fresh one
    assert _lib.lib().tdem_hm_set_wait_budget(e._h, 2_000_000_000) == 0
    e.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
    e.step(20)
    ref = _fresh(hm2d, cfg, st, variant)
    ref.step(20)
    assert e.ledger()["status"] == 0
    a, b = e.state(), ref.state()
    for k in ("pos", "vel", "omega"):
        assert torch.equal(a[k], b[k]), k


def test_grid_barrier_runs_out_and_the_next_launch_is_clean(libs):
    _lib, _ = libs
    from tensordem_gb300.dem3d import DEM3DConfig, IceDEM3D
    kw = dict(nx=20, ny=10, nz=6, breaking_strain=0.004, shear_breaking_strain=0.008, device="cuda")
    sim = IceDEM3D(DEM3DConfig(**kw))
    twin = IceDEM3D(DEM3DConfig(**kw))
    sim.run(5)
    twin.run(5)
    saved = sim.state_dict()
    assert _lib.lib().tdem_icedem3d_set_barrier_spins(sim._handle.ptr, 0) == 0
    with pytest.raises(RuntimeError, match="grid barrier"):
        sim.run(3)
    assert _lib.lib().tdem_icedem3d_set_barrier_spins(sim._handle.ptr, 1 << 24) == 0
    sim.load_state_dict(saved)
    sim.run(10)
    twin.run(10)
    assert torch.equal(sim.positions, twin.positions)
    assert torch.equal(sim.velocities, twin.velocities)
    assert np.array_equal(sim.alive.cpu().numpy(), twin.alive.cpu().numpy())
