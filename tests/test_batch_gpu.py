"""GPU parity of the batched ragged engine (csrc/batch.cu).

* Inside a mixed batch, an FP64 instance matches the FP64 oracle with the
  single-solve engine's bounds: single evaluation 1e-12 normwise, trajectory
  bounds growing with the horizon (chaos), ledger within 1e-6 of the total.
* Bonded FP64 instance in a mixed batch: break table (pairs, modes, break
  evaluations) identical to the oracle's.
* FP32 bonded instance: peak indenter load within 1% of the FP64 oracle;
  before the first break, ledger residual within 1e-6 of the work input.
* With a fixed rebuild interval (rebuild_every) that the displacement bound
  never overrides, an FP32 instance's results are bit-identical alone and in
  any mix, including across admissions and retirements of other instances.
"""

import numpy as np
import pytest
import torch

from tests._hm_cases import bonded_oracle_for, dense_gas, oracle_for, small_sheet

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bt():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300 import batch
    return batch


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _batch(bt, precision=64, every=0, cap=200_000, keys=2_000_000, slots=64):
    return bt.Batch(bt.BatchConfig(particle_capacity=cap, key_capacity=keys, max_instances=slots,
                                   max_neighbors=16, max_bonds=6, precision=precision, rebuild_every=every))


def _inst(bt, cfg, st, bonds=None, strength=None):
    return bt.Instance(cfg, st, bonds, strength)


def _others(bt, precision):
    """Two unrelated instances that share the batch: a slower gas and a sheet."""
    from tensordem_gb300.hm2d import granular_gas_case
    g_cfg, g_st = granular_gas_case(20, seed=21, sigma_v=0.5, precision=precision)
    s_cfg, s_st, s_b, s_s = small_sheet(16, 6, precision=precision, steps=400, speed=5.0)
    return [_inst(bt, g_cfg, g_st), _inst(bt, s_cfg, s_st, s_b, s_s)]


def test_batch_fp64_single_evaluation_matches_oracle(bt):
    cfg, st = dense_gas(24, seed=4, precision=64)
    st["pos"][1] = st["pos"][0] + np.array([st["radius"][0] + st["radius"][1] - 3e-6, 0.0])
    b = _batch(bt)
    for o in _others(bt, 64):
        b.admit(o)
    iid = b.admit(_inst(bt, cfg, st))
    s = b.read(iid)
    o = oracle_for(cfg, st)
    f, tq, _ = o.evaluate(o.pos, o.vel, o.omega, advance=False)
    assert _rel(s["force"], f) <= 1e-12
    assert _rel(s["torque"], tq) <= 1e-12 or np.abs(tq).max() == 0.0
    assert s["ledger"]["status"] == 0


def test_batch_fp64_trajectory_matches_oracle_in_a_mix(bt):
    cfg, st = dense_gas(24, seed=7, precision=64)
    b = _batch(bt)
    others = [b.admit(o) for o in _others(bt, 64)]
    iid = b.admit(_inst(bt, cfg, st))
    o = oracle_for(cfg, st)
    bounds = {1: (1e-14, 1e-12, 1e-12), 50: (1e-11, 1e-7, 1e-6), 200: (1e-9, 1e-5, 1e-4),
              400: (1e-8, 1e-4, 1e-3)}
    done = 0
    for stop, (bp, bv, bf) in bounds.items():
        b.step(stop - done)
        o.step(stop - done)
        done = stop
        s = b.read(iid)
        errs = (_rel(s["pos"], o.pos), _rel(s["vel"], o.vel), _rel(s["force"], o.force))
        print(f"batch fp64 vs oracle after {stop} steps: pos {errs[0]:.2e} vel {errs[1]:.2e} force {errs[2]:.2e}")
        assert errs[0] <= bp and errs[1] <= bv and errs[2] <= bf, (stop, errs)
    led = s["ledger"]
    ref = o.energies()
    assert led["evals"] == 400 and led["status"] == 0
    for k_g, k_o in (("kinetic", "kinetic"), ("potential", "potential"), ("hertz", "elastic_normal"),
                     ("dissipated", "dissipated"), ("total", "total")):
        assert abs(led[k_g] - ref[k_o]) <= 1e-6 * abs(ref["total"]), k_g
    assert b.info()["rebuilds"] >= 2
    for k in others:
        assert b.read(k, state=False)["ledger"]["status"] == 0
    # the many-instance read-back gives the same ledgers as one-by-one reads
    many = b.ledgers([iid, *others])
    for k, got in zip([iid, *others], many):
        one = b.read(k, state=False)["ledger"]
        for name in ("kinetic", "potential", "hertz", "dissipated", "total", "evals", "peak_load"):
            assert got[name] == one[name], (k, name)


def _oracle_bond_table(o):
    order = np.lexsort((o.bj, o.bi))
    return (np.stack((o.bi[order], o.bj[order]), axis=1), o.fail_mode[order].astype(np.int32),
            o.fail_eval[order].astype(np.int32))


def test_batch_bonded_fp64_matches_oracle(bt):
    cfg, st, bonds, strength = small_sheet(24, 8, precision=64, steps=400, speed=20.0)
    b = _batch(bt)
    b.admit(_others(bt, 64)[0])
    iid = b.admit(_inst(bt, cfg, st, bonds, strength))
    o = bonded_oracle_for(cfg, st, bonds, strength)
    table = None
    done = 0
    peak_o = 0.0
    for stop in (1, 100, 200):
        for _ in range(stop - 1 - o.steps):
            o.step(1)
            peak_o = max(peak_o, float(np.hypot(*o.reaction)))
        table = _oracle_bond_table(o)
        o.step(1)
        peak_o = max(peak_o, float(np.hypot(*o.reaction)))
        b.step(stop - done)
        done = stop
        s = b.read(iid)
        errs = (_rel(s["pos"], o.pos), _rel(s["vel"], o.vel))
        print(f"batch fp64 bonded after {stop}: pos {errs[0]:.2e} vel {errs[1]:.2e}")
        assert errs[0] <= 1e-9 and errs[1] <= 1e-6, (stop, errs)
    got = b.bonds(iid)
    pairs, mode, fail = table
    assert np.array_equal(got["pairs"], pairs)
    assert np.array_equal(got["mode"], mode)
    assert np.array_equal(got["fail_eval"], fail)
    assert (mode > 0).sum() > 20
    led, ref = s["ledger"], o.energies()
    scale = max(o.tool_work, 1e-30)
    for k_g, k_o in (("kinetic", "kinetic"), ("bond_elastic", "bond_elastic"),
                     ("fracture_released", "fracture_released"), ("dissipated", "dissipated")):
        assert abs(led[k_g] - ref[k_o]) <= 1e-6 * scale, k_g
    assert abs(led["tool_work"] - o.tool_work) <= 1e-6 * scale
    # the engine's Hertz energy includes the indenter contact
    assert abs(led["hertz"] - ref["elastic_normal"] - ref["tool_elastic"]) <= 1e-6 * scale
    assert abs(led["total"] - ref["total"]) <= 1e-6 * scale
    assert abs(led["peak_load"] - peak_o) <= 1e-9 * peak_o


def test_batch_fp32_bonded_peak_load_within_one_percent(bt):
    cfg, st, bonds, strength = small_sheet(24, 8, precision=32, steps=600, speed=20.0)
    b = _batch(bt, precision=32)
    for o in _others(bt, 32):
        b.admit(o)
    iid = b.admit(_inst(bt, cfg, st, bonds, strength))
    o = bonded_oracle_for(cfg, st, bonds, strength)
    peak_o = 0.0
    for _ in range(300):
        o.step(1)
        peak_o = max(peak_o, float(np.hypot(*o.reaction)))
    b.step(300)
    led = b.read(iid, state=False)["ledger"]
    print("batch fp32 peak load", led["peak_load"], "oracle fp64", peak_o)
    assert abs(led["peak_load"] - peak_o) <= 0.01 * peak_o
    assert abs(led["total"] - o.energies()["total"]) <= 0.02 * o.tool_work


def test_batch_fp32_ledger_residual_before_the_first_break(bt):
    """FP32 bonded instance in a mixed batch (position remainders on, the
    batch default): ledger residual (energies + dissipated + fracture - tool
    work) against the FP64 oracle's within 1e-6 of the work input at every
    checkpoint before the first break (measured 8e-8 to 5.5e-7 in this mix;
    6.8e-7 to 1.8e-6 without remainders)."""
    cfg, st, bonds, strength = small_sheet(24, 8, precision=32, steps=600, speed=5.0)
    b = _batch(bt, precision=32)
    for other in _others(bt, 32):
        b.admit(other)
    iid = b.admit(_inst(bt, cfg, st, bonds, strength))
    cfg64, st64, b64, s64 = small_sheet(24, 8, precision=64, steps=600, speed=5.0)
    o = bonded_oracle_for(cfg64, st64, b64, s64)
    done = 0
    for stop in (100, 200, 300, 400):
        o.step(stop - done)
        b.step(stop - done)
        done = stop
        assert (~o.alive).sum() == 0
        led = b.read(iid, state=False)["ledger"]
        r = (led["total"] - o.energies()["total"]) / o.tool_work
        print(f"batch step {stop}: work {o.tool_work:.1f} J, residual fp32 {r:.2e}")
        assert led["broken"] == 0
        assert abs(r) <= 1e-6, (stop, r)


def _gas(seed, n_side=16):
    from tensordem_gb300.hm2d import granular_gas_case
    return granular_gas_case(n_side, seed=seed, sigma_v=0.1, precision=32)


def _same(a, b):
    for k in ("pos", "vel", "omega", "force", "torque"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("kinetic", "dissipated", "total", "hertz", "evals"):
        assert a["ledger"][k] == b["ledger"][k], k


def test_batch_alone_and_in_mix_are_bit_identical(bt):
    cfg, st = _gas(5)
    alone = _batch(bt, precision=32, every=10)
    ia = alone.admit(_inst(bt, cfg, st))
    alone.step(60)
    ra = alone.read(ia)
    mix = _batch(bt, precision=32, every=10)
    for o in _others(bt, 32):
        mix.admit(o)
    im = mix.admit(_inst(bt, cfg, st))
    mix.step(60)
    rm = mix.read(im)
    assert alone.info()["rebuilds"] == mix.info()["rebuilds"] == 7  # admission + every 10 steps
    _same(ra, rm)


def test_batch_step_variants_bit_identical(bt):
    """Every step-kernel shape (block size, CTAs per SM, tiles per grab of the
    work counter) gives the same bits for each instance of a mix: instance
    sums are formed per tile in tile order, whichever warp took the tile."""
    from tensordem_gb300 import _lib
    runs = []
    for v in range(_lib.lib().tdem_batch_num_variants()):
        b = _batch(bt, precision=32, every=10)
        ids = [b.admit(o) for o in _others(bt, 32)]
        cfg, st = _gas(5)
        ids.append(b.admit(_inst(bt, cfg, st)))
        b.variant = v
        b.step(80)
        assert b.variant == v
        runs.append([b.read(i) for i in ids])
    assert len(runs) == 6
    for got in runs[1:]:
        for a, c in zip(runs[0], got):
            _same(a, c)
            for k in ("bond_elastic", "fracture_released", "tool_work", "peak_load"):
                assert a["ledger"][k] == c["ledger"][k], k


def test_batch_join_and_retire_keep_results_bit_identical(bt):
    a_cfg, a_st = _gas(1)
    b_cfg, b_st = _gas(2, 20)
    c_cfg, c_st = _gas(3, 12)
    refs = {}
    for name, (cfg, st) in {"b": (b_cfg, b_st), "c": (c_cfg, c_st)}.items():
        e = _batch(bt, precision=32, every=10)
        k = e.admit(_inst(bt, cfg, st))
        e.step(60 if name == "b" else 30)
        refs[name] = e.read(k)
    e = _batch(bt, precision=32, every=10)
    ka = e.admit(_inst(bt, a_cfg, a_st))
    kb = e.admit(_inst(bt, b_cfg, b_st))
    e.step(30)
    e.retire(ka)
    kc = e.admit(_inst(bt, c_cfg, c_st))
    assert kc != ka  # the retired slot is reused only after the compaction rebuild
    e.step(30)
    _same(e.read(kb), refs["b"])
    _same(e.read(kc), refs["c"])
    info = e.info()
    assert info["live_instances"] == 2 and info["live_particles"] == b_cfg.n + c_cfg.n
    e.retire(kb)
    e.step(1)
    kd = e.admit(_inst(bt, a_cfg, a_st))
    assert kd in (ka, kb)
    e.step(1)
    assert e.info()["live_particles"] == c_cfg.n + a_cfg.n


def test_batch_capacity_and_argument_errors(bt):
    cfg, st = _gas(4, 16)
    b = _batch(bt, precision=32, cap=300, keys=100_000, slots=2)
    with pytest.raises(RuntimeError):
        b.admit(_inst(bt, cfg, st))  # 256 discs fit, then 256 more do not
        b.admit(_inst(bt, cfg, st))
    bad = np.array([[0, 0]])
    with pytest.raises(ValueError):
        b.admit(_inst(bt, *_gas(6, 4), bonds=bad, strength=np.ones(1)))
    b.step(2)
    assert b.info()["status"] == 0


def test_failed_instance_is_quarantined_and_others_continue(bt):
    """An instance whose state blows up (dt far above its stability limit) is
    reported and frozen; an instance sharing the batch keeps stepping and stays
    within the FP32 tolerance of its solo run (the blow-up can only move the
    shared rebuild times)."""
    from dataclasses import replace
    good_cfg, good_st = _gas(7)
    bad_cfg, bad_st = dense_gas(16, seed=8, precision=32)  # fast, colliding discs
    bad_cfg = replace(bad_cfg, dt=bad_cfg.dt * 200.0)
    solo = _batch(bt, precision=32)
    k0 = solo.admit(_inst(bt, good_cfg, good_st))
    solo.step(80)
    ref = solo.read(k0)
    mix = _batch(bt, precision=32)
    kg = mix.admit(_inst(bt, good_cfg, good_st))
    kb = mix.admit(_inst(bt, bad_cfg, bad_st))
    mix.step(80)
    bad = mix.read(kb, state=False)["ledger"]
    good = mix.read(kg)
    assert bad["status"] != 0  # non-finite or escaped, reported on the instance
    assert good["ledger"]["status"] == 0
    assert np.isfinite(good["pos"]).all()
    assert _rel(good["pos"], ref["pos"]) <= 1e-5
    assert _rel(good["vel"], ref["vel"]) <= 1e-2
    mix.retire(kb)
    mix.step(10)  # the compaction rebuild drops the failed instance
    assert mix.info()["live_particles"] == good_cfg.n
