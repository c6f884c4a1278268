"""Host-side checks of the seeded ensemble generator (no GPU)."""

import math

import numpy as np

from tensordem_gb300.batch import BatchConfig, ensemble_case


def test_ensemble_draws_are_seeded_and_in_range():
    a = ensemble_case(256, seed=0)
    b = ensemble_case(256, seed=0)
    assert a == b
    assert ensemble_case(256, seed=1) != a
    n = np.array([s.n for s in a])
    e = np.array([s.young for s in a])
    mu = np.array([s.mu for s in a])
    assert n.min() >= 100 and n.max() <= 20_000
    assert e.min() >= 1e9 and e.max() <= 70e9
    assert mu.min() >= 0.3 and mu.max() <= 0.7
    assert {s.kind for s in a[0::2]} == {"ice"} and {s.kind for s in a[1::2]} == {"column"}
    # log-uniform: about half the draws below the geometric mean of the bounds
    assert 0.35 < np.mean(n < math.sqrt(100 * 20_000)) < 0.65


def test_instances_are_well_formed():
    for spec in ensemble_case(24, seed=3, n_max=1500):
        inst = spec.build()
        cfg, st = inst.config, inst.state
        assert abs(cfg.n - spec.n) <= 0.2 * spec.n + 8
        box = (cfg.ncx * cfg.cell, cfg.ncy * cfg.cell)
        assert (st["pos"] > 0).all() and (st["pos"][:, 0] < box[0]).all() and (st["pos"][:, 1] < box[1]).all()
        assert cfg.cell >= 2 * st["radius"].max() + cfg.skin
        r = st["radius"]
        assert r.min() >= 0.8 * r.max() / 1.2 * 0.999
        if inst.kind == "column":
            # jittered grid: no two discs overlap at t = 0
            d = np.linalg.norm(st["pos"][:, None, :] - st["pos"][None, :, :], axis=2)
            np.fill_diagonal(d, np.inf)
            assert (d >= r[:, None] + r[None, :]).all()
            assert inst.bonds is None
        else:
            b = inst.bonds
            assert b.shape[1] == 2 and (b[:, 0] < b[:, 1]).all()
            deg = np.bincount(b.ravel(), minlength=cfg.n)
            assert deg.max() <= 6
            assert np.isinf(st["mass"]).sum() == 2 * inst.meta["ny"]  # clamped end columns
            assert cfg.indenter_radius > 0 and cfg.indenter_velocity[1] < 0


def test_batch_config_footprint_is_host_computable():
    cfg = BatchConfig(particle_capacity=1_000_000, key_capacity=2_000_000, max_instances=1024)
    try:
        nbytes = cfg.bytes()
    except RuntimeError:  # the native library is not built in this environment
        return
    assert 400 * 1_000_000 < nbytes < 2000 * 1_000_000


def test_serving_trace_and_budget_sizing():
    from tensordem_gb300.serve import engine_for_budget, make_trace, mean_log_uniform
    tr = make_trace(duration=100.0, rate=5.0, seed=2)
    assert 400 < len(tr) < 600
    arr = np.array([r.arrival for r in tr])
    assert (np.diff(arr) > 0).all() and arr[-1] < 100.0
    assert min(r.n for r in tr) >= 500 and max(r.n for r in tr) <= 200_000
    assert min(r.steps for r in tr) >= 1000 and max(r.steps for r in tr) <= 50_000
    # the offered rate follows load x capacity / E[N S]
    cap = 7e9
    tr2 = make_trace(duration=1000.0, capacity=cap, load=0.8, seed=3)
    want = 0.8 * cap / (mean_log_uniform(500, 200_000) * mean_log_uniform(1000, 50_000))
    assert abs(len(tr2) / 1000.0 - want) < 0.15 * want
    try:
        cfg, per_p, per_k = engine_for_budget(int(150e9))
    except RuntimeError:  # the native library is not built in this environment
        return
    assert cfg.bytes() <= 150e9 and cfg.particle_capacity > 1e8
    assert 300 < per_p < 2000 and 4 < per_k < 64
