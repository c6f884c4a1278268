"""GPU parity of the Hertz-Mindlin engine (csrc/hm2d.cu) against the FP64 oracle.

Tolerances, stated per test:
* candidate pair sets: exact integer equality with a brute-force search,
  except pairs within 1e-6 (FP32) / 1e-12 (FP64) relative of the reach
  boundary, which are reported and must be rare;
* FP64 engine vs oracle: single evaluation 1e-12 normwise; trajectories 1e-9
  normwise after a few hundred steps with collisions and rebuilds;
* FP32 engine vs oracle: single evaluation 2e-3 normwise on forces (the FP32
  overlap of a stiff E = 70 GPa contact carries ~1e-10 m absolute error on
  delta ~ 1e-6 m), energy ledger within 1e-3 of the initial energy.
"""

import math

import numpy as np
import pytest
import torch

from oracle.hm2d import HM2DOracle, HMParams, brute_force_pairs
from tests._hm_cases import dense_gas, oracle_for, two_disc_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hm():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300 import hm2d
    return hm2d


def _np(t):
    return t.detach().cpu().numpy()


def _engine(hm, cfg, st):
    e = hm.HM2D(cfg)
    e.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
    return e


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("precision", [32, 64])
def test_candidate_pairs_match_brute_force(hm, precision):
    cfg, st = dense_gas(40, seed=11, precision=precision, skin=0.3e-3)
    e = _engine(hm, cfg, st)
    e.step(50)
    s = e.state()
    pos = _np(s["pos"])
    got = {tuple(p) for p in e.pairs().tolist()}
    # the list was built at the last rebuild; rebuild now by re-uploading the state
    e.set_state(pos, _np(s["vel"]), _np(s["omega"]), st["radius"], st["mass"], st["inertia"])
    got = {tuple(p) for p in e.pairs().tolist()}
    pos = _np(e.state()["pos"])
    bi, bj = brute_force_pairs(pos, 0.0, st["radius"], skin=cfg.skin)
    want = set(zip(bi.tolist(), bj.tolist()))
    tol = 1e-6 if precision == 32 else 1e-12
    diff = got ^ want
    for i, j in diff:
        d = np.linalg.norm(pos[j] - pos[i])
        reach = st["radius"][i] + st["radius"][j] + cfg.skin
        assert abs(d - reach) <= tol * reach, f"pair {(i, j)} differs away from the reach boundary"
    assert len(diff) <= max(2, len(want) // 10000)
    assert len(want) > cfg.n


def _edge_configurations():
    """2-D counterparts of the reference's neighbour-search configurations
    (tests/test_dem_vectorized_verification.py:94-121): one disc, a touching
    pair, a pair just outside the reach, an overlapping lattice, a dilute and a
    clustered random set, a collinear chain. Equal radii r = 1 mm in a 30 mm
    box; the clustered set is wider than the 3-D original (sigma 4 mm) so no
    disc has more than the engine's 24 candidate slots."""
    r, c = 1e-3, 15e-3
    rng = np.random.default_rng(0)
    g = np.arange(6, dtype=np.float64)
    yy, xx = np.meshgrid(g, g, indexing="ij")
    return {
        "single": np.array([[c, c]]),
        "pair_touching": np.array([[c - r, c], [c + r, c]]),
        "pair_just_outside": np.array([[c - 1.02 * r, c], [c + 1.02 * r, c]]),
        "dense_lattice_overlapping": np.stack([xx.ravel(), yy.ravel()], 1) * (2 * r * 0.99) + 8e-3,
        "random_dilute": rng.uniform(2e-3, 28e-3, (40, 2)),
        "random_clustered": np.clip(c + rng.normal(0.0, 4e-3, (60, 2)), 1.5e-3, 28.5e-3),
        "collinear_chain": np.stack([3e-3 + np.arange(12) * 1.9 * r, np.full(12, c)], 1),
    }


def _positions_case(pos, r=1e-3, box=30e-3, skin=0.02e-3):
    from tensordem_gb300.hm2d import HM2DConfig, grid_for_box, rayleigh_dt
    n = len(pos)
    ncell, cell = grid_for_box(box, r, skin)
    radius = np.full(n, r)
    mass = 2500.0 * math.pi * radius**2 * (2 * radius)
    cfg = HM2DConfig(n=n, ncx=ncell, ncy=ncell, cell=cell, skin=skin, dt=0.2 * rayleigh_dt(r, 2500.0, 70e9, 0.25),
                     young=70e9, poisson=0.25, restitution=0.8, mu=0.5, mu_wall=0.5, precision=64,
                     max_neighbors=24)
    st = dict(pos=np.ascontiguousarray(pos, dtype=np.float64), vel=np.zeros((n, 2)), omega=np.zeros(n),
              radius=radius, mass=mass, inertia=0.5 * mass * radius**2)
    return cfg, st


@pytest.mark.parametrize("name", list(_edge_configurations()))
def test_cell_list_edge_configurations_match_brute_force(hm, name):
    pos = _edge_configurations()[name]
    cfg, st = _positions_case(pos)
    e = _engine(hm, cfg, st)
    got = {tuple(p) for p in e.pairs().tolist()}
    bi, bj = brute_force_pairs(st["pos"], 0.0, st["radius"], skin=cfg.skin)
    want = set(zip(bi.tolist(), bj.tolist()))
    assert got == want, (name, sorted(got ^ want)[:10])
    expected_count = {"single": 0, "pair_touching": 1, "pair_just_outside": 0, "dense_lattice_overlapping": 60,
                      "collinear_chain": 11}
    if name in expected_count:
        assert len(want) == expected_count[name]
    # the engine steps these states without error
    e.step(5)
    assert e.ledger()["status"] == 0


def test_fp64_single_evaluation_matches_oracle(hm):
    cfg, st = dense_gas(24, seed=4, precision=64)
    # push a few pairs into contact at t = 0
    st["pos"][1] = st["pos"][0] + np.array([st["radius"][0] + st["radius"][1] - 3e-6, 0.0])
    e = _engine(hm, cfg, st)
    s = e.state()
    o = oracle_for(cfg, st)
    f, tq, _ = o.evaluate(o.pos, o.vel, o.omega, advance=False)
    assert _rel(_np(s["force"]), f) <= 1e-12
    assert _rel(_np(s["torque"]), tq) <= 1e-12 or np.abs(tq).max() == 0.0


def test_fp64_trajectory_matches_oracle(hm):
    """Step-1 state agrees to rounding; later, stiff collisions amplify the
    last-bit differences of two FP64 programs (chaos), so the bound grows with
    the horizon: 1e-12 after one step, 1e-8 (positions) after 400 steps."""
    cfg, st = dense_gas(24, seed=7, precision=64)
    e = _engine(hm, cfg, st)
    o = oracle_for(cfg, st)
    bounds = {1: (1e-14, 1e-12, 1e-12), 50: (1e-11, 1e-7, 1e-6), 200: (1e-9, 1e-5, 1e-4),
              400: (1e-8, 1e-4, 1e-3)}
    done = 0
    for stop, (bp, bv, bf) in bounds.items():
        e.step(stop - done)
        o.step(stop - done)
        done = stop
        s = e.state()
        errs = (_rel(_np(s["pos"]), o.pos), _rel(_np(s["vel"]), o.vel), _rel(_np(s["force"]), o.force))
        print(f"fp64 vs oracle after {stop} steps: pos {errs[0]:.2e} vel {errs[1]:.2e} force {errs[2]:.2e}")
        assert errs[0] <= bp and errs[1] <= bv and errs[2] <= bf, (stop, errs)
    led = e.ledger()
    ref = o.energies()
    assert led["rebuilds"] >= 2 and o.state.keys.size > 0
    for k in ("kinetic", "potential", "elastic_normal", "dissipated", "total"):
        assert abs(led[k] - ref[k]) <= 1e-6 * abs(ref["total"]), k


@pytest.mark.parametrize("precision", [32, 64])
def test_history_survives_rebuilds_bit_exact(hm, precision):
    """A rebuild re-sorts particles and rebuilds every list; the tangential
    history of every contact must come out bit-identical, keyed by the
    original-id pair (scale_ceiling/kernel.py:250-263)."""
    cfg, st = dense_gas(24, seed=9, precision=precision, skin=0.2e-3)
    e = _engine(hm, cfg, st)
    e.step(120)
    before = e.history()
    assert len(before) > 20
    e.rebuild()
    after = e.history()
    assert before == after
    e.step(1)
    assert e.ledger()["status"] == 0


def test_rebuild_frequency_does_not_change_physics(hm):
    """Rebuilding often or rarely changes only the summation order (FP64)."""
    runs = []
    for skin in (0.005e-3, 0.2e-3):
        cfg, st = dense_gas(24, seed=9, precision=64, skin=skin)
        e = _engine(hm, cfg, st)
        e.step(100)
        runs.append((e.state(), e.ledger()))
    (a, la), (b, lb) = runs
    assert la["rebuilds"] > lb["rebuilds"] + 5
    err = _rel(_np(a["vel"]), _np(b["vel"]))
    print("rebuild-frequency velocity difference", err)
    assert err <= 1e-6
    assert abs(la["dissipated"] - lb["dissipated"]) <= 1e-6 * la["total"]


def test_fp32_single_evaluation_within_tolerance(hm):
    cfg, st = dense_gas(24, seed=4, precision=32)
    st["pos"][1] = st["pos"][0] + np.array([st["radius"][0] + st["radius"][1] - 3e-6, 0.0])
    e = _engine(hm, cfg, st)
    s = e.state()
    # the oracle evaluates at the FP32-representable positions the engine holds
    st64 = dict(st, pos=_np(s["pos"]))
    o = oracle_for(cfg, st64)
    f, tq, _ = o.evaluate(o.pos, o.vel, o.omega, advance=False)
    err = _rel(_np(s["force"]), f)
    print("fp32 single-evaluation normwise force error", err)
    assert err <= 2e-3


def test_fp32_ledger_tracks_oracle(hm):
    cfg, st = dense_gas(24, seed=7, precision=32)
    e = _engine(hm, cfg, st)
    o = oracle_for(cfg, st)
    e0 = o.energies()["total"]
    e.step(300)
    o.step(300)
    led, ref = e.ledger(), o.energies()
    print("fp32 ledger", led, "oracle", ref)
    for k in ("kinetic", "dissipated", "total"):
        assert abs(led[k] - ref[k]) <= 1e-3 * e0, k
    # energy balance of the FP32 run itself
    assert abs(led["total"] - e0) <= 2e-2 * e0


def test_fp32_determinism_and_graph_equivalence(hm):
    digests = []
    for graph in (True, True, False):
        cfg, st = dense_gas(24, seed=8, precision=32)
        e = hm.HM2D(cfg)
        e.use_graph(graph)
        e.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
        e.step(250)
        s = e.state()
        digests.append(tuple(_np(s[k]).tobytes() for k in ("pos", "vel", "omega")))
    assert digests[0] == digests[1] == digests[2]


def test_all_step_variants_bit_identical(hm):
    """Every launch shape the autotuner may pick computes the same state."""
    from tensordem_gb300 import _lib
    outs = []
    for v in range(_lib.lib().tdem_hm_num_variants()):
        cfg, st = dense_gas(20, seed=21, precision=32)
        e = _engine(hm, cfg, st)
        e.variant = v
        e.step(150)
        s = e.state()
        outs.append(tuple(_np(s[k]).tobytes() for k in ("pos", "vel", "omega")))
    assert all(o == outs[0] for o in outs[1:])


def test_autotune_picks_a_variant_and_keeps_running(hm):
    cfg, st = dense_gas(20, seed=22, precision=32)
    e = _engine(hm, cfg, st)
    times = e.autotune(steps=5)
    assert e.variant == min(times, key=times.get)
    e.step(10)
    assert e.ledger()["status"] == 0


def test_momentum_conserved_without_walls_or_gravity(hm):
    cfg, st = dense_gas(24, seed=12, precision=32, walls=0, gravity=(0.0, 0.0))
    e = _engine(hm, cfg, st)
    p0 = (st["mass"][:, None] * st["vel"]).sum(0)
    e.step(300)
    v = _np(e.state()["vel"])
    p1 = (st["mass"][:, None] * v).sum(0)
    scale = (st["mass"][:, None] * np.abs(st["vel"])).sum(0)
    assert np.all(np.abs(p1 - p0) <= 1e-5 * scale)


def test_capacity_overflow_raises(hm):
    cfg, st = dense_gas(16, seed=1, precision=32, skin=0.3e-3, max_neighbors=1)
    e = hm.HM2D(cfg)
    with pytest.raises(RuntimeError, match="capacity"):
        e.set_state(st["pos"], st["vel"], st["omega"], st["radius"], st["mass"], st["inertia"])
        e.step(1)


def test_two_disc_hertz_law_on_gpu(hm):
    st = two_disc_state(delta=2e-6)
    cfg = hm.HM2DConfig(n=2, ncx=4, ncy=4, cell=2.5e-3, skin=0.1e-3, dt=1e-8, young=70e9, poisson=0.25,
                        restitution=1.0, mu=0.0, mu_wall=0.0, gravity=(0.0, 0.0), walls=0, precision=64)
    e = _engine(hm, cfg, st)
    f = _np(e.state()["force"])
    estar = 70e9 / (2 * (1 - 0.25**2))
    expected = (4.0 / 3.0) * estar * math.sqrt(0.5e-3) * (2e-6) ** 1.5
    assert abs(f[0, 0]) == pytest.approx(expected, rel=1e-12)
    assert f[0, 0] == -f[1, 0]


def test_full_size_settling_case_runs(hm):
    cfg, st = hm.granular_gas_case(1024, seed=0)
    e = _engine(hm, cfg, st)
    e.step(20)
    led = e.ledger()
    assert led["evals"] == 20 and led["status"] == 0
    assert math.isfinite(led["total"])


def test_fp64_sum_form_within_the_fp32_bound(hm):
    """The FP64-sum form of the FP32 engine (each particle's force and torque
    terms summed in FP64, sum_precision=64) against the FP64 oracle: the FP32
    single-evaluation bound (2e-3 normwise), and after 100 steps the same
    state as the default float-float form to FP32 rounding (1e-5 of the box)."""
    from dataclasses import replace
    cfg, st = dense_gas(24, seed=4, precision=32)
    st["pos"][1] = st["pos"][0] + np.array([st["radius"][0] + st["radius"][1] - 3e-6, 0.0])
    runs = {}
    for sums in (32, 64):
        e = _engine(hm, replace(cfg, sum_precision=sums), st)
        s = e.state()
        o = oracle_for(cfg, dict(st, pos=_np(s["pos"])))
        f, _, _ = o.evaluate(o.pos, o.vel, o.omega, advance=False)
        err = _rel(_np(s["force"]), f)
        print(f"sum_precision {sums}: single-evaluation normwise force error {err:.2e}")
        assert err <= 2e-3
        e.step(100)
        runs[sums] = _np(e.state()["pos"])
    assert np.abs(runs[32] - runs[64]).max() <= 1e-5 * cfg.box[0]


@pytest.mark.parametrize("remainder", [1, 0])
def test_position_remainder_integrates_free_flight_exactly(hm, remainder):
    """Free flight without forces: each FP32 velocity stays exact, so the
    exact position after N steps is x0 + N dt v (dt and v as the engine holds
    them, FP32). With position remainders the engine's drift keeps the
    rounding of every step (FMA error of dt v, TwoSum error of the sum) and
    carries it across each rebuild's change of cell origin: 5,000 steps and
    501 rebuilds across ~30 cells land within 1e-12 m (measured 5.6e-15 m).
    Plain FP32 offsets lose up to half an ulp of the offset per step
    (measured 1.5e-7 m here)."""
    from dataclasses import replace
    cfg, _ = dense_gas(8, seed=51, precision=32, walls=0, gravity=(0.0, 0.0))
    n = 16
    r = 0.9e-3
    cfg = replace(cfg, n=n, ncx=128, ncy=128, cell=2.2e-3, skin=0.3e-3, dt=1e-5, max_neighbors=4,
                  position_remainder=remainder)
    box = cfg.box[0]
    # sixteen discs on a diagonal, all with the same velocity: never in contact
    pos = np.stack((np.linspace(0.2, 0.6, n), np.linspace(0.15, 0.45, n)), axis=1) * box
    vel = np.tile(np.array([[1.3, 0.7]]), (n, 1))
    mass = 2500.0 * math.pi * r**2 * (2 * r) * np.ones(n)
    state = dict(pos=pos, vel=vel, omega=np.zeros(n), radius=np.full(n, r), mass=mass,
                 inertia=0.5 * mass * r**2)
    e = _engine(hm, cfg, state)
    steps = 5000
    e.step(steps)
    got = _np(e.state()["pos"])
    dt32 = float(np.float32(cfg.dt))
    v32 = vel.astype(np.float32).astype(np.float64)
    exact = pos + steps * (dt32 * v32)
    err = np.abs(got - exact).max()
    print(f"remainder {remainder}: max position error after {steps} steps {err:.2e} m, "
          f"{e.ledger()['rebuilds']:.0f} rebuilds")
    assert e.ledger()["rebuilds"] >= 3
    if remainder:
        assert err <= 1e-12
    else:
        assert err > 1e-11  # the plain offsets do drift: the check above is not vacuous
