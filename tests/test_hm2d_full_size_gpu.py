"""Parity of the Hertz-Mindlin engine at the full 1,048,576-disc settling case.

The case is the seeded 1024 x 1024 polydisperse gas of the throughput
benchmark (radii U[0.8, 1.2] mm, E 70 GPa, nu 0.25, mu 0.5, e 0.8, four
walls, gravity). Following the reference's scale-ceiling checks
(tests/test_scale_ceiling_dem.py:41-80: pair set against brute force, the
Hertz law on the engine's own contacts), at this size:

* the candidate pair set equals an exact search (scipy's KD-tree for
  candidates, then the exact reach test r_i + r_j + skin), FP64 and FP32;
* one FP64 evaluation equals the FP64 oracle to 1e-12 per disc, at the seeded
  state and at the state after the case's 10,000 FP64 steps, when contacts exist;
* the tangential history committed by that evaluation equals the oracle's;
* one FP32 evaluation stays within the engine's stated FP32 bound (2e-3
  normwise on forces; torques to 2e-3 of r_max max|F|).

Exactly comparable geometry: the oracle works in absolute coordinates (up to
2.45 m), the engine in offsets from an integer cell origin. For overlaps of
1e-7 m the two roundings of a centre distance alone differ by ~1e-8 relative.
The FP64 comparisons therefore snap the state's positions and the cell size
to multiples of 2^-32 m (2.3e-10 m, far below any overlap here): every
coordinate, offset and centre difference is then exact on both sides, and
the squared distances (products of integers below 2^24 times 2^-64) are too,
so both sides see the same overlaps and the comparison measures the contact
law and the sums, to 1e-12 of the sum of the magnitudes of each disc's terms.
"""

import numpy as np
import pytest
import torch

from tests._hm_cases import oracle_for

pytestmark = pytest.mark.gpu

Q = 2.0 ** -32


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


def _snapped(hm, cfg, st):
    """Configuration and state with the cell size and positions on the 2^-32 m lattice."""
    cell = round(cfg.cell / Q) * Q
    cfg = hm.HM2DConfig(**{**cfg.__dict__, "cell": cell})
    st = dict(st, pos=np.round(np.asarray(st["pos"]) / Q) * Q)
    return cfg, st


def exact_pairs(pos, radius, skin):
    """All (i, j), i < j, with |x_j - x_i| <= r_i + r_j + skin (KD-tree
    candidates within the largest reach, then the exact test)."""
    from scipy.spatial import cKDTree
    reach = 2.0 * float(radius.max()) + skin
    pr = cKDTree(pos).query_pairs(reach * (1.0 + 1e-9), output_type="ndarray").astype(np.int64).reshape(-1, 2)
    i, j = np.minimum(pr[:, 0], pr[:, 1]), np.maximum(pr[:, 0], pr[:, 1])
    d = pos[j] - pos[i]
    keep = np.sqrt((d * d).sum(axis=1)) <= radius[i] + radius[j] + skin
    return i[keep], j[keep]


def _pair_set(i, j, n):
    return set((i.astype(np.int64) * n + j).tolist())


def _abs_sums(o, pos, vel, omega, total):
    """Per disc, the sum of the magnitudes of its force terms (contacts,
    gravity, and the total, which bounds the wall terms of a disc touching only
    a wall) at an evaluation of the oracle: the scale of its rounding."""
    s = np.abs(o.mass)[:, None] * np.abs(np.asarray(o.p.gravity))[None, :]
    s = np.sqrt((s * s).sum(axis=1)) + np.sqrt((total * total).sum(axis=1))
    i, j = o.candidate_pairs()
    d = pos[j] - pos[i]
    dist = np.sqrt((d * d).sum(axis=1))
    delta = o.radius[i] + o.radius[j] - dist
    act = delta > 0
    if act.any():
        from oracle.hm2d import contact_law
        a = np.flatnonzero(act)
        c = contact_law(o.p, delta[a], d[a] / dist[a, None], o.radius[i[a]], o.radius[j[a]], o.inv_mass[i[a]],
                        o.inv_mass[j[a]], vel[i[a]], vel[j[a]], omega[i[a]], omega[j[a]], np.zeros((len(a), 2)))
        m = np.sqrt((c["f_a"] ** 2).sum(axis=1)) + np.abs(c["f_n"])
        np.add.at(s, i[a], m)
        np.add.at(s, j[a], m)
    return s + 1e-300


@pytest.fixture(scope="module")
def settled(hm):
    """The seeded 1M-disc state after the case's 10,000 FP64 engine steps
    (integer-time velocities), snapped to the 2^-32 m lattice, with its
    configuration."""
    cfg, st = hm.granular_gas_case(1024, seed=0, precision=64)
    e = _engine(hm, cfg, st)
    e.step(10000)
    s = e.state()
    out = dict(st, pos=_np(s["pos"]), vel=_np(s["vel"]), omega=_np(s["omega"]))
    return _snapped(hm, cfg, out)


@pytest.mark.parametrize("precision", [64, 32])
def test_candidate_pairs_equal_exact_search_at_1m(hm, precision):
    cfg, st = hm.granular_gas_case(1024, seed=0, precision=precision)
    e = _engine(hm, cfg, st)
    pos = _np(e.state()["pos"])     # the positions the engine holds (FP32: cell origin + FP32 offset)
    got = e.pairs()
    bi, bj = exact_pairs(pos, st["radius"], cfg.skin)
    n = cfg.n
    g, w = _pair_set(got[:, 0], got[:, 1], n), _pair_set(bi, bj, n)
    diff = g ^ w
    tol = 1e-6 if precision == 32 else 1e-12
    for k in diff:
        i, j = divmod(k, n)
        d = np.linalg.norm(pos[j] - pos[i])
        reach = st["radius"][i] + st["radius"][j] + cfg.skin
        assert abs(d - reach) <= tol * reach, f"pair {(i, j)} differs away from the reach boundary"
    print(f"{precision}-bit candidate pairs at 1M: {len(w)} exact, {len(diff)} at the reach boundary")
    assert len(w) > n // 10 and len(diff) <= len(w) // 100000 + 2
    # after 300 steps and a rebuild
    e.step(300)
    e.rebuild()
    pos = _np(e.state()["pos"])
    got = e.pairs()
    bi, bj = exact_pairs(pos, st["radius"], cfg.skin)
    diff = _pair_set(got[:, 0], got[:, 1], n) ^ _pair_set(bi, bj, n)
    for k in diff:
        i, j = divmod(k, n)
        d = np.linalg.norm(pos[j] - pos[i])
        reach = st["radius"][i] + st["radius"][j] + cfg.skin
        assert abs(d - reach) <= tol * reach


def test_fp64_evaluation_at_the_seeded_state_matches_oracle(hm):
    cfg, st = _snapped(hm, *hm.granular_gas_case(1024, seed=0, precision=64))
    e = _engine(hm, cfg, st)
    s = e.state()
    o = oracle_for(cfg, st)
    f, tq, _ = o.evaluate(o.pos, o.vel, o.omega, advance=False)
    scale = _abs_sums(o, o.pos, o.vel, o.omega, f)
    err = np.abs(_np(s["force"]) - f).max(axis=1) / scale
    print("seeded 1M state: FP64 force error / term scale", float(err.max()))
    assert float(err.max()) <= 1e-12
    assert np.abs(_np(s["torque"]) - tq).max() <= 1e-12 * np.abs(scale).max()


def test_fp64_evaluation_with_contacts_matches_oracle(hm, settled):
    cfg, st = settled
    e = _engine(hm, cfg, st)
    s = e.state()
    o = oracle_for(cfg, st)
    f, tq, _ = o.evaluate(o.pos, o.vel, o.omega, advance=False)
    i, j = o.candidate_pairs()
    d = o.pos[j] - o.pos[i]
    touching = int((np.sqrt((d * d).sum(axis=1)) < o.radius[i] + o.radius[j]).sum())
    scale = _abs_sums(o, o.pos, o.vel, o.omega, f)
    err_f = np.abs(_np(s["force"]) - f).max(axis=1) / scale
    r = o.radius
    err_t = np.abs(_np(s["torque"]) - tq) / (r * scale)
    print(f"1M state after 10000 FP64 steps: {touching} touching pairs; FP64 force error / term scale "
          f"{float(err_f.max()):.2e}, torque {float(err_t.max()):.2e}")
    assert touching > 100
    assert float(err_f.max()) <= 1e-12 and float(err_t.max()) <= 1e-12
    # the history this evaluation commits (the prime evaluation) equals the oracle's
    e.step(1)
    o.prime()
    hist = e.history()
    keys = np.array([a * cfg.n + b for a, b in hist], dtype=np.int64)
    order = np.argsort(keys)
    got = np.array([hist[k] for k in hist])[order] if len(hist) else np.zeros((0, 2))
    nz = np.any(o.state.xi != 0.0, axis=1)
    assert np.array_equal(keys[order], o.state.keys[nz])
    want = o.state.xi[nz]
    err = np.abs(got - want).max(axis=1) / np.maximum(np.abs(want).max(axis=1), 1e-300)
    print(f"history of {len(want)} contacts after the prime evaluation: max relative error {float(err.max()):.2e}")
    assert len(want) > 100 and float(err.max()) <= 1e-12


def test_fp32_evaluation_with_contacts_within_bound(hm, settled):
    cfg64, st = settled
    cfg = hm.HM2DConfig(**{**cfg64.__dict__, "precision": 32})
    e = _engine(hm, cfg, st)
    s = e.state()
    held = dict(st, pos=_np(s["pos"]))   # FP32 cell origin + offset, as held
    o = oracle_for(cfg, held)
    f, tq, _ = o.evaluate(o.pos, o.vel, o.omega, advance=False)
    err = np.abs(_np(s["force"]) - f).max() / np.abs(f).max()
    # torques in units of r max|F|: a torque is a lever times a tangential
    # force, the small difference of the relative velocity and its normal part
    terr = np.abs(_np(s["torque"]) - tq).max() / (st["radius"].max() * np.abs(f).max())
    print(f"1M state: FP32 force error {err:.2e} normwise, torque {terr:.2e} of r max|F|")
    assert err <= 2e-3 and terr <= 2e-3
