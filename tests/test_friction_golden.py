"""Friction law and 2-D rotation conventions pinned to the reference's own functions.

The fixture ``tests/golden/friction_cases.npz`` (written by
``tests/golden/make_friction.py`` from the reference's
``advance_tangential_contact``, ``hertz_mindlin_tangential_force``,
``hertz_mindlin_tangential_stiffness`` and ``reset_tangential_displacement``)
holds 240 contact sequences of 16 steps: stick, slip, reversal and
separation, six materials. Each sequence is replayed free-running (the law's
own history carried from step to step) through

* the oracle's contact law (``oracle.hm2d.contact_law``), on the CPU;
* the CUDA step kernel's contact law (``tdem_hm_contact_law``), FP64 and FP32.

Orientation: the reference accumulates the displacement of partner j
relative to disc i (``disp``); the engine's history is in disc a's
orientation (a = i), so ``xi = -disp`` and the tangential force on a is the
reference's ``k_t disp``. The rotation set checks the contact-point velocity
difference and both torques against the disc engine's own helpers.

Tolerances: FP64, 1e-12 of each sequence's largest |disp| / |F_t| (and of
F_n per step); FP32, 2e-5 of the same scales (overlaps rounded to FP32 carry
6e-8 relative, growing through delta^(3/2) and 16 history increments).
"""

from pathlib import Path

import numpy as np
import pytest

from oracle.hm2d import HMParams, contact_law

FIX = np.load(Path(__file__).resolve().parent / "golden" / "friction_cases.npz")


def _params(m):
    return dict(young=float(FIX["young"][m]), poisson=float(FIX["poisson"][m]), mu=float(FIX["mu_material"][m]))


def _sequences(m):
    return np.flatnonzero(FIX["material"] == m)


def _check_sequence_outputs(xi, ft_a, fn, m_seq, k):
    """Compare one step's outputs for the sequences m_seq against the fixture."""
    disp_ref = FIX["disp_out"][m_seq, k]
    ft_ref = FIX["f_t"][m_seq, k]
    fn_ref = FIX["f_n"][m_seq, k]
    sd = np.abs(FIX["disp_out"][m_seq]).max(axis=(1, 2))[:, None]
    sf = np.abs(FIX["f_t"][m_seq]).max(axis=(1, 2))[:, None]
    e_xi = np.abs(xi + disp_ref) / np.maximum(sd, 1e-300)
    e_ft = np.abs(ft_a - ft_ref) / np.maximum(sf, 1e-300)
    e_fn = np.abs(fn - fn_ref) / np.maximum(fn_ref, 1e-300)
    return float(e_xi.max()), float(e_ft.max()), float(e_fn.max())


def test_fixture_covers_every_regime():
    kinds = FIX["kind"]
    assert not FIX["sliding"][kinds == 0].any()           # stick never slides
    assert FIX["sliding"][kinds == 1].all()               # slip always slides
    assert FIX["sliding"][kinds == 2].any() and not FIX["sliding"][kinds == 2].all()
    assert (FIX["overlap"][kinds == 3] <= 0).any()        # separation opens the contact
    # the stateless saturation agrees with the incremental update
    act = FIX["overlap"] > 0
    assert np.abs(FIX["disp_sat"] - FIX["disp_out"])[act].max() <= 1e-15 * np.abs(FIX["disp_out"]).max()


def test_oracle_contact_law_reproduces_reference_friction():
    worst = np.zeros(3)
    for m in range(len(FIX["young"])):
        seq = _sequences(m)
        pm = _params(m)
        p = HMParams(young=pm["young"], poisson=pm["poisson"], restitution=1.0, mu=pm["mu"], mu_wall=pm["mu"],
                     dt=float(FIX["dt"][seq[0]]), gravity=(0.0, 0.0))
        xi = np.zeros((len(seq), 2))
        n = FIX["normal"][seq]
        for k in range(FIX["overlap"].shape[1]):
            d = FIX["overlap"][seq, k]
            act = d > 0
            new_xi = np.zeros_like(xi)
            ft = np.zeros_like(xi)
            fn = np.zeros(len(seq))
            if act.any():
                a = np.flatnonzero(act)
                zeros2, zeros1 = np.zeros((len(a), 2)), np.zeros(len(a))
                c = contact_law(p, d[a], n[a], FIX["r1"][seq[a]], FIX["r2"][seq[a]], np.ones(len(a)),
                                np.ones(len(a)), zeros2, FIX["v_rel"][seq[a], k], zeros1, zeros1, xi[a])
                new_xi[a] = c["xi"]
                fa = c["f_a"]
                ft[a] = fa - (fa * n[a]).sum(axis=1)[:, None] * n[a]
                fn[a] = c["f_n"]
                np.testing.assert_array_equal(c["sliding"], FIX["sliding"][seq[a], k])
            xi = new_xi
            worst = np.maximum(worst, _check_sequence_outputs(xi, ft, fn, seq, k))
    print("oracle vs reference friction (xi, F_t, F_n):", worst)
    assert worst.max() <= 1e-12


def test_oracle_rotation_conventions_match_the_disc_engine():
    n = FIX["rot_normal"]
    r = FIX["rot_radius"]
    w = FIX["rot_omega"]
    v = FIX["rot_vel"]
    tng = np.stack((-n[:, 1], n[:, 0]), axis=1)
    vrel = v[:, 0] - v[:, 1] + (w[:, 0] * r[:, 0] + w[:, 1] * r[:, 1])[:, None] * tng
    np.testing.assert_allclose(vrel, FIX["rot_vrel"], rtol=0, atol=1e-15 * np.abs(FIX["rot_vrel"]).max())
    f = FIX["rot_force"]
    cr = n[:, 0] * f[:, 1] - n[:, 1] * f[:, 0]
    np.testing.assert_allclose(np.stack((r[:, 0] * cr, r[:, 1] * cr), axis=1), FIX["rot_torque"], rtol=1e-14,
                               atol=1e-15 * np.abs(FIX["rot_torque"]).max())


# ----------------------------------------------------------------------- GPU
def _gpu_replay(precision):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300.hm2d import HM2DConfig, contact_law as gpu_law
    worst = np.zeros(3)
    for m in range(len(FIX["young"])):
        seq = _sequences(m)
        pm = _params(m)
        cfg = HM2DConfig(n=1, ncx=1, ncy=1, cell=1.0, skin=0.0, dt=float(FIX["dt"][seq[0]]), young=pm["young"],
                         poisson=pm["poisson"], restitution=1.0, mu=pm["mu"], mu_wall=pm["mu"], precision=precision)
        xi = np.zeros((len(seq), 2))
        n = FIX["normal"][seq]
        for k in range(FIX["overlap"].shape[1]):
            rows = np.zeros((len(seq), 16))
            rows[:, 0] = FIX["overlap"][seq, k]
            rows[:, 1:3] = n
            rows[:, 3] = FIX["r1"][seq]
            rows[:, 4] = FIX["r2"][seq]
            rows[:, 8:10] = FIX["v_rel"][seq, k]
            rows[:, 11] = 1.0
            rows[:, 12] = 1.0
            rows[:, 13:15] = xi
            out = gpu_law(cfg, rows)
            fa = out[:, 0:2]
            xi = out[:, 3:5]
            ft = fa - (fa * n).sum(axis=1)[:, None] * n
            fn = -(fa * n).sum(axis=1)
            # torque on a = r_a (n x F_a) (the disc engine's lever convention),
            # to rounding of the force's magnitude
            cr = n[:, 0] * fa[:, 1] - n[:, 1] * fa[:, 0]
            tol = 1e-5 if precision == 32 else 1e-13
            assert np.all(np.abs(out[:, 2] - cr) <= tol * np.hypot(fa[:, 0], fa[:, 1]) + 1e-300)
            worst = np.maximum(worst, _check_sequence_outputs(xi, ft, fn, seq, k))
    return worst


@pytest.mark.gpu
def test_cuda_contact_law_fp64_reproduces_reference_friction():
    worst = _gpu_replay(64)
    print("CUDA FP64 vs reference friction (xi, F_t, F_n):", worst)
    assert worst.max() <= 1e-12


@pytest.mark.gpu
def test_cuda_contact_law_fp32_within_bound():
    worst = _gpu_replay(32)
    print("CUDA FP32 vs reference friction (xi, F_t, F_n):", worst)
    assert worst.max() <= 2e-5


@pytest.mark.gpu
def test_cuda_contact_law_rotation_matches_the_disc_engine():
    """Sticking contact (mu large) from zero history: the history after one
    step is the tangential part of the reference's contact-point velocity
    difference (spins included) times dt."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300.hm2d import HM2DConfig, contact_law as gpu_law
    n = FIX["rot_normal"]
    r = FIX["rot_radius"]
    dt = 1e-7
    cfg = HM2DConfig(n=1, ncx=1, ncy=1, cell=1.0, skin=0.0, dt=dt, young=70e9, poisson=0.25, restitution=1.0,
                     mu=1e6, mu_wall=1e6, precision=64)
    rows = np.zeros((len(n), 16))
    rows[:, 0] = 1e-6
    rows[:, 1:3] = n
    rows[:, 3:5] = r
    rows[:, 5:7] = FIX["rot_vel"][:, 0]
    rows[:, 7] = FIX["rot_omega"][:, 0]
    rows[:, 8:10] = FIX["rot_vel"][:, 1]
    rows[:, 10] = FIX["rot_omega"][:, 1]
    rows[:, 11:13] = 1.0
    out = gpu_law(cfg, rows)
    vrel = FIX["rot_vrel"]
    vt = vrel - (vrel * n).sum(axis=1)[:, None] * n
    np.testing.assert_allclose(out[:, 3:5], vt * dt, rtol=0, atol=1e-13 * np.abs(vt * dt).max())
