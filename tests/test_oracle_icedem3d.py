"""CPU pinning of the 3-D oracle and of the host side of the 3-D drop-in.

* The numpy oracle (oracle/icedem3d.py) replays the reference's golden runs
  (tests/golden/dem3d_*.npz, made by the reference IceDEM3D via
  tests/golden/make_golden3d.py): whole trajectories to 1e-12 for the cases
  without transcendental library calls (they are bit-identical), and the
  one-step replay from the reference's own state at every frame for all.
* The host-built topology of tensordem_gb300.dem3d (lattice, bonds, rest
  lengths, fixed set, Weibull thresholds) equals the reference's.
* The ctypes mirrors of the 3-D C structs have the C layout.
"""

import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle.icedem3d import IceDEM3DOracle, Oracle3DConfig
from tests import _icedem3d_parity as P

ROOT = Path(__file__).resolve().parents[1]


def _oracle(g):
    cfg = P.config_dict(g)
    cfg.pop("device")
    x0, pairs = g["initial_positions"], g["pairs"]
    n = len(x0)
    i, j = torch.from_numpy(pairs).T
    ref = torch.from_numpy(x0)[j] - torch.from_numpy(x0)[i]
    rr = ref[:, :, None] * ref[:, None, :]
    cov = torch.zeros((n, 3, 3), dtype=torch.float64)
    cov.index_add_(0, i, rr)
    cov.index_add_(0, j, rr)
    o = IceDEM3DOracle(Oracle3DConfig(**cfg), dt=float(g["dt"]), pinv=torch.linalg.pinv(cov).numpy(),
                       full_rank=(torch.linalg.matrix_rank(cov) >= 3).numpy(),
                       thresholds=g.get("bond_breaking_strain"),
                       zeta=float(g["zeta"]) if "zeta" in g else None)
    o.lateral_velocity = np.asarray(g["lateral_velocity"], dtype=np.float64)
    return o


@pytest.mark.parametrize("name", P.FREE_RUN)
def test_oracle_trajectory(name):
    g = P.load(name)
    o = _oracle(g)
    assert np.array_equal(o.pairs, g["pairs"])
    assert np.array_equal(o.initial_positions, g["initial_positions"])
    assert np.array_equal(o.fixed, g["fixed"])
    loads = g.get("loads")
    s = 0
    for k, target in enumerate(int(x) for x in g["frame_step"]):
        while s < target:
            o.step(None if loads is None else loads[s])
            s += 1
        f, r = o.forces(update_fracture=False, update_history=False)
        for got, want in ((o.positions, g["frame_pos"][k]), (o.velocities, g["frame_vel"][k]),
                          (f, g["frame_force"][k])):
            assert P.normwise(got, want) <= P.RTOL, f"{name} step {target}"
        assert np.array_equal(o.alive, g["frame_alive"][k])
        assert o.time == float(g["frame_time"][k])
    assert np.array_equal(o.failure_mode, g["failure_mode"])
    assert np.array_equal(o.failure_time_s, g["failure_time_s"])
    assert P.normwise(o.failure_energy_J, g["failure_energy_J"]) <= P.RTOL
    assert P.normwise(o.branch_offsets, g["branch_offsets"]) <= P.RTOL
    assert P.normwise(o.damage, g["bond_damage"]) <= P.RTOL
    assert abs(o.bond_dissipation - float(g["bond_dissipation"])) <= P.RTOL * max(1e-300, abs(float(g["bond_dissipation"])))


class _OracleState:
    """The attribute names of the drop-in, mapped onto the oracle's."""

    _MAP = {"_bond_elongation_prev": "elongation_prev", "bond_damage": "damage",
            "_top_platen_tang_disp": "top_tang", "_bottom_platen_tang_disp": "bottom_tang",
            "lateral_platen_pos": "lateral_pos", "cumulative_bond_dissipation_J": "bond_dissipation"}

    def __init__(self, o):
        object.__setattr__(self, "o", o)

    def __getattr__(self, name):
        return getattr(self.o, self._MAP.get(name, name))

    def __setattr__(self, name, value):
        setattr(self.o, self._MAP.get(name, name), value)

    def set_friction_history(self, hist):
        self.o.history = {k: np.asarray(v, dtype=np.float64) for k, v in hist.items()}

    def step(self, loads=None):
        self.o.step(loads)


@pytest.mark.parametrize("name", P.CASES)
def test_oracle_one_step(name):
    g = P.load(name)
    worst = P.replay_one_step(g, _OracleState(_oracle(g)), to_np=np.asarray,
                              to_device=lambda a: np.array(a, copy=True))
    assert worst["pos"] <= P.RTOL


def test_oracle_unit_probes():
    g = P.load("dem3d_unit")
    cfg = P.config_dict(g)
    cfg.pop("device")
    from tensordem_gb300.dem3d import DEM3DConfig
    dt = DEM3DConfig(**{**cfg, "device": "cuda"}).recommended_dt
    for case in ("jitter", "coincident", "stretch", "squeeze", "tool_centre"):
        o = IceDEM3DOracle(Oracle3DConfig(**cfg), dt=dt)
        o.positions = g[f"{case}_pos"].copy()
        o.velocities = g[f"{case}_vel"].copy()
        f, r = o.forces(update_fracture=False, update_history=False)
        scale = max(1.0, np.abs(g[f"{case}_force_probe"]).max())
        assert np.abs(f - g[f"{case}_force_probe"]).max() <= 1e-12 * scale, case
        f2, r2 = o.forces()
        assert np.abs(f2 - g[f"{case}_force"]).max() <= 1e-12 * max(1.0, np.abs(g[f"{case}_force"]).max()), case
        assert np.abs(r2 - g[f"{case}_reaction"]).max() <= 1e-12 * max(1.0, np.abs(g[f"{case}_force"]).max()), case
        assert np.array_equal(o.alive, g[f"{case}_alive"]), case
        assert abs(o.friction_power - float(g[f"{case}_friction_power"])) <= 1e-12 * max(
            1.0, abs(float(g[f"{case}_friction_power"])))


def test_oracle_contacts_match_brute_force():
    """tests/test_dem3d.py:83-98 on the oracle's cell list."""
    g = P.load("dem3d_cylinder")
    o = _oracle(g)
    o.positions = g["frame_pos"][-1].copy()
    got = set(o.candidate_pairs())
    d = np.linalg.norm(o.positions[None] - o.positions[:, None], axis=2)
    i, j = np.nonzero(np.triu(d < 2 * o.config.radius, 1))
    assert set(zip(i.tolist(), j.tolist())) <= got


@pytest.mark.parametrize("name", P.CASES)
def test_dropin_host_topology(name):
    from tensordem_gb300 import dem3d
    g = P.load(name)
    cfg = dem3d.DEM3DConfig(**{**P.config_dict(g), "device": "cuda"})
    assert cfg.recommended_dt == float(g["dt"])
    sim = object.__new__(dem3d.IceDEM3D)
    sim.config = cfg
    host = sim._build_topology()
    assert np.array_equal(host["pairs"].numpy(), g["pairs"])
    assert np.array_equal(host["initial_positions"].numpy(), g["initial_positions"])
    assert np.array_equal(host["fixed"].numpy(), g["fixed"])
    if "bond_breaking_strain" in g:
        assert np.array_equal(host["breaking_strain"].numpy(), g["bond_breaking_strain"])


def test_config_validation():
    from tensordem_gb300.dem3d import DEM3DConfig
    for bad in (dict(nx=1), dict(radius=-1.0), dict(device="cpu"), dict(geometry="sphere"),
                dict(friction_regularization="x"), dict(restitution_coefficient=0.0),
                dict(static_friction_coefficient=0.2, dynamic_friction_coefficient=0.3),
                dict(contact_damping_model="absolute", restitution_coefficient=0.5),
                dict(tangential_model="mindlin_partial_slip"), dict(bond_creep_exponent=-1),
                dict(bond_model="x"), dict(poisson_ratio=0.5)):
        with pytest.raises((ValueError, TypeError)):
            DEM3DConfig(**bad)


def test_struct_layout_matches_c(tmp_path):
    """The ctypes mirrors of the 3-D C-ABI structs have the C sizes and offsets."""
    from tensordem_gb300 import _lib
    src = tmp_path / "layout.c"
    fields = ("nbond", "radius", "branch_k", "cone", "cone_c", "tool_start", "water_level", "cap_denominator",
              "mindlin", "rigid_4e")
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "tdem.h"\nint main(void){\n'
                   'printf("%zu %zu %zu\\n", sizeof(tdem_icedem3d_config), sizeof(tdem_icedem3d_topology),'
                   ' sizeof(tdem_icedem3d_state));\n'
                   + "".join(f'printf("%zu\\n", offsetof(tdem_icedem3d_config, {f}));\n' for f in fields)
                   + "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    sizes = [int(v) for v in out[:3]]
    assert sizes == [ctypes.sizeof(_lib.IceDEM3DConfigC), ctypes.sizeof(_lib.IceDEM3DTopologyC),
                     ctypes.sizeof(_lib.IceDEM3DStateC)]
    assert [int(v) for v in out[3:]] == [getattr(_lib.IceDEM3DConfigC, f).offset for f in fields]


def test_calibrated_damping_ratio_is_the_references():
    """The library's host restatement of the Hertz restitution calibration
    returns the reference's damping ratio bit for bit (contact_calibration.py:219-248)."""
    from tensordem_gb300.dem3d import hertz_damping_ratio_for_restitution
    g = P.load("dem3d_calibrated")
    assert hertz_damping_ratio_for_restitution(0.5) == float(g["zeta"])
    assert hertz_damping_ratio_for_restitution(1.0) == 0.0
    # the calibrated dashpot is stiffer than the linear mapping's (e = 0.5 -> zeta 0.2154)
    assert 0.27 < hertz_damping_ratio_for_restitution(0.5) < 0.30
