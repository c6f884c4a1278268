"""Replay of the golden IceDEM runs against any implementation of the step.

The same replay drives the numpy oracle (CPU tests) and the CUDA path (GPU
tests), so both are held to the reference's own outputs with one set of
tolerances:

* break ledger: ``failure_mode`` and ``failure_time_s`` bit-exact;
  ``failure_extension_m`` / ``failure_energy_J`` within ``RTOL`` normwise;
* positions, velocities, forces, reactions at each recorded frame within
  ``RTOL`` relative to the largest magnitude of that quantity (normwise);
* cumulative accounting within ``RTOL`` of the largest ledger entry of the
  same kind (energies, impulses).
"""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
RTOL = 1e-12


def load(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz", allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def config_dict(g: dict) -> dict:
    return json.loads(str(g["config"]))


def normwise(a, b, floor: float = 0.0) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.abs(b).max(initial=0.0), floor)
    if scale == 0.0:
        return float(np.abs(a - b).max(initial=0.0))
    return float(np.abs(a - b).max(initial=0.0) / scale)


def check_accounting(got: np.ndarray, want: np.ndarray, rtol: float = RTOL) -> None:
    """Energies (first five) and impulses (last eight) compared per group."""
    e_scale = max(np.abs(want[:5]).max(), 1e-300)
    i_scale = max(np.abs(want[5:]).max(), 1e-300)
    assert np.abs(got[:5] - want[:5]).max() <= rtol * e_scale, (got[:5], want[:5])
    assert np.abs(got[5:] - want[5:]).max() <= rtol * i_scale, (got[5:], want[5:])


def replay(g: dict, sim, *, to_np, loads_fn=None, rtol: float = RTOL) -> dict:
    """Run ``sim`` through the golden protocol and compare frame by frame.

    ``sim`` exposes ``forces(loads)``, ``step(loads, load_time=...)``,
    ``positions``, ``velocities``, ``accounting_vector()``, ``bond_alive()``
    and ``failure_ledger()``; ``to_np`` converts its arrays to numpy.
    Returns the worst normwise errors seen, for reporting.
    """
    frames = [int(s) for s in g["frame_step"]]
    last = frames[-1]
    worst = {"pos": 0.0, "vel": 0.0, "force": 0.0, "reaction": 0.0}
    k = 0
    for s in range(last + 1):
        if s == frames[k]:
            loads = None if loads_fn is None else loads_fn(s)
            f, r = sim.forces(loads)
            errs = {
                "pos": normwise(to_np(sim.positions), g["frame_pos"][k]),
                "vel": normwise(to_np(sim.velocities), g["frame_vel"][k]),
                "force": normwise(to_np(f), g["frame_force"][k]),
                "reaction": normwise(to_np(r), g["frame_reaction"][k],
                                     floor=np.abs(g["frame_force"][k]).max()),
            }
            for name, e in errs.items():
                worst[name] = max(worst[name], e)
                assert e <= rtol, f"step {s}: {name} error {e:.3e} > {rtol:.0e}"
            alive = np.asarray(to_np(sim.bond_alive()), dtype=bool)
            assert np.array_equal(alive, g["frame_alive"][k]), f"step {s}: bond state differs"
            check_accounting(np.asarray(sim.accounting_vector()), g["frame_acc"][k], rtol)
            k += 1
        if s < last:
            if loads_fn is None:
                sim.step()
            else:
                sim.step(loads_fn(s), load_time=sim.time)
    mode, t, ext, en = (to_np(x) for x in sim.failure_ledger())
    assert np.array_equal(np.asarray(mode, dtype=np.uint8), g["failure_mode"]), "failure modes differ"
    assert np.array_equal(np.asarray(t), g["failure_time_s"]), "failure times differ"
    assert normwise(ext, g["failure_extension_m"]) <= rtol
    assert normwise(en, g["failure_energy_J"]) <= rtol
    check_accounting(np.asarray(sim.accounting_vector()), g["final_acc"], rtol)
    return worst
