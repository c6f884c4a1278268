"""Continuous batching: every served result equals the same request solved alone.

Requests arrive while others are on the GPU, join at step-block boundaries,
freeze at their own step counts and retire after the block. With a fixed
rebuild interval that divides the block length (and slow enough motion that
the displacement bound never forces an extra rebuild), a request's final
state and ledger are bit-identical to a solve of that request alone.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _alone(bt, req, every, block):
    b = bt.Batch(bt.BatchConfig(particle_capacity=req.n + 64, key_capacity=req.spec.build().keys + 64,
                                max_instances=4, rebuild_every=every))
    iid = b.admit(req.spec.build())
    b.set_steps(iid, req.steps)
    done = 0
    while done < req.steps:
        b.step(block)
        done += block
    return b.read(iid)


def test_served_results_equal_solo_results():
    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from tensordem_gb300 import batch as bt
    from tensordem_gb300.serve import make_trace, serve
    trace = make_trace(duration=0.06, rate=250.0, n_min=200, n_max=2000, s_min=100, s_max=800, seed=1)
    assert len(trace) >= 6
    rep = serve(trace, budget_bytes=int(2e9), block=20, rebuild_every=10, keep_state=True)
    assert rep["completed"] == len(trace) and rep["status_errors"] == 0
    overlapped = 0
    for r in rep["done"]:
        others = [q for q in rep["done"] if q is not r and q.admitted < r.done and q.done > r.admitted]
        overlapped += bool(others)
        solo = _alone(bt, r, 10, 20)
        for k in ("pos", "vel", "omega", "force", "torque"):
            assert np.array_equal(r.state[k], solo[k]), (r.index, k)
        for k in ("kinetic", "dissipated", "total", "evals", "peak_load", "broken"):
            assert r.ledger[k] == solo["ledger"][k], (r.index, k)
        assert r.ledger["evals"] == r.steps
    assert overlapped >= len(trace) // 2  # most requests shared the GPU with others
    lat = rep["latency_s"]
    assert 0 < lat["p50"] <= lat["p95"] <= lat["p99"]
