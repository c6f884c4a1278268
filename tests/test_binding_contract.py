"""The drop-in classes against the reference's frozen binding contract.

The reference's ``binding_contract.verify()`` (src/tensordem/binding_contract.py:414)
checks a class statically: state attributes, properties, methods, parameter
names, kinds, defaults and annotations. ``tests/golden/make_contract_report.py``
runs it on ``IceDEM``, ``CalibratedIceDEM`` and ``IceDEM3D`` and commits the report; this test
checks the committed report, and re-runs ``verify()`` live whenever the
reference package is importable.
"""

import importlib.util
import json
from pathlib import Path

import pytest

REPORT = Path(__file__).resolve().parent / "golden" / "binding_contract_report.json"


def test_committed_report_conforms():
    rep = json.loads(REPORT.read_text())
    for name in ("IceDEM", "CalibratedIceDEM", "IceDEM3D"):
        r = rep["classes"][name]
        assert r["status"] == "CONFORMS" and r["breaking"] == 0 and r["other"] == 0, name
        assert r["checks"] == r["matched"] > 20, name


@pytest.mark.skipif(importlib.util.find_spec("tensordem") is None
                    or importlib.util.find_spec("tensordem.binding_contract") is None,
                    reason="the reference package is not importable here")
def test_live_verify_conforms():
    import sys
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_contract_report
    live = make_contract_report.report()
    for name, r in live["classes"].items():
        assert r["status"] == "CONFORMS" and r["breaking"] == 0, (name, r["findings"])
