"""Check this package's IceDEM classes against the reference's frozen binding contract.

Run where the reference source tree is available::

    PYTHONPATH=<reference>/src python tests/golden/make_contract_report.py

It imports ``tensordem.binding_contract`` (src/tensordem/binding_contract.py)
and runs its ``verify()`` on ``tensordem_gb300.IceDEM`` and
``tensordem_gb300.CalibratedIceDEM`` against the contract's ``IceDEM`` entry,
and on ``tensordem_gb300.IceDEM3D`` against its ``IceDEM3D`` entry.
``verify()`` accepts a class and checks it statically: state attributes,
properties, method names, parameters, kinds and annotations.
Output: tests/golden/binding_contract_report.json.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent / "binding_contract_report.json"


def report() -> dict:
    sys.path.insert(0, str(ROOT))
    from tensordem import binding_contract as bc

    from tensordem_gb300 import CalibratedIceDEM, IceDEM, IceDEM3D
    out = {"contract_version": bc.BINDING_CONTRACT.get("version", bc.BINDING_CONTRACT.get("contract_version")),
           "frozen_fingerprint": bc.FROZEN_FINGERPRINT, "classes": {}}
    for cls, entry in ((IceDEM, "IceDEM"), (CalibratedIceDEM, "IceDEM"), (IceDEM3D, "IceDEM3D")):
        contract = dict(bc.BINDING_CONTRACT)
        contract["entries"] = {entry: bc.BINDING_CONTRACT["entries"][entry]}
        r = bc.verify({entry: cls}, contract=contract)
        out["classes"][cls.__name__] = {k: r[k] for k in ("status", "checks", "matched", "breaking", "other")}
        out["classes"][cls.__name__]["findings"] = r["findings"]
    return out


def main() -> None:
    out = report()
    OUT.write_text(json.dumps(out, indent=1, sort_keys=True, default=str) + "\n")
    print(json.dumps({k: {kk: v[kk] for kk in ("status", "checks", "matched")} for k, v in out["classes"].items()}))


if __name__ == "__main__":
    main()
