"""CPU checks of the C ABI: the library loads and exports every declared symbol.

No compute call is made (there is no GPU here); loading the library only needs
the CUDA runtime shared object.
"""

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> list[str]:
    names = []
    for header in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        names += re.findall(r"\b(tdem_\w+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def library():
    from tensordem_gb300 import build
    path = build.build()
    return ctypes.CDLL(str(path))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "tdem_icedem_step" in names and "tdem_icedem_create" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(library):
    missing = [n for n in declared_functions() if not hasattr(library, n)]
    assert not missing, f"undefined in libtdem_sm103.so: {missing}"


def test_version_and_capacity(library):
    assert library.tdem_version() >= 1
    assert library.tdem_icedem_max_discs() >= 105


def test_variant_counts(library):
    """Host-only queries: twelve single-engine step-kernel variants and six
    batched shapes (block size, CTAs per SM, tiles per work grab)."""
    assert library.tdem_hm_num_variants() == 12
    assert library.tdem_batch_num_variants() == 6


def test_restitution_damping_ratio_is_a_host_routine(library):
    """The calibrated-restitution damping ratio runs on the host (no GPU):
    e = 1 needs no damping, and lower restitution needs more."""
    out = ctypes.c_double()
    ratios = []
    for e in (0.95, 0.7, 0.5, 0.3):
        assert library.tdem_hertz_damping_ratio(ctypes.c_double(e), ctypes.byref(out)) == 0
        ratios.append(out.value)
    assert all(r > 0.0 for r in ratios)
    assert ratios == sorted(ratios)
