"""The C-ABI library loads and exports every entry point include/atm_capi.h
declares (no CUDA call is made: this runs without a GPU)."""

from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions() -> set[str]:
    names = set()
    for header in HEADERS:
        text = header.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(atm_\w+)\s*\(", text, flags=re.M))
    return names


@pytest.fixture(scope="module")
def library_path():
    import build_native

    return build_native.build()


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("atm_create", "atm_destroy", "atm_update", "atm_prepare_frame", "atm_composite",
                     "atm_last_error", "atm_build_lut", "atm_read_lut"):
        assert required in names


def test_library_exports_every_declared_symbol(library_path):
    lib = ctypes.CDLL(str(library_path))
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_library_exports_nothing_else(library_path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(library_path)], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("nm unavailable")
    exported = {line.split()[-1] for line in out.stdout.splitlines() if " T " in line}
    ours = {n for n in exported if n.startswith("atm_")}
    assert ours == declared_functions()


def test_python_binding_matches_header(library_path):
    from planet_renderer_gb300 import _native

    assert set(_native.SIGNATURES) == declared_functions()
    lib = _native.library()
    assert lib.atm_last_error() == b""


def test_struct_layouts_match_between_product_and_oracle():
    from oracle import atm as oracle_atm
    from planet_renderer_gb300 import _native

    assert ctypes.sizeof(_native.AtmParams) == ctypes.sizeof(oracle_atm.AtmParams)
    assert [f[0] for f in _native.AtmParams._fields_] == [f[0] for f in oracle_atm.AtmParams._fields_]
