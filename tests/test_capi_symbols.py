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


STRUCTS = ("AtmParams", "AtmImage", "AtmState", "AtmBuildArgs", "AtmBatchJob", "AtmBatchTuning", "AtmSampleOptions",
           "AtmSurrogate", "AtmPostConfig", "AtmShadeParams", "AtmShadeImages", "AtmRasterMesh", "AtmRasterOutputs",
           "AtmOceanConfig", "AtmOceanImages")


def test_binding_struct_layouts_match_the_header(tmp_path):
    """Every ctypes structure of the binding has the C header's size and the
    same offset for every field (a C program compiled against the header
    prints them)."""

    import shutil

    from planet_renderer_gb300 import _native

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "atm_capi.h"', "int main(void) {"]
    for name in STRUCTS:
        cls = getattr(_native, name)
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{name} {field} %zu\\n", offsetof({name}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    c_side = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        *key, value = line.split()
        c_side[tuple(key)] = int(value)
    for name in STRUCTS:
        cls = getattr(_native, name)
        assert ctypes.sizeof(cls) == c_side[(name, "size")], name
        for field, _ in cls._fields_:
            assert getattr(cls, field).offset == c_side[(name, field)], (name, field)


def test_new_entry_points_reject_bad_arguments_before_any_device_call(library_path):
    """The raster and ocean entry points validate their arguments on the host
    and return ATM_E_INVALID with a message (no GPU is needed to reach it)."""

    from planet_renderer_gb300 import _native

    lib = _native.library()
    out = ctypes.c_void_p()
    assert lib.atm_raster_create(0, 16, 4, 8, ctypes.byref(out)) == _native.ATM_E_INVALID
    assert lib.atm_raster_create(16, 20000, 4, 8, ctypes.byref(out)) == _native.ATM_E_INVALID
    assert b"raster size" in lib.atm_last_error()
    assert lib.atm_raster_create(16, 16, 0, 8, ctypes.byref(out)) == _native.ATM_E_INVALID
    assert lib.atm_raster_terrain(None, None, 0.5, 0.6, 0, None, None, None) == _native.ATM_E_INVALID
    cfg = _native.AtmOceanConfig()
    for field, value, message in (("spectrum_resolution", 100, b"spectrum_resolution"),
                                  ("geometry_cascades", 4, b"geometry_cascades"),
                                  ("wind_speed_mps", 50.0, b"wind_speed")):
        c = _native.AtmOceanConfig()
        c.surface_enabled, c.enabled, c.normal_strength, c.max_visible_depth_m = 1, 1, 0.32, 80.0
        c.spectrum_resolution, c.geometry_cascades, c.wind_speed_mps = 128, 2, 8.0
        c.wave_height_scale, c.choppiness, c.geometry_max_distance_m = 1.0, 0.65, 25000.0
        setattr(c, field, value)
        assert lib.atm_ocean_create(ctypes.byref(c), ctypes.byref(out)) == _native.ATM_E_INVALID
        assert message in lib.atm_last_error(), field
    cfg.albedo[:] = [0.1, 2.0, 0.1]
    assert lib.atm_ocean_create(ctypes.byref(cfg), ctypes.byref(out)) == _native.ATM_E_INVALID
    basis = _native.c_double9(1, 0, 0, 0, 1, 0, 0, 0, 1)
    assert lib.atm_ocean_rasterize(None, None, None, 1.0, 1.0, basis, basis, 0.5, 0.0, 0, None) == _native.ATM_E_INVALID
