"""Display post-process on the CPU: the oracle against the reference's own
postprocess.py (golden vectors made by running it through the float32 Taichi
stand-in, tests/golden/make_golden.py), the configuration's validation
against the reference's, and the C ABI's validation (no CUDA call)."""

from __future__ import annotations

import ctypes
import json
import math
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "postprocess.npz"
DEFAULTS = dict(exposure_ev=0.0, bloom_threshold=1.0, bloom_knee=0.5, bloom_clamp=8.0, bloom_strength=0.08,
                bloom_passes=4)


def golden_cases():
    g = np.load(GOLDEN)
    meta = json.loads(str(g["meta"]))
    for k in range(meta["cases"]):
        args = json.loads(str(g[f"case{k}_args"]))
        yield k, g[f"case{k}_hdr"], g[f"case{k}_display"], args


def test_golden_covers_the_branches():
    seen = {"bloom_off": False, "tone_map_off": False, "no_passes": False, "srgb_linear": False, "odd": False}
    for _, hdr, display, a in golden_cases():
        seen["bloom_off"] |= not a["bloom"]
        seen["tone_map_off"] |= not a["tone_map"]
        seen["no_passes"] |= a["config"].get("bloom_passes", 4) == 0
        seen["srgb_linear"] |= a["tone_map"] and bool((display <= 0.0031308 * 12.92).any())
        seen["odd"] |= a["width"] % 2 == 1 and a["height"] % 2 == 1
    assert all(seen.values()), seen


@pytest.mark.parametrize("case", range(9))
def test_oracle_matches_the_reference_bit_for_bit(case):
    from oracle import postprocess as op

    k, hdr, display, a = list(golden_cases())[case]
    cfg = SimpleNamespace(**{**DEFAULTS, **a["config"]})
    got = op.process(hdr, a["exposure_ev"], cfg, bloom=a["bloom"], tone_map=a["tone_map"])
    assert got.dtype == np.float32 and got.shape == display.shape
    assert np.array_equal(got, display), np.abs(got - display).max()


def test_blur_keeps_a_constant_plane_and_sums_to_one():
    from oracle import postprocess as op

    assert float(op.W0 + 2 * op.W1 + 2 * op.W2) == pytest.approx(1.0, abs=1e-6)
    plane = np.full((7, 5, 3), 0.75, np.float32)
    out = op.blur_vertical(op.blur_horizontal(plane))
    np.testing.assert_allclose(out, 0.75, rtol=1e-6)


def test_display_transform_endpoints():
    from oracle import postprocess as op

    v = np.array([0.0, 1e-4, 0.01, 1.0, 1e6], np.float32)
    d = op.display_from_exposed(v)
    assert d[0] == 0.0 and np.all(np.diff(d) > 0) and d[-1] <= 1.0
    assert d[1] < 0.0031308 * 12.92  # linear sRGB segment


# ---- configuration ------------------------------------------------------------------
@pytest.mark.parametrize("kwargs,message", [
    (dict(exposure_ev=21.0), "exposure_ev must be finite and in [-20, 20]"),
    (dict(exposure_ev=math.nan), "exposure_ev must be finite"),
    (dict(bloom_threshold=-1.0), "bloom_threshold must be finite and non-negative"),
    (dict(bloom_knee=math.inf), "bloom_knee must be finite and non-negative"),
    (dict(bloom_clamp=-0.1), "bloom_clamp must be finite and non-negative"),
    (dict(bloom_strength=math.nan), "bloom_strength must be finite and non-negative"),
    (dict(bloom_passes=9), "bloom_passes must be in 0..8"),
    (dict(bloom_passes=-1), "bloom_passes must be in 0..8"),
])
def test_config_validation_matches_the_reference(kwargs, message):
    from planet_renderer_gb300.postprocess import PostprocessConfig

    with pytest.raises(ValueError, match=message.replace("[", r"\[").replace("]", r"\]")):
        PostprocessConfig(**kwargs)


def test_config_from_mapping():
    from planet_renderer_gb300.postprocess import PostprocessConfig

    assert PostprocessConfig.from_mapping({}) == PostprocessConfig()
    c = PostprocessConfig.from_mapping({"exposure_ev": "1.5", "bloom_passes": 2.0, "bloom_knee": 0})
    assert c.exposure_ev == 1.5 and c.bloom_passes == 2 and isinstance(c.bloom_passes, int) and c.bloom_knee == 0.0


@pytest.mark.parametrize("field,value", [("exposure_ev", 25.0), ("bloom_clamp", -1.0), ("bloom_passes", 12)])
def test_c_abi_rejects_what_the_reference_rejects(field, value):
    """atm_post_create validates before it touches the GPU."""

    from planet_renderer_gb300 import _native

    lib = _native.library()
    cfg = _native.AtmPostConfig(0.0, 1.0, 0.5, 8.0, 0.08, 4)
    setattr(cfg, field, value)
    out = ctypes.c_void_p()
    rc = lib.atm_post_create(ctypes.byref(cfg), 64, 32, ctypes.byref(out))
    assert rc == _native.ATM_E_INVALID and not out.value
    assert field in lib.atm_last_error().decode()
    cfg = _native.AtmPostConfig(0.0, 1.0, 0.5, 8.0, 0.08, 4)
    assert lib.atm_post_create(ctypes.byref(cfg), 0, 32, ctypes.byref(out)) == _native.ATM_E_INVALID


def test_c_abi_shading_rejects_bad_arguments():
    """atm_shade_surface validates before it touches the GPU."""

    from planet_renderer_gb300 import _native

    lib = _native.library()
    params = _native.AtmShadeParams()
    images = _native.AtmShadeImages()
    image = _native.AtmImage(16, 8, 8, 1, 3)
    assert lib.atm_shade_surface(None, ctypes.byref(images), ctypes.byref(image), None) == _native.ATM_E_INVALID
    # every image pointer is required
    assert lib.atm_shade_surface(ctypes.byref(params), ctypes.byref(images), ctypes.byref(image),
                                 None) == _native.ATM_E_INVALID
    assert "null image pointer" in lib.atm_last_error().decode()
    bad = _native.AtmImage(16, 8, 8, 1, 5)  # rejected before any pointer is looked at
    assert lib.atm_shade_surface(ctypes.byref(params), ctypes.byref(images), ctypes.byref(bad),
                                 None) == _native.ATM_E_INVALID
    assert "channels" in lib.atm_last_error().decode()


def test_c_abi_post_process_rejects_null_handles():
    from planet_renderer_gb300 import _native

    lib = _native.library()
    image = _native.AtmImage(16, 8, 8, 1, 3)
    assert lib.atm_post_process(None, None, None, ctypes.byref(image), 0.0, 1, 1, None) == _native.ATM_E_INVALID
    assert lib.atm_post_read_bloom(None, None, None, None) == _native.ATM_E_INVALID
