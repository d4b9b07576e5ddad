"""The ocean coverage oracle (oracle/ocean.py) against the reference's own
kernels (golden vectors of OceanRenderer.rasterize with
_build_directional_spectrum and _rasterize through the float32 Taichi
stand-in, tests/golden/make_golden.py), and the OceanConfig mirror's
validation and JSON mapping (ocean.py:38-190)."""

from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import load_golden

IMAGES = ("depth", "position", "normal", "albedo", "material_weights", "height_m", "water_depth", "seabed_albedo",
          "seabed_normal", "slope_variance", "surface_id", "cell_id")


def golden_case(case):
    data, _ = load_golden("ocean")
    p = f"case{case}_"
    a = json.loads(str(data[p + "args"]))
    inputs = {n: data[p + "in_" + n] for n in IMAGES}
    outputs = {n: data[p + n] for n in IMAGES}
    spectrum = None
    if p + "spectrum_height" in data.files:
        spectrum = tuple(data[p + "spectrum_" + n] for n in ("height", "gradient", "displacement", "jacobian"))
    return a, inputs, outputs, spectrum


@pytest.mark.parametrize("case", [0, 1, 2, 3])
def test_oracle_matches_the_reference_ocean(case):
    from oracle import ocean

    a, inputs, ref, ref_spectrum = golden_case(case)
    cfg = ocean.OceanSettings(**a["config"])
    got, spectrum = ocean.rasterize(inputs, cfg, a["planet_radius_m"], a["camera_altitude_m"], a["planet_frame"],
                                    a["view_basis"], a["tangent_half_fov"], a["time_seconds"], a["debug_mode"])
    if ref_spectrum is not None:
        for name, x, y in zip(("height", "gradient", "displacement", "jacobian"), spectrum, ref_spectrum):
            np.testing.assert_array_equal(x, y, err_msg=name)
    for name in IMAGES:
        np.testing.assert_array_equal(got[name], ref[name], err_msg=name)
    covered = ref["surface_id"] == ocean.OCEAN_SURFACE_ID
    assert covered.sum() > 50
    assert (covered & (inputs["surface_id"] >= 0)).sum() > 5  # the sea in front of terrain pixels
    assert (~covered & (inputs["surface_id"] >= 0)).sum() > 5  # terrain in front of the sea


def test_ocean_config_mirrors_the_reference():
    from planet_renderer_gb300.ocean import OceanConfig, opaque_surface_height_m

    c = OceanConfig()
    assert c.spectrum_resolution == 128 and c.geometry_cascades == 2 and c.albedo == (0.012, 0.055, 0.16)
    for kwargs, message in (({"albedo": (0.1, 0.2)}, "three components"), ({"albedo": (0.1, 2.0, 0.1)}, "0..1"),
                            ({"roughness": 0.01}, "roughness"), ({"spectrum_resolution": 100}, "32, 64, 128 or 256"),
                            ({"wind_speed_mps": 50.0}, "wind_speed"), ({"geometry_cascades": 4}, "geometry_cascades"),
                            ({"absorption_per_m": (0.1, -1.0, 0.1)}, "non-negative"),
                            ({"wind_direction_degrees": float("nan")}, "finite"),
                            ({"refraction_max_offset_pixels": -1.0}, "refraction_max_offset_pixels")):
        with pytest.raises(ValueError, match=message):
            OceanConfig(**kwargs)
    m = OceanConfig.from_mapping({"enabled": 0, "albedo": [0.1, 0.2, 0.3], "spectrum_resolution": "64",
                                  "wind_speed_mps": 12})
    assert m.enabled is False and m.albedo == (0.1, 0.2, 0.3) and m.spectrum_resolution == 64
    assert m.wind_speed_mps == 12.0 and m.choppiness == c.choppiness
    with pytest.raises(ValueError):
        OceanConfig.from_mapping({"albedo": 0.3})
    assert opaque_surface_height_m(-120.0, True) == 0.0 and opaque_surface_height_m(-120.0, False) == -120.0
    assert m.shading().enabled is False
