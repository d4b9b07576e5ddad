"""The terrain raster oracle (oracle/raster.py) against the reference's own
kernels (golden vectors of _clip, _raster_depth_direct and _resolve_raster
run through the float32 Taichi stand-in, tests/golden/make_golden.py)."""

from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import load_golden

FIELDS = ("depth", "position", "albedo", "height_m", "surface_id", "cell_id")


@pytest.mark.parametrize("case", [0, 1, 2, 3])
def test_oracle_matches_the_reference_raster(case):
    from oracle import raster

    data, meta = load_golden("raster")
    a = json.loads(str(data[f"case{case}_args"]))
    p = f"case{case}_"
    g = raster.render(data[p + "view"], data[p + "normal"], data[p + "material"], data[p + "height"],
                      data[p + "cell"], data[p + "triangles"], a["active"], a["near"], a["tangent_half_fov"],
                      a["width"], a["height"], a["mode"], data[p + "slot_level"],
                      2 * a["resolution"] ** 2, a["resolution"], data[p + "skirt_mask"])
    assert g["clipped_count"] == int(data[p + "clipped_count"])
    for name in FIELDS:
        np.testing.assert_array_equal(g[name], data[p + name], err_msg=name)
    np.testing.assert_array_equal(g["normal"], data[p + "gb_normal"])
    np.testing.assert_array_equal(g["material"], data[p + "material_weights"])
    assert (g["surface_id"] >= 0).sum() > 0
