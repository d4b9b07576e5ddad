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


@pytest.mark.parametrize("n", [2, 5, 12, 32])
def test_patch_topology_is_the_reference_topology(n):
    """raster.shared_topology (the triangle list a patch is drawn with) equals
    the reference's _shared_topology (renderer.py:78-100)."""

    from planet_renderer_gb300.raster import shared_topology

    data, _ = load_golden("raster")
    np.testing.assert_array_equal(shared_topology(n), data[f"topology{n}"])


def test_synthetic_terrain_draws_with_skirts():
    """The bench's synthetic terrain frame covers the ground part of the frame
    and its skirts fill the seams between rows of different column spacing
    (checked with the oracle at a small size)."""

    from oracle import raster
    from planet_renderer_gb300.raster import synthetic_terrain

    W, H = 96, 54
    m = synthetic_terrain(W, H, 0.6, rows=4, columns=4, resolution=4, device="cpu")
    a = {k: (v.numpy() if hasattr(v, "numpy") else v) for k, v in m.items()}
    g = raster.render(a["view"], a["normal"], a["material"], a["height_m"], a["cell"], a["triangles"],
                      list(a["active_slots"]), 0.5, 0.6, W, H, 0, a["slot_level"], a["surface_triangles"],
                      a["resolution"], a["skirt_mask"])
    covered = g["surface_id"] >= 0
    assert 0.3 < covered.mean() < 0.9
    assert covered[:, 0].all() and not covered[:, -1].any()  # ground at the bottom, sky at the top
    local = g["surface_id"][covered] % len(a["triangles"])
    assert (local >= a["surface_triangles"]).any()
