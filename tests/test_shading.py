"""Surface shading (the consumer of prepare_frame's surface lighting,
renderer.py:1277-1575): the oracle against the reference's own kernel, run
through the float32 Taichi stand-in on seeded G-buffers (golden vectors from
tests/golden/make_golden.py --only shading)."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "shading.npz"
FIELDS = ("position", "normal", "albedo", "water_depth", "seabed_albedo", "seabed_normal", "slope_variance",
          "surface_id", "terrain_position", "terrain_normal", "terrain_albedo", "terrain_surface_id",
          "sun_transmittance", "sky_radiance")


def _case(k):
    g = np.load(GOLDEN)
    meta = json.loads(str(g["meta"]))
    fields = {n: g[f"case{k}_{n}"] for n in FIELDS}
    return fields, json.loads(str(g[f"case{k}_args"])), g[f"case{k}_surface_hdr"], meta["ocean_surface_id"]


@pytest.mark.parametrize("case", range(5))
def test_oracle_matches_the_reference_bit_for_bit(case):
    from oracle.shading import shade_surface

    fields, args, ref, ocean_id = _case(case)
    got = shade_surface(fields, args, ocean_id)
    assert got.dtype == np.float32 and got.shape == ref.shape
    assert np.array_equal(got, ref), np.abs(got - ref).max()


def test_cases_cover_land_ocean_sky_and_modes():
    from oracle.shading import SKY_COLOR

    fields, args, hdr, ocean_id = _case(3)  # albedo debug mode
    assert args["mode"] == 1
    sid = fields["surface_id"]
    np.testing.assert_array_equal(hdr[sid >= 0], fields["albedo"][sid >= 0])
    np.testing.assert_array_equal(hdr[sid < 0], np.broadcast_to(np.float32(SKY_COLOR), hdr[sid < 0].shape))
    # advanced ocean off: ocean pixels are Lambertian like land; on: they are not
    for k, lambert in ((2, True), (0, False)):
        fields, args, hdr, ocean_id = _case(k)
        n = fields["normal"] / np.linalg.norm(fields["normal"], axis=-1, keepdims=True)
        ndotl = np.maximum(n @ np.asarray(args["sun_global"]), 0.0)[..., None]
        ref = fields["albedo"] * (np.asarray(args["solar_irradiance"]) * fields["sun_transmittance"] * ndotl / np.pi
                                  + fields["sky_radiance"])
        ocean = fields["surface_id"] == ocean_id
        close = np.isclose(hdr[ocean], ref[ocean], rtol=1e-5, atol=1e-7).all(axis=-1)
        assert close.all() if lambert else not close.any()
