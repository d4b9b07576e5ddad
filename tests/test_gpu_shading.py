"""Surface shading on the GPU (atm_shade_surface) against the reference's own
kernel (golden vectors) and the oracle restatement, in both layouts and with
3 or 4 channels.  The kernel follows the reference's float32 operations
without contraction; expf's last bits may differ (tolerance 1e-5 relative)."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "shading.npz"
GBUFFER = ("position", "normal", "albedo", "water_depth", "seabed_albedo", "seabed_normal", "slope_variance",
           "surface_id", "terrain_position", "terrain_normal", "terrain_albedo", "terrain_surface_id")


def _ocean(args):
    from planet_renderer_gb300.shading import OceanShading

    return OceanShading(enabled=bool(args["advanced_ocean_enabled"]), roughness=args["ocean_roughness"],
                        dielectric_f0=args["ocean_f0"], sky_reflection_strength=args["ocean_sky_strength"],
                        absorption_per_m=tuple(args["ocean_absorption"]),
                        scattering_per_m=tuple(args["ocean_scattering"]), max_visible_depth_m=args["ocean_max_depth"],
                        refraction_index=args["ocean_refraction_index"],
                        refraction_strength=args["ocean_refraction_strength"],
                        refraction_max_offset_pixels=args["ocean_refraction_max_offset_pixels"])


def _run(fields, args, ocean_id, channels=3, layout="wh"):
    from planet_renderer_gb300.shading import shade_surface

    def dev(a):
        t = torch.as_tensor(np.ascontiguousarray(a), device="cuda")
        if t.dim() == 3 and channels == 4:
            t = torch.cat([t, torch.full_like(t[..., :1], 9.0)], -1)
        if layout == "hw":
            t = t.transpose(0, 1).contiguous()
        return t

    gb = {n: dev(fields[n]) for n in GBUFFER}
    sun_t, sky = dev(fields["sun_transmittance"]), dev(fields["sky_radiance"])
    out = torch.full_like(sun_t, -1.0)
    shade_surface(gb, sun_t, sky, out, args["sun_global"], args["solar_irradiance"],
                  (args["view_right_global"], args["view_up_global"], args["view_forward_global"]), _ocean(args),
                  args["sun_angular_radius"], args["tangent_half_fov"], args["mode"], layout=layout,
                  ocean_surface_id=ocean_id)
    torch.cuda.synchronize()
    if channels == 4:
        assert bool((out[..., 3] == -1.0).all())
    out = out[..., :3]
    if layout == "hw":
        out = out.transpose(0, 1)
    return out.cpu().numpy()


def test_golden_vectors_of_the_reference():
    g = np.load(GOLDEN)
    meta = json.loads(str(g["meta"]))
    exact = total = 0
    for k in range(meta["cases"]):
        fields = {n: g[f"case{k}_{n}"] for n in GBUFFER + ("sun_transmittance", "sky_radiance")}
        args = json.loads(str(g[f"case{k}_args"]))
        got = _run(fields, args, meta["ocean_surface_id"])
        ref = g[f"case{k}_surface_hdr"]
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-9, err_msg=f"case {k}")
        exact += int((got == ref).sum())
        total += ref.size
    print(f"surface shading golden: {exact}/{total} values bit-identical")


@pytest.mark.parametrize("channels,layout", [(3, "hw"), (4, "wh"), (4, "hw")])
def test_layouts_against_the_oracle(channels, layout):
    from oracle.shading import shade_surface

    g = np.load(GOLDEN)
    meta = json.loads(str(g["meta"]))
    for k in (0, 1):
        fields = {n: g[f"case{k}_{n}"] for n in GBUFFER + ("sun_transmittance", "sky_radiance")}
        args = json.loads(str(g[f"case{k}_args"]))
        got = _run(fields, args, meta["ocean_surface_id"], channels, layout)
        ref = shade_surface(fields, args, meta["ocean_surface_id"])
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-9, err_msg=f"case {k} {channels} {layout}")


def test_argument_checks():
    from planet_renderer_gb300.shading import OceanShading, shade_surface

    g = np.load(GOLDEN)
    fields = {n: torch.as_tensor(g[f"case0_{n}"], device="cuda") for n in GBUFFER}
    args = json.loads(str(g["case0_args"]))
    out = torch.zeros_like(fields["albedo"])
    bad = dict(fields, water_depth=fields["water_depth"][:-1])
    with pytest.raises(ValueError):
        shade_surface(bad, out, out, out, args["sun_global"], args["solar_irradiance"],
                      (args["view_right_global"], args["view_up_global"], args["view_forward_global"]),
                      OceanShading(), 0.0046, 0.577)
