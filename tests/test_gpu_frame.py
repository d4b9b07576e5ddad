"""The fused frame (atm_render_frame): surface lighting, surface shading and
the composite in one pass must give the frame that the separate calls give
(prepare_frame -> shade_surface -> composite, renderer.py:1671-1727), for
the plain composite and for the surrogate composite, in both layouts.  The
shading step itself is pinned to the reference's golden G-buffers by
test_gpu_shading.py; the fused kernel calls the same device function."""

from __future__ import annotations

import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

E = (4.0, 3.9, 3.7)
AR_DEG = 0.266


def _frame(width, height, altitude_m, zenith_deg, azimuth_deg, layout="wh"):
    from planet_renderer_gb300.atmosphere import AtmosphereRenderer, scene
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M, CameraView
    from planet_renderer_gb300.lighting import LightingState

    v = CameraView(altitude_m, zenith_deg, azimuth_deg)
    gb = scene.synthesize_gbuffer(width, height, EARTH_RADIUS_M, v.altitude_m, v.basis, v.tangent_half_fov,
                                  v.sun_local, E, seed=11, device="cuda")
    images = scene.shading_inputs(gb, EARTH_RADIUS_M, v.altitude_m, v.basis)
    images["space_hdr"] = gb["space_hdr"]
    if layout == "hw":
        images = {k: t.transpose(0, 1).contiguous() for k, t in images.items()}
    r = AtmosphereRenderer(width, height, earth_baseline(), layout=layout)
    r.update(EARTH_RADIUS_M, v.camera_radius_m, v.sun_local.copy(), E, AR_DEG)
    args = (EARTH_RADIUS_M, v.camera_radius_m, v.sun_local, E, LightingState(v.sun_local, AR_DEG, E).sun_disk_radiance,
            AR_DEG, v.basis, v.tangent_half_fov, 4.0, 12.0)
    return r, images, args, v


def _separate(r, images, args, v, surrogate=None, check_fraction=0.0):
    from planet_renderer_gb300.shading import OceanShading, shade_surface

    R, cr, sun, E_, disk, ar, basis, tanfov, s0, s1 = args
    r.prepare_frame(images["position"], images["surface_id"], R, cr, sun, E_, ar, basis, tanfov)
    surface_hdr = torch.empty_like(images["position"])
    gbuffer = {k: t for k, t in images.items() if k != "space_hdr"}
    shade_surface(gbuffer, r.surface_sun_transmittance, r.surface_sky_radiance, surface_hdr, sun, E_, basis,
                  OceanShading(), math.radians(ar), tanfov, layout=r.layout)
    hdr = torch.full_like(surface_hdr, -1.0)
    r.radiance_samples(reset=True)  # the composite's samples only (prepare_frame built the aerial volume)
    if surrogate is None:
        r.composite(surface_hdr, images["space_hdr"], images["surface_id"], images["position"], hdr, *args)
    else:
        r.composite_surrogate(surface_hdr, images["space_hdr"], images["surface_id"], images["position"], hdr, *args,
                              surrogate=surrogate, check_fraction=check_fraction, seed=3)
    torch.cuda.synchronize()
    return hdr.cpu().numpy()


def _fused(r, images, args, surrogate=None, check_fraction=0.0):
    gbuffer = {k: t for k, t in images.items() if k != "space_hdr"}
    hdr = torch.full_like(images["position"], -1.0)
    r.render_frame(gbuffer, images["space_hdr"], hdr, *args, surrogate=surrogate, check_fraction=check_fraction,
                   seed=3)
    torch.cuda.synchronize()
    return hdr.cpu().numpy()


@pytest.mark.parametrize("altitude,zenith,layout", [(2000.0, 40.0, "wh"), (50_000.0, 80.0, "hw"),
                                                    (2_000_000.0, 60.0, "wh")])
def test_fused_frame_is_the_separate_calls(altitude, zenith, layout):
    """Plain composite: every pixel of a land-and-ocean frame, and the
    radiance-sample count."""

    r, images, args, v = _frame(256, 144, altitude, zenith, 30.0, layout)
    ref = _separate(r, images, args, v)
    n_ref = r.radiance_samples(reset=True)
    got = _fused(r, images, args)
    n_got = r.radiance_samples(reset=True)
    assert n_got == n_ref > 0
    assert (got >= 0).all()
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-9)
    r.close()


def test_fused_surrogate_frame_is_the_separate_calls():
    """Surrogate composite without networks (every surface pixel through the
    fallback queue, which re-shades it) and with every MLP pixel checked:
    the fused frame equals the separate calls."""

    from planet_renderer_gb300.atmosphere.mlp import Mlp
    from planet_renderer_gb300.atmosphere.surrogate import Surrogate

    r, images, args, v = _frame(256, 144, 2000.0, 40.0, 30.0)
    plain = _separate(r, images, args, v)
    got = _fused(r, images, args, surrogate=Surrogate(None, None))
    np.testing.assert_allclose(got, plain, rtol=1e-5, atol=1e-9)
    sg = Surrogate(Mlp(11, 4, 6, seed=5, device=r.device), None)
    got = _fused(r, images, args, surrogate=sg, check_fraction=1.0)
    np.testing.assert_allclose(got, plain, rtol=1e-5, atol=1e-9)
    ref = _separate(r, images, args, v, surrogate=sg, check_fraction=0.0)
    got = _fused(r, images, args, surrogate=sg, check_fraction=0.0)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-9)
    r.close()


def test_fused_frame_rejects_a_missing_lut_and_image():
    from planet_renderer_gb300.atmosphere import AtmosphereRenderer
    from planet_renderer_gb300.atmosphere.config import earth_baseline

    r, images, args, v = _frame(64, 36, 2000.0, 40.0, 30.0)
    gbuffer = {k: t for k, t in images.items() if k not in ("space_hdr", "albedo")}
    with pytest.raises(ValueError):
        r.render_frame(gbuffer, images["space_hdr"], torch.zeros_like(images["position"]), *args)
    fresh = AtmosphereRenderer(64, 36, earth_baseline())
    gbuffer = {k: t for k, t in images.items() if k != "space_hdr"}
    with pytest.raises(RuntimeError):
        fresh.render_frame(gbuffer, images["space_hdr"], torch.zeros_like(images["position"]), *args)
    fresh.close()
    r.close()
