"""Single-ray oracle entry points (used to judge the learned surrogates)
agree with the LUT and composite kernels they restate."""

from __future__ import annotations

import dataclasses
import math

import numpy as np

E = (4.0, 3.9, 3.7)
AR = math.radians(0.266)
R = 6_360_000.0


def _luts(oracle, cfg):
    tl = oracle.build_transmittance(cfg, R)
    ms = oracle.build_multi_scattering(cfg, R, E, AR, tl)
    return tl, ms


def _cfg():
    from planet_renderer_gb300.atmosphere.config import earth_baseline

    return dataclasses.replace(earth_baseline(), sky_view_lut_width=24, sky_view_lut_height=16)


def test_sky_rays_reproduce_sky_view_texels():
    from oracle.atm import Oracle

    o = Oracle("f64")
    cfg = _cfg()
    tl, ms = _luts(o, cfg)
    alt, sun_cos = 2000.0, 0.3
    lut = o.build_sky_view(cfg, R, alt, sun_cos, E, AR, tl, ms)
    W, H = lut.shape[:2]
    rho = math.sqrt(alt * (2 * R + alt))
    hz = math.pi - math.acos(min(max(rho / (R + alt), 0.0), 1.0))
    rays, idx = [], []
    for x in range(0, W, 5):
        for y in range(H):
            az = (x + 0.5) / W * math.pi
            v = (y + 0.5) / H
            zen = hz * (1 - (1 - 2 * v) ** 2) if v < 0.5 else hz + (math.pi - hz) * (2 * v - 1) ** 2
            rays.append((math.sin(zen) * math.cos(az), math.cos(zen), math.sin(zen) * math.sin(az)))
            idx.append((x, y))
    n = len(rays)
    sun = (math.sqrt(1 - sun_cos ** 2), sun_cos, 0.0)
    got = o.sky_rays(cfg, R, np.full(n, alt), np.array(rays), np.tile(sun, (n, 1)), E, AR, tl, ms)
    ref = np.array([lut[x, y] for x, y in idx])
    np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-15)


def test_surface_rays_reproduce_composite_views():
    from oracle.atm import Oracle
    from planet_renderer_gb300.atmosphere.diagnostics import AtmosphereDiagnosticView as V

    o = Oracle("f64")
    cfg = _cfg()
    tl, ms = _luts(o, cfg)
    W, H, alt = 12, 8, 3000.0
    basis = ((1.0, 0.0, 0.0), (0.0, 0.8, 0.6), (0.0, -0.6, 0.8))
    tanfov = math.tan(math.radians(30))
    sun = np.array([0.3, 0.5, -0.2])
    sun /= np.linalg.norm(sun)
    rng = np.random.default_rng(3)
    # view-space surface points along each pixel ray at 2..60 km
    pos = np.zeros((W, H, 3))
    rays = np.zeros((W, H, 3))
    dist = rng.uniform(2e3, 6e4, (W, H))
    for x in range(W):
        for y in range(H):
            sx = ((x + 0.5) / W * 2 - 1) * W / H
            sy = (y + 0.5) / H * 2 - 1
            vv = np.array([sx, sy, 1.0 / tanfov])
            vv /= np.linalg.norm(vv)
            pos[x, y] = vv * dist[x, y]
            rays[x, y] = np.array(basis[0]) * vv[0] + np.array(basis[1]) * vv[1] + np.array(basis[2]) * vv[2]
    sid = np.zeros((W, H), np.int32)
    zeros = np.zeros((W, H, 3))
    common = dict(config=cfg, scene_hdr=zeros, space_hdr=zeros, surface_id=sid, position_view=pos, bottom_radius=R,
                  camera_altitude=alt, sky_lut_camera_altitude=alt, sun=sun, irradiance=E, disk_radiance=(0, 0, 0),
                  angular_radius_rad=AR, basis=basis, tangent_half_fov=tanfov, star_start=4.0, star_end=12.0,
                  tlut=tl, mslut=ms, svlut=np.zeros((cfg.sky_view_lut_width, cfg.sky_view_lut_height, 3)),
                  aplut=np.zeros((cfg.aerial_lut_width, cfg.aerial_lut_height, cfg.aerial_lut_depth, 3)))
    L_view, _ = o.composite(diagnostic_view=int(V.AERIAL_SCATTERING), **common)
    T_view, _ = o.composite(diagnostic_view=int(V.AERIAL_TRANSMITTANCE), **common)
    n = W * H
    L, T = o.surface_rays(cfg, R, np.full(n, alt), rays.reshape(n, 3), dist.reshape(n), np.tile(sun, (n, 1)), E, AR,
                          tl, ms)
    np.testing.assert_allclose(L, L_view.reshape(n, 3), rtol=1e-7, atol=1e-14)
    np.testing.assert_allclose(T, T_view.reshape(n, 3), rtol=1e-7, atol=1e-14)
