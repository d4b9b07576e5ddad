"""Generate golden vectors by running the reference's own atmosphere code.

    python tests/golden/make_golden.py --reference PATH [--only NAME ...]

PATH is the root of a checkout of the reference project (the directory that
holds ``src/planet_renderer``).

Imports ``planet_renderer.atmosphere`` from the reference checkout with the
float32 Taichi stand-in of ``taichi_f32_shim.py`` installed as ``taichi``, and
drives the reference's public host methods ``AtmosphereRenderer.update``,
``prepare_frame`` and ``composite`` (``atmosphere/renderer.py:2072-2238``),
which launch its kernels unchanged.  Inputs (parameters, G-buffer, camera,
sun) and outputs (every LUT, the surface-lighting fields and ``hdr`` for each
diagnostic view) are written to ``tests/golden/<name>.npz``.

``--precision f64`` runs the same reference source with every f32 replaced
by float64; the oracle's FP64 instance must then agree to rounding level,
which shows the restatement is the reference's algorithm (the f32 fixtures
then bound the rounding noise between two f32 evaluations of it).

Scenarios:
  tiny_earth, tiny_small_planet, tiny_orbit
      the LUT sizes of the reference's own integrated CPU test
      (tests/test_m2_terrain.py:215-230), full 24x16 frames, all 11 views;
  earth_config1
      the Earth workload at full LUT sizes (T 256x64/40 steps, MS 32x32 with
      64 directions x 20 steps, SV 192x108/30 steps, AP 32^3, 48 limb
      intervals): full LUTs, and a 1920x1080 frame sampled at selected pixels;
  earth_cameras
      the same LUTs re-keyed for cameras at 50 km and 2000 km with low suns
      (twilight / terminator), composite sampled at selected pixels;
  postprocess
      the display post-process (src/planet_renderer/postprocess.py) on
      seeded HDR images, nine configurations;
  shading
      the surface shading that consumes prepare_frame's outputs
      (renderer.py:1277-1575) on seeded G-buffers: land, ocean (BRDF,
      refracted seabed) and sky pixels, five configurations.

The script reads the reference only when it runs; the tests read the .npz.
"""

from __future__ import annotations

import argparse
import json
import math
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT / "planet-real-time-render_gb300"))

import taichi_f32_shim as shim  # noqa: E402

TINY_LUTS = dict(
    transmittance_lut_width=16,
    transmittance_lut_height=16,
    multi_scattering_lut_width=8,
    multi_scattering_lut_height=8,
    sky_view_lut_width=16,
    sky_view_lut_height=16,
    aerial_lut_width=4,
    aerial_lut_height=4,
    aerial_lut_depth=8,
    transmittance_steps=4,
    multi_scattering_directions=4,
    multi_scattering_steps=4,
    sky_view_steps=4,
    aerial_steps_per_slice=1,
)


def _import_reference(reference: Path):
    shim.install()
    sys.path.insert(0, str(reference / "src"))
    from planet_renderer.atmosphere import (  # type: ignore
        AtmosphereConfig,
        AtmosphereDiagnosticView,
        AtmosphereRenderer,
    )

    return AtmosphereConfig, AtmosphereDiagnosticView, AtmosphereRenderer


def _fill_field(field, array):
    field.from_numpy(np.asarray(array, dtype=field.data.dtype))


def run_scenario(name, reference, config_kwargs, planet_radius, camera_altitude, sun_zenith_deg, sun_azimuth_deg,
                 yaw_deg, pitch_deg, width, height, sample_pixels=None, seed=2027, reuse=None,
                 views=None, solar_irradiance=(4.0, 3.9, 3.7), sun_angular_radius_degrees=0.266):
    """Run one camera through update/prepare_frame/composite and collect IO."""

    import torch

    from planet_renderer_gb300 import camera as cam
    from planet_renderer_gb300.atmosphere import scene
    from planet_renderer_gb300.lighting import LightingState

    AtmosphereConfig, View, Renderer = _import_reference(reference)
    config = AtmosphereConfig(**config_kwargs)
    renderer = reuse if reuse is not None else Renderer(width, height, config)
    basis = cam.view_basis(yaw_deg, pitch_deg)
    tanfov = cam.tangent_half_fov(60.0)
    sun = cam.sun_from_zenith(sun_zenith_deg, sun_azimuth_deg)
    lighting = LightingState(sun, sun_angular_radius_degrees, solar_irradiance)
    camera_radius = planet_radius + camera_altitude

    if sample_pixels is None:
        pixels = None
        gb = scene.synthesize_gbuffer(width, height, planet_radius, camera_altitude, basis, tanfov, sun,
                                      solar_irradiance, seed=seed)
    else:
        pixels = np.asarray(sample_pixels, dtype=np.int64)
        gb = scene.synthesize_gbuffer(width, height, planet_radius, camera_altitude, basis, tanfov, sun,
                                      solar_irradiance, seed=seed, pixels=torch.as_tensor(pixels))
    gb = {k: v.numpy() for k, v in gb.items()}

    position = shim.Vector.field(3, dtype=shim.f32, shape=(width, height))
    surface = shim.field(dtype=shim.i32, shape=(width, height))
    surface.fill(-1)
    scene_hdr = shim.Vector.field(3, dtype=shim.f32, shape=(width, height))
    space_hdr = shim.Vector.field(3, dtype=shim.f32, shape=(width, height))
    hdr = shim.Vector.field(3, dtype=shim.f32, shape=(width, height))
    if pixels is None:
        _fill_field(position, gb["position_view"])
        _fill_field(surface, gb["surface_id"])
        _fill_field(scene_hdr, gb["scene_hdr"])
        _fill_field(space_hdr, gb["space_hdr"])
    else:
        for k, (x, y) in enumerate(pixels):
            position[x, y] = gb["position_view"][k]
            surface[x, y] = gb["surface_id"][k]
            scene_hdr[x, y] = gb["scene_hdr"][k]
            space_hdr[x, y] = gb["space_hdr"][k]
        shim.restrict_iteration(surface, [tuple(p) for p in pixels])
        shim.restrict_iteration(hdr, [tuple(p) for p in pixels])
        # the reference's per-pixel surface fields are frame sized
        shim.restrict_iteration(renderer.surface_sun_transmittance, [tuple(p) for p in pixels])

    t0 = time.time()
    renderer.update(planet_radius, camera_radius, sun.copy(), solar_irradiance, sun_angular_radius_degrees)
    t_update = time.time() - t0
    t0 = time.time()
    renderer.prepare_frame(position, surface, planet_radius, camera_radius, sun.copy(), solar_irradiance,
                           sun_angular_radius_degrees, basis, tanfov)
    t_prepare = time.time() - t0

    out = {}
    out["transmittance_lut"] = renderer.transmittance_lut.to_numpy()
    out["multi_scattering_lut"] = renderer.multi_scattering_lut.to_numpy()
    out["sky_view_lut"] = renderer.sky_view_lut.to_numpy()
    out["aerial_scattering_lut"] = renderer.aerial_scattering_lut.to_numpy()
    sun_t = renderer.surface_sun_transmittance.to_numpy()
    sky_l = renderer.surface_sky_radiance.to_numpy()
    views = list(View) if views is None else views
    t0 = time.time()
    for view in views:
        hdr.fill(0.0)
        renderer.composite(scene_hdr, space_hdr, surface, position, hdr, planet_radius, camera_radius, sun.copy(),
                           solar_irradiance, lighting.sun_disk_radiance, sun_angular_radius_degrees, basis, tanfov,
                           4.0, 12.0, view)
        result = hdr.to_numpy()
        out[f"hdr_view{int(view)}"] = result if pixels is None else result[pixels[:, 0], pixels[:, 1]]
    t_composite = time.time() - t0
    shim.clear_restrictions()

    if pixels is None:
        out.update({k: v for k, v in gb.items()})
        out["surface_sun_transmittance"] = sun_t
        out["surface_sky_radiance"] = sky_l
    else:
        out.update({k: v for k, v in gb.items()})
        out["pixels"] = pixels.astype(np.int32)
        out["surface_sun_transmittance"] = sun_t[pixels[:, 0], pixels[:, 1]]
        out["surface_sky_radiance"] = sky_l[pixels[:, 0], pixels[:, 1]]

    meta = dict(
        name=name,
        config=dict(config_kwargs),
        planet_radius_m=planet_radius,
        camera_radius_m=camera_radius,
        camera_altitude_m=camera_altitude,
        sun_local=[float(v) for v in sun],
        solar_irradiance=list(solar_irradiance),
        sun_disk_radiance=list(lighting.sun_disk_radiance),
        sun_angular_radius_degrees=sun_angular_radius_degrees,
        view_basis=[[float(v) for v in b] for b in basis],
        tangent_half_fov=tanfov,
        star_contrast=[4.0, 12.0],
        width=width,
        height=height,
        views=[int(v) for v in views],
        seed=seed,
        sky_snapshot_altitude_m=renderer.sky_snapshot_altitude_m,
        sky_snapshot_sun_cosine=renderer.sky_snapshot_sun_cosine,
        rebuilds=[renderer.transmittance_rebuilds, renderer.multi_scattering_rebuilds,
                  renderer.sky_view_rebuilds, renderer.aerial_rebuilds],
        seconds=dict(update=t_update, prepare=t_prepare, composite=t_composite),
        generator="tests/golden/make_golden.py (reference kernels under taichi_f32_shim)",
    )
    out["meta"] = np.array(json.dumps(meta))
    print(f"[{name}] update {t_update:.1f}s prepare {t_prepare:.1f}s composite {t_composite:.1f}s", flush=True)
    return out, renderer


def _sample_pixels(width, height, rng, n_random, column_stride):
    pts = {(int(x), int(y)) for x, y in zip(rng.integers(0, width, n_random), rng.integers(0, height, n_random))}
    for y in range(0, height, column_stride):
        pts.add((width // 2, y))
        pts.add((width // 5, y))
    return sorted(pts)


def model_reference(reference: Path) -> dict:
    """Outputs of the reference's FP64 validation model (atmosphere/model.py):
    shell intervals, transmittance and direct single scattering for seeded
    rays on the Earth set and on the small planet of its own tests."""

    _import_reference(reference)
    from planet_renderer.atmosphere import AtmosphereConfig, AtmosphereModel  # type: ignore

    rng = np.random.default_rng(77)
    out = {}
    sets = {
        "earth": (6_360_000.0, AtmosphereConfig()),
        "small": (50_000.0, AtmosphereConfig(top_altitude_m=15_000.0, rayleigh_scale_height_m=3_000.0,
                                             mie_scale_height_m=800.0, absorption_peak_altitude_m=7_500.0,
                                             absorption_half_width_m=5_000.0)),
    }
    for tag, (radius, cfg) in sets.items():
        model = AtmosphereModel(radius, cfg)
        n = 24
        alt = np.concatenate([[1.0, 10.0, 2000.0], rng.uniform(0.0, 1.5 * cfg.top_altitude_m, n - 3)])
        origins = np.stack([np.zeros(n), radius + alt, np.zeros(n)], axis=1)
        dirs = rng.normal(size=(n, 3))
        dirs[:, 1] = np.where(np.arange(n) % 3 == 0, -np.abs(dirs[:, 1]) * 0.05, dirs[:, 1])
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        suns = rng.normal(size=(n, 3))
        suns /= np.linalg.norm(suns, axis=1, keepdims=True)
        trans, single, starts, ends, ground = [], [], [], [], []
        for o, d, s in zip(origins, dirs, suns):
            iv = model.atmosphere_interval(o, d)
            starts.append(np.nan if iv is None else iv.start_m)
            ends.append(np.nan if iv is None else iv.end_m)
            ground.append(False if iv is None else iv.ends_at_ground)
            trans.append(model.transmittance(o, d, steps=96, ground_is_opaque=True))
            single.append(model.single_scattering(o, d, s, (4.0, 3.9, 3.7), steps=10, sun_steps=10))
        out.update({f"{tag}_origins": origins, f"{tag}_dirs": dirs, f"{tag}_suns": suns,
                    f"{tag}_transmittance": np.array(trans), f"{tag}_single": np.array(single),
                    f"{tag}_start": np.array(starts), f"{tag}_end": np.array(ends),
                    f"{tag}_ground": np.array(ground)})
    out["meta"] = np.array(json.dumps({"name": "model_reference", "radii": {"earth": 6_360_000.0, "small": 50_000.0},
                                       "generator": "reference atmosphere/model.py"}))
    return out


def postprocess_reference(reference: Path) -> dict:
    """The reference's display post-process (src/planet_renderer/postprocess.py)
    run unmodified on seeded HDR images: odd and even sizes, bloom on and
    off, tone mapping on and off, 0-8 blur passes, thresholds and clamps that
    make the soft knee and the bright-pass cap matter."""

    shim.install()
    sys.path.insert(0, str(reference / "src"))
    from planet_renderer.postprocess import PostProcessor, PostprocessConfig  # type: ignore

    rng = np.random.default_rng(4242)
    cases = [
        # (width, height, config kwargs, exposure_ev, bloom, tone_map)
        (24, 16, {}, 0.0, True, True),
        (23, 15, {"bloom_passes": 1}, 1.5, True, True),
        (17, 9, {"bloom_threshold": 0.3, "bloom_knee": 0.2, "bloom_clamp": 2.0, "bloom_strength": 0.5,
                 "bloom_passes": 8}, -2.0, True, True),
        (24, 16, {}, 0.7, False, True),
        (23, 15, {}, 3.0, True, False),
        (9, 5, {"bloom_passes": 0}, 0.0, True, True),
        (1, 1, {"bloom_passes": 2}, 0.0, True, True),
        (16, 11, {"bloom_knee": 0.0, "bloom_strength": 0.25, "bloom_passes": 3}, -0.5, True, True),
        (31, 7, {}, -6.0, True, True),  # dark: the sRGB linear segment
    ]
    out = {}
    for k, (w, h, kw, ev, bloom, tone) in enumerate(cases):
        # linear HDR: log-normal radiance with a few very bright texels (a sun disk)
        hdr = np.exp(rng.normal(-1.0, 1.5, (w, h, 3))).astype(np.float32)
        for _ in range(max(1, w * h // 60)):
            hdr[rng.integers(0, w), rng.integers(0, h)] *= np.float32(rng.uniform(50.0, 5.0e4))
        cfg = PostprocessConfig(**kw)
        pp = PostProcessor(w, h, cfg)
        src = shim.Vector.field(3, dtype=shim.f32, shape=(w, h))
        src.from_numpy(hdr)
        display = shim.Vector.field(3, dtype=shim.f32, shape=(w, h))
        pp.process(src, display, ev, bloom=bloom, tone_map=tone)
        assert np.array_equal(src.to_numpy(), hdr)  # the HDR source is never modified
        out[f"case{k}_hdr"] = hdr
        out[f"case{k}_display"] = display.to_numpy()
        out[f"case{k}_args"] = np.array(json.dumps({"width": w, "height": h, "config": kw, "exposure_ev": ev,
                                                    "bloom": bloom, "tone_map": tone}))
    out["meta"] = np.array(json.dumps({"name": "postprocess", "cases": len(cases),
                                       "generator": "reference postprocess.py through taichi_f32_shim"}))
    return out


def shading_reference(reference: Path) -> dict:
    """The reference's surface shading (PlanetRenderer._shade_surface,
    src/planet_renderer/renderer.py:1277-1575), the consumer of
    prepare_frame's surface_sun_transmittance / surface_sky_radiance, run
    unmodified on seeded G-buffers with land, ocean and sky pixels: the
    Lambert path, the ocean BRDF with refracted seabed reconstruction from the
    terrain snapshot, the flat-ocean fallback and the albedo debug mode."""

    shim.install()
    sys.path.insert(0, str(reference / "src"))
    from planet_renderer.ocean import OCEAN_SURFACE_ID, OceanConfig  # type: ignore
    from planet_renderer.renderer import PlanetRenderer  # type: ignore

    from planet_renderer_gb300 import camera as cam

    ocean = OceanConfig()
    cases = [
        # (width, height, seed, advanced_ocean, mode, refraction strength, max offset px, yaw, pitch)
        (24, 16, 11, 1, 0, ocean.refraction_strength, ocean.refraction_max_offset_pixels, 10.0, -20.0),
        (17, 11, 12, 1, 0, 0.5, 0.3, -40.0, -35.0),  # offsets clamped to 0.3 px
        (24, 16, 13, 0, 0, ocean.refraction_strength, ocean.refraction_max_offset_pixels, 0.0, -10.0),
        (24, 16, 14, 1, 1, ocean.refraction_strength, ocean.refraction_max_offset_pixels, 0.0, -10.0),
        (20, 12, 15, 1, 0, 0.0, ocean.refraction_max_offset_pixels, 75.0, -60.0),
    ]
    out = {}
    for k, (w, h, seed, advanced, mode, strength, max_offset, yaw, pitch) in enumerate(cases):
        rng = np.random.default_rng(seed)
        f32 = np.float32

        def vec_field(values):
            fld = shim.Vector.field(values.shape[-1], dtype=shim.f32, shape=(w, h))
            fld.from_numpy(values.astype(f32))
            return fld

        def scalar_field(values, dtype):
            fld = shim.field(dtype=dtype, shape=(w, h))
            fld.from_numpy(values)
            return fld

        tanfov = cam.tangent_half_fov(60.0)
        basis = cam.view_basis(yaw, pitch)
        # view-space positions along the pixels' rays at 50 m - 3 km
        xs = (np.arange(w) + 0.5) / w * 2.0 - 1.0
        ys = (np.arange(h) + 0.5) / h * 2.0 - 1.0
        aspect = w / h
        rays = np.stack(np.broadcast_arrays(xs[:, None] * tanfov * aspect, ys[None, :] * tanfov,
                                            np.ones((w, h))), -1)
        depth = rng.uniform(50.0, 3000.0, (w, h))
        position = rays * depth[..., None]
        surface_id = np.where(rng.random((w, h)) < 0.5, OCEAN_SURFACE_ID, rng.integers(0, 1000, (w, h)))
        surface_id[:, -2:] = -1  # sky rows at the top
        surface_id = surface_id.astype(np.int32)
        up = np.array([0.0, 1.0, 0.0])
        normal = up + rng.normal(0.0, 0.25, (w, h, 3))
        albedo = rng.uniform(0.02, 0.5, (w, h, 3))
        water_depth = rng.uniform(0.0, 120.0, (w, h))
        seabed_albedo = rng.uniform(0.05, 0.4, (w, h, 3))
        seabed_normal = up + rng.normal(0.0, 0.3, (w, h, 3))
        slope_variance = rng.uniform(0.0, 0.05, (w, h))
        # opaque terrain snapshot: the seabed a little behind the water surface
        terrain_position = position + rays * rng.uniform(0.0, 40.0, (w, h))[..., None]
        terrain_id = np.where(rng.random((w, h)) < 0.85, rng.integers(0, 1000, (w, h)), -1).astype(np.int32)
        terrain_normal = up + rng.normal(0.0, 0.3, (w, h, 3))
        terrain_albedo = rng.uniform(0.05, 0.4, (w, h, 3))
        sun_t = rng.uniform(0.05, 1.0, (w, h, 3))
        sky_l = rng.uniform(0.001, 0.3, (w, h, 3))
        sun = np.array(cam.sun_from_zenith(float(rng.uniform(10.0, 85.0)), float(rng.uniform(0.0, 360.0))))

        renderer = PlanetRenderer.__new__(PlanetRenderer)  # fields only: the kernel reads nothing else
        renderer.width, renderer.height = w, h
        renderer.gbuffer_position = vec_field(position)
        renderer.gbuffer_normal = vec_field(normal)
        renderer.gbuffer_albedo = vec_field(albedo)
        renderer.gbuffer_water_depth_m = scalar_field(water_depth.astype(f32), shim.f32)
        renderer.gbuffer_seabed_albedo = vec_field(seabed_albedo)
        renderer.gbuffer_seabed_normal = vec_field(seabed_normal)
        renderer.gbuffer_ocean_slope_variance = scalar_field(slope_variance.astype(f32), shim.f32)
        renderer.gbuffer_surface_id = scalar_field(surface_id, shim.i32)
        renderer.terrain_position = vec_field(terrain_position)
        renderer.terrain_normal = vec_field(terrain_normal)
        renderer.terrain_albedo = vec_field(terrain_albedo)
        renderer.terrain_surface_id = scalar_field(terrain_id, shim.i32)
        renderer.surface_hdr = shim.Vector.field(3, dtype=shim.f32, shape=(w, h))
        sun_t_field, sky_field = vec_field(sun_t), vec_field(sky_l)
        args = dict(sun_global=tuple(float(v) for v in sun), solar_irradiance=(4.0, 3.9, 3.7),
                    view_right_global=tuple(float(v) for v in basis[0]),
                    view_up_global=tuple(float(v) for v in basis[1]),
                    view_forward_global=tuple(float(v) for v in basis[2]),
                    advanced_ocean_enabled=advanced, ocean_roughness=ocean.roughness, ocean_f0=ocean.dielectric_f0,
                    ocean_sky_strength=ocean.sky_reflection_strength,
                    ocean_absorption=tuple(ocean.absorption_per_m), ocean_scattering=tuple(ocean.scattering_per_m),
                    ocean_max_depth=ocean.max_visible_depth_m, ocean_refraction_index=ocean.refraction_index,
                    ocean_refraction_strength=float(strength), ocean_refraction_max_offset_pixels=float(max_offset),
                    sun_angular_radius=math.radians(0.266), tangent_half_fov=float(tanfov), mode=mode)
        renderer._shade_surface(args["sun_global"], args["solar_irradiance"], sun_t_field, sky_field,
                                *(args[n] for n in ("view_right_global", "view_up_global", "view_forward_global",
                                                   "advanced_ocean_enabled", "ocean_roughness", "ocean_f0",
                                                   "ocean_sky_strength", "ocean_absorption", "ocean_scattering",
                                                   "ocean_max_depth", "ocean_refraction_index",
                                                   "ocean_refraction_strength",
                                                   "ocean_refraction_max_offset_pixels", "sun_angular_radius",
                                                   "tangent_half_fov", "mode")))
        for name, fld in (("position", renderer.gbuffer_position), ("normal", renderer.gbuffer_normal),
                          ("albedo", renderer.gbuffer_albedo), ("water_depth", renderer.gbuffer_water_depth_m),
                          ("seabed_albedo", renderer.gbuffer_seabed_albedo),
                          ("seabed_normal", renderer.gbuffer_seabed_normal),
                          ("slope_variance", renderer.gbuffer_ocean_slope_variance),
                          ("surface_id", renderer.gbuffer_surface_id),
                          ("terrain_position", renderer.terrain_position),
                          ("terrain_normal", renderer.terrain_normal), ("terrain_albedo", renderer.terrain_albedo),
                          ("terrain_surface_id", renderer.terrain_surface_id),
                          ("sun_transmittance", sun_t_field), ("sky_radiance", sky_field),
                          ("surface_hdr", renderer.surface_hdr)):
            out[f"case{k}_{name}"] = fld.to_numpy()
        out[f"case{k}_args"] = np.array(json.dumps(args))
    out["meta"] = np.array(json.dumps({"name": "shading", "cases": len(cases), "ocean_surface_id": OCEAN_SURFACE_ID,
                                       "generator": "reference renderer.py _shade_surface through taichi_f32_shim"}))
    return out


RASTER_CASES = [
    # (width, height, patches, resolution, active slots, mode, tangent_half_fov, near, seed, skirt masks)
    (40, 24, 3, 4, (2, 0, 1), 0, 0.57735, 0.5, 21, (0b0101, 0, 0b1111)),
    (33, 19, 2, 3, (1, 0), 1, 0.45, 2.0, 22, (0, 0)),     # height-band view, narrower field of view
    (40, 24, 3, 4, (0, 2), 2, 0.57735, 0.5, 23, (0b0010, 0b1000, 0)),  # LOD-level hue view, one slot inactive
    (24, 24, 2, 5, (0, 1), 3, 0.8, 1.0, 24, (0b1111, 0b1111)),      # slot-hash view
]


# (width, height, seed, camera altitude m, pitch deg, yaw deg, time s, debug mode, OceanConfig overrides)
OCEAN_CASES = [
    (40, 24, 21, 30.0, -4.0, 20.0, 3.7, 0, dict(spectrum_resolution=32)),  # waves displace the near field
    (36, 20, 22, 5000.0, -2.0, -50.0, 11.0, 1, dict(spectrum_resolution=32)),  # reseeded grazing rays
    (32, 18, 23, 120.0, -8.0, 140.0, 0.0, 3, dict(enabled=False, spectrum_resolution=32)),  # flat sea level
    (30, 18, 24, 0.5, -1.0, 75.0, 42.5, 2, dict(spectrum_resolution=64, wind_direction_degrees=-120.0,
                                               choppiness=1.0, geometry_cascades=3, wind_speed_mps=14.0,
                                               wave_height_scale=1.6, normal_strength=0.8)),
]


def ocean_reference(reference: Path) -> dict:
    """The reference's ocean coverage pass (OceanRenderer.rasterize with
    _build_directional_spectrum and _rasterize, src/planet_renderer/ocean.py
    :193-771) run unmodified on seeded G-buffers holding terrain pixels in
    front of and behind the sea surface and sky: near-field wave geometry by
    fixed-point sphere solves, the reseeded outer sphere for a high camera's
    grazing rays, the flat sea level with the advanced path off, a camera
    below the crests, the debug colourings."""

    shim.install()
    sys.path.insert(0, str(reference / "src"))
    from planet_renderer.ocean import OCEAN_SURFACE_ID, OceanConfig, OceanRenderer  # type: ignore

    from planet_renderer_gb300 import camera as cam

    out = {}
    for k, (w, h, seed, altitude, pitch, yaw, time_s, mode, overrides) in enumerate(OCEAN_CASES):
        rng = np.random.default_rng(seed)
        f32 = np.float32
        config = OceanConfig(**overrides)
        ocean = OceanRenderer(w, h, config)
        tanfov = cam.tangent_half_fov(60.0)
        basis = cam.view_basis(yaw, pitch)
        # the camera's local frame in planet coordinates: a seeded rotation
        q = np.linalg.qr(rng.normal(size=(3, 3)))[0]
        frame = (q[:, 0], q[:, 1], np.cross(q[:, 0], q[:, 1]))
        xs = (np.arange(w) + 0.5) / w * 2.0 - 1.0
        ys = (np.arange(h) + 0.5) / h * 2.0 - 1.0
        rays = np.stack(np.broadcast_arrays(xs[:, None] * tanfov * w / h, ys[None, :] * tanfov,
                                            np.ones((w, h))), -1)
        depth = rng.uniform(1.0, 4.0, (w, h)) * np.exp(rng.uniform(0.0, 9.0, (w, h)))
        sid = np.where(rng.random((w, h)) < 0.6, rng.integers(0, 5000, (w, h)), -1).astype(np.int32)
        g = {
            "depth": depth.astype(f32),
            "position": (rays * depth[..., None]).astype(f32),
            "normal": (np.array([0.0, 1.0, 0.0]) + rng.normal(0.0, 0.3, (w, h, 3))).astype(f32),
            "albedo": rng.uniform(0.02, 0.6, (w, h, 3)).astype(f32),
            "material_weights": rng.dirichlet(np.ones(4), (w, h)).astype(f32),
            "height_m": rng.uniform(-200.0, 900.0, (w, h)).astype(f32),
            "water_depth": rng.uniform(0.0, 50.0, (w, h)).astype(f32),
            "seabed_albedo": rng.uniform(0.0, 0.3, (w, h, 3)).astype(f32),
            "seabed_normal": rng.normal(0.0, 1.0, (w, h, 3)).astype(f32),
            "slope_variance": rng.uniform(0.0, 0.1, (w, h)).astype(f32),
            "surface_id": sid,
            "cell_id": rng.integers(0, 1 << 20, (w, h)).astype(np.int32),
        }
        fields = {}
        for name, values in g.items():
            if values.ndim == 3:
                fld = shim.Vector.field(values.shape[-1], dtype=shim.f32, shape=(w, h))
            else:
                fld = shim.field(dtype=shim.i32 if values.dtype == np.int32 else shim.f32, shape=(w, h))
            fld.from_numpy(values)
            fields[name] = fld
        radius = 6_371_000.0
        ocean.rasterize(*(fields[n] for n in ("depth", "position", "normal", "albedo", "material_weights",
                                               "height_m", "water_depth", "seabed_albedo", "seabed_normal",
                                               "slope_variance", "surface_id", "cell_id")),
                        radius, altitude, frame, basis, tanfov, time_s, mode)
        pre = f"case{k}_"
        for name, values in g.items():
            out[pre + "in_" + name] = values
            out[pre + name] = fields[name].to_numpy()
        if config.enabled:
            out[pre + "spectrum_height"] = ocean.spectrum_height.to_numpy()
            out[pre + "spectrum_gradient"] = ocean.spectrum_gradient.to_numpy()
            out[pre + "spectrum_displacement"] = ocean.spectrum_displacement.to_numpy()
            out[pre + "spectrum_jacobian"] = ocean.spectrum_displacement_jacobian.to_numpy()
        out[pre + "args"] = np.array(json.dumps({
            "width": w, "height": h, "planet_radius_m": radius, "camera_altitude_m": altitude,
            "planet_frame": [list(map(float, v)) for v in frame], "view_basis": [list(map(float, v)) for v in basis],
            "tangent_half_fov": float(tanfov), "time_seconds": time_s, "debug_mode": mode, "config": overrides}))
    out["meta"] = np.array(json.dumps({"name": "ocean", "cases": len(OCEAN_CASES), "ocean_surface_id": OCEAN_SURFACE_ID,
                                       "generator": "reference ocean.py OceanRenderer.rasterize through "
                                                    "taichi_f32_shim"}))
    return out


RASTER_TOPOLOGIES = (2, 5, 12, 32)


def raster_mesh(w, h, patches, resolution, seed):
    """Seeded terrain patches in view space (x right, y up, z forward): a
    heightfield grid of (resolution + 1)^2 vertices per patch in front of
    and below the camera, wide enough to cross every frustum plane and the
    near plane; odd patches wound the other way (culled as back faces)."""

    rng = np.random.default_rng(seed)
    side = resolution + 1
    n_vert = side * side
    view = np.zeros((patches, n_vert, 3), np.float32)
    for p in range(patches):
        x0, z0 = rng.uniform(-90.0, -40.0), rng.uniform(-6.0, 4.0) + 20.0 * p
        span = rng.uniform(90.0, 140.0)
        for j in range(side):
            for i in range(side):
                x = x0 + span * i / resolution
                z = z0 + span * j / resolution
                y = -12.0 + 0.02 * z + rng.normal(0.0, 0.4)
                view[p, j * side + i] = (x, y, z)
    normal = np.zeros_like(view)
    normal[..., 1] = 1.0
    normal += rng.normal(0.0, 0.2, normal.shape).astype(np.float32)
    material = rng.dirichlet(np.ones(4), (patches, n_vert)).astype(np.float32)
    height = rng.uniform(-1500.0, 4500.0, (patches, n_vert)).astype(np.float32)
    cell = rng.integers(0, 10_000, (patches, n_vert)).astype(np.int32)
    tris = []
    for j in range(resolution):
        for i in range(resolution):
            a, b, c, d = j * side + i, j * side + i + 1, (j + 1) * side + i, (j + 1) * side + i + 1
            tris += [(a, b, c), (b, d, c)]
    # skirts: four edges of 2 * resolution triangles each, double-sided (here
    # the surface triangles re-wound, so that culled ones render as skirts)
    for k in range(8 * resolution):
        a, b, c = tris[k % len(tris)]
        tris.append((a, c, b))
    triangles = np.array(tris, np.int32)
    for p in range(1, patches, 2):  # a back-facing patch: swap the winding of its vertices' rows
        view[p] = view[p].reshape(side, side, 3)[:, ::-1].reshape(n_vert, 3)
    return view, normal, material, height, cell, triangles


def raster_reference(reference: Path) -> dict:
    """The reference's terrain raster (PlanetRenderer._clip, _emit,
    _raster_depth_direct, _resolve_raster, _surface_color;
    src/planet_renderer/renderer.py:628-1269) run unmodified on seeded view-space
    patches: triangles inside the frustum, crossing its side planes and the
    near plane (Sutherland-Hodgman), trivially rejected and back-facing ones,
    the atomic depth-key raster and the resolve into the G-buffer, in the lit
    albedo mode and the three debug colourings."""

    shim.install()
    sys.path.insert(0, str(reference / "src"))
    from planet_renderer.renderer import (DEPTH_KEY_SENTINEL, MAX_CLIPPED_TRIANGLES,  # type: ignore
                                          PlanetRenderer, _shared_topology)

    out = {}
    for n in RASTER_TOPOLOGIES:  # the patch topology the terrain backend's patches are drawn with
        out[f"topology{n}"] = np.asarray(_shared_topology(n), np.int32)
    for k, (w, h, patches, resolution, active, mode, tf, near, seed, skirts) in enumerate(RASTER_CASES):
        view, normal, material, height, cell, triangles = raster_mesh(w, h, patches, resolution, seed)
        n_vert = view.shape[1]
        r = PlanetRenderer.__new__(PlanetRenderer)  # fields only: the kernels read nothing else
        r.width, r.height = w, h
        r.resolution = resolution
        r.local_triangle_count = len(triangles)
        r.surface_triangle_count = 2 * resolution * resolution
        r.local_triangles = shim.Vector.field(3, dtype=shim.i32, shape=len(triangles))
        r.local_triangles.from_numpy(triangles)
        r.active_slot_ids = shim.field(dtype=shim.i32, shape=patches)
        r.active_slot_ids.from_numpy(np.array(list(active) + [0] * (patches - len(active)), np.int32))
        r.active_slot_count = shim.field(dtype=shim.i32, shape=())
        r.active_slot_count[None] = len(active)
        r.slot_skirt_mask = shim.field(dtype=shim.i32, shape=patches)
        r.slot_skirt_mask.from_numpy(np.array(skirts, np.int32))
        for name, values, n in (("view", view, 3), ("frame_normal", normal, 3), ("frame_material", material, 4)):
            fld = shim.Vector.field(n, dtype=shim.f32, shape=(patches, n_vert))
            fld.from_numpy(values)
            setattr(r, name, fld)
        r.frame_height_m = shim.field(dtype=shim.f32, shape=(patches, n_vert))
        r.frame_height_m.from_numpy(height)
        r.frame_cell = shim.field(dtype=shim.i32, shape=(patches, n_vert))
        r.frame_cell.from_numpy(cell)
        cap = patches * len(triangles) * MAX_CLIPPED_TRIANGLES
        r.raster_capacity = cap
        for name, n, dt in (("rv", 3, shim.f32), ("rn", 3, shim.f32), ("rm", 4, shim.f32), ("screen", 3, shim.f32),
                            ("edge_equation", 3, shim.f32)):
            setattr(r, name, shim.Vector.field(n, dtype=dt, shape=(cap, 3)))
        r.rh = shim.field(dtype=shim.f32, shape=(cap, 3))
        r.rc = shim.field(dtype=shim.i32, shape=(cap, 3))
        r.source = shim.field(dtype=shim.i32, shape=cap)
        r.inv_area = shim.field(dtype=shim.f32, shape=cap)
        r.edge_top_left = shim.Vector.field(3, dtype=shim.i32, shape=cap)
        r.clipped_count = shim.field(dtype=shim.i32, shape=())
        r.depth_key = shim.field(dtype=shim.u64, shape=(w, h))
        r.depth_key.fill(DEPTH_KEY_SENTINEL)
        r.depth = shim.field(dtype=shim.f32, shape=(w, h))
        for name, n in (("gbuffer_position", 3), ("gbuffer_normal", 3), ("gbuffer_albedo", 3),
                        ("gbuffer_material_weights", 4)):
            setattr(r, name, shim.Vector.field(n, dtype=shim.f32, shape=(w, h)))
        r.gbuffer_height_m = shim.field(dtype=shim.f32, shape=(w, h))
        r.gbuffer_surface_id = shim.field(dtype=shim.i32, shape=(w, h))
        r.gbuffer_surface_id.fill(-1)
        r.gbuffer_surface_cell_id = shim.field(dtype=shim.i32, shape=(w, h))
        r.gbuffer_surface_cell_id.fill(-1)
        slot_level = np.arange(patches, dtype=np.int32) * 3 + 1

        class _Terrain:  # the only TerrainRenderer field _surface_color reads (LOD-level view)
            pass

        r.terrain_renderer = _Terrain()
        r.terrain_renderer.slot_level = shim.field(dtype=shim.i32, shape=patches)
        r.terrain_renderer.slot_level.from_numpy(slot_level)
        r._clip(near, tf)
        r._raster_depth_direct(False)
        r._resolve_raster(mode, False)
        pre = f"case{k}_"
        for name, values in (("view", view), ("normal", normal), ("material", material), ("height", height),
                             ("cell", cell), ("triangles", triangles), ("slot_level", slot_level),
                             ("skirt_mask", np.array(skirts, np.int32))):
            out[pre + name] = values
        out[pre + "clipped_count"] = np.array(int(r.clipped_count[None]))
        for name, fld in (("depth", r.depth), ("position", r.gbuffer_position), ("gb_normal", r.gbuffer_normal),
                          ("albedo", r.gbuffer_albedo), ("material_weights", r.gbuffer_material_weights),
                          ("height_m", r.gbuffer_height_m), ("surface_id", r.gbuffer_surface_id),
                          ("cell_id", r.gbuffer_surface_cell_id)):
            out[pre + name] = fld.to_numpy()
        out[pre + "args"] = np.array(json.dumps({"width": w, "height": h, "patches": patches,
                                                 "resolution": resolution, "active": list(active), "mode": mode,
                                                 "tangent_half_fov": tf, "near": near, "seed": seed}))
    out["meta"] = np.array(json.dumps({"name": "raster", "cases": len(RASTER_CASES),
                                       "generator": "reference renderer.py _clip/_raster_depth_direct/_resolve_raster "
                                                    "through taichi_f32_shim"}))
    return out


def earth_config1_kwargs():
    return dict(
        mie_extinction_per_m=(3.996e-6 + 4.4e-6,) * 3,
        sky_view_lut_height=108,
        multi_scattering_directions=64,
        multi_scattering_steps=20,
        sky_view_steps=30,
        aerial_lut_height=32,
        aerial_horizon_raymarch_steps=48,
    )


def main() -> None:
    parser = argparse.ArgumentParser()
    parser.add_argument("--reference", type=Path, required=True,
                        help="root of the reference checkout (holds src/planet_renderer)")
    parser.add_argument("--only", nargs="*")
    parser.add_argument("--precision", choices=("f32", "f64"), default="f32",
                        help="f64 runs the same reference source in double (tiny scenarios only)")
    args = parser.parse_args()
    shim.set_precision(args.precision)
    suffix = "" if args.precision == "f32" else "_f64"
    wanted = set(args.only or [])

    def want(name):
        return not wanted or name in wanted

    if want("tiny_earth"):
        out, _ = run_scenario("tiny_earth", args.reference, TINY_LUTS, 6_360_000.0, 1000.0, 40.0, 25.0, 0.0, -30.0,
                              24, 16, seed=5)
        np.savez_compressed(HERE / f"tiny_earth{suffix}.npz", **out)
    if want("tiny_small_planet"):
        kwargs = dict(TINY_LUTS, top_altitude_m=15_000.0, rayleigh_scale_height_m=3_000.0, mie_scale_height_m=800.0,
                      absorption_peak_altitude_m=7_500.0, absorption_half_width_m=5_000.0)
        out, _ = run_scenario("tiny_small_planet", args.reference, kwargs, 50_000.0, 3000.0, 91.0, 30.0, 10.0, -10.0,
                              24, 16, seed=11)
        np.savez_compressed(HERE / f"tiny_small_planet{suffix}.npz", **out)
    if want("tiny_orbit"):
        out, _ = run_scenario("tiny_orbit", args.reference, dict(TINY_LUTS, aerial_horizon_raymarch_steps=16),
                              6_360_000.0, 2_000_000.0, 95.0, 60.0, 0.0, -35.0, 24, 16, seed=7)
        np.savez_compressed(HERE / f"tiny_orbit{suffix}.npz", **out)
    if want("model_reference") and args.precision == "f32":
        np.savez_compressed(HERE / "model_reference.npz", **model_reference(args.reference))
    if want("shading") and args.precision == "f32":
        np.savez_compressed(HERE / "shading.npz", **shading_reference(args.reference))
    if want("ocean") and args.precision == "f32":
        np.savez_compressed(HERE / "ocean.npz", **ocean_reference(args.reference))
    if want("raster") and args.precision == "f32":
        np.savez_compressed(HERE / "raster.npz", **raster_reference(args.reference))
    if want("postprocess") and args.precision == "f32":
        np.savez_compressed(HERE / "postprocess.npz", **postprocess_reference(args.reference))
    renderer = None
    if args.precision == "f64":
        return
    if want("earth_config1") or want("earth_cameras"):
        rng = np.random.default_rng(1234)
        pixels = _sample_pixels(1920, 1080, rng, 60, 60)
        out, renderer = run_scenario("earth_config1", args.reference, earth_config1_kwargs(), 6_360_000.0, 2000.0,
                                     45.0, 30.0, 0.0, -35.0, 1920, 1080, sample_pixels=pixels, seed=2027,
                                     views=[0, 1, 2, 6, 8])
        np.savez_compressed(HERE / "earth_config1.npz", **out)
    if want("earth_cameras"):
        for altitude, zenith, azimuth, tag in ((50_000.0, 88.0, 140.0, "50km"), (2_000_000.0, 95.0, 60.0, "2000km")):
            rng = np.random.default_rng(int(altitude))
            pixels = _sample_pixels(1920, 1080, rng, 60, 60)
            out, renderer = run_scenario(f"earth_camera_{tag}", args.reference, earth_config1_kwargs(), 6_360_000.0,
                                         altitude, zenith, azimuth, 0.0, -35.0, 1920, 1080, sample_pixels=pixels,
                                         seed=2027, reuse=renderer, views=[0, 2])
            # T and MS are unchanged from earth_config1 (same keys); keep the file small
            out.pop("transmittance_lut")
            out.pop("multi_scattering_lut")
            np.savez_compressed(HERE / f"earth_camera_{tag}.npz", **out)


if __name__ == "__main__":
    main()
