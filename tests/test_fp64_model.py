"""FP64 model: the reference's known answers and its validation model.

* Known answers of the reference's own tests, restated:
  tests/test_m3_atmosphere.py:24-99 (ray-sphere roots, shell interval and
  opaque ground, density and transmittance ranges, single scattering) and
  tests/test_m0_geometry.py:87-107 (disk radiance integrates to irradiance).
* The numpy FP64 model agrees with the reference's atmosphere/model.py outputs
  (tests/golden/model_reference.npz) to 1e-12.
* The FP32 transmittance LUT's quadrature error against a 4096-step FP64
  quadrature of the same rays is stated and bounded.
"""

from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import load_golden


def _small_model():
    from oracle.atm_fp64 import AtmosphereModelFP64
    from planet_renderer_gb300.atmosphere.config import AtmosphereConfig

    return AtmosphereModelFP64(50_000.0, AtmosphereConfig(top_altitude_m=15_000.0, rayleigh_scale_height_m=3_000.0,
                                                          mie_scale_height_m=800.0, absorption_peak_altitude_m=7_500.0,
                                                          absorption_half_width_m=5_000.0))


def test_ray_sphere_roots_from_outside_and_inside():
    from oracle.atm_fp64 import ray_sphere_roots

    outside = ray_sphere_roots(np.array([0.0, 70_000.0, 0.0]), np.array([0.0, -1.0, 0.0]), 65_000.0)
    np.testing.assert_allclose(outside, (5_000.0, 135_000.0), atol=1e-8)
    inside = ray_sphere_roots(np.array([0.0, 55_000.0, 0.0]), np.array([0.0, 1.0, 0.0]), 65_000.0)
    np.testing.assert_allclose(inside, (-120_000.0, 10_000.0), atol=1e-8)


def test_shell_interval_stops_at_opaque_ground():
    model = _small_model()
    down = model.atmosphere_interval(np.array([0.0, 51_000.0, 0.0]), np.array([0.0, -1.0, 0.0]))
    assert down is not None and down.ends_at_ground
    assert math.isclose(down.end_m, 1_000.0, abs_tol=1e-8)
    up = model.atmosphere_interval(np.array([0.0, 50_000.0, 0.0]), np.array([0.0, 1.0, 0.0]))
    assert up is not None and not up.ends_at_ground
    assert math.isclose(up.end_m, 15_000.0, abs_tol=1e-8)


def test_density_and_transmittance_ranges():
    model = _small_model()
    sea = [float(v) for v in model.density(0.0)]
    high = [float(v) for v in model.density(12_000.0)]
    assert sea[0] > high[0] >= 0.0 and sea[1] > high[1] >= 0.0
    origin = np.array([0.0, 50_001.0, 0.0])
    t = model.transmittance(origin, np.array([0.0, 1.0, 0.0]), steps=64)
    assert np.isfinite(t).all() and np.all((0.0 <= t) & (t <= 1.0)) and t[2] < t[0]
    blocked = model.transmittance(origin, np.array([0.0, -1.0, 0.0]), steps=16, ground_is_opaque=True)
    np.testing.assert_array_equal(blocked, np.zeros(3))


def test_single_scattering_is_finite_and_non_negative():
    model = _small_model()
    L = model.single_scattering(np.array([0.0, 50_010.0, 0.0]), np.array([0.0, 0.2, 1.0]),
                                np.array([0.0, 0.7, 0.7]), (4.0, 3.9, 3.7), steps=12, sun_steps=12)
    assert np.isfinite(L).all() and np.all(L >= 0.0) and float(L.max()) > 0.0


def test_solar_disk_radiance_integrates_to_irradiance():
    from planet_renderer_gb300.lighting import LightingState

    state = LightingState(np.array([0.0, 1.0, 0.0]), 0.266, (4.0, 3.9, 3.7))
    integrated = np.asarray(state.sun_disk_radiance) * state.sun_projected_solid_angle_sr
    np.testing.assert_allclose(integrated, state.solar_irradiance, rtol=1e-12)
    smaller = LightingState(np.array([0.0, 1.0, 0.0]), 0.133, state.solar_irradiance)
    assert smaller.sun_disk_radiance[0] > state.sun_disk_radiance[0]
    with pytest.raises(ValueError):
        LightingState(np.array([0.0, 1.0, 0.0]), 9.0, (1.0, 1.0, 1.0))


def test_fp64_model_matches_reference_model():
    from oracle.atm_fp64 import AtmosphereModelFP64
    from planet_renderer_gb300.atmosphere.config import AtmosphereConfig

    data, meta = load_golden("model_reference")
    configs = {
        "earth": AtmosphereConfig(),
        "small": AtmosphereConfig(top_altitude_m=15_000.0, rayleigh_scale_height_m=3_000.0, mie_scale_height_m=800.0,
                                  absorption_peak_altitude_m=7_500.0, absorption_half_width_m=5_000.0),
    }
    for tag, cfg in configs.items():
        model = AtmosphereModelFP64(meta["radii"][tag], cfg)
        for k, (o, d, s) in enumerate(zip(data[f"{tag}_origins"], data[f"{tag}_dirs"], data[f"{tag}_suns"])):
            iv = model.atmosphere_interval(o, d)
            if np.isnan(data[f"{tag}_start"][k]):
                assert iv is None
            else:
                assert iv is not None
                np.testing.assert_allclose([iv.start_m, iv.end_m], [data[f"{tag}_start"][k], data[f"{tag}_end"][k]],
                                           rtol=1e-12, atol=1e-6)
                assert iv.ends_at_ground == bool(data[f"{tag}_ground"][k])
            np.testing.assert_allclose(model.transmittance(o, d, steps=96, ground_is_opaque=True),
                                       data[f"{tag}_transmittance"][k], rtol=1e-12, atol=1e-300)
            np.testing.assert_allclose(model.single_scattering(o, d, s, (4.0, 3.9, 3.7), steps=10, sun_steps=10),
                                       data[f"{tag}_single"][k], rtol=1e-10, atol=1e-300)


def test_transmittance_lut_quadrature_error_is_stated(oracle_f32, oracle_f64):
    """40 warped steps (the reference's quadrature) vs 4096 uniform FP64 steps
    on every texel ray of the Earth transmittance LUT."""

    from oracle.atm_fp64 import AtmosphereModelFP64
    from planet_renderer_gb300.atmosphere.config import earth_baseline

    cfg = earth_baseline()
    R = 6_360_000.0
    converged = AtmosphereModelFP64(R, cfg).transmittance_lut_converged(cfg.transmittance_lut_width,
                                                                        cfg.transmittance_lut_height)
    lut64 = oracle_f64.build_transmittance(cfg, R)
    lut32 = oracle_f32.build_transmittance(cfg, R)
    mask = converged > 1e-6  # texels carrying visible light
    err64 = np.abs(lut64 - converged)[mask] / converged[mask]
    err32 = np.abs(lut32 - converged)[mask] / converged[mask]
    # the 40-step warped quadrature itself; f32 adds little on top
    assert np.median(err64) < 2e-3
    assert np.percentile(err64, 99) < 5e-2
    assert np.percentile(err32, 99) < np.percentile(err64, 99) + 1e-3
