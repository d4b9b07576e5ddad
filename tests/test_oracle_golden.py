"""Pin the CPU oracle to the reference.

The golden vectors were produced by the reference's own kernel source
(``atmosphere/renderer.py``) driven through its public methods
(tests/golden/make_golden.py).  Two checks:

* float64: the reference source run in double and the oracle's FP64 instance
  agree to 1e-9 relative on every LUT, surface field and diagnostic view -
  the oracle is the reference's algorithm, operation for operation;
* float32: the oracle's FP32 instance agrees with the reference run in
  float32 within the parity criterion (1e-3 relative per channel plus 1e-5
  of the channel peak for rounding noise far below the peak).
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_parity, load_golden, parity_report
from scenario import Scenario, oracle_stages, oracle_stages_with_luts

TINY = ["tiny_earth", "tiny_small_planet", "tiny_orbit"]


def _compare(out: dict, data, what: str, rtol=1e-3, atol_frac=1e-5):
    reports = {}
    for key, got in out.items():
        reports[key] = assert_parity(got, data[key], f"{what}:{key}", rtol=rtol, atol_frac=atol_frac)
    return reports


@pytest.mark.parametrize("name", TINY)
def test_oracle_f64_is_the_reference_algorithm(name, oracle_f64):
    data, meta = load_golden(name + "_f64")
    sc = Scenario(data, meta)
    out = oracle_stages(sc, oracle_f64)
    assert set(out) >= {"transmittance_lut", "multi_scattering_lut", "sky_view_lut", "aerial_scattering_lut"}
    assert len([k for k in out if k.startswith("hdr_view")]) == 11
    _compare(out, data, name, rtol=1e-9, atol_frac=1e-12)


@pytest.mark.parametrize("name", TINY)
def test_oracle_f32_matches_reference_f32(name, oracle_f32):
    data, meta = load_golden(name)
    _compare(oracle_stages(Scenario(data, meta), oracle_f32), data, name)


def test_oracle_chain_matches_reference_host_logic(oracle_f32):
    """update/prepare_frame/composite of the oracle's host restatement
    reproduce the reference outputs and rebuild counters."""

    from oracle.atm import OracleAtmosphere

    data, meta = load_golden("tiny_earth")
    sc = Scenario(data, meta)
    o = OracleAtmosphere(sc.W, sc.H, sc.config)
    o.update(sc.R, sc.cr, sc.sun.copy(), sc.E, sc.ar_deg)
    f = sc.frame
    o.prepare_frame(f["position_view"], f["surface_id"], sc.R, sc.cr, sc.sun, sc.E, sc.ar_deg, sc.basis, sc.tanfov)
    for key in ("transmittance_lut", "multi_scattering_lut", "sky_view_lut", "aerial_scattering_lut"):
        assert_parity(getattr(o, key), data[key], key)
    hdr, samples = o.composite(f["scene_hdr"], f["space_hdr"], f["surface_id"], f["position_view"], sc.R, sc.cr,
                               sc.sun, sc.E, sc.disk, sc.ar_deg, sc.basis, sc.tanfov, 4.0, 12.0, 0)
    assert_parity(hdr, data["hdr_view0"], "composite")
    assert samples > 0
    assert [o.transmittance_rebuilds, o.multi_scattering_rebuilds, o.sky_view_rebuilds,
            o.aerial_rebuilds] == meta["rebuilds"]
    assert o.sky_snapshot_altitude_m == meta["sky_snapshot_altitude_m"]
    assert o.sky_snapshot_sun_cosine == meta["sky_snapshot_sun_cosine"]


@pytest.mark.parametrize("name", ["earth_config1"])
def test_oracle_f32_full_size_earth(name, oracle_f32):
    data, meta = load_golden(name)
    _compare(oracle_stages(Scenario(data, meta), oracle_f32), data, name)


@pytest.mark.parametrize("name", ["earth_camera_50km", "earth_camera_2000km"])
def test_oracle_f32_cameras(name, oracle_f32):
    base, _ = load_golden("earth_config1")
    data, meta = load_golden(name)
    out = oracle_stages_with_luts(Scenario(data, meta), oracle_f32, base["transmittance_lut"],
                                  base["multi_scattering_lut"])
    _compare(out, data, name)


def test_parity_criterion_rejects_a_planted_error(oracle_f32):
    """A 0.2% error planted in one oracle texel must fail the criterion."""

    data, meta = load_golden("tiny_earth")
    sc = Scenario(data, meta)
    lut = oracle_f32.build_transmittance(sc.config, sc.R)
    lut[3, 5, 1] *= 1.002
    assert parity_report(lut, data["transmittance_lut"])["max_excess"] > 1.0
