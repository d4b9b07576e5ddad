"""Single-LUT kernels with the camera 3 m above the ground, against the
float64 oracle with the reference's own float32 deviation allowed (the
reference's float32 segment weight cancels there; see
test_weight_conditioning.py)."""

from __future__ import annotations

import pytest

from conftest import assert_exact_parity
from near_ground import CAMERA_ALTITUDE_M, SUN_LOCAL, TAN_HALF_FOV, VIEW_BASIS, FRAME, oracle_aerial, setting

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("param_set", [0, 1])
def test_gpu_aerial_next_to_the_ground(param_set):
    from oracle.atm import Oracle
    from planet_renderer_gb300.atmosphere import AtmosphereRenderer

    cfg, radius = setting(param_set)
    r = AtmosphereRenderer(FRAME[0], FRAME[1], cfg)
    r.build_lut("transmittance", planet_radius_m=radius)
    r.build_lut("multi_scattering", planet_radius_m=radius)
    r.build_lut("aerial", planet_radius_m=radius, camera_altitude_m=CAMERA_ALTITUDE_M, sun_local=SUN_LOCAL,
                view_basis=VIEW_BASIS, tangent_half_fov=TAN_HALF_FOV)
    got = r.aerial_scattering_lut.to_torch().cpu().numpy()
    r.close()
    rep = assert_exact_parity(got, oracle_aerial(Oracle("f32"), cfg, radius), oracle_aerial(Oracle("f64"), cfg, radius),
                              f"aerial, set {param_set}")
    # the kernels' series weight tracks float64 closely, not just within the allowance
    assert rep["max_rel_vs_exact"] < 1e-3, rep
