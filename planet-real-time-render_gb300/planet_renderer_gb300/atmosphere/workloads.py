"""Named workloads of the atmosphere path (the frames the bench and the
parity tests run).

``frame_chain_cameras``: the full plain per-frame chain at 1920x1080 - three
cameras at 2 km, 50 km and 2000 km altitude, pitch -35 deg, vertical FOV
60 deg, sun zenith uniform in [0, 100] deg.  The three zeniths are drawn from
the three thirds of that range (stratified, seeded, randomly assigned to the
cameras) so every run holds a daylight, a low-sun and a twilight view;
azimuths are uniform in [0, 360).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .. import camera

EARTH_RADIUS_M = 6_360_000.0
SOLAR_IRRADIANCE = (4.0, 3.9, 3.7)  # configs/earth.json lighting block
SUN_ANGULAR_RADIUS_DEG = 0.266
STAR_CONTRAST = (4.0, 12.0)
VERTICAL_FOV_DEG = 60.0
PITCH_DEG = -35.0


@dataclass(frozen=True)
class CameraView:
    altitude_m: float
    sun_zenith_deg: float
    sun_azimuth_deg: float
    yaw_deg: float = 0.0
    pitch_deg: float = PITCH_DEG

    @property
    def camera_radius_m(self) -> float:
        return EARTH_RADIUS_M + self.altitude_m

    @property
    def basis(self):
        return camera.view_basis(self.yaw_deg, self.pitch_deg)

    @property
    def sun_local(self) -> np.ndarray:
        return camera.sun_from_zenith(self.sun_zenith_deg, self.sun_azimuth_deg)

    @property
    def tangent_half_fov(self) -> float:
        return camera.tangent_half_fov(VERTICAL_FOV_DEG)


def frame_chain_cameras(seed: int = 2027) -> list[CameraView]:
    rng = np.random.default_rng(seed)
    strata = rng.permutation(3)
    views = []
    for altitude, stratum in zip((2_000.0, 50_000.0, 2_000_000.0), strata):
        zenith = float((stratum + rng.uniform()) * 100.0 / 3.0)
        azimuth = float(rng.uniform(0.0, 360.0))
        views.append(CameraView(altitude, zenith, azimuth))
    return views
