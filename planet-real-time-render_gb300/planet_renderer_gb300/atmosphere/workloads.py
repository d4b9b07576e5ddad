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


def surrogate_sweep_cameras(seed: int = 2027, frames: int = 64) -> list[CameraView]:
    """Cameras of the aerial-surrogate frame workload: altitude log-uniform
    1 m - 4000 km, sun zenith uniform 0-100 deg, sun azimuth uniform, the
    frame chain's pitch and field of view.  Seeded."""

    rng = np.random.default_rng(seed)
    altitude = np.exp(rng.uniform(np.log(1.0), np.log(4.0e6), frames))
    zenith = rng.uniform(0.0, 100.0, frames)
    azimuth = rng.uniform(0.0, 360.0, frames)
    return [CameraView(float(a), float(z), float(b)) for a, z, b in zip(altitude, zenith, azimuth)]


# ---- batched LUT builds ----------------------------------------------------
SKY_VIEW_SIZES = ((96, 54), (128, 72), (192, 108), (256, 144), (384, 216))
AERIAL_SIDES = (16, 24, 32, 48, 64)


def batched_lut_sets():
    """(config, planet radius) of the two parameter sets of the batch."""

    from .config import EARTH_RADIUS_M as R_EARTH, SMALL_PLANET_RADIUS_M, earth_baseline, small_planet

    return [(earth_baseline(), R_EARTH), (small_planet(), SMALL_PLANET_RADIUS_M)]


def batched_lut_jobs(seed: int = 2027, snapshots: int = 256, cameras: int = 16):
    """Jobs of the batched LUT-build workload: ``snapshots`` time snapshots
    (sun zenith uniform 0-110 deg, azimuth uniform 0-360 deg) x ``cameras``
    cameras (altitude log-uniform 1 m - 4000 km, yaw uniform, pitch uniform
    -45..10 deg) x both parameter sets; each (snapshot, camera, set) gets a
    sky-view LUT (96x54 .. 384x216) and an aerial volume (16^3 .. 64^3) with
    sizes drawn uniformly from those ladders.  Seeded."""

    from .batch import AERIAL, SKY_VIEW, BatchJob

    rng = np.random.default_rng(seed)
    zen = rng.uniform(0.0, 110.0, snapshots)
    azi = rng.uniform(0.0, 360.0, snapshots)
    alt = np.exp(rng.uniform(np.log(1.0), np.log(4.0e6), cameras))
    yaw = rng.uniform(0.0, 360.0, cameras)
    pitch = rng.uniform(-45.0, 10.0, cameras)
    tanfov = camera.tangent_half_fov(VERTICAL_FOV_DEG)
    bases = [camera.view_basis(float(y), float(p)) for y, p in zip(yaw, pitch)]
    jobs = []
    for s in range(snapshots):
        sun = camera.sun_from_zenith(float(zen[s]), float(azi[s]))
        sun_cos = float(np.float32(np.clip(sun[1], -1.0, 1.0)))
        for c in range(cameras):
            basis = tuple(tuple(float(v) for v in b) for b in bases[c])
            for param_set in (0, 1):
                sw, sh = SKY_VIEW_SIZES[rng.integers(len(SKY_VIEW_SIZES))]
                side = AERIAL_SIDES[rng.integers(len(AERIAL_SIDES))]
                jobs.append(BatchJob(SKY_VIEW, param_set, sw, sh, 1, camera_altitude_m=float(alt[c]),
                                     sun_zenith_cosine=sun_cos))
                jobs.append(BatchJob(AERIAL, param_set, side, side, side, camera_altitude_m=float(alt[c]),
                                     sun_local=tuple(float(v) for v in sun), view_basis=basis,
                                     tangent_half_fov=tanfov))
    return jobs
