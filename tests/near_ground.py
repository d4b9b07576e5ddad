"""A camera standing on the ground: the geometry where the reference's float32
segment weight (1 - exp(-x)) / ext cancels.  Shared by the CPU test of that
cancellation and the GPU tests that compare against the float64 oracle."""

from __future__ import annotations

import dataclasses
import math

import numpy as np

E = (4.0, 3.9, 3.7)
SUN_ANGULAR_RADIUS_DEG = 0.266
CAMERA_ALTITUDE_M = 2.916895486054149
SUN_LOCAL = (0.04380585497325674, 0.9696900953977097, 0.24037921282349434)
VIEW_BASIS = ((-0.6799216978786049, 0.0, -0.7332847228422771),
              (0.3650675345397183, 0.8672617950955044, -0.3385006262812744),
              (0.6359498250483027, -0.49785236643780595, -0.589670112226582))
TAN_HALF_FOV = math.tan(math.radians(30.0))
FRAME = (1920, 1080)
SIDE = 24


def setting(param_set: int):
    """(config with a SIDE^3 aerial volume, planet radius) of parameter set
    0 (Earth) or 1 (the 50 km planet)."""

    from planet_renderer_gb300.atmosphere.workloads import batched_lut_sets

    cfg, radius = batched_lut_sets()[param_set]
    return dataclasses.replace(cfg, aerial_lut_width=SIDE, aerial_lut_height=SIDE, aerial_lut_depth=SIDE), radius


def oracle_aerial(oracle, cfg, radius) -> np.ndarray:
    f32 = oracle.precision == "f32"
    ar = math.radians(SUN_ANGULAR_RADIUS_DEG)
    tl = oracle.build_transmittance(cfg, radius)
    ms = oracle.build_multi_scattering(cfg, radius, E, float(np.float32(ar)) if f32 else ar, tl)
    return oracle.build_aerial(cfg, FRAME[0], FRAME[1], radius, CAMERA_ALTITUDE_M, SUN_LOCAL, E, ar, VIEW_BASIS,
                               TAN_HALF_FOV, tl, ms)
