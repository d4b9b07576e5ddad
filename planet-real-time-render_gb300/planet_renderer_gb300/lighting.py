"""Host-side solar lighting state (reference ``lighting.py:11-55``).

``sun_disk_radiance`` is the uniform-disk radiance whose projected solid
angle integral equals the irradiance: ``L = E / (pi sin^2 alpha)``.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def _unit(value) -> np.ndarray:
    vector = np.asarray(value, dtype=np.float64)
    length = float(np.linalg.norm(vector))
    if vector.shape != (3,) or not np.isfinite(vector).all() or length <= 1.0e-12:
        raise ValueError("direction must be three finite values of non-zero length")
    return vector / length


@dataclass(frozen=True)
class LightingState:
    sun_direction_global: np.ndarray
    sun_angular_radius_degrees: float
    solar_irradiance: tuple[float, float, float]

    def __post_init__(self) -> None:
        object.__setattr__(self, "sun_direction_global", _unit(self.sun_direction_global))
        if not 0.01 <= self.sun_angular_radius_degrees <= 5.0:
            raise ValueError("sun angular radius must be in 0.01..5 degrees")
        if len(self.solar_irradiance) != 3 or not all(
            math.isfinite(v) and v >= 0.0 for v in self.solar_irradiance
        ):
            raise ValueError("solar irradiance must contain three finite values")

    @property
    def sun_solid_angle_sr(self) -> float:
        return 2.0 * math.pi * (1.0 - math.cos(math.radians(self.sun_angular_radius_degrees)))

    @property
    def sun_projected_solid_angle_sr(self) -> float:
        return math.pi * math.sin(math.radians(self.sun_angular_radius_degrees)) ** 2

    @property
    def sun_disk_radiance(self) -> tuple[float, float, float]:
        omega = self.sun_projected_solid_angle_sr
        return tuple(v / omega for v in self.solar_irradiance)  # type: ignore[return-value]
