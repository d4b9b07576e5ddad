"""Configuration contract of one spherical atmosphere.

Same fields, defaults, validation and JSON mapping as the reference's
``AtmosphereConfig`` (``src/planet_renderer/atmosphere/config.py:29-259``), so
a caller's existing config objects and JSON ``atmosphere`` blocks work
unchanged.  Lengths are metres, coefficients 1/m.  The planet radius is not
part of the config; it is passed per call, as in the reference.
"""

from __future__ import annotations

import math
from dataclasses import asdict, dataclass, fields
from typing import Mapping

Rgb = tuple[float, float, float]

# (field, low, high, message) integer ranges checked by the reference
# (atmosphere/config.py:97-128).
_INT_RANGES = (
    ("transmittance_lut_width", 16, 2048, "transmittance LUT width must be in 16..2048"),
    ("transmittance_lut_height", 16, 1024, "transmittance LUT height must be in 16..1024"),
    ("sky_view_lut_width", 16, 2048, "sky-view LUT width must be in 16..2048"),
    ("sky_view_lut_height", 16, 2048, "sky-view LUT height must be in 16..2048"),
    ("multi_scattering_lut_width", 8, 256, "multi-scattering LUT width must be in 8..256"),
    ("multi_scattering_lut_height", 8, 256, "multi-scattering LUT height must be in 8..256"),
    ("aerial_lut_width", 4, 256, "aerial LUT width must be in 4..256"),
    ("aerial_lut_height", 4, 256, "aerial LUT height must be in 4..256"),
    ("aerial_lut_depth", 8, 256, "aerial LUT depth must be in 8..256"),
    ("transmittance_steps", 4, 256, "transmittance_steps must be in 4..256"),
    ("multi_scattering_directions", 4, 128, "multi_scattering_directions must be in 4..128"),
    ("multi_scattering_steps", 4, 128, "multi_scattering_steps must be in 4..128"),
    ("sky_view_steps", 4, 256, "sky_view_steps must be in 4..256"),
    ("aerial_steps_per_slice", 1, 16, "aerial_steps_per_slice must be in 1..16"),
    ("aerial_horizon_raymarch_steps", 4, 64, "aerial_horizon_raymarch_steps must be in 4..64"),
    ("aerial_terminator_substeps", 2, 16, "aerial_terminator_substeps must be in 2..16"),
)

_RGB_FIELDS = (
    "rayleigh_scattering_per_m",
    "mie_scattering_per_m",
    "mie_extinction_per_m",
    "absorption_extinction_per_m",
    "ground_albedo",
)

_POSITIVE_FIELDS = (
    "top_altitude_m",
    "rayleigh_scale_height_m",
    "mie_scale_height_m",
    "absorption_half_width_m",
)


def _rgb(value: object, name: str, default: Rgb) -> Rgb:
    source = default if value is None else value
    if not isinstance(source, (list, tuple)) or len(source) != 3:
        raise ValueError(f"atmosphere.{name} must contain three values")
    result = tuple(float(component) for component in source)
    if not all(math.isfinite(c) and c >= 0.0 for c in result):
        raise ValueError(f"atmosphere.{name} must be finite and non-negative")
    return result  # type: ignore[return-value]


@dataclass(frozen=True)
class AtmosphereConfig:
    """Optical parameters and LUT quality for one spherical atmosphere."""

    top_altitude_m: float = 100_000.0
    rayleigh_scattering_per_m: Rgb = (5.802e-6, 13.558e-6, 33.100e-6)
    rayleigh_scale_height_m: float = 8_000.0
    mie_scattering_per_m: Rgb = (3.996e-6, 3.996e-6, 3.996e-6)
    mie_extinction_per_m: Rgb = (4.440e-6, 4.440e-6, 4.440e-6)
    mie_scale_height_m: float = 1_200.0
    mie_phase_g: float = 0.80
    absorption_extinction_per_m: Rgb = (0.650e-6, 1.881e-6, 0.085e-6)
    absorption_peak_altitude_m: float = 25_000.0
    absorption_half_width_m: float = 15_000.0
    ground_albedo: Rgb = (0.10, 0.10, 0.10)
    transmittance_lut_width: int = 256
    transmittance_lut_height: int = 64
    multi_scattering_lut_width: int = 32
    multi_scattering_lut_height: int = 32
    sky_view_lut_width: int = 192
    sky_view_lut_height: int = 256
    aerial_lut_width: int = 32
    aerial_lut_height: int = 18
    aerial_lut_depth: int = 32
    transmittance_steps: int = 40
    multi_scattering_directions: int = 16
    multi_scattering_steps: int = 12
    sky_view_steps: int = 24
    aerial_steps_per_slice: int = 2
    aerial_horizon_raymarch_steps: int = 12
    aerial_terminator_substeps: int = 8

    def __post_init__(self) -> None:
        for name in _RGB_FIELDS:
            values = getattr(self, name)
            if len(values) != 3 or not all(
                math.isfinite(v) and v >= 0.0 for v in values
            ):
                raise ValueError(
                    f"atmosphere.{name} must contain three non-negative values"
                )
        if any(v > 1.0 for v in self.ground_albedo):
            raise ValueError("atmosphere.ground_albedo must remain in [0, 1]")
        for name in _POSITIVE_FIELDS:
            value = getattr(self, name)
            if not math.isfinite(value) or value <= 0.0:
                raise ValueError(f"atmosphere.{name} must be positive and finite")
        if not 0.0 <= self.absorption_peak_altitude_m <= self.top_altitude_m:
            raise ValueError("atmosphere absorption peak must lie inside the shell")
        if not -0.99 < self.mie_phase_g < 0.99:
            raise ValueError("atmosphere.mie_phase_g must be in (-0.99, 0.99)")
        if any(
            s > e for s, e in zip(self.mie_scattering_per_m, self.mie_extinction_per_m)
        ):
            raise ValueError("Mie scattering cannot exceed Mie extinction")
        for name, low, high, message in _INT_RANGES:
            if not low <= getattr(self, name) <= high:
                raise ValueError(message)

    @classmethod
    def from_mapping(cls, values: Mapping[str, object]) -> "AtmosphereConfig":
        """Build from a JSON ``atmosphere`` block; missing keys take defaults."""

        defaults = cls()
        kwargs: dict[str, object] = {}
        for f in fields(cls):
            if f.name in _RGB_FIELDS:
                kwargs[f.name] = _rgb(values.get(f.name), f.name, getattr(defaults, f.name))
            elif isinstance(getattr(defaults, f.name), int):
                kwargs[f.name] = int(values.get(f.name, getattr(defaults, f.name)))
            else:
                kwargs[f.name] = float(values.get(f.name, getattr(defaults, f.name)))
        return cls(**kwargs)  # type: ignore[arg-type]

    def to_mapping(self) -> dict[str, object]:
        out = asdict(self)
        for name in _RGB_FIELDS:
            out[name] = list(out[name])
        return out


# Named parameter sets of the workloads this package is measured on.
def earth_baseline() -> AtmosphereConfig:
    """Earth-like set with LUT sizes and step counts of the plain LUT-build
    workload: Mie extinction = scattering 3.996e-6 + absorption 4.4e-6
    (the reference's earth.json uses 4.44e-6 instead); Sky-view 192x108 with 30
    steps; Multi-scattering 64 directions x 20 steps; AP 32x32x32; 48 limb
    intervals and 8 terminator substeps as in earth.json."""

    return AtmosphereConfig(
        mie_extinction_per_m=(3.996e-6 + 4.4e-6,) * 3,
        sky_view_lut_width=192,
        sky_view_lut_height=108,
        multi_scattering_directions=64,
        multi_scattering_steps=20,
        sky_view_steps=30,
        aerial_lut_width=32,
        aerial_lut_height=32,
        aerial_lut_depth=32,
        aerial_horizon_raymarch_steps=48,
        aerial_terminator_substeps=8,
    )


def earth_reference() -> AtmosphereConfig:
    """The reference's configs/earth.json atmosphere block."""

    return AtmosphereConfig(
        sky_view_lut_width=192,
        sky_view_lut_height=256,
        aerial_lut_width=96,
        aerial_lut_height=54,
        aerial_lut_depth=64,
        aerial_horizon_raymarch_steps=48,
    )


def small_planet() -> AtmosphereConfig:
    """Stylised small planet (R = 50 km): top 60 km, Rayleigh H 1.5 km,
    Mie H 0.3 km, the Earth set's coefficients and ozone tent (25 km +/-
    15 km, inside the 60 km shell, so the reference validation accepts it)."""

    return AtmosphereConfig(
        top_altitude_m=60_000.0,
        rayleigh_scale_height_m=1_500.0,
        mie_scale_height_m=300.0,
        mie_extinction_per_m=(3.996e-6 + 4.4e-6,) * 3,
        sky_view_lut_height=108,
        multi_scattering_directions=64,
        multi_scattering_steps=20,
        sky_view_steps=30,
        aerial_lut_height=32,
        aerial_horizon_raymarch_steps=48,
    )


SMALL_PLANET_RADIUS_M = 50_000.0
EARTH_RADIUS_M = 6_360_000.0
