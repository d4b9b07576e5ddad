"""Drop-in ocean coverage: ``OceanConfig`` and ``OceanRenderer`` with the
reference's fields, validation and ``rasterize`` call
(``src/planet_renderer/ocean.py:38-771``), backed by the sm_103a kernels of
libplanet_atm (``atm_ocean_*`` in the C ABI).

``rasterize`` runs after the terrain raster: per frame it builds the
three-cascade directional wave spectrum, then intersects every pixel's view
ray with the sea-level sphere (near-field crests by fixed-point sphere
solves) and, where the sea is nearer than the terrain, overwrites the
G-buffer with the water surface: view position, footprint-filtered wave
normal, unresolved slope variance, and the seabed colour, normal and water
depth taken from the terrain pixel it covers.  Images are torch CUDA
tensors ``(W, H, ...)`` - the layout of the reference's Taichi fields - or
``(H, W, ...)`` with ``layout="hw"``; work is enqueued on the current CUDA
stream.  There is no CPU path.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, fields
from typing import Mapping

import numpy as np
import torch

from . import _native
from .shading import OCEAN_SURFACE_ID, OceanShading

CASCADES = 3
_HEIGHTS_M = (0.62, 0.14, 0.025)  # per-cascade wave heights (ocean.py:20)

# (field, lower, upper, message) of the range checks (ocean.py:67-110)
_RANGES = (
    ("roughness", 0.02, 1.0, "ocean.roughness must be in 0.02..1"),
    ("normal_strength", 0.0, 1.0, "ocean.normal_strength must be in 0..1"),
    ("sky_reflection_strength", 0.0, 1.0, "ocean.sky_reflection_strength must be in 0..1"),
    ("dielectric_f0", 0.0, 0.2, "ocean.dielectric_f0 must be in 0..0.2"),
    ("wind_speed_mps", 0.1, 40.0, "ocean.wind_speed_mps must be in 0.1..40"),
    ("wave_height_scale", 0.0, 4.0, "ocean.wave_height_scale must be in 0..4"),
    ("choppiness", 0.0, 1.0, "ocean.choppiness must be in 0..1"),
    ("geometry_cascades", 0, CASCADES, "ocean.geometry_cascades must be in 0..3"),
    ("refraction_index", 1.0, 2.0, "ocean.refraction_index must be in 1..2"),
    ("refraction_strength", 0.0, 1.0, "ocean.refraction_strength must be in 0..1"),
)


def opaque_surface_height_m(terrain_height_m: float, ocean_enabled: bool) -> float:
    """The first opaque radial surface for camera and atmosphere queries
    (ocean.py:27-35): sea level caps the terrain from below when the sea is
    drawn."""

    h = float(terrain_height_m)
    return max(h, 0.0) if ocean_enabled else h


@dataclass(frozen=True)
class OceanConfig:
    """Sea-level coverage and the water material (ocean.py:38-190).
    ``surface_enabled`` draws the sea-level boundary; ``enabled`` selects
    the wave and BRDF path (off: a flat diffuse sea level)."""

    surface_enabled: bool = True
    enabled: bool = True
    albedo: tuple = (0.012, 0.055, 0.16)
    roughness: float = 0.12
    normal_strength: float = 0.32
    sky_reflection_strength: float = 1.0
    dielectric_f0: float = 0.02
    absorption_per_m: tuple = (0.14, 0.055, 0.022)
    scattering_per_m: tuple = (0.0025, 0.005, 0.012)
    max_visible_depth_m: float = 80.0
    spectrum_resolution: int = 128
    wind_speed_mps: float = 8.0
    wind_direction_degrees: float = 35.0
    wave_height_scale: float = 1.0
    choppiness: float = 0.65
    geometry_cascades: int = 2
    geometry_max_distance_m: float = 25_000.0
    refraction_index: float = 1.333
    refraction_strength: float = 1.0
    refraction_max_offset_pixels: float = 48.0

    def __post_init__(self) -> None:
        if len(self.albedo) != 3:
            raise ValueError("ocean.albedo must contain three components")
        if not all(0.0 <= float(a) <= 1.0 for a in self.albedo):
            raise ValueError("ocean.albedo components must be in 0..1")
        checks = {name: (lo, hi, msg) for name, lo, hi, msg in _RANGES}
        for name in ("roughness", "normal_strength", "sky_reflection_strength", "dielectric_f0"):
            lo, hi, msg = checks[name]
            if not lo <= getattr(self, name) <= hi:
                raise ValueError(msg)
        for name in ("absorption_per_m", "scattering_per_m"):
            values = getattr(self, name)
            if len(values) != 3 or min(float(v) for v in values) < 0.0:
                raise ValueError(f"ocean.{name} must contain three non-negative values")
        if self.max_visible_depth_m <= 0.0:
            raise ValueError("ocean.max_visible_depth_m must be positive")
        if self.spectrum_resolution not in (32, 64, 128, 256):
            raise ValueError("ocean.spectrum_resolution must be 32, 64, 128 or 256")
        lo, hi, msg = checks["wind_speed_mps"]
        if not lo <= self.wind_speed_mps <= hi:
            raise ValueError(msg)
        if not math.isfinite(self.wind_direction_degrees):
            raise ValueError("ocean.wind_direction_degrees must be finite")
        for name in ("wave_height_scale", "choppiness", "geometry_cascades"):
            lo, hi, msg = checks[name]
            if not lo <= getattr(self, name) <= hi:
                raise ValueError(msg)
        if self.geometry_max_distance_m < 0.0:
            raise ValueError("ocean.geometry_max_distance_m must be non-negative")
        for name in ("refraction_index", "refraction_strength"):
            lo, hi, msg = checks[name]
            if not lo <= getattr(self, name) <= hi:
                raise ValueError(msg)
        if self.refraction_max_offset_pixels < 0.0:
            raise ValueError("ocean.refraction_max_offset_pixels must be non-negative")

    @classmethod
    def from_mapping(cls, values: Mapping[str, object]) -> "OceanConfig":
        """The ``ocean`` block of a scene JSON (ocean.py:111-190): absent keys
        take the defaults, values are coerced to the fields' types."""

        defaults = cls()
        raw = values.get("albedo", list(defaults.albedo))
        if not isinstance(raw, (list, tuple)) or len(raw) != 3:
            raise ValueError("ocean.albedo must contain three components")
        kwargs = {}
        for f in fields(cls):
            default = getattr(defaults, f.name)
            value = values.get(f.name, default)
            if isinstance(default, bool):
                kwargs[f.name] = bool(value)
            elif isinstance(default, tuple):
                kwargs[f.name] = tuple(float(v) for v in value)
            else:
                kwargs[f.name] = type(default)(value)
        return cls(**kwargs)

    def wind_amplitude_scale(self) -> float:
        return min(max(self.wind_speed_mps / 8.0, 0.25), 2.0)

    def shading(self) -> OceanShading:
        """The fields the surface shading reads."""

        return OceanShading(enabled=self.enabled, roughness=self.roughness, dielectric_f0=self.dielectric_f0,
                            sky_reflection_strength=self.sky_reflection_strength,
                            absorption_per_m=tuple(self.absorption_per_m),
                            scattering_per_m=tuple(self.scattering_per_m),
                            max_visible_depth_m=self.max_visible_depth_m, refraction_index=self.refraction_index,
                            refraction_strength=self.refraction_strength,
                            refraction_max_offset_pixels=self.refraction_max_offset_pixels)

    def native(self) -> _native.AtmOceanConfig:
        c = _native.AtmOceanConfig()
        c.surface_enabled = int(bool(self.surface_enabled))
        c.enabled = int(bool(self.enabled))
        c.albedo[:] = [float(v) for v in self.albedo]
        c.normal_strength = float(self.normal_strength)
        c.max_visible_depth_m = float(self.max_visible_depth_m)
        c.spectrum_resolution = int(self.spectrum_resolution)
        c.geometry_cascades = int(self.geometry_cascades)
        c.wind_speed_mps = float(self.wind_speed_mps)
        c.wind_direction_degrees = float(self.wind_direction_degrees)
        c.wave_height_scale = float(self.wave_height_scale)
        c.choppiness = float(self.choppiness)
        c.geometry_max_distance_m = float(self.geometry_max_distance_m)
        return c


# the G-buffer images of rasterize, in the reference's argument order, with
# (dtype, floats per element: -1 = the frame's channels, 0 = one scalar)
_IMAGES = (("depth", torch.float32, 0), ("position", torch.float32, -1), ("normal", torch.float32, -1),
           ("albedo", torch.float32, -1), ("material_weights", torch.float32, 4), ("height_m", torch.float32, 0),
           ("water_depth", torch.float32, 0), ("seabed_albedo", torch.float32, -1),
           ("seabed_normal", torch.float32, -1), ("slope_variance", torch.float32, 0),
           ("surface_id", torch.int32, 0), ("cell_id", torch.int32, 0))


def _element_strides(t: torch.Tensor, per_element: int, layout: str) -> tuple:
    sx, sy = (t.stride(0), t.stride(1)) if layout == "wh" else (t.stride(1), t.stride(0))
    if sx % per_element or sy % per_element:
        raise ValueError("image strides must be whole elements")
    return sx // per_element, sy // per_element


class OceanRenderer:
    """Rasterises an analytic sea-level sphere into the shared G-buffer
    (ocean.py:193-771)."""

    def __init__(self, width: int, height: int, config: OceanConfig, layout: str = "wh",
                 device: str | torch.device | None = None):
        if layout not in ("wh", "hw"):
            raise ValueError("layout must be 'wh' (Taichi field layout) or 'hw'")
        self.width, self.height = int(width), int(height)
        self.config = config
        self.layout = layout
        self.device = torch.device(device if device is not None else "cuda")
        if self.device.type == "cuda" and self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        scale = config.wave_height_scale * config.wind_amplitude_scale()
        self.max_geometry_displacement_m = sum(_HEIGHTS_M[:config.geometry_cascades]) * scale
        self._lib = _native.library()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.check(self._lib.atm_ocean_create(ctypes.byref(config.native()), ctypes.byref(h)))
        self._handle = h

    def rasterize(self, depth, position_view, normal_global, albedo, material_weights, height_m, water_depth_m,
                  seabed_albedo, seabed_normal, slope_variance, surface_id, surface_cell_id, planet_radius_m: float,
                  camera_altitude_m: float, planet_frame, view_basis, tangent_half_fov: float, time_seconds: float,
                  debug_mode: int) -> None:
        """OceanRenderer.rasterize (ocean.py:686-762) on the frame's G-buffer
        tensors, in the reference's argument order.  ``planet_frame`` is the
        camera's (east, up, north) in planet coordinates, ``view_basis`` its
        (right, up, forward) in the local frame."""

        tensors = (depth, position_view, normal_global, albedo, material_weights, height_m, water_depth_m,
                   seabed_albedo, seabed_normal, slope_variance, surface_id, surface_cell_id)
        image = self._image(tensors)
        imgs = _native.AtmOceanImages(*[ctypes.c_void_p(t.data_ptr()) for t in tensors])
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _native.check(self._lib.atm_ocean_rasterize(
            self._handle, ctypes.byref(imgs), ctypes.byref(image), float(planet_radius_m), float(camera_altitude_m),
            _native.d9(planet_frame), _native.d9(view_basis), float(tangent_half_fov), float(time_seconds),
            int(debug_mode), ctypes.c_void_p(stream)))

    def rasterize_gbuffer(self, gbuffer: dict, *args, **kwargs) -> None:
        """``rasterize`` over a dict holding the images under the names
        ``depth``, ``position``, ``normal``, ``albedo``, ``material_weights``,
        ``height_m``, ``water_depth``, ``seabed_albedo``, ``seabed_normal``,
        ``slope_variance``, ``surface_id`` and ``cell_id``."""

        self.rasterize(*(gbuffer[name] for name, _, _ in _IMAGES), *args, **kwargs)

    def _image(self, tensors) -> _native.AtmImage:
        ref = tensors[1]
        if not isinstance(ref, torch.Tensor) or ref.dim() != 3 or ref.shape[2] not in (3, 4) or ref.stride(2) != 1:
            raise ValueError("position_view must be a float32 CUDA tensor (W, H, 3|4) with contiguous channels")
        channels = int(ref.shape[2])
        dims = (int(ref.shape[0]), int(ref.shape[1])) if self.layout == "wh" else (int(ref.shape[1]),
                                                                                  int(ref.shape[0]))
        if dims != (self.width, self.height):
            raise ValueError(f"G-buffer is {dims[0]}x{dims[1]}, the ocean renderer {self.width}x{self.height}")
        strides = _element_strides(ref, channels, self.layout)
        for t, (name, dtype, per) in zip(tensors, _IMAGES):
            per = channels if per < 0 else per
            if not isinstance(t, torch.Tensor) or t.dtype != dtype or t.device != self.device:
                raise ValueError(f"{name} must be a {dtype} tensor on {self.device}")
            shape = tuple(t.shape[:2]) if self.layout == "wh" else (int(t.shape[1]), int(t.shape[0]))
            if shape != dims or t.dim() != (3 if per else 2) or (per and (t.shape[2] != per or t.stride(2) != 1)):
                raise ValueError(f"{name} must have the frame's shape with {per or 1} values per pixel")
            if _element_strides(t, per or 1, self.layout) != strides:
                raise ValueError(f"{name} must share the G-buffer's element strides")
        return _native.AtmImage(self.width, self.height, strides[0], strides[1], channels)

    def spectrum(self) -> dict:
        """The last frame's wave spectrum as numpy arrays indexed [cascade,
        x, y] (synchronises the current stream)."""

        n = self.config.spectrum_resolution
        out = {"height": np.zeros((CASCADES, n, n), np.float32), "gradient": np.zeros((CASCADES, n, n, 2), np.float32),
               "displacement": np.zeros((CASCADES, n, n, 2), np.float32),
               "jacobian": np.zeros((CASCADES, n, n, 4), np.float32)}
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _native.check(self._lib.atm_ocean_read_spectrum(self._handle, *(a.ctypes.data for a in out.values()),
                                                        ctypes.c_void_p(stream)))
        return out

    def close(self) -> None:
        if self._handle:
            self._lib.atm_ocean_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["OCEAN_SURFACE_ID", "OceanConfig", "OceanRenderer", "opaque_surface_height_m"]
