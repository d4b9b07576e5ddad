"""Surface shading that consumes ``AtmosphereRenderer.prepare_frame``'s
``surface_sun_transmittance`` / ``surface_sky_radiance``: the reference's
``PlanetRenderer._shade_surface`` (``src/planet_renderer/renderer.py
:1277-1575``) over ``atm_shade_surface``, with the same arguments.

Land pixels are Lambertian under the transmitted sun plus the sky radiance.
Ocean pixels (advanced ocean on) add a GGX-style sun specular, Fresnel sky
reflection and a water body over the seabed, reconstructed along the refracted
view ray from the opaque terrain snapshot.  Images are torch CUDA tensors
``(W, H, ...)`` - the layout of the reference's Taichi fields - or ``(H, W,
...)`` with ``layout="hw"``; work is enqueued on the current CUDA stream.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from . import _native

OCEAN_SURFACE_ID = 2_147_000_000  # ocean.py:17

FLOAT_IMAGES = ("position", "normal", "albedo", "seabed_albedo", "seabed_normal", "terrain_position",
                "terrain_normal", "terrain_albedo")
SCALAR_IMAGES = ("water_depth", "slope_variance")
ID_IMAGES = ("surface_id", "terrain_surface_id")
# the G-buffer and terrain-snapshot images of a shading call (the rest of
# _native.SHADE_IMAGES are the surface lighting and the output)
GBUFFER_IMAGES = ("position", "normal", "albedo", "water_depth", "seabed_albedo", "seabed_normal", "slope_variance",
                  "surface_id", "terrain_position", "terrain_normal", "terrain_albedo", "terrain_surface_id")


@dataclass(frozen=True)
class OceanShading:
    """The OceanConfig fields the shading reads (ocean.py:38-65), with their
    defaults; ``enabled`` is the advanced-ocean switch."""

    enabled: bool = True
    roughness: float = 0.12
    dielectric_f0: float = 0.02
    sky_reflection_strength: float = 1.0
    absorption_per_m: tuple = (0.14, 0.055, 0.022)
    scattering_per_m: tuple = (0.0025, 0.005, 0.012)
    max_visible_depth_m: float = 80.0
    refraction_index: float = 1.333
    refraction_strength: float = 1.0
    refraction_max_offset_pixels: float = 48.0


def _element_strides(t: torch.Tensor, per_element: int, layout: str) -> tuple:
    sx, sy = (t.stride(0), t.stride(1)) if layout == "wh" else (t.stride(1), t.stride(0))
    if sx % per_element or sy % per_element:
        raise ValueError("image strides must be whole elements")
    return sx // per_element, sy // per_element


def shade_arguments(images: dict, ref: torch.Tensor, sun_global, solar_irradiance, view_basis_global,
                    ocean: OceanShading, sun_angular_radius: float, tangent_half_fov: float, mode: int = 0,
                    layout: str = "wh", ocean_surface_id: int = OCEAN_SURFACE_ID, names=None):
    """Checked native arguments of a shading call: (AtmShadeParams,
    AtmShadeImages, AtmImage).  ``images`` maps the names of ``names``
    (default: every image of ``_native.SHADE_IMAGES``) to tensors sharing
    ``ref``'s frame shape, channels and strides; images left out of ``names``
    are passed as null."""

    if layout not in ("wh", "hw"):
        raise ValueError("layout must be 'wh' (Taichi field layout) or 'hw'")
    names = tuple(names or _native.SHADE_IMAGES)
    missing = [n for n in names if n not in images]
    if missing:
        raise ValueError(f"missing images: {missing}")
    if not isinstance(ref, torch.Tensor) or ref.dim() != 3 or ref.shape[2] not in (3, 4) or ref.stride(2) != 1:
        raise ValueError("the frame's images must be float32 CUDA tensors (W, H, 3|4) with contiguous channels")
    channels = int(ref.shape[2])
    dims = (int(ref.shape[0]), int(ref.shape[1])) if layout == "wh" else (int(ref.shape[1]), int(ref.shape[0]))
    strides = _element_strides(ref, channels, layout)
    for name in names:
        t = images[name]
        scalar = name in SCALAR_IMAGES or name in ID_IMAGES
        dtype = torch.int32 if name in ID_IMAGES else torch.float32
        if not isinstance(t, torch.Tensor) or t.device != ref.device or t.dtype != dtype:
            raise ValueError(f"{name} must be a {dtype} CUDA tensor on the frame's device")
        shape = tuple(t.shape[:2]) if layout == "wh" else (int(t.shape[1]), int(t.shape[0]))
        if t.dim() != (2 if scalar else 3) or shape != dims:
            raise ValueError(f"{name} must have the frame's shape")
        if scalar:
            if _element_strides(t, 1, layout) != strides:
                raise ValueError(f"{name} must share the images' element strides")
        elif t.shape[2] != channels or t.stride(2) != 1 or _element_strides(t, channels, layout) != strides:
            raise ValueError(f"{name} must share the frame's channels and strides")
    p = _native.AtmShadeParams()
    p.sun_global[:] = [float(v) for v in sun_global]
    p.solar_irradiance[:] = [float(v) for v in solar_irradiance]
    right, up, forward = view_basis_global
    p.view_right_global[:] = [float(v) for v in right]
    p.view_up_global[:] = [float(v) for v in up]
    p.view_forward_global[:] = [float(v) for v in forward]
    p.advanced_ocean_enabled = 1 if ocean.enabled else 0
    p.mode = int(mode)
    p.ocean_roughness = float(ocean.roughness)
    p.ocean_f0 = float(ocean.dielectric_f0)
    p.ocean_sky_strength = float(ocean.sky_reflection_strength)
    p.ocean_absorption[:] = [float(v) for v in ocean.absorption_per_m]
    p.ocean_scattering[:] = [float(v) for v in ocean.scattering_per_m]
    p.ocean_max_depth = float(ocean.max_visible_depth_m)
    p.ocean_refraction_index = float(ocean.refraction_index)
    p.ocean_refraction_strength = float(ocean.refraction_strength)
    p.ocean_refraction_max_offset_pixels = float(ocean.refraction_max_offset_pixels)
    p.sun_angular_radius = float(sun_angular_radius)
    p.tangent_half_fov = float(tangent_half_fov)
    p.ocean_surface_id = int(ocean_surface_id)
    ptrs = _native.AtmShadeImages(*[ctypes.c_void_p(images[n].data_ptr() if n in names else None)
                                    for n in _native.SHADE_IMAGES])
    return p, ptrs, _native.AtmImage(dims[0], dims[1], strides[0], strides[1], channels)


def shade_surface(gbuffer: dict, sun_transmittance: torch.Tensor, sky_radiance: torch.Tensor,
                  surface_hdr: torch.Tensor, sun_global, solar_irradiance, view_basis_global,
                  ocean: OceanShading, sun_angular_radius: float, tangent_half_fov: float, mode: int = 0,
                  layout: str = "wh", ocean_surface_id: int = OCEAN_SURFACE_ID) -> None:
    """_shade_surface (renderer.py:1277-1575) into ``surface_hdr``.  ``gbuffer``
    holds the G-buffer and terrain-snapshot images named as in
    ``_native.SHADE_IMAGES``; ``view_basis_global`` the camera's right, up and
    forward directions in the global frame; ``sun_angular_radius`` radians."""

    images = dict(gbuffer, sun_transmittance=sun_transmittance, sky_radiance=sky_radiance, surface_hdr=surface_hdr)
    p, ptrs, image = shade_arguments(images, surface_hdr, sun_global, solar_irradiance, view_basis_global, ocean,
                                     sun_angular_radius, tangent_half_fov, mode, layout, ocean_surface_id)
    lib = _native.library()
    _native.check(lib.atm_shade_surface(ctypes.byref(p), ctypes.byref(ptrs), ctypes.byref(image),
                                        ctypes.c_void_p(torch.cuda.current_stream(surface_hdr.device).cuda_stream)))
