"""ctypes binding of the CPU oracle (``atm_oracle.cpp``) - TEST INFRASTRUCTURE.

Only the tests, the smoke check and the bench's CPU-baseline leg use this
module, as the checker; the product never imports it.

``OracleAtmosphere`` restates the reference's host-side logic of
``AtmosphereRenderer`` (``src/planet_renderer/atmosphere/renderer.py``:
``update`` :2072-2137 with its cache keys and f64->f32 rounding points,
``prepare_frame`` :2139-2187, ``composite`` :2189-2238, ``set_luts_frozen``
:2057-2070) on top of the oracle kernels, in numpy arrays of the Taichi field
layout ``(W, H[, D], 3)``.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import fields
from pathlib import Path

import numpy as np

from . import build_oracle

_LIB = None


class AtmParams(ctypes.Structure):
    """Mirror of ``AtmParams`` in include/atm_capi.h."""

    _fields_ = [
        ("top_altitude_m", ctypes.c_double),
        ("rayleigh_scattering_per_m", ctypes.c_double * 3),
        ("rayleigh_scale_height_m", ctypes.c_double),
        ("mie_scattering_per_m", ctypes.c_double * 3),
        ("mie_extinction_per_m", ctypes.c_double * 3),
        ("mie_scale_height_m", ctypes.c_double),
        ("mie_phase_g", ctypes.c_double),
        ("absorption_extinction_per_m", ctypes.c_double * 3),
        ("absorption_peak_altitude_m", ctypes.c_double),
        ("absorption_half_width_m", ctypes.c_double),
        ("ground_albedo", ctypes.c_double * 3),
        ("transmittance_lut_width", ctypes.c_int32),
        ("transmittance_lut_height", ctypes.c_int32),
        ("multi_scattering_lut_width", ctypes.c_int32),
        ("multi_scattering_lut_height", ctypes.c_int32),
        ("sky_view_lut_width", ctypes.c_int32),
        ("sky_view_lut_height", ctypes.c_int32),
        ("aerial_lut_width", ctypes.c_int32),
        ("aerial_lut_height", ctypes.c_int32),
        ("aerial_lut_depth", ctypes.c_int32),
        ("transmittance_steps", ctypes.c_int32),
        ("multi_scattering_directions", ctypes.c_int32),
        ("multi_scattering_steps", ctypes.c_int32),
        ("sky_view_steps", ctypes.c_int32),
        ("aerial_steps_per_slice", ctypes.c_int32),
        ("aerial_horizon_raymarch_steps", ctypes.c_int32),
        ("aerial_terminator_substeps", ctypes.c_int32),
    ]


class CompositeArgs(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
        ("diagnostic_view", ctypes.c_int32),
        ("bottom", ctypes.c_double),
        ("cam_alt", ctypes.c_double),
        ("sky_alt", ctypes.c_double),
        ("ar", ctypes.c_double),
        ("tanfov", ctypes.c_double),
        ("star_start", ctypes.c_double),
        ("star_end", ctypes.c_double),
        ("sun", ctypes.c_double * 3),
        ("E", ctypes.c_double * 3),
        ("disk", ctypes.c_double * 3),
        ("right", ctypes.c_double * 3),
        ("up", ctypes.c_double * 3),
        ("fwd", ctypes.c_double * 3),
    ]


def params_from_config(config) -> AtmParams:
    """Fill AtmParams from any object with AtmosphereConfig's field names."""

    p = AtmParams()
    for name, ctype in AtmParams._fields_:
        value = getattr(config, name)
        if isinstance(value, (tuple, list)):
            getattr(p, name)[:] = [float(v) for v in value]
        elif ctype is ctypes.c_int32:
            setattr(p, name, int(value))
        else:
            setattr(p, name, float(value))
    return p


def library() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        lib = ctypes.CDLL(str(path))
        _LIB = lib
    return _LIB


def _d3(values) -> ctypes.Array:
    return (ctypes.c_double * 3)(*[float(v) for v in values])


def _ptr(array: np.ndarray):
    assert array.flags["C_CONTIGUOUS"]
    return array.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """Kernel-level oracle.  ``precision`` "f32" mirrors Taichi f32; "f64"
    is the same algorithm in double."""

    def __init__(self, precision: str = "f32", threads: int | None = None, series_weight: bool = False):
        if precision not in ("f32", "f64"):
            raise ValueError(precision)
        self.precision = precision
        self.dtype = np.float32 if precision == "f32" else np.float64
        # series_weight: NOT the reference - the segment weight by its Taylor
        # series where the reference's formula cancels (a diagnostic variant)
        self.series_weight = bool(series_weight)
        self.lib = library()
        if threads:
            self.lib.orc_set_threads(int(threads))

    def _fn(self, name):
        self.lib.orc_set_series_weight(int(self.series_weight))
        return getattr(self.lib, f"orc_{name}_{self.precision}")

    def _arr(self, a) -> np.ndarray:
        return np.ascontiguousarray(a, dtype=self.dtype)

    def build_transmittance(self, config, bottom_radius: float) -> np.ndarray:
        p = params_from_config(config)
        out = np.zeros((config.transmittance_lut_width, config.transmittance_lut_height, 3), self.dtype)
        fn = self._fn("build_transmittance")
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_double, ctypes.c_void_p]
        fn(ctypes.byref(p), float(bottom_radius), _ptr(out))
        return out

    def build_multi_scattering(self, config, bottom_radius, irradiance, angular_radius_rad, tlut):
        p = params_from_config(config)
        tlut = self._arr(tlut)
        out = np.zeros((config.multi_scattering_lut_width, config.multi_scattering_lut_height, 3), self.dtype)
        fn = self._fn("build_multi_scattering")
        fn.restype = ctypes.c_int64
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_double, ctypes.c_double * 3, ctypes.c_double,
                       ctypes.c_void_p, ctypes.c_void_p]
        n = fn(ctypes.byref(p), float(bottom_radius), _d3(irradiance), float(angular_radius_rad), _ptr(tlut),
               _ptr(out))
        return out

    def build_sky_view(self, config, bottom_radius, camera_altitude, sun_zenith_cosine, irradiance,
                       angular_radius_rad, tlut, mslut):
        p = params_from_config(config)
        tlut, mslut = self._arr(tlut), self._arr(mslut)
        out = np.zeros((config.sky_view_lut_width, config.sky_view_lut_height, 3), self.dtype)
        fn = self._fn("build_sky_view")
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                       ctypes.c_double * 3, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        fn(ctypes.byref(p), float(bottom_radius), float(camera_altitude), float(sun_zenith_cosine), _d3(irradiance),
           float(angular_radius_rad), _ptr(tlut), _ptr(mslut), _ptr(out))
        return out

    def build_aerial(self, config, width, height, bottom_radius, camera_altitude, sun, irradiance,
                     angular_radius_rad, basis, tangent_half_fov, tlut, mslut):
        p = params_from_config(config)
        tlut, mslut = self._arr(tlut), self._arr(mslut)
        out = np.zeros((config.aerial_lut_width, config.aerial_lut_height, config.aerial_lut_depth, 3), self.dtype)
        fn = self._fn("build_aerial")
        d3 = ctypes.c_double * 3
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, d3,
                       d3, ctypes.c_double, d3, d3, d3, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                       ctypes.c_void_p]
        right, up, forward = basis
        fn(ctypes.byref(p), int(width), int(height), float(bottom_radius), float(camera_altitude), _d3(sun),
           _d3(irradiance), float(angular_radius_rad), _d3(right), _d3(up), _d3(forward), float(tangent_half_fov),
           _ptr(tlut), _ptr(mslut), _ptr(out))
        return out

    def prepare_surface(self, config, position_view, surface_id, bottom_radius, camera_altitude, sun,
                        angular_radius_rad, basis, tlut, mslut):
        p = params_from_config(config)
        pos = self._arr(position_view)
        sid = np.ascontiguousarray(surface_id, dtype=np.int32)
        W, H = sid.shape
        tlut, mslut = self._arr(tlut), self._arr(mslut)
        sun_t = np.zeros((W, H, 3), self.dtype)
        sky = np.zeros((W, H, 3), self.dtype)
        fn = self._fn("prepare_surface")
        d3 = ctypes.c_double * 3
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                       ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double, d3,
                       ctypes.c_double, d3, d3, d3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                       ctypes.c_void_p]
        right, up, forward = basis
        fn(ctypes.byref(p), W, H, H, 1, 3, _ptr(pos), _ptr(sid), float(bottom_radius), float(camera_altitude),
           _d3(sun), float(angular_radius_rad), _d3(right), _d3(up), _d3(forward), _ptr(tlut), _ptr(mslut),
           _ptr(sun_t), _ptr(sky))
        return sun_t, sky

    def sky_rays(self, config, bottom_radius, altitudes, rays, suns, irradiance, angular_radius_rad, tlut, mslut):
        """Sky radiance along each ray (n, 3) from its altitude (n,), sun (n, 3)."""

        p = params_from_config(config)
        h, r, s = self._arr(altitudes), self._arr(rays), self._arr(suns)
        n = h.shape[0]
        out = np.zeros((n, 3), self.dtype)
        fn = self._fn("sky_rays")
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_double, ctypes.c_int] + [ctypes.c_void_p] * 3 + \
            [ctypes.c_double * 3, ctypes.c_double] + [ctypes.c_void_p] * 3
        fn(ctypes.byref(p), float(bottom_radius), n, _ptr(h), _ptr(r), _ptr(s), _d3(irradiance),
           float(angular_radius_rad), _ptr(self._arr(tlut)), _ptr(self._arr(mslut)), _ptr(out))
        return out

    def surface_rays(self, config, bottom_radius, altitudes, rays, surface_distances, suns, irradiance,
                     angular_radius_rad, tlut, mslut):
        """(in-scattering, transmittance) (n, 3) each of camera-to-surface segments."""

        p = params_from_config(config)
        h, r, d, s = (self._arr(a) for a in (altitudes, rays, surface_distances, suns))
        n = h.shape[0]
        L = np.zeros((n, 3), self.dtype)
        T = np.zeros((n, 3), self.dtype)
        fn = self._fn("surface_rays")
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_double, ctypes.c_int] + [ctypes.c_void_p] * 4 + \
            [ctypes.c_double * 3, ctypes.c_double] + [ctypes.c_void_p] * 4
        fn(ctypes.byref(p), float(bottom_radius), n, _ptr(h), _ptr(r), _ptr(d), _ptr(s), _d3(irradiance),
           float(angular_radius_rad), _ptr(self._arr(tlut)), _ptr(self._arr(mslut)), _ptr(L), _ptr(T))
        return L, T

    def composite(self, config, scene_hdr, space_hdr, surface_id, position_view, bottom_radius,
                  camera_altitude, sky_lut_camera_altitude, sun, irradiance, disk_radiance, angular_radius_rad,
                  basis, tangent_half_fov, star_start, star_end, diagnostic_view, tlut, mslut, svlut, aplut,
                  pixel_list=None, out=None, margin_out=None):
        """Returns (hdr, radiance_samples).  ``pixel_list`` (n,) int32 linear
        indices x*H + y restricts the pixels computed (others left as in
        ``out``, zero by default).  ``margin_out`` (W, H) float64 receives per
        computed pixel the smallest distance (m) of any density evaluation's
        altitude from the profile's cutoffs (0 and the shell top)."""

        p = params_from_config(config)
        sid = np.ascontiguousarray(surface_id, dtype=np.int32)
        W, H = sid.shape
        scene, space, pos = self._arr(scene_hdr), self._arr(space_hdr), self._arr(position_view)
        tlut, mslut, svlut, aplut = (self._arr(a) for a in (tlut, mslut, svlut, aplut))
        hdr = np.zeros((W, H, 3), self.dtype) if out is None else out
        a = CompositeArgs()
        a.width, a.height, a.diagnostic_view = W, H, int(diagnostic_view)
        a.bottom, a.cam_alt, a.sky_alt = float(bottom_radius), float(camera_altitude), float(sky_lut_camera_altitude)
        a.ar, a.tanfov = float(angular_radius_rad), float(tangent_half_fov)
        a.star_start, a.star_end = float(star_start), float(star_end)
        a.sun[:] = [float(v) for v in sun]
        a.E[:] = [float(v) for v in irradiance]
        a.disk[:] = [float(v) for v in disk_radiance]
        right, up, forward = basis
        a.right[:] = [float(v) for v in right]
        a.up[:] = [float(v) for v in up]
        a.fwd[:] = [float(v) for v in forward]
        fn = self._fn("composite")
        fn.restype = ctypes.c_int64
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.POINTER(CompositeArgs), ctypes.c_int, ctypes.c_int,
                       ctypes.c_int] + [ctypes.c_void_p] * 9 + [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
        if pixel_list is None:
            plist, n = None, 0
        else:
            plist = np.ascontiguousarray(pixel_list, dtype=np.int32)
            n = plist.size
        samples = fn(ctypes.byref(p), ctypes.byref(a), H, 1, 3, _ptr(scene), _ptr(space), _ptr(sid), _ptr(pos),
                     _ptr(tlut), _ptr(mslut), _ptr(svlut), _ptr(aplut), _ptr(hdr),
                     None if plist is None else _ptr(plist), n,
                     None if margin_out is None else _ptr(margin_out))
        return hdr, int(samples)


def sun_disk_radiance(irradiance, angular_radius_degrees):
    omega = math.pi * math.sin(math.radians(angular_radius_degrees)) ** 2
    return tuple(float(v) / omega for v in irradiance)


class OracleAtmosphere:
    """Host-logic restatement of the reference AtmosphereRenderer on the oracle."""

    def __init__(self, width: int, height: int, config, precision: str = "f32"):
        self.width, self.height, self.config = int(width), int(height), config
        self.kernels = Oracle(precision)
        dt = self.kernels.dtype
        c = config
        self.transmittance_lut = np.zeros((c.transmittance_lut_width, c.transmittance_lut_height, 3), dt)
        self.multi_scattering_lut = np.zeros((c.multi_scattering_lut_width, c.multi_scattering_lut_height, 3), dt)
        self.sky_view_lut = np.zeros((c.sky_view_lut_width, c.sky_view_lut_height, 3), dt)
        self.aerial_scattering_lut = np.zeros(
            (c.aerial_lut_width, c.aerial_lut_height, c.aerial_lut_depth, 3), dt)
        self.surface_sun_transmittance = np.zeros((self.width, self.height, 3), dt)
        self.surface_sky_radiance = np.zeros((self.width, self.height, 3), dt)
        self._planet_radius_key = None
        self._multi_scattering_key = None
        self._sky_key = None
        self.luts_frozen = False
        self.sky_snapshot_altitude_m = None
        self.sky_snapshot_sun_cosine = None
        self.aerial_snapshot_altitude_m = None
        self._aerial_available = False
        self.transmittance_rebuilds = 0
        self.multi_scattering_rebuilds = 0
        self.sky_view_rebuilds = 0
        self.aerial_rebuilds = 0

    def set_luts_frozen(self, frozen: bool) -> None:
        frozen = bool(frozen)
        if self.luts_frozen and not frozen:
            self._sky_key = None
        self.luts_frozen = frozen

    def update(self, planet_radius_m, camera_radius_m, sun_local, solar_irradiance, sun_angular_radius_degrees):
        planet_radius = float(planet_radius_m)
        camera_radius = float(camera_radius_m)
        sun = np.array(sun_local, dtype=np.float64)
        sun /= max(float(np.linalg.norm(sun)), 1.0e-12)
        ar = float(np.float32(math.radians(sun_angular_radius_degrees)))
        if self._planet_radius_key != planet_radius:
            self.transmittance_lut = self.kernels.build_transmittance(self.config, planet_radius)
            self._planet_radius_key = planet_radius
            self._multi_scattering_key = None
            self._sky_key = None
            self.transmittance_rebuilds += 1
        irradiance_key = tuple(float(v) for v in solar_irradiance)
        ms_key = (planet_radius, irradiance_key, ar)
        if ms_key != self._multi_scattering_key:
            self.multi_scattering_lut = self.kernels.build_multi_scattering(
                self.config, planet_radius, solar_irradiance, ar, self.transmittance_lut)
            self._multi_scattering_key = ms_key
            self._sky_key = None
            self.multi_scattering_rebuilds += 1
        alt_key = float(np.float32(max(camera_radius - planet_radius, 0.0)))
        zen_key = float(np.float32(np.clip(sun[1], -1.0, 1.0)))
        sky_key = (alt_key, zen_key, irradiance_key + (ar,))
        if sky_key != self._sky_key and (not self.luts_frozen or self._sky_key is None):
            self.sky_view_lut = self.kernels.build_sky_view(
                self.config, planet_radius, alt_key, zen_key, solar_irradiance, ar, self.transmittance_lut,
                self.multi_scattering_lut)
            self._sky_key = sky_key
            self.sky_snapshot_altitude_m = alt_key
            self.sky_snapshot_sun_cosine = zen_key
            self.sky_view_rebuilds += 1

    def prepare_frame(self, position_view, surface_id, planet_radius_m, camera_radius_m, sun_local,
                      solar_irradiance, sun_angular_radius_degrees, view_basis, tangent_half_fov):
        cam_alt = max(float(camera_radius_m) - float(planet_radius_m), 0.0)
        ar = math.radians(sun_angular_radius_degrees)
        self.surface_sun_transmittance, self.surface_sky_radiance = self.kernels.prepare_surface(
            self.config, position_view, surface_id, planet_radius_m, cam_alt, sun_local, ar, view_basis,
            self.transmittance_lut, self.multi_scattering_lut)
        if not self.luts_frozen or not self._aerial_available:
            self.aerial_scattering_lut = self.kernels.build_aerial(
                self.config, self.width, self.height, planet_radius_m, cam_alt, sun_local, solar_irradiance, ar,
                view_basis, tangent_half_fov, self.transmittance_lut, self.multi_scattering_lut)
            self.aerial_snapshot_altitude_m = float(camera_radius_m) - float(planet_radius_m)
            self._aerial_available = True
            self.aerial_rebuilds += 1

    def composite(self, scene_hdr, space_hdr, surface_id, position_view, planet_radius_m, camera_radius_m,
                  sun_local, solar_irradiance, sun_disk_radiance_rgb, sun_angular_radius_degrees, view_basis,
                  tangent_half_fov, star_contrast_start, star_contrast_end, diagnostic_view=0, pixel_list=None,
                  margin_out=None):
        cam_alt = max(float(camera_radius_m) - float(planet_radius_m), 0.0)
        sky_alt = cam_alt if self.sky_snapshot_altitude_m is None else self.sky_snapshot_altitude_m
        return self.kernels.composite(
            self.config, scene_hdr, space_hdr, surface_id, position_view, planet_radius_m, cam_alt, sky_alt,
            sun_local, solar_irradiance, sun_disk_radiance_rgb, math.radians(sun_angular_radius_degrees),
            view_basis, tangent_half_fov, star_contrast_start, star_contrast_end, int(diagnostic_view),
            self.transmittance_lut, self.multi_scattering_lut, self.sky_view_lut, self.aerial_scattering_lut,
            pixel_list=pixel_list, margin_out=margin_out)
