"""ctypes binding of libplanet_atm (the C ABI declared in include/atm_capi.h).

The library is built in-tree by ``build_native.py`` (``__graft_entry__.build()``
runs it).  There is no CPU fallback: if the library is missing or cannot be
loaded, :func:`library` raises ``RuntimeError``.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

LIBRARY_PATH = Path(__file__).resolve().parent / "lib" / "libplanet_atm.so"

ATM_OK = 0
ATM_E_INVALID = -1
ATM_E_CUDA = -2
ATM_E_NOMEM = -3
ATM_E_STATE = -4
ATM_E_TIMEOUT = -5

LUT_TRANSMITTANCE = 0
LUT_MULTI_SCATTERING = 1
LUT_SKY_VIEW = 2
LUT_AERIAL = 3

c_double3 = ctypes.c_double * 3
c_double9 = ctypes.c_double * 9


class AtmParams(ctypes.Structure):
    _fields_ = [
        ("top_altitude_m", ctypes.c_double),
        ("rayleigh_scattering_per_m", c_double3),
        ("rayleigh_scale_height_m", ctypes.c_double),
        ("mie_scattering_per_m", c_double3),
        ("mie_extinction_per_m", c_double3),
        ("mie_scale_height_m", ctypes.c_double),
        ("mie_phase_g", ctypes.c_double),
        ("absorption_extinction_per_m", c_double3),
        ("absorption_peak_altitude_m", ctypes.c_double),
        ("absorption_half_width_m", ctypes.c_double),
        ("ground_albedo", c_double3),
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

    @classmethod
    def from_config(cls, config) -> "AtmParams":
        p = cls()
        for name, ctype in cls._fields_:
            value = getattr(config, name)
            if isinstance(value, (tuple, list)):
                getattr(p, name)[:] = [float(v) for v in value]
            elif ctype is ctypes.c_int32:
                setattr(p, name, int(value))
            else:
                setattr(p, name, float(value))
        return p


class AtmImage(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
        ("stride_x", ctypes.c_int64),
        ("stride_y", ctypes.c_int64),
        ("channels", ctypes.c_int32),
    ]


class AtmState(ctypes.Structure):
    _fields_ = [
        ("luts_frozen", ctypes.c_int32),
        ("has_sky_snapshot", ctypes.c_int32),
        ("sky_snapshot_altitude_m", ctypes.c_double),
        ("sky_snapshot_sun_cosine", ctypes.c_double),
        ("has_aerial_snapshot", ctypes.c_int32),
        ("aerial_snapshot_altitude_m", ctypes.c_double),
        ("transmittance_rebuilds", ctypes.c_int64),
        ("multi_scattering_rebuilds", ctypes.c_int64),
        ("sky_view_rebuilds", ctypes.c_int64),
        ("aerial_rebuilds", ctypes.c_int64),
    ]


class AtmBuildArgs(ctypes.Structure):
    _fields_ = [
        ("planet_radius_m", ctypes.c_double),
        ("camera_altitude_m", ctypes.c_double),
        ("sun_zenith_cosine", ctypes.c_double),
        ("sun_local", c_double3),
        ("solar_irradiance", c_double3),
        ("sun_angular_radius_rad", ctypes.c_double),
        ("view_basis", c_double9),
        ("tangent_half_fov", ctypes.c_double),
        ("frame_width", ctypes.c_int32),
        ("frame_height", ctypes.c_int32),
    ]


class AtmBatchJob(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("param_set", ctypes.c_int32),
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
        ("depth", ctypes.c_int32),
        ("frame_width", ctypes.c_int32),
        ("frame_height", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("output_offset", ctypes.c_int64),
        ("camera_altitude_m", ctypes.c_double),
        ("sun_zenith_cosine", ctypes.c_double),
        ("sun_local", c_double3),
        ("view_basis", c_double9),
        ("tangent_half_fov", ctypes.c_double),
    ]


class AtmBatchTuning(ctypes.Structure):
    _fields_ = [
        ("sky_view_texels_per_item", ctypes.c_int32),
        ("aerial_columns_per_item", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
    ]


class AtmSampleOptions(ctypes.Structure):
    _fields_ = [
        ("shell_top_fraction", ctypes.c_double),
        ("surface_fraction", ctypes.c_double),
        ("surface_min_m", ctypes.c_double),
        ("surface_max_m", ctypes.c_double),
        ("start_min_m", ctypes.c_double),
        ("start_max_m", ctypes.c_double),
        ("sun_angle_fraction", ctypes.c_double),
        ("sun_angle_max_degrees", ctypes.c_double),
    ]


class AtmSurrogate(ctypes.Structure):
    _fields_ = [
        ("aerial", ctypes.c_void_p),
        ("sky", ctypes.c_void_p),
        ("aerial_above_shell", ctypes.c_void_p),
        ("scale_height_range", ctypes.c_double * 4),
        ("trained_planet_radius_m", ctypes.c_double),
        ("trained_top_altitude_m", ctypes.c_double),
        ("check_fraction", ctypes.c_double),
        ("aerial_floor", ctypes.c_double),
        ("aerial_floor_t", ctypes.c_double),
        ("sky_floor", ctypes.c_double),
        ("twilight_cosine", ctypes.c_double),
        ("sky_twilight_cosine", ctypes.c_double),
        ("limb_degrees", ctypes.c_double),
        ("seed", ctypes.c_uint32),
        ("tc_wait_polls", ctypes.c_int32),
        ("stats", ctypes.c_void_p),
        ("gate_terminator", ctypes.c_int32),
        ("calibration_tile", ctypes.c_int32),
    ]


ATM_SKY_PIXELS_PLAIN, ATM_SKY_PIXELS_NET, ATM_SKY_PIXELS_LUT = 0, 1, 2
ATM_SURROGATE_SKY = 0
ATM_SURROGATE_AERIAL = 1


class AtmShadeParams(ctypes.Structure):
    _fields_ = [
        ("sun_global", c_double3),
        ("solar_irradiance", c_double3),
        ("view_right_global", c_double3),
        ("view_up_global", c_double3),
        ("view_forward_global", c_double3),
        ("advanced_ocean_enabled", ctypes.c_int32),
        ("mode", ctypes.c_int32),
        ("ocean_roughness", ctypes.c_double),
        ("ocean_f0", ctypes.c_double),
        ("ocean_sky_strength", ctypes.c_double),
        ("ocean_absorption", c_double3),
        ("ocean_scattering", c_double3),
        ("ocean_max_depth", ctypes.c_double),
        ("ocean_refraction_index", ctypes.c_double),
        ("ocean_refraction_strength", ctypes.c_double),
        ("ocean_refraction_max_offset_pixels", ctypes.c_double),
        ("sun_angular_radius", ctypes.c_double),
        ("tangent_half_fov", ctypes.c_double),
        ("ocean_surface_id", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


SHADE_IMAGES = ("position", "normal", "albedo", "water_depth", "seabed_albedo", "seabed_normal", "slope_variance",
                "surface_id", "terrain_position", "terrain_normal", "terrain_albedo", "terrain_surface_id",
                "sun_transmittance", "sky_radiance", "surface_hdr")


class AtmShadeImages(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in SHADE_IMAGES]


class AtmPostConfig(ctypes.Structure):
    _fields_ = [
        ("exposure_ev", ctypes.c_double),
        ("bloom_threshold", ctypes.c_double),
        ("bloom_knee", ctypes.c_double),
        ("bloom_clamp", ctypes.c_double),
        ("bloom_strength", ctypes.c_double),
        ("bloom_passes", ctypes.c_int32),
    ]

class AtmRasterMesh(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in ("view", "normal", "material", "height_m", "cell", "triangles",
                                                     "active_slots", "skirt_mask", "slot_level")] + [
        (name, ctypes.c_int32) for name in ("patches", "vertices_per_patch", "triangles_per_patch",
                                            "surface_triangles_per_patch", "resolution", "n_active")]


RASTER_OUTPUTS = ("depth", "position", "normal", "albedo", "material_weights", "height_m", "surface_id", "cell_id",
                  "terrain_position", "terrain_normal", "terrain_albedo", "terrain_surface_id")


class AtmRasterOutputs(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in RASTER_OUTPUTS]


class AtmOceanConfig(ctypes.Structure):
    _fields_ = [
        ("surface_enabled", ctypes.c_int32),
        ("enabled", ctypes.c_int32),
        ("albedo", ctypes.c_double * 3),
        ("normal_strength", ctypes.c_double),
        ("max_visible_depth_m", ctypes.c_double),
        ("spectrum_resolution", ctypes.c_int32),
        ("geometry_cascades", ctypes.c_int32),
        ("wind_speed_mps", ctypes.c_double),
        ("wind_direction_degrees", ctypes.c_double),
        ("wave_height_scale", ctypes.c_double),
        ("choppiness", ctypes.c_double),
        ("geometry_max_distance_m", ctypes.c_double),
    ]


OCEAN_IMAGES = ("depth", "position", "normal", "albedo", "material_weights", "height_m", "water_depth",
                "seabed_albedo", "seabed_normal", "slope_variance", "surface_id", "cell_id")


class AtmOceanImages(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in OCEAN_IMAGES]


_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_D = ctypes.c_double

# name -> (restype, argtypes); the exported entry points of atm_capi.h
SIGNATURES = {
    "atm_last_error": (ctypes.c_char_p, []),
    "atm_create": (ctypes.c_int, [ctypes.POINTER(AtmParams), _I32, _I32, ctypes.POINTER(_P)]),
    "atm_destroy": (ctypes.c_int, [_P]),
    "atm_set_luts_frozen": (ctypes.c_int, [_P, _I32]),
    "atm_get_state": (ctypes.c_int, [_P, ctypes.POINTER(AtmState)]),
    "atm_update": (ctypes.c_int, [_P, _D, _D, c_double3, c_double3, _D, _P]),
    "atm_prepare_frame": (
        ctypes.c_int,
        [_P, _P, _P, ctypes.POINTER(AtmImage), _D, _D, c_double3, c_double3, _D, c_double9, _D, _P, _P, _P],
    ),
    "atm_composite": (
        ctypes.c_int,
        [_P, _P, _P, _P, _P, _P, ctypes.POINTER(AtmImage), _D, _D, c_double3, c_double3, c_double3, _D, c_double9,
         _D, _D, _D, _I32, _P],
    ),
    "atm_build_lut": (ctypes.c_int, [_P, _I32, ctypes.POINTER(AtmBuildArgs), _P]),
    "atm_lut_info": (ctypes.c_int, [_P, _I32, ctypes.POINTER(_I32), ctypes.POINTER(_P)]),
    "atm_read_lut": (ctypes.c_int, [_P, _I32, _P, _P]),
    "atm_load_lut": (ctypes.c_int, [_P, _I32, _P, _P]),
    "atm_read_sample_counter": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.c_uint64), _P]),
    "atm_check": (ctypes.c_int, [_P, _P]),
    "atm_sky_pixels": (ctypes.c_int, [_P, _I32, _P, ctypes.POINTER(AtmImage), _D, _D, c_double3, c_double3, _D,
                                      c_double9, _D, ctypes.POINTER(AtmSurrogate), _P]),
    "atm_batch_create": (
        ctypes.c_int,
        [ctypes.POINTER(AtmParams), ctypes.POINTER(ctypes.c_double), _I32, c_double3, _D, ctypes.POINTER(_P), _P],
    ),
    "atm_batch_destroy": (ctypes.c_int, [_P]),
    "atm_batch_build": (
        ctypes.c_int,
        [_P, ctypes.POINTER(AtmBatchJob), _I32, _P, ctypes.c_int64, ctypes.POINTER(AtmBatchTuning), _P],
    ),
    "atm_batch_read_samples": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.c_uint64), _P]),
    "atm_batch_static_lut": (ctypes.c_int, [_P, _I32, _I32, ctypes.POINTER(_P)]),
    "atm_mlp_create": (ctypes.c_int, [_I32, _I32, _I32, ctypes.c_uint64, ctypes.POINTER(_P)]),
    "atm_mlp_destroy": (ctypes.c_int, [_P]),
    "atm_mlp_info": (ctypes.c_int, [_P, ctypes.POINTER(_I32), ctypes.POINTER(_P)]),
    "atm_mlp_reset_optimizer": (ctypes.c_int, [_P, _P]),
    "atm_mlp_get_params": (ctypes.c_int, [_P, _P, _P]),
    "atm_mlp_set_params": (ctypes.c_int, [_P, _P, _P]),
    "atm_mlp_gradient": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int64, _P, _P, _P]),
    "atm_mlp_train_step": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int64, ctypes.c_float, ctypes.c_float,
                                          ctypes.c_float, ctypes.c_float, _P, _P]),
    "atm_mlp_pack_bf16": (ctypes.c_int, [_P, _P]),
    "atm_mlp_forward": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, _I32, _P]),
    "atm_surrogate_samples": (ctypes.c_int, [_P, _I32, ctypes.c_int64, ctypes.c_uint64,
                                             ctypes.POINTER(AtmSampleOptions), ctypes.c_double * 4, _P, _P, _P]),
    "atm_composite_surrogate": (
        ctypes.c_int,
        [_P, _P, _P, _P, _P, _P, ctypes.POINTER(AtmImage), _D, _D, c_double3, c_double3, c_double3, _D, c_double9,
         _D, _D, _D, ctypes.POINTER(AtmSurrogate), _P],
    ),
    "atm_post_create": (ctypes.c_int, [ctypes.POINTER(AtmPostConfig), _I32, _I32, ctypes.POINTER(_P)]),
    "atm_post_destroy": (ctypes.c_int, [_P]),
    "atm_post_process": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(AtmImage), _D, _I32, _I32, _P]),
    "atm_post_read_bloom": (ctypes.c_int, [_P, ctypes.POINTER(_I32), _P, _P]),
    "atm_shade_surface": (ctypes.c_int, [ctypes.POINTER(AtmShadeParams), ctypes.POINTER(AtmShadeImages),
                                         ctypes.POINTER(AtmImage), _P]),
    "atm_render_frame": (
        ctypes.c_int,
        [_P, ctypes.POINTER(AtmShadeParams), ctypes.POINTER(AtmShadeImages), _P, _P, ctypes.POINTER(AtmImage), _D, _D,
         c_double3, c_double3, c_double3, _D, c_double9, _D, _D, _D, ctypes.POINTER(AtmSurrogate), _P],
    ),
    "atm_raster_create": (ctypes.c_int, [_I32, _I32, _I32, _I32, ctypes.POINTER(_P)]),
    "atm_raster_destroy": (ctypes.c_int, [_P]),
    "atm_raster_terrain": (ctypes.c_int, [_P, ctypes.POINTER(AtmRasterMesh), _D, _D, _I32,
                                          ctypes.POINTER(AtmRasterOutputs), ctypes.POINTER(AtmImage), _P]),
    "atm_raster_emitted": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64), _P]),
    "atm_ocean_create": (ctypes.c_int, [ctypes.POINTER(AtmOceanConfig), ctypes.POINTER(_P)]),
    "atm_ocean_destroy": (ctypes.c_int, [_P]),
    "atm_ocean_rasterize": (ctypes.c_int, [_P, ctypes.POINTER(AtmOceanImages), ctypes.POINTER(AtmImage), _D, _D,
                                           c_double9, c_double9, _D, _D, _I32, _P]),
    "atm_ocean_read_spectrum": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "atm_composite_noalloc": (
        ctypes.c_int,
        [ctypes.POINTER(AtmParams), _P, _P, _P, _P, _P, _P, _P, _P, ctypes.POINTER(AtmImage), _D, _D, _D, c_double3,
         c_double3, c_double3, _D, c_double9, _D, _D, _D, _P, _P],
    ),
}

_LIB: ctypes.CDLL | None = None


def library() -> ctypes.CDLL:
    """Load libplanet_atm.so (raises RuntimeError if it is not built)."""

    global _LIB
    if _LIB is not None:
        return _LIB
    path = Path(os.environ.get("PLANET_ATM_LIBRARY", LIBRARY_PATH))
    if not path.exists():
        raise RuntimeError(
            f"libplanet_atm.so not found at {path}; build it with "
            "`python planet-real-time-render_gb300/build_native.py` (needs nvcc)"
        )
    lib = ctypes.CDLL(str(path))
    for name, (restype, argtypes) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _LIB = lib
    return lib


class AtmError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{message} (code {code})")
        self.code = code


def check(rc: int) -> None:
    """Raise on a non-zero return code: ValueError for invalid arguments."""

    if rc == ATM_OK:
        return
    message = (library().atm_last_error() or b"").decode(errors="replace")
    if rc == ATM_E_INVALID:
        raise ValueError(message)
    raise AtmError(rc, message)


def d3(values) -> ctypes.Array:
    return c_double3(*[float(v) for v in values])


def d9(basis) -> ctypes.Array:
    flat = [float(v) for vec in basis for v in vec]
    if len(flat) != 9:
        raise ValueError("view_basis must be three 3-vectors (right, up, forward)")
    return c_double9(*flat)
