"""Drop-in ``AtmosphereRenderer`` backed by the sm_103a kernels of libplanet_atm.

Same constructor, methods, arguments and public attributes as the reference's
Taichi class (``src/planet_renderer/atmosphere/renderer.py:42-2238``):

* ``update``, ``prepare_frame``, ``composite``, ``set_luts_frozen`` - the cache
  keys, float rounding points and rebuild counters are implemented natively
  (``atm_update`` & co. in the C ABI) and behave as the reference's;
* ``transmittance_lut``, ``multi_scattering_lut``, ``sky_view_lut`` and
  ``aerial_scattering_lut`` expose ``to_numpy()`` in the Taichi field layout
  ``(W, H[, D], 3)``, like the reference's ``ti.Vector.field`` objects;
* ``surface_sun_transmittance`` / ``surface_sky_radiance`` are renderer-owned
  CUDA tensors of the frame layout.

Images are torch CUDA float32 tensors shaped ``(W, H, 3|4)`` - the layout of the
reference's fields - or ``(H, W, 3|4)`` when the renderer is created with
``layout="hw"``; ``surface_id`` is int32 ``(W, H)`` / ``(H, W)``.  Work is
enqueued on the current torch CUDA stream and never synchronises the host.
There is no CPU path: without the native library the constructor raises.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from .. import _native
from .config import AtmosphereConfig
from .diagnostics import AtmosphereDiagnosticView

_KINDS = {
    "transmittance": _native.LUT_TRANSMITTANCE,
    "multi_scattering": _native.LUT_MULTI_SCATTERING,
    "sky_view": _native.LUT_SKY_VIEW,
    "aerial": _native.LUT_AERIAL,
}


def _stream_handle(device: torch.device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class LutField:
    """One LUT of a renderer, readable like the reference's Taichi field."""

    def __init__(self, renderer: "AtmosphereRenderer", kind: int):
        self._renderer = renderer
        self.kind = kind
        dims = (ctypes.c_int32 * 3)()
        ptr = ctypes.c_void_p()
        _native.check(renderer._lib.atm_lut_info(renderer._handle, kind, dims, ctypes.byref(ptr)))
        self.dims = tuple(int(v) for v in dims)
        self.device_ptr = int(ptr.value or 0)

    @property
    def shape(self) -> tuple[int, ...]:
        w, h, d = self.dims
        return (w, h) if kind_is_2d(self.kind) else (w, h, d)

    def to_torch(self) -> torch.Tensor:
        """Copy into a new CUDA tensor of shape ``shape + (3,)``."""

        r = self._renderer
        out = torch.empty(self.shape + (3,), dtype=torch.float32, device=r.device)
        _native.check(r._lib.atm_read_lut(r._handle, self.kind, ctypes.c_void_p(out.data_ptr()),
                                          _stream_handle(r.device)))
        return out

    def to_numpy(self) -> np.ndarray:
        return self.to_torch().cpu().numpy()

    def from_torch(self, values: torch.Tensor) -> None:
        r = self._renderer
        src = values.to(device=r.device, dtype=torch.float32).contiguous()
        if tuple(src.shape) != self.shape + (3,):
            raise ValueError(f"expected shape {self.shape + (3,)}, got {tuple(src.shape)}")
        _native.check(r._lib.atm_load_lut(r._handle, self.kind, ctypes.c_void_p(src.data_ptr()),
                                          _stream_handle(r.device)))
        torch.cuda.current_stream(r.device).synchronize()

    def from_numpy(self, values: np.ndarray) -> None:
        self.from_torch(torch.as_tensor(np.asarray(values, dtype=np.float32)))


def kind_is_2d(kind: int) -> bool:
    return kind != _native.LUT_AERIAL


class AtmosphereRenderer:
    """Spherical Rayleigh/Mie/ozone atmosphere through GPU LUTs (GB300).

    LUT geometry is planet-centred; the composite reconstructs rays in the
    camera's local East-Up-North frame with the camera at the origin and the
    planet centre at ``(0, -camera_radius, 0)``.
    """

    def __init__(self, width: int, height: int, config: AtmosphereConfig, device=None, layout: str = "wh"):
        if layout not in ("wh", "hw"):
            raise ValueError("layout must be 'wh' (Taichi field layout) or 'hw'")
        self._lib = _native.library()
        self.width = int(width)
        self.height = int(height)
        self.config = config
        self.layout = layout
        self.device = torch.device(device if device is not None else f"cuda:{torch.cuda.current_device()}")
        if self.device.type != "cuda":
            raise ValueError("AtmosphereRenderer runs on a CUDA device only")
        torch.cuda.init()
        self._handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            params = _native.AtmParams.from_config(config)
            _native.check(self._lib.atm_create(ctypes.byref(params), self.width, self.height,
                                               ctypes.byref(self._handle)))
        self.transmittance_lut = LutField(self, _native.LUT_TRANSMITTANCE)
        self.multi_scattering_lut = LutField(self, _native.LUT_MULTI_SCATTERING)
        self.sky_view_lut = LutField(self, _native.LUT_SKY_VIEW)
        self.aerial_scattering_lut = LutField(self, _native.LUT_AERIAL)
        frame = (self.width, self.height, 3) if layout == "wh" else (self.height, self.width, 3)
        self.surface_sun_transmittance = torch.zeros(frame, dtype=torch.float32, device=self.device)
        self.surface_sky_radiance = torch.zeros(frame, dtype=torch.float32, device=self.device)

    def close(self) -> None:
        handle = getattr(self, "_handle", None)
        if handle is not None and handle.value:
            self._lib.atm_destroy(handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state (reference renderer.py:97-116) ---------------------------------
    def _state(self) -> _native.AtmState:
        s = _native.AtmState()
        _native.check(self._lib.atm_get_state(self._handle, ctypes.byref(s)))
        return s

    @property
    def luts_frozen(self) -> bool:
        return bool(self._state().luts_frozen)

    @property
    def sky_snapshot_altitude_m(self):
        s = self._state()
        return s.sky_snapshot_altitude_m if s.has_sky_snapshot else None

    @property
    def sky_snapshot_sun_cosine(self):
        s = self._state()
        return s.sky_snapshot_sun_cosine if s.has_sky_snapshot else None

    @property
    def aerial_snapshot_altitude_m(self):
        s = self._state()
        return s.aerial_snapshot_altitude_m if s.has_aerial_snapshot else None

    @property
    def transmittance_rebuilds(self) -> int:
        return int(self._state().transmittance_rebuilds)

    @property
    def multi_scattering_rebuilds(self) -> int:
        return int(self._state().multi_scattering_rebuilds)

    @property
    def sky_view_rebuilds(self) -> int:
        return int(self._state().sky_view_rebuilds)

    @property
    def aerial_rebuilds(self) -> int:
        return int(self._state().aerial_rebuilds)

    # ---- images ------------------------------------------------------------
    def _image(self, floats: list[torch.Tensor], ids: torch.Tensor | None) -> _native.AtmImage:
        img = None
        for t in floats:
            if not isinstance(t, torch.Tensor) or t.device != self.device or t.dtype != torch.float32:
                raise ValueError("images must be float32 CUDA tensors on the renderer's device")
            if t.dim() != 3 or t.shape[2] not in (3, 4) or t.stride(2) != 1:
                raise ValueError("images must have shape (W, H, 3|4) with contiguous channels")
            c = int(t.shape[2])
            if t.stride(0) % c or t.stride(1) % c:
                raise ValueError("image strides must be whole pixels")
            if self.layout == "wh":
                dims, sx, sy = (t.shape[0], t.shape[1]), t.stride(0) // c, t.stride(1) // c
            else:
                dims, sx, sy = (t.shape[1], t.shape[0]), t.stride(1) // c, t.stride(0) // c
            this = (int(dims[0]), int(dims[1]), int(sx), int(sy), c)
            if img is None:
                img = this
            elif this != img:
                raise ValueError("all images of one call must share shape, strides and channels")
        if ids is None:  # a call without a G-buffer
            return _native.AtmImage(img[0], img[1], img[2], img[3], img[4])
        if not isinstance(ids, torch.Tensor) or ids.device != self.device or ids.dtype != torch.int32:
            raise ValueError("surface_id must be an int32 CUDA tensor on the renderer's device")
        id_strides = (ids.stride(0), ids.stride(1)) if self.layout == "wh" else (ids.stride(1), ids.stride(0))
        if ids.dim() != 2 or id_strides != (img[2], img[3]):
            raise ValueError("surface_id must match the images' pixel strides")
        return _native.AtmImage(img[0], img[1], img[2], img[3], img[4])

    # ---- reference methods -----------------------------------------------------
    def set_luts_frozen(self, frozen: bool) -> None:
        """Freeze or resume view-dependent LUT regeneration (renderer.py:2057-2070)."""

        _native.check(self._lib.atm_set_luts_frozen(self._handle, 1 if frozen else 0))

    def update(self, planet_radius_m: float, camera_radius_m: float, sun_local, solar_irradiance,
               sun_angular_radius_degrees: float) -> None:
        """Regenerate only LUTs invalidated by atmosphere, altitude or sun state."""

        if isinstance(sun_local, np.ndarray) and sun_local.dtype == np.float64 and sun_local.shape == (3,):
            # the reference normalises a float64 array argument in place
            sun_local /= max(float(np.linalg.norm(sun_local)), 1.0e-12)
        _native.check(self._lib.atm_update(self._handle, float(planet_radius_m), float(camera_radius_m),
                                           _native.d3(sun_local), _native.d3(solar_irradiance),
                                           float(sun_angular_radius_degrees), _stream_handle(self.device)))

    def prepare_frame(self, position_view, surface_id, planet_radius_m: float, camera_radius_m: float, sun_local,
                      solar_irradiance, sun_angular_radius_degrees: float, view_basis,
                      tangent_half_fov: float) -> None:
        """Surface-lighting inputs and the aerial-perspective volume."""

        img = self._image([position_view, self.surface_sun_transmittance, self.surface_sky_radiance], surface_id)
        _native.check(self._lib.atm_prepare_frame(
            self._handle, ctypes.c_void_p(position_view.data_ptr()), ctypes.c_void_p(surface_id.data_ptr()),
            ctypes.byref(img), float(planet_radius_m), float(camera_radius_m), _native.d3(sun_local),
            _native.d3(solar_irradiance), float(sun_angular_radius_degrees), _native.d9(view_basis),
            float(tangent_half_fov), ctypes.c_void_p(self.surface_sun_transmittance.data_ptr()),
            ctypes.c_void_p(self.surface_sky_radiance.data_ptr()), _stream_handle(self.device)))

    def composite(self, scene_hdr, space_hdr, surface_id, position_view, hdr, planet_radius_m: float,
                  camera_radius_m: float, sun_local, solar_irradiance, sun_disk_radiance,
                  sun_angular_radius_degrees: float, view_basis, tangent_half_fov: float,
                  star_contrast_start: float, star_contrast_end: float,
                  diagnostic_view: AtmosphereDiagnosticView = AtmosphereDiagnosticView.COMPOSITE) -> None:
        """Write the atmosphere composite (or a diagnostic view) into ``hdr``."""

        img = self._image([scene_hdr, space_hdr, position_view, hdr], surface_id)
        _native.check(self._lib.atm_composite(
            self._handle, ctypes.c_void_p(scene_hdr.data_ptr()), ctypes.c_void_p(space_hdr.data_ptr()),
            ctypes.c_void_p(surface_id.data_ptr()), ctypes.c_void_p(position_view.data_ptr()),
            ctypes.c_void_p(hdr.data_ptr()), ctypes.byref(img), float(planet_radius_m), float(camera_radius_m),
            _native.d3(sun_local), _native.d3(solar_irradiance), _native.d3(sun_disk_radiance),
            float(sun_angular_radius_degrees), _native.d9(view_basis), float(tangent_half_fov),
            float(star_contrast_start), float(star_contrast_end), int(diagnostic_view),
            _stream_handle(self.device)))

    # ---- extensions ------------------------------------------------------------
    def composite_surrogate(self, scene_hdr, space_hdr, surface_id, position_view, hdr, planet_radius_m: float,
                            camera_radius_m: float, sun_local, solar_irradiance, sun_disk_radiance,
                            sun_angular_radius_degrees: float, view_basis, tangent_half_fov: float,
                            star_contrast_start: float, star_contrast_end: float, surrogate,
                            stats: torch.Tensor | None = None, check_fraction: float = 0.01,
                            seed: int = 0) -> None:
        """COMPOSITE view with the learned surrogates (``surrogate``: a
        :class:`~planet_renderer_gb300.atmosphere.surrogate.Surrogate`).  The
        plain integrator re-integrates ``check_fraction`` of the MLP pixels;
        ``stats`` (8 floats on the device, accumulated) receives their error
        and the pixel counts of each path."""

        img = self._image([scene_hdr, space_hdr, position_view, hdr], surface_id)
        if stats is not None and (stats.device != self.device or stats.dtype != torch.float32 or stats.numel() < 8):
            raise ValueError("stats must be a float32 tensor of 8 elements on the renderer's device")
        sg = surrogate.native(check_fraction=check_fraction, seed=seed,
                              stats=None if stats is None else stats.data_ptr(),
                              camera_altitude_m=float(camera_radius_m) - float(planet_radius_m))
        _native.check(self._lib.atm_composite_surrogate(
            self._handle, ctypes.c_void_p(scene_hdr.data_ptr()), ctypes.c_void_p(space_hdr.data_ptr()),
            ctypes.c_void_p(surface_id.data_ptr()), ctypes.c_void_p(position_view.data_ptr()),
            ctypes.c_void_p(hdr.data_ptr()), ctypes.byref(img), float(planet_radius_m), float(camera_radius_m),
            _native.d3(sun_local), _native.d3(solar_irradiance), _native.d3(sun_disk_radiance),
            float(sun_angular_radius_degrees), _native.d9(view_basis), float(tangent_half_fov),
            float(star_contrast_start), float(star_contrast_end), ctypes.byref(sg), _stream_handle(self.device)))

    def build_lut(self, kind: str, *, planet_radius_m: float, camera_altitude_m: float = 0.0,
                  sun_zenith_cosine: float = 1.0, sun_local=(0.0, 1.0, 0.0), solar_irradiance=(4.0, 3.9, 3.7),
                  sun_angular_radius_degrees: float = 0.266, view_basis=((1, 0, 0), (0, 1, 0), (0, 0, 1)),
                  tangent_half_fov: float = math.tan(math.radians(30.0))) -> None:
        """Rebuild one LUT from explicit inputs, bypassing cache keys and counters."""

        a = _native.AtmBuildArgs()
        a.planet_radius_m = float(planet_radius_m)
        a.camera_altitude_m = float(camera_altitude_m)
        a.sun_zenith_cosine = float(sun_zenith_cosine)
        a.sun_local[:] = [float(v) for v in sun_local]
        a.solar_irradiance[:] = [float(v) for v in solar_irradiance]
        a.sun_angular_radius_rad = math.radians(sun_angular_radius_degrees)
        a.view_basis[:] = [float(v) for vec in view_basis for v in vec]
        a.tangent_half_fov = float(tangent_half_fov)
        a.frame_width, a.frame_height = self.width, self.height
        _native.check(self._lib.atm_build_lut(self._handle, _KINDS[kind], ctypes.byref(a),
                                              _stream_handle(self.device)))

    def render_frame(self, gbuffer: dict, space_hdr, hdr, planet_radius_m: float, camera_radius_m: float,
                     sun_local, solar_irradiance, sun_disk_radiance, sun_angular_radius_degrees: float, view_basis,
                     tangent_half_fov: float, star_contrast_start: float, star_contrast_end: float, *,
                     sun_global=None, view_basis_global=None, ocean=None, shade_mode: int = 0,
                     ocean_surface_id: int | None = None, surrogate=None, stats: torch.Tensor | None = None,
                     check_fraction: float = 0.01, seed: int = 0) -> None:
        """``prepare_frame`` -> surface shading -> ``composite`` (COMPOSITE
        view) in one pass over the pixels, the surface lighting and shaded
        colour of each pixel kept in registers (``atm_render_frame``).
        ``gbuffer`` holds the shading's G-buffer and terrain-snapshot images
        (``shading.GBUFFER_IMAGES``; ``position`` and ``surface_id`` are the
        composite's ``position_view`` and ``surface_id``).  ``sun_global`` and
        ``view_basis_global`` default to the local ones (a global frame equal
        to the camera's local frame).  With ``surrogate`` the composite is
        ``composite_surrogate``'s.  The aerial volume and the public surface
        lighting images are not updated."""

        from .. import shading

        ocean = ocean or shading.OceanShading()
        names = shading.GBUFFER_IMAGES
        p, ptrs, image = shading.shade_arguments(
            gbuffer, hdr, sun_local if sun_global is None else sun_global, solar_irradiance,
            view_basis if view_basis_global is None else view_basis_global, ocean,
            math.radians(sun_angular_radius_degrees), tangent_half_fov, shade_mode, self.layout,
            shading.OCEAN_SURFACE_ID if ocean_surface_id is None else ocean_surface_id, names=names)
        img = self._image([space_hdr, hdr, gbuffer["position"]], gbuffer["surface_id"])
        if (img.width, img.height) != (image.width, image.height):
            raise ValueError("images must have the renderer's frame shape")
        sg = None
        if surrogate is not None:
            if stats is not None and (stats.device != self.device or stats.dtype != torch.float32
                                      or stats.numel() < 8):
                raise ValueError("stats must be a float32 tensor of 8 elements on the renderer's device")
            sg = surrogate.native(check_fraction=check_fraction, seed=seed,
                                  stats=None if stats is None else stats.data_ptr(),
                                  camera_altitude_m=float(camera_radius_m) - float(planet_radius_m))
        _native.check(self._lib.atm_render_frame(
            self._handle, ctypes.byref(p), ctypes.byref(ptrs), ctypes.c_void_p(space_hdr.data_ptr()),
            ctypes.c_void_p(hdr.data_ptr()), ctypes.byref(img), float(planet_radius_m), float(camera_radius_m),
            _native.d3(sun_local), _native.d3(solar_irradiance), _native.d3(sun_disk_radiance),
            float(sun_angular_radius_degrees), _native.d9(view_basis), float(tangent_half_fov),
            float(star_contrast_start), float(star_contrast_end), None if sg is None else ctypes.byref(sg),
            _stream_handle(self.device)))

    def sky_pixels(self, radiance, planet_radius_m: float, camera_radius_m: float, sun_local, solar_irradiance,
                   sun_angular_radius_degrees: float, view_basis, tangent_half_fov: float, mode: str = "plain",
                   surrogate=None, check_fraction: float = 0.01, seed: int = 0) -> None:
        """Sky radiance along every pixel's view ray into ``radiance``
        (``(W, H, 3|4)`` float32, the renderer's layout): ``mode`` "plain" the
        sky-view march per pixel, "net" the sky network of ``surrogate`` with
        the plain march where a gate trips, "lut" the sky-view LUT of the last
        ``update``.  In "net" mode with the surrogate's ``calibration_tile``
        set, a seeded ``check_fraction`` of the network pixels also take the
        plain march (and keep it), and each tile's mean log ratio of plain to
        network radiance rescales the tile's other network pixels."""

        code = {"plain": _native.ATM_SKY_PIXELS_PLAIN, "net": _native.ATM_SKY_PIXELS_NET,
                "lut": _native.ATM_SKY_PIXELS_LUT}[mode]
        img = self._image([radiance], None)
        sg = None if surrogate is None else surrogate.native(check_fraction=check_fraction, seed=seed)
        _native.check(self._lib.atm_sky_pixels(
            self._handle, code, ctypes.c_void_p(radiance.data_ptr()), ctypes.byref(img), float(planet_radius_m),
            float(camera_radius_m), _native.d3(sun_local), _native.d3(solar_irradiance),
            float(sun_angular_radius_degrees), _native.d9(view_basis), float(tangent_half_fov),
            None if sg is None else ctypes.byref(sg), _stream_handle(self.device)))

    def check(self) -> None:
        """Synchronise the stream and raise the device-side errors of earlier
        calls (``AtmError`` with ``ATM_E_TIMEOUT`` when a tensor-core wait of
        ``composite_surrogate`` gave up: those pixels took the plain
        integrator).  Clears what it reports."""

        _native.check(self._lib.atm_check(self._handle, _stream_handle(self.device)))

    def radiance_samples(self, reset: bool = False) -> int:
        """Radiance samples evaluated by composites (synchronises the stream)."""

        out = ctypes.c_uint64()
        _native.check(self._lib.atm_read_sample_counter(self._handle, 1 if reset else 0, ctypes.byref(out),
                                                        _stream_handle(self.device)))
        return int(out.value)
