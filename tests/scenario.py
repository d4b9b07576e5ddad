"""Drive a golden scenario through the oracle or through the GPU renderer.

Two modes, both producing dicts keyed like the golden fixtures:

* ``stages``: every kernel fed the reference's own upstream outputs (its
  LUTs), so each kernel is compared in isolation;
* ``chain``: the public ``update -> prepare_frame -> composite`` sequence from
  scratch, as the reference's frame scheduler calls it.

Scenarios sampled at a subset of pixels of a large frame are run on a frame
that is sky everywhere else; only the sampled pixels are compared.
"""

from __future__ import annotations

import math

import numpy as np

LUT_KEYS = ("transmittance_lut", "multi_scattering_lut", "sky_view_lut", "aerial_scattering_lut")
KINDS = ("transmittance", "multi_scattering", "sky_view", "aerial")


class Scenario:
    def __init__(self, data, meta):
        from planet_renderer_gb300.atmosphere.config import AtmosphereConfig

        self.data, self.meta = data, meta
        self.config = AtmosphereConfig(**meta["config"])
        self.W, self.H = meta["width"], meta["height"]
        self.R = meta["planet_radius_m"]
        self.cr = meta["camera_radius_m"]
        self.sun = np.array(meta["sun_local"], dtype=np.float64)
        self.E = tuple(meta["solar_irradiance"])
        self.disk = tuple(meta["sun_disk_radiance"])
        self.ar_deg = meta["sun_angular_radius_degrees"]
        self.basis = [np.array(b) for b in meta["view_basis"]]
        self.tanfov = meta["tangent_half_fov"]
        self.views = meta["views"]
        self.pixels = data["pixels"] if "pixels" in data.files else None
        self.frame = self._full_frame()

    def _full_frame(self):
        d = self.data
        if self.pixels is None:
            return {k: d[k] for k in ("position_view", "surface_id", "scene_hdr", "space_hdr")}
        W, H = self.W, self.H
        frame = {
            "position_view": np.zeros((W, H, 3), np.float32),
            "surface_id": np.full((W, H), -1, np.int32),
            "scene_hdr": np.zeros((W, H, 3), np.float32),
            "space_hdr": np.zeros((W, H, 3), np.float32),
        }
        xs, ys = self.pixels[:, 0], self.pixels[:, 1]
        for k in frame:
            frame[k][xs, ys] = d[k]
        return frame

    def select(self, image):
        """Pixels of a (W, H, ...) image that the fixture holds."""

        if self.pixels is None:
            return image
        return image[self.pixels[:, 0], self.pixels[:, 1]]

    @property
    def cam_alt(self):
        return max(self.cr - self.R, 0.0)

    @property
    def sun_cos_key(self):
        return float(np.float32(np.clip(self.sun[1] / np.linalg.norm(self.sun), -1.0, 1.0)))

    @property
    def alt_key(self):
        return float(np.float32(self.cam_alt))

    def ar_rad(self):
        return math.radians(self.ar_deg)

    def ar_key(self):
        return float(np.float32(math.radians(self.ar_deg)))


# ---- oracle -------------------------------------------------------------------
def oracle_stages(sc: Scenario, oracle) -> dict:
    d = sc.data
    out = {}
    if "transmittance_lut" in d.files:
        out["transmittance_lut"] = oracle.build_transmittance(sc.config, sc.R)
        T, M = d["transmittance_lut"], d["multi_scattering_lut"]
        out["multi_scattering_lut"] = oracle.build_multi_scattering(sc.config, sc.R, sc.E, sc.ar_key(), T)
    else:
        T = M = None
    return _oracle_view_stages(sc, oracle, out, T, M)


def _oracle_view_stages(sc, oracle, out, T, M):
    d = sc.data
    if T is None:
        return out
    out["sky_view_lut"] = oracle.build_sky_view(sc.config, sc.R, sc.alt_key, sc.sun_cos_key, sc.E, sc.ar_key(), T, M)
    out["aerial_scattering_lut"] = oracle.build_aerial(sc.config, sc.W, sc.H, sc.R, sc.cam_alt, sc.sun, sc.E,
                                                       sc.ar_rad(), sc.basis, sc.tanfov, T, M)
    f = sc.frame
    st, sky = oracle.prepare_surface(sc.config, f["position_view"], f["surface_id"], sc.R, sc.cam_alt, sc.sun,
                                     sc.ar_rad(), sc.basis, T, M)
    out["surface_sun_transmittance"] = sc.select(st)
    out["surface_sky_radiance"] = sc.select(sky)
    plist = None
    if sc.pixels is not None:
        plist = (sc.pixels[:, 0].astype(np.int64) * sc.H + sc.pixels[:, 1]).astype(np.int32)
    for v in sc.views:
        hdr, _ = oracle.composite(sc.config, f["scene_hdr"], f["space_hdr"], f["surface_id"], f["position_view"],
                                  sc.R, sc.cam_alt, sc.alt_key, sc.sun, sc.E, sc.disk, sc.ar_rad(), sc.basis,
                                  sc.tanfov, 4.0, 12.0, v, T, M, d["sky_view_lut"], d["aerial_scattering_lut"],
                                  pixel_list=plist)
        out[f"hdr_view{v}"] = sc.select(hdr)
    return out


def oracle_stages_with_luts(sc: Scenario, oracle, T, M) -> dict:
    """View-dependent stages with explicit T / MS inputs (fixtures that do not
    carry them reuse another fixture's)."""

    return _oracle_view_stages(sc, oracle, {}, T, M)


# ---- GPU ---------------------------------------------------------------------------
def _torch_frame(sc: Scenario, device):
    import torch

    return {k: torch.as_tensor(v).to(device) for k, v in sc.frame.items()}


def gpu_stages(sc: Scenario, T=None, M=None) -> dict:
    """Each kernel of the GPU renderer fed the reference's upstream LUTs."""

    import torch

    from planet_renderer_gb300.atmosphere import AtmosphereRenderer

    d = sc.data
    r = AtmosphereRenderer(sc.W, sc.H, sc.config)
    dev = r.device
    out = {}
    T = d["transmittance_lut"] if T is None and "transmittance_lut" in d.files else T
    M = d["multi_scattering_lut"] if M is None and "multi_scattering_lut" in d.files else M
    if "transmittance_lut" in d.files:
        r.build_lut("transmittance", planet_radius_m=sc.R)
        out["transmittance_lut"] = r.transmittance_lut.to_numpy()
        r.transmittance_lut.from_numpy(T)
        r.build_lut("multi_scattering", planet_radius_m=sc.R, solar_irradiance=sc.E,
                    sun_angular_radius_degrees=math.degrees(sc.ar_key()))
        out["multi_scattering_lut"] = r.multi_scattering_lut.to_numpy()
    r.transmittance_lut.from_numpy(T)
    r.multi_scattering_lut.from_numpy(M)
    r.build_lut("sky_view", planet_radius_m=sc.R, camera_altitude_m=sc.alt_key, sun_zenith_cosine=sc.sun_cos_key,
                solar_irradiance=sc.E, sun_angular_radius_degrees=math.degrees(sc.ar_key()))
    out["sky_view_lut"] = r.sky_view_lut.to_numpy()
    r.build_lut("aerial", planet_radius_m=sc.R, camera_altitude_m=sc.cam_alt, sun_local=sc.sun,
                solar_irradiance=sc.E, sun_angular_radius_degrees=sc.ar_deg, view_basis=sc.basis,
                tangent_half_fov=sc.tanfov)
    out["aerial_scattering_lut"] = r.aerial_scattering_lut.to_numpy()
    r.sky_view_lut.from_numpy(d["sky_view_lut"])
    r.aerial_scattering_lut.from_numpy(d["aerial_scattering_lut"])
    f = _torch_frame(sc, dev)
    # prepare_frame also rebuilds the aerial volume: read the surface fields only
    r.prepare_frame(f["position_view"], f["surface_id"], sc.R, sc.cr, sc.sun, sc.E, sc.ar_deg, sc.basis, sc.tanfov)
    out["surface_sun_transmittance"] = sc.select(r.surface_sun_transmittance.cpu().numpy())
    out["surface_sky_radiance"] = sc.select(r.surface_sky_radiance.cpu().numpy())
    r.aerial_scattering_lut.from_numpy(d["aerial_scattering_lut"])
    hdr = torch.zeros_like(f["scene_hdr"])
    for v in sc.views:
        hdr.zero_()
        r.composite(f["scene_hdr"], f["space_hdr"], f["surface_id"], f["position_view"], hdr, sc.R, sc.cr, sc.sun,
                    sc.E, sc.disk, sc.ar_deg, sc.basis, sc.tanfov, 4.0, 12.0, v)
        out[f"hdr_view{v}"] = sc.select(hdr.cpu().numpy())
    r.close()
    return out


def gpu_chain(sc: Scenario):
    """update -> prepare_frame -> composite through the public API."""

    import torch

    from planet_renderer_gb300.atmosphere import AtmosphereRenderer

    r = AtmosphereRenderer(sc.W, sc.H, sc.config)
    f = _torch_frame(sc, r.device)
    r.update(sc.R, sc.cr, sc.sun.copy(), sc.E, sc.ar_deg)
    r.prepare_frame(f["position_view"], f["surface_id"], sc.R, sc.cr, sc.sun, sc.E, sc.ar_deg, sc.basis, sc.tanfov)
    out = {k: getattr(r, k).to_numpy() for k in LUT_KEYS}
    out["surface_sun_transmittance"] = sc.select(r.surface_sun_transmittance.cpu().numpy())
    out["surface_sky_radiance"] = sc.select(r.surface_sky_radiance.cpu().numpy())
    hdr = torch.zeros_like(f["scene_hdr"])
    for v in sc.views:
        r.composite(f["scene_hdr"], f["space_hdr"], f["surface_id"], f["position_view"], hdr, sc.R, sc.cr, sc.sun,
                    sc.E, sc.disk, sc.ar_deg, sc.basis, sc.tanfov, 4.0, 12.0, v)
        out[f"hdr_view{v}"] = sc.select(hdr.cpu().numpy())
    return out, r
