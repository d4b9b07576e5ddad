"""FP64 numpy quadrature of the atmosphere model - TEST INFRASTRUCTURE.

Restates the reference's double-precision validation model
``src/planet_renderer/atmosphere/model.py`` (ray-sphere roots :38-55, shell
interval :90-119, density :68-80, extinction :82-88, uniform-midpoint
transmittance :121-143, phases :145-157, direct single scattering with a
point sun and opaque ground :159-213), vectorised over rays, plus converged
quadratures used to state the error of the FP32 LUTs:

* ``transmittance_lut_converged``: every texel ray of the transmittance LUT
  (the reference's distance parameterisation, renderer.py:410-432) integrated
  with ``steps`` uniform midpoint steps in float64.

Used only by tests as a checker.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class RayInterval:
    start_m: float
    end_m: float
    ends_at_ground: bool = False


def _unit(v) -> np.ndarray:
    v = np.asarray(v, dtype=np.float64)
    n = float(np.linalg.norm(v))
    if v.shape != (3,) or not np.isfinite(v).all() or n <= 1.0e-15:
        raise ValueError("directions must be finite non-zero 3-vectors")
    return v / n


def ray_sphere_roots(origin, direction, radius_m):
    """Ordered ray parameters of a planet-centred sphere, or None (model.py:38-55)."""

    p = np.asarray(origin, dtype=np.float64)
    d = _unit(direction)
    b = float(p @ d)
    disc = b * b - (float(p @ p) - radius_m * radius_m)
    if disc < -1.0e-12 * max(radius_m * radius_m, 1.0):
        return None
    root = math.sqrt(max(disc, 0.0))
    return -b - root, -b + root


class AtmosphereModelFP64:
    def __init__(self, planet_radius_m: float, config):
        if not math.isfinite(planet_radius_m) or planet_radius_m <= 1.0:
            raise ValueError("planet radius must be positive and finite")
        self.R = float(planet_radius_m)
        self.top = self.R + config.top_altitude_m
        self.c = config
        self.beta_r = np.asarray(config.rayleigh_scattering_per_m, dtype=np.float64)
        self.beta_ms = np.asarray(config.mie_scattering_per_m, dtype=np.float64)
        self.beta_me = np.asarray(config.mie_extinction_per_m, dtype=np.float64)
        self.beta_o = np.asarray(config.absorption_extinction_per_m, dtype=np.float64)

    # -- profiles ------------------------------------------------------------
    def density(self, h):
        """(rayleigh, mie, ozone) densities; zero outside [0, top] (vectorised)."""

        h = np.asarray(h, dtype=np.float64)
        c = self.c
        hc = np.clip(h, 0.0, c.top_altitude_m)
        inside = (h >= 0.0) & (h <= c.top_altitude_m)
        r = np.where(inside, np.exp(-hc / c.rayleigh_scale_height_m), 0.0)
        m = np.where(inside, np.exp(-hc / c.mie_scale_height_m), 0.0)
        o = np.where(inside, np.maximum(1.0 - np.abs(hc - c.absorption_peak_altitude_m) /
                                        c.absorption_half_width_m, 0.0), 0.0)
        return r, m, o

    def extinction(self, h):
        r, m, o = self.density(h)
        return (np.multiply.outer(r, self.beta_r) + np.multiply.outer(m, self.beta_me) +
                np.multiply.outer(o, self.beta_o))

    # -- geometry --------------------------------------------------------------
    def atmosphere_interval(self, origin, direction, maximum_distance_m=math.inf):
        p = np.asarray(origin, dtype=np.float64)
        d = _unit(direction)
        outer = ray_sphere_roots(p, d, self.top)
        if outer is None or outer[1] <= 0.0:
            return None
        start = max(outer[0], 0.0)
        end = min(outer[1], float(maximum_distance_m))
        ground = ray_sphere_roots(p, d, self.R)
        at_ground = False
        if ground is not None:
            eps = max(1.0e-6, self.R * 1.0e-12)
            hits = [t for t in ground if t > start + eps]
            if hits and min(hits) < end:
                end = min(hits)
                at_ground = True
        if end <= start:
            return None
        return RayInterval(start, end, at_ground)

    # -- transport ---------------------------------------------------------------
    def transmittance(self, origin, direction, maximum_distance_m=math.inf, steps=128, ground_is_opaque=False):
        interval = self.atmosphere_interval(origin, direction, maximum_distance_m)
        if interval is None:
            return np.ones(3)
        if ground_is_opaque and interval.ends_at_ground:
            return np.zeros(3)
        d = _unit(direction)
        p = np.asarray(origin, dtype=np.float64)
        n = max(int(steps), 1)
        step = (interval.end_m - interval.start_m) / n
        t = interval.start_m + (np.arange(n) + 0.5) * step
        pts = p[None, :] + t[:, None] * d[None, :]
        h = np.linalg.norm(pts, axis=1) - self.R
        tau = self.extinction(h).sum(axis=0) * step
        return np.exp(-np.minimum(tau, 80.0))

    @staticmethod
    def rayleigh_phase(c):
        return 3.0 * (1.0 + c * c) / (16.0 * math.pi)

    def mie_phase(self, c):
        g = self.c.mie_phase_g
        den = max(1.0 + g * g - 2.0 * g * c, 1.0e-8)
        return 3.0 * (1.0 - g * g) * (1.0 + c * c) / (8.0 * math.pi * (2.0 + g * g) * den ** 1.5)

    def single_scattering(self, origin, view, sun, irradiance, steps=64, sun_steps=64):
        interval = self.atmosphere_interval(origin, view)
        if interval is None:
            return np.zeros(3)
        v = _unit(view)
        s = _unit(sun)
        p0 = np.asarray(origin, dtype=np.float64)
        n = max(int(steps), 1)
        step = (interval.end_m - interval.start_m) / n
        cosv = float(np.clip(v @ s, -1.0, 1.0))
        pr, pm = self.rayleigh_phase(cosv), self.mie_phase(cosv)
        E = np.asarray(irradiance, dtype=np.float64)
        view_t = np.ones(3)
        radiance = np.zeros(3)
        for k in range(n):
            t = interval.start_m + (k + 0.5) * step
            point = p0 + v * t
            h = float(np.linalg.norm(point) - self.R)
            r, m, _ = (float(x) for x in self.density(h))
            sun_t = self.transmittance(point, s, steps=sun_steps, ground_is_opaque=True)
            source = E * sun_t * (self.beta_r * r * pr + self.beta_ms * m * pm)
            ext = self.extinction(h)
            seg_t = np.exp(-np.minimum(ext * step, 80.0))
            integral = np.where(ext > 1.0e-12, (1.0 - seg_t) / np.maximum(ext, 1e-300), step)
            radiance += view_t * source * integral
            view_t *= seg_t
        return np.maximum(radiance, 0.0)

    # -- converged references for the FP32 LUTs -------------------------------------
    def transmittance_lut_rays(self, width, height):
        """Texel rays of the transmittance LUT in float64 (renderer.py:410-432):
        returns altitude, cosine and length of each texel's ray, shape (W, H)."""

        top_h = self.c.top_altitude_m
        R = self.R
        u = (np.arange(width) + 0.5) / width
        v = (np.arange(height) + 0.5) / height
        U, V = np.meshgrid(u, v, indexing="ij")
        sh = math.sqrt(top_h * (2.0 * R + top_h))
        rho = sh * V
        h = rho * rho / (np.sqrt(rho * rho + R * R) + R)
        dmin = top_h - h
        dmax = rho + sh
        dist = dmin + U * (dmax - dmin)
        cos = np.where(dist > 1e-6, ((top_h - h) * (2.0 * R + top_h + h) - dist * dist) /
                       (2.0 * (R + h) * np.maximum(dist, 1e-300)), 1.0)
        return h, np.clip(cos, -1.0, 1.0), dist

    def transmittance_lut_converged(self, width, height, steps=4096, chunk=16):
        """Transmittance of every texel ray, ``steps`` uniform midpoints (W, H, 3)."""

        h, cos, dist = self.transmittance_lut_rays(width, height)
        R = self.R
        out = np.empty((width, height, 3))
        frac = (np.arange(steps) + 0.5) / steps
        for x0 in range(0, width, chunk):
            hh, cc, dd = h[x0:x0 + chunk], cos[x0:x0 + chunk], dist[x0:x0 + chunk]
            t = dd[..., None] * frac  # (w, H, steps)
            a = hh[..., None]
            # altitude along the ray without cancellation: |p|^2 - R^2 = a(2R+a) + 2(R+a) cos t + t^2
            delta = a * (2.0 * R + a) + 2.0 * (R + a) * cc[..., None] * t + t * t
            alt = delta / (np.sqrt(R * R + delta) + R)
            r, m, o = self.density(alt)
            step = (dd / steps)[..., None]
            tau = np.stack([(r * b + m * bm + o * bo) * step for b, bm, bo in
                            zip(self.beta_r, self.beta_me, self.beta_o)], axis=-1).sum(axis=2)
            out[x0:x0 + chunk] = np.exp(-np.minimum(tau, 80.0))
        return out
