"""Seeded synthetic G-buffer for the full-frame workloads.

Stands in for the reference's terrain raster + ocean passes (the G-buffer
producers of ``renderer.py:1603-1663``, which are not part of this package):
each pixel's camera ray is intersected with a sphere of radius ``R``
displaced by a seeded 6-octave fBm height field of +/- ``amplitude_m``; rays
that miss are sky pixels (``surface_id = -1``).  Output tensors use the
Taichi field layout ``(W, H, ...)`` of the reference's G-buffer fields:

* ``position_view``  (W, H, 3) f32 - hit position in view space
  (right, up, forward), as ``gbuffer_position`` (``renderer.py:1150``);
* ``surface_id``     (W, H)    i32 - 0 surface, -1 sky;
* ``scene_hdr``      (W, H, 3) f32 - a lit albedo standing in for
  ``surface_hdr``;
* ``space_hdr``      (W, H, 3) f32 - sparse seeded stars.

Works on any torch device; the search runs in float32 with the
cancellation-free altitude form so an Earth-radius sphere resolves metres.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

_MASK32 = 0xFFFFFFFF


def _hash3(ix: torch.Tensor, iy: torch.Tensor, iz: torch.Tensor, seed: int) -> torch.Tensor:
    """32-bit integer hash of lattice points -> uniform floats in [-1, 1]."""

    h = (ix * 0x8DA6B343) ^ (iy * 0xD8163841) ^ (iz * 0xCB1AB31F) ^ (seed * 0x9E3779B1)
    h = h & _MASK32
    h = h ^ (h >> 15)
    h = (h * 0x2C1B3C6D) & _MASK32
    h = h ^ (h >> 12)
    h = (h * 0x297A2D39) & _MASK32
    h = h ^ (h >> 15)
    return (h.to(torch.float32) / float(_MASK32)) * 2.0 - 1.0


def _value_noise(p: torch.Tensor, seed: int) -> torch.Tensor:
    """Trilinear value noise with smoothstep fade; p is (..., 3) float32."""

    cell = torch.floor(p)
    f = p - cell
    s = f * f * (3.0 - 2.0 * f)
    i = cell.to(torch.int64)
    ix, iy, iz = i[..., 0], i[..., 1], i[..., 2]
    sx, sy, sz = s[..., 0], s[..., 1], s[..., 2]
    result = torch.zeros_like(sx)
    for dx in (0, 1):
        wx = sx if dx else 1.0 - sx
        for dy in (0, 1):
            wy = sy if dy else 1.0 - sy
            for dz in (0, 1):
                wz = sz if dz else 1.0 - sz
                result = result + wx * wy * wz * _hash3(ix + dx, iy + dy, iz + dz, seed)
    return result


@dataclass(frozen=True)
class Terrain:
    """fBm height field on the unit sphere: height(n) in [-amplitude, amplitude]."""

    seed: int = 2027
    octaves: int = 6
    amplitude_m: float = 4_000.0
    base_frequency: float = 64.0
    offset: tuple[float, float, float] = (0.0, 0.0, 0.0)

    def height(self, unit: torch.Tensor) -> torch.Tensor:
        offset = torch.tensor(self.offset, dtype=torch.float32, device=unit.device)
        total = torch.zeros(unit.shape[:-1], dtype=torch.float32, device=unit.device)
        norm = 0.0
        amp = 1.0
        freq = self.base_frequency
        for octave in range(self.octaves):
            total = total + amp * _value_noise(unit * freq + offset * (octave + 1), self.seed + octave)
            norm += amp
            amp *= 0.5
            freq *= 2.0
        return (total / norm) * self.amplitude_m


def terrain_below(camera_altitude_m: float, seed: int = 2027, amplitude_m: float = 4_000.0,
                  clearance_m: float = 300.0) -> Terrain:
    """A terrain whose height under the camera is at least ``clearance_m``
    below it (the camera sits on the +y axis of the planet frame); the noise
    domain offset is drawn from ``seed`` until that holds."""

    rng = np.random.default_rng(seed)
    nadir = torch.tensor([[0.0, 1.0, 0.0]], dtype=torch.float32)
    terrain = Terrain(seed=seed, amplitude_m=amplitude_m)
    for _ in range(256):
        if float(terrain.height(nadir)[0]) < camera_altitude_m - clearance_m:
            return terrain
        offset = tuple(float(v) for v in rng.uniform(-1000.0, 1000.0, 3))
        terrain = Terrain(seed=seed, amplitude_m=amplitude_m, offset=offset)
    return terrain


def _shell_roots(h0: float, cosv: torch.Tensor, shell: float, radius: float):
    """Stable ray/sphere roots for a ray from altitude h0 (float64)."""

    orad = radius + h0
    hl = orad * cosv
    c = (h0 - shell) * (2.0 * radius + h0 + shell)
    disc = hl * hl - c
    hit = disc >= 0.0
    root = torch.sqrt(torch.clamp(disc, min=0.0))
    sign = torch.where(hl < 0.0, -1.0, 1.0)
    q = -hl - sign * root
    safe_q = torch.where(q.abs() > 1e-12, q, torch.ones_like(q))
    r0 = torch.where(q.abs() > 1e-12, q, -hl - root)
    r1 = torch.where(q.abs() > 1e-12, c / safe_q, -hl + root)
    return torch.minimum(r0, r1), torch.maximum(r0, r1), hit


def pixel_rays(width: int, height: int, basis, tangent_half_fov: float, xs: torch.Tensor, ys: torch.Tensor):
    """Camera rays (float64, local EUN) of pixels (xs, ys), as the composite
    builds them (reference ``atmosphere/renderer.py:1850-1859``)."""

    right, up, forward = (torch.as_tensor(v, dtype=torch.float64, device=xs.device) for v in basis)
    aspect = width / height
    su = (xs.to(torch.float64) + 0.5) / width
    sv = (ys.to(torch.float64) + 0.5) / height
    sx = (su * 2.0 - 1.0) * aspect
    sy = sv * 2.0 - 1.0
    rays = right * sx[:, None] + up * sy[:, None] + forward / tangent_half_fov
    return rays / torch.linalg.norm(rays, dim=1, keepdim=True)


def _march(terrain: Terrain, radius: float, cam_alt: float, rays: torch.Tensor, steps: int = 96,
           bisections: int = 28) -> tuple[torch.Tensor, torch.Tensor]:
    """Distance to the first terrain crossing along each ray, and a hit mask."""

    amp = terrain.amplitude_m
    cosv = rays[:, 1]
    outer_n, outer_f, outer_hit = _shell_roots(cam_alt, cosv, amp, radius)
    inner_n, _, inner_hit = _shell_roots(cam_alt, cosv, -amp, radius)
    t0 = torch.clamp(outer_n, min=0.0)
    t1 = torch.where(inner_hit & (inner_n > 0.0), inner_n, outer_f)
    valid = outer_hit & (t1 > t0)
    t0 = torch.where(valid, t0, torch.zeros_like(t0))
    t1 = torch.where(valid, t1, torch.ones_like(t1))

    rays32 = rays.to(torch.float32)
    cos32 = rays32[:, 1]
    cam_center = torch.tensor([0.0, radius + cam_alt, 0.0], dtype=torch.float64, device=rays.device)

    def signed(t: torch.Tensor) -> torch.Tensor:
        # altitude along the ray without subtracting Earth-scale radii
        a = cam_alt
        delta = a * (2.0 * radius + a) + 2.0 * (radius + a) * cosv * t + t * t
        alt = delta / (torch.sqrt(torch.clamp(radius * radius + delta, min=0.0)) + radius)
        point = cam_center + rays * t[:, None]
        unit = (point / torch.linalg.norm(point, dim=1, keepdim=True)).to(torch.float32)
        return alt - terrain.height(unit).to(torch.float64)

    del rays32, cos32
    prev_t = t0.clone()
    prev_f = signed(prev_t)
    lo = torch.full_like(t0, float("nan"))
    hi = torch.full_like(t0, float("nan"))
    found = torch.zeros_like(valid)
    for k in range(1, steps + 1):
        frac = (k / steps) ** 2
        t = t0 + (t1 - t0) * frac
        f = signed(t)
        crossing = valid & ~found & (prev_f > 0.0) & (f <= 0.0)
        lo = torch.where(crossing, prev_t, lo)
        hi = torch.where(crossing, t, hi)
        found = found | crossing
        prev_t, prev_f = t, f
    lo = torch.where(found, lo, t0)
    hi = torch.where(found, hi, t1)
    for _ in range(bisections):
        mid = 0.5 * (lo + hi)
        above = signed(mid) > 0.0
        lo = torch.where(above, mid, lo)
        hi = torch.where(above, hi, mid)
    return hi, found


def synthesize_gbuffer(width: int, height: int, planet_radius_m: float, camera_altitude_m: float, basis,
                       tangent_half_fov: float, sun_local, solar_irradiance=(4.0, 3.9, 3.7), seed: int = 2027,
                       terrain: Terrain | None = None, pixels: torch.Tensor | None = None,
                       device: str | torch.device = "cpu", chunk: int = 1 << 20) -> dict[str, torch.Tensor]:
    """Build the G-buffer of one camera.

    ``pixels`` (n, 2) int64 selects pixel coordinates (x, y); the outputs are
    then (n, ...) instead of (W, H, ...).
    """

    device = torch.device(device)
    if terrain is None:
        terrain = terrain_below(camera_altitude_m, seed=seed)
    if pixels is None:
        xs = torch.arange(width, device=device).repeat_interleave(height)
        ys = torch.arange(height, device=device).repeat(width)
    else:
        pixels = torch.as_tensor(pixels, device=device, dtype=torch.int64)
        xs, ys = pixels[:, 0], pixels[:, 1]
    n = xs.numel()
    position = torch.zeros(n, 3, dtype=torch.float32, device=device)
    surface = torch.full((n,), -1, dtype=torch.int32, device=device)
    scene = torch.zeros(n, 3, dtype=torch.float32, device=device)
    right, up, forward = (torch.as_tensor(v, dtype=torch.float64, device=device) for v in basis)
    sun = torch.as_tensor(np.asarray(sun_local, dtype=np.float64), device=device)
    sun = sun / torch.linalg.norm(sun)
    albedo = torch.tensor([0.16, 0.20, 0.12], dtype=torch.float64, device=device)
    irradiance = torch.as_tensor(solar_irradiance, dtype=torch.float64, device=device)
    cam_center = torch.tensor([0.0, planet_radius_m + camera_altitude_m, 0.0], dtype=torch.float64, device=device)
    for begin in range(0, n, chunk):
        end = min(begin + chunk, n)
        rays = pixel_rays(width, height, basis, tangent_half_fov, xs[begin:end], ys[begin:end])
        t, hit = _march(terrain, planet_radius_m, camera_altitude_m, rays)
        local = rays * t[:, None]
        view = torch.stack([local @ right, local @ up, local @ forward], dim=1)
        position[begin:end] = torch.where(hit[:, None], view, torch.zeros_like(view)).to(torch.float32)
        surface[begin:end] = torch.where(hit, 0, -1).to(torch.int32)
        normal = cam_center + local
        normal = normal / torch.linalg.norm(normal, dim=1, keepdim=True)
        lambert = torch.clamp(normal @ sun, min=0.0) + 0.05
        lit = albedo * irradiance / math.pi * lambert[:, None]
        scene[begin:end] = torch.where(hit[:, None], lit, torch.zeros_like(lit)).to(torch.float32)
    # sparse stars: about 1% of pixels, radiance 0.02..0.3
    star_u = (_hash3(xs, ys, torch.zeros_like(xs), seed + 911) + 1.0) * 0.5
    star_l = 0.02 + 0.28 * (_hash3(xs, ys, torch.ones_like(xs), seed + 913) + 1.0) * 0.5
    star = torch.where(star_u < 0.01, star_l, torch.zeros_like(star_l))
    space = torch.stack([star, star * 0.95, star * 1.05], dim=1).to(torch.float32)
    out = {"position_view": position, "surface_id": surface, "scene_hdr": scene, "space_hdr": space}
    if pixels is None:
        out = {k: v.reshape((width, height) + tuple(v.shape[1:])) for k, v in out.items()}
    return out


def shading_inputs(gbuffer: dict, planet_radius_m: float, camera_altitude_m: float, basis,
                   ocean_surface_id: int = 2_147_000_000) -> dict[str, torch.Tensor]:
    """Land-and-ocean surface-shading inputs for a G-buffer of
    :func:`synthesize_gbuffer` (the images ``shading.shade_surface`` reads
    besides the surface lighting).  The global frame is the camera's local
    frame.  The sea level is the median radius of the frame's hits: hits
    below it are ocean (``ocean_surface_id``; water depth = how far below),
    the rest land, so about half the surface takes the ocean BRDF.  Normals
    are radial; the terrain snapshot is the hit surface itself.  A timing
    and fusion workload, not a terrain model."""

    pos = gbuffer["position_view"]
    sid = gbuffer["surface_id"]
    device = pos.device
    right, up, forward = (torch.as_tensor(v, dtype=torch.float32, device=device) for v in basis)
    local = pos[..., 0:1] * right + pos[..., 1:2] * up + pos[..., 2:3] * forward
    local[..., 1] += float(planet_radius_m + camera_altitude_m)
    radius = torch.linalg.norm(local.double(), dim=-1)
    normal = (local.double() / radius[..., None].clamp_min(1.0)).float()
    hit = sid >= 0
    sea = torch.median(radius[hit]) if bool(hit.any()) else torch.tensor(float(planet_radius_m), device=device)
    depth = (sea - radius).float().clamp_min(0.0)
    ocean = hit & (depth > 0.0)
    one = torch.ones_like(pos[..., :1])
    land_albedo = torch.tensor([0.16, 0.20, 0.12], device=device) * one
    ocean_albedo = torch.tensor([0.02, 0.05, 0.08], device=device) * one
    albedo = torch.where(ocean[..., None], ocean_albedo, land_albedo)
    surface_id = torch.where(ocean, torch.full_like(sid, ocean_surface_id), sid)
    return {
        "position": pos, "normal": normal, "albedo": albedo,
        "water_depth": torch.where(ocean, depth, torch.zeros_like(depth)).contiguous(),
        "seabed_albedo": torch.tensor([0.30, 0.28, 0.20], device=device) * one, "seabed_normal": normal,
        "slope_variance": torch.full_like(depth, 0.01), "surface_id": surface_id.contiguous(),
        "terrain_position": pos, "terrain_normal": normal, "terrain_albedo": land_albedo.contiguous(),
        "terrain_surface_id": torch.where(hit, torch.zeros_like(sid), sid).contiguous(),
    }
