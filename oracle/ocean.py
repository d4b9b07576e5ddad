"""CPU restatement (test infrastructure) of the reference's ocean coverage
pass, OceanRenderer (src/planet_renderer/ocean.py:193-771): the
per-frame directional wave spectrum (_build_directional_spectrum :260-337)
and the sea-level sphere's coverage of the G-buffer (_rasterize :517-684,
with _near_sphere_distance :339-362, _cascade_axes :364-381,
_sample_spectrum_texture :383-425 and _sample_spectrum :427-515), driven
as OceanRenderer.rasterize (:686-762) drives them.

numpy float32, operation by operation in the reference's order (Python
constants folded to float32 where Taichi folds them), vectorised over
texels and pixels with branches as masks; fields are (W, H[, n]) indexed
[x, y] like the reference's Taichi fields.  Used only by tests, never by
the product path."""

from __future__ import annotations

import math

import numpy as np

F = np.float32
OCEAN_SURFACE_ID = 2_147_000_000  # ocean.py:17
CASCADES = 3
PERIODS_M = (2048.0, 256.0, 32.0)  # ocean.py:19-25, the wave spectrum's table
HEIGHTS_M = (0.62, 0.14, 0.025)
MODE_X = (3, 4, 4, 5, 5, 3, 2, 1, -1, -2, -3, -4)
MODE_Y = (1, 1, 2, 1, 2, 2, 3, 4, 4, 3, 2, 1)
WEIGHTS = (1.0, 0.82, 0.72, 0.60, 0.52, 0.68, 0.55, 0.42, 0.36, 0.31, 0.27, 0.22)
PHASES = (0.31, 1.73, 3.11, 4.67, 0.93, 2.39, 5.21, 3.83, 1.17, 5.72, 2.83, 4.09)
TWO_PI = F(2.0 * math.pi)
PI = F(math.pi)


def wind_amplitude_scale(wind_speed_mps: float) -> float:
    return min(max(wind_speed_mps / 8.0, 0.25), 2.0)


def slope_variances(wave_height_scale: float, wind_speed_mps: float) -> tuple:
    """Per-cascade slope variance of the spectrum (float64, :235-258)."""

    weight_sum = sum(WEIGHTS)
    scale = wave_height_scale * wind_amplitude_scale(wind_speed_mps)
    out = []
    for period, band in zip(PERIODS_M, HEIGHTS_M):
        var = 0.0
        for mx, my, w in zip(MODE_X, MODE_Y, WEIGHTS):
            amp = band * scale * w / weight_sum
            k = 2.0 * math.pi * math.hypot(mx, my) / period
            var += 0.5 * (amp * k) ** 2
        out.append(var)
    return tuple(out)


def max_geometry_displacement(wave_height_scale, wind_speed_mps, geometry_cascades) -> float:
    return sum(HEIGHTS_M[:geometry_cascades]) * wave_height_scale * wind_amplitude_scale(wind_speed_mps)


def build_spectrum(resolution: int, time_seconds: float, amplitude_scale: float, choppiness: float):
    """_build_directional_spectrum: height (3, N, N), gradient (3, N, N, 2),
    displacement (3, N, N, 2) and displacement Jacobian (3, N, N, 4),
    indexed [cascade, x, y]."""

    n = int(resolution)
    t = F(time_seconds)
    amp_scale = F(amplitude_scale)
    chop = F(choppiness)
    weight_sum = F(float(sum(WEIGHTS)))
    idx = np.arange(n)
    X, Y = np.meshgrid(idx, idx, indexing="ij")
    u = (X.astype(F) + F(0.5)) / F(n)
    v = (Y.astype(F) + F(0.5)) / F(n)
    height = np.zeros((CASCADES, n, n), F)
    grad = np.zeros((CASCADES, n, n, 2), F)
    disp = np.zeros((CASCADES, n, n, 2), F)
    jac = np.zeros((CASCADES, n, n, 4), F)
    for c in range(CASCADES):
        period = F(PERIODS_M[c])
        h = np.zeros((n, n), F)
        g = np.zeros((n, n, 2), F)
        d = np.zeros((n, n, 2), F)
        j = np.zeros((n, n, 4), F)
        for m in range(len(MODE_X)):
            kx, ky = F(MODE_X[m]), F(MODE_Y[m])
            mode_length = np.sqrt(kx * kx + ky * ky)
            wave_number = TWO_PI * mode_length / period
            omega = np.sqrt(F(9.81) * wave_number)
            phase = TWO_PI * (kx * u + ky * v) + F(PHASES[m]) - omega * t
            amplitude = F(HEIGHTS_M[c]) * amp_scale * F(WEIGHTS[m]) / weight_sum
            cos_p, sin_p = np.cos(phase), np.sin(phase)
            h = h + amplitude * cos_p
            derivative = -amplitude * sin_p * F(2.0) * PI
            g = g + np.stack([derivative * kx / period, derivative * ky / period], -1)
            inv_len = np.maximum(mode_length, F(1.0e-6))
            direction = (kx / inv_len, ky / inv_len)
            wave_vector = (TWO_PI * kx / period, TWO_PI * ky / period)
            choppy = chop * amplitude
            s = -choppy * sin_p
            d = d + np.stack([s * direction[0], s * direction[1]], -1)
            js = -choppy * cos_p
            j = j + np.stack([js * (direction[0] * wave_vector[0]), js * (direction[0] * wave_vector[1]),
                              js * (direction[1] * wave_vector[0]), js * (direction[1] * wave_vector[1])], -1)
        height[c], grad[c], disp[c], jac[c] = h, g, d, j
    return height, grad, disp, jac


def _dot(a, b):
    acc = a[..., 0] * b[..., 0]
    for k in range(1, a.shape[-1]):
        acc = acc + a[..., k] * b[..., k]
    return acc


def _norm(a):
    return np.sqrt(_dot(a, a))


def _normalized(a):
    return (F(1.0) / (_norm(a) + F(0.0)))[..., None] * a


def _v(x):
    return np.asarray(x, F)


def near_sphere_distance(altitude, ray_cosine, radius):
    """_near_sphere_distance: the cancellation-resistant near hit (-1: none)."""

    altitude, ray_cosine, radius = (np.asarray(a, F) for a in (altitude, ray_cosine, radius))
    origin_radius = radius + altitude
    half_linear = origin_radius * ray_cosine
    constant = altitude * (F(2.0) * radius + altitude)
    disc = half_linear * half_linear - constant
    root = np.sqrt(np.maximum(disc, F(0.0)))
    q = -half_linear - np.where(half_linear >= F(0.0), root, -root)
    root0 = -half_linear - root
    root1 = -half_linear + root
    big = np.abs(q) > F(1.0e-12)
    with np.errstate(divide="ignore", invalid="ignore"):
        root0 = np.where(big, q, root0)
        root1 = np.where(big, constant / np.where(big, q, F(1.0)), root1)
    near = np.minimum(root0, root1)
    far = np.maximum(root0, root1)
    dist = np.where(near > F(0.0), near, np.where(far > F(0.0), far, F(-1.0)))
    return np.where(disc >= F(0.0), dist, F(-1.0)).astype(F)


def cascade_axes(cascade, wind_radians):
    base = (((1.0, 0.0, 0.0), (0.0, 0.0, 1.0)), ((0.0, 1.0, 0.0), (1.0, 0.0, 0.0)),
            ((0.0, 0.0, 1.0), (0.0, 1.0, 0.0)))[cascade]
    bu, bv = _v(base[0]), _v(base[1])
    w = F(wind_radians)
    c, s = np.cos(w), np.sin(w)
    return bu * c + bv * s, -bu * s + bv * c


def sample_texture(spec, cascade, uv):
    """_sample_spectrum_texture: periodic bilinear sample of one cascade at
    uv (..., 2); returns height, gradient (.., 2), displacement (.., 2),
    Jacobian (.., 4)."""

    height, grad, disp, jac = spec
    n = height.shape[1]
    wrapped = uv - np.floor(uv)
    texel = wrapped * F(n) - F(0.5)
    base = np.floor(texel).astype(np.int64)
    frac = texel - base.astype(F)
    x0 = (base[..., 0] % n + n) % n
    y0 = (base[..., 1] % n + n) % n
    x1, y1 = (x0 + 1) % n, (y0 + 1) % n
    fx, fy = frac[..., 0], frac[..., 1]

    def bil(a):
        a = a[cascade]
        a00, a10, a01, a11 = a[x0, y0], a[x1, y0], a[x0, y1], a[x1, y1]
        if a00.ndim > fx.ndim:
            gx, gy = fx[..., None], fy[..., None]
        else:
            gx, gy = fx, fy
        r0 = a00 * (F(1.0) - gx) + a10 * gx
        r1 = a01 * (F(1.0) - gx) + a11 * gx
        return r0 * (F(1.0) - gy) + r1 * gy

    return bil(height), bil(grad), bil(disp), bil(jac)


def sample_spectrum(spec, global_offset, radial, phase_offsets, wind_radians, footprint, geometry_only,
                    geometry_cascades, variances):
    """_sample_spectrum: summed wave height, resolved surface slope (.., 3)
    and unresolved slope variance over the cascades."""

    shape = global_offset.shape[:-1]
    height = np.zeros(shape, F)
    slope = np.zeros(shape + (3,), F)
    unresolved = np.zeros(shape, F)
    periods = _v(PERIODS_M)
    var = _v(variances)
    min_wavelengths = periods / F(5.5)
    for c in range(CASCADES):
        if geometry_only and not c < geometry_cascades:
            continue
        axis_u, axis_v = cascade_axes(c, wind_radians)
        base_uv = np.stack([F(phase_offsets[c, 0]) + _dot(global_offset, np.broadcast_to(axis_u, global_offset.shape))
                            / periods[c],
                            F(phase_offsets[c, 1]) + _dot(global_offset, np.broadcast_to(axis_v, global_offset.shape))
                            / periods[c]], -1)
        uv = base_uv
        for _ in range(2):
            _, _, band_disp, _ = sample_texture(spec, c, uv)
            uv = base_uv - band_disp / periods[c]
        band_h, band_g, _, band_j = sample_texture(spec, c, uv)
        if geometry_only:
            height = height + band_h
            continue
        spw = min_wavelengths[c] / np.maximum(footprint, F(0.01))
        resolved = np.minimum(np.maximum((spw - F(2.0)) / F(4.0), F(0.0)), F(1.0))
        resolved = resolved * resolved * (F(3.0) - F(2.0) * resolved)
        m00 = F(1.0) + band_j[..., 0]
        m01 = band_j[..., 1]
        m10 = band_j[..., 2]
        m11 = F(1.0) + band_j[..., 3]
        det = m00 * m11 - m01 * m10
        safe = np.where(np.abs(det) < F(0.15), np.where(det >= F(0.0), F(0.15), F(-0.15)), det)
        mg0 = (m11 * band_g[..., 0] - m10 * band_g[..., 1]) / safe
        mg1 = (-m01 * band_g[..., 0] + m00 * band_g[..., 1]) / safe
        tu = axis_u - radial * _dot(radial, np.broadcast_to(axis_u, radial.shape))[..., None]
        tv = axis_v - radial * _dot(radial, np.broadcast_to(axis_v, radial.shape))[..., None]
        slope = slope + (tu * mg0[..., None] + tv * mg1[..., None]) * resolved[..., None]
        unresolved = unresolved + var[c] * (F(1.0) - resolved * resolved)
    return height, slope, unresolved


class OceanSettings:
    """The OceanConfig fields the coverage pass reads (ocean.py:38-110)."""

    def __init__(self, enabled=True, albedo=(0.012, 0.055, 0.16), normal_strength=0.32, max_visible_depth_m=80.0,
                 spectrum_resolution=128, wind_speed_mps=8.0, wind_direction_degrees=35.0, wave_height_scale=1.0,
                 choppiness=0.65, geometry_cascades=2, geometry_max_distance_m=25_000.0, surface_enabled=True):
        self.enabled = enabled
        self.albedo = albedo
        self.normal_strength = normal_strength
        self.max_visible_depth_m = max_visible_depth_m
        self.spectrum_resolution = spectrum_resolution
        self.wind_speed_mps = wind_speed_mps
        self.wind_direction_degrees = wind_direction_degrees
        self.wave_height_scale = wave_height_scale
        self.choppiness = choppiness
        self.geometry_cascades = geometry_cascades
        self.geometry_max_distance_m = geometry_max_distance_m
        self.surface_enabled = surface_enabled


def phase_offsets(up, planet_radius_m, wind_radians):
    """The per-cascade texture offsets of the sea anchor (float64, :709-726)."""

    anchor = np.asarray(up, np.float64) * float(planet_radius_m)
    out = np.zeros((CASCADES, 2), F)
    c, s = math.cos(wind_radians), math.sin(wind_radians)
    base = (((1.0, 0.0, 0.0), (0.0, 0.0, 1.0)), ((0.0, 1.0, 0.0), (1.0, 0.0, 0.0)),
            ((0.0, 0.0, 1.0), (0.0, 1.0, 0.0)))
    for k, (bu, bv) in enumerate(base):
        bu, bv = np.asarray(bu, np.float64), np.asarray(bv, np.float64)
        au = bu * c + bv * s
        av = -bu * s + bv * c
        out[k, 0] = (anchor.dot(au) / PERIODS_M[k]) % 1.0
        out[k, 1] = (anchor.dot(av) / PERIODS_M[k]) % 1.0
    return out


def rasterize(g: dict, cfg: OceanSettings, planet_radius_m, camera_altitude_m, planet_frame, view_basis,
              tangent_half_fov, time_seconds, debug_mode=0, spectrum=None) -> dict:
    """OceanRenderer.rasterize on the G-buffer ``g`` (numpy fields as the
    reference's: depth, position, normal, albedo, material_weights, height_m,
    water_depth, seabed_albedo, seabed_normal, slope_variance, surface_id,
    cell_id).  Returns the updated copy and the spectrum."""

    g = {k: np.array(v, copy=True) for k, v in g.items()}
    if not cfg.surface_enabled:
        return g, None
    amp_scale = cfg.wave_height_scale * wind_amplitude_scale(cfg.wind_speed_mps)
    if cfg.enabled and spectrum is None:
        spectrum = build_spectrum(cfg.spectrum_resolution, time_seconds, amp_scale, cfg.choppiness)
    wind = math.radians(cfg.wind_direction_degrees)
    east, up, north = (_v(a) for a in planet_frame)
    right, view_up, forward = (_v(a) for a in view_basis)
    offsets = phase_offsets(planet_frame[1], planet_radius_m, wind)
    variances = slope_variances(cfg.wave_height_scale, cfg.wind_speed_mps)
    max_disp = F(max_geometry_displacement(cfg.wave_height_scale, cfg.wind_speed_mps, cfg.geometry_cascades)
                 if cfg.enabled else 0.0)
    geom_max = F(cfg.geometry_max_distance_m if cfg.enabled else 0.0)
    R = F(planet_radius_m)
    alt = F(max(camera_altitude_m, 0.0))
    tf = F(tangent_half_fov)
    wind_f = F(wind)
    W, H = g["surface_id"].shape
    aspect = F(W) / F(H)
    origin = np.array([0.0, R + alt, 0.0], F)
    X, Y = np.meshgrid(np.arange(W), np.arange(H), indexing="ij")
    su = (X.astype(F) + F(0.5)) / F(W)
    sv = (Y.astype(F) + F(0.5)) / F(H)
    sx = (su * F(2.0) - F(1.0)) * aspect
    sy = sv * F(2.0) - F(1.0)
    ray_view = _normalized(np.stack([sx, sy, np.full_like(sx, F(1.0) / tf)], -1))
    ray_local = (right * ray_view[..., 0:1] + view_up * ray_view[..., 1:2]) + forward * ray_view[..., 2:3]
    distance = near_sphere_distance(alt, ray_local[..., 1], R)
    reseed = (distance <= F(0.1)) & (max_disp > F(0.0)) & (alt > max_disp)
    if reseed.any():
        distance = np.where(reseed, near_sphere_distance(alt - max_disp, ray_local[..., 1], R + max_disp), distance)
    geo = (distance > F(0.1)) & (distance <= geom_max)
    geo_cascades = cfg.geometry_cascades

    def to_global(vl):
        return (east * vl[..., 0:1] + up * vl[..., 1:2]) + north * vl[..., 2:3]

    def offset_global(vl):
        return (east * vl[..., 0:1] + up * (vl[..., 1:2] - R)) + north * vl[..., 2:3]

    if geo.any() and spectrum is not None:
        for _ in range(3):
            cand = origin + ray_local * distance[..., None]
            radial_local = cand / np.maximum(_norm(cand), F(1.0))[..., None]
            radial_global = _normalized(to_global(radial_local))
            goff = offset_global(cand)
            wave_h, _, _ = sample_spectrum(spectrum, goff, radial_global, offsets, wind_f, F(0.0), True,
                                           geo_cascades, variances)
            displaced = near_sphere_distance(alt - wave_h, ray_local[..., 1], R + wave_h)
            distance = np.where(geo & (displaced > F(0.1)), displaced, distance)
    elif geo.any():
        # geometry cascades sample an unbuilt spectrum only when the advanced
        # path is off, where geometry_max_distance is 0: nothing is displaced
        pass
    hit = distance > F(0.1)
    ocean_view = ray_view * distance[..., None]
    sid = g["surface_id"]
    nearer = hit & ((sid < 0) | (ocean_view[..., 2] < g["depth"]))
    max_depth = F(cfg.max_visible_depth_m)
    has_seabed = sid >= 0
    seabed_distance = np.where(has_seabed, _norm(g["position"][..., :3].astype(F)), distance + max_depth)
    seabed_color = np.where(has_seabed[..., None], g["albedo"][..., :3], _v((0.025, 0.035, 0.025)))
    optical = np.minimum(np.maximum(seabed_distance - distance, F(0.0)), max_depth)
    ocean_local = origin + ray_local * distance[..., None]
    radial_local = ocean_local / np.maximum(_norm(ocean_local), F(1.0))[..., None]
    radial_global = _normalized(to_global(radial_local))
    seabed_normal = np.where(has_seabed[..., None], g["normal"][..., :3], radial_global)
    goff = offset_global(ocean_local)
    footprint = distance * F(2.0) * tf / F(H)
    slope = np.zeros_like(goff)
    unresolved = np.zeros(distance.shape, F)
    if cfg.enabled:
        _, slope, unresolved = sample_spectrum(spectrum, goff, radial_global, offsets, wind_f, footprint, False,
                                               geo_cascades, variances)
    water_normal = _normalized(radial_global - slope * F(cfg.normal_strength))
    color = {1: (0.02, 0.63, 0.82), 2: (0.05, 0.18, 0.70), 3: (0.04, 0.35, 0.62)}.get(int(debug_mode), cfg.albedo)
    m = nearer
    m3 = m[..., None]
    g["depth"] = np.where(m, ocean_view[..., 2], g["depth"]).astype(F)
    g["position"] = np.where(m3, ocean_view, g["position"]).astype(F)
    g["normal"] = np.where(m3, water_normal, g["normal"]).astype(F)
    g["albedo"] = np.where(m3, _v(color), g["albedo"]).astype(F)
    g["material_weights"] = np.where(m3, F(0.0), g["material_weights"]).astype(F)
    g["height_m"] = np.where(m, _norm(ocean_local) - R, g["height_m"]).astype(F)
    g["water_depth"] = np.where(m, optical, g["water_depth"]).astype(F)
    g["seabed_albedo"] = np.where(m3, seabed_color, g["seabed_albedo"]).astype(F)
    g["seabed_normal"] = np.where(m3, seabed_normal, g["seabed_normal"]).astype(F)
    g["slope_variance"] = np.where(m, unresolved, g["slope_variance"]).astype(F)
    g["surface_id"] = np.where(m, OCEAN_SURFACE_ID, sid).astype(np.int32)
    g["cell_id"] = np.where(m, -1, g["cell_id"]).astype(np.int32)
    return g, spectrum
