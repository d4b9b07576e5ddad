"""CPU restatement (test infrastructure) of the reference's surface shading,
PlanetRenderer._shade_surface (src/planet_renderer/renderer.py:1277-1575):
the consumer of prepare_frame's surface_sun_transmittance and
surface_sky_radiance.  Land pixels are Lambertian under the transmitted sun
and the sky radiance; ocean pixels (advanced ocean on) add a GGX-style sun
specular, Fresnel sky reflection and a water body over the seabed, whose
albedo, normal and depth are reconstructed along the refracted view ray from
the opaque terrain snapshot.  numpy float32, operation by operation in the
reference's order (vectorised over pixels, branches as masks); fields are
(W, H[, 3]) indexed [x, y] like the reference's Taichi fields.  Used only by
tests, never by the product path."""

from __future__ import annotations

import math

import numpy as np

F = np.float32
SKY_COLOR = (0.00015, 0.0002, 0.00035)  # renderer.py:1302


def _dot(a, b):
    """((a0 b0 + a1 b1) + a2 b2), the reference's float32 order."""

    acc = a[..., 0] * b[..., 0]
    for k in range(1, a.shape[-1]):
        acc = acc + a[..., k] * b[..., k]
    return acc


def _norm(a):
    return np.sqrt(_dot(a, a))


def _normalized(a):
    # Taichi: (1 / (norm + 0)) * v
    return (F(1.0) / _norm(a))[..., None] * a


def _vec(args, name):
    return np.asarray([F(v) for v in args[name]], dtype=F)


def shade_surface(fields: dict, args: dict, ocean_surface_id: int) -> np.ndarray:
    """surface_hdr of _shade_surface for the G-buffer `fields` (keys as in
    tests/golden/shading.npz: position, normal, albedo, water_depth,
    seabed_albedo, seabed_normal, slope_variance, surface_id,
    terrain_position, terrain_normal, terrain_albedo, terrain_surface_id,
    sun_transmittance, sky_radiance) and the kernel's arguments `args`."""

    g = {k: np.asarray(v) for k, v in fields.items()}
    sid = g["surface_id"]
    W, H = sid.shape
    sun = _vec(args, "sun_global")
    E = _vec(args, "solar_irradiance")
    right, up, fwd = (_vec(args, n) for n in ("view_right_global", "view_up_global", "view_forward_global"))
    f0 = F(args["ocean_f0"])
    roughness = F(args["ocean_roughness"])
    sky_strength = F(args["ocean_sky_strength"])
    absorption, scattering = _vec(args, "ocean_absorption"), _vec(args, "ocean_scattering")
    max_depth = F(args["ocean_max_depth"])
    ior = F(args["ocean_refraction_index"])
    strength = F(args["ocean_refraction_strength"])
    max_offset = F(args["ocean_refraction_max_offset_pixels"])
    ang = F(args["sun_angular_radius"])
    tanfov = F(args["tangent_half_fov"])
    mode = int(args["mode"])
    advanced = int(args["advanced_ocean_enabled"])
    pi = F(math.pi)

    color = np.broadcast_to(np.asarray(SKY_COLOR, dtype=F), (W, H, 3)).copy()
    surface = sid >= 0
    albedo = g["albedo"].astype(F)
    if mode != 0:
        color[surface] = albedo[surface]
        return np.maximum(color, F(0.0))

    with np.errstate(all="ignore"):
        T = g["sun_transmittance"].astype(F)
        L_sky = g["sky_radiance"].astype(F)
        normal = _normalized(g["normal"].astype(F))
        ndotl = np.maximum(_dot(normal, np.broadcast_to(sun, normal.shape)), F(0.0))
        direct = E * T * ndotl[..., None]
        lambert = albedo * (direct / pi + L_sky)
        color = np.where(surface[..., None], lambert, color)

        ocean = surface & (sid == ocean_surface_id) & (advanced != 0)
        if not ocean.any():
            return np.maximum(color, F(0.0))
        position = g["position"].astype(F)
        px, py, pz = position[..., 0:1], position[..., 1:2], position[..., 2:3]
        view_direction = -_normalized(right * px + up * py + fwd * pz)
        ndotv = np.maximum(_dot(normal, view_direction), F(1.0e-4))
        half_sum = view_direction + sun
        half_vector = half_sum / np.maximum(_norm(half_sum), F(1.0e-5))[..., None]
        ndoth = np.maximum(_dot(normal, half_vector), F(0.0))
        vdoth = np.maximum(_dot(view_direction, half_vector), F(0.0))
        omv = F(1.0) - ndotv
        fresnel_view = f0 + (F(1.0) - f0) * (omv * omv * omv * omv * omv)
        omh = F(1.0) - vdoth
        fresnel_sun = f0 + (F(1.0) - f0) * (omh * omh * omh * omh * omh)
        base_alpha = roughness * roughness
        solar_slope_variance = np.tan(ang) ** 2
        alpha2 = base_alpha * base_alpha + g["slope_variance"].astype(F) + solar_slope_variance
        alpha2 = np.minimum(np.maximum(alpha2, F(1.0e-5)), F(1.0))
        denominator = ndoth * ndoth * (alpha2 - F(1.0)) + F(1.0)
        distribution = alpha2 / np.maximum(pi * denominator * denominator, F(1.0e-5))
        effective_roughness = np.sqrt(np.sqrt(alpha2))
        geometry_k = (effective_roughness + F(1.0)) ** 2 / F(8.0)
        geometry_v = ndotv / np.maximum(ndotv * (F(1.0) - geometry_k) + geometry_k, F(1.0e-5))
        geometry_l = ndotl / np.maximum(ndotl * (F(1.0) - geometry_k) + geometry_k, F(1.0e-5))
        sun_specular = (E * T * distribution[..., None] * geometry_v[..., None] * geometry_l[..., None]
                        * fresnel_sun[..., None] * ndotl[..., None]
                        / np.maximum(F(4.0) * ndotv * ndotl, F(1.0e-4))[..., None])
        reflected_sky = L_sky * fresnel_view[..., None] * sky_strength
        water_depth = np.minimum(g["water_depth"].astype(F), max_depth)
        seabed_albedo = g["seabed_albedo"].astype(F)
        seabed_normal = _normalized(g["seabed_normal"].astype(F))

        # refraction into the water and seabed reconstruction (:1388-1520)
        incident_view = _normalized(position)
        normal_view = _normalized(np.stack([_dot(normal, np.broadcast_to(v, normal.shape)) for v in (right, up, fwd)],
                                           -1))
        cos_incident = np.maximum(-_dot(incident_view, normal_view), F(0.0))
        eta = F(1.0) / ior
        discriminant = F(1.0) - eta * eta * (F(1.0) - cos_incident * cos_incident)
        bent = _normalized(eta * incident_view
                           + (eta * cos_incident - np.sqrt(discriminant))[..., None] * normal_view)
        refracted_view = np.where((discriminant > F(0.0))[..., None], bent, incident_view)
        refracted_view = _normalized(incident_view * (F(1.0) - strength) + refracted_view * strength)
        vertical_depth = water_depth * np.maximum(-_dot(incident_view, normal_view), F(0.05))
        refracted_distance = np.minimum(vertical_depth / np.maximum(-_dot(refracted_view, normal_view), F(0.05)),
                                        max_depth * F(2.0))
        endpoint = position + refracted_view * refracted_distance[..., None]
        project = (endpoint[..., 2] > F(0.1)) & (strength > F(0.0))
        aspect = F(W) / F(H)
        sx = (endpoint[..., 0] / (endpoint[..., 2] * tanfov * aspect) * F(0.5) + F(0.5)) * F(W) - F(0.5)
        sy = (endpoint[..., 1] / (endpoint[..., 2] * tanfov) * F(0.5) + F(0.5)) * F(H) - F(0.5)
        qx = np.broadcast_to(np.arange(W, dtype=F)[:, None], (W, H))
        qy = np.broadcast_to(np.arange(H, dtype=F)[None, :], (W, H))
        dx, dy = sx - qx, sy - qy
        delta_length = np.sqrt(dx * dx + dy * dy)
        clamp = delta_length > max_offset
        k = max_offset / np.maximum(delta_length, F(1.0e-5))
        dx, dy = np.where(clamp, dx * k, dx), np.where(clamp, dy * k, dy)
        sx, sy = np.where(clamp, qx + dx, sx), np.where(clamp, qy + dy, sy)
        bx = np.floor(sx)
        by = np.floor(sy)
        fx, fy = sx - bx, sy - by
        bx = np.where(np.isfinite(bx), bx, 0).astype(np.int64)
        by = np.where(np.isfinite(by), by, 0).astype(np.int64)
        acc_albedo = np.zeros((W, H, 3), F)
        acc_normal = np.zeros((W, H, 3), F)
        acc_position = np.zeros((W, H, 3), F)
        acc_weight = np.zeros((W, H), F)
        t_id, t_pos = g["terrain_surface_id"], g["terrain_position"].astype(F)
        t_alb, t_nrm = g["terrain_albedo"].astype(F), g["terrain_normal"].astype(F)
        for oy in (0, 1):
            for ox in (0, 1):
                ix, iy = bx + ox, by + oy
                inside = (ix >= 0) & (ix < W) & (iy >= 0) & (iy < H)
                cx, cy = np.clip(ix, 0, W - 1), np.clip(iy, 0, H - 1)
                candidate = t_pos[cx, cy]
                distance = _norm(candidate - position)
                valid = (inside & (t_id[cx, cy] >= 0) & (candidate[..., 2] > position[..., 2] + F(0.01))
                         & (distance <= max_depth * F(2.0)))
                wx = (F(1.0) - fx) if ox == 0 else fx
                wy = (F(1.0) - fy) if oy == 0 else fy
                weight = wx * wy
                use = (valid & project)[..., None]
                acc_albedo = np.where(use, acc_albedo + t_alb[cx, cy] * weight[..., None], acc_albedo)
                acc_normal = np.where(use, acc_normal + t_nrm[cx, cy] * weight[..., None], acc_normal)
                acc_position = np.where(use, acc_position + candidate * weight[..., None], acc_position)
                acc_weight = np.where(use[..., 0], acc_weight + weight, acc_weight)
        found = project & (acc_weight > F(0.25))
        inv = F(1.0) / acc_weight
        seabed_albedo = np.where(found[..., None], acc_albedo * inv[..., None], seabed_albedo)
        seabed_normal = np.where(found[..., None], _normalized(acc_normal * inv[..., None]), seabed_normal)
        seabed_position = acc_position * inv[..., None]
        water_depth = np.where(found, np.minimum(_norm(seabed_position - position), max_depth), water_depth)

        # water body (:1521-1574)
        water_extinction = absorption + scattering
        water_transmission = np.exp(-water_extinction * water_depth[..., None])
        seabed_ndotl = np.maximum(_dot(seabed_normal, np.broadcast_to(sun, seabed_normal.shape)), F(0.0))
        seabed_direct = E * T * seabed_ndotl[..., None]
        lit_seabed = seabed_albedo * (seabed_direct / pi + L_sky)
        seabed = lit_seabed * water_transmission
        scattering_albedo = scattering / np.maximum(water_extinction, F(1.0e-6))
        incident_water = L_sky + direct / F(4.0 * math.pi)
        water_scattering = incident_water * scattering_albedo * (F(1.0) - water_transmission)
        water_body = (seabed + water_scattering) * (F(1.0) - fresnel_view)[..., None]
        ocean_color = water_body + reflected_sky + sun_specular
        color = np.where(ocean[..., None], ocean_color, color)
    return np.maximum(color, F(0.0)).astype(F)
