"""Per-ray geometry of far cameras in compensated float32.

Seen from many planet radii, r^2 - R^2 along a grazing ray cancels the
camera's ~r_cam^2 terms.  The kernels pivot such rays at the closest approach
and form r_c^2 - R^2 and (R + top)^2 - r_c^2 as differences of squares from
r_c = (R + h0) sin v carried as a float pair (two-sum, FMA two-product), and
the sun term p(t_c) . sun from the closest-approach point.  These tests
restate that float32 sequence in numpy (an FMA of two floats is exact in
float64 and then rounds once) and check it against float64 on the same float32
inputs across both limbs: a few float ulps of the quantity itself, where the
plain float32 form keeps no digit."""

from __future__ import annotations

import numpy as np
import pytest

f32 = np.float32


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    err = f32(f32(a - f32(s - bb)) + f32(b - bb))
    return s, err


def fma32(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def compensated(bottom, top, h0, sinv, cosv):
    """The float32 operation sequence of the far-camera ray setup."""

    o, o_lo = two_sum(bottom, h0)
    rc = f32(o * sinv)
    rc_lo = f32(fma32(o, sinv, -rc) + f32(o_lo * sinv))
    bt, bt_lo = two_sum(bottom, top)
    dg = f32(f32(bottom - rc) - rc_lo)
    dt = f32(f32(f32(bt - rc) + bt_lo) - rc_lo)
    disc_ground = f32(dg * f32(bottom + rc))
    disc_top = f32(dt * f32(bt + rc))
    t0 = -fma32(o, cosv, f32(o_lo * cosv))
    return disc_ground, disc_top, t0


def exact(bottom, top, h0, sinv, cosv):
    b, t = np.float64(bottom), np.float64(top)
    o = b + np.float64(h0)
    rc = o * np.float64(sinv)
    return (b - rc) * (b + rc), (b + t - rc) * (b + t + rc), -o * np.float64(cosv)


def grazing_rays(bottom, top, h0, n=400):
    """Ray sines around the ground and top limbs, float32."""

    o = np.float64(bottom) + h0
    out = []
    for shell in (bottom, bottom + top):
        s_limb = shell / o
        for k in np.geomspace(1e-9, 1e-2, n // 2):
            for sgn in (-1.0, 1.0):
                s = min(s_limb * (1.0 + sgn * k), 1.0)
                out.append(f32(s))
    sinv = np.array(out, dtype=np.float32)
    cosv = (-np.sqrt(1.0 - sinv.astype(np.float64) ** 2)).astype(np.float32)
    return sinv, cosv


@pytest.mark.parametrize("bottom,top,h0", [
    (50_000.0, 60_000.0, 1_867_260.0),     # small planet, camera ~37 radii up
    (50_000.0, 60_000.0, 241_214.0),
    (6_360_000.0, 100_000.0, 12_000_000.0),  # Earth from ~2 radii up
])
def test_compensated_differences_of_squares(bottom, top, h0):
    bottom, top, h0 = f32(bottom), f32(top), f32(h0)
    sinv, cosv = grazing_rays(bottom, top, h0)
    worst_g = worst_t = worst_naive = 0.0
    for s, c in zip(sinv, cosv):
        dg, dt, t0 = compensated(bottom, top, h0, s, c)
        eg, et, e0 = exact(bottom, top, h0, s, c)
        # error against the float32 spacing of the quantity itself (+ the
        # absolute floor of the product's low part, ~2^-48 r_cam^2)
        floor = 2.0 ** -46 * float(np.float64(bottom + h0) ** 2)
        worst_g = max(worst_g, abs(float(dg) - eg) / (abs(eg) * 2.0 ** -23 + floor))
        worst_t = max(worst_t, abs(float(dt) - et) / (abs(et) * 2.0 ** -23 + floor))
        assert abs(float(t0) - e0) <= 2.0 ** -22 * abs(e0)
        # the plain float32 form r_c^2 - R^2
        rc = f32(f32(bottom + h0) * s)
        naive = f32(f32(bottom * bottom) - f32(rc * rc))
        worst_naive = max(worst_naive, abs(float(naive) - eg) / (abs(eg) * 2.0 ** -23 + floor))
    assert worst_g <= 4.0 and worst_t <= 4.0, (worst_g, worst_t)
    assert worst_naive > 1e3, worst_naive


def test_sun_term_from_the_closest_point():
    """p(t0) . sun through the closest-approach point: error ~ulp(r_c), not
    ~ulp(r_cam)."""

    rng = np.random.default_rng(3)
    bottom, h0 = f32(50_000.0), f32(1_867_260.0)
    o_y = f32(bottom + h0)
    worst = 0.0
    for _ in range(2000):
        ray = rng.normal(size=3)
        ray[1] = -abs(ray[1]) * 40.0  # looking down at the planet
        ray = (ray / np.linalg.norm(ray)).astype(np.float32)
        sun = rng.normal(size=3)
        sun = (sun / np.linalg.norm(sun)).astype(np.float32)
        sinv = f32(np.sqrt(np.float64(ray[0]) ** 2 + np.float64(ray[2]) ** 2))
        _, _, t0 = compensated(bottom, f32(60_000.0), h0, sinv, ray[1])
        c = (f32(t0 * ray[0]), fma32(t0, ray[1], o_y), f32(t0 * ray[2]))
        s0 = f32(f32(f32(c[0] * sun[0]) + f32(c[1] * sun[1])) + f32(c[2] * sun[2]))
        ref = np.float64(o_y) * sun[1] + np.float64(t0) * np.dot(ray.astype(np.float64), sun.astype(np.float64))
        rc = np.float64(o_y) * np.float64(sinv)
        worst = max(worst, abs(float(s0) - ref) / (rc * 2.0 ** -24))
    assert worst <= 16.0, worst
