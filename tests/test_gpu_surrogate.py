"""Learned surrogates: training samples against the oracle, training by the
package's kernels, the surrogate composite's queue and gates, its error
against the FP64 oracle and what it gains over the plain integrator (the
method without it)."""

from __future__ import annotations

import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

E = (4.0, 3.9, 3.7)
AR_DEG = 0.266


@pytest.fixture(scope="module")
def source():
    from planet_renderer_gb300.atmosphere.surrogate import SampleSource, parameter_grid

    s = SampleSource(parameter_grid(rayleigh=(6000.0, 10000.0), mie=(800.0, 1600.0)))
    yield s
    s.close()


@pytest.fixture(scope="module")
def trained(source):
    """Both networks at a reduced training budget (seconds)."""

    from planet_renderer_gb300.atmosphere.surrogate import AERIAL, SKY, Surrogate, train

    aerial, ra = train(source, AERIAL, n_samples=2**21, batch=16384, epochs=60, lr=4e-3, seed=3, log_every=50)
    sky, rs = train(source, SKY, n_samples=2**21, batch=16384, epochs=60, lr=4e-3, seed=4, log_every=50)
    return Surrogate(aerial, sky, source.planet_radius_m, source.top_altitude_m, source.scale_height_range), ra, rs


# ---- feature decoding (the generator's maps, numpy float64) ------------------------
def _decode(x, top, R, scale_height_range, kind):
    x = x.astype(np.float64)
    h = top * ((x[:, 0] + 1.0) * 0.5) ** 2
    rho = np.sqrt(h * (2 * R + h))
    hz = math.pi - np.arccos(np.clip(rho / (R + h), 0.0, 1.0))
    v = (x[:, 1] + 1.0) * 0.5
    zen = np.where(v < 0.5, hz * (1 - (1 - 2 * v) ** 2), hz + (math.pi - hz) * (2 * v - 1) ** 2)
    hc = -rho / (R + h)
    u = (x[:, 2] + 1.0) * 0.5
    mu_s = np.where(u < 0.5, hc - (hc + 1) * (1 - 2 * u) ** 2, hc + (1 - hc) * (2 * u - 1) ** 2)
    mu_s = np.clip(mu_s, -1, 1)
    cphi = x[:, 3]
    ss, sphi = np.sqrt(np.maximum(1 - mu_s ** 2, 0)), np.sqrt(np.maximum(1 - cphi ** 2, 0))
    ray = np.stack([np.sin(zen), np.cos(zen), np.zeros_like(zen)], 1)
    sun = np.stack([ss * cphi, mu_s, ss * sphi], 1)
    lo_r, hi_r, lo_m, hi_m = scale_height_range
    hr = np.exp(math.log(lo_r) + (x[:, 4] + 1) * 0.5 * (math.log(hi_r) - math.log(lo_r)))
    hm = np.exp(math.log(lo_m) + (x[:, 5] + 1) * 0.5 * (math.log(hi_m) - math.log(lo_m)))
    length = 2.0e6 ** ((x[:, 6] + 1) * 0.5) if kind == 1 else None
    return h, ray, sun, hr, hm, length


def test_samples_are_deterministic_and_in_the_box(source):
    from planet_renderer_gb300.atmosphere.surrogate import AERIAL, SKY

    for kind in (SKY, AERIAL):
        x1, y1 = source.samples(kind, 4096, 5)
        x2, y2 = source.samples(kind, 8192, 5)
        torch.cuda.synchronize()
        assert torch.equal(x1, x2[:4096]) and torch.equal(y1, y2[:4096])
        assert float(x1.abs().max()) <= 1.0 + 1e-6
        assert bool(torch.isfinite(y1).all())


@pytest.mark.parametrize("kind", [0, 1])
def test_samples_match_the_oracle_integrator(source, kind):
    """Targets of the GPU generator against the oracle's single-ray
    restatement of the same integrals at the decoded geometry."""

    from oracle.atm import Oracle
    from planet_renderer_gb300.atmosphere.surrogate import FLOOR, MAX_DEPTH

    x, y = source.samples(kind, 1536, 11)
    x, y = x.cpu().numpy(), y.cpu().numpy()
    h, ray, sun, hr, hm, length = _decode(x, source.top_altitude_m, source.planet_radius_m,
                                          source.scale_height_range, kind)
    # FP64: the reference's float32 segment weight rounds the in-scattering of
    # thin high-altitude segments to zero, the kernels' series weight does not
    o = Oracle("f64")
    ar = math.radians(AR_DEG)
    ref = np.zeros_like(y, dtype=np.float64)
    for cfg in source.configs:
        m = (np.abs(hr - cfg.rayleigh_scale_height_m) < 1.0) & (np.abs(hm - cfg.mie_scale_height_m) < 1.0)
        if not m.any():
            continue
        tl = o.build_transmittance(cfg, source.planet_radius_m)
        ms = o.build_multi_scattering(cfg, source.planet_radius_m, E, ar, tl)
        if kind == 0:
            L = o.sky_rays(cfg, source.planet_radius_m, h[m], ray[m], sun[m], E, ar, tl, ms)
            ref[m] = np.log(L / np.array(E) + FLOOR)
        else:
            L, T = o.surface_rays(cfg, source.planet_radius_m, h[m], ray[m], length[m], sun[m], E, ar, tl, ms)
            ref[m, :3] = np.log(L / np.array(E) + FLOOR)
            ref[m, 3:] = np.minimum(-np.log(np.maximum(T.astype(np.float64), 1e-30)), MAX_DEPTH)
    d = np.abs(y - ref)
    # radiance targets: ln differences = relative differences; decoding the
    # features back to geometry in float64 moves rays by ~1e-7, which only
    # matters for the rare ray grazing the ground
    assert np.median(d[:, :3]) < 1e-4, np.median(d[:, :3])
    assert np.quantile(d[:, :3], 0.99) < 5e-3, np.quantile(d[:, :3], 0.99)
    if kind == 1:
        live = ref[:, 3:] < 10
        assert np.quantile(d[:, 3:][live], 0.99) < 5e-3


def _point_features_match(x, fs, fh, top, R, ray, sun, h, t):
    """Features fs (sun cosine, u mapping) and fh (altitude) of the point at
    distance t along each ray against float64 geometry."""

    p = np.stack([ray[:, 0] * t, R + h + ray[:, 1] * t, ray[:, 2] * t], 1)
    r = np.linalg.norm(p, axis=1)
    he = np.clip(r - R, 0.0, top)
    mu = np.sum(p * sun, axis=1) / r
    got_h = top * ((x[:, fh].astype(np.float64) + 1.0) * 0.5) ** 2
    assert np.max(np.abs(got_h - he) / (3.0 + 1e-4 * he)) <= 1.0
    hc = -np.sqrt(got_h * (2 * R + got_h)) / (R + got_h)
    u = (x[:, fs].astype(np.float64) + 1.0) * 0.5
    got_mu = np.where(u < 0.5, hc - (hc + 1) * (1 - 2 * u) ** 2, hc + (1 - hc) * (2 * u - 1) ** 2)
    assert np.max(np.abs(got_mu - np.clip(mu, -1, 1))) <= 2e-4


def test_aerial_segment_end_features(source):
    """Aerial features 7-10: sun cosine and altitude at the segment's end (the
    shell-clipped length) and middle, against the decoded geometry."""

    from planet_renderer_gb300.atmosphere.surrogate import AERIAL

    x, _ = source.samples(AERIAL, 4096, 13, 0.25, 0.5)
    x = x.cpu().numpy()
    assert x.shape[1] == 11
    top, R = source.top_altitude_m, source.planet_radius_m
    h, ray, sun, _, _, length = _decode(x, top, R, source.scale_height_range, AERIAL)
    b = (R + h) * ray[:, 1]
    t_top = -b + np.sqrt(np.maximum(b * b - ((R + h) ** 2 - (R + top) ** 2), 0.0))
    end = np.minimum(length, t_top)
    _point_features_match(x, 7, 8, top, R, ray, sun, h, end)
    _point_features_match(x, 9, 10, top, R, ray, sun, h, 0.5 * end)


def test_sky_ray_end_features(source):
    """Sky features 6-9: sun cosine and altitude where the march ends (top or
    ground) and at its lowest point."""

    from planet_renderer_gb300.atmosphere.surrogate import SKY

    x, _ = source.samples(SKY, 4096, 17)
    x = x.cpu().numpy()
    assert x.shape[1] == 10
    top, R = source.top_altitude_m, source.planet_radius_m
    h, ray, sun, _, _, _ = _decode(x, top, R, source.scale_height_range, SKY)
    b = (R + h) * ray[:, 1]
    t_top = -b + np.sqrt(np.maximum(b * b - ((R + h) ** 2 - (R + top) ** 2), 0.0))
    dg = b * b - ((R + h) ** 2 - R ** 2)
    t_g = -b - np.sqrt(np.maximum(dg, 0.0))
    # rays decoded within ~1e-7 rad of the horizon may hit or miss the ground
    grazing = np.abs(dg) < 1e-6 * (R + h) ** 2
    x, h, ray, sun, b, t_top, dg, t_g = (v[~grazing] for v in (x, h, ray, sun, b, t_top, dg, t_g))
    end = np.where((dg >= 0) & (ray[:, 1] < 0) & (t_g > 0), t_g, t_top)
    _point_features_match(x, 6, 7, top, R, ray, sun, h, end)
    _point_features_match(x, 8, 9, top, R, ray, sun, h, np.clip(-b, 0.0, end))


def test_training_learns_both_networks(trained):
    """Held-out errors at the reduced test budget (the bench states those of
    the full budget); BF16 inference stays close to the FP32 network."""

    _, ra, rs = trained
    for rep in (ra, rs):
        b, f = rep.held_out["bf16"], rep.held_out["f32"]
        assert b["radiance_rel_mean"] < 1.5 * f["radiance_rel_mean"] + 0.01, rep.held_out
        assert rep.loss[-1][1] < 0.05 * rep.loss[0][1], rep.loss
    # sky: over the input box; aerial: over segments ending at a surface (what frames evaluate)
    assert rs.held_out["bf16"]["radiance_rel_mean"] < 0.15, rs.held_out
    assert ra.held_out["bf16_surface"]["radiance_rel_mean"] < 0.35, ra.held_out
    assert ra.held_out["bf16_surface"]["composite_rel_mean"] < 0.08, ra.held_out


# ---- frames ---------------------------------------------------------------------------
def _frame(width, height, altitude_m, zenith_deg, azimuth_deg, seed=7):
    from planet_renderer_gb300.atmosphere import AtmosphereRenderer, scene
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.workloads import CameraView, EARTH_RADIUS_M
    from planet_renderer_gb300.lighting import LightingState

    v = CameraView(altitude_m, zenith_deg, azimuth_deg)
    r = AtmosphereRenderer(width, height, earth_baseline())
    gb = scene.synthesize_gbuffer(width, height, EARTH_RADIUS_M, v.altitude_m, v.basis, v.tangent_half_fov,
                                  v.sun_local, E, seed=seed, device=r.device)
    light = LightingState(v.sun_local, AR_DEG, E)
    r.update(EARTH_RADIUS_M, v.camera_radius_m, v.sun_local.copy(), E, AR_DEG)
    r.prepare_frame(gb["position_view"], gb["surface_id"], EARTH_RADIUS_M, v.camera_radius_m, v.sun_local, E, AR_DEG,
                    v.basis, v.tangent_half_fov)
    args = (EARTH_RADIUS_M, v.camera_radius_m, v.sun_local, E, light.sun_disk_radiance, AR_DEG, v.basis,
            v.tangent_half_fov, 4.0, 12.0)
    return r, gb, args, v


def _plain(r, gb, args):
    hdr = torch.zeros_like(gb["scene_hdr"])
    r.composite(gb["scene_hdr"], gb["space_hdr"], gb["surface_id"], gb["position_view"], hdr, *args)
    return hdr


def _surrogate(r, gb, args, sg, check_fraction=0.0, scene=None):
    hdr = torch.zeros_like(gb["scene_hdr"])
    stats = torch.zeros(8, dtype=torch.float32, device=r.device)
    r.composite_surrogate(gb["scene_hdr"] if scene is None else scene, gb["space_hdr"], gb["surface_id"],
                          gb["position_view"], hdr, *args, surrogate=sg, stats=stats, check_fraction=check_fraction,
                          seed=9)
    torch.cuda.synchronize()
    return hdr, stats


def test_without_networks_the_surrogate_composite_is_the_plain_one():
    from planet_renderer_gb300.atmosphere.surrogate import Surrogate

    r, gb, args, _ = _frame(320, 180, 2000.0, 40.0, 30.0)
    plain = _plain(r, gb, args)
    got, stats = _surrogate(r, gb, args, Surrogate(None, None))
    # every surface pixel goes through the queue and the plain integrator
    np.testing.assert_allclose(got.cpu().numpy(), plain.cpu().numpy(), rtol=2e-5, atol=1e-9)
    n_surface = int((gb["surface_id"] >= 0).sum())
    assert int(stats[3]) <= n_surface and int(stats[4]) == 0 and int(stats[5]) == 0
    r.close()


def test_checked_pixels_keep_the_plain_result(trained):
    """check_fraction = 1 re-integrates every MLP pixel: the frame is the
    plain frame (sky network off: sky pixels read the LUT as the plain
    composite does), and every MLP surface pixel was counted and judged."""

    from planet_renderer_gb300.atmosphere.surrogate import Surrogate, stats_summary

    sg_full, _, _ = trained
    sg = Surrogate(sg_full.aerial, None, sg_full.planet_radius_m, sg_full.top_altitude_m, sg_full.scale_height_range)
    r, gb, args, _ = _frame(320, 180, 2000.0, 40.0, 30.0)
    plain = _plain(r, gb, args)
    got, stats = _surrogate(r, gb, args, sg, check_fraction=1.0)
    np.testing.assert_allclose(got.cpu().numpy(), plain.cpu().numpy(), rtol=2e-5, atol=1e-9)
    s = stats_summary(stats)
    n_surface = int((gb["surface_id"] >= 0).sum())
    assert s["checked"] == s["mlp_surface"] > 0
    assert s["mlp_surface"] + s["gated_surface"] <= n_surface
    assert 0.0 < s["check_rel_mean"] < 0.2
    r.close()


def test_tensor_core_timeout_takes_the_plain_path_and_is_reported(trained):
    """A wait bound of no polls makes every tensor-core completion wait give
    up at once.  Every MLP pixel must then take the plain path (surface pixels
    the limb integrator, sky pixels the sky-view LUT: the frame equals the
    plain frame), the timed-out tiles are counted, and the handle's next
    check reports ATM_E_TIMEOUT once, whether or not stats were passed."""

    from planet_renderer_gb300._native import ATM_E_TIMEOUT, AtmError
    from planet_renderer_gb300.atmosphere.surrogate import Surrogate

    sg_full, _, _ = trained
    sg = Surrogate(sg_full.aerial, sg_full.sky, sg_full.planet_radius_m, sg_full.top_altitude_m,
                   sg_full.scale_height_range)
    r, gb, args, _ = _frame(320, 180, 2000.0, 40.0, 30.0)
    plain = _plain(r, gb, args)
    r.check()
    sg.tc_wait_polls = -1
    got, stats = _surrogate(r, gb, args, sg)
    np.testing.assert_allclose(got.cpu().numpy(), plain.cpu().numpy(), rtol=2e-5, atol=1e-9)
    n_tiles = ((320 + 15) // 16) * ((180 + 15) // 16) * 2
    assert 0 < int(stats[7]) <= n_tiles
    assert int(stats[4]) == 0 and int(stats[5]) == 0  # no pixel kept a network output
    with pytest.raises(AtmError) as err:
        r.check()
    assert err.value.code == ATM_E_TIMEOUT
    r.check()  # reported once, then cleared
    hdr = torch.zeros_like(gb["scene_hdr"])
    r.composite_surrogate(gb["scene_hdr"], gb["space_hdr"], gb["surface_id"], gb["position_view"], hdr, *args,
                          surrogate=sg, stats=None, check_fraction=0.0)
    with pytest.raises(AtmError):
        r.check()
    # the library's own bound: no timeout, the networks' outputs are used
    sg.tc_wait_polls = 0
    _, stats = _surrogate(r, gb, args, sg)
    r.check()
    assert int(stats[7]) == 0 and int(stats[4]) > 0
    r.close()


def _fp64_pixels(r, gb, args, v, pixels, diagnostic_view=0, scene=None):
    """FP64 oracle composite at the given (x, y) pixels (own FP64 LUTs)."""

    from oracle.atm import Oracle
    from planet_renderer_gb300.atmosphere.config import earth_baseline

    o = Oracle("f64")
    cfg = earth_baseline()
    R, cr, sun, E_, disk, ar_deg, basis, tanfov, s0, s1 = args
    alt = cr - R
    ar = math.radians(ar_deg)
    tl = o.build_transmittance(cfg, R)
    ms = o.build_multi_scattering(cfg, R, E_, ar, tl)
    sv = o.build_sky_view(cfg, R, alt, float(sun[1]), E_, ar, tl, ms)
    W, H = r.width, r.height
    ap = np.zeros((cfg.aerial_lut_width, cfg.aerial_lut_height, cfg.aerial_lut_depth, 3))
    if diagnostic_view == 8:  # the froxel view reads the FP64 aerial volume
        ap = o.build_aerial(cfg, W, H, R, alt, sun, E_, ar, basis, tanfov, tl, ms)
    f = {k: gb[k].cpu().numpy().astype(np.float64) for k in ("scene_hdr", "space_hdr", "position_view")}
    if scene is not None:
        f["scene_hdr"] = scene
    plist = (pixels[:, 0].astype(np.int64) * H + pixels[:, 1]).astype(np.int32)
    hdr, _ = o.composite(cfg, f["scene_hdr"], f["space_hdr"], gb["surface_id"].cpu().numpy(), f["position_view"], R,
                         alt, alt, sun, E_, disk, ar, basis, tanfov, s0, s1, diagnostic_view, tl, ms, sv, ap,
                         pixel_list=plist)
    return hdr[pixels[:, 0], pixels[:, 1]]


def _rel(got, ref, floor):
    return np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor), axis=-1)


@pytest.mark.parametrize("altitude,zenith", [(2000.0, 40.0), (50_000.0, 60.0)])
def test_surrogate_frame_against_fp64(trained, altitude, zenith):
    """Composite radiance of the surrogate frame against the FP64 oracle at
    sampled surface pixels; the plain FP32 frame's own error is the yardstick.
    (The bench states the error of the fully trained networks.)"""

    sg, _, _ = trained
    r, gb, args, v = _frame(640, 360, altitude, zenith, 30.0)
    plain = _plain(r, gb, args).cpu().numpy()
    sg.calibration_tile = 0
    raw, _ = _surrogate(r, gb, args, sg, check_fraction=0.01)
    sg.calibration_tile = 64
    got, _ = _surrogate(r, gb, args, sg, check_fraction=0.01)
    raw, got = raw.cpu().numpy(), got.cpu().numpy()
    pixels = _surface_pixels(gb, 400)
    ref = _fp64_pixels(r, gb, args, v, pixels)
    floor = 1e-4 * np.abs(ref).max()
    e_mlp = _rel(got[pixels[:, 0], pixels[:, 1]], ref, floor)
    e_raw = _rel(raw[pixels[:, 0], pixels[:, 1]], ref, floor)
    e_plain = _rel(plain[pixels[:, 0], pixels[:, 1]], ref, floor)
    print(f"{altitude} m: plain {np.mean(e_plain):.2e} raw {np.mean(e_raw):.4f} calibrated {np.mean(e_mlp):.4f}")
    assert np.median(e_plain) < 1e-3
    # the reduced test budget (60 epochs); the bench states the fully trained
    # networks' error over the 64-frame sweep against the 1e-2 target
    assert np.mean(e_mlp) <= np.mean(e_raw) * 1.05
    assert np.mean(e_mlp) < 0.02, (np.mean(e_mlp), np.quantile(e_mlp, 0.99))
    r.close()


def _surface_pixels(gb, n, seed=1):
    sid = gb["surface_id"].cpu().numpy()
    xs, ys = np.nonzero(sid >= 0)
    pick = np.random.default_rng(seed).choice(len(xs), size=min(n, len(xs)), replace=False)
    return np.stack([xs[pick], ys[pick]], 1)


def test_calibration_corrects_a_biased_network(trained):
    """A planted bias: the aerial network's log-radiance outputs shifted by
    ln 1.2 (in-scattering about 20% high).  The calibration from the 1%
    checked pixels (64-pixel tiles) must take most of it out: against FP64
    at sampled surface pixels its mean error is below a third of the
    uncalibrated one; sky pixels are not touched."""

    from planet_renderer_gb300.atmosphere.mlp import Mlp
    from planet_renderer_gb300.atmosphere.surrogate import Surrogate

    sg_full, _, _ = trained
    biased = Mlp(11, 4, 6, device=sg_full.aerial.device)
    p = sg_full.aerial.params()
    p[-6:-3] += math.log(1.2)
    biased.set_params(p)
    sg = Surrogate(biased, None, sg_full.planet_radius_m, sg_full.top_altitude_m, sg_full.scale_height_range)
    r, gb, args, v = _frame(640, 360, 2000.0, 40.0, 30.0)
    sg.calibration_tile = 0
    raw, _ = _surrogate(r, gb, args, sg, check_fraction=0.01)
    sg.calibration_tile = 64
    cal, stats = _surrogate(r, gb, args, sg, check_fraction=0.01)
    raw, cal = raw.cpu().numpy(), cal.cpu().numpy()
    sky = gb["surface_id"].cpu().numpy() < 0
    np.testing.assert_array_equal(cal[sky], raw[sky])
    pixels = _surface_pixels(gb, 400)
    ref = _fp64_pixels(r, gb, args, v, pixels)
    floor = 1e-4 * np.abs(ref).max()
    e_raw = _rel(raw[pixels[:, 0], pixels[:, 1]], ref, floor).mean()
    e_cal = _rel(cal[pixels[:, 0], pixels[:, 1]], ref, floor).mean()
    print(f"planted 20% bias: raw {e_raw:.4f} calibrated {e_cal:.4f}")
    assert e_raw > 0.05
    assert e_cal < e_raw / 3.0, (e_raw, e_cal)
    r.close()


def test_surrogate_frame_gains_over_the_plain_integrator(trained):
    """What the network gains over the method without it (the plain limb
    integrator of every surface pixel): the surrogate composite of a
    3840x2160 frame from 2 km, with its 1% checks and the calibration pass,
    is at least three times as fast (the target), with its error against
    FP64 stated by test_surrogate_frame_against_fp64."""

    sg, _, _ = trained
    r, gb, args, _ = _frame(3840, 2160, 2000.0, 40.0, 30.0)
    hdr = torch.zeros_like(gb["scene_hdr"])

    def timed(fn, reps=5):
        for _ in range(2):
            fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    plain = timed(lambda: r.composite(gb["scene_hdr"], gb["space_hdr"], gb["surface_id"], gb["position_view"], hdr,
                                      *args))
    mlp = timed(lambda: r.composite_surrogate(gb["scene_hdr"], gb["space_hdr"], gb["surface_id"], gb["position_view"],
                                              hdr, *args, surrogate=sg, check_fraction=0.01, seed=1))
    print(f"4K composite: plain {plain:.3f} ms, surrogate {mlp:.3f} ms, {plain / mlp:.2f}x")
    assert plain / mlp > 3.0, (plain, mlp)
    r.close()


# ---- the learned sky-view workload: sky radiance of every pixel ---------------------
def _sky_frame(width=320, height=180, altitude_m=2000.0, zenith_deg=40.0, pitch_deg=15.0):
    from planet_renderer_gb300 import camera
    from planet_renderer_gb300.atmosphere import AtmosphereRenderer
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M

    r = AtmosphereRenderer(width, height, earth_baseline())
    sun = camera.sun_from_zenith(zenith_deg, 30.0)
    basis = camera.view_basis(0.0, pitch_deg)
    tanfov = camera.tangent_half_fov(60.0)
    cr = EARTH_RADIUS_M + altitude_m
    r.update(EARTH_RADIUS_M, cr, sun.copy(), E, AR_DEG)
    args = (EARTH_RADIUS_M, cr, sun, E, AR_DEG, basis, tanfov)
    return r, args


def _sky(r, args, mode, surrogate=None):
    out = torch.full((r.width, r.height, 3), -1.0, device=r.device)
    r.sky_pixels(out, *args, mode=mode, surrogate=surrogate)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_sky_pixels_plain_matches_the_oracle_march():
    """The plain per-pixel integrator is the sky-view LUT's march along each
    pixel's own ray: against the oracle's restatement (float32) at every
    pixel of a small frame looking above and below the horizon, with the
    radiance-sample count."""

    from conftest import assert_parity
    from oracle.atm import Oracle
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.scene import pixel_rays

    r, args = _sky_frame(96, 54, pitch_deg=5.0)
    R, cr, sun, E_, ar_deg, basis, tanfov = args
    r.radiance_samples(reset=True)
    got = _sky(r, args, "plain")
    assert r.radiance_samples() == 96 * 54 * earth_baseline().sky_view_steps
    xs = torch.arange(96).repeat_interleave(54)
    ys = torch.arange(54).repeat(96)
    rays = pixel_rays(96, 54, basis, tanfov, xs, ys).double().numpy()
    o = Oracle("f32")
    cfg = earth_baseline()
    ar = math.radians(ar_deg)
    tl = o.build_transmittance(cfg, R)
    ms = o.build_multi_scattering(cfg, R, E_, ar, tl)
    ref = o.sky_rays(cfg, R, np.full(len(rays), cr - R), rays, np.tile(sun, (len(rays), 1)), E_, ar, tl, ms)
    assert_parity(got.reshape(-1, 3), ref, "sky pixels (plain)")
    r.close()


def test_sky_pixels_lut_is_the_composite_sky():
    """The LUT mode is the plain composite's sky radiance: a frame of sky
    pixels with no scene or stars composites to the same values away from
    the sun's disk."""

    from planet_renderer_gb300.lighting import LightingState

    r, args = _sky_frame(160, 90, pitch_deg=20.0)
    R, cr, sun, E_, ar_deg, basis, tanfov = args
    got = _sky(r, args, "lut")
    zero = torch.zeros((160, 90, 3), device=r.device)
    sid = torch.full((160, 90), -1, dtype=torch.int32, device=r.device)
    hdr = torch.zeros_like(zero)
    r.prepare_frame(zero, sid, R, cr, sun, E_, ar_deg, basis, tanfov)
    r.composite(zero, zero, sid, zero, hdr, R, cr, sun, E_, LightingState(sun, ar_deg, E_).sun_disk_radiance, ar_deg,
                basis, tanfov, 4.0, 12.0)
    from planet_renderer_gb300.atmosphere.scene import pixel_rays

    rays = pixel_rays(160, 90, basis, tanfov, torch.arange(160).repeat_interleave(90),
                      torch.arange(90).repeat(160)).numpy().reshape(160, 90, 3)
    away = np.degrees(np.arccos(np.clip(rays @ np.asarray(sun), -1, 1))) > 3.0  # outside the disk's smoothing
    assert away.mean() > 0.9
    np.testing.assert_array_equal(np.maximum(got, 0.0)[away], hdr.cpu().numpy()[away])
    r.close()


def test_sky_pixels_network_against_the_plain_integrator(trained):
    """The network mode at the reduced training budget: close to the plain
    integrator at every pixel (the bench states the full budget's error
    against FP64); with every pixel gated it is the plain integrator; with no
    polls allowed it falls back to the plain integrator and reports the
    timeout."""

    from planet_renderer_gb300._native import ATM_E_TIMEOUT, AtmError
    from planet_renderer_gb300.atmosphere.surrogate import Surrogate

    sg_full, _, _ = trained
    sg = Surrogate(None, sg_full.sky, sg_full.planet_radius_m, sg_full.top_altitude_m, sg_full.scale_height_range)
    r, args = _sky_frame(320, 180, pitch_deg=15.0)
    plain = _sky(r, args, "plain")
    floor = 1e-4 * np.abs(plain).max()
    rel = lambda img: np.max(np.abs(img - plain) / np.maximum(np.abs(plain), floor), axis=-1)
    sg.calibration_tile = 0
    e_raw = rel(_sky(r, args, "net", sg))
    sg.calibration_tile = 32  # 32x32 tiles: about 10 checks each at 1%
    e = rel(_sky(r, args, "net", sg))
    print(f"sky network: raw {np.mean(e_raw):.4f} calibrated {np.mean(e):.4f}")
    # the reduced training budget (the sky network's held-out error bound of
    # test_training_learns_both_networks is 0.15); the calibration from the
    # 1% checked pixels must not make it worse
    assert np.mean(e_raw) < 0.25, (np.mean(e_raw), np.quantile(e_raw, 0.99))
    assert np.mean(e) <= np.mean(e_raw) * 1.02, (np.mean(e), np.mean(e_raw))
    sg.sky_twilight_cosine = 1.0  # gate every pixel
    np.testing.assert_allclose(_sky(r, args, "net", sg), plain, rtol=1e-6, atol=0)
    sg.sky_twilight_cosine = 0.1
    sg.tc_wait_polls = -1
    np.testing.assert_allclose(_sky(r, args, "net", sg), plain, rtol=1e-6, atol=0)
    with pytest.raises(AtmError) as err:
        r.check()
    assert err.value.code == ATM_E_TIMEOUT
    r.close()
