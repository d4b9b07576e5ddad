"""Algorithmic operation counts of the atmosphere kernels (test infrastructure).

    python oracle/count_flops.py [--stride 16]

Runs the oracle's op-counting instantiation (every add/sub, mul, div, sqrt
and transcendental of the reference algorithm, ``atm_oracle.cpp`` CountF) on
the full-frame workload: Earth parameter set at the plain LUT-build sizes,
1920x1080, the three cameras of ``workloads.frame_chain_cameras`` (2 km /
50 km / 2000 km altitude, pitch -35 deg, stratified sun zeniths, seed 2027).  The composite is
counted on every ``stride``-th pixel in x and y and scaled to the frame.
Prints per-kernel totals and per-radiance-sample figures; FLOP counts
add/sub + mul + div + sqrt as one each (an FMA in the source is two).
"""

from __future__ import annotations

import argparse
import ctypes
import json
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "planet-real-time-render_gb300"))

from oracle.atm import AtmParams, CompositeArgs, library, params_from_config, sun_disk_radiance  # noqa: E402

OPS = ["add", "mul", "div", "sqrt", "exp", "acos", "cos_sin", "pow", "atan2"]


def bench_cameras(seed: int = 2027):
    from planet_renderer_gb300.atmosphere.workloads import frame_chain_cameras

    return [(v.altitude_m, v.sun_zenith_deg, v.sun_azimuth_deg) for v in frame_chain_cameras(seed)]


def _counts(lib, reset=True):
    out = (ctypes.c_uint64 * 9)()
    lib.orc_op_counts(out, 1 if reset else 0)
    return dict(zip(OPS, [int(v) for v in out]))


def _flops(c):
    return c["add"] + c["mul"] + c["div"] + c["sqrt"]


def count(stride: int = 16, width: int = 1920, height: int = 1080) -> dict:
    import torch

    from planet_renderer_gb300 import camera
    from planet_renderer_gb300.atmosphere import scene
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from oracle.atm import Oracle

    lib = library()
    lib.orc_set_threads(1)
    f32 = Oracle("f32")
    cfg = earth_baseline()
    p = params_from_config(cfg)
    R = 6_360_000.0
    E = (4.0, 3.9, 3.7)
    ar_deg = 0.266
    ar = math.radians(ar_deg)
    ar_key = float(np.float32(ar))
    d3 = ctypes.c_double * 3
    vp = ctypes.c_void_p

    def ptr(a):
        return a.ctypes.data_as(vp)

    result = {}
    _counts(lib)
    tlut = np.zeros((cfg.transmittance_lut_width, cfg.transmittance_lut_height, 3), np.float32)
    lib.orc_build_transmittance_cnt.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_double, vp]
    lib.orc_build_transmittance_cnt(ctypes.byref(p), R, ptr(tlut))
    c = _counts(lib)
    n = cfg.transmittance_lut_width * cfg.transmittance_lut_height * cfg.transmittance_steps
    result["transmittance"] = {"ops": c, "samples": n, "flop_per_sample": _flops(c) / n}

    tlut = f32.build_transmittance(cfg, R)
    ms = np.zeros((cfg.multi_scattering_lut_width, cfg.multi_scattering_lut_height, 3), np.float32)
    fn = lib.orc_build_multi_scattering_cnt
    fn.restype = ctypes.c_int64
    fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_double, d3, ctypes.c_double, vp, vp]
    n = fn(ctypes.byref(p), R, d3(*E), ar_key, ptr(tlut), ptr(ms))
    c = _counts(lib)
    result["multi_scattering"] = {"ops": c, "samples": int(n), "flop_per_sample": _flops(c) / n}
    mslut = f32.build_multi_scattering(cfg, R, E, ar_key, tlut)

    per_camera = []
    for altitude, zenith, azimuth in bench_cameras():
        basis = camera.view_basis(0.0, -35.0)
        tanfov = camera.tangent_half_fov(60.0)
        sun = camera.sun_from_zenith(zenith, azimuth)
        alt_key = float(np.float32(altitude))
        sun_cos = float(np.float32(sun[1]))
        # sky-view
        sv = np.zeros((cfg.sky_view_lut_width, cfg.sky_view_lut_height, 3), np.float32)
        fn = lib.orc_build_sky_view_cnt
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_double, ctypes.c_double, ctypes.c_double, d3,
                       ctypes.c_double, vp, vp, vp]
        fn(ctypes.byref(p), R, alt_key, sun_cos, d3(*E), ar_key, ptr(tlut), ptr(mslut), ptr(sv))
        c_sv = _counts(lib)
        # aerial
        ap = np.zeros((cfg.aerial_lut_width, cfg.aerial_lut_height, cfg.aerial_lut_depth, 3), np.float32)
        fn = lib.orc_build_aerial_cnt
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, d3,
                       d3, ctypes.c_double, d3, d3, d3, ctypes.c_double, vp, vp, vp]
        fn(ctypes.byref(p), width, height, R, altitude, d3(*sun), d3(*E), ar, d3(*basis[0]), d3(*basis[1]),
           d3(*basis[2]), tanfov, ptr(tlut), ptr(mslut), ptr(ap))
        c_ap = _counts(lib)
        # composite on a pixel grid
        xs, ys = np.meshgrid(np.arange(stride // 2, width, stride), np.arange(stride // 2, height, stride),
                             indexing="ij")
        pix = np.stack([xs.ravel(), ys.ravel()], 1)
        gb = scene.synthesize_gbuffer(width, height, R, altitude, basis, tanfov, sun, E, pixels=torch.as_tensor(pix))
        frame = {k: np.zeros((width, height) + tuple(v.shape[1:]), np.float32 if k != "surface_id" else np.int32)
                 for k, v in gb.items()}
        frame["surface_id"][:] = -1
        for k, v in gb.items():
            frame[k][pix[:, 0], pix[:, 1]] = v.numpy()
        plist = (pix[:, 0] * height + pix[:, 1]).astype(np.int32)
        sv32 = f32.build_sky_view(cfg, R, alt_key, sun_cos, E, ar_key, tlut, mslut)
        ap32 = f32.build_aerial(cfg, width, height, R, altitude, sun, E, ar, basis, tanfov, tlut, mslut)
        a = CompositeArgs()
        a.width, a.height, a.diagnostic_view = width, height, 0
        a.bottom, a.cam_alt, a.sky_alt, a.ar, a.tanfov = R, altitude, alt_key, ar, tanfov
        a.star_start, a.star_end = 4.0, 12.0
        a.sun[:], a.E[:], a.disk[:] = list(sun), list(E), list(sun_disk_radiance(E, ar_deg))
        a.right[:], a.up[:], a.fwd[:] = list(basis[0]), list(basis[1]), list(basis[2])
        hdr = np.zeros((width, height, 3), np.float32)
        fn = lib.orc_composite_cnt
        fn.restype = ctypes.c_int64
        fn.argtypes = [ctypes.POINTER(AtmParams), ctypes.POINTER(CompositeArgs), ctypes.c_int, ctypes.c_int,
                       ctypes.c_int] + [vp] * 9 + [vp, ctypes.c_int64]
        samples = fn(ctypes.byref(p), ctypes.byref(a), height, 1, 3, ptr(frame["scene_hdr"]), ptr(frame["space_hdr"]),
                     ptr(frame["surface_id"]), ptr(frame["position_view"]), ptr(tlut), ptr(mslut), ptr(sv32),
                     ptr(ap32), ptr(hdr), ptr(plist), plist.size)
        c_co = _counts(lib)
        scale = (width * height) / plist.size
        surface_frac = float((gb["surface_id"].numpy() >= 0).mean())
        per_camera.append({
            "altitude_m": altitude, "sun_zenith_deg": zenith, "sun_azimuth_deg": azimuth,
            "sky_view": {"ops": c_sv, "flop": _flops(c_sv)},
            "aerial": {"ops": c_ap, "flop": _flops(c_ap)},
            "composite": {"ops_subset": c_co, "samples_subset": int(samples), "pixels_subset": int(plist.size),
                          "frame_flop_est": _flops(c_co) * scale, "frame_samples_est": samples * scale,
                          "surface_fraction": surface_frac,
                          "flop_per_sample": _flops(c_co) / max(samples, 1)},
        })
    result["cameras"] = per_camera
    tot_f = sum(c["composite"]["frame_flop_est"] for c in per_camera)
    tot_s = sum(c["composite"]["frame_samples_est"] for c in per_camera)
    result["composite_flop_per_sample"] = tot_f / tot_s
    lib.orc_set_threads(0)
    return result


if __name__ == "__main__":
    parser = argparse.ArgumentParser()
    parser.add_argument("--stride", type=int, default=16)
    args = parser.parse_args()
    print(json.dumps(count(args.stride), indent=1))
