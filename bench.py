#!/usr/bin/env python
"""Benchmark of the GB300 atmosphere path (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one "step": 16 passes over the three cameras): the plain
per-frame chain of the reference's frame scheduler (atmosphere/renderer.py
update -> prepare_frame -> composite) at 1920x1080 FP32 for the three
cameras of ``workloads.frame_chain_cameras``
(2 km, 50 km, 2000 km altitude; pitch -35 deg; stratified sun zeniths in
[0, 100] deg; seed 2027) on a seeded fBm G-buffer (+/- 4 km).  Per camera the
chain is: sky-view LUT rebuild (a moving camera changes its key every frame),
surface lighting + aerial-perspective volume, composite.  Transmittance and
multi-scattering LUTs depend only on the parameter set and are built once.
Each camera's chain is captured in a CUDA graph and replayed.

Metric: radiance samples per second (one constant-source segment of the
reference's _scattering_segment, counted on the device by the kernels), and
frame milliseconds.  ``e2e`` is the same metric through the public Python API
(AtmosphereRenderer) with host buffers: pinned host -> device copies of the
G-buffer inputs and the device -> host copy of ``hdr`` inside the timed
region.  ``roofline`` is for the composite kernel, which dominates the step:
it is FP32/SFU-bound, so its roofline is FP32 throughput (algorithmic FLOPs
counted by ``oracle/count_flops.py`` over the same workload) against
152 SMs x 128 lanes x 2 FLOP x the SM clock sampled during the run;
``roofline_hbm`` gives its algorithmic DRAM bytes against the measured copy
bandwidth.  ``cpu_baseline`` times the oracle (a port of the reference's
algorithm, OpenMP over all host cores) on a bounded sample of the workload.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "planet-real-time-render_gb300", ROOT):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "atm. radiance samples/s & 4K frame ms: MLP vs plain integrator at ≤1e-2 rel err"
UNIT = "radiance samples/s"
WIDTH, HEIGHT = 1920, 1080
SEED = 2027
# Algorithmic FP32 operations (add/sub + mul + div + sqrt, an FMA counting 2)
# per radiance sample of the composite, over this workload, from
# `python oracle/count_flops.py --stride 32` (op-counting instantiation of the
# oracle restatement); includes the per-pixel and per-interval set-up.
COMPOSITE_FLOP_PER_SAMPLE = 406.16
# DRAM bytes a composite pixel must move: position 12 + surface_id 4 +
# scene 12 + space 12 read, hdr 12 written (LUTs stay in L2).
COMPOSITE_BYTES_PER_PIXEL = 52
# DRAM bytes (read + write) of one k_composite launch of the 2 km camera at
# 1920x1080, from `ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum`
# on `bench.py --profile-case frame1080p` (58,468,352 + 3,072,256)
COMPOSITE_DRAM_BYTES_1080P = 58_468_352 + 3_072_256
MLP_CHECK_FRACTION = 0.01  # share of MLP pixels the plain path re-integrates
# A step is this many passes of the three cameras' chains (48 frames of
# 1080p, ~57 ms): with the usual 20 timed steps the timed region lasts over a
# second.  Every pass redoes the whole chain (sky-view rebuild, surface
# lighting, aerial volume, composite) on inputs larger than L2.
PASSES_PER_STEP = 16
SMS, FP32_LANES = 152, 128


def _peaks() -> dict:
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        return json.loads(path.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


class ClockSampler:
    """nvidia-smi clock/throttle sampling at 200 ms during a timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.file.seek(0)
        rows = [line.split(",") for line in self.file.read().splitlines() if line.count(",") >= 8]
        os.unlink(self.file.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for name, value in zip(names, r[5:9]):
                if "Active" in value and "Not" not in value:
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _setup_chain(device, width, height):
    import torch

    from planet_renderer_gb300.atmosphere import AtmosphereRenderer, scene
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.workloads import (EARTH_RADIUS_M, SOLAR_IRRADIANCE,
                                                            SUN_ANGULAR_RADIUS_DEG, frame_chain_cameras)
    from planet_renderer_gb300.lighting import LightingState

    cfg = earth_baseline()
    views = frame_chain_cameras(SEED)
    r = AtmosphereRenderer(width, height, cfg, device=device)
    frames = []
    for v in views:
        gb = scene.synthesize_gbuffer(width, height, EARTH_RADIUS_M, v.altitude_m, v.basis, v.tangent_half_fov,
                                      v.sun_local, SOLAR_IRRADIANCE, seed=SEED, device=device)
        gb["hdr"] = torch.zeros_like(gb["scene_hdr"])
        light = LightingState(v.sun_local, SUN_ANGULAR_RADIUS_DEG, SOLAR_IRRADIANCE)
        frames.append((v, gb, light))
    sun0 = views[0].sun_local
    r.update(EARTH_RADIUS_M, views[0].camera_radius_m, sun0.copy(), SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG)
    torch.cuda.synchronize(device)
    return r, cfg, frames


def _chain(r, v, gb, light):
    """One frame of the plain chain for camera view v: update (the sky-view
    LUT rebuilds, its key changes with every camera) -> prepare_frame ->
    composite, as the reference's frame scheduler calls them."""

    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG

    sun = v.sun_local
    r.update(EARTH_RADIUS_M, v.camera_radius_m, sun, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG)
    r.prepare_frame(gb["position_view"], gb["surface_id"], EARTH_RADIUS_M, v.camera_radius_m, sun, SOLAR_IRRADIANCE,
                    SUN_ANGULAR_RADIUS_DEG, v.basis, v.tangent_half_fov)
    r.composite(gb["scene_hdr"], gb["space_hdr"], gb["surface_id"], gb["position_view"], gb["hdr"], EARTH_RADIUS_M,
                v.camera_radius_m, sun, SOLAR_IRRADIANCE, light.sun_disk_radiance, SUN_ANGULAR_RADIUS_DEG, v.basis,
                v.tangent_half_fov, 4.0, 12.0)


def _f32(x):
    import numpy as np

    return np.float32(x)


def _capture(r, frames, device):
    import torch

    graphs = []
    side = torch.cuda.Stream(device)
    side.wait_stream(torch.cuda.current_stream(device))
    with torch.cuda.stream(side):
        for v, gb, light in frames:  # warm-up outside capture
            _chain(r, v, gb, light)
    torch.cuda.current_stream(device).wait_stream(side)
    torch.cuda.synchronize(device)
    for v, gb, light in frames:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            _chain(r, v, gb, light)
        graphs.append(g)
    torch.cuda.synchronize(device)
    return graphs


def _timed_graph_region(graphs, steps, device):
    import torch

    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    start.record()
    for _ in range(steps):
        for g in graphs:
            g.replay()
    end.record()
    torch.cuda.synchronize(device)
    return start.elapsed_time(end)


def _composite_kernel_times(r, frames, reps, device):
    """CUDA-event duration of each composite launch (eager, same stream)."""

    import torch

    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG

    per_camera = []
    for v, gb, light in frames:
        _chain(r, v, gb, light)
        events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in events:
            a.record()
            r.composite(gb["scene_hdr"], gb["space_hdr"], gb["surface_id"], gb["position_view"], gb["hdr"],
                        EARTH_RADIUS_M, v.camera_radius_m, v.sun_local, SOLAR_IRRADIANCE, light.sun_disk_radiance,
                        SUN_ANGULAR_RADIUS_DEG, v.basis, v.tangent_half_fov, 4.0, 12.0)
            b.record()
        torch.cuda.synchronize(device)
        per_camera.append(statistics.mean(a.elapsed_time(b) for a, b in events))
    return per_camera


def _e2e(r, frames, steps, warmup, device):
    """Public API with pinned host buffers, copies inside the timed region.

    Copies run on a copy stream ordered by events against the compute
    stream, so camera k+1's upload and camera k-1's read-back overlap camera
    k's kernels (the renderer's LUTs serialise the cameras on the compute
    stream).  Each step ends with every hdr image back in host memory."""

    import torch

    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG

    host = []
    h2d = d2h = 0
    for v, gb, light in frames:
        hin = {k: gb[k].cpu().pin_memory() for k in ("position_view", "surface_id", "scene_hdr", "space_hdr")}
        hout = torch.empty(gb["hdr"].shape, dtype=torch.float32, pin_memory=True)
        dev = {k: torch.empty_like(gb[k]) for k in hin}
        dev["hdr"] = torch.empty_like(gb["hdr"])
        host.append((v, light, hin, hout, dev))
        h2d += sum(t.numel() * t.element_size() for t in hin.values())
        d2h += hout.numel() * hout.element_size()
    compute = torch.cuda.current_stream(device)
    copy = torch.cuda.Stream(device)

    def step(k):
        uploaded = []
        with torch.cuda.stream(copy):
            for _, _, hin, _, dev in host:
                for name, t in hin.items():
                    dev[name].copy_(t, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(copy)
                uploaded.append(ev)
        for (v, light, hin, hout, dev), ev in zip(host, uploaded):
            compute.wait_event(ev)
            radius = v.camera_radius_m + (0.5 if k % 2 else 0.0)  # moving camera: new sky-view key
            r.update(EARTH_RADIUS_M, radius, v.sun_local, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG)
            r.prepare_frame(dev["position_view"], dev["surface_id"], EARTH_RADIUS_M, radius, v.sun_local,
                            SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG, v.basis, v.tangent_half_fov)
            r.composite(dev["scene_hdr"], dev["space_hdr"], dev["surface_id"], dev["position_view"], dev["hdr"],
                        EARTH_RADIUS_M, radius, v.sun_local, SOLAR_IRRADIANCE, light.sun_disk_radiance,
                        SUN_ANGULAR_RADIUS_DEG, v.basis, v.tangent_half_fov, 4.0, 12.0)
            done = torch.cuda.Event()
            done.record(compute)
            copy.wait_event(done)
            with torch.cuda.stream(copy):
                hout.copy_(dev["hdr"], non_blocking=True)
        copy.synchronize()
        compute.synchronize()

    for k in range(warmup):
        step(k)
    r.radiance_samples(reset=True)
    t0 = time.perf_counter()
    for k in range(steps):
        step(k)
    elapsed = time.perf_counter() - t0
    samples = r.radiance_samples(reset=True)
    return elapsed, samples, h2d, d2h


def _cpu_baseline(frames_cpu, cfg, stride, threads=None):
    """Oracle port over all host cores on every stride-th pixel (x and y)."""

    import numpy as np

    from oracle.atm import Oracle
    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG

    o = Oracle("f32", threads=threads)
    cores = int(o.lib.orc_max_threads())
    R = EARTH_RADIUS_M
    ar = math.radians(SUN_ANGULAR_RADIUS_DEG)
    ar_key = float(np.float32(ar))
    t0 = time.perf_counter()
    tl = o.build_transmittance(cfg, R)
    ms = o.build_multi_scattering(cfg, R, SOLAR_IRRADIANCE, ar_key, tl)
    t_static = time.perf_counter() - t0
    samples, seconds, pixels = 0, 0.0, 0
    for v, host, light in frames_cpu:
        W, H = host["surface_id"].shape
        xs, ys = np.meshgrid(np.arange(0, W, stride), np.arange(0, H, stride), indexing="ij")
        plist = (xs.ravel() * H + ys.ravel()).astype(np.int32)
        t0 = time.perf_counter()
        sv = o.build_sky_view(cfg, R, float(np.float32(v.altitude_m)), float(np.float32(v.sun_local[1])),
                              SOLAR_IRRADIANCE, ar_key, tl, ms)
        ap = o.build_aerial(cfg, W, H, R, v.altitude_m, v.sun_local, SOLAR_IRRADIANCE, ar, v.basis,
                            v.tangent_half_fov, tl, ms)
        _, n = o.composite(cfg, host["scene_hdr"], host["space_hdr"], host["surface_id"], host["position_view"], R,
                           v.altitude_m, float(np.float32(v.altitude_m)), v.sun_local, SOLAR_IRRADIANCE,
                           light.sun_disk_radiance, ar, v.basis, v.tangent_half_fov, 4.0, 12.0, 0, tl, ms, sv, ap,
                           pixel_list=plist)
        seconds += time.perf_counter() - t0
        sv_n = cfg.sky_view_lut_width * cfg.sky_view_lut_height * cfg.sky_view_steps
        ap_n = cfg.aerial_lut_width * cfg.aerial_lut_height * cfg.aerial_lut_depth * cfg.aerial_steps_per_slice
        samples += n + sv_n + ap_n
        pixels += plist.size
    return {
        "value": samples / seconds,
        "unit": UNIT,
        "cores": cores,
        "kind": "port",
        "sample": (f"oracle FP32 restatement (oracle/atm_oracle.cpp, OpenMP) on the same 3-camera frame chain: "
                   f"full sky-view + aerial LUTs and the composite of every {stride}th pixel in x and y "
                   f"({pixels} px); {samples} radiance samples in {seconds:.2f} s "
                   f"(sky-view/aerial counted as texels x steps); static T+MS build {t_static:.2f} s not timed"),
        "seconds": seconds,
    }


def run_reference(args) -> None:
    """The reference arm: the reference algorithm's CPU implementation (the
    oracle port: Taichi cannot be installed here) on all host cores."""

    world, rank, _ = _dist()
    if rank != 0:
        return
    import torch

    from oracle import build_oracle
    from planet_renderer_gb300.atmosphere import scene
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG
    from planet_renderer_gb300.atmosphere.workloads import frame_chain_cameras
    from planet_renderer_gb300.lighting import LightingState

    build_oracle.build()
    cfg = earth_baseline()
    frames = []
    for v in frame_chain_cameras(SEED):
        gb = scene.synthesize_gbuffer(WIDTH, HEIGHT, EARTH_RADIUS_M, v.altitude_m, v.basis, v.tangent_half_fov,
                                      v.sun_local, SOLAR_IRRADIANCE, seed=SEED,
                                      device="cuda" if torch.cuda.is_available() else "cpu")
        frames.append((v, {k: t.cpu().numpy() for k, t in gb.items()},
                       LightingState(v.sun_local, SUN_ANGULAR_RADIUS_DEG, SOLAR_IRRADIANCE)))
    values, secs = [], []
    for _ in range(args.warmup):
        _cpu_baseline(frames, cfg, args.ref_stride * 2)
    for _ in range(args.steps):
        b = _cpu_baseline(frames, cfg, args.ref_stride)
        values.append(b["value"])
        secs.append(b["seconds"])
    value = statistics.mean(values)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": _config_block(), "cpu_baseline": {k: v for k, v in b.items() if k != "seconds"} | {"value": value},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_note": "Taichi (the reference's runtime) is not installable on this box; the reference arm runs "
                          "the oracle restatement of its kernels, pinned to the reference's own source by golden "
                          "vectors (tests/golden)",
    }
    print(json.dumps(line), flush=True)


def _config_block(extra=None) -> dict:
    block = {
        "workload": "plain per-frame chain (sky-view rebuild + surface lighting + aerial volume + composite), "
                    "1920x1080 FP32, 3 cameras (2 km / 50 km / 2000 km, pitch -35 deg, stratified sun zenith "
                    "0-100 deg), seeded fBm G-buffer +/-4 km, CUDA graph per camera",
        "width": WIDTH, "height": HEIGHT, "cameras": 3, "passes_per_step": PASSES_PER_STEP, "seed": SEED,
        "params": "Earth: R 6360 km, top 100 km, Mie ext 8.396e-6; T 256x64/40, MS 32x32 64 dirs x 20 steps, "
                  "SV 192x108/30, AP 32x32x32 x2, 48 limb intervals, 8 terminator substeps",
        "l2": "inputs larger than L2 (3 cameras x 108 MB of G-buffer + hdr per step)",
    }
    if extra:
        block.update(extra)
    return block


def main() -> None:
    parser = argparse.ArgumentParser()
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=20,
                        help=f"timed steps of {PASSES_PER_STEP} passes of the 3-camera 1080p chain each")
    parser.add_argument("--warmup", type=int, default=5)
    parser.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    parser.add_argument("--cpu-stride", type=int, default=1,
                        help="cpu_baseline leg: composite every n-th pixel in x and y")
    parser.add_argument("--ref-stride", type=int, default=4,
                        help="reference arm: pixel stride of each step's bounded sample")
    parser.add_argument("--no-cpu-baseline", action="store_true")
    parser.add_argument("--no-4k", action="store_true")
    parser.add_argument("--no-batch", action="store_true")
    parser.add_argument("--no-mlp", action="store_true", help="skip the surrogate frame (training + timing)")
    parser.add_argument("--mlp-epochs", type=int, default=400, help="surrogate training epochs (2^22 samples)")
    parser.add_argument("--no-post", action="store_true", help="skip the 4K display post-process timing")
    parser.add_argument("--no-luts", action="store_true", help="skip the plain LUT-build timing")
    parser.add_argument("--no-raster", action="store_true", help="skip the 4K terrain raster timing")
    parser.add_argument("--mlp-sweep", type=int, default=64,
                        help="also run the aerial-surrogate frame workload over this many 4K frames with cameras "
                             "log-uniform 1 m - 4000 km (e.g. 64)")
    parser.add_argument("--profile-case", choices=sorted(PROFILE_CASES),
                        help="run one small case for an ncu capture instead of the benchmark (prints one line)")
    args = parser.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return
    if args.profile_case:
        PROFILE_CASES[args.profile_case](args)
        return

    import torch
    import torch.distributed as dist

    world, rank, local = _dist()
    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)
    if world > 1:
        dist.init_process_group("nccl", device_id=device)

    r, cfg, frames = _setup_chain(device, WIDTH, HEIGHT)
    graphs = _capture(r, frames, device)
    # radiance samples per step (device counters of the captured kernels)
    r.radiance_samples(reset=True)
    for g in graphs:
        g.replay()
    samples_per_step = PASSES_PER_STEP * r.radiance_samples(reset=True)
    for _ in range(args.warmup * PASSES_PER_STEP):
        for g in graphs:
            g.replay()
    torch.cuda.synchronize(device)
    sampler = ClockSampler(local)
    if world > 1:
        dist.barrier()
    sampler.start()
    ms_total = _timed_graph_region(graphs, args.steps * PASSES_PER_STEP, device)
    clocks = sampler.stop()
    if world > 1:
        dist.barrier()
        t = torch.tensor([ms_total], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_total = float(t.item())
    ms_per_step = ms_total / args.steps
    value = world * samples_per_step * args.steps / (ms_total / 1e3)

    # per-launch composite timing for the roofline
    r.radiance_samples(reset=True)
    comp_samples = []
    for v, gb, light in frames:
        _chain(r, v, gb, light)
    for v, gb, light in frames:
        r.radiance_samples(reset=True)
        r.composite(gb["scene_hdr"], gb["space_hdr"], gb["surface_id"], gb["position_view"], gb["hdr"],
                    *_composite_args(v, light))
        comp_samples.append(r.radiance_samples(reset=True))
    comp_ms = _composite_kernel_times(r, frames, 20, device)
    flops = [n * COMPOSITE_FLOP_PER_SAMPLE for n in comp_samples]
    achieved_tflops = sum(flops) / (sum(comp_ms) / 1e3) / 1e12
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    peak_tflops = SMS * FP32_LANES * 2 * sm_mhz * 1e6 / 1e12
    peaks = _peaks()
    comp_bytes = WIDTH * HEIGHT * COMPOSITE_BYTES_PER_PIXEL
    achieved_gbs = comp_bytes / (statistics.mean(comp_ms) / 1e3) / 1e9

    e2e_steps = 100
    e2e_s, e2e_samples, h2d, d2h = _e2e(r, frames, e2e_steps, 2, device)

    leg_s = {}  # wall seconds of each leg (host time, including its checks against the FP64 oracle)

    def leg(name, skip, fn):
        if skip:
            return None
        t0 = time.perf_counter()
        out = fn()
        leg_s[name] = round(time.perf_counter() - t0, 1)
        return out

    luts = leg("lut_build", args.no_luts, lambda: _lut_builds(device, args))
    frame_4k = leg("frame_4k", args.no_4k, lambda: _frame_4k(device, args))
    batch = leg("batch", args.no_batch, lambda: _batch(device, args))
    post = leg("postprocess_4k", args.no_post, lambda: _postprocess_4k(device, args))
    shade = leg("shading_4k", args.no_post, lambda: _shading_4k(device, args))
    raster = leg("raster_4k", args.no_raster, lambda: _raster_4k(device, args))
    mesh_frame = (frame_4k or {}).pop("mesh_4k", None)
    if mesh_frame is None:
        mesh_frame = leg("frame_from_mesh_4k", args.no_raster, lambda: _frame_from_mesh_4k(device, args))

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        host_frames = [(v, {k: gb[k].cpu().numpy() for k in ("position_view", "surface_id", "scene_hdr",
                                                               "space_hdr")}, light) for v, gb, light in frames]
        # repeat the bounded sample until about 8 s of CPU work (at most 4 passes)
        runs = [_cpu_baseline(host_frames, cfg, args.cpu_stride)]
        while sum(b["seconds"] for b in runs) < 8.0 and len(runs) < 4:
            runs.append(_cpu_baseline(host_frames, cfg, args.cpu_stride))
        cpu = runs[-1]
        cpu["value"] = statistics.mean(b["value"] for b in runs)
        cpu["sample"] += f"; {len(runs)} passes, {sum(b['seconds'] for b in runs):.1f} s in total"
        cpu.pop("seconds")

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": _config_block(),
            "frame_ms_1080p": ms_per_step / (3.0 * PASSES_PER_STEP),
            "lut_build": luts,
            "frame_ms_4k": frame_4k,
            "batch": batch,
            "postprocess_4k": post,
            "shading_4k": shade,
            "raster_4k": raster,
            "frame_from_mesh_4k": mesh_frame,
            "samples_per_step": samples_per_step,
            "e2e": {"value": world * e2e_samples / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s / e2e_steps,
                    "path": "AtmosphereRenderer.update/prepare_frame/composite, pinned host buffers, "
                            "uploads/read-backs on a copy stream overlapping the other cameras' kernels"},
            "gpu_launches": 12 * PASSES_PER_STEP * args.steps,
            "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": peak_tflops, "unit": "TFLOP/s",
                         "frac": achieved_tflops / peak_tflops, "traffic": COMPOSITE_DRAM_BYTES_1080P, "traffic_unit": "bytes per launch (2 km camera, ncu)",
                         "kernel": "k_composite",
                         "peak_source": f"derived: {SMS} SMs x {FP32_LANES} FP32 lanes x 2 x median SM clock "
                                        f"{sm_mhz:.0f} MHz sampled during the run",
                         "algorithmic": f"{COMPOSITE_FLOP_PER_SAMPLE} FLOP per radiance sample x "
                                        f"{sum(comp_samples)} samples over 3 launches",
                         "launch_ms": comp_ms},
            "roofline_hbm": {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                             "frac": achieved_gbs / peaks["hbm_gbs"],
                             "note": f"{COMPOSITE_BYTES_PER_PIXEL} B per pixel algorithmic; of "
                                     f"{'fallback' if peaks.get('fallback') else 'measured'} copy bandwidth"},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "leg_seconds": leg_s,
        }
        line.update(_summary(frame_4k, luts, ms_total / 1e3))
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def _summary(frame_4k, luts, timed_s) -> dict:
    """Short top-level keys that close the line: the surrogate's headline
    (4K frames of the three cameras; the 64-frame sweep when it ran) and the
    LUT build, next to the length of the timed region."""

    out = {"timed_region_s": timed_s}
    if luts:
        out["lut_build_us"] = {k: round(luts[k]["us"], 2) for k in ("transmittance", "multi_scattering",
                                                                     "sky_view", "aerial")}
    if frame_4k:
        out["plain_4k_ms"] = frame_4k["plain_ms"]
        if frame_4k.get("mlp_ms"):
            err = frame_4k["error_vs_fp64"]
            out.update({
                "mlp_4k_ms": frame_4k["mlp_ms"], "mlp_4k_speedup": frame_4k["speedup"],
                "mlp_4k_err_mean": err["all"]["mlp"]["mean"], "mlp_4k_err_p99": err["all"]["mlp"]["p99"],
                "mlp_4k_err_worst_camera": max(c["mlp"]["mean"] for c in err["cameras"]),
                "plain_4k_err_mean": err["all"]["plain"]["mean"],
            })
        sky = frame_4k.get("sky_4k")
        if sky:
            out.update({"sky_4k_net_speedup_vs_plain": sky["net_speedup_vs_plain"],
                        "sky_4k_net_err_mean": sky["error_vs_fp64"]["net"]["mean"],
                        "sky_4k_net_uncalibrated_err_mean": sky["error_vs_fp64"]["net_uncalibrated"]["mean"],
                        "sky_4k_net_ms": sky["net_ms"], "sky_4k_plain_ms": sky["plain_ms"]})
        fused = frame_4k.get("fused_4k")
        if fused:
            out.update({k: fused[k] for k in ("separate_plain_ms", "fused_plain_ms", "separate_mlp_ms",
                                              "fused_mlp_ms") if k in fused})
        sweep = frame_4k.get("sweep")
        if sweep:
            out.update({
                "sweep_frames": sweep["frames"], "sweep_speedup": sweep["speedup"],
                "sweep_err_mean": sweep["error_vs_fp64"]["mlp"]["mean"],
                "sweep_err_p99": sweep["error_vs_fp64"]["mlp"]["p99"],
                "sweep_err_worst_frame": max(c["mlp_error_mean"] for c in sweep["cameras"]),
            })
    return out


def _composite_args(v, light):
    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG

    return (EARTH_RADIUS_M, v.camera_radius_m, v.sun_local, SOLAR_IRRADIANCE, light.sun_disk_radiance,
            SUN_ANGULAR_RADIUS_DEG, v.basis, v.tangent_half_fov, 4.0, 12.0)


POST_BYTES_PER_PIXEL = 36  # float3 HDR read by the extract and by the resolve, float3 display written


def _lut_builds(device, args) -> dict:
    """The plain LUT build (Earth parameters, FP32): each of the four LUT
    kernels at its configured size for a camera at 2 km with the sun at
    45 deg zenith, timed alone with CUDA events over repeated launches.
    Samples are the analytic counts of each build (texels x steps; the
    multi-scattering build: texels x directions x steps)."""

    import torch

    from planet_renderer_gb300 import camera
    from planet_renderer_gb300.atmosphere import AtmosphereRenderer
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG

    cfg = earth_baseline()
    r = AtmosphereRenderer(WIDTH, HEIGHT, cfg, device=device)
    sun = camera.sun_from_zenith(45.0, 0.0)
    kw = dict(planet_radius_m=EARTH_RADIUS_M, camera_altitude_m=2000.0, sun_zenith_cosine=float(sun[1]),
              sun_local=sun, solar_irradiance=SOLAR_IRRADIANCE, sun_angular_radius_degrees=SUN_ANGULAR_RADIUS_DEG,
              view_basis=camera.view_basis(0.0, -35.0), tangent_half_fov=camera.tangent_half_fov(60.0))
    counts = {
        "transmittance": cfg.transmittance_lut_width * cfg.transmittance_lut_height * cfg.transmittance_steps,
        "multi_scattering": cfg.multi_scattering_lut_width * cfg.multi_scattering_lut_height
                            * cfg.multi_scattering_directions * cfg.multi_scattering_steps,
        "sky_view": cfg.sky_view_lut_width * cfg.sky_view_lut_height * cfg.sky_view_steps,
        "aerial": cfg.aerial_lut_width * cfg.aerial_lut_height * cfg.aerial_lut_depth * cfg.aerial_steps_per_slice,
    }
    reps = 200
    out = {"workload": "plain LUT build, Earth (Mie ext 8.396e-6), camera 2 km, sun zenith 45 deg: T 256x64/40, "
                       "MS 32x32 x 64 dirs x 20, SV 192x108/30, AP 32^3 x 2; each kernel launched alone "
                       f"{reps} times (LUTs stay in L2)"}
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    total_us = 0.0
    for kind in ("transmittance", "multi_scattering", "sky_view", "aerial"):
        for _ in range(max(args.warmup, 3)):
            r.build_lut(kind, **kw)
        torch.cuda.synchronize(device)
        start.record()
        for _ in range(reps):
            r.build_lut(kind, **kw)
        end.record()
        torch.cuda.synchronize(device)
        us = start.elapsed_time(end) * 1e3 / reps
        total_us += us
        out[kind] = {"us": us, "samples": counts[kind], "samples_per_s": counts[kind] / (us * 1e-6)}
    out["all_four_us"] = total_us
    out["samples_per_s"] = sum(counts.values()) / (total_us * 1e-6)
    r.close()
    return out


def _postprocess_4k(device, args) -> dict:
    """The display post-process that follows the atmosphere stage
    (PostProcessor, reference postprocess.py) on 3840x2160 HDR frames with
    the default configuration (4 bloom passes) and tone mapping: device time
    per frame with CUDA events, two HDR frames alternated."""

    import torch

    from planet_renderer_gb300.postprocess import PostprocessConfig, PostProcessor

    width, height = 3840, 2160
    g = torch.Generator(device=device).manual_seed(SEED)
    hdrs = [torch.exp(torch.randn((width, height, 3), device=device, generator=g) * 1.5 - 1.0) for _ in range(2)]
    display = torch.empty_like(hdrs[0])
    config = PostprocessConfig()
    pp = PostProcessor(width, height, config, device=device)
    for i in range(args.warmup):
        pp.process(hdrs[i % 2], display, 0.0, bloom=True, tone_map=True)
    steps = 50
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    start.record()
    for i in range(steps):
        pp.process(hdrs[i % 2], display, 0.0, bloom=True, tone_map=True)
    end.record()
    torch.cuda.synchronize(device)
    eager_ms = start.elapsed_time(end) / steps
    # the same frames as CUDA graphs (one per HDR source): the six launches replay as one
    graphs = _capture_fn([(h,) for h in hdrs], device,
                         lambda h: pp.process(h, display, 0.0, bloom=True, tone_map=True))
    for _ in range(3):
        for gr in graphs:
            gr.replay()
    ms = _timed_graph_region(graphs, steps // 2, device) / (2 * (steps // 2))
    del graphs
    peaks = _peaks()
    gbs = width * height * POST_BYTES_PER_PIXEL / (ms / 1e3) / 1e9
    out = {
        "workload": "3840x2160 float3 HDR -> display: bloom extract at half resolution, 4 fused blur passes, "
                    "resolve (exposure, bilinear bloom, ACES, sRGB); two HDR frames alternated (each frame's "
                    "300 MB of traffic exceeds L2)",
        "ms": ms, "eager_ms": eager_ms, "graph": True, "steps": steps, "launches_per_frame": 2 + config.bloom_passes,
        "algorithmic_bytes_per_pixel": POST_BYTES_PER_PIXEL, "achieved_gbs": gbs, "hbm_peak_gbs": peaks["hbm_gbs"],
        "frac": gbs / peaks["hbm_gbs"],
    }
    pp.close()
    del hdrs, display
    torch.cuda.empty_cache()
    return out


SHADE_BYTES_LAND = 84     # position 12 + normal 12 + albedo 12 + id 4 + sun T 12 + sky 12 read, hdr 12 written
SHADE_BYTES_OCEAN = 148   # + water depth 4, seabed albedo 12 and normal 12, slope 4, 4 terrain taps ~32


def _shading_4k(device, args, steps=20) -> dict:
    """Surface shading (shading.shade_surface, the consumer of prepare_frame's
    surface lighting) at 3840x2160 on the land-and-ocean inputs of the 2 km
    camera's fBm G-buffer: device time per frame with CUDA events."""

    import torch

    from planet_renderer_gb300.atmosphere import scene
    from planet_renderer_gb300.atmosphere.workloads import (EARTH_RADIUS_M, SOLAR_IRRADIANCE,
                                                            SUN_ANGULAR_RADIUS_DEG)
    from planet_renderer_gb300.shading import OceanShading, shade_surface

    width, height = 3840, 2160
    r, cfg, frames = _setup_chain(device, width, height)
    v, gb, light = frames[0]
    _chain(r, v, gb, light)
    inputs = scene.shading_inputs(gb, EARTH_RADIUS_M, v.altitude_m, v.basis)
    out = torch.empty_like(gb["scene_hdr"])
    run = lambda: shade_surface(inputs, r.surface_sun_transmittance, r.surface_sky_radiance, out, v.sun_local,
                                SOLAR_IRRADIANCE, v.basis, OceanShading(), math.radians(SUN_ANGULAR_RADIUS_DEG),
                                v.tangent_half_fov)
    for _ in range(args.warmup):
        run()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    start.record()
    for _ in range(steps):
        run()
    end.record()
    torch.cuda.synchronize(device)
    ms = start.elapsed_time(end) / steps
    n_ocean = int((inputs["water_depth"] > 0).sum())
    n_land = int((inputs["surface_id"] == 0).sum())
    algo = n_land * SHADE_BYTES_LAND + n_ocean * SHADE_BYTES_OCEAN
    peaks = _peaks()
    res = {"workload": "3840x2160 surface shading of the 2 km camera's fBm G-buffer (hits below the sphere are "
                       "ocean: BRDF, refraction, seabed taps; the rest Lambertian land)",
           "ms": ms, "land_px": n_land, "ocean_px": n_ocean, "algorithmic_bytes": algo,
           "achieved_gbs": algo / (ms / 1e3) / 1e9, "frac": algo / (ms / 1e3) / 1e9 / peaks["hbm_gbs"]}
    r.close()
    del gb, inputs, out
    torch.cuda.empty_cache()
    return res


RASTER_TRI_BYTES = 228  # one emitted triangle record (atm::RasterTri)
RASTER_VERTEX_BYTES = 48  # view 12, normal 12, material 16, height 4, cell 4
RASTER_COVERED_BYTES = 68  # depth, position, normal, albedo (3 floats), material (4), height, ids
RASTER_KEY_BYTES = 16  # the depth key's clear and its read by the resolve


def _raster_4k(device, args, steps=20) -> dict:
    """The terrain raster (clip, depth keys, resolve; the atmosphere stage's
    G-buffer producer) at 3840x2160 over the synthetic ground-camera terrain:
    the reference renderer's default patch budget (256 patches of 12 cells)
    and a dense one (1024 patches of 32 cells), 2 km above ground looking 8
    degrees down to 80 km.  Device time per frame with CUDA events."""

    import torch

    from planet_renderer_gb300.raster import TerrainRaster, synthetic_terrain

    width, height, tf = 3840, 2160, math.tan(math.radians(30.0))
    out = {}
    for name, rows, cols, res in (("default_256x12", 16, 16, 12), ("dense_1024x32", 32, 32, 32)):
        mesh = synthetic_terrain(width, height, tf, rows=rows, columns=cols, resolution=res, seed=SEED, device=device)
        patches, tpp = rows * cols, int(mesh["triangles"].shape[0])
        r = TerrainRaster(width, height, patches, tpp, device=device)
        g = r.allocate_gbuffer(3)
        run = lambda: r.render(mesh, 0.5, tf, g)
        for _ in range(args.warmup):
            run()
        emitted = r.emitted()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        start.record()
        for _ in range(steps):
            run()
        end.record()
        torch.cuda.synchronize(device)
        ms = start.elapsed_time(end) / steps
        covered = int((g["surface_id"] >= 0).sum())
        pixels = width * height
        algo = (patches * int(mesh["view"].shape[1]) * RASTER_VERTEX_BYTES + 2 * emitted * RASTER_TRI_BYTES
                + pixels * RASTER_KEY_BYTES + covered * RASTER_COVERED_BYTES + (pixels - covered) * 8)
        peaks = _peaks()
        out[name] = {"ms": ms, "source_triangles": patches * tpp, "emitted": emitted, "covered_px": covered,
                     "algorithmic_bytes": algo, "achieved_gbs": algo / (ms / 1e3) / 1e9,
                     "frac": algo / (ms / 1e3) / 1e9 / peaks["hbm_gbs"]}
        r.close()
        del mesh, g
        torch.cuda.empty_cache()
    out["workload"] = ("3840x2160 terrain raster (clip + depth keys + resolve) of a 2 km ground camera's synthetic "
                       "terrain, 60 degree vertical field of view, near 0.5 m")
    return out


def _frame_from_mesh_4k(device, args, sg=None, steps=10) -> dict:
    """A whole 3840x2160 frame from terrain patches to the display image, in
    the reference renderer's order (renderer.py:1626-1735): terrain raster
    with the snapshot -> ocean coverage -> atmosphere update -> fused surface
    lighting + shading + composite -> display post-process.  The ground
    camera 30 m above sea level looks 6 degrees down over the synthetic
    coast (the default patch budget, 256 patches of 12 cells; 200 m relief
    rising inland, its valleys below sea level are sea), sun 35 degrees up.  One CUDA graph per frame;
    device ms per frame and per stage.  With ``sg`` the atmosphere stage also
    runs with the surrogate composite, and its frame's error against the
    plain frame is stated."""

    import numpy as np
    import torch

    from planet_renderer_gb300 import camera as cam
    from planet_renderer_gb300.atmosphere import AtmosphereRenderer
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.workloads import (EARTH_RADIUS_M, SOLAR_IRRADIANCE,
                                                            SUN_ANGULAR_RADIUS_DEG)
    from planet_renderer_gb300.lighting import LightingState
    from planet_renderer_gb300.ocean import OCEAN_SURFACE_ID, OceanConfig, OceanRenderer
    from planet_renderer_gb300.postprocess import PostprocessConfig, PostProcessor
    from planet_renderer_gb300.raster import TerrainRaster, synthetic_terrain

    W, H, tf, alt = 3840, 2160, math.tan(math.radians(30.0)), 30.0
    mesh = synthetic_terrain(W, H, tf, altitude_m=alt, pitch_degrees=6.0, relief_m=200.0, base_height_m=0.0,
                             rise_m_per_km=10.0, seed=SEED, device=device)
    basis = mesh["view_basis"]
    frame = (np.array([1.0, 0.0, 0.0]), np.array([0.0, 1.0, 0.0]), np.array([0.0, 0.0, 1.0]))
    sun = cam.sun_local(150.0, 35.0)
    light = LightingState(sun, SUN_ANGULAR_RADIUS_DEG, SOLAR_IRRADIANCE)
    raster = TerrainRaster(W, H, int(mesh["view"].shape[0]), int(mesh["triangles"].shape[0]), device=device)
    g = raster.allocate_gbuffer(3, snapshot=True, ocean=True)
    sea = OceanRenderer(W, H, OceanConfig(), device=device)
    atm = AtmosphereRenderer(W, H, earth_baseline(), device=device)
    post = PostProcessor(W, H, PostprocessConfig(), device=device)
    space_hdr = torch.zeros(W, H, 3, device=device)
    hdr = torch.zeros(W, H, 3, device=device)
    display = torch.zeros(W, H, 3, device=device)
    R = EARTH_RADIUS_M
    args_atm = (R, R + alt, sun, SOLAR_IRRADIANCE, light.sun_disk_radiance, SUN_ANGULAR_RADIUS_DEG, basis, tf, 4.0,
                12.0)
    stages = {
        "raster": lambda: raster.render(mesh, 0.5, tf, g),
        "ocean": lambda: sea.rasterize_gbuffer(g, R, alt, frame, basis, tf, 12.5, 0),
        "atmosphere": lambda: (atm.update(R, R + alt, sun, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG),
                               atm.render_frame(g, space_hdr, hdr, *args_atm)),
        "post": lambda: post.process(hdr, display, 0.0, bloom=True, tone_map=True),
    }
    whole = lambda: [fn() for fn in stages.values()]
    timed = list(stages.items()) + [("frame", whole)]
    if sg is not None:
        stages_mlp = dict(stages, atmosphere=lambda: (
            atm.update(R, R + alt, sun, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG),
            atm.render_frame(g, space_hdr, hdr, *args_atm, surrogate=sg, check_fraction=MLP_CHECK_FRACTION,
                             seed=SEED)))
        timed += [("atmosphere_mlp", stages_mlp["atmosphere"]),
                  ("frame_mlp", lambda: [fn() for fn in stages_mlp.values()])]
    out = {"workload": "3840x2160 frame from terrain patches to display: raster + snapshot, ocean coverage, "
                       "atmosphere update, fused lighting + shading + composite, bloom + tone map; ground camera "
                       "30 m above sea level, 256 patches x 12 cells, default ocean; CUDA graphs"}
    if sg is not None:
        whole()
        plain_hdr = hdr.clone()
        [fn() for fn in stages_mlp.values()]
        surface = (g["surface_id"] >= 0)
        ref = plain_hdr[surface].double()
        floor = 1e-4 * float(ref.abs().max())
        rel = ((hdr[surface].double() - ref).abs() / ref.abs().clamp_min(floor)).max(dim=-1).values
        out["mlp_err_vs_plain"] = {"mean": float(rel.mean()), "p99": float(torch.quantile(rel.float()[::97], 0.99))}
    for name, fn in timed:
        graphs = _capture_fn([()], device, fn)
        for _ in range(3):
            graphs[0].replay()
        out[f"{name}_ms"] = _timed_graph_region(graphs, steps, device) / steps
        del graphs
    sid = g["surface_id"]
    out["sea_px"] = int((sid == OCEAN_SURFACE_ID).sum())
    out["terrain_px"] = int(((sid >= 0) & (sid != OCEAN_SURFACE_ID)).sum())
    out["emitted_triangles"] = raster.emitted()
    out["display_finite"] = bool(torch.isfinite(display).all())
    for o in (raster, sea, atm, post):
        o.close()
    del g, mesh
    torch.cuda.empty_cache()
    return out


def _batch(device, args) -> dict:
    """Batched LUT builds: 256 snapshots x 16 cameras x 2 parameter sets, a
    sky-view LUT and an aerial volume each (16,384 LUTs of uneven sizes) in
    one persistent launch per step, tiles from the autotuner."""

    import torch

    from planet_renderer_gb300.atmosphere import autotune
    from planet_renderer_gb300.atmosphere.batch import SKY_VIEW, BatchedLutBuilder
    from planet_renderer_gb300.atmosphere.workloads import batched_lut_jobs, batched_lut_sets

    sets = batched_lut_sets()
    jobs = batched_lut_jobs(SEED)
    builder = BatchedLutBuilder(sets, device=device)
    tuning, report = autotune.tune(builder, jobs)
    prepared = builder.prepare(jobs)
    arena = torch.empty((prepared[1], 4), dtype=torch.float32, device=device)
    for _ in range(2):
        builder.build(jobs, tuning, arena=arena, prepared=prepared)
    torch.cuda.synchronize(device)
    builder.samples(reset=True)
    steps = 5
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(steps):
        builder.build(jobs, tuning, arena=arena, prepared=prepared)
    end.record()
    torch.cuda.synchronize(device)
    ms = start.elapsed_time(end) / steps
    samples = builder.samples(reset=True) / steps
    sky_keys = {j.sky_key() for j in jobs if j.kind == SKY_VIEW}
    n_sky = sum(1 for j in jobs if j.kind == SKY_VIEW)
    out = {
        "workload": "256 snapshots (sun zenith 0-110 deg) x 16 cameras (1 m - 4000 km) x 2 parameter sets "
                    "(Earth, 50 km planet); sky-view 96x54..384x216 and aerial 16^3..64^3 per (snapshot, camera, "
                    "set); one persistent launch",
        "luts": len(jobs), "ms_per_batch": ms, "luts_per_s": len(jobs) / (ms / 1e3),
        "samples_per_batch": samples, "samples_per_s": samples / (ms / 1e3),
        "sky_view_luts_raw": n_sky, "sky_view_luts_deduped": len(sky_keys),
        "arena_gb": prepared[1] * 16 / 1e9,
        "tuning": tuning.__dict__, "tuning_cached": report.get("cached", False), "steps": steps,
    }
    del arena
    builder.close()
    torch.cuda.empty_cache()
    return out


def _chain_surrogate(r, v, gb, light, sg, stats):
    """One frame of the surrogate chain: the plain chain with the composite
    replaced by atm_composite_surrogate (1% of the MLP pixels re-integrated)."""

    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG

    sun = v.sun_local
    r.update(EARTH_RADIUS_M, v.camera_radius_m, sun, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG)
    r.prepare_frame(gb["position_view"], gb["surface_id"], EARTH_RADIUS_M, v.camera_radius_m, sun, SOLAR_IRRADIANCE,
                    SUN_ANGULAR_RADIUS_DEG, v.basis, v.tangent_half_fov)
    r.composite_surrogate(gb["scene_hdr"], gb["space_hdr"], gb["surface_id"], gb["position_view"], gb["hdr"],
                          *_composite_args(v, light), surrogate=sg, stats=stats, check_fraction=MLP_CHECK_FRACTION,
                          seed=SEED)


def _capture_fn(frames, device, fn):
    import torch

    side = torch.cuda.Stream(device)
    side.wait_stream(torch.cuda.current_stream(device))
    with torch.cuda.stream(side):
        for f in frames:  # warm-up outside capture
            fn(*f)
    torch.cuda.current_stream(device).wait_stream(side)
    torch.cuda.synchronize(device)
    graphs = []
    for f in frames:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            fn(*f)
        graphs.append(g)
    torch.cuda.synchronize(device)
    return graphs


def _sparse_inputs(gb, pix, width, height):
    """The G-buffer images the FP64 oracle composite reads, as full-size
    float64 / int32 host arrays holding only the pixels `pix` (n, 2): the
    oracle touches no other element, and untouched zero pages cost nothing."""

    import numpy as np
    import torch

    dev = gb["surface_id"].device
    px = torch.as_tensor(pix[:, 0], device=dev)
    py = torch.as_tensor(pix[:, 1], device=dev)
    full = {}
    for k in ("scene_hdr", "space_hdr", "position_view"):
        a = np.zeros((width, height, 3), np.float64)
        a[pix[:, 0], pix[:, 1]] = gb[k][px, py].cpu().numpy()
        full[k] = a
    sid = np.zeros((width, height), np.int32)
    sid[pix[:, 0], pix[:, 1]] = gb["surface_id"][px, py].cpu().numpy()
    return full, sid


def _fp64_error(r, cfg, frames, images, n_pixels=1500):
    """Relative error (max over RGB, floor 1e-4 of the sample's peak) of each
    camera's image against the FP64 oracle composite at n_pixels random
    pixels; the oracle builds its own FP64 LUTs."""

    import numpy as np

    from oracle.atm import Oracle
    from planet_renderer_gb300.atmosphere.workloads import EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG

    o = Oracle("f64")
    ar = math.radians(SUN_ANGULAR_RADIUS_DEG)
    tl = o.build_transmittance(cfg, EARTH_RADIUS_M)
    ms = o.build_multi_scattering(cfg, EARTH_RADIUS_M, SOLAR_IRRADIANCE, ar, tl)
    W, H = r.width, r.height
    rng = np.random.default_rng(SEED)
    per_cam, all_errs = [], {k: [] for k in images[0]}
    for (v, gb, light), imgs in zip(frames, images):
        alt = v.altitude_m
        sv = o.build_sky_view(cfg, EARTH_RADIUS_M, alt, float(v.sun_local[1]), SOLAR_IRRADIANCE, ar, tl, ms)
        ap = np.zeros((cfg.aerial_lut_width, cfg.aerial_lut_height, cfg.aerial_lut_depth, 3))
        pix = np.stack([rng.integers(0, W, n_pixels), rng.integers(0, H, n_pixels)], 1)
        full, sid = _sparse_inputs(gb, pix, W, H)
        plist = (pix[:, 0].astype(np.int64) * H + pix[:, 1]).astype(np.int32)
        hdr, _ = o.composite(cfg, full["scene_hdr"], full["space_hdr"], sid, full["position_view"], EARTH_RADIUS_M,
                             alt, alt, v.sun_local, SOLAR_IRRADIANCE, light.sun_disk_radiance, ar, v.basis,
                             v.tangent_half_fov, 4.0, 12.0, 0, tl, ms, sv, ap, pixel_list=plist)
        ref = hdr[pix[:, 0], pix[:, 1]]
        floor = 1e-4 * np.abs(ref).max()
        cam = {"altitude_m": alt}
        for name, img in imgs.items():
            e = np.max(np.abs(img[pix[:, 0], pix[:, 1]] - ref) / np.maximum(np.abs(ref), floor), axis=1)
            all_errs[name].append(e)
            cam[name] = {"mean": float(e.mean()), "p99": float(np.quantile(e, 0.99))}
        per_cam.append(cam)
    total = {}
    for name, es in all_errs.items():
        e = np.concatenate(es)
        total[name] = {"mean": float(e.mean()), "p99": float(np.quantile(e, 0.99)), "max": float(e.max())}
    return {"pixels_per_camera": n_pixels, "all": total, "cameras": per_cam}


def _frame_4k(device, args) -> dict:
    """Plain chain and surrogate chain at 3840x2160 for the same cameras:
    frame ms (graph replay), the surrogate's training, gate statistics and
    both frames' error against the FP64 oracle."""

    import time

    import torch

    from planet_renderer_gb300.atmosphere.surrogate import stats_summary, train_surrogate

    r, cfg, frames = _setup_chain(device, 3840, 2160)
    graphs = _capture(r, frames, device)
    for _ in range(3):
        for g in graphs:
            g.replay()
    steps = 20
    plain_ms = _timed_graph_region(graphs, steps, device) / steps / 3.0
    plain_imgs = []
    for v, gb, light in frames:
        _chain(r, v, gb, light)
        plain_imgs.append(gb["hdr"].cpu().numpy().astype("float64"))
    del graphs
    out = {"plain_ms": plain_ms, "mlp_ms": None, "steps": steps}
    if args.no_mlp:
        return out
    t0 = time.perf_counter()
    trained, reports = train_surrogate(epochs=args.mlp_epochs, batch=16384, seed=SEED, log_every=0, device=device)
    torch.cuda.synchronize(device)
    train_s = time.perf_counter() - t0
    sg = _frame_surrogate(trained)
    stats = torch.zeros(8, dtype=torch.float32, device=device)
    fn = lambda v, gb, light: _chain_surrogate(r, v, gb, light, sg, stats)
    graphs = _capture_fn(frames, device, fn)
    for _ in range(3):
        for g in graphs:
            g.replay()
    mlp_ms = _timed_graph_region(graphs, steps, device) / steps / 3.0
    stats.zero_()
    for g in graphs:
        g.replay()
    torch.cuda.synchronize(device)
    gate = stats_summary(stats)
    images = []
    for (v, gb, light), plain in zip(frames, plain_imgs):
        _chain_surrogate(r, v, gb, light, sg, None)
        images.append({"plain": plain, "mlp": gb["hdr"].cpu().numpy().astype("float64")})
    err = _fp64_error(r, cfg, frames, images)
    out.update({
        "mlp_ms": mlp_ms, "speedup": plain_ms / mlp_ms, "error_vs_fp64": err,
        "gate": {**gate, "check_fraction": MLP_CHECK_FRACTION},
        "training": {"seconds": train_s, "networks": len(reports), "samples_per_network": 2**22, "batch": 16384,
                     "epochs": args.mlp_epochs, "steps_per_network": reports["sky"].steps,
                     "held_out": {name: rep.held_out for name, rep in reports.items()}},
        "networks": "aerial 11->4x64->6 (one per camera-altitude band inside the shell: 0-100 m, 100 m-3 km, "
                    "3-25 km, 25-100 km; one above the shell), sky 10->3x64->3; SiLU; BF16 operands on tcgen05 "
                    "with FP32 accumulators in tensor memory; in frames the sky pixels read the sky-view LUT",
        "gates": {"twilight_cosine": sg.twilight_cosine, "terminator": bool(sg.gate_terminator),
                  "limb_degrees": sg.limb_degrees},
    })
    del graphs
    if args.mlp_sweep:
        out["sweep"] = _mlp_sweep(r, cfg, sg, args.mlp_sweep, device)
    del r, frames
    torch.cuda.empty_cache()
    out["sky_4k"] = _sky_4k(device, args, trained)
    out["fused_4k"] = _frame_fused_4k(device, args, sg)
    if not args.no_raster:
        out["mesh_4k"] = _frame_from_mesh_4k(device, args, sg)
    return out


def _frame_surrogate(trained):
    """The surrogate of the frames: the aerial networks of `trained` (its
    altitude bands and the network above the shell) with the sky pixels on
    the sky-view LUT, as the plain frame has them (a LUT tap is cheaper than
    the sky network and exact to the plain frame), and the terminator gate."""

    from planet_renderer_gb300.atmosphere.surrogate import Surrogate

    sg = Surrogate(trained.aerial, None, trained.planet_radius_m, trained.top_altitude_m, trained.scale_height_range,
                   trained.aerial_spec, None, trained.aerial_above_shell, aerial_bands=trained.aerial_bands)
    sg.gate_terminator = True
    return sg


def _frame_fused_4k(device, args, sg) -> dict:
    """The reference's frame order at 3840x2160 for the three frame-chain
    cameras on land-and-ocean shading inputs: update -> prepare_frame ->
    shade_surface -> composite as separate calls, against update ->
    render_frame (surface lighting, shading and composite fused in one
    pass), each with the plain composite and with the surrogate composite;
    CUDA-graph replays, device ms per frame."""

    import torch

    from planet_renderer_gb300.atmosphere import scene
    from planet_renderer_gb300.atmosphere.workloads import (EARTH_RADIUS_M, SOLAR_IRRADIANCE,
                                                            SUN_ANGULAR_RADIUS_DEG)
    from planet_renderer_gb300.shading import OceanShading, shade_surface

    r, cfg, frames = _setup_chain(device, 3840, 2160)
    shaded = []
    for v, gb, light in frames:
        images = scene.shading_inputs(gb, EARTH_RADIUS_M, v.altitude_m, v.basis)
        shaded.append((v, gb, light, images, torch.empty_like(gb["scene_hdr"])))
    ar = math.radians(SUN_ANGULAR_RADIUS_DEG)

    def separate(v, gb, light, images, surface_hdr, surrogate):
        sun = v.sun_local
        r.update(EARTH_RADIUS_M, v.camera_radius_m, sun, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG)
        r.prepare_frame(images["position"], images["surface_id"], EARTH_RADIUS_M, v.camera_radius_m, sun,
                        SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG, v.basis, v.tangent_half_fov)
        shade_surface(images, r.surface_sun_transmittance, r.surface_sky_radiance, surface_hdr, sun,
                      SOLAR_IRRADIANCE, v.basis, OceanShading(), ar, v.tangent_half_fov)
        if surrogate is None:
            r.composite(surface_hdr, gb["space_hdr"], images["surface_id"], images["position"], gb["hdr"],
                        *_composite_args(v, light))
        else:
            r.composite_surrogate(surface_hdr, gb["space_hdr"], images["surface_id"], images["position"], gb["hdr"],
                                  *_composite_args(v, light), surrogate=surrogate, check_fraction=MLP_CHECK_FRACTION,
                                  seed=SEED)

    def fused(v, gb, light, images, surface_hdr, surrogate):
        r.update(EARTH_RADIUS_M, v.camera_radius_m, v.sun_local, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG)
        r.render_frame(images, gb["space_hdr"], gb["hdr"], *_composite_args(v, light), surrogate=surrogate,
                       check_fraction=MLP_CHECK_FRACTION, seed=SEED)

    out = {"workload": "3840x2160, frame-chain cameras, land-and-ocean shading inputs (sea level at the median hit "
                       "radius): update -> prepare_frame -> shade_surface -> composite as separate calls vs update "
                       "-> render_frame (lighting, shading and composite fused); CUDA graphs"}
    steps = 10
    for name, fn in (("separate", separate), ("fused", fused)):
        for label, surrogate in (("plain", None), ("mlp", sg)):
            if surrogate is None and label == "mlp":
                continue
            graphs = _capture_fn(shaded, device, lambda *f: fn(*f, surrogate))
            for _ in range(3):
                for g in graphs:
                    g.replay()
            out[f"{name}_{label}_ms"] = _timed_graph_region(graphs, steps, device) / steps / 3.0
            del graphs
    r.check()
    r.close()
    del shaded, frames
    torch.cuda.empty_cache()
    return out


SKY_ALTITUDES_M = (2_000.0, 20_000.0, 60_000.0)


def _sky_4k(device, args, sg, n_pixels=1500) -> dict:
    """The learned sky-view workload: the sky radiance of every pixel of a
    3840x2160 view (cameras at 2, 20 and 60 km, pitch +15 deg, the frame-chain
    workload's sun positions) by the plain integrator per pixel (the
    sky-view march along each pixel's ray), by the sky network (plain where a
    gate trips), and by the reference's sky-view LUT lookup; device ms per
    frame and each one's error against the FP64 oracle's march."""

    import numpy as np
    import torch

    from oracle.atm import Oracle
    from planet_renderer_gb300 import camera
    from planet_renderer_gb300.atmosphere import AtmosphereRenderer
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.scene import pixel_rays
    from planet_renderer_gb300.atmosphere.workloads import (EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG,
                                                            frame_chain_cameras)

    width, height = 3840, 2160
    cfg = earth_baseline()
    r = AtmosphereRenderer(width, height, cfg, device=device)
    out = torch.empty((width, height, 3), device=device)
    o = Oracle("f64")
    ar = math.radians(SUN_ANGULAR_RADIUS_DEG)
    tl = o.build_transmittance(cfg, EARTH_RADIUS_M)
    ms = o.build_multi_scattering(cfg, EARTH_RADIUS_M, SOLAR_IRRADIANCE, ar, tl)
    rng = np.random.default_rng(SEED + 2)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = {"plain": 0.0, "net": 0.0, "net_uncalibrated": 0.0, "lut": 0.0}
    tile = sg.calibration_tile
    errors = {k: [] for k in times}
    cams = []
    basis = camera.view_basis(0.0, 15.0)
    tanfov = camera.tangent_half_fov(60.0)
    for alt, v in zip(SKY_ALTITUDES_M, frame_chain_cameras(SEED)):
        cr = EARTH_RADIUS_M + alt
        sun = v.sun_local
        r.update(EARTH_RADIUS_M, cr, sun.copy(), SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG)
        a = (EARTH_RADIUS_M, cr, sun, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG, basis, tanfov)
        xs = torch.as_tensor(rng.integers(0, width, n_pixels))
        ys = torch.as_tensor(rng.integers(0, height, n_pixels))
        rays = pixel_rays(width, height, basis, tanfov, xs, ys).numpy()
        ref = o.sky_rays(cfg, EARTH_RADIUS_M, np.full(n_pixels, alt), rays, np.tile(sun, (n_pixels, 1)),
                         SOLAR_IRRADIANCE, ar, tl, ms)
        floor = 1e-4 * np.abs(ref).max()
        cam = {"altitude_m": alt, "sun_zenith_deg": v.sun_zenith_deg}
        for mode in times:
            # the network with the calibration from 1% checked pixels, and without it
            sg.calibration_tile = 0 if mode == "net_uncalibrated" else tile
            kind = "net" if mode.startswith("net") else mode
            run = lambda: r.sky_pixels(out, *a, mode=kind, surrogate=sg if kind == "net" else None, seed=SEED)
            for _ in range(3):
                run()
            torch.cuda.synchronize(device)
            start.record()
            for _ in range(10):
                run()
            end.record()
            torch.cuda.synchronize(device)
            ms_mode = start.elapsed_time(end) / 10
            times[mode] += ms_mode
            got = out[xs.to(device), ys.to(device)].cpu().numpy().astype(np.float64)
            e = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor), axis=1)
            errors[mode].append(e)
            cam[f"{mode}_ms"] = ms_mode
            cam[f"{mode}_err_mean"] = float(e.mean())
        cams.append(cam)
    sg.calibration_tile = tile
    r.check()
    r.close()
    del out
    torch.cuda.empty_cache()
    err = {k: {"mean": float(np.concatenate(v).mean()), "p99": float(np.quantile(np.concatenate(v), 0.99))}
           for k, v in errors.items()}
    n = len(SKY_ALTITUDES_M)
    return {"workload": "sky radiance of every pixel of 3840x2160 views (cameras 2 / 20 / 60 km, pitch +15 deg, "
                        "frame-chain sun positions): plain per-pixel sky-view march vs sky network (plain where "
                        "|sun cosine| < 0.1 or within 0.5 deg of the limb; 1% of its pixels checked by the march "
                        f"and {tile}-pixel tiles calibrated from them; also without the calibration) vs sky-view "
                        "LUT lookup",
            "plain_ms": times["plain"] / n, "net_ms": times["net"] / n,
            "net_uncalibrated_ms": times["net_uncalibrated"] / n, "lut_lookup_ms": times["lut"] / n,
            "net_speedup_vs_plain": times["plain"] / times["net"], "error_vs_fp64": err,
            "pixels_per_camera": n_pixels, "cameras": cams}


def _mlp_sweep(r, cfg, sg, n_frames, device, n_pixels=300) -> dict:
    """The aerial-surrogate frame workload as configured: n_frames frames of
    the fBm G-buffer at the renderer's size with cameras log-uniform 1 m -
    4000 km (surrogate_sweep_cameras).  Per frame the plain and the surrogate
    chain are timed with CUDA events after one untimed call each (which also
    rebuilds the camera's sky-view LUT), and both images are compared with the
    FP64 oracle at n_pixels random pixels."""

    import numpy as np
    import torch

    from oracle.atm import Oracle
    from planet_renderer_gb300.atmosphere import scene
    from planet_renderer_gb300.atmosphere.surrogate import stats_summary
    from planet_renderer_gb300.atmosphere.workloads import (EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG,
                                                            surrogate_sweep_cameras)
    from planet_renderer_gb300.lighting import LightingState

    o = Oracle("f64")
    ar = math.radians(SUN_ANGULAR_RADIUS_DEG)
    tl = o.build_transmittance(cfg, EARTH_RADIUS_M)
    ms = o.build_multi_scattering(cfg, EARTH_RADIUS_M, SOLAR_IRRADIANCE, ar, tl)
    ap = np.zeros((cfg.aerial_lut_width, cfg.aerial_lut_height, cfg.aerial_lut_depth, 3))
    W, H = r.width, r.height
    rng = np.random.default_rng(SEED + 1)
    stats = torch.zeros(8, dtype=torch.float32, device=device)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    totals = {"plain": 0.0, "mlp": 0.0}
    errors = {"plain": [], "mlp": []}
    cameras = []
    for v in surrogate_sweep_cameras(SEED, n_frames):
        gb = scene.synthesize_gbuffer(W, H, EARTH_RADIUS_M, v.altitude_m, v.basis, v.tangent_half_fov, v.sun_local,
                                      SOLAR_IRRADIANCE, seed=SEED, device=device)
        gb["hdr"] = torch.zeros_like(gb["scene_hdr"])
        light = LightingState(v.sun_local, SUN_ANGULAR_RADIUS_DEG, SOLAR_IRRADIANCE)
        pix = np.stack([rng.integers(0, W, n_pixels), rng.integers(0, H, n_pixels)], 1)
        px, py = torch.as_tensor(pix[:, 0], device=device), torch.as_tensor(pix[:, 1], device=device)
        values, ms_cam = {}, {}
        runs = (("plain", lambda: _chain(r, v, gb, light)),
                ("mlp", lambda: _chain_surrogate(r, v, gb, light, sg, stats)))
        for name, fn in runs:
            fn()
            torch.cuda.synchronize(device)
            start.record()
            fn()
            end.record()
            torch.cuda.synchronize(device)
            ms_cam[name] = start.elapsed_time(end)
            totals[name] += ms_cam[name]
            values[name] = gb["hdr"][px, py].cpu().numpy().astype(np.float64)
        alt = v.altitude_m
        sv = o.build_sky_view(cfg, EARTH_RADIUS_M, alt, float(v.sun_local[1]), SOLAR_IRRADIANCE, ar, tl, ms)
        full, sid = _sparse_inputs(gb, pix, W, H)
        plist = (pix[:, 0].astype(np.int64) * H + pix[:, 1]).astype(np.int32)
        hdr, _ = o.composite(cfg, full["scene_hdr"], full["space_hdr"], sid, full["position_view"], EARTH_RADIUS_M,
                             alt, alt, v.sun_local, SOLAR_IRRADIANCE, light.sun_disk_radiance, ar, v.basis,
                             v.tangent_half_fov, 4.0, 12.0, 0, tl, ms, sv, ap, pixel_list=plist)
        ref = hdr[pix[:, 0], pix[:, 1]]
        floor = 1e-4 * np.abs(ref).max()
        cam = {"altitude_m": alt, "sun_zenith_deg": v.sun_zenith_deg, **{f"{k}_ms": t for k, t in ms_cam.items()}}
        for name, got in values.items():
            e = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor), axis=1)
            errors[name].append(e)
            cam[f"{name}_error_mean"] = float(e.mean())
        cameras.append(cam)
        del gb, full
    error = {name: {"mean": float(np.concatenate(es).mean()), "p99": float(np.quantile(np.concatenate(es), 0.99))}
             for name, es in errors.items()}
    return {"frames": n_frames, "width": W, "height": H, "pixels_per_frame": n_pixels,
            "plain_ms_mean": totals["plain"] / n_frames, "mlp_ms_mean": totals["mlp"] / n_frames,
            "speedup": totals["plain"] / totals["mlp"], "error_vs_fp64": error, "gate": stats_summary(stats),
            "cameras": cameras}


# ---- small cases for ncu captures (python bench.py --profile-case NAME) ------
# Each runs its kernels a few times on one workload of the benchmark, so that
# `ncu -k regex:<kernel> -s <skip> -c <count>` captures a warm launch.


def _profile_frame(args, width, height, camera):
    import torch

    device = torch.device("cuda:0")
    torch.cuda.set_device(device)
    r, cfg, frames = _setup_chain(device, width, height)
    v, gb, light = frames[camera]
    for _ in range(3):
        _chain(r, v, gb, light)
    torch.cuda.synchronize(device)
    return r, frames


def _profile_frame_1080p(args):
    """Plain chain, 1080p, the 2 km camera: k_sky_view, k_prepare_surface,
    k_aerial, k_composite three times each."""

    _profile_frame(args, WIDTH, HEIGHT, 0)
    print("profile case frame1080p: 3 chains of the 2 km camera at 1920x1080")


def _profile_frame_4k_mlp(args):
    """Surrogate chain at 4K for the 2 km camera, networks trained for
    --mlp-epochs epochs (the kernels' cost does not depend on how well the
    networks are trained): k_composite_surrogate and k_surrogate_fallback
    three times each, after the training kernels."""

    import torch

    from planet_renderer_gb300.atmosphere.surrogate import train_surrogate

    device = torch.device("cuda:0")
    torch.cuda.set_device(device)
    r, cfg, frames = _setup_chain(device, 3840, 2160)
    trained, _ = train_surrogate(epochs=args.mlp_epochs, batch=16384, seed=SEED, log_every=0, device=device,
                                 sky=False)
    sg = _frame_surrogate(trained)
    v, gb, light = frames[0]
    for _ in range(3):
        _chain_surrogate(r, v, gb, light, sg, None)
    torch.cuda.synchronize(device)
    r.check()
    print(f"profile case frame4k_mlp: 3 surrogate chains of the 2 km camera at 3840x2160 "
          f"({args.mlp_epochs} training epochs)")


def _profile_luts(args):
    """The four plain LUT builds of the Earth workload, three times each."""

    args.warmup = 0
    out = _lut_builds(__import__("torch").device("cuda:0"), argparse.Namespace(warmup=3))
    print("profile case luts:", {k: round(out[k]["us"], 2) for k in ("transmittance", "multi_scattering",
                                                                      "sky_view", "aerial")})


def _profile_batch(args):
    """One persistent batched build of the first 512 jobs of the batched
    workload (a mix of sky-view LUTs and aerial volumes of both parameter
    sets), tiles from the autotuner's defaults, three launches."""

    import torch

    from planet_renderer_gb300.atmosphere.batch import BatchedLutBuilder, Tuning
    from planet_renderer_gb300.atmosphere.workloads import batched_lut_jobs, batched_lut_sets

    device = torch.device("cuda:0")
    builder = BatchedLutBuilder(batched_lut_sets(), device=device)
    jobs = batched_lut_jobs(SEED)[:512]
    tuning = Tuning(64, 4, 3)
    for _ in range(3):
        builder.build(jobs, tuning)
    torch.cuda.synchronize(device)
    builder.close()
    print("profile case batch: 3 launches over 512 jobs")


def _profile_train(args):
    """MLP training and batch inference of the aerial network (11 -> 4x64 ->
    6): 8 Adam steps of 16,384 samples (k_mlp_grad, k_reduce_partials,
    k_adam), then tcgen05 and mma.sync forwards of 2^20 samples."""

    import torch

    from planet_renderer_gb300.atmosphere.mlp import Mlp

    device = torch.device("cuda:0")
    torch.cuda.set_device(device)
    g = torch.Generator(device=device).manual_seed(SEED)
    net = Mlp(11, 4, 6, seed=3, device=device)
    x = torch.rand((16384, 11), device=device, generator=g) * 2 - 1
    t = torch.randn((16384, 6), device=device, generator=g)
    for _ in range(8):
        net.train_step(x, t, lr=1e-3)
    net.pack()
    xb = torch.rand((1 << 20, 11), device=device, generator=g) * 2 - 1
    for precision in ("bf16_tc", "bf16") * 3:
        net.forward(xb, precision)
    torch.cuda.synchronize(device)
    print("profile case train: 8 Adam steps, 3 tcgen05 + 3 mma.sync forwards of 2^20 samples")


def _profile_post(args):
    """The display post-process at 4K (default configuration), three frames."""

    args.steps = 0
    _postprocess_4k(__import__("torch").device("cuda:0"), argparse.Namespace(warmup=3, steps=0))
    print("profile case post4k")


def _profile_shade(args):
    """Surface shading at 4K on the synthetic land-and-ocean G-buffer of the
    2 km camera, three launches."""

    out = _shading_4k(__import__("torch").device("cuda:0"), argparse.Namespace(warmup=3), steps=3)
    print("profile case shade4k:", round(out["ms"], 3), "ms")


def _profile_sky_tiles(args):
    """The learned sky-view workload at 4K (cameras 2 / 20 / 60 km) with the
    sky network trained as the bench trains it, for calibration tiles of 32
    and 64 pixels with 1, 2 and 4% checked pixels, and without the
    calibration: device ms and mean error against the FP64 march at 1,500
    pixels per camera.  (Tiles of 16 pixels hold too few checks at 1%: 3.2%
    error; 128 pixels: 1.44%.)"""

    import numpy as np
    import torch

    from oracle.atm import Oracle
    from planet_renderer_gb300 import camera
    from planet_renderer_gb300.atmosphere import AtmosphereRenderer
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.scene import pixel_rays
    from planet_renderer_gb300.atmosphere.surrogate import (DEFAULT_SPECS, SKY, SampleSource, Surrogate,
                                                            parameter_grid, train)
    from planet_renderer_gb300.atmosphere.workloads import (EARTH_RADIUS_M, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG,
                                                            frame_chain_cameras)

    device = torch.device("cuda:0")
    torch.cuda.set_device(device)
    source = SampleSource(parameter_grid(), device=device)
    net, _ = train(source, SKY, 2**22, 16384, args.mlp_epochs, lr=4e-3, seed=SEED + 1, spec=DEFAULT_SPECS[SKY],
                   log_every=0)
    sg = Surrogate(None, net, source.planet_radius_m, source.top_altitude_m, source.scale_height_range)
    source.close()
    width, height = 3840, 2160
    cfg = earth_baseline()
    r = AtmosphereRenderer(width, height, cfg, device=device)
    out = torch.empty((width, height, 3), device=device)
    o = Oracle("f64")
    ar = math.radians(SUN_ANGULAR_RADIUS_DEG)
    tl = o.build_transmittance(cfg, EARTH_RADIUS_M)
    ms = o.build_multi_scattering(cfg, EARTH_RADIUS_M, SOLAR_IRRADIANCE, ar, tl)
    rng = np.random.default_rng(SEED + 2)
    basis = camera.view_basis(0.0, 15.0)
    tanfov = camera.tangent_half_fov(60.0)
    tiles = ((0, 0.01), (32, 0.01), (64, 0.01), (32, 0.02), (64, 0.02), (32, 0.04))  # (tile, check fraction)
    res = {t: {"ms": 0.0, "err": []} for t in tiles}
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for alt, v in zip(SKY_ALTITUDES_M, frame_chain_cameras(SEED)):
        cr = EARTH_RADIUS_M + alt
        r.update(EARTH_RADIUS_M, cr, v.sun_local.copy(), SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG)
        a = (EARTH_RADIUS_M, cr, v.sun_local, SOLAR_IRRADIANCE, SUN_ANGULAR_RADIUS_DEG, basis, tanfov)
        xs = torch.as_tensor(rng.integers(0, width, 1500))
        ys = torch.as_tensor(rng.integers(0, height, 1500))
        rays = pixel_rays(width, height, basis, tanfov, xs, ys).numpy()
        ref = o.sky_rays(cfg, EARTH_RADIUS_M, np.full(1500, alt), rays, np.tile(v.sun_local, (1500, 1)),
                         SOLAR_IRRADIANCE, ar, tl, ms)
        floor = 1e-4 * np.abs(ref).max()
        for t in tiles:
            sg.calibration_tile = t[0]
            run = lambda: r.sky_pixels(out, *a, mode="net", surrogate=sg, seed=SEED, check_fraction=t[1])
            for _ in range(3):
                run()
            torch.cuda.synchronize(device)
            start.record()
            for _ in range(10):
                run()
            end.record()
            torch.cuda.synchronize(device)
            res[t]["ms"] += start.elapsed_time(end) / 10 / len(SKY_ALTITUDES_M)
            got = out[xs.to(device), ys.to(device)].cpu().numpy().astype(np.float64)
            res[t]["err"].append(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor), axis=1))
    r.close()
    print("profile case sky4k_tiles:", {t: {"ms": round(v["ms"], 4), "err_mean": round(float(np.concatenate(
        v["err"]).mean()), 5)} for t, v in res.items()})


def _profile_raster(args):
    """The terrain raster at 4K, both patch budgets, three frames each."""

    out = _raster_4k(__import__("torch").device("cuda:0"), argparse.Namespace(warmup=3), steps=3)
    print("profile case raster4k:", {k: round(v["ms"], 3) for k, v in out.items() if isinstance(v, dict)})


def _profile_mesh_frame(args):
    """The whole 4K frame from terrain patches to display, three frames."""

    out = _frame_from_mesh_4k(__import__("torch").device("cuda:0"), argparse.Namespace(warmup=3), steps=3)
    print("profile case meshframe4k:", {k: v for k, v in out.items() if k != "workload"})


PROFILE_CASES = {
    "raster4k": _profile_raster,
    "sky4k_tiles": _profile_sky_tiles,
    "meshframe4k": _profile_mesh_frame,
    "frame1080p": _profile_frame_1080p,
    "frame4k_mlp": _profile_frame_4k_mlp,
    "luts": _profile_luts,
    "batch": _profile_batch,
    "train": _profile_train,
    "post4k": _profile_post,
    "shade4k": _profile_shade,
}


if __name__ == "__main__":
    main()
