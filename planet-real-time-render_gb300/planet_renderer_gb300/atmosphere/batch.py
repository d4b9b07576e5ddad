"""Batched sky-view / aerial-perspective LUT builds in one persistent launch.

The reference builds one LUT per kernel launch (``atmosphere/renderer.py``
``_build_sky_view`` :1208 and ``_build_aerial_perspective`` :1304); a batch
here holds many time snapshots x cameras x parameter sets with uneven LUT
sizes and builds them all with one launch of ``atm_batch_build``.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from .. import _native

SKY_VIEW = _native.LUT_SKY_VIEW
AERIAL = _native.LUT_AERIAL


@dataclass(frozen=True)
class BatchJob:
    """One LUT of a batch (what one reference kernel launch computes)."""

    kind: int                 # SKY_VIEW or AERIAL
    param_set: int
    width: int
    height: int
    depth: int = 1
    camera_altitude_m: float = 0.0
    sun_zenith_cosine: float = 1.0           # sky-view (f32-rounded key)
    sun_local: tuple = (0.0, 1.0, 0.0)       # aerial
    view_basis: tuple = ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0))
    tangent_half_fov: float = math.tan(math.radians(30.0))
    frame_width: int = 1920
    frame_height: int = 1080

    @property
    def texels(self) -> int:
        return self.width * self.height * self.depth

    def samples(self, config) -> int:
        """Upper bound of radiance samples (every ray valid)."""

        if self.kind == SKY_VIEW:
            return self.texels * config.sky_view_steps
        return self.texels * config.aerial_steps_per_slice

    def sky_key(self):
        return (self.param_set, float(np.float32(self.camera_altitude_m)), float(np.float32(self.sun_zenith_cosine)))


@dataclass
class Tuning:
    sky_view_texels_per_item: int = 16
    aerial_columns_per_item: int = 4
    blocks_per_sm: int = 3

    def native(self) -> _native.AtmBatchTuning:
        return _native.AtmBatchTuning(self.sky_view_texels_per_item, self.aerial_columns_per_item,
                                      self.blocks_per_sm)


@dataclass
class BatchResult:
    arena: torch.Tensor            # (texels, 4) float32, every LUT at its offset
    offsets: list[int] = field(default_factory=list)
    jobs: list[BatchJob] = field(default_factory=list)

    def lut(self, index: int) -> torch.Tensor:
        """Job ``index``'s LUT in the Taichi field layout (W, H[, D], 3)."""

        j = self.jobs[index]
        o = self.offsets[index]
        v = self.arena[o:o + j.texels, :3].reshape(j.depth, j.height, j.width, 3)
        v = v.permute(2, 1, 0, 3)
        return v[:, :, 0] if j.kind == SKY_VIEW else v


class BatchedLutBuilder:
    """Parameter sets (config, planet radius) sharing irradiance and sun size."""

    def __init__(self, sets, solar_irradiance=(4.0, 3.9, 3.7), sun_angular_radius_degrees=0.266, device=None):
        self._lib = _native.library()
        self.device = torch.device(device if device is not None else f"cuda:{torch.cuda.current_device()}")
        self.sets = list(sets)
        params = (_native.AtmParams * len(self.sets))(*[_native.AtmParams.from_config(c) for c, _ in self.sets])
        radii = (ctypes.c_double * len(self.sets))(*[float(r) for _, r in self.sets])
        self._handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.check(self._lib.atm_batch_create(params, radii, len(self.sets), _native.d3(solar_irradiance),
                                                     float(sun_angular_radius_degrees), ctypes.byref(self._handle),
                                                     self._stream()))

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def close(self):
        if getattr(self, "_handle", None) is not None and self._handle.value:
            self._lib.atm_batch_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def layout(jobs):
        offsets, total = [], 0
        for j in jobs:
            offsets.append(total)
            total += j.texels
        return offsets, total

    def native_jobs(self, jobs, offsets):
        arr = (_native.AtmBatchJob * len(jobs))()
        for a, j, o in zip(arr, jobs, offsets):
            a.kind, a.param_set = j.kind, j.param_set
            a.width, a.height, a.depth = j.width, j.height, j.depth
            a.frame_width, a.frame_height = j.frame_width, j.frame_height
            a.output_offset = o
            a.camera_altitude_m = float(j.camera_altitude_m)
            a.sun_zenith_cosine = float(j.sun_zenith_cosine)
            a.sun_local[:] = [float(v) for v in j.sun_local]
            a.view_basis[:] = [float(v) for vec in j.view_basis for v in vec]
            a.tangent_half_fov = float(j.tangent_half_fov)
        return arr

    def build(self, jobs, tuning: Tuning | None = None, arena: torch.Tensor | None = None,
              prepared=None) -> BatchResult:
        """Build every job's LUT in one launch (asynchronous on the current stream)."""

        tuning = tuning or Tuning()
        if prepared is None:
            offsets, total = self.layout(jobs)
            native = self.native_jobs(jobs, offsets)
        else:
            offsets, total, native = prepared
        if arena is None:
            arena = torch.empty((total, 4), dtype=torch.float32, device=self.device)
        if arena.shape[0] < total or arena.dtype != torch.float32 or not arena.is_contiguous():
            raise ValueError("arena must be a contiguous float32 (texels, 4) CUDA tensor large enough for the jobs")
        t = tuning.native()
        _native.check(self._lib.atm_batch_build(self._handle, native, len(jobs), ctypes.c_void_p(arena.data_ptr()),
                                                arena.shape[0], ctypes.byref(t), self._stream()))
        return BatchResult(arena, offsets, list(jobs))

    def prepare(self, jobs):
        """Host-side job table, reusable across builds of the same jobs."""

        offsets, total = self.layout(jobs)
        return offsets, total, self.native_jobs(jobs, offsets)

    def samples(self, reset: bool = False) -> int:
        out = ctypes.c_uint64()
        _native.check(self._lib.atm_batch_read_samples(self._handle, 1 if reset else 0, ctypes.byref(out),
                                                       self._stream()))
        return int(out.value)


def partition_jobs(jobs, configs, world_size: int, rank: int):
    """Jobs of ``rank`` when a batch is spread over ``world_size`` GPUs:
    greedy longest-first assignment by radiance-sample count, so every rank
    gets a near-equal share; no data moves between ranks (independent LUTs).
    Returns the indices of this rank's jobs, in their original order."""

    if not 0 <= rank < world_size:
        raise ValueError("rank must be in [0, world_size)")
    order = sorted(range(len(jobs)), key=lambda i: -jobs[i].samples(configs[jobs[i].param_set]))
    load = [0] * world_size
    owner = [0] * len(jobs)
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += jobs[i].samples(configs[jobs[i].param_set])
    return [i for i in range(len(jobs)) if owner[i] == rank]
