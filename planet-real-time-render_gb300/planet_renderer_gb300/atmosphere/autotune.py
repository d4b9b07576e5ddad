"""Autotuner of the batched LUT builder's work split.

Times candidate ``Tuning`` values (texels per sky-view work item, columns per
aerial work item, resident blocks per SM) on a sample of a batch's jobs with
CUDA events, keeps the fastest and caches it in a JSON file keyed by the GPU,
the native library build and the batch's job mix, so later runs with the same
mix skip the search.
"""

from __future__ import annotations

import hashlib
import json
import os
from collections import Counter
from pathlib import Path

import torch

from .. import _native
from .batch import BatchedLutBuilder, Tuning

CANDIDATES = [
    Tuning(sv, ap, b)
    for sv in (4, 16, 64)
    for ap in (1, 4, 16)
    for b in (2, 3)
]


def cache_path() -> Path:
    base = os.environ.get("PLANET_ATM_AUTOTUNE_CACHE")
    if base:
        return Path(base)
    root = Path(os.environ.get("XDG_CACHE_HOME", Path.home() / ".cache"))
    return root / "planet_renderer_gb300" / "autotune.json"


def mix_key(jobs, device) -> str:
    """GPU name, SM count, library build and job-mix histogram, hashed."""

    props = torch.cuda.get_device_properties(device)
    lib = _native.LIBRARY_PATH
    build = f"{lib.stat().st_size}:{int(lib.stat().st_mtime)}" if lib.exists() else "none"
    mix = Counter((j.kind, j.width, j.height, j.depth) for j in jobs)
    text = json.dumps([props.name, props.multi_processor_count, build, sorted(mix.items())])
    return hashlib.sha256(text.encode()).hexdigest()[:24]


def _time(builder: BatchedLutBuilder, prepared, jobs, tuning: Tuning, arena, reps: int) -> float:
    builder.build(jobs, tuning, arena=arena, prepared=prepared)  # warm-up
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(reps):
        builder.build(jobs, tuning, arena=arena, prepared=prepared)
    end.record()
    torch.cuda.synchronize(builder.device)
    return start.elapsed_time(end) / reps


def tune(builder: BatchedLutBuilder, jobs, sample_every: int = 8, reps: int = 2, use_cache: bool = True,
         candidates=None) -> tuple[Tuning, dict]:
    """Best tuning for ``jobs`` and a report {tuning: ms} of the search."""

    key = mix_key(jobs, builder.device)
    path = cache_path()
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        t = cache[key]["tuning"]
        return Tuning(**t), {"cached": True, "key": key}
    subset = jobs[::max(sample_every, 1)]
    prepared = builder.prepare(subset)
    arena = torch.empty((prepared[1], 4), dtype=torch.float32, device=builder.device)
    report = {}
    best, best_ms = None, float("inf")
    for t in candidates or CANDIDATES:
        ms = _time(builder, prepared, subset, t, arena, reps)
        report[f"{t.sky_view_texels_per_item}/{t.aerial_columns_per_item}/{t.blocks_per_sm}"] = ms
        if ms < best_ms:
            best, best_ms = t, ms
    builder.samples(reset=True)
    if use_cache:
        cache[key] = {"tuning": best.__dict__, "ms_on_sample": best_ms, "sample_every": sample_every}
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1))
        os.replace(tmp, path)
    return best, {"cached": False, "key": key, "search_ms": report}
