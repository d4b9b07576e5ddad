"""Batched LUT builds (one persistent launch) vs the single-LUT kernels and
the oracle; autotuner cache."""

from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import assert_exact_parity, assert_parity

pytestmark = pytest.mark.gpu


def _small_batch():
    from planet_renderer_gb300.atmosphere.workloads import batched_lut_jobs, batched_lut_sets

    return batched_lut_sets(), batched_lut_jobs(seed=11, snapshots=3, cameras=3)


def test_batch_matches_single_lut_kernels():
    import dataclasses

    import torch

    from planet_renderer_gb300.atmosphere import AtmosphereRenderer
    from planet_renderer_gb300.atmosphere.batch import AERIAL, SKY_VIEW, BatchedLutBuilder, Tuning

    sets, jobs = _small_batch()
    builder = BatchedLutBuilder(sets)
    builder.samples(reset=True)
    result = builder.build(jobs, Tuning(16, 4, 3))
    torch.cuda.synchronize()
    batch_samples = builder.samples(reset=True)
    single_samples = 0
    for i, j in enumerate(jobs):
        cfg, radius = sets[j.param_set]
        if j.kind == SKY_VIEW:
            cfg = dataclasses.replace(cfg, sky_view_lut_width=j.width, sky_view_lut_height=j.height)
        else:
            cfg = dataclasses.replace(cfg, aerial_lut_width=j.width, aerial_lut_height=j.height,
                                      aerial_lut_depth=j.depth)
        r = AtmosphereRenderer(j.frame_width, j.frame_height, cfg)
        r.build_lut("transmittance", planet_radius_m=radius)
        r.build_lut("multi_scattering", planet_radius_m=radius)
        r.radiance_samples(reset=True)
        if j.kind == SKY_VIEW:
            r.build_lut("sky_view", planet_radius_m=radius, camera_altitude_m=j.camera_altitude_m,
                        sun_zenith_cosine=j.sun_zenith_cosine)
            ref = r.sky_view_lut.to_torch()
        else:
            r.build_lut("aerial", planet_radius_m=radius, camera_altitude_m=j.camera_altitude_m,
                        sun_local=j.sun_local, view_basis=j.view_basis, tangent_half_fov=j.tangent_half_fov)
            ref = r.aerial_scattering_lut.to_torch()
        single_samples += r.radiance_samples(reset=True)
        got = result.lut(i)
        # same device functions in another kernel: FMA contraction may differ in the last bits,
        # amplified up to ~1e-5 at texels grazing the limb
        assert_parity(got.cpu().numpy(), ref.cpu().numpy(), f"job {i} kind {j.kind} {j.width}x{j.height}x{j.depth}",
                      rtol=1e-4, atol_frac=1e-6)
        r.close()
    assert batch_samples == single_samples
    builder.close()


def test_batch_matches_oracle():
    """Batched LUTs against the oracle.  The small batch holds cameras 3 m
    above the ground, where the reference's float32 segment weight cancels:
    the comparison is against the float64 oracle with the reference's own
    float32 deviation allowed (``assert_exact_parity``)."""
    import dataclasses

    import torch

    from oracle.atm import Oracle
    from planet_renderer_gb300.atmosphere.batch import SKY_VIEW, BatchedLutBuilder, Tuning

    sets, jobs = _small_batch()
    builder = BatchedLutBuilder(sets)
    result = builder.build(jobs, Tuning(64, 1, 2))
    torch.cuda.synchronize()
    E = (4.0, 3.9, 3.7)
    oracles = {"f32": (Oracle("f32"), float(np.float32(math.radians(0.266)))),
               "f64": (Oracle("f64"), math.radians(0.266))}
    for i in (0, 1, 2, 3, len(jobs) - 2, len(jobs) - 1):
        j = jobs[i]
        cfg, radius = sets[j.param_set]
        refs = {}
        for prec, (oracle, ar) in oracles.items():
            tl = oracle.build_transmittance(cfg, radius)
            ms = oracle.build_multi_scattering(cfg, radius, E, ar, tl)
            if j.kind == SKY_VIEW:
                c = dataclasses.replace(cfg, sky_view_lut_width=j.width, sky_view_lut_height=j.height)
                refs[prec] = oracle.build_sky_view(c, radius, j.camera_altitude_m, j.sun_zenith_cosine, E, ar, tl, ms)
            else:
                c = dataclasses.replace(cfg, aerial_lut_width=j.width, aerial_lut_height=j.height,
                                        aerial_lut_depth=j.depth)
                refs[prec] = oracle.build_aerial(c, j.frame_width, j.frame_height, radius, j.camera_altitude_m,
                                                 j.sun_local, E, math.radians(0.266), j.view_basis,
                                                 j.tangent_half_fov, tl, ms)
        assert_exact_parity(result.lut(i).cpu().numpy(), refs["f32"], refs["f64"], f"batch job {i}")
    builder.close()


def test_batch_rejects_bad_jobs():
    import dataclasses

    import torch

    from planet_renderer_gb300.atmosphere.batch import BatchedLutBuilder

    sets, jobs = _small_batch()
    builder = BatchedLutBuilder(sets)
    arena = torch.empty((10, 4), device="cuda")
    with pytest.raises(ValueError):
        builder.build(jobs[:1], arena=arena)  # arena too small
    with pytest.raises(ValueError):
        builder.build([dataclasses.replace(jobs[0], param_set=7)])
    with pytest.raises(ValueError):
        builder.build([dataclasses.replace(jobs[0], width=4)])
    builder.close()


def test_autotuner_picks_and_caches(tmp_path, monkeypatch):
    from planet_renderer_gb300.atmosphere import autotune
    from planet_renderer_gb300.atmosphere.batch import BatchedLutBuilder, Tuning

    monkeypatch.setenv("PLANET_ATM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    sets, jobs = _small_batch()
    builder = BatchedLutBuilder(sets)
    cands = [Tuning(4, 1, 2), Tuning(64, 8, 3)]
    best, report = autotune.tune(builder, jobs, sample_every=1, reps=1, candidates=cands)
    assert not report["cached"] and best in cands and len(report["search_ms"]) == 2
    again, report2 = autotune.tune(builder, jobs, sample_every=1, reps=1, candidates=cands)
    assert report2["cached"] and again == best
    builder.close()
