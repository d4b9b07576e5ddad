"""Display post-process on the GPU (PostProcessor through atm_post_process)
against the reference's own outputs (golden vectors) and the oracle
restatement: the kernels follow the reference's float32 operations without
contraction, so results agree to the last bit except where powf's last bit
differs in the sRGB segment (tolerance 4 ulp at 1.0)."""

from __future__ import annotations

import json
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "postprocess.npz"
DEFAULTS = dict(exposure_ev=0.0, bloom_threshold=1.0, bloom_knee=0.5, bloom_clamp=8.0, bloom_strength=0.08,
                bloom_passes=4)
DISPLAY_ATOL = 4 * 2.0 ** -24 * 2  # 4 ulp at 1.0


def _processor(width, height, config, layout="wh"):
    from planet_renderer_gb300.postprocess import PostprocessConfig, PostProcessor

    return PostProcessor(width, height, PostprocessConfig(**config), layout=layout)


def _run(pp, hdr_np, ev, bloom, tone_map, channels=3, layout="wh"):
    hdr = torch.as_tensor(hdr_np, device="cuda")
    if layout == "hw":
        hdr = hdr.permute(1, 0, 2).contiguous()
    if channels == 4:
        hdr = torch.cat([hdr, torch.full_like(hdr[..., :1], 7.0)], dim=-1).contiguous()
    before = hdr.clone()
    display = torch.full_like(hdr, -1.0)
    pp.process(hdr, display, ev, bloom=bloom, tone_map=tone_map)
    torch.cuda.synchronize()
    assert torch.equal(hdr, before), "the HDR source was modified"
    out = display[..., :3]
    if layout == "hw":
        out = out.permute(1, 0, 2)
    if channels == 4:
        assert bool((display[..., 3] == -1.0).all()), "the fourth channel was written"
    return out.cpu().numpy()


def test_golden_vectors_of_the_reference():
    g = np.load(GOLDEN)
    meta = json.loads(str(g["meta"]))
    exact = total = 0
    for k in range(meta["cases"]):
        a = json.loads(str(g[f"case{k}_args"]))
        pp = _processor(a["width"], a["height"], a["config"])
        got = _run(pp, g[f"case{k}_hdr"], a["exposure_ev"], a["bloom"], a["tone_map"])
        ref = g[f"case{k}_display"]
        np.testing.assert_allclose(got, ref, rtol=0, atol=DISPLAY_ATOL, err_msg=f"case {k}: {a}")
        exact += int((got == ref).sum())
        total += ref.size
        pp.close()
    print(f"post-process golden: {exact}/{total} values bit-identical")


@pytest.mark.parametrize("width,height,channels,layout", [(321, 187, 3, "wh"), (320, 180, 4, "wh"),
                                                          (97, 61, 3, "hw"), (2, 3, 4, "hw")])
def test_against_the_oracle(width, height, channels, layout):
    from oracle import postprocess as op

    rng = np.random.default_rng(width * 1000 + height)
    hdr = np.exp(rng.normal(-1.0, 2.0, (width, height, 3))).astype(np.float32)
    hdr[rng.integers(0, width, 20), rng.integers(0, height, 20)] *= np.float32(2.0e4)
    config = dict(bloom_threshold=0.8, bloom_knee=0.3, bloom_clamp=6.0, bloom_strength=0.2, bloom_passes=5)
    cfg = SimpleNamespace(**{**DEFAULTS, **config})
    pp = _processor(width, height, config, layout)
    for ev, bloom, tone_map in ((0.5, True, True), (-3.0, True, True), (0.0, False, True), (2.0, True, False)):
        got = _run(pp, hdr, ev, bloom, tone_map, channels, layout)
        ref = op.process(hdr, ev, cfg, bloom=bloom, tone_map=tone_map)
        np.testing.assert_allclose(got, ref, rtol=0, atol=DISPLAY_ATOL, err_msg=f"ev {ev} bloom {bloom}")
    pp.close()


def test_bloom_plane_against_the_oracle():
    """The half-resolution bloom after extraction and the blur passes."""

    from oracle import postprocess as op

    width, height = 203, 117
    rng = np.random.default_rng(3)
    hdr = np.exp(rng.normal(0.0, 1.5, (width, height, 3))).astype(np.float32)
    for passes in (1, 4, 8):
        config = dict(bloom_passes=passes)
        cfg = SimpleNamespace(**{**DEFAULTS, **config})
        pp = _processor(width, height, config)
        _run(pp, hdr, 1.0, True, True)
        got = pp.bloom_plane().cpu().numpy()
        a = op.extract(hdr, float(np.float32(2.0)), cfg)
        for _ in range(passes):
            a = op.blur_vertical(op.blur_horizontal(a))
        assert got.shape == a.shape
        np.testing.assert_allclose(got, a, rtol=2.0 ** -22, atol=0)
        pp.close()


def test_4k_frame_is_finite_and_in_range():
    width, height = 3840, 2160
    g = torch.Generator(device="cuda").manual_seed(5)
    hdr = torch.exp(torch.randn((width, height, 3), device="cuda", generator=g) * 1.5 - 1.0)
    display = torch.empty_like(hdr)
    pp = _processor(width, height, {})
    pp.process(hdr, display, 0.0, bloom=True, tone_map=True)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(display).all()) and float(display.min()) >= 0.0 and float(display.max()) <= 1.0
    pp.close()


def test_image_checks():
    pp = _processor(64, 32, {})
    hdr = torch.zeros((64, 32, 3), device="cuda")
    with pytest.raises(ValueError):
        pp.process(hdr, torch.zeros((32, 64, 3), device="cuda"), 0.0, bloom=True, tone_map=True)
    with pytest.raises(ValueError):
        pp.process(torch.zeros((63, 32, 3), device="cuda"), torch.zeros((63, 32, 3), device="cuda"), 0.0,
                   bloom=True, tone_map=True)
    pp.close()
