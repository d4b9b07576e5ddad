"""CPU restatement (test infrastructure) of the reference's display
post-process, src/planet_renderer/postprocess.py: bloom extraction at half
resolution with a soft threshold, separable 5-tap blur passes, bilinear bloom
resolve, ACES fit and sRGB encoding.  numpy float32, operation by operation
in the reference's order, with its clamps and edge rules; images are (W, H, 3)
indexed [x, y] like the reference's Taichi fields.  Used only by tests and the
bench's checks, never by the product path."""

from __future__ import annotations

import numpy as np

F = np.float32

# postprocess.py:126-129 (blur weights, centre / +-1 / +-2)
W0, W1, W2 = F(0.38774), F(0.24477), F(0.06136)


def display_from_exposed(value: np.ndarray) -> np.ndarray:
    """_display_from_exposed, postprocess.py:56-73: ACES fit, then sRGB."""

    value = np.maximum(value, F(0.0))
    a, b, c, d, e = F(2.51), F(0.03), F(2.43), F(0.59), F(0.14)
    mapped = np.clip((value * (a * value + b)) / (value * (c * value + d) + e), F(0.0), F(1.0))
    lo = mapped * F(12.92)
    hi = F(1.055) * np.power(mapped, F(1.0 / 2.4)) - F(0.055)
    return np.where(mapped <= F(0.0031308), lo, hi).astype(F)


def soft_threshold(value: np.ndarray, threshold: float, knee: float, clamp: float) -> np.ndarray:
    """PostProcessor._soft_threshold, postprocess.py:88-107."""

    brightness = np.maximum(value[..., 0], np.maximum(value[..., 1], value[..., 2]))
    soft = np.clip(brightness - F(threshold) + F(knee), F(0.0), F(2.0 * knee))
    soft = soft * soft / F(max(4.0 * knee, 1.0e-6))
    contribution = np.maximum(brightness - F(threshold), soft)
    contribution = contribution / np.maximum(brightness, F(1.0e-6))
    result = value * contribution[..., None]
    peak = np.maximum(result[..., 0], np.maximum(result[..., 1], result[..., 2]))
    return (result * np.minimum(F(1.0), F(clamp) / np.maximum(peak, F(1.0e-6)))[..., None]).astype(F)


def half_size(width: int, height: int) -> tuple[int, int]:
    """PostProcessor.__init__, postprocess.py:78-86."""

    return max((int(width) + 1) // 2, 1), max((int(height) + 1) // 2, 1)


def extract(hdr: np.ndarray, exposure_multiplier: float, cfg) -> np.ndarray:
    """_extract, postprocess.py:110-119: 2x2 box at half resolution, edge
    clamped, times 0.25 x exposure, soft threshold."""

    W, H = hdr.shape[:2]
    hw, hh = half_size(W, H)
    xs, ys = np.arange(hw), np.arange(hh)
    value = np.zeros((hw, hh, 3), F)
    for ox in (0, 1):
        for oy in (0, 1):
            sx = np.minimum(xs * 2 + ox, W - 1)
            sy = np.minimum(ys * 2 + oy, H - 1)
            value = value + hdr[sx][:, sy, :3]
    value = value * (F(0.25) * F(exposure_multiplier))
    return soft_threshold(value, cfg.bloom_threshold, cfg.bloom_knee, cfg.bloom_clamp)


def blur_horizontal(a: np.ndarray) -> np.ndarray:
    """_blur_horizontal, postprocess.py:121-129 (indices clamped)."""

    hw = a.shape[0]
    x = np.arange(hw)
    at = lambda k: a[np.clip(x + k, 0, hw - 1)]
    return (at(0) * W0 + at(-1) * W1 + at(1) * W1 + at(-2) * W2 + at(2) * W2).astype(F)


def blur_vertical(b: np.ndarray) -> np.ndarray:
    """_blur_vertical, postprocess.py:131-139."""

    hh = b.shape[1]
    y = np.arange(hh)
    at = lambda k: b[:, np.clip(y + k, 0, hh - 1)]
    return (at(0) * W0 + at(-1) * W1 + at(1) * W1 + at(-2) * W2 + at(2) * W2).astype(F)


def sample_bloom(bloom: np.ndarray, width: int, height: int) -> np.ndarray:
    """_sample_bloom, postprocess.py:141-153, at every pixel centre
    (u, v) = ((x + 0.5) / W, (y + 0.5) / H)."""

    hw, hh = bloom.shape[:2]
    u = (np.arange(width, dtype=F) + F(0.5)) / F(width)
    v = (np.arange(height, dtype=F) + F(0.5)) / F(height)
    px = u * F(hw) - F(0.5)
    py = v * F(hh) - F(0.5)
    fpx, fpy = np.floor(px), np.floor(py)
    x0 = np.clip(fpx.astype(np.int64), 0, hw - 1)
    y0 = np.clip(fpy.astype(np.int64), 0, hh - 1)
    x1 = np.minimum(x0 + 1, hw - 1)
    y1 = np.minimum(y0 + 1, hh - 1)
    fx = np.clip(px - fpx, F(0.0), F(1.0))[:, None, None]
    fy = np.clip(py - fpy, F(0.0), F(1.0))[None, :, None]
    b00, b10 = bloom[x0][:, y0], bloom[x1][:, y0]
    b01, b11 = bloom[x0][:, y1], bloom[x1][:, y1]
    low = b00 * (F(1.0) - fx) + b10 * fx
    high = b01 * (F(1.0) - fx) + b11 * fx
    return (low * (F(1.0) - fy) + high * fy).astype(F)


def process(hdr: np.ndarray, exposure_ev: float, cfg, *, bloom: bool, tone_map: bool) -> np.ndarray:
    """PostProcessor.process + _resolve, postprocess.py:155-207.  hdr is
    (W, H, >=3) float32; returns the (W, H, 3) display image."""

    hdr = np.asarray(hdr, F)
    W, H = hdr.shape[:2]
    em = F(2.0 ** float(exposure_ev) if tone_map else 1.0)
    use_bloom = bool(bloom and cfg.bloom_passes > 0 and cfg.bloom_strength > 0.0)
    value = hdr[..., :3] * em
    if use_bloom:
        a = extract(hdr, float(em), cfg)
        for _ in range(cfg.bloom_passes):
            a = blur_vertical(blur_horizontal(a))
        value = value + sample_bloom(a, W, H) * F(cfg.bloom_strength)
    if tone_map:
        return display_from_exposed(value)
    return np.clip(value, F(0.0), F(1.0)).astype(F)
