"""Drop-in display post-process: ``PostprocessConfig`` and ``PostProcessor``
with the reference's constructor, fields, validation and ``process`` call
(``src/planet_renderer/postprocess.py:10-207``), backed by the sm_103a
kernels of libplanet_atm (``atm_post_*`` in the C ABI).

``process(hdr, display, exposure_ev, *, bloom, tone_map)`` reads a linear HDR
image and writes the display image: bloom at half resolution (2x2 extract
with a soft threshold and a bright-pass cap, then ``bloom_passes`` separable
5-tap blurs), exposure, bilinear bloom, ACES fit and sRGB encoding.  Images
are torch CUDA float32 tensors ``(W, H, 3|4)`` - the layout of the
reference's Taichi fields - or ``(H, W, 3|4)`` with ``layout="hw"``; work is
enqueued on the current torch CUDA stream.  There is no CPU path.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Mapping

import torch

from . import _native


@dataclass(frozen=True)
class PostprocessConfig:
    """Display parameters kept separate from physical scene radiance
    (postprocess.py:10-53); the same fields, defaults, checks and messages."""

    exposure_ev: float = 0.0
    bloom_threshold: float = 1.0
    bloom_knee: float = 0.5
    bloom_clamp: float = 8.0
    bloom_strength: float = 0.08
    bloom_passes: int = 4

    def __post_init__(self) -> None:
        if not math.isfinite(self.exposure_ev) or not -20.0 <= self.exposure_ev <= 20.0:
            raise ValueError("postprocess.exposure_ev must be finite and in [-20, 20]")
        for name in ("bloom_threshold", "bloom_knee", "bloom_clamp", "bloom_strength"):
            value = getattr(self, name)
            if not math.isfinite(value) or value < 0.0:
                raise ValueError(f"postprocess.{name} must be finite and non-negative")
        if not 0 <= self.bloom_passes <= 8:
            raise ValueError("postprocess.bloom_passes must be in 0..8")

    @classmethod
    def from_mapping(cls, values: Mapping[str, object]) -> "PostprocessConfig":
        defaults = cls()
        return cls(**{name: type(getattr(defaults, name))(values.get(name, getattr(defaults, name)))
                      for name in ("exposure_ev", "bloom_threshold", "bloom_knee", "bloom_clamp",
                                   "bloom_strength", "bloom_passes")})

    def native(self) -> _native.AtmPostConfig:
        return _native.AtmPostConfig(float(self.exposure_ev), float(self.bloom_threshold), float(self.bloom_knee),
                                     float(self.bloom_clamp), float(self.bloom_strength), int(self.bloom_passes))


class PostProcessor:
    """Half-resolution bloom followed by the sole display transform
    (postprocess.py:75-207)."""

    def __init__(self, width: int, height: int, config: PostprocessConfig, device=None, layout: str = "wh"):
        if layout not in ("wh", "hw"):
            raise ValueError("layout must be 'wh' (Taichi field layout) or 'hw'")
        self._lib = _native.library()
        self.width = int(width)
        self.height = int(height)
        self.half_width = max((self.width + 1) // 2, 1)
        self.half_height = max((self.height + 1) // 2, 1)
        self.config = config
        self.layout = layout
        self.device = torch.device(device if device is not None else f"cuda:{torch.cuda.current_device()}")
        if self.device.type != "cuda":
            raise ValueError("PostProcessor runs on a CUDA device only")
        self._handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            cfg = config.native()
            _native.check(self._lib.atm_post_create(ctypes.byref(cfg), self.width, self.height,
                                                    ctypes.byref(self._handle)))

    def close(self) -> None:
        if getattr(self, "_handle", None) is not None and self._handle.value:
            self._lib.atm_post_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _image(self, hdr: torch.Tensor, display: torch.Tensor) -> _native.AtmImage:
        spec = None
        for t in (hdr, display):
            if not isinstance(t, torch.Tensor) or t.device != self.device or t.dtype != torch.float32:
                raise ValueError("images must be float32 CUDA tensors on the post-processor's device")
            if t.dim() != 3 or t.shape[2] not in (3, 4) or t.stride(2) != 1:
                raise ValueError("images must have shape (W, H, 3|4) with contiguous channels")
            c = int(t.shape[2])
            if t.stride(0) % c or t.stride(1) % c:
                raise ValueError("image strides must be whole pixels")
            if self.layout == "wh":
                this = (int(t.shape[0]), int(t.shape[1]), t.stride(0) // c, t.stride(1) // c, c)
            else:
                this = (int(t.shape[1]), int(t.shape[0]), t.stride(1) // c, t.stride(0) // c, c)
            if spec is None:
                spec = this
            elif this != spec:
                raise ValueError("hdr and display must share shape, strides and channels")
        return _native.AtmImage(*spec)

    def process(self, hdr: torch.Tensor, display: torch.Tensor, exposure_ev: float, *, bloom: bool,
                tone_map: bool) -> None:
        """Convert one HDR frame without ever modifying the HDR source."""

        image = self._image(hdr, display)
        _native.check(self._lib.atm_post_process(
            self._handle, ctypes.c_void_p(hdr.data_ptr()), ctypes.c_void_p(display.data_ptr()), ctypes.byref(image),
            float(exposure_ev), 1 if bloom else 0, 1 if tone_map else 0,
            ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)))

    def bloom_plane(self) -> torch.Tensor:
        """Copy of the half-resolution bloom of the last ``process`` that ran
        bloom, shape ``(half_width, half_height, 3)`` like the reference's
        ``bloom_a`` field."""

        out = torch.empty((self.half_height, self.half_width, 4), dtype=torch.float32, device=self.device)
        dims = (ctypes.c_int32 * 2)()
        _native.check(self._lib.atm_post_read_bloom(self._handle, dims, ctypes.c_void_p(out.data_ptr()),
                                                    ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)))
        return out[..., :3].permute(1, 0, 2).contiguous()
