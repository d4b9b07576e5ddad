"""Small MLPs trained and evaluated by the package's own CUDA kernels.

``Mlp(n_in, n_hidden, n_out)``: n_in -> [64 SiLU] x n_hidden -> n_out.
Training uses the fused FP32 forward/backward kernel and Adam
(``atm_mlp_train_step``); inference runs FP32 on CUDA cores or BF16 on tensor
cores with FP32 accumulation (``atm_mlp_forward``).  Checkpoints hold the
parameters, the Adam state is re-initialised on load.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np
import torch

from .. import _native

HIDDEN = 64


def layer_shapes(n_in: int, n_hidden: int, n_out: int):
    """(out, in) of each layer, in parameter order."""

    dims = [n_in] + [HIDDEN] * n_hidden + [n_out]
    return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]


class Mlp:
    def __init__(self, n_in: int, n_hidden: int, n_out: int, seed: int = 0, device=None):
        self._lib = _native.library()
        self.n_in, self.n_hidden, self.n_out = int(n_in), int(n_hidden), int(n_out)
        self.device = torch.device(device if device is not None else f"cuda:{torch.cuda.current_device()}")
        self._handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.check(self._lib.atm_mlp_create(self.n_in, self.n_hidden, self.n_out, int(seed),
                                                   ctypes.byref(self._handle)))
        n = ctypes.c_int32()
        _native.check(self._lib.atm_mlp_info(self._handle, ctypes.byref(n), None))
        self.n_params = int(n.value)
        self._loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        self._packed = False

    def _s(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    @staticmethod
    def _p(t: torch.Tensor):
        return ctypes.c_void_p(t.data_ptr())

    def close(self):
        if getattr(self, "_handle", None) is not None and self._handle.value:
            self._lib.atm_mlp_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check_io(self, x: torch.Tensor, width: int, name: str) -> torch.Tensor:
        if x.device != self.device or x.dtype != torch.float32 or x.dim() != 2 or x.shape[1] != width:
            raise ValueError(f"{name} must be a float32 CUDA tensor of shape (n, {width})")
        return x.contiguous()

    # -- parameters --------------------------------------------------------------
    def params(self) -> torch.Tensor:
        out = torch.empty(self.n_params, dtype=torch.float32, device=self.device)
        _native.check(self._lib.atm_mlp_get_params(self._handle, self._p(out), self._s()))
        return out

    def set_params(self, values) -> None:
        v = torch.as_tensor(values, dtype=torch.float32).to(self.device).contiguous()
        if v.numel() != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters")
        _native.check(self._lib.atm_mlp_set_params(self._handle, self._p(v), self._s()))
        _native.check(self._lib.atm_mlp_reset_optimizer(self._handle, self._s()))
        torch.cuda.current_stream(self.device).synchronize()
        self._packed = False

    def save(self, path) -> None:
        np.savez(Path(path), params=self.params().cpu().numpy(),
                 shape=np.array([self.n_in, self.n_hidden, self.n_out]))

    @classmethod
    def load(cls, path, device=None) -> "Mlp":
        data = np.load(Path(path))
        n_in, n_hidden, n_out = (int(v) for v in data["shape"])
        m = cls(n_in, n_hidden, n_out, device=device)
        m.set_params(data["params"])
        return m

    # -- training ------------------------------------------------------------------
    def _weights(self, weights, n):
        if weights is None:
            return None
        w = self._check_io(weights, self.n_out, "weights")
        if w.shape[0] != n:
            raise ValueError("weights must have one row per sample")
        return w

    def gradient(self, inputs: torch.Tensor, targets: torch.Tensor, weights: torch.Tensor | None = None):
        """(gradient of the batch's mean weighted squared error, summed
        weighted squared error); no update."""

        x = self._check_io(inputs, self.n_in, "inputs")
        y = self._check_io(targets, self.n_out, "targets")
        w = self._weights(weights, x.shape[0])
        g = torch.empty(self.n_params, dtype=torch.float32, device=self.device)
        _native.check(self._lib.atm_mlp_gradient(self._handle, self._p(x), self._p(y),
                                                 None if w is None else self._p(w), x.shape[0], self._p(g),
                                                 self._p(self._loss), self._s()))
        return g, self._loss.clone()

    def train_step(self, inputs, targets, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, weights=None) -> torch.Tensor:
        """One Adam step; returns the batch's summed (weighted) squared error (device)."""

        x = self._check_io(inputs, self.n_in, "inputs")
        y = self._check_io(targets, self.n_out, "targets")
        w = self._weights(weights, x.shape[0])
        _native.check(self._lib.atm_mlp_train_step(self._handle, self._p(x), self._p(y),
                                                   None if w is None else self._p(w), x.shape[0], float(lr),
                                                   float(betas[0]), float(betas[1]), float(eps), self._p(self._loss),
                                                   self._s()))
        self._packed = False
        return self._loss

    # -- inference -------------------------------------------------------------------
    def pack(self) -> None:
        """Copy the current parameters into the BF16 tensor-core layout."""

        if not self._packed:
            _native.check(self._lib.atm_mlp_pack_bf16(self._handle, self._s()))
            self._packed = True

    def forward(self, inputs: torch.Tensor, precision: str = "f32", out: torch.Tensor | None = None) -> torch.Tensor:
        x = self._check_io(inputs, self.n_in, "inputs")
        if out is None:
            out = torch.empty((x.shape[0], self.n_out), dtype=torch.float32, device=self.device)
        if precision in ("bf16", "bf16_tc"):
            self.pack()
        code = {"f32": 0, "bf16": 1, "bf16_tc": 2}[precision]
        _native.check(self._lib.atm_mlp_forward(self._handle, self._p(x), self._p(out), x.shape[0], code, self._s()))
        return out

    @property
    def handle(self):
        return self._handle
