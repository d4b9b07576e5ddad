"""MLP kernels: FP32 gradients vs the FP64 oracle, FP32 / BF16 forward,
training progress, checkpoint round trip."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _net(n_in, n_hidden, n_out, seed=1):
    from planet_renderer_gb300.atmosphere.mlp import Mlp

    return Mlp(n_in, n_hidden, n_out, seed=seed)


@pytest.mark.parametrize("shape,weighted", [((6, 3, 3), False), ((11, 4, 6), False), ((3, 1, 2), False),
                                            ((11, 4, 6), True), ((16, 2, 8), False)])
def test_gradient_matches_fp64_oracle(shape, weighted):
    import torch

    from oracle import mlp_fp64
    from planet_renderer_gb300.atmosphere.mlp import layer_shapes

    n_in, n_hidden, n_out = shape
    net = _net(*shape)
    rng = np.random.default_rng(7)
    n = 1000  # several training CTAs and a ragged last tile
    x = rng.uniform(-1.0, 1.0, (n, n_in)).astype(np.float32)
    t = rng.normal(0.0, 1.0, (n, n_out)).astype(np.float32)
    w = rng.uniform(0.0, 2.0, (n, n_out)).astype(np.float32) if weighted else None
    g, sq = net.gradient(torch.as_tensor(x, device="cuda"), torch.as_tensor(t, device="cuda"),
                         None if w is None else torch.as_tensor(w, device="cuda"))
    params = net.params().cpu().numpy().astype(np.float64)
    shapes = layer_shapes(n_in, n_hidden, n_out)
    ref = mlp_fp64.gradient(params, shapes, x, t, w)
    got = g.cpu().numpy().astype(np.float64)
    scale = np.abs(ref).max()
    assert np.max(np.abs(got - ref)) <= 1e-4 * scale, np.max(np.abs(got - ref)) / scale
    ref_sq = np.sum((1.0 if w is None else w) * (mlp_fp64.forward(params, shapes, x) - t) ** 2)
    assert abs(float(sq.item()) - ref_sq) <= 1e-4 * ref_sq
    net.close()


def test_forward_fp32_and_bf16():
    import torch

    from oracle import mlp_fp64
    from planet_renderer_gb300.atmosphere.mlp import layer_shapes

    net = _net(11, 4, 6)
    rng = np.random.default_rng(9)
    x = rng.uniform(-1.0, 1.0, (4099, 11)).astype(np.float32)
    xt = torch.as_tensor(x, device="cuda")
    f32 = net.forward(xt, "f32").cpu().numpy()
    bf16 = net.forward(xt, "bf16").cpu().numpy()
    ref = mlp_fp64.forward(net.params().cpu().numpy(), layer_shapes(11, 4, 6), x)
    scale = np.abs(ref).max()
    assert np.max(np.abs(f32 - ref)) <= 1e-5 * scale
    # bf16 operands (8-bit mantissa), fp32 accumulation
    assert np.sqrt(np.mean((bf16 - ref) ** 2)) <= 2e-2 * np.sqrt(np.mean(ref ** 2))
    net.close()


def test_training_reduces_loss_and_checkpoint_round_trip(tmp_path):
    import torch

    from planet_renderer_gb300.atmosphere.mlp import Mlp

    net = _net(3, 2, 2, seed=4)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((65536, 3), device="cuda", generator=g) * 2 - 1
    y = torch.stack([torch.sin(2 * x[:, 0]) * x[:, 1], torch.cos(x[:, 2]) + x[:, 0] ** 2], dim=1)
    first = None
    for k in range(300):
        loss = float(net.train_step(x, y, lr=3e-3).item()) / y.numel()
        first = loss if first is None else first
    assert loss < 0.05 * first
    net.save(tmp_path / "net.npz")
    again = Mlp.load(tmp_path / "net.npz")
    assert torch.equal(again.params(), net.params())
    assert torch.equal(again.forward(x[:100]), net.forward(x[:100]))
    net.close()
    again.close()


@pytest.mark.parametrize("shape", [(11, 4, 6), (6, 3, 3), (16, 2, 8)])
def test_forward_tcgen05_matches_mma_sync(shape):
    """The tcgen05 forward (accumulators in tensor memory) against the
    mma.sync forward of the same BF16 weights and the FP64 network."""

    import torch

    from oracle import mlp_fp64
    from planet_renderer_gb300.atmosphere.mlp import layer_shapes

    net = _net(*shape, seed=3)
    rng = np.random.default_rng(11)
    x = rng.uniform(-1.0, 1.0, (1000, shape[0])).astype(np.float32)  # ragged last tile of 128
    xt = torch.as_tensor(x, device="cuda")
    mma = net.forward(xt, "bf16").cpu().numpy()
    tc = net.forward(xt, "bf16_tc").cpu().numpy()
    ref = mlp_fp64.forward(net.params().cpu().numpy(), layer_shapes(*shape), x)
    scale = np.sqrt(np.mean(ref ** 2))
    assert np.sqrt(np.mean((tc - mma) ** 2)) <= 2e-3 * scale, np.sqrt(np.mean((tc - mma) ** 2)) / scale
    assert np.sqrt(np.mean((tc - ref) ** 2)) <= 2e-2 * scale
    net.close()
