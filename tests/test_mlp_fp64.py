"""The FP64 MLP oracle's analytic gradient agrees with finite differences."""

from __future__ import annotations

import numpy as np


import pytest


@pytest.mark.parametrize("weighted", [False, True])
def test_fp64_analytic_gradient_matches_finite_differences(weighted):
    from oracle import mlp_fp64
    from planet_renderer_gb300.atmosphere.mlp import layer_shapes

    rng = np.random.default_rng(3)
    shapes = layer_shapes(7, 2, 6)
    n = sum(o * i + o for o, i in shapes)
    params = rng.normal(0.0, 0.3, n)
    x = rng.uniform(-1, 1, (40, 7))
    t = rng.normal(0.0, 1.0, (40, 6))
    w = rng.uniform(0.0, 2.0, (40, 6)) if weighted else None
    g = mlp_fp64.gradient(params, shapes, x, t, w)
    idx = rng.choice(n, 60, replace=False)
    fd = mlp_fp64.finite_difference(params, shapes, x, t, idx, weights=w)
    np.testing.assert_allclose(g[idx], fd, rtol=1e-5, atol=1e-8)
