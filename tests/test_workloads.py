"""Seeded workload definitions (no GPU): the surrogate frame sweep's cameras."""

from __future__ import annotations

import numpy as np


def test_surrogate_sweep_cameras_are_seeded_and_in_range():
    from planet_renderer_gb300.atmosphere.workloads import PITCH_DEG, surrogate_sweep_cameras

    a = surrogate_sweep_cameras(7, 64)
    b = surrogate_sweep_cameras(7, 64)
    assert len(a) == 64 and a == b
    alt = np.array([v.altitude_m for v in a])
    assert alt.min() >= 1.0 and alt.max() <= 4.0e6
    # log-uniform: about half of the cameras below the geometric middle (2 km)
    assert 20 <= int((alt < 2000.0).sum()) <= 44
    assert all(0.0 <= v.sun_zenith_deg <= 100.0 and v.pitch_deg == PITCH_DEG for v in a)
