"""Host-side camera geometry in the local East-Up-North frame.

``view_basis(yaw, pitch)`` follows the reference's
``PlanetCamera.view_basis_local`` (``camera.py:24-33``); ``sun_local`` follows
the azimuth/elevation convention of ``cli.py:80-94``.  All float64.
"""

from __future__ import annotations

import math

import numpy as np

UP = np.array([0.0, 1.0, 0.0])


def _normalize(v: np.ndarray) -> np.ndarray:
    return v / float(np.linalg.norm(v))


def view_basis(yaw_degrees: float, pitch_degrees: float):
    """Return (right, view_up, forward) for a camera with this yaw/pitch."""

    yaw = math.radians(yaw_degrees)
    pitch = math.radians(float(np.clip(pitch_degrees, -89.0, 89.0)))
    horizontal = np.array([math.sin(yaw), 0.0, math.cos(yaw)])
    forward = _normalize(horizontal * math.cos(pitch) + UP * math.sin(pitch))
    right = _normalize(np.cross(UP, forward))
    view_up = _normalize(np.cross(forward, right))
    return right, view_up, forward


def sun_local(azimuth_degrees: float, elevation_degrees: float) -> np.ndarray:
    az = math.radians(azimuth_degrees)
    el = math.radians(elevation_degrees)
    return np.array(
        [math.sin(az) * math.cos(el), math.sin(el), math.cos(az) * math.cos(el)]
    )


def sun_from_zenith(zenith_degrees: float, azimuth_degrees: float = 0.0) -> np.ndarray:
    return sun_local(azimuth_degrees, 90.0 - zenith_degrees)


def tangent_half_fov(vertical_fov_degrees: float) -> float:
    return math.tan(math.radians(vertical_fov_degrees) / 2.0)
