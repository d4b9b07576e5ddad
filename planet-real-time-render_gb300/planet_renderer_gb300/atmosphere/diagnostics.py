"""Composite diagnostic views (reference ``atmosphere/diagnostics.py:12-60``).

The integer values are part of the C ABI (``ATM_VIEW_*`` in atm_capi.h) and
equal the reference's enum values.
"""

from __future__ import annotations

from enum import IntEnum


class AtmosphereDiagnosticView(IntEnum):
    """Select what the composite writes into ``hdr``."""

    COMPOSITE = 0
    SKY_VIEW = 1
    CAMERA_TRANSMITTANCE = 2
    TRANSMITTANCE_LUT = 3
    MULTI_SCATTERING_LUT = 4
    AERIAL_SCATTERING = 5
    AERIAL_TRANSMITTANCE = 6
    SURFACE_MASK = 7
    AERIAL_FROXEL_ONLY = 8
    AERIAL_DIRECT_ONLY = 9
    AERIAL_BLEND_WEIGHT = 10

    @property
    def label(self) -> str:
        return _LABELS[self]

    @property
    def is_radiance(self) -> bool:
        """Whether this view holds radiance (needs exposure and tone mapping)."""

        return self in _RADIANCE

    @property
    def uses_bloom(self) -> bool:
        """Bloom belongs to the final composition only."""

        return self is AtmosphereDiagnosticView.COMPOSITE


_LABELS = {
    AtmosphereDiagnosticView.COMPOSITE: "Composite",
    AtmosphereDiagnosticView.SKY_VIEW: "Sky-view radiance",
    AtmosphereDiagnosticView.CAMERA_TRANSMITTANCE: "Camera transmittance",
    AtmosphereDiagnosticView.TRANSMITTANCE_LUT: "Transmittance LUT",
    AtmosphereDiagnosticView.MULTI_SCATTERING_LUT: "Multi-scattering LUT",
    AtmosphereDiagnosticView.AERIAL_SCATTERING: "Aerial scattering",
    AtmosphereDiagnosticView.AERIAL_TRANSMITTANCE: "Aerial transmittance",
    AtmosphereDiagnosticView.SURFACE_MASK: "Surface mask",
    AtmosphereDiagnosticView.AERIAL_FROXEL_ONLY: "Aerial froxel only",
    AtmosphereDiagnosticView.AERIAL_DIRECT_ONLY: "Aerial direct only",
    AtmosphereDiagnosticView.AERIAL_BLEND_WEIGHT: "Aerial blend weight",
}

_RADIANCE = frozenset(
    {
        AtmosphereDiagnosticView.COMPOSITE,
        AtmosphereDiagnosticView.SKY_VIEW,
        AtmosphereDiagnosticView.MULTI_SCATTERING_LUT,
        AtmosphereDiagnosticView.AERIAL_SCATTERING,
        AtmosphereDiagnosticView.AERIAL_FROXEL_ONLY,
        AtmosphereDiagnosticView.AERIAL_DIRECT_ONLY,
    }
)

__all__ = ["AtmosphereDiagnosticView"]
