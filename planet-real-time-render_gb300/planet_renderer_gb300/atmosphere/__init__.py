"""Spherical Rayleigh/Mie/ozone atmosphere on GB300.

Same public names as the reference's ``planet_renderer.atmosphere``.  The
renderer module loads the native library on first use, so importing the
config, diagnostics or scene helpers needs no GPU.
"""

from .config import AtmosphereConfig
from .diagnostics import AtmosphereDiagnosticView

__all__ = ["AtmosphereConfig", "AtmosphereDiagnosticView", "AtmosphereRenderer"]


def __getattr__(name):
    if name == "AtmosphereRenderer":
        from .renderer import AtmosphereRenderer

        return AtmosphereRenderer
    raise AttributeError(name)
