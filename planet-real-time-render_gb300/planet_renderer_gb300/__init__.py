"""GB300-native atmosphere hot path of the planet renderer.

``planet_renderer_gb300.atmosphere`` mirrors the reference package
``planet_renderer.atmosphere``: ``AtmosphereConfig``, ``AtmosphereDiagnosticView``
and ``AtmosphereRenderer`` (whose LUT builds and composite run as sm_103a CUDA
kernels behind the C ABI of ``include/atm_capi.h``).
"""

__version__ = "0.1.0"
