"""atm_composite_noalloc: the composite for callers that may not allocate
device memory (an engine or plugin host owning every allocation, a real-time
frame loop that cannot take an allocation's synchronisation, a fixed memory
budget).  Called through the C ABI, it must give the same image and the same
radiance-sample count as atm_composite on the same inputs, on two calls in a
row (the second call reuses the library's fixed scratch array).

Collected last (file name) so that a run stopping at the first failure has
run every other test first; it also passes alone in a fresh process.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import assert_parity

pytestmark = pytest.mark.gpu


def test_noalloc_composite_matches_composite_twice():
    import torch

    from oracle.atm import sun_disk_radiance
    from planet_renderer_gb300 import _native
    from planet_renderer_gb300.atmosphere import AtmosphereRenderer, scene
    from planet_renderer_gb300.atmosphere.config import earth_baseline
    from planet_renderer_gb300.atmosphere.workloads import frame_chain_cameras

    W, H = 320, 180
    cfg = earth_baseline()
    R = 6_360_000.0
    E = (4.0, 3.9, 3.7)
    disk = sun_disk_radiance(E, 0.266)
    lib = _native.library()
    params = _native.AtmParams.from_config(cfg)
    for view in frame_chain_cameras(2027):
        cr = view.camera_radius_m
        sun = view.sun_local
        gb = scene.synthesize_gbuffer(W, H, R, view.altitude_m, view.basis, view.tangent_half_fov, sun, E,
                                      device="cuda")
        r = AtmosphereRenderer(W, H, cfg)
        r.update(R, cr, sun.copy(), E, 0.266)
        r.prepare_frame(gb["position_view"], gb["surface_id"], R, cr, sun, E, 0.266, view.basis,
                        view.tangent_half_fov)
        ref = torch.zeros_like(gb["scene_hdr"])
        r.radiance_samples(reset=True)
        r.composite(gb["scene_hdr"], gb["space_hdr"], gb["surface_id"], gb["position_view"], ref, R, cr, sun, E,
                    disk, 0.266, view.basis, view.tangent_half_fov, 4.0, 12.0)
        ref_samples = r.radiance_samples(reset=True)
        luts = [r.transmittance_lut.device_ptr, r.multi_scattering_lut.device_ptr, r.sky_view_lut.device_ptr]
        image = _native.AtmImage(W, H, gb["scene_hdr"].stride(0) // 3, gb["scene_hdr"].stride(1) // 3, 3)
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        for call in range(2):
            out = torch.full_like(gb["scene_hdr"], float("nan"))
            count = torch.zeros(1, dtype=torch.int64, device="cuda")
            rc = lib.atm_composite_noalloc(
                ctypes.byref(params), *(ctypes.c_void_p(p) for p in luts),
                ctypes.c_void_p(gb["scene_hdr"].data_ptr()), ctypes.c_void_p(gb["space_hdr"].data_ptr()),
                ctypes.c_void_p(gb["surface_id"].data_ptr()), ctypes.c_void_p(gb["position_view"].data_ptr()),
                ctypes.c_void_p(out.data_ptr()), ctypes.byref(image), R, cr, r.sky_snapshot_altitude_m,
                _native.d3(sun), _native.d3(E), _native.d3(disk), 0.266, _native.d9(view.basis),
                view.tangent_half_fov, 4.0, 12.0, ctypes.c_void_p(count.data_ptr()), stream)
            _native.check(rc)
            torch.cuda.synchronize()
            assert_parity(out.cpu().numpy(), ref.cpu().numpy(), f"noalloc call {call}")
            assert int(count.item()) == ref_samples, (call, int(count.item()), ref_samples)
        r.close()


def test_noalloc_rejects_frames_beyond_its_scratch():
    import torch

    from planet_renderer_gb300 import _native
    from planet_renderer_gb300.atmosphere.config import earth_baseline

    lib = _native.library()
    params = _native.AtmParams.from_config(earth_baseline())
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    p = ctypes.c_void_p(dummy.data_ptr())
    image = _native.AtmImage(8192, 4096, 4096, 1, 3)  # 131,072 tiles > 65,536
    rc = lib.atm_composite_noalloc(ctypes.byref(params), p, p, p, p, p, p, p, p, ctypes.byref(image), 6.36e6,
                                   6.361e6, 1000.0, _native.d3((0, 1, 0)), _native.d3((4, 4, 4)),
                                   _native.d3((1, 1, 1)), 0.266, _native.d9(((1, 0, 0), (0, 1, 0), (0, 0, 1))),
                                   0.5, 4.0, 12.0, None, None)
    assert rc == _native.ATM_E_INVALID
    assert b"65536 tiles" in lib.atm_last_error()
