"""The terrain raster (atm_raster_terrain through TerrainRaster) against the
reference's own kernels (the golden G-buffers of _clip,
_raster_depth_direct and _resolve_raster, tests/golden/raster.npz) and
against the float32 oracle (oracle/raster.py) on larger seeded meshes.

Bar: bit-exact.  The only allowed difference is the winner of an exact depth
tie: the emitted stream's order comes from an atomic counter here and from
the reference's own atomic counter there (the reference's _emit appends with
ti.atomic_add), so at a pixel where several triangles have the same depth
bits any of them may win.  Such pixels keep the same depth bits (checked
everywhere), and their winner must be one of the tied triangles the oracle
lists.  These meshes have many: their skirt slots repeat surface triangles
with the other winding (double-sided duplicates)."""

from __future__ import annotations

import json

import numpy as np
import pytest
import torch

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _mesh_tensors(view, normal, material, height, cell, triangles, active, skirt_mask, slot_level,
                  surface_triangles, resolution):
    d = "cuda"
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=d)
    return {"view": t(view, torch.float32), "normal": t(normal, torch.float32),
            "material": t(material, torch.float32), "height_m": t(height, torch.float32),
            "cell": t(cell, torch.int32), "triangles": t(triangles, torch.int32),
            "active_slots": t(np.asarray(active, np.int32), torch.int32),
            "skirt_mask": None if skirt_mask is None else t(skirt_mask, torch.int32),
            "slot_level": None if slot_level is None else t(slot_level, torch.int32),
            "surface_triangles": surface_triangles, "resolution": resolution}


def _render(mesh, width, height, near, tf, mode, layout="wh", channels=3):
    """One frame through TerrainRaster with the terrain snapshot written in
    the same pass; the snapshot must equal the G-buffer it copies."""

    from planet_renderer_gb300.raster import TerrainRaster

    r = TerrainRaster(width, height, mesh["view"].shape[0], mesh["triangles"].shape[0], layout=layout)
    g = r.allocate_gbuffer(channels, snapshot=True)
    r.render(mesh, near, tf, g, view_mode=mode)
    count = r.emitted()
    out = {k: v.cpu().numpy() for k, v in g.items()}
    if layout == "hw":
        out = {k: np.swapaxes(v, 0, 1) for k, v in out.items()}
    for k in ("position", "normal", "albedo", "terrain_position", "terrain_normal", "terrain_albedo"):
        out[k] = out[k][..., :3]
    np.testing.assert_array_equal(out["terrain_surface_id"], out["surface_id"])
    cov = out["surface_id"] >= 0
    for k in ("position", "normal", "albedo"):
        np.testing.assert_array_equal(out["terrain_" + k][cov], out[k][cov])
    r.close()
    return out, count


def _compare(got, ref, ties):
    """Bit equality of every G-buffer image at covered pixels; at pixels
    whose winner differs, the depth bits are equal and the winner is one of
    the oracle's tied triangles.  Returns the number of such pixels."""

    sid_ref, sid = ref["surface_id"], got["surface_id"]
    np.testing.assert_array_equal(sid >= 0, sid_ref >= 0, err_msg="coverage")
    np.testing.assert_array_equal(got["cell_id"][sid < 0], -1)
    cov = sid_ref >= 0
    np.testing.assert_array_equal(got["depth"][cov].view(np.uint32), ref["depth"][cov].view(np.uint32),
                                  err_msg="depth")
    same = cov & (sid == sid_ref)
    for name in ("depth", "position", "normal", "albedo", "material_weights", "height_m", "cell_id"):
        a, b = got[name][same], ref[name][same]
        if a.dtype == np.float32:
            a, b = a.view(np.uint32), b.view(np.uint32)
        np.testing.assert_array_equal(a, b, err_msg=name)
    xs, ys = np.nonzero(cov & ~same)
    for x, y in zip(xs, ys):
        assert int(sid[x, y]) in ties.get((int(x), int(y)), ()), (x, y, sid[x, y], sid_ref[x, y])
    return len(xs)


@pytest.mark.parametrize("case", [0, 1, 2, 3])
def test_raster_matches_the_reference_golden(case):
    data, _ = load_golden("raster")
    a = json.loads(str(data[f"case{case}_args"]))
    p = f"case{case}_"
    res = a["resolution"]
    mesh = _mesh_tensors(data[p + "view"], data[p + "normal"], data[p + "material"], data[p + "height"],
                         data[p + "cell"], data[p + "triangles"], a["active"], data[p + "skirt_mask"],
                         data[p + "slot_level"], 2 * res * res, res)
    got, count = _render(mesh, a["width"], a["height"], a["near"], a["tangent_half_fov"], a["mode"])
    assert count == int(data[p + "clipped_count"])
    ref = {k: data[p + k] for k in ("depth", "position", "albedo", "height_m", "surface_id", "cell_id",
                                    "material_weights")}
    ref["normal"] = data[p + "gb_normal"]
    assert (ref["surface_id"] >= 0).sum() > 0
    from oracle import raster

    ties = raster.render(data[p + "view"], data[p + "normal"], data[p + "material"], data[p + "height"],
                         data[p + "cell"], data[p + "triangles"], a["active"], a["near"], a["tangent_half_fov"],
                         a["width"], a["height"], a["mode"], data[p + "slot_level"], 2 * res * res, res,
                         data[p + "skirt_mask"])["ties"]
    _compare(got, ref, ties)


def _terrain(patches, res, seed, wind_odd=True):
    """Seeded heightfield patches in view space ahead of and below the camera
    (crossing the near plane and the side planes), with skirts."""

    rng = np.random.default_rng(seed)
    side = res + 1
    nv = side * side
    view = np.zeros((patches, nv, 3), np.float32)
    for p in range(patches):
        x0, z0 = rng.uniform(-90.0, -40.0), rng.uniform(-6.0, 4.0) + 14.0 * p
        span = rng.uniform(90.0, 140.0)
        i = np.arange(side)
        X, Z = np.broadcast_arrays(x0 + span * i[None, :] / res, z0 + span * i[:, None] / res)
        Y = -12.0 + 0.02 * Z + rng.normal(0.0, 0.6, (side, side))
        view[p] = np.stack([X, Y, Z], -1).reshape(nv, 3)
    normal = np.zeros_like(view)
    normal[..., 1] = 1.0
    normal += rng.normal(0.0, 0.2, normal.shape).astype(np.float32)
    material = rng.dirichlet(np.ones(4), (patches, nv)).astype(np.float32)
    height = rng.uniform(-1500.0, 4500.0, (patches, nv)).astype(np.float32)
    cell = rng.integers(0, 1 << 30, (patches, nv)).astype(np.int32)
    tris = []
    for j in range(res):
        for i in range(res):
            a, b, c, d = j * side + i, j * side + i + 1, (j + 1) * side + i, (j + 1) * side + i + 1
            tris += [(a, b, c), (b, d, c)]
    surface = len(tris)
    for k in range(8 * res):  # skirt slots: re-wound surface triangles (double-sided)
        a, b, c = tris[(k * 7) % surface]
        tris.append((a, c, b))
    if wind_odd:
        for p in range(1, patches, 2):
            view[p] = view[p].reshape(side, side, 3)[:, ::-1].reshape(nv, 3)
    skirt = rng.integers(0, 16, patches).astype(np.int32)
    level = rng.integers(0, 20, patches).astype(np.int32)
    return view, normal, material, height, cell, np.array(tris, np.int32), skirt, level, surface


@pytest.mark.parametrize("mode,layout,channels", [(0, "wh", 3), (1, "hw", 4), (2, "wh", 4), (3, "hw", 3)])
def test_raster_matches_the_oracle(mode, layout, channels):
    from oracle import raster

    W, H, patches, res = 240, 136, 24, 12
    view, normal, material, height, cell, tris, skirt, level, surface = _terrain(patches, res, 7 + mode)
    active = [s for s in range(patches) if s % 5 != 3][::-1]  # a subset, out of order
    near, tf = 0.5, 0.62
    ref = raster.render(view, normal, material, height, cell, tris, active, near, tf, W, H, mode, level, surface,
                        res, skirt)
    ref["material_weights"] = ref.pop("material")
    mesh = _mesh_tensors(view, normal, material, height, cell, tris, active, skirt, level, surface, res)
    got, count = _render(mesh, W, H, near, tf, mode, layout, channels)
    assert count == ref["clipped_count"]
    assert (ref["surface_id"] >= 0).mean() > 0.2
    _compare(got, ref, ref["ties"])


def test_raster_drops_slots_and_vertices_outside_the_mesh():
    """Active slots and vertex indices outside the mesh draw nothing (no
    out-of-bounds read): the frame equals the reference's with those slots
    left out and that triangle degenerate (culled)."""

    from oracle import raster

    W, H, patches, res = 64, 40, 4, 4
    view, normal, material, height, cell, tris, skirt, level, surface = _terrain(patches, res, 3, wind_odd=False)
    bad = tris.copy()
    bad[1] = (0, 1, 10_000)
    culled = tris.copy()
    culled[1] = (0, 0, 0)
    mesh = _mesh_tensors(view, normal, material, height, cell, bad, [0, 99, -1, 3], skirt, level, surface, res)
    got, count = _render(mesh, W, H, 0.5, 0.62, 0)
    ref = raster.render(view, normal, material, height, cell, culled, [0, 3], 0.5, 0.62, W, H, 0, level, surface,
                        res, skirt)
    ref["material_weights"] = ref.pop("material")
    assert count == ref["clipped_count"] > 0
    _compare(got, ref, ref["ties"])


def test_raster_rejects_bad_arguments():
    from planet_renderer_gb300.raster import TerrainRaster

    view, normal, material, height, cell, tris, skirt, level, surface = _terrain(2, 2, 1)
    mesh = _mesh_tensors(view, normal, material, height, cell, tris, [0, 1], skirt, None, surface, 2)
    r = TerrainRaster(32, 16, 2, len(tris))
    g = r.allocate_gbuffer()
    with pytest.raises(ValueError):
        r.render(mesh, 0.5, 0.6, g, view_mode=2)  # mode 2 without slot levels
    with pytest.raises(ValueError):
        r.render(mesh, -1.0, 0.6, g)
    with pytest.raises(ValueError):
        r.render(mesh, 0.5, 0.6, {k: v for k, v in g.items() if k != "albedo"})
    other = TerrainRaster(16, 16, 2, len(tris))
    with pytest.raises(ValueError):
        other.render(mesh, 0.5, 0.6, g)
    r.close()
    other.close()
