"""The terrain raster that produces the atmosphere stage's G-buffer: the
reference's ``PlanetRenderer`` triangle path (``src/planet_renderer/renderer.py
:628-1269``) over ``atm_raster_terrain``.

One frame is ``_clip`` (back-face culling of surface triangles, skirts drawn
from both sides, trivial reject, Sutherland-Hodgman against the near plane
and the four frustum sides, fan triangulation into the emitted stream),
``_raster_depth_direct`` (each covered pixel centre takes the atomic 64-bit
minimum of ``depth bits << 32 | triangle``) and ``_resolve_raster`` (the
nearest triangle's perspective-correct view position, normal, material
weights and height, the dominant vertex's cell id and the albedo of the
debug view).  The reference's tiled pixel path (``_bin`` / ``_raster_pixel``)
chooses the same nearest triangle per pixel; this class runs the
triangle-driven path for every frame.

Images are torch CUDA tensors ``(W, H, ...)`` - the layout of the reference's
Taichi fields - or ``(H, W, ...)`` with ``layout="hw"``; work is enqueued on
the current CUDA stream.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _native

MAX_CLIPPED_TRIANGLES = 6  # renderer.py:37
# G-buffer images the raster writes, with (dtype, floats per element; 0 = one scalar)
OUTPUTS = {"depth": (torch.float32, 0), "position": (torch.float32, -1), "normal": (torch.float32, -1),
           "albedo": (torch.float32, -1), "material_weights": (torch.float32, 4), "height_m": (torch.float32, 0),
           "surface_id": (torch.int32, 0), "cell_id": (torch.int32, 0)}
# the opaque terrain snapshot the ocean shading reads (written when all four are given)
SNAPSHOT = {"terrain_position": (torch.float32, -1), "terrain_normal": (torch.float32, -1),
            "terrain_albedo": (torch.float32, -1), "terrain_surface_id": (torch.int32, 0)}
# the rest of a frame's G-buffer, written by the ocean coverage pass
OCEAN_EXTRA = {"water_depth": (torch.float32, 0), "seabed_albedo": (torch.float32, -1),
               "seabed_normal": (torch.float32, -1), "slope_variance": (torch.float32, 0)}


def shared_topology(resolution: int) -> np.ndarray:
    """The patch topology the raster draws (``_shared_topology``,
    renderer.py:78-100): two triangles per grid cell of the (resolution + 1)^2
    surface vertices, then per edge (bottom, right, top, left, walked so the
    skirt faces outwards) two triangles per segment joining the edge's surface
    vertices to that edge's row of skirt vertices, which follow the surface
    vertices in the patch's vertex stream."""

    n = int(resolution)
    side = n + 1
    cells = np.arange(n)
    a = (cells[:, None] * side + cells[None, :]).ravel()  # row-major cells: a = y * side + x
    surface = np.stack([np.stack([a, a + 1, a + side], 1), np.stack([a + 1, a + side + 1, a + side], 1)],
                       1).reshape(-1, 3)
    i = np.arange(side)
    edges = (i, i * side + n, (n * side + i)[::-1], (i * side)[::-1])
    skirts = []
    for k, edge in enumerate(edges):
        base = side * side + k * side
        s0, s1 = edge[:-1], edge[1:]
        c0, c1 = base + cells, base + cells + 1
        skirts.append(np.stack([np.stack([s0, c0, s1], 1), np.stack([s1, c0, c1], 1)], 1).reshape(-1, 3))
    return np.concatenate([surface] + skirts).astype(np.int32)


def synthetic_terrain(width: int, height: int, tangent_half_fov: float, altitude_m: float = 2000.0,
                      pitch_degrees: float = 8.0, rows: int = 16, columns: int = 16, resolution: int = 12,
                      far_m: float = 80_000.0, planet_radius_m: float = 6_371_000.0, seed: int = 0,
                      relief_m: float = 380.0, base_height_m: float = 150.0, rise_m_per_km: float = 0.0,
                      device: str | torch.device = "cuda") -> dict:
    """A seeded terrain frame in camera view space for ``render``: rows x
    columns patches of ``resolution`` cells a side tiling the ground in the
    view frustum from the camera's foot to ``far_m`` (rows growing
    geometrically with distance, as a distance-based LOD does), heights from
    a few octaves of sinusoids (largest amplitude ``relief_m``, mean
    ``base_height_m``, rising ``rise_m_per_km`` with distance) over the
    planet's curvature drop, outward
    skirts below every edge, material weights by height and slope.  Vertex
    positions are in view space (x right, y up, z forward; the camera looks
    ``pitch_degrees`` down), normals in the camera's local East-Up-North frame
    (the global frame when the planet frame is the identity), as the
    reference's patch streams hold them.  Stands in for the terrain backend's
    patch stream (the LOD system is not part of this library)."""

    rng = np.random.default_rng(seed)
    n, side = int(resolution), int(resolution) + 1
    near_z = max(altitude_m / math.tan(math.radians(pitch_degrees) + math.atan(tangent_half_fov)), 1.0)
    growth = (far_m / near_z) ** (1.0 / rows)
    tx = tangent_half_fov * width / height
    t = np.linspace(0.0, 1.0, side)
    phases = rng.uniform(0.0, 2.0 * math.pi, (6, 2))
    waves = [(1.0 / (900.0 * 2.2 ** -k), relief_m * 0.5 ** k) for k in range(6)]

    def ground(x, z):
        h = np.zeros_like(x)
        dhx, dhz = np.zeros_like(x), np.zeros_like(x)
        for k, (f, amp) in enumerate(waves):
            u, v = f * x + phases[k, 0], f * z * 0.83 + phases[k, 1]
            h += amp * np.sin(u) * np.cos(v)
            dhx += amp * f * np.cos(u) * np.cos(v)
            dhz -= amp * f * 0.83 * np.sin(u) * np.sin(v)
        return h + base_height_m + rise_m_per_km * 1e-3 * z, dhx, dhz + rise_m_per_km * 1e-3

    view, normal, material, hgt, cell = [], [], [], [], []
    pitch = math.radians(pitch_degrees)
    up = np.array([0.0, math.cos(pitch), math.sin(pitch)])
    fwd = np.array([0.0, -math.sin(pitch), math.cos(pitch)])
    for r in range(rows):
        z0, z1 = near_z * growth ** r * (0.0 if r == 0 else 1.0), near_z * growth ** (r + 1)
        half = 1.15 * tx * z1 + 200.0
        for c in range(columns):
            x0, x1 = -half + 2.0 * half * c / columns, -half + 2.0 * half * (c + 1) / columns
            X, Z = np.meshgrid(x0 + (x1 - x0) * t, z0 + (z1 - z0) * t)
            h, dhx, dhz = ground(X, Z)
            drop = (X * X + Z * Z) / (2.0 * planet_radius_m)
            Y = h - altitude_m - drop
            nrm = np.stack([-dhx, np.ones_like(X), -dhz], -1)
            nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
            pts = np.stack([X, Y, Z], -1).reshape(-1, 3)
            nr = nrm.reshape(-1, 3)
            hh = h.reshape(-1)
            skirt_depth = 0.02 * (z1 - z0) + 5.0
            ring = np.concatenate([np.arange(side), np.arange(side) * side + n, n * side + np.arange(side),
                                   np.arange(side) * side])
            pts = np.concatenate([pts, pts[ring] - [0.0, skirt_depth, 0.0]])
            nr = np.concatenate([nr, nr[ring]])
            hh = np.concatenate([hh, hh[ring] - skirt_depth])
            slope = 1.0 - nr[:, 1]
            snow = np.clip((hh - 450.0) / 150.0, 0.0, 1.0)
            rock = np.clip(slope * 6.0, 0.0, 1.0) * (1.0 - snow)
            arid = np.clip(hh / 600.0, 0.0, 1.0) * (1.0 - rock - snow)
            fertile = np.clip(1.0 - arid - rock - snow, 0.0, 1.0)
            view.append(np.stack([pts[:, 0], pts @ up, pts @ fwd], -1))
            normal.append(nr)
            material.append(np.stack([fertile, arid, rock, snow], -1))
            hgt.append(hh)
            cell.append((r * columns + c) * 4096 + np.arange(len(hh)))
    patches = rows * columns
    f32 = lambda a: torch.as_tensor(np.asarray(a, np.float32), device=device)
    i32 = lambda a: torch.as_tensor(np.asarray(a, np.int32), device=device)
    return {"view": f32(view), "normal": f32(normal), "material": f32(material), "height_m": f32(hgt),
            "cell": i32(cell), "triangles": i32(shared_topology(n)), "active_slots": i32(np.arange(patches)),
            "skirt_mask": i32(np.full(patches, 15)), "slot_level": i32(rows - 1 - np.arange(patches) // columns),
            "surface_triangles": 2 * n * n, "resolution": n,
            "view_basis": (np.array([1.0, 0.0, 0.0]), up, fwd)}


def _element_strides(t: torch.Tensor, per_element: int, layout: str) -> tuple:
    sx, sy = (t.stride(0), t.stride(1)) if layout == "wh" else (t.stride(1), t.stride(0))
    if sx % per_element or sy % per_element:
        raise ValueError("image strides must be whole elements")
    return sx // per_element, sy // per_element


class TerrainRaster:
    """The raster buffers of one frame size (``renderer.py:200-236``): the
    emitted-triangle stream of ``max_patches * triangles_per_patch * 6``
    triangles and the per-pixel depth keys."""

    def __init__(self, width: int, height: int, max_patches: int, triangles_per_patch: int,
                 layout: str = "wh", device: str | torch.device = "cuda"):
        if layout not in ("wh", "hw"):
            raise ValueError("layout must be 'wh' (Taichi field layout) or 'hw'")
        self.width, self.height = int(width), int(height)
        self.max_patches, self.triangles_per_patch = int(max_patches), int(triangles_per_patch)
        self.layout = layout
        self.device = torch.device(device)
        if self.device.type == "cuda" and self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self._lib = _native.library()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.check(self._lib.atm_raster_create(self.width, self.height, self.max_patches,
                                                      self.triangles_per_patch, ctypes.byref(h)))
        self._handle = h

    @property
    def capacity(self) -> int:
        return self.max_patches * self.triangles_per_patch * MAX_CLIPPED_TRIANGLES

    def allocate_gbuffer(self, channels: int = 3, snapshot: bool = False, ocean: bool = False) -> dict:
        """Empty G-buffer images of this raster's size and layout; with
        ``snapshot`` also the terrain snapshot, with ``ocean`` also the
        images the ocean pass adds (a whole frame's G-buffer)."""

        dims = (self.width, self.height) if self.layout == "wh" else (self.height, self.width)
        out = {}
        images = dict(OUTPUTS, **(SNAPSHOT if snapshot else {}), **(OCEAN_EXTRA if ocean else {}))
        for name, (dtype, per) in images.items():
            per = channels if per < 0 else per
            shape = dims + ((per,) if per else ())
            out[name] = torch.zeros(shape, dtype=dtype, device=self.device)
        for name in ("surface_id", "cell_id", "terrain_surface_id"):
            if name in out:
                out[name].fill_(-1)
        return out

    def _image(self, gbuffer: dict) -> _native.AtmImage:
        missing = [n for n in OUTPUTS if n not in gbuffer]
        if missing:
            raise ValueError(f"missing G-buffer images: {missing}")
        ref = gbuffer["position"]
        if not isinstance(ref, torch.Tensor) or ref.dim() != 3 or ref.shape[2] not in (3, 4) or ref.stride(2) != 1:
            raise ValueError("position must be a float32 CUDA tensor (W, H, 3|4) with contiguous channels")
        channels = int(ref.shape[2])
        dims = (int(ref.shape[0]), int(ref.shape[1])) if self.layout == "wh" else (int(ref.shape[1]),
                                                                                  int(ref.shape[0]))
        if dims != (self.width, self.height):
            raise ValueError(f"G-buffer is {dims[0]}x{dims[1]}, the raster {self.width}x{self.height}")
        strides = _element_strides(ref, channels, self.layout)
        snapshot = [n for n in SNAPSHOT if n in gbuffer]
        if snapshot and len(snapshot) != len(SNAPSHOT):
            raise ValueError(f"the terrain snapshot needs all of {list(SNAPSHOT)}")
        for name, (dtype, per) in dict(OUTPUTS, **{n: SNAPSHOT[n] for n in snapshot}).items():
            t = gbuffer[name]
            per = channels if per < 0 else per
            if not isinstance(t, torch.Tensor) or t.dtype != dtype or t.device != self.device:
                raise ValueError(f"{name} must be a {dtype} tensor on {self.device}")
            shape = tuple(t.shape[:2]) if self.layout == "wh" else (int(t.shape[1]), int(t.shape[0]))
            if shape != dims or t.dim() != (3 if per else 2) or (per and (t.shape[2] != per or t.stride(2) != 1)):
                raise ValueError(f"{name} must have the frame's shape with {per or 1} values per pixel")
            if _element_strides(t, per or 1, self.layout) != strides:
                raise ValueError(f"{name} must share the G-buffer's element strides")
        return _native.AtmImage(self.width, self.height, strides[0], strides[1], channels)

    def render(self, mesh: dict, near: float, tangent_half_fov: float, gbuffer: dict, view_mode: int = 0) -> None:
        """One frame's _clip + _raster_depth_direct + _resolve_raster into
        ``gbuffer`` (images named as ``OUTPUTS``).  ``mesh`` holds CUDA
        tensors: ``view``, ``normal`` (patches, vertices, 3), ``material``
        (patches, vertices, 4), ``height_m`` (patches, vertices) float32,
        ``cell`` (patches, vertices), ``triangles`` (triangles, 3) and
        ``active_slots`` int32, optional ``skirt_mask`` and ``slot_level``
        (patches,) int32, and the ints ``surface_triangles`` and
        ``resolution``.  ``view_mode``: 0 lit albedo, 1 height bands, 2 LOD
        level, 3 patch hash.  When ``gbuffer`` also holds the ``SNAPSHOT``
        images the same pass writes the terrain snapshot
        (_snapshot_terrain_gbuffer) into them."""

        image = self._image(gbuffer)
        view = mesh["view"]
        patches, vertices = int(view.shape[0]), int(view.shape[1])
        tri = mesh["triangles"]

        def arr(name, dtype, shape, optional=False):
            t = mesh.get(name)
            if t is None:
                if optional:
                    return None
                raise ValueError(f"mesh needs {name}")
            if not isinstance(t, torch.Tensor) or t.dtype != dtype or t.device != self.device:
                raise ValueError(f"mesh {name} must be a {dtype} tensor on {self.device}")
            if tuple(t.shape) != shape or not t.is_contiguous():
                raise ValueError(f"mesh {name} must be a contiguous {shape} tensor")
            return t

        f32, i32 = torch.float32, torch.int32
        active = mesh["active_slots"]
        n_active = int(active.numel())
        tensors = {
            "view": arr("view", f32, (patches, vertices, 3)),
            "normal": arr("normal", f32, (patches, vertices, 3)),
            "material": arr("material", f32, (patches, vertices, 4)),
            "height_m": arr("height_m", f32, (patches, vertices)),
            "cell": arr("cell", i32, (patches, vertices)),
            "triangles": arr("triangles", i32, (int(tri.shape[0]), 3)),
            "active_slots": arr("active_slots", i32, (n_active,)),
            "skirt_mask": arr("skirt_mask", i32, (patches,), optional=True),
            "slot_level": arr("slot_level", i32, (patches,), optional=True),
        }
        m = _native.AtmRasterMesh()
        for name, t in tensors.items():
            setattr(m, name, None if t is None else t.data_ptr())
        m.patches, m.vertices_per_patch, m.triangles_per_patch = patches, vertices, int(tri.shape[0])
        m.surface_triangles_per_patch = int(mesh.get("surface_triangles", tri.shape[0]))
        m.resolution = int(mesh.get("resolution", 1))
        m.n_active = n_active
        outs = _native.AtmRasterOutputs(*[ctypes.c_void_p(gbuffer[n].data_ptr() if n in gbuffer else None)
                                          for n in _native.RASTER_OUTPUTS])
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _native.check(self._lib.atm_raster_terrain(self._handle, ctypes.byref(m), float(near), float(tangent_half_fov),
                                                   int(view_mode), ctypes.byref(outs), ctypes.byref(image),
                                                   ctypes.c_void_p(stream)))

    def emitted(self) -> int:
        """Triangles the last frame emitted (``clipped_count``; synchronises
        the current stream).  Above ``capacity`` means some were dropped."""

        n = ctypes.c_int64()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _native.check(self._lib.atm_raster_emitted(self._handle, ctypes.byref(n), ctypes.c_void_p(stream)))
        return int(n.value)

    def close(self) -> None:
        if self._handle:
            self._lib.atm_raster_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
