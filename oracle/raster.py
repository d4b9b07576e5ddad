"""CPU restatement of the reference's terrain raster, the G-buffer producer
that precedes the atmosphere stage.  TEST INFRASTRUCTURE ONLY: the checker
of the sm_103a raster kernels; nothing in the product imports it.

Follows src/planet_renderer/renderer.py in float32, operation for
operation (numpy float32 scalars, no fused multiply-add):

* ``_clip`` (:731-901): back-face culling of surface triangles, the
  clip-code trivial reject, and Sutherland-Hodgman clipping against the near
  plane and the four frustum sides with attribute interpolation;
* ``_emit`` (:628-686): projection to pixels snapped to 1/256, the signed
  area, edge equations and the top-left flags;
* ``_raster_depth_direct`` (:1158-1206): per covered pixel centre the
  perspective depth and the atomic minimum of the key (depth bits << 32 | q);
* ``_resolve_raster`` (:1208-1267) with ``_surface_color`` (:1008-1058) and
  ``_height_band`` (:976-1006): perspective-correct attributes of the winning
  triangle, the dominant vertex's cell id and the albedo of the view mode.

Triangles are emitted in source order here; the GPU emits them in the order
its atomic counter hands out slots, which changes the key's low bits and so
only the winner of an exact depth tie.
"""

from __future__ import annotations

import math

import numpy as np

F = np.float32
MAX_CLIP_VERTICES = 8
MAX_CLIPPED_TRIANGLES = 6
SENTINEL = (1 << 64) - 1


def _v(*a):
    return np.array(a, dtype=F)


def _dot(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def _cross(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], dtype=F)


def _normalized(v):
    invlen = F(1) / (np.sqrt(_dot(v, v)) + F(0))
    return (invlen * v).astype(F)


def _clip_code(p, near, tan_x, tan_y):
    code = 0
    if p[2] < near:
        code |= 1
    if p[0] < -p[2] * tan_x:
        code |= 2
    if p[0] > p[2] * tan_x:
        code |= 4
    if p[1] < -p[2] * tan_y:
        code |= 8
    if p[1] > p[2] * tan_y:
        code |= 16
    return code


def _clip_distance(p, plane, near, tan_x, tan_y):
    if plane == 0:
        return p[2] - near
    if plane == 1:
        return p[0] + p[2] * tan_x
    if plane == 2:
        return -p[0] + p[2] * tan_x
    if plane == 3:
        return p[1] + p[2] * tan_y
    return -p[1] + p[2] * tan_y


def _edge_coeff(a, b):
    return _v(a[1] - b[1], b[0] - a[0], (b[1] - a[1]) * a[0] - (b[0] - a[0]) * a[1])


def _top_left(a, b, orientation):
    dx = (b[0] - a[0]) * orientation
    dy = (b[1] - a[1]) * orientation
    return int((dy > 0.0) or (dy == 0.0 and dx < 0.0))


class Triangles:
    """The emitted triangle stream (the reference's rv, rn, rm, rh, rc,
    screen, source, edge_equation, inv_area, edge_top_left)."""

    def __init__(self):
        self.rows = []

    def emit(self, src, v, n, m, h, c, tf, width, height):
        aspect = F(width) / F(height)
        screen = np.zeros((3, 3), F)
        for k in range(3):
            p = v[k]
            px = (p[0] / (p[2] * tf * aspect) * F(0.5) + F(0.5)) * F(width)
            py = (p[1] / (p[2] * tf) * F(0.5) + F(0.5)) * F(height)
            px = np.floor(px * F(256.0) + F(0.5)) / F(256.0)
            py = np.floor(py * F(256.0) + F(0.5)) / F(256.0)
            screen[k] = (px, py, p[2])
        a, b, cc = screen[0, :2], screen[1, :2], screen[2, :2]
        area = (b[0] - a[0]) * (cc[1] - a[1]) - (b[1] - a[1]) * (cc[0] - a[0])
        abs_area = np.abs(area)
        sg = F(1.0) if area > 0.0 else F(-1.0)
        inv_area = F(1.0) / abs_area if abs_area > 1e-8 else F(0.0)
        eq = np.stack([_edge_coeff(b, cc) * sg, _edge_coeff(cc, a) * sg, _edge_coeff(a, b) * sg]).astype(F)
        tl = (_top_left(b, cc, sg), _top_left(cc, a, sg), _top_left(a, b, sg))
        self.rows.append(dict(v=np.array(v, F), n=np.array(n, F), m=np.array(m, F), h=np.array(h, F),
                              c=np.array(c, np.int64), screen=screen, src=int(src), eq=eq, inv_area=F(inv_area),
                              tl=tl))


def clip(view, normal, material, height, cell, triangles, active, near, tf, width, height_px, capacity,
         surface_triangles=None, resolution=1, skirt_mask=None):
    """_clip over the active slots' triangles; returns the emitted stream.
    Triangles from ``surface_triangles`` on are skirts: four edges of
    2 * ``resolution`` triangles, edge e enabled by bit e of the slot's
    ``skirt_mask``, never culled as back faces."""

    out = Triangles()
    stc = len(triangles) if surface_triangles is None else int(surface_triangles)
    near, tf = F(near), F(tf)
    aspect = F(width) / F(height_px)
    tan_x, tan_y = tf * aspect, tf
    ltc = len(triangles)
    for active_source in range(len(active) * ltc):
        slot = int(active[active_source // ltc])
        local_id = active_source % ltc
        source_id = slot * ltc + local_id
        skirt_edge = (local_id - stc) // (resolution * 2)
        if not (local_id < stc or (skirt_edge >= 0 and skirt_mask is not None
                                   and int(skirt_mask[slot]) & (1 << skirt_edge))):
            continue
        ids = triangles[local_id]
        p0, p1, p2 = (view[slot, i].astype(F) for i in ids)
        if local_id < stc and not (_dot(_cross(p1 - p0, p2 - p0), -p0) < 0.0):
            continue  # a back-facing surface triangle (skirts are double-sided)
        c0, c1, c2 = (_clip_code(p, near, tan_x, tan_y) for p in (p0, p1, p2))
        if c0 & c1 & c2:
            continue
        nn = [normal[slot, i].astype(F) for i in ids]
        mm = [material[slot, i].astype(F) for i in ids]
        hh = [F(height[slot, i]) for i in ids]
        ce = [int(cell[slot, i]) for i in ids]

        def emit(v, n, m, h, c):
            if len(out.rows) < capacity:
                out.emit(source_id, v, n, m, h, c, tf, width, height_px)
            else:
                out.rows.append(None)  # counted, not stored (the reference's s >= capacity)

        if (c0 | c1 | c2) == 0:
            emit([p0, p1, p2], nn, mm, hh, ce)
            continue
        pos = [[None] * MAX_CLIP_VERTICES for _ in range(2)]
        nrm = [[None] * MAX_CLIP_VERTICES for _ in range(2)]
        mat = [[None] * MAX_CLIP_VERTICES for _ in range(2)]
        hgt = [[None] * MAX_CLIP_VERTICES for _ in range(2)]
        cel = [[None] * MAX_CLIP_VERTICES for _ in range(2)]
        for k in range(3):
            pos[0][k], nrm[0][k], mat[0][k], hgt[0][k], cel[0][k] = [p0, p1, p2][k], nn[k], mm[k], hh[k], ce[k]
        count, read = 3, 0
        for plane in range(5):
            write = 1 - read
            oc = 0
            for vertex in range(count):
                prev = (vertex + count - 1) % count
                cp, pp = pos[read][vertex], pos[read][prev]
                cd = _clip_distance(cp, plane, near, tan_x, tan_y)
                pd = _clip_distance(pp, plane, near, tan_x, tan_y)
                ci, pi = cd >= 0.0, pd >= 0.0
                if ci != pi and oc < MAX_CLIP_VERTICES:
                    den = pd - cd
                    t = pd / den if np.abs(den) > 1e-20 else F(0.0)
                    pos[write][oc] = (pp + (cp - pp) * t).astype(F)
                    nrm[write][oc] = _normalized((nrm[read][prev] + (nrm[read][vertex] - nrm[read][prev]) * t)
                                                 .astype(F))
                    mat[write][oc] = (mat[read][prev] + (mat[read][vertex] - mat[read][prev]) * t).astype(F)
                    hgt[write][oc] = F(hgt[read][prev] + (hgt[read][vertex] - hgt[read][prev]) * t)
                    cel[write][oc] = cel[read][vertex] if ci else cel[read][prev]
                    oc += 1
                if ci and oc < MAX_CLIP_VERTICES:
                    pos[write][oc], nrm[write][oc] = cp, nrm[read][vertex]
                    mat[write][oc], hgt[write][oc], cel[write][oc] = mat[read][vertex], hgt[read][vertex], \
                        cel[read][vertex]
                    oc += 1
            count, read = oc, write
        for tri in range(min(max(count - 2, 0), MAX_CLIPPED_TRIANGLES)):
            idx = (0, tri + 1, tri + 2)
            emit([pos[read][i] for i in idx], [nrm[read][i] for i in idx], [mat[read][i] for i in idx],
                 [hgt[read][i] for i in idx], [cel[read][i] for i in idx])
    return out


FERTILE, ARID, ROCK = _v(0.10, 0.34, 0.075), _v(0.44, 0.31, 0.13), _v(0.34, 0.32, 0.30)
SNOW, SAND = _v(0.92, 0.95, 0.98), _v(0.72, 0.60, 0.34)
DEEP_OCEAN, SHALLOW_OCEAN = _v(0.012, 0.055, 0.16), _v(0.015, 0.34, 0.46)
BAND = {"deep_water": _v(0.015, 0.12, 0.34), "shallow_water": _v(0.02, 0.63, 0.82), "beach": _v(0.82, 0.78, 0.48),
        "lowland": _v(0.16, 0.58, 0.22), "upland": _v(0.48, 0.42, 0.16), "rock": _v(0.43, 0.39, 0.35),
        "snow": _v(0.94, 0.96, 0.98)}


def _mix(a, b, t):
    return (a * (F(1.0) - t) + b * t).astype(F)


def _clamp01(x):
    return F(min(max(x, F(0.0)), F(1.0)))


def height_band(h):
    B = BAND
    if h < -250.0:
        return _mix(B["deep_water"], B["shallow_water"], _clamp01((h + F(5000.0)) / F(4750.0)))
    if h < 0.0:
        return B["shallow_water"].copy()
    if h < 120.0:
        return _mix(B["beach"], B["lowland"], _clamp01(h / F(120.0)))
    if h < 1400.0:
        return _mix(B["lowland"], B["upland"], _clamp01((h - F(120.0)) / F(1280.0)))
    if h < 3000.0:
        return _mix(B["upland"], B["rock"], _clamp01((h - F(1400.0)) / F(1600.0)))
    return _mix(B["rock"], B["snow"], _clamp01((h - F(3000.0)) / F(1400.0)))


def surface_color(h, m, slot, mode, slot_level):
    color = (((FERTILE * m[0] + ARID * m[1]) + ROCK * m[2]) + SNOW * m[3]).astype(F)
    if h < 0.0:
        color = _mix(SHALLOW_OCEAN, DEEP_OCEAN, _clamp01(-h / F(4200.0)))
    elif h < 140.0:
        color = _mix(SAND, color, _clamp01(h / F(140.0)))
    if mode == 1:
        color = height_band(h)
    elif mode == 2:
        hue = F(int(slot_level[slot]) % 6) / F(6.0)
        color = np.minimum(np.maximum(_v(np.abs(hue * F(6.0) - F(3.0)) - F(1.0), F(2.0) - np.abs(hue * F(6.0) - F(2.0)),
                                         F(2.0) - np.abs(hue * F(6.0) - F(4.0))), F(0.0)), F(1.0)).astype(F)
    elif mode == 3:
        value = F((slot * 1103515245 + 12345) & 255) / F(255.0)
        fr = lambda x: F(x - np.floor(x))
        color = _v(value, fr(value * F(0.73) + F(0.21)), fr(value * F(0.37) + F(0.61)))
    return color


def raster(tris: Triangles, width, height, local_triangle_count, mode=0, slot_level=None):
    """_raster_depth_direct then _resolve_raster; returns the G-buffer."""

    key = np.full((width, height), SENTINEL, dtype=object)
    # every triangle covering a pixel, by depth bits: the exact-depth ties,
    # where the winner is the atomic order's (the lowest stream index here)
    cover = {}
    for q, t in enumerate(tris.rows):
        if t is None or not t["inv_area"] > 0.0:
            continue
        a, b, c = t["screen"]
        x0 = max(int(np.floor(min(a[0], b[0], c[0]))), 0)
        x1 = min(int(np.ceil(max(a[0], b[0], c[0]))), width - 1)
        y0 = max(int(np.floor(min(a[1], b[1], c[1]))), 0)
        y1 = min(int(np.ceil(max(a[1], b[1], c[1]))), height - 1)
        for x in range(x0, x1 + 1):
            for y in range(y0, y1 + 1):
                e = _edges(t, x, y)
                if not _inside(t, e):
                    continue
                l = e * t["inv_area"]
                z = F(1.0) / max(l[0] / a[2] + l[1] / b[2] + l[2] / c[2], F(1e-20))
                k = (int(np.array(z, F).view(np.uint32)) << 32) | q
                key[x, y] = min(key[x, y], k)
                cover.setdefault((x, y), []).append(k)
    g = {"depth": np.zeros((width, height), F), "position": np.zeros((width, height, 3), F),
         "normal": np.zeros((width, height, 3), F), "albedo": np.zeros((width, height, 3), F),
         "material": np.zeros((width, height, 4), F), "height_m": np.zeros((width, height), F),
         "surface_id": np.full((width, height), -1, np.int32), "cell_id": np.full((width, height), -1, np.int32),
         "ties": {}}
    for x in range(width):
        for y in range(height):
            k = key[x, y]
            if k == SENTINEL:
                continue
            q = k & 0xFFFFFFFF
            z = np.array(k >> 32, np.uint32).view(F)[()]
            tied = [c & 0xFFFFFFFF for c in cover[(x, y)] if c >> 32 == k >> 32]
            if len(tied) > 1:
                g["ties"][(x, y)] = sorted({int(tris.rows[c]["src"]) for c in tied})
            t = tris.rows[q]
            a, b, c = t["screen"]
            l = _edges(t, x, y) * t["inv_area"]
            w = _v(l[0] * z / a[2], l[1] * z / b[2], l[2] * z / c[2])
            lerp = lambda v: ((v[0] * w[0] + v[1] * w[1]) + v[2] * w[2]).astype(F)
            bh = F((t["h"][0] * w[0] + t["h"][1] * w[1]) + t["h"][2] * w[2])
            vi = 0
            if w[1] > w[0]:
                vi = 1
            if w[2] > w[vi]:
                vi = 2
            src = t["src"]
            g["depth"][x, y] = z
            g["surface_id"][x, y] = src
            g["cell_id"][x, y] = int(t["c"][vi])
            g["position"][x, y] = lerp(t["v"])
            g["normal"][x, y] = _normalized(lerp(t["n"]))
            g["material"][x, y] = lerp(t["m"])
            g["height_m"][x, y] = bh
            g["albedo"][x, y] = surface_color(bh, lerp(t["m"]), src // local_triangle_count, mode, slot_level)
    return g


def _edges(t, x, y):
    px, py = F(x) + F(0.5), F(y) + F(0.5)
    e = t["eq"]
    return _v((e[0, 0] * px + e[0, 1] * py) + e[0, 2], (e[1, 0] * px + e[1, 1] * py) + e[1, 2],
              (e[2, 0] * px + e[2, 1] * py) + e[2, 2])


def _inside(t, e):
    tl = t["tl"]
    return ((e[0] > 0.0 or (e[0] == 0.0 and tl[0] != 0)) and (e[1] > 0.0 or (e[1] == 0.0 and tl[1] != 0))
            and (e[2] > 0.0 or (e[2] == 0.0 and tl[2] != 0)))


def render(view, normal, material, height, cell, triangles, active, near, tf, width, height_px, mode=0,
           slot_level=None, surface_triangles=None, resolution=1, skirt_mask=None):
    """The whole terrain raster of one frame: clip/emit, depth keys, resolve."""

    capacity = view.shape[0] * len(triangles) * MAX_CLIPPED_TRIANGLES
    tris = clip(view, normal, material, height, cell, triangles, active, near, tf, width, height_px, capacity,
                surface_triangles, resolution, skirt_mask)
    g = raster(tris, width, height_px, len(triangles), mode, slot_level)
    g["clipped_count"] = len(tris.rows)
    return g
