"""Seeded patch sets for the multi-right-hand-side radiosity gather.

`room(seed, n_patches, n_configs)` builds a furnished room (shell, tables,
chairs, cabinets, a sofa and a bed) out of axis-aligned or yawed boxes, cuts
every visible face into near-square quads, and returns:

    tri       T x 9   occluder triangles (two per quad, every quad)
    pos, nrm  n x 3   patch centres and outward unit normals
    area      n       patch areas
    albedo    n x 3   per-surface albedo, uniform(0.3, 0.8) per channel
    emission  n x 3C  C light configurations (RGB each): 1-3 lamps chosen
                      from ceiling panels and wall windows, seeded colours

With n_patches = 32768 the mesh has about 65k triangles. When more quads than
n_patches exist, a seeded subset (kept in surface order) becomes the patch
set; all quads stay occluders.
"""
from __future__ import annotations

import math

import numpy as np


def _box_rects(cx, cy, z0, sx, sy, sz, yaw, bottom):
    """Faces of a box as (corner, u, v) with cross(u, v) pointing outwards."""
    c, s = math.cos(yaw), math.sin(yaw)
    ex = np.array([c, s, 0.0]) * sx
    ey = np.array([-s, c, 0.0]) * sy
    ez = np.array([0.0, 0.0, sz])
    o = np.array([cx, cy, z0]) - 0.5 * ex - 0.5 * ey
    rects = [
        (o + ez, ex, ey),              # top (+z)
        (o, ey, ex),                   # bottom (-z)
        (o, ez, ey),                   # -x side: cross(ez, ey) = -ex
        (o + ex, ey, ez),              # +x side
        (o, ex, ez),                   # -y side: cross(ex, ez) = -ey
        (o + ey, ez, ex),              # +y side
    ]
    if not bottom:
        rects.pop(1)
    return rects


def _room_rects(W, D, H):
    """Inward-facing shell of a W x D x H room."""
    X, Y, Z = np.array([W, 0, 0.0]), np.array([0, D, 0.0]), np.array([0, 0, H * 1.0])
    O = np.zeros(3)
    return [
        (O, X, Y),              # floor, normal +z
        (O + Z, Y, X),          # ceiling, normal -z
        (O, Y, Z),              # x = 0 wall, normal +x
        (O + X, Z, Y),          # x = W wall, normal -x
        (O, Z, X),              # y = 0 wall, normal +y
        (O + Y, X, Z),          # y = D wall, normal -y
    ]


def _furniture(rng, W, D):
    out = []   # (cx, cy, z0, sx, sy, sz, yaw, bottom)

    def spot(margin):
        return rng.uniform(margin, W - margin), rng.uniform(margin, D - margin)

    for _ in range(3):   # tables: top + 4 legs
        cx, cy = spot(1.2)
        yaw = rng.uniform(0, math.pi)
        tw, td = rng.uniform(1.2, 1.8), rng.uniform(0.7, 1.0)
        out.append((cx, cy, 0.72, tw, td, 0.05, yaw, True))
        c, s = math.cos(yaw), math.sin(yaw)
        for fx in (-0.45, 0.45):
            for fy in (-0.4, 0.4):
                lx, ly = fx * tw, fy * td
                out.append((cx + c * lx - s * ly, cy + s * lx + c * ly, 0.0, 0.06, 0.06, 0.72, yaw, False))
    for _ in range(6):   # chairs: seat, back, legs
        cx, cy = spot(0.6)
        yaw = rng.uniform(0, 2 * math.pi)
        c, s = math.cos(yaw), math.sin(yaw)
        out.append((cx, cy, 0.45, 0.45, 0.45, 0.05, yaw, True))
        out.append((cx - s * 0.2, cy + c * 0.2, 0.5, 0.45, 0.05, 0.5, yaw, True))
        for fx in (-0.18, 0.18):
            for fy in (-0.18, 0.18):
                out.append((cx + c * fx - s * fy, cy + s * fx + c * fy, 0.0, 0.04, 0.04, 0.45, yaw, False))
    for k in range(3):   # cabinets / shelves against the walls
        w = rng.uniform(0.8, 1.6)
        if k % 2 == 0:
            out.append((rng.uniform(1, W - 1), 0.25, 0.0, w, 0.4, rng.uniform(1.0, 2.2), 0.0, False))
        else:
            out.append((W - 0.25, rng.uniform(1, D - 1), 0.0, 0.4, w, rng.uniform(1.0, 2.2), 0.0, False))
    cx, cy = spot(1.5)   # sofa: base + back
    yaw = rng.uniform(0, 2 * math.pi)
    c, s = math.cos(yaw), math.sin(yaw)
    out.append((cx, cy, 0.0, 2.0, 0.9, 0.45, yaw, False))
    out.append((cx - s * 0.35, cy + c * 0.35, 0.45, 2.0, 0.2, 0.4, yaw, True))
    cx, cy = spot(1.4)   # bed
    out.append((cx, cy, 0.0, 2.0, 1.6, 0.5, rng.uniform(0, math.pi), False))
    return out


def _tessellate(rects, step):
    """Quads of each rectangle: centres, normals, areas, corner quads, surface index."""
    cen, nrm, area, quads, sid = [], [], [], [], []
    for k, (o, u, v) in enumerate(rects):
        lu, lv = np.linalg.norm(u), np.linalg.norm(v)
        nu, nv = max(1, int(round(lu / step))), max(1, int(round(lv / step)))
        du, dv = u / nu, v / nv
        n = np.cross(u, v)
        n = n / np.linalg.norm(n)
        a, b = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
        a, b = a.ravel()[:, None], b.ravel()[:, None]
        p00 = o + a * du + b * dv
        quads.append(np.stack([p00, p00 + du, p00 + du + dv, p00 + dv], axis=1))
        cen.append(p00 + 0.5 * du + 0.5 * dv)
        nrm.append(np.repeat(n[None], len(p00), 0))
        area.append(np.full(len(p00), np.linalg.norm(np.cross(du, dv))))
        sid.append(np.full(len(p00), k))
    return (np.concatenate(cen), np.concatenate(nrm), np.concatenate(area), np.concatenate(quads),
            np.concatenate(sid))


def room(seed: int = 1, n_patches: int = 32768, n_configs: int = 64, size=(10.0, 8.0, 3.5)) -> dict:
    rng = np.random.default_rng(seed)
    W, D, H = size
    rects = _room_rects(W, D, H)
    for f in _furniture(rng, W, D):
        rects += _box_rects(*f)
    albedo_s = rng.uniform(0.3, 0.8, (len(rects), 3))
    total = sum(np.linalg.norm(np.cross(u, v)) for _, u, v in rects)
    step = math.sqrt(total / n_patches)
    while True:
        cen, nrm, area, quads, sid = _tessellate(rects, step)
        if len(cen) >= n_patches:
            break
        step *= 0.97
    tri = np.concatenate([quads[:, [0, 1, 2]], quads[:, [0, 2, 3]]], axis=0).reshape(-1, 9)
    keep = np.sort(rng.choice(len(cen), n_patches, replace=False))
    cen, nrm, area, sid = cen[keep], nrm[keep], area[keep], sid[keep]
    albedo = albedo_s[sid]

    # lamps: 8 ceiling panels and 4 wall windows, as (surface index, centre, half extent)
    lamps = []
    for _ in range(8):
        lamps.append((1, np.array([rng.uniform(1, W - 1), rng.uniform(1, D - 1), H]), 0.6))
    for _ in range(4):
        w = int(rng.integers(2, 6))
        o, u, v = rects[w]
        c = o + u * rng.uniform(0.25, 0.75) + v * rng.uniform(0.45, 0.75)
        lamps.append((w, c, 0.8))
    members = []
    for s, c, h in lamps:
        m = np.nonzero((sid == s) & np.all(np.abs(cen - c) <= h + 1e-6, axis=1))[0]
        if len(m) == 0:   # coarse patch sets: nearest patch of that surface
            cand = np.nonzero(sid == s)[0]
            m = cand[[np.argmin(np.linalg.norm(cen[cand] - c, axis=1))]]
        members.append(m)
    E = np.zeros((n_patches, 3 * n_configs), np.float32)
    for k in range(n_configs):
        chosen = rng.choice(len(lamps), int(rng.integers(1, 4)), replace=False)
        for li in chosen:
            col = rng.uniform(0.4, 1.0, 3) * rng.uniform(2.0, 10.0)
            E[members[li], 3 * k:3 * k + 3] += col.astype(np.float32)
    return {
        "tri": tri.astype(np.float32),
        "pos": cen.astype(np.float32),
        "nrm": nrm.astype(np.float32),
        "area": area.astype(np.float32),
        "albedo": albedo.astype(np.float32),
        "emission": E,
        "surfaces": len(rects),
        "seed": seed,
    }
